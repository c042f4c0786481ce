// GpuWorld: a drop-in World whose internalStep runs on a GB300 through
// libcannon_gpu.so.
//
// The scene is built with the reference's own API (World, Body, Sphere, Box,
// Plane, ConvexPolyhedron, Cylinder, Material, ContactMaterial,
// PointToPointConstraint, HingeConstraint, DistanceConstraint, GSSolver).
// A body with several shapes (Body.addShape) sends its first shape as the
// body's shape and the others, with their offsets and orientations, through
// cp_world_desc.body_shapes.  On the first step, and after markDirty(), the bodies, shapes, materials and
// constraints are packed into a cp_world_desc and uploaded.  Every
// internalStep after that pushes World.time / stepnumber (cp_world_set_time)
// and the per-step body fields an app may have changed (cp_world_set_states:
// pose, velocities, forces, sleep state), runs one cp_world_internal_step,
// and writes back the per-step fields World.internalStep changes
// (lib/world/world_class.dart:433-701; cp_world_get_states).  World.step
// (world_class.dart:392-430) is not overridden: it keeps the only clock,
// adding dt (fixed mode) or timeSinceLastCalled (interpolating mode) after
// the internal steps, and interpolates the written-back poses itself.
// Fields outside cp_body_state (mass, damping, shapes, materials, factors,
// the world inertia of a body the app rotated) travel only with markDirty().
//
// This file is written for a maintainer; it is not compiled in this
// repository (no Dart or Flutter SDK is present).  The C side checks every
// descriptor and returns a status; a failing status throws a StateError with
// the library's message.
import 'dart:ffi';

import 'package:cannon_physics/cannon_physics.dart';
import 'package:ffi/ffi.dart';

import 'src/cannon_gpu_ffi.dart';

class GpuWorld extends World {
  GpuWorld({
    super.gravity,
    super.frictionGravity,
    super.allowSleep,
    super.broadphase,
    super.solver,
    super.quatNormalizeFast,
    super.quatNormalizeSkip,
    this.libraryPath = 'libcannon_gpu.so',
    this.device = 0,
  });

  final String libraryPath;
  final int device;

  CannonGpu? _api;
  Pointer<CpCtx> _ctx = nullptr;
  int _worldId = -1;
  bool _dirty = true;
  Pointer<CpBodyDesc> _bodyBuf = nullptr;
  int _bodyCap = 0;
  // each body's first shape and its first entry in the extra-shape table,
  // as last uploaded
  List<int> _firstShape = const [];
  List<int> _extraFirst = const [];
  List<Shape> _shapeList = const [];  // shape index -> Shape, as uploaded
  Pointer<CpBodyState> _stateBuf = nullptr;
  int _stateCap = 0;

  /// Call after adding or removing bodies, shapes, materials or constraints,
  /// or after changing a body field other than the ones a step writes.
  void markDirty() => _dirty = true;

  CannonGpu get _lib {
    final api = _api ??= CannonGpu(DynamicLibrary.open(libraryPath));
    if (_ctx == nullptr) {
      if (api.abiVersion() != cpAbiVersion) {
        throw StateError('libcannon_gpu ABI ${api.abiVersion()} != $cpAbiVersion');
      }
      final cfg = calloc<CpConfig>();
      final out = calloc<Pointer<CpCtx>>();
      try {
        cfg.ref.device = device;
        _check(api.create(cfg, out));
        _ctx = out.value;
      } finally {
        calloc.free(cfg);
        calloc.free(out);
      }
    }
    return api;
  }

  void _check(int status) {
    if (status != cpOk) throw StateError('cannon_gpu: ${_api!.errorText()}');
  }

  @override
  void internalStep(double dt) {
    final api = _lib;
    if (_dirty) _upload(api);
    // sleepTick inside the step reads World.time as World.step holds it
    _check(api.worldSetTime(_ctx, _worldId, time, stepnumber, accumulator));
    _packStates();
    _check(api.worldSetStates(_ctx, _worldId, _stateBuf, bodies.length));
    _check(api.worldInternalStep(_ctx, _worldId, dt, 1));
    _check(api.worldGetStates(_ctx, _worldId, _stateBuf, bodies.length));
    _unpackStates();
    // World.internalStep's own counter (world_class.dart:680); time is left
    // to World.step
    stepnumber += 1;
    this.dt = dt;
  }

  // ---------------------------------------------------------------- raycasts
  // World.raycastClosest / Any / All (world_class.dart:248-278) answered by
  // cp_world_raycast on the device copy of the world.  The bodies' per-step
  // fields are pushed first, as before a step.

  /// Hits of RAY_ALL beyond this many per ray are dropped.
  int raycastAllMaxHits = 64;

  List<CpRayHit> _cast(Vector3 from, Vector3 to, RayOptions? options, int mode, Arena arena, Pointer<Int32> count) {
    final api = _lib;
    if (_dirty) _upload(api);
    _packStates();
    _check(api.worldSetStates(_ctx, _worldId, _stateBuf, bodies.length));
    final ray = arena<CpRay>();
    _set3(ray.ref.from, from);
    _set3(ray.ref.to, to);
    ray.ref.collisionFilterGroup = options?.collisionFilterGroup ?? -1;
    ray.ref.collisionFilterMask = options?.collisionFilterMask ?? -1;
    ray.ref.skipBackfaces = (options?.skipBackfaces ?? true) ? 1 : 0;
    ray.ref.checkCollisionResponse = (options?.checkCollisionResponse ?? true) ? 1 : 0;
    final maxHits = mode == cpRayAll ? raycastAllMaxHits : 1;
    final hits = arena<CpRayHit>(maxHits);
    _check(api.worldRaycast(_ctx, _worldId, ray, 1, mode, hits, maxHits, count));
    final n = mode == cpRayAll ? (count.value < maxHits ? count.value : maxHits) : 1;
    return [for (var k = 0; k < n; k++) hits[k]];
  }

  void _fill(RaycastResult r, CpRayHit h, Vector3 from, Vector3 to) {
    r.reset();
    r.hitFaceIndex = h.hitFaceIndex;
    if (h.hasHit == 0) return;
    r.set(from, to, Vector3(h.hitNormal[0], h.hitNormal[1], h.hitNormal[2]),
        Vector3(h.hitPoint[0], h.hitPoint[1], h.hitPoint[2]), _shapeList[h.shape], bodies[h.body], h.distance);
    r.hasHit = true;
  }

  @override
  bool raycastClosest([Vector3? from, Vector3? to, RayOptions? options, RaycastResult? result]) =>
      _castOne(from, to, options, result, cpRayClosest);

  @override
  bool raycastAny([Vector3? from, Vector3? to, RayOptions? options, RaycastResult? result]) =>
      _castOne(from, to, options, result, cpRayAny);

  bool _castOne(Vector3? from, Vector3? to, RayOptions? options, RaycastResult? result, int mode) {
    final f = from ?? options?.from ?? Vector3.zero();
    final t = to ?? options?.to ?? Vector3.zero();
    final arena = Arena();
    try {
      final h = _cast(f, t, options, mode, arena, arena<Int32>())[0];
      if (result != null) _fill(result, h, f, t);
      return h.hasHit != 0;
    } finally {
      arena.releaseAll();
    }
  }

  @override
  bool raycastAll([Vector3? from, Vector3? to, RayOptions? options, RaycastCallback? callback]) {
    final f = from ?? options?.from ?? Vector3.zero();
    final t = to ?? options?.to ?? Vector3.zero();
    final arena = Arena();
    try {
      final count = arena<Int32>();
      final hits = _cast(f, t, options, cpRayAll, arena, count);
      final r = RaycastResult();
      for (final h in hits) {
        _fill(r, h, f, t);
        callback?.call(r);
      }
      return count.value > 0;
    } finally {
      arena.releaseAll();
    }
  }

  /// Releases the device world and the context.
  void dispose() {
    final api = _api;
    if (api == null) return;
    if (_worldId >= 0) api.worldDestroy(_ctx, _worldId);
    if (_ctx != nullptr) api.destroy(_ctx);
    if (_bodyBuf != nullptr) calloc.free(_bodyBuf);
    if (_stateBuf != nullptr) calloc.free(_stateBuf);
    _worldId = -1;
    _ctx = nullptr;
    _bodyBuf = nullptr;
    _stateBuf = nullptr;
  }

  // ---------------------------------------------------------------- packing

  static int _shapeType(Shape s) {
    switch (s.type) {
      case ShapeType.sphere:
        return cpShapeSphere;
      case ShapeType.plane:
        return cpShapePlane;
      case ShapeType.box:
        return cpShapeBox;
      case ShapeType.convex:
        return cpShapeConvex;
      case ShapeType.cylinder:
        return cpShapeCylinder;
      case ShapeType.capsule:
        return cpShapeCapsule;
      case ShapeType.cone:
        return cpShapeCone;
      case ShapeType.sizedPlane:
        return cpShapeSizedPlane;
      default:
        throw UnsupportedError('GpuWorld: shape type ${s.type} is not on the GPU path');
    }
  }

  void _ensureBodyBuf() {
    if (_bodyCap >= bodies.length) return;
    if (_bodyBuf != nullptr) calloc.free(_bodyBuf);
    _bodyCap = bodies.length < 16 ? 16 : bodies.length;
    _bodyBuf = calloc<CpBodyDesc>(_bodyCap);
  }

  void _upload(CannonGpu api) {
    if (_worldId >= 0) {
      _check(api.worldDestroy(_ctx, _worldId));
      _worldId = -1;
    }
    final arena = Arena();
    try {
      // materials: every Material reachable from shapes, bodies and contact
      // materials, in first-seen order
      final mats = <Material>[];
      int matIndex(Material? m) {
        if (m == null) return -1;
        final i = mats.indexOf(m);
        if (i >= 0) return i;
        mats.add(m);
        return mats.length - 1;
      }

      // every body's shapes in Body.shapes order: the first is the body's
      // `shape`, the others (a compound body) go to the extra-shape table
      _firstShape = List<int>.filled(bodies.length, -1);
      _extraFirst = List<int>.filled(bodies.length, 0);
      var numShapes = 0, numExtra = 0;
      for (var i = 0; i < bodies.length; i++) {
        final n = bodies[i].shapes.length;
        if (n > 0) {
          _firstShape[i] = numShapes;
          _extraFirst[i] = numExtra;
          numShapes += n;
          numExtra += n - 1;
        }
      }
      final shapes = arena<CpShapeDesc>(numShapes == 0 ? 1 : numShapes);
      final bodyShapes = arena<CpBodyShape>(numExtra == 0 ? 1 : numExtra);
      final vertexBuffers = <Pointer<Float>>[];
      _ensureBodyBuf();
      final shapeList = <Shape>[];
      for (var i = 0; i < bodies.length; i++) {
        final b = bodies[i];
        for (var k = 0; k < b.shapes.length; k++) {
          shapeList.add(b.shapes[k]);
          if (k == 0) continue;
          final e = bodyShapes[_extraFirst[i] + k - 1];
          e.shape = _firstShape[i] + k;
          _set3(e.offset, b.shapeOffsets[k]);
          _setQ(e.orientation, b.shapeOrientations[k]);
        }
        matIndex(b.material);
      }
      _shapeList = shapeList;
      for (var i = 0; i < shapeList.length; i++) {
        final s = shapeList[i];
        final d = shapes[i];
        d.type = _shapeType(s);
        d.collisionFilterGroup = s.collisionFilterGroup;
        d.collisionFilterMask = s.collisionFilterMask;
        d.collisionResponse = s.collisionResponse ? 1 : 0;
        d.material = matIndex(s.material);
        d.boundingSphereRadius = s.boundingSphereRadius;
        if (s is Sphere) d.radius = s.radius;
        if (s is Box) {
          d.halfExtents[0] = s.halfExtents.x;
          d.halfExtents[1] = s.halfExtents.y;
          d.halfExtents[2] = s.halfExtents.z;
        }
        if (s is Cylinder) {
          d.radiusTop = s.radiusTop;
          d.radiusBottom = s.radiusBottom;
          d.height = s.height;
          d.numSegments = s.numSegments;
        } else if (s is ConvexPolyhedron) {
          final nv = s.vertices.length;
          final verts = arena<Float>(3 * nv);
          for (var k = 0; k < nv; k++) {
            verts[3 * k] = s.vertices[k].x;
            verts[3 * k + 1] = s.vertices[k].y;
            verts[3 * k + 2] = s.vertices[k].z;
          }
          final nf = s.faces.length;
          final sizes = arena<Int32>(nf);
          var total = 0;
          for (var f = 0; f < nf; f++) {
            sizes[f] = s.faces[f].length;
            total += s.faces[f].length;
          }
          final idx = arena<Int32>(total);
          var o = 0;
          for (final face in s.faces) {
            for (final v in face) {
              idx[o++] = v;
            }
          }
          d.numVertices = nv;
          d.numFaces = nf;
          d.vertices = verts;
          d.faceSizes = sizes;
          d.faceIndices = idx;
          final axes = s.uniqueAxes;
          if (axes != null) {
            final ax = arena<Float>(3 * axes.length);
            for (var k = 0; k < axes.length; k++) {
              ax[3 * k] = axes[k].x;
              ax[3 * k + 1] = axes[k].y;
              ax[3 * k + 2] = axes[k].z;
            }
            d.hasAxes = 1;
            d.numAxes = axes.length;
            d.axes = ax;
          }
          vertexBuffers.add(verts);
        }
        _check(api.shapeSetup(d));
      }
      _packBodies(materialIndex: matIndex);

      final cmats = arena<CpContactMaterial>(contactmaterials.isEmpty ? 1 : contactmaterials.length);
      for (var k = 0; k < contactmaterials.length; k++) {
        final cm = contactmaterials[k];
        _fillContactMaterial(cmats[k], cm, matIndex(cm.materials[0]), matIndex(cm.materials[1]));
      }
      final mtab = arena<CpMaterial>(mats.isEmpty ? 1 : mats.length);
      for (var k = 0; k < mats.length; k++) {
        mtab[k].friction = mats[k].friction;
        mtab[k].restitution = mats[k].restitution;
      }

      final cons = arena<CpConstraintDesc>(constraints.isEmpty ? 1 : constraints.length);
      for (var k = 0; k < constraints.length; k++) {
        _fillConstraint(cons[k], constraints[k]);
      }

      final w = arena<CpWorldDesc>();
      final r = w.ref;
      r.numBodies = bodies.length;
      r.numShapes = numShapes;
      r.numMaterials = mats.length;
      r.numContactMaterials = contactmaterials.length;
      r.numConstraints = constraints.length;
      r.allowSleep = allowSleep ? 1 : 0;
      r.quatNormalizeSkip = quatNormalizeSkip;
      r.quatNormalizeFast = quatNormalizeFast ? 1 : 0;
      // GSSolver, or SplitSolver over a GSSolver with the SplitSolver's
      // iterations and tolerance (split_solver.dart:91-92); equation ids
      // continue from Equation.idCounter
      r.solverIterations = solver.iterations;
      r.solverTolerance = solver.tolerance;
      r.solver = solver is SplitSolver ? cpSolverSplit : cpSolverGs;
      r.equationIdCounter = Equation.idCounter;
      r.useBoundingBoxes = broadphase.useBoundingBoxes ? 1 : 0;
      r.enableFrictionReduction = narrowphase.enableFrictionReduction ? 1 : 0;
      final bp = broadphase;
      if (bp is SAPBroadphase) {
        r.broadphase = cpBroadSap;
        r.sapAxis = bp.axisIndex.index;
      } else if (bp is GridBroadphase) {
        r.broadphase = cpBroadGrid;
        r.gridN[0] = bp.nx;
        r.gridN[1] = bp.ny;
        r.gridN[2] = bp.nz;
        r.gridAabbMin[0] = bp.aabbMin.x;
        r.gridAabbMin[1] = bp.aabbMin.y;
        r.gridAabbMin[2] = bp.aabbMin.z;
        r.gridAabbMax[0] = bp.aabbMax.x;
        r.gridAabbMax[1] = bp.aabbMax.y;
        r.gridAabbMax[2] = bp.aabbMax.z;
      } else {
        r.broadphase = cpBroadNaive;
      }
      r.stepnumber = stepnumber;
      r.time = time;
      r.gravity[0] = gravity.x;
      r.gravity[1] = gravity.y;
      r.gravity[2] = gravity.z;
      final fg = frictionGravity;
      if (fg != null) {
        r.hasFrictionGravity = 1;
        r.frictionGravity[0] = fg.x;
        r.frictionGravity[1] = fg.y;
        r.frictionGravity[2] = fg.z;
      }
      r.bodies = _bodyBuf;
      r.shapes = shapes;
      r.materials = mtab;
      r.contactMaterials = cmats;
      r.constraints = cons;
      r.sapAxisList = nullptr;
      r.bodyShapes = bodyShapes;
      r.numBodyShapes = numExtra;
      _fillContactMaterial(r.defaultContactMaterial, defaultContactMaterial, -1, -1);

      final id = arena<Int32>();
      _check(api.worldCreate(_ctx, w, id));
      _worldId = id.value;
      _dirty = false;
    } finally {
      arena.releaseAll();
    }
  }

  static void _fillContactMaterial(CpContactMaterial d, ContactMaterial cm, int a, int b) {
    d.materialA = a;
    d.materialB = b;
    d.friction = cm.friction;
    d.restitution = cm.restitution;
    d.contactStiffness = cm.contactEquationStiffness;
    d.contactRelaxation = cm.contactEquationRelaxation;
    d.frictionStiffness = cm.frictionEquationStiffness;
    d.frictionRelaxation = cm.frictionEquationRelaxation;
  }

  void _fillConstraint(CpConstraintDesc d, Constraint c) {
    d.bodyA = bodies.indexOf(c.bodyA);
    d.bodyB = bodies.indexOf(c.bodyB);
    d.collideConnected = c.collideConnected ? 1 : 0;
    final eq = c.equations.first;
    d.firstEquationId = eq.id;
    d.spookStiffness = eq.stiffness;
    d.spookRelaxation = eq.relaxation;
    d.spookTimeStep = 1 / 60;
    d.maxForce = eq.maxForce;
    if (c is LockConstraint) {
      // the local frames the constructor stored (lock_constraint.dart:26-76)
      d.type = cpConLock;
      _set3(d.pivotA, c.pivotA);
      _set3(d.pivotB, c.pivotB);
      final axes = [c.xA, c.xB, c.yA, c.yB, c.zA, c.zB];
      for (var v = 0; v < 6; v++) {
        d.lockAxes[v][0] = axes[v].x;
        d.lockAxes[v][1] = axes[v].y;
        d.lockAxes[v][2] = axes[v].z;
      }
    } else if (c is ConeTwistConstraint) {
      d.type = cpConConeTwist;
      _set3(d.pivotA, c.pivotA);
      _set3(d.pivotB, c.pivotB);
      _set3(d.axisA, c.axisA);
      _set3(d.axisB, c.axisB);
      d.angle = c.angle;
      d.twistAngle = c.twistAngle;
    } else if (c is SpringConstraint) {
      // rest length: the bodies' distance when the world is uploaded (the
      // constructor's value is private to the reference library); the row's
      // force bound is the stiffness
      d.type = cpConSpring;
      d.distance = -1;
      d.maxForce = c.stiffness;
    } else if (c is HingeConstraint) {
      d.type = cpConHinge;
      _set3(d.pivotA, c.pivotA);
      _set3(d.pivotB, c.pivotB);
      _set3(d.axisA, c.axisA);
      _set3(d.axisB, c.axisB);
      d.motorEnabled = c.motorEquation.enabled ? 1 : 0;
      d.motorTargetVelocity = c.motorTargetVelocity ?? 0;
      d.motorMaxForce = c.motorEquation.maxForce;
    } else if (c is PointToPointConstraint) {
      d.type = cpConPointToPoint;
      _set3(d.pivotA, c.pivotA);
      _set3(d.pivotB, c.pivotB);
    } else if (c is DistanceConstraint) {
      d.type = cpConDistance;
      d.distance = c.distance;
    } else {
      throw UnsupportedError('GpuWorld: ${c.runtimeType} is not on the GPU path');
    }
  }

  static void _set3(Array<Float> a, Vector3 v) {
    a[0] = v.x;
    a[1] = v.y;
    a[2] = v.z;
  }

  void _packBodies({int Function(Material?)? materialIndex}) {
    _ensureBodyBuf();
    for (var i = 0; i < bodies.length; i++) {
      final b = bodies[i];
      final d = _bodyBuf[i];
      _set3(d.position, b.position);
      d.quaternion[0] = b.quaternion.x;
      d.quaternion[1] = b.quaternion.y;
      d.quaternion[2] = b.quaternion.z;
      d.quaternion[3] = b.quaternion.w;
      _set3(d.velocity, b.velocity);
      _set3(d.angularVelocity, b.angularVelocity);
      _set3(d.force, b.force);
      _set3(d.torque, b.torque);
      _set3(d.linearFactor, b.linearFactor);
      _set3(d.angularFactor, b.angularFactor);
      _set3(d.invInertia, b.invInertia);
      for (var k = 0; k < 9; k++) {
        d.invInertiaWorld[k] = b.invInertiaWorld.storage[k];
      }
      _set3(d.aabbLower, b.aabb.lowerBound);
      _set3(d.aabbUpper, b.aabb.upperBound);
      if (b.shapes.isNotEmpty) {
        _set3(d.shapeOffset, b.shapeOffsets[0]);
        _setQ(d.shapeOrientation, b.shapeOrientations[0]);
      } else {
        _set3(d.shapeOffset, Vector3.zero());
        _setQ(d.shapeOrientation, Quaternion(0, 0, 0, 1));
      }
      _set3(d.previousPosition, b.previousPosition);
      d.previousQuaternion[0] = b.previousQuaternion.x;
      d.previousQuaternion[1] = b.previousQuaternion.y;
      d.previousQuaternion[2] = b.previousQuaternion.z;
      d.previousQuaternion[3] = b.previousQuaternion.w;
      d.mass = b.mass;
      d.invMass = b.invMass;
      d.linearDamping = b.linearDamping;
      d.angularDamping = b.angularDamping;
      d.sleepSpeedLimit = b.sleepSpeedLimit;
      d.sleepTimeLimit = b.sleepTimeLimit.toDouble();
      d.timeLastSleepy = b.timeLastSleepy.toDouble();
      d.boundingRadius = b.boundingRadius;
      d.type = b.type.index;
      d.sleepState = b.sleepState.index;
      d.allowSleep = b.allowSleep ? 1 : 0;
      d.wakeUpAfterNarrowphase = b.wakeUpAfterNarrowphase ? 1 : 0;
      d.collisionFilterGroup = b.collisionFilterGroup;
      d.collisionFilterMask = b.collisionFilterMask;
      d.collisionResponse = b.collisionResponse ? 1 : 0;
      d.isTrigger = b.isTrigger ? 1 : 0;
      if (materialIndex != null) d.material = materialIndex(b.material);
      d.shape = _firstShape[i];
      d.extraShapesFirst = _extraFirst[i];
      d.extraShapesCount = b.shapes.isEmpty ? 0 : b.shapes.length - 1;
      d.fixedRotation = b.fixedRotation ? 1 : 0;
      d.aabbNeedsUpdate = b.aabbNeedsUpdate ? 1 : 0;
    }
  }

  void _ensureStateBuf() {
    if (_stateCap >= bodies.length) return;
    if (_stateBuf != nullptr) calloc.free(_stateBuf);
    _stateCap = bodies.length < 16 ? 16 : bodies.length;
    _stateBuf = calloc<CpBodyState>(_stateCap);
  }

  static void _setQ(Array<Float> a, Quaternion q) {
    a[0] = q.x;
    a[1] = q.y;
    a[2] = q.z;
    a[3] = q.w;
  }

  void _packStates() {
    _ensureStateBuf();
    for (var i = 0; i < bodies.length; i++) {
      final b = bodies[i];
      final d = _stateBuf[i];
      _set3(d.position, b.position);
      _setQ(d.quaternion, b.quaternion);
      _set3(d.velocity, b.velocity);
      _set3(d.angularVelocity, b.angularVelocity);
      _set3(d.force, b.force);
      _set3(d.torque, b.torque);
      _set3(d.previousPosition, b.previousPosition);
      _setQ(d.previousQuaternion, b.previousQuaternion);
      _set3(d.interpolatedPosition, b.interpolatedPosition);
      _setQ(d.interpolatedQuaternion, b.interpolatedQuaternion);
      d.sleepState = b.sleepState.index;
      d.wakeUpAfterNarrowphase = b.wakeUpAfterNarrowphase ? 1 : 0;
      d.aabbNeedsUpdate = b.aabbNeedsUpdate ? 1 : 0;
      d.timeLastSleepy = b.timeLastSleepy.toDouble();
    }
  }

  void _unpackStates() {
    for (var i = 0; i < bodies.length; i++) {
      final b = bodies[i];
      final d = _stateBuf[i];
      b.position.setValues(d.position[0], d.position[1], d.position[2]);
      b.quaternion.setValues(d.quaternion[0], d.quaternion[1], d.quaternion[2], d.quaternion[3]);
      b.velocity.setValues(d.velocity[0], d.velocity[1], d.velocity[2]);
      b.angularVelocity.setValues(d.angularVelocity[0], d.angularVelocity[1], d.angularVelocity[2]);
      b.force.setZero();
      b.torque.setZero();
      b.previousPosition.setValues(d.previousPosition[0], d.previousPosition[1], d.previousPosition[2]);
      b.previousQuaternion.setValues(
          d.previousQuaternion[0], d.previousQuaternion[1], d.previousQuaternion[2], d.previousQuaternion[3]);
      b.aabbNeedsUpdate = d.aabbNeedsUpdate != 0;
      b.sleepState = BodySleepStates.values[d.sleepState];
      b.timeLastSleepy = d.timeLastSleepy;
      b.wakeUpAfterNarrowphase = d.wakeUpAfterNarrowphase != 0;
    }
  }
}
