// dart:ffi mirror of include/cannon_gpu.h.
//
// Struct layouts follow the C header field by field; the C side checks the
// ABI version at load time (cp_abi_version).  Nothing here allocates device
// memory: the library owns it, and every pointer passed in is read or written
// only during the call.
import 'dart:ffi';

const int cpAbiVersion = 4;

const int cpOk = 0;
const int cpErrArg = 1;
const int cpErrCapacity = 2;
const int cpErrNonfinite = 3;
const int cpErrTimeout = 4;
const int cpErrOom = 5;
const int cpErrCuda = 6;
const int cpErrUnsupported = 7;

const int cpShapeSphere = 0, cpShapePlane = 1, cpShapeBox = 2, cpShapeConvex = 3, cpShapeCylinder = 4;
const int cpShapeCapsule = 5, cpShapeCone = 6, cpShapeSizedPlane = 7;
const int cpBroadNaive = 0, cpBroadSap = 1, cpBroadGrid = 2;
const int cpConPointToPoint = 0, cpConHinge = 1, cpConDistance = 2;
const int cpConLock = 3, cpConConeTwist = 4, cpConSpring = 5;
const int cpSolverGs = 0, cpSolverSplit = 1;

final class CpShapeDesc extends Struct {
  @Int32() external int type;
  @Int32() external int collisionFilterGroup;
  @Int32() external int collisionFilterMask;
  @Int32() external int collisionResponse;
  @Int32() external int material;
  @Int32() external int numSegments;
  @Double() external double radius;
  @Double() external double radiusTop;
  @Double() external double radiusBottom;
  @Double() external double height;
  @Array(3) external Array<Float> halfExtents;
  @Int32() external int numVertices;
  @Int32() external int numFaces;
  @Int32() external int numAxes;
  @Int32() external int hasAxes;
  external Pointer<Float> vertices;
  external Pointer<Int32> faceSizes;
  external Pointer<Int32> faceIndices;
  external Pointer<Float> axes;
  @Double() external double boundingSphereRadius;
}

final class CpBodyDesc extends Struct {
  @Array(3) external Array<Float> position;
  @Array(4) external Array<Float> quaternion;
  @Array(3) external Array<Float> velocity;
  @Array(3) external Array<Float> angularVelocity;
  @Array(3) external Array<Float> force;
  @Array(3) external Array<Float> torque;
  @Array(3) external Array<Float> linearFactor;
  @Array(3) external Array<Float> angularFactor;
  @Array(3) external Array<Float> invInertia;
  @Array(9) external Array<Float> invInertiaWorld;
  @Array(3) external Array<Float> aabbLower;
  @Array(3) external Array<Float> aabbUpper;
  @Array(3) external Array<Float> shapeOffset;
  @Array(4) external Array<Float> shapeOrientation;
  @Array(3) external Array<Float> previousPosition;
  @Array(4) external Array<Float> previousQuaternion;
  @Double() external double mass;
  @Double() external double invMass;
  @Double() external double linearDamping;
  @Double() external double angularDamping;
  @Double() external double sleepSpeedLimit;
  @Double() external double sleepTimeLimit;
  @Double() external double timeLastSleepy;
  @Double() external double boundingRadius;
  @Int32() external int type;
  @Int32() external int sleepState;
  @Int32() external int allowSleep;
  @Int32() external int wakeUpAfterNarrowphase;
  @Int32() external int collisionFilterGroup;
  @Int32() external int collisionFilterMask;
  @Int32() external int collisionResponse;
  @Int32() external int isTrigger;
  @Int32() external int material;
  @Int32() external int shape;
  @Int32() external int fixedRotation;
  @Int32() external int aabbNeedsUpdate;
  @Array(3) external Array<Float> interpolatedPosition;
  @Array(4) external Array<Float> interpolatedQuaternion;
  @Int32() external int extraShapesFirst;
  @Int32() external int extraShapesCount;
}

/// cp_body_shape: a compound body's second, third, ... shape.
final class CpBodyShape extends Struct {
  @Int32() external int shape;
  @Array(3) external Array<Float> offset;
  @Array(4) external Array<Float> orientation;
}

final class CpBodyState extends Struct {
  @Array(3) external Array<Float> position;
  @Array(4) external Array<Float> quaternion;
  @Array(3) external Array<Float> velocity;
  @Array(3) external Array<Float> angularVelocity;
  @Array(3) external Array<Float> force;
  @Array(3) external Array<Float> torque;
  @Array(3) external Array<Float> previousPosition;
  @Array(4) external Array<Float> previousQuaternion;
  @Array(3) external Array<Float> interpolatedPosition;
  @Array(4) external Array<Float> interpolatedQuaternion;
  @Int32() external int sleepState;
  @Int32() external int wakeUpAfterNarrowphase;
  @Int32() external int aabbNeedsUpdate;
  @Int32() external int pad0;
  @Double() external double timeLastSleepy;
}

final class CpMaterial extends Struct {
  @Double() external double friction;
  @Double() external double restitution;
}

final class CpContactMaterial extends Struct {
  @Int32() external int materialA;
  @Int32() external int materialB;
  @Double() external double friction;
  @Double() external double restitution;
  @Double() external double contactStiffness;
  @Double() external double contactRelaxation;
  @Double() external double frictionStiffness;
  @Double() external double frictionRelaxation;
}

final class CpConstraintDesc extends Struct {
  @Int32() external int type;
  @Int32() external int bodyA;
  @Int32() external int bodyB;
  @Int32() external int collideConnected;
  @Int32() external int motorEnabled;
  @Int32() external int pad0;
  @Array(3) external Array<Float> pivotA;
  @Array(3) external Array<Float> pivotB;
  @Array(3) external Array<Float> axisA;
  @Array(3) external Array<Float> axisB;
  @Double() external double distance;
  @Double() external double maxForce;
  @Double() external double motorTargetVelocity;
  @Double() external double motorMaxForce;
  @Double() external double spookStiffness;
  @Double() external double spookRelaxation;
  @Double() external double spookTimeStep;
  @Array(6, 3) external Array<Array<Float>> lockAxes;
  @Double() external double angle;
  @Double() external double twistAngle;
  @Int64() external int firstEquationId;
}

final class CpWorldDesc extends Struct {
  @Int32() external int numBodies;
  @Int32() external int numShapes;
  @Int32() external int numMaterials;
  @Int32() external int numContactMaterials;
  @Int32() external int numConstraints;
  @Int32() external int allowSleep;
  @Int32() external int quatNormalizeSkip;
  @Int32() external int quatNormalizeFast;
  @Int32() external int solverIterations;
  @Int32() external int broadphase;
  @Int32() external int useBoundingBoxes;
  @Int32() external int sapAxis;
  @Array(3) external Array<Int32> gridN;
  @Int32() external int enableFrictionReduction;
  @Int32() external int hasFrictionGravity;
  @Int32() external int stepnumber;
  @Double() external double solverTolerance;
  @Double() external double time;
  @Array(3) external Array<Float> gravity;
  @Array(3) external Array<Float> frictionGravity;
  @Array(3) external Array<Float> gridAabbMin;
  @Array(3) external Array<Float> gridAabbMax;
  external Pointer<CpBodyDesc> bodies;
  external Pointer<CpShapeDesc> shapes;
  external Pointer<CpMaterial> materials;
  external Pointer<CpContactMaterial> contactMaterials;
  external Pointer<CpConstraintDesc> constraints;
  external Pointer<Int32> sapAxisList;
  external CpContactMaterial defaultContactMaterial;
  external Pointer<CpBodyShape> bodyShapes;
  @Int32() external int numBodyShapes;
  @Int32() external int solver;
  @Int64() external int equationIdCounter;
}

/// cp_ray: one ray of World.raycastClosest / Any / All.
final class CpRay extends Struct {
  @Array(3) external Array<Float> from;
  @Array(3) external Array<Float> to;
  @Int32() external int collisionFilterGroup;
  @Int32() external int collisionFilterMask;
  @Int32() external int skipBackfaces;
  @Int32() external int checkCollisionResponse;
}

/// cp_ray_hit: a RaycastResult.
final class CpRayHit extends Struct {
  @Int32() external int hasHit;
  @Int32() external int body;
  @Int32() external int shape;
  @Int32() external int hitFaceIndex;
  @Array(3) external Array<Float> hitPoint;
  @Array(3) external Array<Float> hitNormal;
  @Double() external double distance;
}

const int cpRayClosest = 0, cpRayAny = 1, cpRayAll = 2;

final class CpStepInfo extends Struct {
  @Int64() external int stepnumber;
  @Double() external double time;
  @Int32() external int numPairs;
  @Int32() external int numContacts;
  @Int32() external int numRows;
  @Int32() external int iterations;
  @Int32() external int status;
  @Int32() external int numBodies;
  @Int32() external int numLevels;
  @Int32() external int substeps;
  @Double() external double accumulator;
}

final class CpConfig extends Struct {
  @Int32() external int device;
  @Int32() external int blockThreads;
  @Int64() external int arenaBytes;
}

final class CpCtx extends Opaque {}

/// The entry points of libcannon_gpu.so that the drop-in uses.
class CannonGpu {
  CannonGpu(DynamicLibrary lib)
      : abiVersion = lib.lookupFunction<Int32 Function(), int Function()>('cp_abi_version'),
        lastError = lib.lookupFunction<Pointer<Uint8> Function(), Pointer<Uint8> Function()>('cp_last_error'),
        shapeSetup = lib.lookupFunction<Int32 Function(Pointer<CpShapeDesc>), int Function(Pointer<CpShapeDesc>)>(
            'cp_shape_setup'),
        bodySetup = lib.lookupFunction<
            Int32 Function(Pointer<CpShapeDesc>, Int32, Pointer<CpBodyShape>, Int32, Pointer<CpBodyDesc>, Int32),
            int Function(Pointer<CpShapeDesc>, int, Pointer<CpBodyShape>, int, Pointer<CpBodyDesc>, int)>('cp_body_setup'),
        create = lib.lookupFunction<Int32 Function(Pointer<CpConfig>, Pointer<Pointer<CpCtx>>),
            int Function(Pointer<CpConfig>, Pointer<Pointer<CpCtx>>)>('cp_create'),
        destroy = lib.lookupFunction<Int32 Function(Pointer<CpCtx>), int Function(Pointer<CpCtx>)>('cp_destroy'),
        worldCreate = lib.lookupFunction<Int32 Function(Pointer<CpCtx>, Pointer<CpWorldDesc>, Pointer<Int32>),
            int Function(Pointer<CpCtx>, Pointer<CpWorldDesc>, Pointer<Int32>)>('cp_world_create'),
        worldDestroy = lib.lookupFunction<Int32 Function(Pointer<CpCtx>, Int32), int Function(Pointer<CpCtx>, int)>(
            'cp_world_destroy'),
        worldStep = lib.lookupFunction<Int32 Function(Pointer<CpCtx>, Int32, Double, Int32),
            int Function(Pointer<CpCtx>, int, double, int)>('cp_world_step'),
        worldGetBodies = lib.lookupFunction<Int32 Function(Pointer<CpCtx>, Int32, Pointer<CpBodyDesc>, Int32),
            int Function(Pointer<CpCtx>, int, Pointer<CpBodyDesc>, int)>('cp_world_get_bodies'),
        worldSetBodies = lib.lookupFunction<Int32 Function(Pointer<CpCtx>, Int32, Pointer<CpBodyDesc>, Int32),
            int Function(Pointer<CpCtx>, int, Pointer<CpBodyDesc>, int)>('cp_world_set_bodies'),
        worldGetInfo = lib.lookupFunction<Int32 Function(Pointer<CpCtx>, Int32, Pointer<CpStepInfo>),
            int Function(Pointer<CpCtx>, int, Pointer<CpStepInfo>)>('cp_world_get_info'),
        worldInternalStep = lib.lookupFunction<Int32 Function(Pointer<CpCtx>, Int32, Double, Int32),
            int Function(Pointer<CpCtx>, int, double, int)>('cp_world_internal_step'),
        worldSetTime = lib.lookupFunction<Int32 Function(Pointer<CpCtx>, Int32, Double, Int64, Double),
            int Function(Pointer<CpCtx>, int, double, int, double)>('cp_world_set_time'),
        worldGetStates = lib.lookupFunction<Int32 Function(Pointer<CpCtx>, Int32, Pointer<CpBodyState>, Int32),
            int Function(Pointer<CpCtx>, int, Pointer<CpBodyState>, int)>('cp_world_get_states'),
        worldSetStates = lib.lookupFunction<Int32 Function(Pointer<CpCtx>, Int32, Pointer<CpBodyState>, Int32),
            int Function(Pointer<CpCtx>, int, Pointer<CpBodyState>, int)>('cp_world_set_states'),
        worldStepStatic = lib.lookupFunction<Int32 Function(Pointer<CpCtx>, Int32, Double, Int32),
            int Function(Pointer<CpCtx>, int, double, int)>('cp_world_step_static'),
        batchStep = lib.lookupFunction<Int32 Function(Pointer<CpCtx>, Pointer<Int32>, Int32, Double, Int32),
            int Function(Pointer<CpCtx>, Pointer<Int32>, int, double, int)>('cp_batch_step'),
        worldRaycast = lib.lookupFunction<
            Int32 Function(Pointer<CpCtx>, Int32, Pointer<CpRay>, Int32, Int32, Pointer<CpRayHit>, Int32, Pointer<Int32>),
            int Function(Pointer<CpCtx>, int, Pointer<CpRay>, int, int, Pointer<CpRayHit>, int, Pointer<Int32>)>(
            'cp_world_raycast');

  final int Function() abiVersion;
  final Pointer<Uint8> Function() lastError;
  final int Function(Pointer<CpShapeDesc>) shapeSetup;
  final int Function(Pointer<CpShapeDesc>, int, Pointer<CpBodyShape>, int, Pointer<CpBodyDesc>, int) bodySetup;
  final int Function(Pointer<CpConfig>, Pointer<Pointer<CpCtx>>) create;
  final int Function(Pointer<CpCtx>) destroy;
  final int Function(Pointer<CpCtx>, Pointer<CpWorldDesc>, Pointer<Int32>) worldCreate;
  final int Function(Pointer<CpCtx>, int) worldDestroy;
  final int Function(Pointer<CpCtx>, int, double, int) worldStep;
  final int Function(Pointer<CpCtx>, int, Pointer<CpBodyDesc>, int) worldGetBodies;
  final int Function(Pointer<CpCtx>, int, Pointer<CpBodyDesc>, int) worldSetBodies;
  final int Function(Pointer<CpCtx>, int, Pointer<CpStepInfo>) worldGetInfo;

  /// World.internalStep on the device: stepnumber advances, time does not.
  final int Function(Pointer<CpCtx>, int, double, int) worldInternalStep;

  /// World.time, World.stepnumber and World.accumulator of the device world.
  final int Function(Pointer<CpCtx>, int, double, int, double) worldSetTime;

  /// The per-step Body fields only (cp_body_state).
  final int Function(Pointer<CpCtx>, int, Pointer<CpBodyState>, int) worldGetStates;
  final int Function(Pointer<CpCtx>, int, Pointer<CpBodyState>, int) worldSetStates;

  /// `worldStep` without device allocation (fixed step scratch; a world too
  /// large for it, or a step that overflows a list, returns CP_ERR_CAPACITY).
  final int Function(Pointer<CpCtx>, int, double, int) worldStepStatic;

  /// Many independent worlds stepped together: ids, count, dt, steps.
  final int Function(Pointer<CpCtx>, Pointer<Int32>, int, double, int) batchStep;

  /// Rays against a world's resident state: ctx, world, rays, n, mode, hits,
  /// max hits per ray (RAY_ALL), counts (RAY_ALL).
  final int Function(Pointer<CpCtx>, int, Pointer<CpRay>, int, int, Pointer<CpRayHit>, int, Pointer<Int32>) worldRaycast;

  /// The thread-local message of the last failing call.
  String errorText() {
    final p = lastError();
    final bytes = <int>[];
    for (var i = 0; p[i] != 0; i++) {
      bytes.add(p[i]);
    }
    return String.fromCharCodes(bytes);
  }
}
