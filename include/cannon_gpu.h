/*
 * cannon_gpu.h -- C ABI of the GB300 World.step engine for cannon_physics.
 *
 * The reference (Dart package cannon_physics 0.0.2) has no FFI.  Its pluggable
 * seams are Dart objects hung on World: `World.internalStep(double dt)`
 * (lib/world/world_class.dart:433-701), `Broadphase.collisionPairs`
 * (lib/collision/broadphase.dart:39), `Narrowphase.getContacts`
 * (lib/world/narrow_phase.dart:634) and `Solver.solve`
 * (lib/solver/gs_solver.dart:74).  A Dart `GpuWorld extends World` overrides
 * `internalStep` and reaches the entry points below through dart:ffi; every
 * entry point names the reference code it stands in for.
 *
 * Conventions
 *  - Every call returns a status (CP_OK or a CP_ERR_* code); `cp_last_error`
 *    gives a thread-local message for the last failing call.
 *  - No pointer passed in is retained after the call returns; host buffers are
 *    read or written only during the call.
 *  - Vector fields are binary32 because the reference stores Vector3,
 *    Quaternion and Matrix3 components in Float32List (package:vector_math);
 *    scalars (mass, damping, radii, time) are binary64 like Dart doubles.
 *  - Matrix3 storage is the 9-float array the reference indexes as
 *    e[3*row+col] (lib/math/mat3.dart:9-108).
 *  - Calls on one context are serialized by the context.
 */
#ifndef CANNON_GPU_H
#define CANNON_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CP_ABI_VERSION 4

/* status codes */
#define CP_OK               0
#define CP_ERR_ARG          1   /* invalid argument or descriptor */
#define CP_ERR_CAPACITY     2   /* a scratch capacity was exceeded (state left as before the step) */
#define CP_ERR_NONFINITE    3   /* NaN/Inf found in body state after a step */
#define CP_ERR_TIMEOUT      4   /* a bounded device-side wait gave up */
#define CP_ERR_OOM          5   /* device or host allocation failed */
#define CP_ERR_CUDA         6   /* CUDA runtime error */
#define CP_ERR_UNSUPPORTED  7   /* feature outside the supported subset */

/* ShapeType order of lib/rigid_body_shapes/shape.dart:6-18 (the order decides
 * which shape is passed first to a narrowphase resolver). */
enum cp_shape_type {
  CP_SHAPE_SPHERE = 0,
  CP_SHAPE_PLANE = 1,
  CP_SHAPE_BOX = 2,
  CP_SHAPE_CONVEX = 3,
  CP_SHAPE_CYLINDER = 4,
  CP_SHAPE_CAPSULE = 5,             /* Capsule, Cone and SizedPlane are ConvexPolyhedrons with */
  CP_SHAPE_CONE = 6,                /* their own ShapeType: their hulls are given as for CONVEX */
  CP_SHAPE_SIZED_PLANE = 7
};

/* BodyTypes / BodySleepStates, lib/objects/rigid_body.dart:15-16 */
enum cp_body_type { CP_BODY_DYNAMIC = 0, CP_BODY_STATIC = 1, CP_BODY_KINEMATIC = 2 };
enum cp_sleep_state { CP_AWAKE = 0, CP_SLEEPY = 1, CP_SLEEPING = 2 };

/* Broadphase plugins: NaiveBroadphase (lib/collision/naive_broadphase.dart),
 * SAPBroadphase (lib/collision/sap_broadphase.dart), GridBroadphase
 * (lib/collision/grid_broadphase.dart, with per-bin lists and a working pair
 * de-duplication; the reference version throws on its first step). */
enum cp_broadphase_kind { CP_BROAD_NAIVE = 0, CP_BROAD_SAP = 1, CP_BROAD_GRID = 2 };

/* Constraint classes, lib/constraints/*.dart */
enum cp_constraint_type {
  CP_CON_POINT_TO_POINT = 0,
  CP_CON_HINGE = 1,
  CP_CON_DISTANCE = 2,
  CP_CON_LOCK = 3,                  /* lock_constraint.dart */
  CP_CON_CONE_TWIST = 4,            /* cone_twist_constraint.dart */
  CP_CON_SPRING = 5                 /* spring_constraint.dart */
};

/* World.solver: GSSolver (lib/solver/gs_solver.dart) or SplitSolver over a
 * GSSolver with the same iterations and tolerance (lib/solver/split_solver.dart:
 * islands of non-static bodies, each solved on its own with its equations in
 * descending Equation.id order).  A SPLIT world keeps the reference's equation
 * ids: constraint equations take their constructor's ids
 * (cp_constraint_desc.first_equation_id ..), contact and friction equations
 * are drawn from the same last-in-first-out object pools the reference
 * recycles them through (world_class.dart:506-527, narrow_phase.dart:492-586). */
enum cp_solver_kind { CP_SOLVER_GS = 0, CP_SOLVER_SPLIT = 1 };

/* Equation classes appearing as solver rows, lib/equations/*.dart */
enum cp_row_kind { CP_ROW_CONTACT = 0, CP_ROW_FRICTION = 1, CP_ROW_ROTATIONAL = 2, CP_ROW_MOTOR = 3 };

/* Shape (lib/rigid_body_shapes/{sphere,plane,box,convex_polyhedron,cylinder,
 * capsule,cone,sized_plane}.dart).  A CONVEX, CAPSULE, CONE or SIZED_PLANE
 * shape lists its hull as the reference's constructor built it: `vertices`
 * (3 floats each), `face_sizes` (vertex count per face) and `face_indices`
 * (concatenated faces); `axes` (3 floats each) is the optional `uniqueAxes`
 * list (has_axes=0 means null).  A Lathe is a CONVEX shape. */
typedef struct cp_shape_desc {
  int32_t type;
  int32_t collision_filter_group;   /* Shape default -1 */
  int32_t collision_filter_mask;    /* Shape default -1 */
  int32_t collision_response;       /* default 1 */
  int32_t material;                 /* index into cp_world_desc.materials, -1 = null */
  int32_t num_segments;             /* cylinder */
  double radius;                    /* sphere */
  double radius_top, radius_bottom, height;  /* cylinder */
  float half_extents[3];            /* box */
  int32_t num_vertices, num_faces, num_axes, has_axes;  /* convex */
  const float* vertices;
  const int32_t* face_sizes;
  const int32_t* face_indices;
  const float* axes;
  double bounding_sphere_radius;    /* output of cp_shape_setup */
} cp_shape_desc;

/* A body's second, third, ... shape (Body.addShape(shape, offset,
 * orientation), lib/objects/rigid_body.dart:348-369): an entry of
 * cp_world_desc.body_shapes.  A body has at most CP_MAX_BODY_SHAPES shapes,
 * its first included. */
#define CP_MAX_BODY_SHAPES 65535
typedef struct cp_body_shape {
  int32_t shape;                    /* index into cp_world_desc.shapes */
  float offset[3];
  float orientation[4];
} cp_body_shape;

/* Body state (lib/objects/rigid_body.dart:27-260).  Its first shape is
 * `shape` at `shape_offset` / `shape_orientation` in the body frame; the
 * shapes added after it (a compound body) are body_shapes[
 * extra_shapes_first .. extra_shapes_first + extra_shapes_count) of the
 * world (or of the table given to cp_body_setup), in Body.shapes order. */
typedef struct cp_body_desc {
  float position[3];
  float quaternion[4];              /* x, y, z, w */
  float velocity[3];
  float angular_velocity[3];
  float force[3];
  float torque[3];
  float linear_factor[3];
  float angular_factor[3];
  float inv_inertia[3];
  float inv_inertia_world[9];
  float aabb_lower[3];
  float aabb_upper[3];
  float shape_offset[3];
  float shape_orientation[4];
  float previous_position[3];
  float previous_quaternion[4];
  double mass, inv_mass;
  double linear_damping, angular_damping;
  double sleep_speed_limit, sleep_time_limit, time_last_sleepy;
  double bounding_radius;
  int32_t type, sleep_state, allow_sleep, wake_up_after_narrowphase;
  int32_t collision_filter_group, collision_filter_mask, collision_response, is_trigger;
  int32_t material;                 /* -1 = null */
  int32_t shape;                    /* index into cp_world_desc.shapes */
  int32_t fixed_rotation, aabb_needs_update;
  /* Body.interpolatedPosition / interpolatedQuaternion (rigid_body.dart:135,190),
   * written by cp_world_step_interpolated */
  float interpolated_position[3];
  float interpolated_quaternion[4];
  int32_t extra_shapes_first, extra_shapes_count;
} cp_body_desc;

/* The Body fields one World.step changes or an app typically sets between
 * steps (applyForce, a new velocity, a teleport, a wake-up), moved without
 * the rest of the record: what a Dart GpuWorld exchanges every step. */
typedef struct cp_body_state {
  float position[3];
  float quaternion[4];
  float velocity[3];
  float angular_velocity[3];
  float force[3];
  float torque[3];
  float previous_position[3];
  float previous_quaternion[4];
  float interpolated_position[3];
  float interpolated_quaternion[4];
  int32_t sleep_state;
  int32_t wake_up_after_narrowphase;
  int32_t aabb_needs_update;
  int32_t pad0;
  double time_last_sleepy;
} cp_body_state;

/* Material (lib/material/material.dart): -1 means "not set". */
typedef struct cp_material {
  double friction, restitution;
} cp_material;

/* ContactMaterial (lib/material/contact_material.dart:63-101). */
typedef struct cp_contact_material {
  int32_t material_a, material_b;   /* ignored for the world default */
  double friction, restitution;
  double contact_stiffness, contact_relaxation;
  double friction_stiffness, friction_relaxation;
} cp_contact_material;

/* Constraint (lib/constraints/*.dart).  spook_* are the Equation SPOOK
 * parameters of the constraint rows; the reference constructor uses
 * (1e7, 4, 1/60) whatever the step size (lib/equations/equation_class.dart:38).
 * The local vectors are those the reference's constructor stored:
 *   POINT_TO_POINT  pivot_a, pivot_b; rows x, y, z
 *   HINGE           + axis_a, axis_b (normalised here); rows x, y, z, two
 *                   rotational, motor
 *   DISTANCE        distance (<0: the bodies' current distance); one row
 *   LOCK            pivot_a, pivot_b and lock_axes = xA, xB, yA, yB, zA, zB;
 *                   rows x, y, z, rotational (xA, yB), (yA, zB), (zA, xB)
 *   CONE_TWIST      pivot_a, pivot_b, axis_a, axis_b, angle, twist_angle;
 *                   rows x, y, z, cone, twist
 *   SPRING          distance = the rest length, max_force = the stiffness
 *                   (the row's force bound); one row
 */
typedef struct cp_constraint_desc {
  int32_t type, body_a, body_b, collide_connected;
  int32_t motor_enabled, pad0;
  float pivot_a[3], pivot_b[3];
  float axis_a[3], axis_b[3];
  double distance;                  /* DistanceConstraint; <0 = use the current distance */
  double max_force;
  double motor_target_velocity, motor_max_force;
  double spook_stiffness, spook_relaxation, spook_time_step;
  float lock_axes[6][3];            /* LockConstraint xA, xB, yA, yB, zA, zB */
  double angle, twist_angle;        /* ConeTwistConstraint */
  int64_t first_equation_id;        /* SPLIT: Equation.id of the first row; the others follow */
} cp_constraint_desc;

/* World (lib/world/world_class.dart:135-162) plus solver/broadphase settings. */
typedef struct cp_world_desc {
  int32_t num_bodies, num_shapes, num_materials, num_contact_materials, num_constraints;
  int32_t allow_sleep, quat_normalize_skip, quat_normalize_fast;
  int32_t solver_iterations;        /* Solver.iterations, default 10 */
  int32_t broadphase;               /* cp_broadphase_kind */
  int32_t use_bounding_boxes;       /* Broadphase.useBoundingBoxes */
  int32_t sap_axis;                 /* 0 = x, 1 = y, 2 = z */
  int32_t grid_n[3];
  int32_t enable_friction_reduction;
  int32_t has_friction_gravity;
  int32_t stepnumber;
  double solver_tolerance;          /* default 1e-7 */
  double time;
  float gravity[3];
  float friction_gravity[3];
  float grid_aabb_min[3], grid_aabb_max[3];
  const cp_body_desc* bodies;
  const cp_shape_desc* shapes;
  const cp_material* materials;
  const cp_contact_material* contact_materials;
  const cp_constraint_desc* constraints;
  const int32_t* sap_axis_list;     /* optional persisted SAP order, NULL = body order */
  cp_contact_material default_contact_material;
  const cp_body_shape* body_shapes; /* shapes after each body's first (compound bodies) */
  int32_t num_body_shapes;
  int32_t solver;                   /* cp_solver_kind */
  /* SPLIT: Equation.idCounter when the world is handed over (the ids of the
   * contact and friction equations created from then on follow it; the
   * equation pools start empty) */
  int64_t equation_id_counter;
} cp_world_desc;

/* One narrowphase contact, in the order the reference appends them. */
typedef struct cp_contact {
  int32_t bi, bj;                   /* ContactEquation.bi / .bj body indices */
  int32_t si, sj;                   /* ContactEquation.si / .sj shape indices */
  float ni[3], ri[3], rj[3];
  int32_t enabled, pair;            /* pair = index in the broadphase pair list */
  double restitution;
} cp_contact;

/* One solver row, in World.internalStep's equation order (friction,
 * contact, constraint rows). */
typedef struct cp_row {
  int32_t kind, bi, bj, pad;
  double B, inv_c, lambda, multiplier, min_force, max_force, eps;
  int64_t id;                       /* Equation.id under the SPLIT solver, else -1 */
} cp_row;

typedef struct cp_step_info {
  int64_t stepnumber;
  double time;
  int32_t num_pairs, num_contacts, num_rows, iterations;
  int32_t status, num_bodies;
  int32_t num_levels;               /* dependency levels of the last solve (rows of a level share no dynamic body) */
  int32_t substeps;                 /* internal steps taken by the last cp_world_step_interpolated */
  double accumulator;               /* World.accumulator (world_class.dart:119) */
} cp_step_info;

typedef struct cp_config {
  int32_t device;                   /* CUDA device ordinal */
  int32_t block_threads;            /* 0 = autotuned */
  int64_t arena_bytes;              /* 0 = grow on demand */
} cp_config;

typedef struct cp_ctx cp_ctx;

/* ---- host-side setup (Body / Shape constructors) ------------------------ */

/* Shape constructor work: Sphere/Box/Cylinder/ConvexPolyhedron init and
 * updateBoundingSphereRadius (sphere.dart:119-144, box.dart:21-126,
 * cylinder.dart:222-294, convex_polyhedron.dart:80-185,648-660).  Fills
 * shape->bounding_sphere_radius. */
int cp_shape_setup(cp_shape_desc* shape);

/* Body(mass, position, quaternion) followed by addShape(shape, offset,
 * orientation) for each of its shapes, for each of `num_bodies` bodies:
 * updateMassProperties (rigid_body.dart:587-609, inertia from the AABB of
 * all the body's shapes) and updateBoundingRadius (:395-412).  Reads mass,
 * position, quaternion, shape, shape_offset, shape_orientation, the extra
 * shapes (body_shapes, may be NULL when no body has any), fixed_rotation and
 * type (-1 = derive from mass); writes inv_mass, type, inertia-derived
 * fields, aabb, bounding_radius, previous_* and aabb_needs_update.  Other
 * fields are left as given (callers start from the Body constructor
 * defaults). */
int cp_body_setup(const cp_shape_desc* shapes, int32_t num_shapes, const cp_body_shape* body_shapes, int32_t num_body_shapes,
                  cp_body_desc* bodies, int32_t num_bodies);

/* ---- context and worlds ------------------------------------------------- */

int cp_create(const cp_config* cfg, cp_ctx** out);
int cp_destroy(cp_ctx* ctx);

/* Pack a World (bodies, shapes, materials, constraints, settings) into
 * device memory.  Replaces World.addBody/addConstraint/addContactMaterial as
 * the way state reaches the step (world_class.dart:224,282-299,343-348). */
int cp_world_create(cp_ctx* ctx, const cp_world_desc* desc, int32_t* world_id);
int cp_world_destroy(cp_ctx* ctx, int32_t world_id);

/* World.step(dt) in fixed mode, nsteps times: internalStep then time += dt
 * (world_class.dart:392-399,433-701).  The world keeps its own copy of
 * World.time and World.stepnumber (set at cp_world_create and by
 * cp_world_set_time); sleepTick reads that time, as the reference does. */
int cp_world_step(cp_ctx* ctx, int32_t world_id, double dt, int32_t nsteps);

/* World.internalStep(dt), nsteps times (world_class.dart:433-701): stepnumber
 * advances by one per step, time does not; sleepTick reads the world's
 * current time.  This is the call for a binding that overrides
 * World.internalStep and lets World.step keep the clock: push World.time with
 * cp_world_set_time before it, and World.step adds dt (fixed mode) or
 * timeSinceLastCalled (interpolating mode) itself afterwards. */
int cp_world_internal_step(cp_ctx* ctx, int32_t world_id, double dt, int32_t nsteps);

/* World.step(dt, timeSinceLastCalled, maxSubSteps), the interpolating form
 * (world_class.dart:400-430): the accumulator gains timeSinceLastCalled;
 * internal steps run while it holds a whole dt (at most max_sub_steps, and
 * none after the steps so far took longer than dt of wall-clock time, as the
 * reference bails out); the remainder is kept modulo dt; every body's
 * interpolated position (previousPosition.lerp) and quaternion
 * (previousQuaternion.slerp, Quaternion.slerp quaternion.dart:118-168) are
 * written for t = accumulator / dt and previousQuaternion is normalised;
 * then time += timeSinceLastCalled.  *substeps (may be NULL) receives the
 * number of internal steps taken.  The slerp's acos and sin are the device's
 * (within 2 ulp of the C library's), so interpolated quaternions can differ
 * from a host computation in the last binary32 bit; every other field is
 * exact. */
int cp_world_step_interpolated(cp_ctx* ctx, int32_t world_id, double dt, double time_since_last_called,
                               int32_t max_sub_steps, int32_t* substeps);

/* Overwrite World.time, World.stepnumber and World.accumulator
 * (world_class.dart:74-80,119) of a device world, e.g. from the host
 * World object before cp_world_internal_step. */
int cp_world_set_time(cp_ctx* ctx, int32_t world_id, double time, int64_t stepnumber, double accumulator);

/* cp_world_step without any allocation.  It has no counterpart in the
 * reference (Dart allocates as it pleases).
 *
 * Who needs it: callers that must not allocate device memory while they
 * step.  One example is a frame loop with a hard deadline, where
 * cudaMalloc / cudaFree can synchronise the whole device.  Another is a
 * server whose device memory was fixed when a request was admitted.
 * cp_world_step may allocate: when a step overflows the world's pair,
 * contact or row capacity, it regrows the world's scratch and re-runs the
 * step.
 *
 * What it does: it gives the same results as cp_world_step, bit for bit.
 * The per-step lists (pairs, contacts, rows, levels, solver scratch) live
 * in one file-scope device array of CP_STATIC_SCRATCH_BYTES (64 MiB), not
 * in the world's own scratch.  At the end of the call the last step's
 * pairs, contacts and rows are copied (device to device, on the context's
 * stream) into the world's own lists, so cp_world_get_pairs / get_contacts
 * / get_rows / get_info report them as they do after cp_world_step.
 *
 * Limits:
 *  - A world whose lists, at its current capacities, need more than that
 *    array is rejected with CP_ERR_CAPACITY before anything runs.  This is
 *    roughly 11 KB per body: a 4096-body world fits, 10,000 bodies do not.
 *  - A step that overflows a capacity is not regrown.  The world's bodies
 *    are left as they were at the start of that step (only their cached
 *    AABBs may be refreshed), its status is cleared, its pair, contact and
 *    row lists read back empty, and the call returns CP_ERR_CAPACITY.
 *    cp_world_step can then take that step and grow the capacities.
 *
 * Set-up: the first call on a device takes the array's address with
 * cudaGetSymbolAddress, with that device current.  Make that first call
 * before any stream capture.
 *
 * Start state: nothing in the array needs to start at zero.  Every step
 * writes each list before reading it.  The work-queue counters the kernels
 * take work from are cleared before every step.
 *
 * Concurrency: every context on a device shares the one array.  Calls whose
 * GPU work overlaps race on it; for example, calls on two contexts of one
 * device, which run on different streams.  Calls on one context never
 * overlap: they are serialised on its stream. */
#define CP_STATIC_SCRATCH_BYTES (64u * 1024u * 1024u)
int cp_world_step_static(cp_ctx* ctx, int32_t world_id, double dt, int32_t nsteps);

/* ---- event feed (World events, lib/world/world_class.dart:593-610,703-770) --
 *
 * The reference dispatches, inside World.internalStep, a `collide` event to
 * both bodies of every contact (its collision matrices alias, so every
 * contact counts as a first contact), and then beginContact / endContact /
 * beginShapeContact / endShapeContact for the body and shape pairs whose
 * overlap started or ended since the previous step (OverlapKeeper,
 * lib/collision/overlap_keeper.dart; kinematic / static pairs whose shapes
 * overlap count too, through getContacts' justTest call).  With the feed on,
 * every step of the world records those events in that order; the O(N^3)
 * collision matrix and the O(K^2) insertion sorts are replaced by sorted
 * key sets built from the step's contact and pair lists on the host. */
enum cp_event_type {
  CP_EV_COLLIDE = 0,             /* a = contact.bi, b = contact.bj, contact = its index in the step's contacts */
  CP_EV_BEGIN_CONTACT = 1,       /* a, b: bodies (the lower id first, as OverlapKeeper unpacks its keys) */
  CP_EV_END_CONTACT = 2,
  CP_EV_BEGIN_SHAPE_CONTACT = 3, /* a, b: shapes (lower id first) */
  CP_EV_END_SHAPE_CONTACT = 4
};
typedef struct cp_event {
  int32_t type, a, b, contact;
  int64_t stepnumber;               /* World.stepnumber after the step that raised it */
} cp_event;

/* Turn a world's event feed on or off (off by default: it costs a
 * device-to-host copy of the step's lists and a synchronisation per step).
 * body_ids / shape_ids (may be NULL: the indices) give the Body.id and
 * Shape.id values the overlap keys sort by, so events of one step come in
 * the reference's order; ids must be below 65536 (the reference packs two
 * into one key).  Turning the feed on starts with empty overlap sets. */
int cp_world_set_events(cp_ctx* ctx, int32_t world_id, int32_t on, const int32_t* body_ids, const int32_t* shape_ids);
/* Drains the world's recorded events (oldest first).  CP_ERR_CAPACITY with
 * *count set when more than cap are waiting (nothing is drained then). */
int cp_world_get_events(cp_ctx* ctx, int32_t world_id, cp_event* out, int32_t cap, int32_t* count);

/* ---- raycasts over the resident state -------------------------------------
 * World.raycastClosest / raycastAny / raycastAll (lib/world/world_class.dart:
 * 248-278) through Ray.intersectWorld (lib/collision/ray_class.dart:163-199),
 * one ray per record, all against the world as it stands.  Like the
 * reference, a raycast refreshes the AABBs of the bodies that need it (and
 * re-sorts a SAPBroadphase's axis list), and a GridBroadphase world answers
 * no hits (GridBroadphase has no aabbQuery).  Capsule, Cone and SizedPlane
 * shapes have no ray intersector in the reference and are never hit. */
typedef struct cp_ray {
  float from[3], to[3];
  int32_t collision_filter_group;   /* RayOptions: default -1 */
  int32_t collision_filter_mask;    /* default -1 */
  int32_t skip_backfaces;           /* intersectWorld default 1 */
  int32_t check_collision_response; /* default 1 */
} cp_ray;

enum cp_ray_mode { CP_RAY_CLOSEST = 0, CP_RAY_ANY = 1, CP_RAY_ALL = 2 };

/* RaycastResult (lib/collision/raycast_result.dart); after reset() a miss
 * reads has_hit 0, body / shape -1, hit_face_index -1, distance -1.  As in
 * the reference, hit_face_index of a CLOSEST result is that of the last hit
 * reported, kept or not. */
typedef struct cp_ray_hit {
  int32_t has_hit, body, shape, hit_face_index;
  float hit_point[3];
  float hit_normal[3];
  double distance;
} cp_ray_hit;

/* Casts n rays.  CLOSEST / ANY: hits[r] is ray r's result (max_hits and counts
 * are not used).  ALL: the hits of ray r in report order go to
 * hits[r * max_hits ..] (at most max_hits of them) and counts[r] is their
 * number (it may exceed max_hits: the rest are dropped). */
int cp_world_raycast(cp_ctx* ctx, int32_t world_id, const cp_ray* rays, int32_t n, int32_t mode, cp_ray_hit* hits,
                     int32_t max_hits, int32_t* counts);

/* Read back / overwrite body state (Body fields). */
int cp_world_get_bodies(cp_ctx* ctx, int32_t world_id, cp_body_desc* out, int32_t n);
int cp_world_set_bodies(cp_ctx* ctx, int32_t world_id, const cp_body_desc* in, int32_t n);

/* Read back / overwrite only the per-step fields of cp_body_state (about a
 * third of a cp_body_desc).  set_states writes every field of the record
 * (aabb_needs_update and wake_up_after_narrowphase set or clear the body's
 * flags); other Body fields keep their device values. */
int cp_world_get_states(cp_ctx* ctx, int32_t world_id, cp_body_state* out, int32_t n);
int cp_world_set_states(cp_ctx* ctx, int32_t world_id, const cp_body_state* in, int32_t n);

/* Last step's broadphase pairs (worldStepP1/P2, world_class.dart:481-499),
 * contacts (World.contacts) and solver rows (Solver.equations with B, 1/C,
 * lambda and multiplier, gs_solver.dart:105-176). */
int cp_world_get_pairs(cp_ctx* ctx, int32_t world_id, int32_t* p1, int32_t* p2, int32_t cap, int32_t* count);
int cp_world_get_contacts(cp_ctx* ctx, int32_t world_id, cp_contact* out, int32_t cap, int32_t* count);
int cp_world_get_rows(cp_ctx* ctx, int32_t world_id, cp_row* out, int32_t cap, int32_t* count);
int cp_world_get_info(cp_ctx* ctx, int32_t world_id, cp_step_info* out);

/* SAP axisList order (sap_broadphase.dart:11), kept across steps. */
int cp_world_get_sap_order(cp_ctx* ctx, int32_t world_id, int32_t* out, int32_t n);

/* ---- batched form ------------------------------------------------------- */

/* Step many independent worlds together: one persistent fused launch per
 * step, the nsteps sequence captured in a CUDA graph and replayed.  Each
 * world's result equals cp_world_step on that world alone. */
int cp_batch_step(cp_ctx* ctx, const int32_t* world_ids, int32_t n, double dt, int32_t nsteps);

/* Per-step host I/O of a batch, the way a game or RL loop drives it.
 * The bodies of the listed worlds are concatenated in list order
 * (`total_bodies` = the sum of their body counts).
 * set_forces overwrites Body.force / Body.torque (6 floats per body: force
 * xyz, torque xyz), i.e. what applyForce / applyTorque accumulated on the host
 * before World.step (rigid_body.dart:472-525);
 * get_poses reads position xyz, quaternion xyzw, velocity xyz and angular
 * velocity xyz (13 floats per body), what a Dart GpuWorld writes back into
 * its Body objects after each step.  Host buffers may be pinned or pageable;
 * each call is one host-device copy plus one scatter / gather launch. */
int cp_batch_set_forces(cp_ctx* ctx, const int32_t* world_ids, int32_t n, const float* ft, int64_t total_bodies);
int cp_batch_get_poses(cp_ctx* ctx, const int32_t* world_ids, int32_t n, float* out, int64_t total_bodies);

/* Number of this library's GPU kernel launches issued by this context so far
 * (two per batched or single-world step, plus the status and I/O kernels;
 * memory copies and sets are not counted). */
int64_t cp_kernel_launches(cp_ctx* ctx);

/* The CUDA stream (cudaStream_t) all work of the context runs on, so callers
 * can order their own work or time with events on it. */
int cp_get_stream(cp_ctx* ctx, void** stream);

/* The batch autotuner's choice: every kernel variant (threads per block and
 * register budget) gives identical results, so the first cp_batch_step calls
 * on a world set each time one variant on the live steps and later calls use
 * the fastest.  Writes the chosen variant (-1 while tuning), its block size
 * and up to n per-variant ms/step; returns the number of variants. */
int cp_autotune_info(cp_ctx* ctx, int32_t* variant, int32_t* threads, double* ms, int32_t n);

/* Pin the batched kernel variant (0 .. number of variants - 1), or -1 to
 * return to autotuning. */
int cp_set_variant(cp_ctx* ctx, int32_t variant);

/* The World.profile breakdown (world_class.dart:27-41) of every step since
 * the previous call, as SM cycles summed over thread blocks, in 8 slots:
 * prepare, broadphase, narrowphase, contact rows + wake-ups + solve set-up,
 * row assembly (computeB / computeC), solver levels, Gauss-Seidel sweeps,
 * velocity update + integrate + sleep.  Shares, not wall time.  With n >= 40
 * it also writes 16 narrowphase-resolver thread-cycle sums and 16 call
 * counts (resolver kinds: 1 sphere-sphere, 2 sphere-plane, 3 sphere-box,
 * 4 sphere-convex, 5 plane-box, 6 plane-convex, 7 box-box, 8 box-convex,
 * 9 convex-convex; 10-12 pairs settled by a binary32 no-contact test);
 * those are counted only while cp_set_resolver_profile is on. */
int cp_phase_profile(cp_ctx* ctx, double* cycles, int32_t n);

/* Turn the per-resolver cycle and call counts on (1) or off (0, the
 * default).  The switch is per device, not per context: it applies to every
 * step launched on the context's device afterwards.  Counting costs a few per
 * cent of a step.  No counterpart in the reference (its World.profile has no
 * per-resolver breakdown). */
int cp_set_resolver_profile(cp_ctx* ctx, int32_t on);

/* Batched path: worlds are handed to thread blocks in groups of consecutive
 * (similar-size) worlds holding up to `bodies` bodies (at most 8 worlds);
 * the solver sweeps of a group share barriers.  0 = one world per group. */
int cp_set_group_bodies(cp_ctx* ctx, int32_t bodies);

/* cp_world_step, cp_world_internal_step and cp_world_step_interpolated on a
 * world of at least `bodies` bodies spread the world over the whole GPU: each
 * phase runs as a grid-wide kernel over its bodies, pairs, contacts or rows,
 * and only the dependency levels and the Gauss-Seidel sweeps stay on one
 * block.  The results are the same bits as on one block.  Default 1024;
 * 0 keeps every world on one block.  No counterpart in the reference. */
int cp_set_wide_bodies(cp_ctx* ctx, int32_t bodies);

/* The Gauss-Seidel sweeps of a world stepped over the whole GPU run either
 * level by level or on a slot schedule across sweeps (the same bits either
 * way).  0 (default): the schedule where it pays (the last solve ran every
 * sweep, the schedule saves two thirds of the level steps, its tables fit);
 * 1: the schedule wherever its tables fit; -1: always level by level.  A
 * test switch; no counterpart in the reference. */
int cp_set_sweep_schedule(cp_ctx* ctx, int32_t mode);

/* Filter check, a test switch with no counterpart in the reference (off by
 * default; per device).  Where a binary32 filter settles a pair without the
 * reference's binary64 arithmetic (the no-contact certificates of
 * sphere-plane, sphere-box and plane-hull pairs; the separating-axis bound
 * and the candidate axes of hull pairs), the step also runs the unfiltered
 * binary64 computation and compares: the resolver's contact count for a
 * certificate, and the separation verdict and the chosen axis (bit for bit)
 * for findSeparatingAxis.  Steps run several times slower while it is on.
 * cp_filter_check_counts reads the pairs checked and the disagreements since
 * the last reset. */
int cp_set_filter_check(cp_ctx* ctx, int32_t on);
int cp_filter_check_counts(cp_ctx* ctx, int64_t* checked, int64_t* disagreed, int32_t reset);

/* Device time (CUDA events on the context stream) of the batched-step graph
 * launches since the previous call, and how many step launches they held. */
int cp_batch_profile(cp_ctx* ctx, double* graph_ms, int64_t* step_launches);

/* ---- served form ---------------------------------------------------------
 *
 * No counterpart in the reference.  A request server on one device: a
 * request is one world plus a horizon (nsteps steps at dt).  The server keeps
 * admitted worlds resident in HBM and admits queued requests (first come,
 * first served) while their state and step scratch fit `hbm_budget_bytes`.
 * Every admitted world advances up to `steps_per_tick` steps per launch
 * sequence, together with all other admitted worlds, so requests that arrive
 * while others run share the device with them (continuous batching).  A
 * world stops at its own horizon.  Its result is the same, bit for bit, as
 * stepping it alone with cp_world_step.
 *
 * The server owns its own context and thread; submit, poll, wait, result,
 * cancel and stats may be called from any thread. */
typedef struct cp_server cp_server;

typedef struct cp_serve_config {
  int32_t device;
  int32_t steps_per_tick;           /* 0 = 2 */
  int64_t hbm_budget_bytes;         /* device memory admitted worlds may hold at once */
  int64_t max_active_bodies;        /* 0 = no cap; else admission also stops at this many bodies stepping */
  int32_t variant;                  /* kernel variant pair, -1 = default */
  int32_t group_bodies;             /* world grouping of the solve kernel, 0 = default */
  /* a world whose pair, contact or row list would have to grow beyond this
   * many entries (its step scratch beyond what admission counted on) fails
   * alone with CP_ERR_CAPACITY; the other requests of its ticks go on.
   * 0 = no limit */
  int64_t max_list_entries;
  /* wide_lanes > 0: worlds of at least wide_bodies bodies (0 = 1024) are
   * not batched into the ticks; each of wide_lanes lanes steps one at a time
   * to its horizon, spread over the whole GPU (cp_set_wide_bodies), on a
   * stream of its own, concurrently with the ticks.  This lowers a large
   * world's latency on an idle server but costs throughput under load: a
   * lane steps one world at a time.  0 or -1 = no lanes (every world joins
   * the ticks) */
  int32_t wide_bodies;
  int32_t wide_lanes;
} cp_serve_config;

/* request states */
#define CP_REQ_PENDING   0
#define CP_REQ_ACTIVE    1
#define CP_REQ_DONE      2
#define CP_REQ_FAILED    3
#define CP_REQ_CANCELLED 4

typedef struct cp_serve_stats {
  int64_t submitted, admitted, completed, failed, cancelled;
  int64_t pending, active, ticks;
  int64_t bytes_in_use, bytes_peak, bytes_budget;
  int64_t body_steps;               /* bodies x steps of the completed requests */
  double span_s;                    /* first submission to last completion */
  double device_s;                  /* time inside step launch sequences */
  double p50_ms, p99_ms, mean_ms, max_ms;  /* latency: submission to result ready */
} cp_serve_stats;

int cp_serve_start(const cp_serve_config* cfg, cp_server** out);
int cp_serve_stop(cp_server* server);
/* Copies the world during the call.  CP_ERR_CAPACITY if the world alone needs
 * more than the whole budget. */
int cp_serve_submit(cp_server* server, const cp_world_desc* desc, double dt, int32_t nsteps, int64_t* ticket);
int cp_serve_poll(cp_server* server, int64_t ticket, int32_t* state);
/* Blocks until the request finished (done, failed or cancelled);
 * timeout_s < 0 waits without limit, else CP_ERR_TIMEOUT when it runs out. */
int cp_serve_wait(cp_server* server, int64_t ticket, double timeout_s, int32_t* state);
/* Copies a finished request's bodies and final step info and releases it. */
int cp_serve_result(cp_server* server, int64_t ticket, cp_body_desc* out, int32_t n, cp_step_info* info);
/* A queued request is dropped; an admitted one is retired at the end of the
 * current tick without a result. */
int cp_serve_cancel(cp_server* server, int64_t ticket);
/* Counters and latency percentiles since the previous reset. */
int cp_serve_get_stats(cp_server* server, cp_serve_stats* out, int32_t reset);

const char* cp_last_error(void);
int cp_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif /* CANNON_GPU_H */
