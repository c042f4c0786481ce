/*
 * cannon_oracle.h -- C API of the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  The oracle is a sequential C++ restatement of
 * cannon_physics' World.step (Dart, lib/world/world_class.dart:433-701 and
 * everything it calls).  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline legs load it, to compare the GPU path's results with and to
 * time the CPU baseline.  Nothing in the cannon_physics_gb300 package links or
 * calls it.
 *
 * Arithmetic contract ("mode R"): every scalar is an IEEE binary64 value and
 * every Vector3 / Quaternion / Matrix3 component is rounded to binary32 at the
 * point where the reference stores it (package:vector_math keeps those
 * components in Float32List).  Build with -ffp-contract=off.
 *
 * Parity status: the reference ships no tests, golden vectors or fixtures and
 * cannot run in this environment (Dart/Flutter SDK absent), so the oracle is
 * pinned only by analytic known-answer tests (free fall, resting contact,
 * symmetric stacks) -- "parity unpinned" against the reference itself.
 */
#ifndef CANNON_ORACLE_H
#define CANNON_ORACLE_H

#include "cannon_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_world orc_world;

int orc_shape_setup(cp_shape_desc* shape);
int orc_body_setup(const cp_shape_desc* shapes, int32_t num_shapes, const cp_body_shape* body_shapes, int32_t num_body_shapes,
                   cp_body_desc* bodies, int32_t num_bodies);

orc_world* orc_world_create(const cp_world_desc* desc);
void orc_world_destroy(orc_world* w);
int orc_world_step(orc_world* w, double dt, int32_t nsteps);
int orc_world_internal_step(orc_world* w, double dt, int32_t nsteps);
int orc_world_step_interpolated(orc_world* w, double dt, double time_since_last_called, int32_t max_sub_steps, int32_t* substeps);
int orc_world_set_time(orc_world* w, double time, int64_t stepnumber, double accumulator);
/* Overwrite the bodies / the persisted SAP order (e.g. with a GPU world's
 * state, to time or check the oracle from the same step). */
int orc_world_set_bodies(orc_world* w, const cp_body_desc* in, int32_t n);
/* Record World's events (collide, begin / end contact, begin / end shape
 * contact) in dispatch order, restating the reference's collision matrix
 * and OverlapKeeper; ids as in cp_world_set_events. */
int orc_world_set_events(orc_world* w, int32_t on, const int32_t* body_ids, const int32_t* shape_ids);
int orc_world_get_events(orc_world* w, cp_event* out, int32_t cap, int32_t* count);
int orc_world_set_sap_order(orc_world* w, const int32_t* in, int32_t n);
int orc_world_get_bodies(orc_world* w, cp_body_desc* out, int32_t n);
int orc_world_get_pairs(orc_world* w, int32_t* p1, int32_t* p2, int32_t cap, int32_t* count);
int orc_world_get_contacts(orc_world* w, cp_contact* out, int32_t cap, int32_t* count);
int orc_world_get_rows(orc_world* w, cp_row* out, int32_t cap, int32_t* count);
int orc_world_get_info(orc_world* w, cp_step_info* out);
int orc_world_get_sap_order(orc_world* w, int32_t* out, int32_t n);
int orc_world_raycast(orc_world* w, const cp_ray* rays, int32_t n, int32_t mode, cp_ray_hit* hits, int32_t max_hits,
                      int32_t* counts);

/* Step many independent worlds on `threads` host threads (one world per
 * thread at a time); used for the CPU baseline of the batched form. */
int orc_worlds_step_parallel(orc_world** worlds, int32_t n, double dt, int32_t nsteps, int32_t threads);

/* Convex hull tables the oracle derives for a shape (vertices, face normals,
 * unique edges), for host-side parity tests of hull construction. */
int orc_shape_hull(const cp_shape_desc* shape, float* verts, int32_t vcap, int32_t* nv,
                   float* normals, int32_t ncap, int32_t* nf, float* edges, int32_t ecap, int32_t* ne);

#ifdef __cplusplus
}
#endif
#endif
