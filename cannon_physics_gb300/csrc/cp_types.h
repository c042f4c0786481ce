// cp_types.h -- device-resident world layout shared by the host runtime
// (cp_host.cpp) and the step kernels (cp_step.cu).
//
// One World is a set of arrays in device memory.  Bodies are 432-byte
// records: every phase of a step touches a handful of fields of a body, and
// pairs and solver rows gather bodies by index, so a record per body keeps
// those gathers to a few cache lines.  Scratch (pairs, contacts, rows,
// solver levels) belongs to the world and keeps the last step's lists for
// cp_world_get_pairs / get_contacts / get_rows.
#pragma once
#include <cstdint>

#include <vector_types.h>

#include "../../include/cannon_gpu.h"

#define CP_MAX_HULL_VERTS 32
#define CP_MAX_FACE_VERTS 16
#define CP_MAX_CLIP 48
#define CP_MAX_PAIR_CONTACTS 32
#define CP_NUM_PHASES 8
#define CP_PROFILE_SLOTS (CP_NUM_PHASES + 32)

// body flags
#define BF_ALLOW_SLEEP 1
#define BF_WAKE 2
#define BF_RESPONSE 4
#define BF_TRIGGER 8
#define BF_FIXED_ROT 16
#define BF_AABB_DIRTY 32

// step status bits (DWorldParams.status)
#define ST_PAIRS_OVERFLOW 1
#define ST_CONTACTS_OVERFLOW 2
#define ST_ROWS_OVERFLOW 4
#define ST_LEVELS_OVERFLOW 8
#define ST_HULL_OVERFLOW 16
#define ST_BINS_OVERFLOW 32
#define ST_NONFINITE 64
#define ST_TIMEOUT 128
#define ST_JOBS_OVERFLOW 256  // shape-pair jobs of compound bodies

struct __align__(16) DBody {
  float pos[4];     // Body.position
  float quat[4];    // Body.quaternion (x, y, z, w)
  float vel[4];     // Body.velocity
  float avel[4];    // Body.angularVelocity
  float force[4];   // Body.force
  float torque[4];  // Body.torque
  float iw[12];     // Body.invInertiaWorld, e[3*row+col]
  float inv_inertia[4];
  float lin_factor[4];
  float ang_factor[4];
  float aabb_lo[4];
  float aabb_hi[4];
  float shape_off[4];
  float shape_quat[4];
  float prev_pos[4];
  float prev_quat[4];
  double mass, inv_mass, lin_damp, ang_damp;
  double sleep_speed_limit, sleep_time_limit, time_last_sleepy, bounding_radius;
  int type, sleep_state, flags, group;
  int mask, material, shape, pad0;
  float brad32;  // bounding_radius rounded to float (broadphase filter only)
  int xs0, nxs;   // a compound body's further shapes: bshapes[xs0 .. xs0 + nxs)
  int pad1;
  float interp_pos[4];   // Body.interpolatedPosition
  float interp_quat[4];  // Body.interpolatedQuaternion
};

struct __align__(16) DShape {
  int type, group, mask, response;
  int material, hull, plane_done, pad1;
  double radius, bsr;
  float he[4];
  float plane_n[4];  // Plane.worldNormal, computed once by the grid broadphase (plane.dart:182-187)
};

// Convex hull tables (ConvexPolyhedron: vertices, faces, faceNormals,
// uniqueEdges), plus the per-face data the clipping code derives every time
// in the reference: the connected faces of each face and -n.v0.
struct __align__(16) DHull {
  int v0, nv, f0, nf;        // vertices [v0, v0+nv), faces [f0, f0+nf)
  int e0, ne, has_axes, is_box;  // unique edges [e0, e0+ne); is_box: vertices are (+-he)
  int cf0, ncf, ce0, nce;    // canonical faces / edges: hcanon[cf0 ..), hcanon[ce0 ..)
  double he[4];              // box half extents (binary32 values)
};
struct __align__(16) DFace {
  int i0, n;     // vertex indices hfi[i0 .. i0+n)
  int c0, nc;    // connected faces hconn[c0 .. c0+nc)
  float normal[4];
  double dnormal[4];   // the same normal in binary64
  double plane_const;
  int canon, pad[3];   // the face whose normal is this one's exact negation (earlier), or itself
};

struct DMaterial { double friction, restitution; };

struct DContactMaterial {
  double friction, restitution, cs, cr, fs, fr;
  double ca, cb, ceps, fa, fb, feps;  // SPOOK a, b, eps for contact / friction rows at the current dt
};

struct __align__(16) DConstraint {
  int type, a, b, collide;
  int row0, nrows, motor, pad;
  float piv_a[4], piv_b[4], axis_a[4], axis_b[4];
  float loc[6][4];  // LockConstraint local axes xA, xB, yA, yB, zA, zB
  double distance, max_force, motor_target, motor_max_force;
  double sa, sb, seps;  // SPOOK params of the constraint rows
  // cos(maxAngle) of the rotational rows, from libm: rows 0-2 take cos_rot[0]
  // (a cone-twist's twist row takes cos_rot[1])
  double cos_rot[2];
  double pad2;
  // per-step geometry
  float ri[4], rj[4], n[4];
  float rot_a[3][4], rot_b[3][4];  // world axes (axisA, axisB) of the rotational rows
  float ma[4], mb[4];              // motor axes
  long long first_id;              // SplitSolver: Equation.id of row 0 (the others follow)
  long long pad3;
};

struct __align__(16) DContact {
  int bi, bj, si, sj;
  float ni[4], ri[4], rj[4];
  int enabled, pair, cm, frow;  // frow: index of the first friction candidate, -1 if none
  double restitution;
  double slip;  // mug * reducedMass
};

// A solver row.  The Jacobian entries are binary32 values (JacobianElement
// stores Vector3s).
struct __align__(16) DRow {
  float gaS[4], gaR[4], gbS[4], gbR[4];
  float iMaR[4], iMbR[4];  // invInertiaWorldSolve * rotational Jacobians (the addToWlambda temp)
  double B, invC, eps, minF, maxF, lambda;
  double imA, imB;          // invMassSolve of bi, bj
  double mult;              // Equation.multiplier = lambda / h
  int bi, bj, kind, src;
};

struct __align__(16) DBodyScr {
  float xs[4];   // shape world position
  float qs[4];   // shape world orientation
  float vl[4];   // vlambda (x, y, z; w unused)
  float wl[4];   // wlambda
  float imf[4];  // force * invMassSolve (computeGiMf)
  float iit[4];  // invInertiaWorldSolve * torque
  double im_solve;
  int active, last_level;
};

struct __align__(16) DWorldParams {
  double time, tolerance, dt_cached;
  long long stepnumber;
  float gravity[4], fgrav[4];
  float grid_min[4], grid_max[4];
  int nb, nshapes, nmat, ncm;
  int ncons, ncon_rows, iterations, broadphase;
  int sap_axis, use_bb, allow_sleep, qn_skip;
  int qn_fast, has_fgrav, grid_nx, grid_ny;
  int grid_nz, nbins, status, last_iterations;
  int num_pairs, num_contacts, num_rows, num_levels;
  int pairs_cap, contacts_cap, rows_cap, bins_cap;
  int grid_plane_done, n_nocollide, fric_reduction, events;
  float grid_plane_n[4];
  long long step_limit;  // the step kernels leave the world alone once stepnumber reaches this
  int compound, jobs_cap;  // some body has several shapes; capacity of the shape-pair job list
  int num_jobs, pad3;  // narrowphase jobs of the last step (shape pairs; the pairs without compound bodies)
  // SplitSolver: on; sizes of the contact / friction equation pools (stacks
  // of ids); set by the pre-step kernel when it ran the whole step itself
  int split, pool_c, pool_f, presolved;
  long long id_counter;  // Equation.idCounter
  long long pad5;
};

// A compound body's second, third, ... shape (Body.shapes[1..] with its
// offset and orientation)
struct __align__(16) DBodyShape {
  int shape, pad[3];
  float off[4];
  float quat[4];
};

// Counters of a step of one world spread over the whole GPU (the wide
// kernels, cp_wide.cu): what the one-block kernels keep in shared memory.
struct __align__(16) DWide {
  int run;        // the step runs: status clear and below the step limit
  int overflow;   // ST_* bits found during this step
  int n_pairs, n_cand_pairs, n_contacts, n_fric;
  int n_cand, n_rows, n_levels, iters;
  int n_queued, n_queued2, nh_padded, cursor;
  int check[4];   // first failed index check of the sweep kernel: code, index, bound
  int kcnt[16], kpos[16];
  int total, n_jobs;  // n_jobs: narrowphase jobs of a compound world
  int sched;          // this step's sweeps run on the slot schedule (k_w_sched)
  int n_slots;        // its slots
  int early;          // the last solve stopped before its last sweep (0 at the first step)
  int slow;           // steps left on the level-by-level sweeps after a schedule that saved too little
  int pad[2];
};

// Buffers of the slot-scheduled sweeps of a wide world (its own allocation,
// sized for `rows` rows, `iters` sweeps and `nb` bodies; null when absent).
// Instance i = s * n_rows + p is sweep s of the row at level position p.
struct DSched {
  double* lam;        // [iters * rows] lambda after each instance
  double* absdl;      // [iters * rows] |dlambda| by sweep and row-list index (the exit tests sum them)
  int* slot;          // [iters * rows] the instance's slot (-1: skipped by a failed index check)
  unsigned char* first;  // [iters * rows] bit 0 / 1: the instance is the first of its sweep on bi / bj
  int* items;         // [iters * rows] instances ordered by slot
  int* ends;          // [iters * rows + 1] end of each slot in items
  int* body_t;        // [nb] slot of the body's last instance
  int* body_s;        // [nb] sweep of the body's last instance (-1: no row touches it)
  unsigned char* act; // [rows] bit 0 / 1: the row's bi / bj takes velocity updates
  float* ckpt;        // [iters * nb * 6] vlambda, wlambda of a body before its first instance of a sweep
  int rows, iters, nb;
  int mode;           // cp_set_sweep_schedule: 0 where it pays, 1 wherever it fits, -1 never
};
#define CP_WIDE_SCAN_BLOCKS 128

struct DWorld {
  DWorldParams* P;
  DBody* bodies;
  DShape* shapes;
  DHull* hulls;
  DFace* faces;
  float* hverts;   // float4 per vertex
  float* hedges;   // float4 per unique edge
  double* hvd;     // vertices, binary64 (4 per vertex)
  double* hed;     // unique edges, binary64 (4 per edge)
  int* hcanon;     // canonical face / edge index lists
  float* haxes;    // unused by the step (uniqueAxes only gate face tests)
  int* hfi;        // face vertex indices
  int* hconn;      // connected faces
  DMaterial* mats;
  int* cm_table;   // nmat*nmat -> contact material index or -1
  DContactMaterial* cms;  // [0] = world default
  DConstraint* cons;
  int* nocollide;  // body pairs (a, b) of constraints with collideConnected == false
  double* dpow;    // per body: pow(1 - linearDamping, dt), pow(1 - angularDamping, dt) for the cached dt
  DBodyShape* bshapes;  // compound bodies' further shapes
  // scratch
  DBodyScr* bscr;
  // Sphere-broadphase records, one per body, written by the prepare phase:
  // brec = (position, bounding radius rounded to binary32, its sign bit set
  // for a static or sleeping body), bgm = (collisionFilterGroup,
  // collisionFilterMask); consecutive bodies in consecutive memory.
  float4* brec;
  int2* bgm;
  // per chunk of 32 consecutive bodies: the box of their bounding spheres,
  // rounded outward (cbox[2c] = lower corner, cbox[2c + 1] = upper corner
  // with the largest radius in w)
  float4* cbox;
  int* sap_order;
  int* sap_tmp;
  int* pair_a;
  int* pair_b;
  int* pair_cnt;
  int* pair_tstart;
  int* pair_flag;   // event feed: 1 for a kinematic/static job whose shapes overlap (the reference's justTest)
  // Narrowphase jobs of a compound world: one per shape pair of a body pair,
  // pair-major (getContacts' loops, narrow_phase.dart:654-676); job j is
  // shape slot job_sh >> 16 of pair job_pair[j]'s first body against slot
  // job_sh & 0xffff of its second (slot 0: the body's first shape).  In a
  // world without compound bodies a job is a pair.  pair_cnt, pair_tstart,
  // pair_flag and the queues are indexed by job.
  int* job_pair;
  int* job_sh;
  // SplitSolver: the equation pools (persistent, outside the step scratch),
  // the step's equation ids, islands and the rows in descending id order
  long long* pool_c;   // contact equation ids, bottom first (capacity contacts_cap)
  long long* pool_f;   // friction equation ids (capacity 2 * contacts_cap)
  long long* ct_id;    // per contact
  long long* fr_id;    // per friction candidate
  long long* row_id;   // per row
  long long* sort_key; // bitonic sort of the rows by id: keys, then row indices
  int* sort_val;
  int sort_n;          // power of two >= rows_cap
  int* isl_par;        // per body: union-find parent, then the island (its smallest body), -1 static
  int* isl_rows;       // per island: rows
  int* isl_iter;       // per island: -1 while it sweeps, then its iterations
  double* isl_sum;     // per island: the sweep's sum of |dlambda|
  int* row_isl;        // per row: island
  int* job_att;        // per narrowphase job: 1 when spherePlane took an equation object for it
  int* job_base;       // per job: contact objects taken before it (scan)
  int* heavy;       // pairs queued for a resolver, (kind << 28) | pair; later scan scratch
  int* heavy2;      // queued pairs sorted by resolver kind (pairs + 16 * 32 slots)
  DContact* ctmp;
  DContact* contacts;
  int* cscr;       // per-contact scratch (contacts_cap + 1)
  int* cand;       // row candidate -> kept row index, or -1
  DRow* rows;
  double* absdl;
  int* level_of;
  int* level_rows;
  int* level_start;
  int* level_cursor;
  float* sap_key;
  int* bin_cnt;    // grid: per-bin counts / cursors (nbins + 1)
  int* bin_start;  // nbins + 1
  int* bin_body;   // bins_cap entries, bodies of each bin in body order
  float* bin_acc;  // nx + ny + nz accumulated bin-centre offsets
  long long* hkeys;  // pair de-duplication hash (hash_cap)
  int* hvals;
  int hash_cap;
  // The solver rows again, in level order (position p = rank of the row in
  // level_rows) and as separate arrays, so that the threads sweeping a level
  // read consecutive memory: sw_j[f * sw_cap + p], f < 5, the 18 binary32
  // Jacobian values (gaS, gaR, gbS, gbR, iMaR, iMbR); sw_d[f * sw_cap + p],
  // f < 4: (B, invC), (eps, lambda), (imA, imB), (minF, maxF); sw_b: (bi, bj);
  // sw_orig: the row index.
  float4* sw_j;
  double2* sw_d;
  int2* sw_b;
  int* sw_orig;
  int sw_cap;
  DWide* wide;      // counters of a wide step
  int* wpart;       // per-block partial sums of the wide scans (CP_WIDE_SCAN_BLOCKS + 1)
  float* wvel;      // wide sweeps: vlambda, wlambda (6 floats per body) when they do not fit in shared memory
  unsigned char* wflag;  // wide sweeps: solve flag per body
  DSched sched;          // slot-scheduled wide sweeps (zeroed when not allocated)
};
