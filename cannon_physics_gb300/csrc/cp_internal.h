// cp_internal.h -- host-side records shared by the C ABI (cp_host.cpp) and
// the request server (cp_serve.cpp).  Not part of the public interface.
#pragma once

#include <cuda_runtime.h>

#include <climits>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/cannon_gpu.h"
#include "cp_kernels.h"
#include "cp_types.h"

#define CP_WIDE_BODIES_DEFAULT 1024

namespace cpi {

// Sub-arrays of one device allocation, each 256-byte aligned.
struct Layout {
  size_t off = 0;
  size_t take(size_t bytes) {
    size_t o = (off + 255) & ~(size_t)255;
    off = o + bytes;
    return o;
  }
};

struct WorldRec {
  bool live = false;
  char* state = nullptr;   // device: params, bodies, shapes, hulls, materials, constraints, sap order, damping
  char* scratch = nullptr; // device: per-step lists
  long long* pool = nullptr;  // device, SplitSolver: contact then friction equation pools (ids)
  int pool_cap = 0;           // contact pool capacity (the friction pool holds twice as many)
  bool split = false;         // SplitSolver
  int iterations = 0;         // GSSolver.iterations
  char* sched_mem = nullptr;  // device: the slot-scheduled wide sweeps' buffers (DSched), made at the first wide step
  size_t sched_bytes = 0;
  long long sched_skip_rows = -1;  // row capacity for which the buffers were too large or could not be had
  size_t state_bytes = 0, scratch_bytes = 0;
  bool pooled = false;     // state and scratch come from the context's memory pool
  DWorld dw{};
  int nb = 0, nshapes = 0, nmat = 0, ncm = 0, ncons = 0, ncon_rows = 0;
  int n_nocollide = 0;
  int broadphase = 0, nbins = 0;
  int pairs_cap = 0, contacts_cap = 0, rows_cap = 0, bins_cap = 0;
  int jobs_cap = 0;   // shape-pair jobs (compound worlds only)
  bool compound = false;
  std::vector<cp_body_shape> body_shapes;  // the world's extra-shape table
  long long step_limit = LLONG_MAX;  // the kernels leave the world alone at this step number
  double dt_cached = -1.0;
  double accumulator = 0.0;  // World.accumulator of the interpolating World.step
  int last_substeps = 0;     // internal steps of the last interpolating step
  std::vector<double> lin_damp, ang_damp;
  std::vector<int> body_shape;  // each body's shape index (justTest overlaps of the event feed)
  std::vector<int> body_xs0;    // each body's first entry in body_shapes (its extra shapes)
  // event feed
  bool events = false;
  std::vector<int> body_ids, shape_ids;                // the ids overlap keys sort by
  std::vector<unsigned long long> body_keys, shape_keys;  // overlaps of the last step, sorted
  std::vector<cp_event> event_queue;
  std::vector<DContactMaterial> cms;  // host copy for SPOOK updates
};

// Offsets of the state sub-arrays inside a world's state allocation.
struct StateOffsets {
  size_t P, bodies, shapes, hulls, faces, hverts, hedges, hfi, hvd, hed, hcanon, hconn;
  size_t mats, cm_table, cms, cons, nocollide, dpow, sap_order, bshapes;
};

// A world checked and laid out on the host, ready to be copied to the device:
// everything cp_world_create does except the device work.
struct PreparedWorld {
  WorldRec w;
  std::vector<char> host;  // image of the state allocation
  StateOffsets off{};
};

// Records the message of a failing call for cp_last_error (thread-local)
// and returns `code`.
int fail(int code, const char* fmt, ...);
const char* last_error();

}  // namespace cpi

struct cp_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  // When set, world allocations come from this stream-ordered pool (no
  // device-wide synchronisation on allocate or free).
  cudaMemPool_t pool = nullptr;
  std::vector<cpi::WorldRec> worlds;
  DWorld* d_worlds = nullptr;
  int d_worlds_cap = 0;
  int* d_ids = nullptr;
  int d_ids_cap = 0;
  int* d_queue = nullptr;
  int* d_one = nullptr;  // world id of the plain path
  // pinned staging of the plain path: the world id it uploads, the index
  // check record and the world's parameters before and after its launches,
  // read back with one stream synchronisation per call
  struct PlainStage {
    int id, pad;
    int chk[4];
    DWorldParams before, after;
  };
  PlainStage* h_plain = nullptr;
  int plain_id = -1;  // the id d_one holds (-1: unknown)
  int* d_one_group = nullptr;  // {0, 1}: the plain path's single group
  int* d_gstart = nullptr;  // batched path: group boundaries into d_ids
  int ngroups = 0;
  int group_bodies = 640;   // a group gathers consecutive (similar-size) worlds up to this many bodies
  int plain_variant = 2 * cpk_num_solve_variants();  // (pre 128x4, solve 128x4) for single small worlds
  // cp_world_step on a world of at least this many bodies runs the wide
  // kernels (the world spread over the whole GPU); 0: never
  int wide_bodies = CP_WIDE_BODIES_DEFAULT;
  int sched_mode = 0;  // cp_set_sweep_schedule
  // a world whose pair, contact, row or bin list would grow beyond this many
  // entries fails with CP_ERR_CAPACITY instead (0: no limit)
  long long list_cap_limit = 0;
  long long* d_status = nullptr;  // 4 per world after a batched call, then 4 per world before it
  int d_status_cap = 0;
  std::vector<int> dev_order, dev_gstart;  // what d_ids and d_gstart hold
  int sms = 0;
  std::vector<int> blocks_pre, blocks_solve;  // resident blocks per SM, per kernel variant
  // autotuner: one timed step per kernel variant, then the fastest
  std::vector<double> tune_ms;   // ms/step per (pre, solve) variant pair timed so far
  std::vector<int> tune_plan;    // variant pairs still to time in this round
  int tune_next = 0;
  int best = -1;
  std::vector<int> tune_ids;
  long long tune_calls = 0;  // batched calls on this world set
  int forced = -1;
  long long launches = 0;
  std::mutex mu;
  // batched host I/O
  int* d_io_ids = nullptr;
  long long* d_io_first = nullptr;
  int io_cap = 0;
  float* d_io = nullptr;
  long long io_floats = 0;
  std::vector<int> io_ids;  // ids whose offsets are on the device
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // staging of cp_world_get_states / set_states
  cp_body_state* d_states = nullptr;
  int states_cap = 0;
  void* d_rays = nullptr;  // raycast scratch: rays, then hits, then counts
  size_t rays_bytes = 0;
  double graph_ms = 0.0;
  long long graph_step_launches = 0;
  // batched-step graph cache
  cudaGraphExec_t graph = nullptr;
  std::vector<int> graph_ids;
  double graph_dt = 0;
  int graph_steps = 0;
  int graph_variant = -1;
};

namespace cpi {

// All of these expect the context's mutex to be held by the caller, except
// prepare_world, which touches no context.
int prepare_world(const cp_world_desc* d, PreparedWorld& out);
int commit_world(cp_ctx* c, PreparedWorld& p, int* world_id);
int destroy_world(cp_ctx* c, int id);
// Steps a world set `nsteps` times; worlds stop at their step limit.  With
// `use_graph` the launch sequence is captured and replayed while the set, dt
// and step count repeat; without it the kernels are launched directly.
// With `failed`, a world that cannot complete its steps (a capacity beyond
// its limit, a failed regrowth) is listed there and the others complete;
// without it the first such world's error is returned.
int step_worlds(cp_ctx* c, const int* ids, int n, double dt, int nsteps, bool use_graph, std::vector<int>* failed = nullptr);
// World.step(dt) nsteps times on one world (cp_world_step without the
// argument checks): the wide kernels for a world of at least wide_bodies
// bodies, the one-block kernels otherwise; capacities grow as needed.
int world_step_plain(cp_ctx* c, int id, double dt, int nsteps);
int read_bodies(cp_ctx* c, int id, cp_body_desc* out);
int read_info(cp_ctx* c, int id, cp_step_info* out);
// Creates the context's memory pool (release threshold: never) if absent.
int enable_pool(cp_ctx* c);

}  // namespace cpi
