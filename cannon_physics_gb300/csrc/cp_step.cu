// cp_step.cu -- one World.step (lib/world/world_class.dart:433-701) per
// thread block, as a persistent kernel that pulls worlds from a queue: the
// batched form, the served form and the plain path for worlds small enough
// for one block (the phases themselves are in cp_phases.cuh).
#include <cuda_runtime.h>

#include <mutex>

#include "cp_kernels.h"
#include "cp_narrow.cuh"
#include "cp_cc.cuh"
#include "cp_types.h"
#include "cp_phases.cuh"


// Per-phase SM cycles summed over blocks (World.profile's breakdown,
// world_class.dart:27-41); read with cp_phase_profile.
__device__ unsigned long long g_phase_cycles[CP_NUM_PHASES];
// per narrowphase resolver kind: summed thread cycles and calls, counted
// only while g_res_profile is set (cpk_set_resolver_profile): the per-pair
// shared-memory atomics cost a few per cent of a step
__device__ unsigned long long g_res_cycles[16];
__device__ unsigned long long g_res_calls[16];
__device__ int g_res_profile;



// A group of worlds in one block: the state one world keeps between its
// pre-solve phases and its post-solve phases.
#define CP_GROUP_MAX 8
#define CP_SOLVE_MAX_WARPS 8  // solve kernels run at most 256 threads per block
struct __align__(16) Slot {
  DWorld W;
  DWorldParams P;
  int n_pairs, n_contacts, n_rows, n_levels;
  int ok, done, iters, id;
};

// The solve kernel checks every index it derives from a world's level lists
// before it uses it.  A failed check skips the access and records the first
// failure here as {code, world id, index, bound}; the host reads and clears
// it after each launch sequence and reports it as an error.
__device__ int g_check[4];

DI bool index_ok(int code, int world, int idx, int bound) {
  if ((unsigned)idx < (unsigned)bound) return true;
  if (atomicCAS(&g_check[0], 0, code) == 0) {
    g_check[1] = world;
    g_check[2] = idx;
    g_check[3] = bound;
  }
  return false;
}

// GSSolver sweeps (gs_solver.dart:122-155) of all worlds of a group at once:
// level l of every unfinished world runs between the same two barriers, so a
// barrier waits for many independent rows instead of a few.  Each world keeps
// its own iteration count and convergence test.
// Rows of a level handed to a thread: position p in the world's sweep
// arrays and the row's body pair (checked where it is used), or k = -1.
struct LevelRow {
  int k, p;
  int2 bb;
  int r;  // the row's index in the row list (sw_orig)
};

// The first row of level `slot` (a ring entry of per-world level bounds)
// that falls to this thread (both halves of a split level take the same
// rows), with its body pair and row-list index loaded and the rest of its
// record prefetched to L2.  Prepared one level ahead and consumed one level
// later, so that none of these loads lies on a level's path.
DI LevelRow level_row(const Slot* slots, int K, const int* lb, const int* lc) {
  LevelRow R{-1, 0, make_int2(0, 0), -1};
  int total = 0;
  for (int k = 0; k < K; k++) total += lc[k];
  const int half = BT >> 1;
  int off = total <= half ? (int)threadIdx.x % half : (int)threadIdx.x, k = 0;
  while (k < K && off >= lc[k]) { off -= lc[k]; k++; }
  if (k >= K) return R;
  const Slot& sl = slots[k];
  const DWorld& W = sl.W;
  const int p = lb[k] + off;
  if (!index_ok(8, sl.id, p, sl.n_rows)) return R;
  const int cap = W.sw_cap;
#pragma unroll
  for (int q = 0; q < 5; q++) asm volatile("prefetch.global.L2 [%0];" ::"l"(W.sw_j + q * cap + p));
#pragma unroll
  for (int q = 0; q < 4; q++) asm volatile("prefetch.global.L2 [%0];" ::"l"(W.sw_d + q * cap + p));
  R.k = k;
  R.p = p;
  R.bb = W.sw_b[p];
  R.r = W.sw_orig[p];
  return R;
}
DI bool row_bodies_ok(const Slot& sl, int2 bb) {
  return index_ok(5, sl.id, bb.x, sl.P.nb) && index_ok(6, sl.id, bb.y, sl.P.nb);
}

// GSSolver sweeps (gs_solver.dart:122-155) of all worlds of a group at once:
// level l of every unfinished world runs between the same two barriers, so a
// barrier waits for many independent rows instead of a few.  Each world keeps
// its own iteration count and convergence test.
// s_acc: CP_GROUP_MAX * blockDim.x per-thread, per-world sums of |dlambda|
// over a sweep (in shared memory: eight binary64 accumulators in registers
// make the kernel spill); vref: where each world's vlambda / wlambda live.
DI void joint_solve(Smem& S, Slot* slots, int K, double* s_acc, const VelRef* vref) {
  __shared__ double s_part[CP_GROUP_MAX][CP_SOLVE_MAX_WARPS];
  // ring of per-world level bounds: during level l, entry (l+2)%3 is filled
  // for level l+2 and entry (l+1)%3 (filled during level l-1) is read
  __shared__ int s_lb[3][CP_GROUP_MAX], s_lc[3][CP_GROUP_MAX];
  // halves of G*Wlambda exchanged between the two threads of a split row
  __shared__ double s_gx[CP_SOLVE_MAX_WARPS * 32];
  __shared__ int s_ax[CP_SOLVE_MAX_WARPS * 32];
  for (int sweep = 0;; sweep++) {
    int active = 0, Lmax = 0;
    for (int k = 0; k < K; k++) {
      const Slot& sl = slots[k];
      if (sl.ok && !sl.done && sl.n_rows > 0) {
        active |= 1 << k;
        Lmax = max(Lmax, sl.n_levels);
      }
    }
    if (!active) break;
    // level bounds of world threadIdx.x at level l (count 0 once its levels
    // are done): loaded during one level, checked and published at its end
    auto bounds_load = [&](int l, int& b0, int& e0) {
      b0 = e0 = 0;
      if (threadIdx.x < K && (active >> threadIdx.x & 1) && l < slots[threadIdx.x].n_levels) {
        b0 = slots[threadIdx.x].W.level_start[l];
        e0 = slots[threadIdx.x].W.level_start[l + 1];
      }
    };
    auto bounds_store = [&](int l, int e, int b0, int e0) {
      if (threadIdx.x < K) {
        const int k = threadIdx.x;
        const Slot& sl = slots[k];
        int b = 0, c = 0;
        // a level is a non-empty sub-range of [0, n_rows)
        if ((active >> k & 1) && l < sl.n_levels && index_ok(1, sl.id, b0, sl.n_rows) &&
            index_ok(2, sl.id, e0 - 1 - b0, sl.n_rows - b0)) {
          b = b0;
          c = e0 - b0;
        }
        s_lb[e][k] = b;
        s_lc[e][k] = c;
      }
    };
    {
      int b0, e0, b1, e1;
      bounds_load(0, b0, e0);
      bounds_load(1, b1, e1);
      bounds_store(0, 0, b0, e0);
      bounds_store(1, 1, b1, e1);
    }
    __syncthreads();
    LevelRow nxt = level_row(slots, K, s_lb[0], s_lc[0]);
#pragma unroll
    for (int k = 0; k < CP_GROUP_MAX; k++) s_acc[k * BT + threadIdx.x] = 0.0;
    for (int l = 0; l < Lmax; l++) {
      const int e = l % 3;
      const LevelRow cur = nxt;
      int b2, e2;
      bounds_load(l + 2, b2, e2);
      nxt = level_row(slots, K, s_lb[(l + 1) % 3], s_lc[(l + 1) % 3]);
      const int* lb = s_lb[e];
      const int* lc = s_lc[e];
      int total = 0;
      for (int k = 0; k < K; k++) total += lc[k];
      const int half = BT >> 1;
      if (total <= half) {
        // split level (see gs_row_sw): row threadIdx.x % half, side 0 (bi)
        // on threads [0, half), side 1 (bj) on [half, BT)
        const int side = threadIdx.x >= half;
        const int partner = side ? threadIdx.x - half : threadIdx.x + half;
        const bool mine = (int)threadIdx.x - side * half < total && cur.k >= 0 && row_bodies_ok(slots[cur.k], cur.bb);
        RowRec R;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f), w = v;
        float4* pme = nullptr;
        bool act = false;
        double g = 0.0;
        if (mine) {
          R = load_row(slots[cur.k].W, cur.p);
          pme = vl_of(vref[cur.k], side ? cur.bb.y : cur.bb.x);
          v = pme[0];
          w = pme[1];
          act = v.w != 0.f;
          if (act) g = side ? half_b(R, v, w) : half_a(R, v, w);
        }
        s_gx[threadIdx.x] = g;
        s_ax[threadIdx.x] = act;
        __syncthreads();
        if (mine) {
          const int k = cur.k;
          const Slot& sl = slots[k];
          const DWorld& W = sl.W;
          const double go = s_gx[partner];
          const bool ao = s_ax[partner] != 0;
          const double dl = side ? row_dl(R, go, ao, g, act) : row_dl(R, g, act, go, ao);
          const bool same = cur.bb.x == cur.bb.y;
          if (side == 0) {
            W.sw_d[W.sw_cap + cur.p].y = R.d1.y + dl;
            if (act) update_a(pme, v, w, R, dl);
            if (same && ao) update_b(pme, pme[0], pme[1], R, dl);  // the same body, after its first update
            const int r = cur.r;
            if (index_ok(4, sl.id, r, sl.n_rows)) {
              const double a = dl > 0.0 ? dl : -dl;
              W.absdl[r] = a;
              s_acc[k * BT + threadIdx.x] += a;
            }
          } else if (act && !same) {
            update_b(pme, v, w, R, dl);
          }
        }
      } else {
        for (int x = threadIdx.x; x < total; x += BT) {
          int k, p, r;
          int2 bb;
          if (x == (int)threadIdx.x) {
            if (cur.k < 0) continue;  // a failed index check (recorded)
            k = cur.k;
            p = cur.p;
            bb = cur.bb;
            r = cur.r;
          } else {
            int off = x;
            k = 0;
            while (k < K - 1 && off >= lc[k]) { off -= lc[k]; k++; }
            const Slot& sl = slots[k];
            if (!index_ok(3, sl.id, off, lc[k])) continue;
            p = lb[k] + off;
            if (!index_ok(8, sl.id, p, sl.n_rows)) continue;
            bb = sl.W.sw_b[p];
            r = sl.W.sw_orig[p];
          }
          const Slot& sl = slots[k];
          if (!row_bodies_ok(sl, bb)) continue;
          const DWorld& W = sl.W;
          // the row-list index only places |dlambda|; checked after the row
          // so that its load does not delay the row's own
          double a = gs_row_sw(W, vref[k], p, bb);
          if (!index_ok(4, sl.id, r, sl.n_rows)) continue;
          W.absdl[r] = a;
          s_acc[k * BT + threadIdx.x] += a;
        }
      }
      bounds_store(l + 2, (l + 2) % 3, b2, e2);
      __syncthreads();
    }
    // per-world convergence: (sum of |dlambda| in row order)^2 < tol^2, with
    // the order-free block sum deciding unless it lies within the rounding
    // band of the threshold (then the ordered sum decides)
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < CP_GROUP_MAX; k++) {
      double v = s_acc[k * BT + threadIdx.x];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
      if (lane == 0) s_part[k][wid] = v;
    }
    __syncthreads();
    if (threadIdx.x < K) {
      const int k = threadIdx.x;
      Slot& sl = slots[k];
      if (active >> k & 1) {
        double sp = 0.0;
        for (int w = 0; w < (int)NWARP; w++) sp += s_part[k][w];
        const int nrows = sl.n_rows;
        const double tol2 = sl.P.tolerance * sl.P.tolerance;
        double band = 2.2 * (double)nrows * 1.1102230246251565e-16;
        double hi = sp * (1.0 + band), lo = sp * (1.0 - band);
        int conv;
        if (hi * hi * (1.0 + 4.5e-16) < tol2) conv = 1;
        else if (lo * lo * (1.0 - 4.5e-16) >= tol2 && lo >= 0.0) conv = 0;
        else {
          double t = 0.0;
          for (int r = 0; r < nrows; r++) t += sl.W.absdl[r];
          conv = t * t < tol2;
        }
        if (conv) {
          sl.done = 1;
          sl.iters = sweep;
        } else if (sweep + 1 >= sl.P.iterations) {
          sl.done = 1;
          sl.iters = sl.P.iterations;
        }
      }
    }
    __syncthreads();
  }
}

// Kernel 1 of a step: one world per block, everything up to the solver's
// sweeps (pairs, contacts, rows, levels).  Register-hungry (the resolvers).
// Dynamic shared memory: CP_LEVEL_CHUNK row pairs, then the level table of
// up to last_cap bodies.
template <int THREADS, int MINB>
__global__ void __launch_bounds__(THREADS, MINB) k_step_pre(const DWorld* __restrict__ worlds, const int* __restrict__ ids, int n,
                                                           double dt, double time_inc, int* __restrict__ queue, int last_cap) {
  static_assert(THREADS <= 256, "the naive broadphase's count buffers hold 8 warps");
  __shared__ Smem S;
  extern __shared__ int2 s_dyn[];
  int2* s_pairs = s_dyn;
  int* s_last = (int*)(s_dyn + CP_LEVEL_CHUNK);
  if (threadIdx.x < CP_NUM_PHASES) S.t_acc[threadIdx.x] = 0;
  if (threadIdx.x < 16) { S.r_cyc[threadIdx.x] = 0; S.r_cnt[threadIdx.x] = 0; }
  if (threadIdx.x == 0) {
    S.rprof = *(volatile int*)&g_res_profile;
    S.cursor_p = &S.cursor;
    S.overflow_p = &S.overflow;
  }
  for (;;) {
    if (threadIdx.x == 0) S.wi = atomicAdd(queue, 1);
    __syncthreads();
    const int wi = S.wi;
    if (wi >= n) break;
    if (threadIdx.x == 0) {
      S.W = worlds[ids[wi]];
      S.P = *S.W.P;
    }
    __syncthreads();
    if (S.P.status == 0 && S.P.stepnumber < S.P.step_limit) {
      bool ok = step_pre(S, s_last, last_cap, s_pairs, dt);
      if (threadIdx.x == 0) {
        DWorldParams* gp = S.W.P;
        gp->num_pairs = S.n_pairs;
        gp->num_jobs = S.n_jobs;
        gp->num_contacts = S.n_contacts;
        gp->num_rows = ok ? S.n_rows : 0;
        gp->num_levels = ok ? S.n_levels : 0;
        gp->presolved = 0;
        if (!ok) gp->status = S.overflow;
      }
      // a SplitSolver world finishes its step here; the solve kernel skips it
      if (ok && S.P.split) step_split_rest(S, dt, time_inc);
    }
    __syncthreads();
  }
  if (threadIdx.x < CP_NUM_PHASES) atomicAdd(&g_phase_cycles[threadIdx.x], (unsigned long long)S.t_acc[threadIdx.x]);
  if (threadIdx.x < 16 && S.rprof) {
    atomicAdd(&g_res_cycles[threadIdx.x], S.r_cyc[threadIdx.x]);
    atomicAdd(&g_res_calls[threadIdx.x], (unsigned long long)S.r_cnt[threadIdx.x]);
  }
}

// Kernel 2 of a step: the solver sweeps, velocity update, integration and
// sleep for groups of worlds (ids[gstart[g] .. gstart[g+1])).  The sweeps of a
// group share barriers (joint_solve); this kernel needs few registers, so
// many blocks share an SM and hide the binary64 latency of each other's rows.
template <int THREADS, int MINB>
__global__ void __launch_bounds__(THREADS, MINB) k_step_solve(const DWorld* __restrict__ worlds, const int* __restrict__ ids,
                                                             const int* __restrict__ gstart, int ngroups, double dt,
                                                             double time_inc, int* __restrict__ queue) {
  static_assert(THREADS <= 32 * CP_SOLVE_MAX_WARPS, "solve block too wide");
  __shared__ Smem S;
  __shared__ Slot slots[CP_GROUP_MAX];
  __shared__ double s_acc[CP_GROUP_MAX * THREADS];
  __shared__ VelRef s_vref[CP_GROUP_MAX];
  __shared__ int s_voff[CP_GROUP_MAX];  // body offset in s_vel, -1: global memory
  // vlambda / wlambda of the group's bodies while it sweeps (two float4 per
  // body); a group with more bodies than fit keeps them in global memory
  extern __shared__ float4 s_vel[];
  unsigned dyn_bytes;
  asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(dyn_bytes));
  const int vcap = (int)(dyn_bytes / (2 * sizeof(float4)));
  if (threadIdx.x < CP_NUM_PHASES) S.t_acc[threadIdx.x] = 0;
  for (;;) {
    if (threadIdx.x == 0) S.wi = atomicAdd(queue, 1);
    __syncthreads();
    const int g = S.wi;
    if (g >= ngroups) break;
    const int k0 = gstart[g];
    int K = gstart[g + 1] - k0;
    if (!index_ok(7, -1, K - 1, CP_GROUP_MAX)) K = 0;
    if (threadIdx.x < K) {
      Slot& sl = slots[threadIdx.x];
      sl.id = ids[k0 + threadIdx.x];
      sl.W = worlds[sl.id];
      sl.P = *sl.W.P;
      sl.ok = sl.P.status == 0 && sl.P.stepnumber < sl.P.step_limit && !sl.P.presolved;
      sl.n_rows = sl.ok ? sl.P.num_rows : 0;
      sl.n_levels = sl.P.num_levels;
      sl.done = 0;
      sl.iters = 0;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      int vo = 0;
      for (int k = 0; k < K; k++) {
        const Slot& sl = slots[k];
        if (sl.n_rows > 0 && vo + sl.P.nb <= vcap) {
          s_voff[k] = vo;
          s_vref[k] = VelRef{s_vel + 2 * vo, 2};
          vo += sl.P.nb;
        } else {
          s_voff[k] = -1;
          s_vref[k] = vel_global(sl.W);
        }
      }
    }
    __syncthreads();
    for (int k = 0; k < K; k++) {
      if (s_voff[k] < 0) continue;
      const DWorld& W = slots[k].W;
      float4* sv = s_vel + 2 * s_voff[k];
      for (int i = threadIdx.x; i < slots[k].P.nb; i += BT) {
        const float4* gv = (const float4*)W.bscr[i].vl;
        sv[2 * i] = gv[0];
        sv[2 * i + 1] = gv[1];
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) S.t_last = clock64();
    joint_solve(S, slots, K, s_acc, s_vref);
    for (int k = 0; k < K; k++) {
      if (s_voff[k] < 0) continue;
      const DWorld& W = slots[k].W;
      const float4* sv = s_vel + 2 * s_voff[k];
      for (int i = threadIdx.x; i < slots[k].P.nb; i += BT) {
        float4* gv = (float4*)W.bscr[i].vl;
        gv[0] = sv[2 * i];
        gv[1] = sv[2 * i + 1];
      }
    }
    __syncthreads();
    tick(S, 6);
    for (int k = 0; k < K; k++) {
      if (!slots[k].ok) continue;
      if (threadIdx.x == 0) {
        S.W = slots[k].W;
        S.P = slots[k].P;
        S.n_rows = slots[k].n_rows;
      }
      __syncthreads();
      if (S.n_rows > 0) ph_solve_apply(S, dt);
      ph_integrate(S, dt);
      if (threadIdx.x == 0) {
        DWorldParams* gp = S.W.P;
        gp->last_iterations = slots[k].iters;
        gp->stepnumber = S.P.stepnumber + 1;
        gp->time = S.P.time + time_inc;
      }
      tick(S, 7);
      __syncthreads();
    }
  }
  if (threadIdx.x == 6 || threadIdx.x == 7) atomicAdd(&g_phase_cycles[threadIdx.x], (unsigned long long)S.t_acc[threadIdx.x]);
}

// ---------------------------------------------------------------------------
// Kernel 2, warp-centric form.  Every warp takes a pool of up to
// CP_GROUP_MAX worlds from the queue and runs their GSSolver sweeps with no
// block barrier: each round fills the warp's 32 lanes with rows from the
// current level of any of its worlds (rows of one level of one world share
// no dynamic body, and rows of different worlds share nothing), and a world
// moves on to its next level, or its next sweep, as soon as its current
// level is done.  Every world still sees its rows level by level, sweep by
// sweep, so results are those of the block form; the warp's lanes stay busy
// instead of waiting for the slowest level of a block.
#define WS_MAX_ROUNDS (1 << 26)

template <int WARPS, int MINB>
__global__ void __launch_bounds__(WARPS * 32, MINB) k_step_solve_w(const DWorld* __restrict__ worlds, const int* __restrict__ ids,
                                                                  const int* __restrict__ gstart, int ngroups, double dt,
                                                                  double time_inc, int* __restrict__ queue) {
  __shared__ Slot s_slot[WARPS][CP_GROUP_MAX];
  __shared__ int s_cur[WARPS][CP_GROUP_MAX];    // next level position to hand out
  __shared__ int s_end[WARPS][CP_GROUP_MAX];    // end of the current level
  __shared__ int s_lev[WARPS][CP_GROUP_MAX];    // current level
  __shared__ int s_sweep[WARPS][CP_GROUP_MAX];  // current sweep
  __shared__ int s_live[WARPS][CP_GROUP_MAX];   // 1: sweeping, 2: sweep just finished, 0: done
  const unsigned FULL = 0xffffffffu;
  const int wp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  Slot* sl = s_slot[wp];
  int* cur = s_cur[wp];
  int* end = s_end[wp];
  int* lev = s_lev[wp];
  int* swp = s_sweep[wp];
  int* live = s_live[wp];
  for (;;) {
    int g = 0;
    if (lane == 0) g = atomicAdd(queue, 1);
    g = __shfl_sync(FULL, g, 0);
    if (g >= ngroups) break;
    const int k0 = gstart[g];
    int K = gstart[g + 1] - k0;
    if (!index_ok(7, -1, K - 1, CP_GROUP_MAX)) K = 0;
    if (lane < K) {
      Slot& t = sl[lane];
      t.id = ids[k0 + lane];
      t.W = worlds[t.id];
      t.P = *t.W.P;
      t.ok = t.P.status == 0 && t.P.stepnumber < t.P.step_limit && !t.P.presolved;
      t.n_rows = t.ok ? t.P.num_rows : 0;
      t.n_levels = t.P.num_levels;
      t.iters = 0;
      int run = t.n_rows > 0 && t.P.iterations > 0 && t.n_levels > 0;
      int b = 0, e = 0;
      if (run) {
        b = t.W.level_start[0];
        e = t.W.level_start[1];
        if (!index_ok(1, t.id, b, t.n_rows) || !index_ok(2, t.id, e - 1 - b, t.n_rows - b)) run = 0;
      }
      live[lane] = run;
      lev[lane] = 0;
      swp[lane] = 0;
      cur[lane] = b;
      end[lane] = e;
    }
    __syncwarp();
    double part[CP_GROUP_MAX];
#pragma unroll
    for (int k = 0; k < CP_GROUP_MAX; k++) part[k] = 0.0;
    for (int round = 0;; round++) {
      // rows on offer: the rest of every live world's current level
      int pre[CP_GROUP_MAX + 1];
      pre[0] = 0;
#pragma unroll
      for (int k = 0; k < CP_GROUP_MAX; k++) pre[k + 1] = pre[k] + ((k < K && live[k] == 1) ? end[k] - cur[k] : 0);
      const int total = pre[CP_GROUP_MAX];
      if (total == 0) break;
      if (round >= WS_MAX_ROUNDS) {
        index_ok(8, sl[0].id, round, WS_MAX_ROUNDS);
        break;
      }
      if (lane < total) {
        int k = 0;
        while (k < K - 1 && lane >= pre[k + 1]) k++;
        const Slot& t = sl[k];
        const DWorld& W = t.W;
        const int p = cur[k] + lane - pre[k];
        if (index_ok(3, t.id, p, t.n_rows)) {
          const int r = W.sw_orig[p];
          const int2 bb = W.sw_b[p];
          if (index_ok(4, t.id, r, t.n_rows) && index_ok(5, t.id, bb.x, t.P.nb) && index_ok(6, t.id, bb.y, t.P.nb)) {
            const double a = gs_row_sw(W, vel_global(W), p, bb);
            W.absdl[r] = a;
#pragma unroll
            for (int kk = 0; kk < CP_GROUP_MAX; kk++)
              if (kk == k) part[kk] += a;
          }
        }
      }
      __syncwarp();
      // the lanes took the first 32 rows on offer
      if (lane < K && live[lane] == 1) {
        const int k = lane;
        const int take = min(end[k] - cur[k], max(0, 32 - pre[k]));
        cur[k] += take;
        if (cur[k] == end[k]) {
          const Slot& t = sl[k];
          if (lev[k] + 1 < t.n_levels) {
            lev[k]++;
            const int e = t.W.level_start[lev[k] + 1];
            if (index_ok(2, t.id, e - 1 - cur[k], t.n_rows - cur[k])) end[k] = e;
            else live[k] = 0;
          } else {
            live[k] = 2;
          }
        }
      }
      __syncwarp();
      // worlds whose sweep just ended: (sum of |dlambda| in row order)^2 <
      // tol^2, decided by the warp sum unless it lies within the rounding
      // band of the threshold (then by the ordered sum)
#pragma unroll
      for (int k = 0; k < CP_GROUP_MAX; k++) {
        if (k < K && live[k] == 2) {
          double v = part[k];
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(FULL, v, o);
          part[k] = 0.0;
          if (lane == 0) {
            Slot& t = sl[k];
            const int nrows = t.n_rows;
            const double tol2 = t.P.tolerance * t.P.tolerance;
            const double band = 2.2 * (double)nrows * 1.1102230246251565e-16;
            const double hi = v * (1.0 + band), lo = v * (1.0 - band);
            int conv;
            if (hi * hi * (1.0 + 4.5e-16) < tol2) conv = 1;
            else if (lo * lo * (1.0 - 4.5e-16) >= tol2 && lo >= 0.0) conv = 0;
            else {
              double sum = 0.0;
              for (int r = 0; r < nrows; r++) sum += t.W.absdl[r];
              conv = sum * sum < tol2;
            }
            const int sweep = swp[k];
            if (conv) {
              live[k] = 0;
              t.iters = sweep;
            } else if (sweep + 1 >= t.P.iterations) {
              live[k] = 0;
              t.iters = t.P.iterations;
            } else {
              swp[k] = sweep + 1;
              lev[k] = 0;
              cur[k] = t.W.level_start[0];
              end[k] = t.W.level_start[1];
              live[k] = 1;
            }
          }
          __syncwarp();
        }
      }
    }
    // velocities, multipliers, integration and sleep of each world
    const double invDt = 1 / dt;
    for (int k = 0; k < K; k++) {
      const Slot& t = sl[k];
      if (!t.ok) continue;
      const DWorld& W = t.W;
      if (t.n_rows > 0) {
        for (int i = lane; i < t.P.nb; i += 32) apply_body(W, i);
        for (int p = lane; p < t.n_rows; p += 32) apply_row(W, p, invDt);
      }
      __syncwarp();
      const bool qn = (t.P.stepnumber % (long long)(t.P.qn_skip + 1)) == 0;
      for (int i = lane; i < t.P.nb; i += 32) integrate_body(W, t.P, i, dt, qn, t.P.time);
      if (lane == 0) {
        DWorldParams* gp = W.P;
        gp->last_iterations = t.iters;
        gp->stepnumber = t.P.stepnumber + 1;
        gp->time = t.P.time + time_inc;
      }
      __syncwarp();
    }
  }
}

__global__ void k_gather_status(const DWorld* __restrict__ worlds, const int* __restrict__ ids, int n, long long* out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const DWorldParams* p = worlds[ids[i]].P;
  out[4 * i + 0] = p->status;
  out[4 * i + 1] = p->stepnumber;
  out[4 * i + 2] = p->num_pairs;
  out[4 * i + 3] = ((long long)p->num_contacts << 32) | (unsigned)p->num_rows;
}

__global__ void k_clear_status(const DWorld* __restrict__ worlds, const int* __restrict__ ids, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) worlds[ids[i]].P->status = 0;
}

// ---------------------------------------------------------------------------

cudaError_t cpk_gather_status(const DWorld* d_worlds, const int* d_ids, int n, long long* d_out, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  k_gather_status<<<(n + 255) / 256, 256, 0, stream>>>(d_worlds, d_ids, n, d_out);
  return cudaGetLastError();
}

cudaError_t cpk_clear_status(const DWorld* d_worlds, const int* d_ids, int n, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  k_clear_status<<<(n + 255) / 256, 256, 0, stream>>>(d_worlds, d_ids, n);
  return cudaGetLastError();
}

__global__ void k_scatter_forces(const DWorld* __restrict__ worlds, const int* __restrict__ ids, const long long* __restrict__ first,
                                 const float* __restrict__ in) {
  const DWorld& W = worlds[ids[blockIdx.x]];
  const int nb = W.P->nb;
  const float* src = in + 6 * first[blockIdx.x];
  for (int i = threadIdx.x; i < nb; i += blockDim.x) {
    DBody& b = W.bodies[i];
    b.force[0] = src[6 * i]; b.force[1] = src[6 * i + 1]; b.force[2] = src[6 * i + 2];
    b.torque[0] = src[6 * i + 3]; b.torque[1] = src[6 * i + 4]; b.torque[2] = src[6 * i + 5];
  }
}

__global__ void k_gather_poses(const DWorld* __restrict__ worlds, const int* __restrict__ ids, const long long* __restrict__ first,
                               float* __restrict__ out) {
  const DWorld& W = worlds[ids[blockIdx.x]];
  const int nb = W.P->nb;
  float* dst = out + 13 * first[blockIdx.x];
  for (int i = threadIdx.x; i < nb; i += blockDim.x) {
    const DBody& b = W.bodies[i];
    float* o = dst + 13 * i;
    o[0] = b.pos[0]; o[1] = b.pos[1]; o[2] = b.pos[2];
    o[3] = b.quat[0]; o[4] = b.quat[1]; o[5] = b.quat[2]; o[6] = b.quat[3];
    o[7] = b.vel[0]; o[8] = b.vel[1]; o[9] = b.vel[2];
    o[10] = b.avel[0]; o[11] = b.avel[1]; o[12] = b.avel[2];
  }
}

cudaError_t cpk_scatter_forces(const DWorld* d_worlds, const int* d_ids, const long long* d_first, int n, const float* d_in,
                               cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  k_scatter_forces<<<n, 128, 0, stream>>>(d_worlds, d_ids, d_first, d_in);
  return cudaGetLastError();
}

cudaError_t cpk_gather_poses(const DWorld* d_worlds, const int* d_ids, const long long* d_first, int n, float* d_out,
                             cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  k_gather_poses<<<n, 128, 0, stream>>>(d_worlds, d_ids, d_first, d_out);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// World.step's interpolation (world_class.dart:420-428) and the per-step
// body state exchange of a single world

// Quaternion.slerp (quaternion.dart:118-168) in binary64, each component
// stored to binary32; acos and sin are the CUDA math library's
DI q4 qslerp(q4 a, q4 b, double t) {
  const double ax = F(a.x), ay = F(a.y), az = F(a.z), aw = F(a.w);
  double bx = F(b.x), by = F(b.y), bz = F(b.z), bw = F(b.w);
  double cosom = ax * bx + ay * by + az * bz + aw * bw;
  if (cosom < 0.0) {
    cosom = -cosom;
    bx = -bx; by = -by; bz = -bz; bw = -bw;
  }
  double s0, s1;
  if (1.0 - cosom > 0.000001) {
    const double omega = acos(cosom);
    const double sinom = sin(omega);
    s0 = sin((1.0 - t) * omega) / sinom;
    s1 = sin(t * omega) / sinom;
  } else {
    s0 = 1.0 - t;
    s1 = t;
  }
  return q4{rf(s0 * ax + s1 * bx), rf(s0 * ay + s1 * by), rf(s0 * az + s1 * bz), rf(s0 * aw + s1 * bw)};
}

__global__ void k_interpolate(const DWorld* __restrict__ world, int nb, double t) {
  DBody* bodies = world->bodies;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nb; i += gridDim.x * blockDim.x) {
    DBody& b = bodies[i];
    const q4 pq = ld4q(b.prev_quat);
    st3(b.interp_pos, lerp(ld3(b.prev_pos), ld3(b.pos), t));  // previousPosition.lerp(position, t, ...)
    st4q(b.interp_quat, qslerp(pq, ld4q(b.quat), t));
    st4q(b.prev_quat, qnormalize(pq));                          // previousQuaternion.normalize()
  }
}

cudaError_t cpk_interpolate(const DWorld* d_world, int nb, double t, cudaStream_t stream) {
  if (nb <= 0) return cudaSuccess;
  k_interpolate<<<(nb + 255) / 256, 256, 0, stream>>>(d_world, nb, t);
  return cudaGetLastError();
}

__global__ void k_states(const DWorld* __restrict__ world, int nb, cp_body_state* __restrict__ buf, int to_device) {
  DBody* bodies = world->bodies;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nb; i += gridDim.x * blockDim.x) {
    DBody& b = bodies[i];
    cp_body_state& s = buf[i];
    if (to_device) {
      for (int k = 0; k < 3; k++) {
        b.pos[k] = s.position[k]; b.vel[k] = s.velocity[k]; b.avel[k] = s.angular_velocity[k];
        b.force[k] = s.force[k]; b.torque[k] = s.torque[k]; b.prev_pos[k] = s.previous_position[k];
        b.interp_pos[k] = s.interpolated_position[k];
      }
      for (int k = 0; k < 4; k++) {
        b.quat[k] = s.quaternion[k]; b.prev_quat[k] = s.previous_quaternion[k]; b.interp_quat[k] = s.interpolated_quaternion[k];
      }
      b.sleep_state = s.sleep_state;
      b.time_last_sleepy = s.time_last_sleepy;
      b.flags = (b.flags & ~(BF_AABB_DIRTY | BF_WAKE)) | (s.aabb_needs_update ? BF_AABB_DIRTY : 0) |
                (s.wake_up_after_narrowphase ? BF_WAKE : 0);
    } else {
      for (int k = 0; k < 3; k++) {
        s.position[k] = b.pos[k]; s.velocity[k] = b.vel[k]; s.angular_velocity[k] = b.avel[k];
        s.force[k] = b.force[k]; s.torque[k] = b.torque[k]; s.previous_position[k] = b.prev_pos[k];
        s.interpolated_position[k] = b.interp_pos[k];
      }
      for (int k = 0; k < 4; k++) {
        s.quaternion[k] = b.quat[k]; s.previous_quaternion[k] = b.prev_quat[k]; s.interpolated_quaternion[k] = b.interp_quat[k];
      }
      s.sleep_state = b.sleep_state;
      s.time_last_sleepy = b.time_last_sleepy;
      s.aabb_needs_update = (b.flags & BF_AABB_DIRTY) != 0;
      s.wake_up_after_narrowphase = (b.flags & BF_WAKE) != 0;
      s.pad0 = 0;
    }
  }
}

cudaError_t cpk_states(const DWorld* d_world, int nb, cp_body_state* d_buf, int to_device, cudaStream_t stream) {
  if (nb <= 0) return cudaSuccess;
  k_states<<<(nb + 255) / 256, 256, 0, stream>>>(d_world, nb, d_buf, to_device);
  return cudaGetLastError();
}


// ---------------------------------------------------------------------------
// Static step scratch for cp_world_step_static: a file-scope device array, so
// stepping through it needs no device allocation.  Its address is taken once
// per device, with that device current, by the first cpk_static_scratch call.
static __device__ __align__(256) unsigned char g_static_scratch[CP_STATIC_SCRATCH_BYTES];

namespace {
std::mutex g_static_mu;
void* g_static_addr[CP_MAX_DEVICES] = {};
}  // namespace

cudaError_t cpk_static_scratch(int device, void** ptr, size_t* bytes) {
  *ptr = nullptr;
  *bytes = 0;
  if (device < 0 || device >= CP_MAX_DEVICES) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_static_mu);
  if (!g_static_addr[device]) {
    int cur = -1;
    cudaError_t e = cudaGetDevice(&cur);
    if (e != cudaSuccess) return e;
    if (cur != device) return cudaErrorInvalidDevice;
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess) return e;
    g_static_addr[device] = p;
  }
  *ptr = g_static_addr[device];
  *bytes = sizeof(g_static_scratch);
  return cudaSuccess;
}

cudaError_t cpk_read_check_async(int* out, cudaStream_t stream) {
  return cudaMemcpyFromSymbolAsync(out, g_check, sizeof(int) * 4, 0, cudaMemcpyDeviceToHost, stream);
}

cudaError_t cpk_read_check(int out[4]) {
  cudaError_t e = cudaMemcpyFromSymbol(out, g_check, sizeof(int) * 4);
  if (e == cudaSuccess && out[0] != 0) {
    int z[4] = {0, 0, 0, 0};
    e = cudaMemcpyToSymbol(g_check, z, sizeof(z));
  }
  return e;
}

cudaError_t cpk_phase_cycles(unsigned long long* out, bool reset) {
  cudaError_t e = cudaMemcpyFromSymbol(out, g_phase_cycles, sizeof(unsigned long long) * CP_NUM_PHASES);
  if (e == cudaSuccess) e = cudaMemcpyFromSymbol(out + CP_NUM_PHASES, g_res_cycles, sizeof(unsigned long long) * 16);
  if (e == cudaSuccess) e = cudaMemcpyFromSymbol(out + CP_NUM_PHASES + 16, g_res_calls, sizeof(unsigned long long) * 16);
  if (e == cudaSuccess && reset) {
    unsigned long long z[16] = {0};
    e = cudaMemcpyToSymbol(g_phase_cycles, z, sizeof(unsigned long long) * CP_NUM_PHASES);
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_res_cycles, z, sizeof(z));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_res_calls, z, sizeof(z));
  }
  return e;
}

cudaError_t cpk_filter_check(int on) { return cudaMemcpyToSymbol(g_filter_check, &on, sizeof(int)); }

cudaError_t cpk_filter_counts(unsigned long long out[2], bool reset) {
  cudaError_t e = cudaMemcpyFromSymbol(out, g_filter_count, 2 * sizeof(unsigned long long));
  if (e == cudaSuccess && reset) {
    const unsigned long long z[2] = {0, 0};
    e = cudaMemcpyToSymbol(g_filter_count, z, sizeof(z));
  }
  return e;
}

cudaError_t cpk_set_resolver_profile(int on) {
  const int v = on ? 1 : 0;
  return cudaMemcpyToSymbol(g_res_profile, &v, sizeof(v));
}

// Kernel variants (block threads, minimum resident blocks per SM) for each
// of the two kernels: the register budget, and with it the number of blocks
// that hide each other's waits, differs between them.  All compute
// identical results.
struct PreVariant {
  void (*fn)(const DWorld*, const int*, int, double, double, int*, int);
  int threads;
  int minb;
};
struct SolveVariant {
  void (*fn)(const DWorld*, const int*, const int*, int, double, double, int*);
  int threads;
  int minb;
  int per_warp;  // each warp takes its own group (k_step_solve_w)
};
static const PreVariant kPre[] = {
    {k_step_pre<256, 1>, 256, 1}, {k_step_pre<128, 2>, 128, 2}, {k_step_pre<128, 4>, 128, 4},
    {k_step_pre<64, 8>, 64, 8},   {k_step_pre<256, 2>, 256, 2}, {k_step_pre<32, 16>, 32, 16},
};
static const SolveVariant kSolve[] = {
    {k_step_solve<128, 4>, 128, 4, 0},     {k_step_solve<128, 8>, 128, 8, 0},     {k_step_solve<256, 4>, 256, 4, 0},
    {k_step_solve<128, 6>, 128, 6, 0},     {k_step_solve<64, 16>, 64, 16, 0},     {k_step_solve_w<4, 4>, 128, 4, 1},
    {k_step_solve<64, 12>, 64, 12, 0},     {k_step_solve_w<8, 4>, 256, 4, 1},
};
static const int kNumPre = sizeof(kPre) / sizeof(kPre[0]);
static const int kNumSolve = sizeof(kSolve) / sizeof(kSolve[0]);

int cpk_num_variants() { return kNumPre * kNumSolve; }
int cpk_num_pre_variants() { return kNumPre; }
int cpk_num_solve_variants() { return kNumSolve; }

int cpk_variant_threads(int v) { return kPre[v / kNumSolve].threads; }
int cpk_solve_threads(int v) { return kSolve[v % kNumSolve].threads; }
int cpk_solve_group_limit(int v, int group_bodies) {
  const SolveVariant& V = kSolve[v % kNumSolve];
  return V.per_warp ? group_bodies : (int)((long long)group_bodies * V.threads / 128);
}

// body capacity of the pre kernel's shared level table for a launch whose
// largest world has max_nb bodies, and the dynamic shared memory it takes
static int last_cap_for(int max_nb) { return max_nb < 1 ? 1 : (max_nb < CP_SMEM_LEVEL_MAX ? max_nb : CP_SMEM_LEVEL_MAX); }
static size_t pre_smem(int last_cap) { return sizeof(int2) * CP_LEVEL_CHUNK + sizeof(int) * (size_t)last_cap; }

// shared memory for the solve kernel's vlambda / wlambda: the bodies of a
// default-size group (CP_SOLVE_VEL_BODIES per 128 threads)
#define CP_SOLVE_VEL_BODIES 640
static size_t solve_smem(const SolveVariant& V) {
  return V.per_warp ? 0 : (size_t)CP_SOLVE_VEL_BODIES * V.threads / 128 * 2 * sizeof(float4);
}

int cpk_pre_blocks_per_sm(int variant, int max_nb) {
  const PreVariant& P = kPre[variant / kNumSolve];
  int b = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, P.fn, P.threads, pre_smem(last_cap_for(max_nb)));
  return b < 1 ? 1 : b;
}

cudaError_t cpk_launch_step(const DWorld* d_worlds, const int* d_ids, const int* d_gstart, int ngroups, double dt, double time_inc,
                            int* d_queue, int grid_pre, int grid_solve, cudaStream_t stream, int variant, int n, int max_nb) {
  cudaError_t e = cudaMemsetAsync(d_queue, 0, 2 * sizeof(int), stream);
  if (e != cudaSuccess) return e;
  const PreVariant& P = kPre[variant / kNumSolve];
  const SolveVariant& V = kSolve[variant % kNumSolve];
  const int cap = last_cap_for(max_nb);
  P.fn<<<grid_pre, P.threads, pre_smem(cap), stream>>>(d_worlds, d_ids, n, dt, time_inc, d_queue, cap);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  V.fn<<<grid_solve, V.threads, solve_smem(V), stream>>>(d_worlds, d_ids, d_gstart, ngroups, dt, time_inc, d_queue + 1);
  return cudaGetLastError();
}

void cpk_max_resident_blocks(int variant, int* pre, int* solve) {
  const PreVariant& P = kPre[variant / kNumSolve];
  const SolveVariant& V = kSolve[variant % kNumSolve];
  *pre = 0;
  *solve = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(pre, P.fn, P.threads, pre_smem(last_cap_for(512)));
  // static plus dynamic shared memory above 48 KB needs the kernel's opt-in
  cudaFuncSetAttribute((const void*)V.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)solve_smem(V));
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(solve, V.fn, V.threads, solve_smem(V));
}
