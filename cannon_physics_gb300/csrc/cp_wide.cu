// cp_wide.cu -- one large World.step (lib/world/world_class.dart:433-701)
// spread over the whole GPU.
//
// A world of thousands of bodies holds tens of thousands of broadphase pairs
// and contacts; one thread block (cp_step.cu) runs them on one SM of 152.
// Here every phase is a grid-wide kernel over its items (bodies, list
// positions, pairs, contacts, rows), built from the same per-item functions
// as the one-block kernels (cp_phases.cuh), so the results are the same bits.
// Counts that the one-block kernels keep in shared memory live in the
// world's DWide record; ordered outputs come from grid-wide exclusive scans
// (per-block partial sums, then each block scans its chunk from its prefix).
// Two phases stay on one block: the dependency levels (each row's level
// depends on every earlier row on its bodies) and the Gauss-Seidel sweeps
// (level after level, sweep after sweep), which run with vlambda / wlambda
// in shared memory and each thread's next row record loaded a level ahead.
//
// Every kernel starts by reading the world's run flag and overflow bits, so
// after a capacity overflow the rest of the step does nothing and the body
// state is left as it was before the step (the host regrows and re-runs).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>

#include "cp_kernels.h"
#include "cp_phases.cuh"

#define WT 256  // threads per block of the grid-wide kernels
#define WIDE_LOOP(i, n) for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += gridDim.x * blockDim.x)

// The block's copy of the world descriptor and parameters; false when the
// step does not run (status set, step limit reached) or has overflowed.
// the narrowphase's job count: the pairs, or a compound world's shape pairs
DI int wide_jobs(const DWorld& W) { return W.P->compound ? W.wide->n_jobs : W.wide->n_pairs; }

DI bool wide_enter(Smem& S, const DWorld* dw) {
  if (threadIdx.x == 0) {
    S.W = *dw;
    S.P = *S.W.P;
    S.rprof = 0;
    S.cursor_p = &S.W.wide->cursor;
    S.overflow_p = &S.W.wide->overflow;
    const DWide* x = S.W.wide;
    S.wi = x->run && x->overflow == 0;
  }
  __syncthreads();
  return S.wi != 0;
}

// ---------------------------------------------------------------------------
// scans: a[0..n) -> exclusive prefix sums in place, n read from device memory

__global__ void k_w_scan1(const DWorld* dw, int* a, const int* n_ptr) {
  __shared__ Smem S;
  if (!wide_enter(S, dw)) return;
  const int n = *n_ptr;
  const int chunk = (n + gridDim.x - 1) / gridDim.x;
  const int b0 = min(n, (int)blockIdx.x * chunk), b1 = min(n, b0 + chunk);
  int s = 0;
  for (int i = b0 + threadIdx.x; i < b1; i += BT) s += a[i];
  int tot;
  block_excl_scan(S, s, tot);
  if (threadIdx.x == 0) S.W.wpart[blockIdx.x] = tot;
}

// total -> *out (and *out2 when given); with cap >= 0, a total above cap
// sets overflow bit `bit`
__global__ void k_w_scan2(const DWorld* dw, int* a, const int* n_ptr, int* out, int* out2, int cap, int bit) {
  __shared__ Smem S;
  if (!wide_enter(S, dw)) return;
  const int n = *n_ptr;
  const int chunk = (n + gridDim.x - 1) / gridDim.x;
  const int b0 = min(n, (int)blockIdx.x * chunk), b1 = min(n, b0 + chunk);
  int pre = 0;
  for (int k = threadIdx.x; k < (int)blockIdx.x; k += BT) pre += S.W.wpart[k];
  int tot;
  block_excl_scan(S, pre, tot);
  pre = tot;  // sum of the partials before this block
  const int mine = block_scan_array(S, a + b0, b1 - b0);
  for (int i = b0 + threadIdx.x; i < b1; i += BT) a[i] += pre;
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) {
    const int total = pre + mine;
    *out = total;
    if (out2) *out2 = total;
    if (cap >= 0 && total > cap) atomicOr(&S.W.wide->overflow, bit);
  }
}

static cudaError_t wide_scan(const DWorld* dw, int* a, const int* n_ptr, int* out, int* out2, int cap, int bit,
                             cudaStream_t st) {
  k_w_scan1<<<CP_WIDE_SCAN_BLOCKS, WT, 0, st>>>(dw, a, n_ptr);
  k_w_scan2<<<CP_WIDE_SCAN_BLOCKS, WT, 0, st>>>(dw, a, n_ptr, out, out2, cap, bit);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// step start and the state-change boundary

__global__ void k_w_begin(const DWorld* dw) {
  const DWorld W = *dw;
  const DWorldParams& P = *W.P;
  DWide* x = W.wide;
  if (threadIdx.x == 0) {
    x->run = P.status == 0 && P.stepnumber < P.step_limit;
    x->overflow = 0;
    x->n_pairs = x->n_cand_pairs = x->n_contacts = x->n_fric = 0;
    x->n_cand = x->n_rows = x->n_levels = x->iters = 0;
    x->n_queued = x->n_queued2 = x->nh_padded = x->cursor = 0;
    x->total = x->n_jobs = 0;
  }
  if (threadIdx.x < 16) { x->kcnt[threadIdx.x] = 0; x->kpos[threadIdx.x] = 0; }
}

// After the rows are listed and before any body state changes: an overflow
// ends the step here, with the step's counts recorded as the one-block
// kernels record them.
__global__ void k_w_mid(const DWorld* dw) {
  const DWorld W = *dw;
  DWide* x = W.wide;
  if (!x->run) return;
  DWorldParams* P = W.P;
  P->num_pairs = x->n_pairs;
  P->num_jobs = wide_jobs(W);
  P->num_contacts = x->n_contacts;
  if (x->overflow) {
    P->num_rows = 0;
    P->num_levels = 0;
    P->status = x->overflow;
    x->run = 0;
  }
}

__global__ void k_w_end(const DWorld* dw, double time_inc) {
  const DWorld W = *dw;
  DWide* x = W.wide;
  if (!x->run) return;
  DWorldParams* P = W.P;
  P->num_rows = x->n_rows;
  P->num_levels = x->n_levels;
  P->last_iterations = x->iters;
  P->stepnumber = P->stepnumber + 1;
  P->time = P->time + time_inc;
}

// ---------------------------------------------------------------------------
// prepare, broadphase

__global__ void k_w_prepare(const DWorld* dw) {
  __shared__ Smem S;
  if (!wide_enter(S, dw)) return;
  WIDE_LOOP(i, S.P.nb) prepare_body(S.W, S.P, i);
}

// SAP: stable re-sort of the persisted list by aabb.lowerBound[axis]
// (sap_broadphase.dart:66-79): the new rank of position p is
// #{keys < key_p} + #{q < p : key_q == key_p}, where insertion sort leaves it
__global__ void k_w_sap_key(const DWorld* dw) {
  __shared__ Smem S;
  if (!wide_enter(S, dw)) return;
  const DWorld& W = S.W;
  WIDE_LOOP(p, S.P.nb) W.sap_key[p] = W.bodies[W.sap_order[p]].aabb_lo[S.P.sap_axis];
}

#define SAP_TILE 1024
__global__ void k_w_sap_rank(const DWorld* dw) {
  __shared__ Smem S;
  __shared__ float s_key[SAP_TILE];
  if (!wide_enter(S, dw)) return;
  const DWorld& W = S.W;
  const int nb = S.P.nb;
  for (int p0 = blockIdx.x * BT; p0 < nb; p0 += gridDim.x * BT) {
    const int p = p0 + threadIdx.x;
    const float kp = p < nb ? W.sap_key[p] : 0.f;
    int r = 0;
    for (int q0 = 0; q0 < nb; q0 += SAP_TILE) {
      const int m = min(SAP_TILE, nb - q0);
      __syncthreads();
      for (int q = threadIdx.x; q < m; q += BT) s_key[q] = W.sap_key[q0 + q];
      __syncthreads();
      for (int q = 0; q < m; q++) {
        const float kq = s_key[q];
        r += (kq < kp) || (kq == kp && q0 + q < p);
      }
    }
    if (p < nb) W.sap_tmp[r] = W.sap_order[p];
  }
}

__global__ void k_w_sap_copy(const DWorld* dw) {
  __shared__ Smem S;
  if (!wide_enter(S, dw)) return;
  WIDE_LOOP(p, S.P.nb) S.W.sap_order[p] = S.W.sap_tmp[p];
}

// SAPBroadphase.collisionPairs' scan from list position i (sap_broadphase.dart:
// 149-165) by one warp, 32 list positions at a time: `continue` on a pair
// the filter rejects, `break` at the first remaining pair whose bounds are
// apart (the lowest such lane), a pair for every earlier lane that
// intersects.  Counts the pairs, or writes them from pair_cnt[i] on.  A
// plane (infinite bounds, it sorts first and pairs with every body) scans
// the whole list 32 times faster than a thread alone would.
DI int sap_scan_warp(const DWorld& W, const DWorldParams& P, int i, bool write) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int nb = P.nb, axis = P.sap_axis;
  const int ai = W.sap_order[i];
  const DBody& bi = W.bodies[ai];
  const int out = write ? W.pair_cnt[i] : 0;
  int count = 0;
  for (int j0 = i + 1; j0 < nb; j0 += 32) {
    const int j = j0 + lane;
    const int aj = j < nb ? W.sap_order[j] : 0;
    const DBody& bj = W.bodies[aj];
    const bool np = j < nb && need_pair(bi, bj);
    const bool brk = np && !check_bounds(bi, bj, axis);
    const unsigned bm = __ballot_sync(FULL, brk);
    const int first = bm ? __ffs(bm) - 1 : 32;
    const bool hit = np && lane < first && intersection_test(P, bi, bj);
    const unsigned hm = __ballot_sync(FULL, hit);
    if (write && hit) {
      const int o = out + count + __popc(hm & ((1u << lane) - 1u));
      W.pair_a[o] = ai;
      W.pair_b[o] = aj;
    }
    count += __popc(hm);
    if (bm) break;
  }
  return count;
}

__global__ void k_w_sap_pairs(const DWorld* dw, int write) {
  __shared__ Smem S;
  if (!wide_enter(S, dw)) return;
  if (write && S.W.wide->n_cand_pairs > S.P.pairs_cap) return;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < S.P.nb; i += nwarps) {
    const int c = sap_scan_warp(S.W, S.P, i, write != 0);
    if (!write && (threadIdx.x & 31) == 0) S.W.pair_cnt[i] = c;
  }
}

// Naive: the i > j triangle in order (naive_broadphase.dart:14-33).  Block b
// takes a contiguous range of the triangle; pass 0 counts its pairs into
// wpart[b], pass 1 (after a scan of wpart) writes them from its offset in
// the same order, BT * 4 candidates at a time.
DI void naive_tile_bodies(const Smem& S, long long k0, long long T, int& bits, int& cnt, int& i, int& j) {
  const DWorld& W = S.W;
  bits = cnt = 0;
  i = j = 0;
  if (k0 >= T) return;
  i = (int)((1.0f + sqrtf(1.0f + 8.0f * (float)k0)) * 0.5f);
  while ((long long)i * (i - 1) / 2 > k0) i--;
  while ((long long)(i + 1) * i / 2 <= k0) i++;
  j = (int)(k0 - (long long)i * (i - 1) / 2);
  int ii = i, jj = j;
  for (int m = 0; m < 4 && k0 + m < T; m++) {
    const DBody& A = W.bodies[ii];
    const DBody& B = W.bodies[jj];
    if (need_pair(A, B) && intersection_test(S.P, A, B)) {
      bits |= 1 << m;
      cnt++;
    }
    if (++jj == ii) { ii++; jj = 0; }
  }
}

__global__ void k_w_naive(const DWorld* dw, int pass) {
  __shared__ Smem S;
  if (!wide_enter(S, dw)) return;
  const DWorld& W = S.W;
  const int nb = S.P.nb;
  const long long T = (long long)nb * (nb - 1) / 2;
  const long long chunk = (T + gridDim.x - 1) / gridDim.x;
  const long long c0 = min(T, (long long)blockIdx.x * chunk), c1 = min(T, c0 + chunk);
  if (pass == 1 && W.wide->n_cand_pairs > S.P.pairs_cap) return;
  int out = pass == 1 ? W.wpart[blockIdx.x] : 0;
  if (!S.P.use_bb) {  // bounding spheres: the prepare phase's records
    int i = 0, j = 0, buf = 0;
    NaiveRow R;
    R.init();
    if (c0 < c1) naive_from_flat(c0 + threadIdx.x, i, j);
    for (long long k0 = c0; k0 < c1; k0 += (long long)NAIVE_SUB * BT)
      out += naive_tile(S, k0, c1, pass == 1, out, S.P.pairs_cap, i, j, R, buf);
    if (pass == 0 && threadIdx.x == 0) W.wpart[blockIdx.x] = out;
    return;
  }
  for (long long tile = c0; tile < c1; tile += BT * 4) {
    const long long k0 = tile + (long long)threadIdx.x * 4;
    int bits, cnt, i, j;
    naive_tile_bodies(S, k0, c1, bits, cnt, i, j);
    int tot;
    const int pre = block_excl_scan(S, cnt, tot);
    if (pass == 1 && cnt) {
      int o = out + pre, ii = i, jj = j;
      for (int m = 0; m < 4; m++) {
        if (bits & (1 << m)) { W.pair_a[o] = ii; W.pair_b[o] = jj; o++; }
        if (++jj == ii) { ii++; jj = 0; }
      }
    }
    out += tot;
  }
  if (pass == 0 && threadIdx.x == 0) W.wpart[blockIdx.x] = out;
}

// scan of the naive per-block counts (one block)
__global__ void __launch_bounds__(1024) k_w_naive_scan(const DWorld* dw, int nblocks) {
  __shared__ Smem S;
  if (!wide_enter(S, dw)) return;
  const int total = block_scan_array(S, S.W.wpart, nblocks);
  if (threadIdx.x == 0) {
    S.W.wide->n_cand_pairs = total;
    S.W.wide->n_pairs = total;
    if (total > S.P.pairs_cap) atomicOr(&S.W.wide->overflow, ST_PAIRS_OVERFLOW);
  }
}

// Grid (repaired GridBroadphase, grid_broadphase.dart:59-239)
__global__ void k_w_grid_zero(const DWorld* dw) {
  __shared__ Smem S;
  if (!wide_enter(S, dw)) return;
  WIDE_LOOP(b, S.P.grid_nx * S.P.grid_ny * S.P.grid_nz) S.W.bin_cnt[b] = 0;
}

__global__ void k_w_grid_bin(const DWorld* dw, int pass) {
  __shared__ Smem S;
  if (!wide_enter(S, dw)) return;
  double c[10];
  grid_consts(S.P, c);
  WIDE_LOOP(i, S.P.nb) grid_bin_body(S.W, S.P, c, i, pass);
}

__global__ void __launch_bounds__(1024) k_w_grid_planes(const DWorld* dw, int pass) {
  __shared__ Smem S;
  if (!wide_enter(S, dw)) return;
  double c[10];
  grid_consts(S.P, c);
  grid_bin_planes(S, c, pass);
}

__global__ void k_w_grid_starts(const DWorld* dw) {
  __shared__ Smem S;
  if (!wide_enter(S, dw)) return;
  const int nBins = S.P.grid_nx * S.P.grid_ny * S.P.grid_nz;
  WIDE_LOOP(b, nBins) S.W.bin_start[b] = S.W.bin_cnt[b];
  if (blockIdx.x == 0 && threadIdx.x == 0) S.W.bin_start[nBins] = S.W.wide->total;
}

__global__ void k_w_grid_sort(const DWorld* dw) {
  __shared__ Smem S;
  if (!wide_enter(S, dw)) return;
  WIDE_LOOP(b, S.P.grid_nx * S.P.grid_ny * S.P.grid_nz) grid_sort_bin(S.W, b);
}

__global__ void k_w_grid_pairs(const DWorld* dw, int write) {
  __shared__ Smem S;
  if (!wide_enter(S, dw)) return;
  WIDE_LOOP(b, S.P.grid_nx * S.P.grid_ny * S.P.grid_nz) {
    const int c = grid_bin_pairs(S.W, S.P, b, write != 0);
    if (!write) S.W.bin_cnt[b] = c;
  }
}

__global__ void k_w_grid_check(const DWorld* dw) {
  const DWorld W = *dw;
  DWide* x = W.wide;
  if (!x->run || x->overflow) return;
  const int total = x->n_cand_pairs;
  if (total > W.P->pairs_cap || 2 * total > W.hash_cap) atomicOr(&x->overflow, ST_PAIRS_OVERFLOW);
}

__global__ void k_w_hash(const DWorld* dw, int op) {
  __shared__ Smem S;
  if (!wide_enter(S, dw)) return;
  const DWorld& W = S.W;
  if (op == 0) {
    WIDE_LOOP(h, W.hash_cap) grid_hash_clear(W, h);
  } else if (op == 1) {
    WIDE_LOOP(k, W.wide->n_cand_pairs) grid_hash_insert(W, k);
  } else {
    WIDE_LOOP(k, W.wide->n_cand_pairs) grid_hash_keep(W, k);
  }
}

// stable compaction of the kept candidate pairs (grid de-duplication,
// constraint-pair removal): n_cand_pairs candidates, n_pairs kept
__global__ void k_w_compact(const DWorld* dw) {
  __shared__ Smem S;
  if (!wide_enter(S, dw)) return;
  const int n = S.W.wide->n_cand_pairs, kept = S.W.wide->n_pairs;
  WIDE_LOOP(k, n) compact_pair(S.W, k, n, kept);
}

// constraint-pair removal (world_class.dart:487-499)
__global__ void k_w_nocollide(const DWorld* dw) {
  __shared__ Smem S;
  if (!wide_enter(S, dw)) return;
  const DWorld& W = S.W;
  const int nn = S.P.n_nocollide;
  if (blockIdx.x == 0 && threadIdx.x == 0) W.wide->n_cand_pairs = W.wide->n_pairs;
  WIDE_LOOP(k, W.wide->n_pairs) {
    int a = W.pair_a[k], b = W.pair_b[k];
    int keep = 1;
    for (int c = 0; c < nn; c++) {
      int ca = W.nocollide[2 * c], cb = W.nocollide[2 * c + 1];
      if ((ca == a && cb == b) || (cb == a && ca == b)) keep = 0;
    }
    W.pair_cnt[k] = keep;
    W.pair_tstart[k] = a;
    W.heavy[k] = b;
  }
}

// ---------------------------------------------------------------------------
// narrowphase

// a compound world's jobs: count per pair, then (after a scan) the list
__global__ void k_w_jobs(const DWorld* dw, int fill) {
  __shared__ Smem S;
  if (!wide_enter(S, dw)) return;
  if (fill) {
    WIDE_LOOP(k, S.W.wide->n_pairs) pair_jobs_fill(S.W, k, S.W.pair_cnt[k]);
  } else {
    WIDE_LOOP(k, S.W.wide->n_pairs) S.W.pair_cnt[k] = pair_jobs(S.W, k);
  }
}

__global__ void k_w_narrow_first(const DWorld* dw) {
  __shared__ Smem S;
  if (!wide_enter(S, dw)) return;
  WIDE_LOOP(k, wide_jobs(S.W)) narrow_first(S, k, &S.W.wide->n_queued);
}

__global__ void k_w_kind_count(const DWorld* dw) {
  __shared__ Smem S;
  __shared__ int s_cnt[16];
  if (!wide_enter(S, dw)) return;
  if (threadIdx.x < 16) s_cnt[threadIdx.x] = 0;
  __syncthreads();
  WIDE_LOOP(h, S.W.wide->n_queued) atomicAdd(&s_cnt[(unsigned)S.W.heavy[h] >> 28], 1);
  __syncthreads();
  if (threadIdx.x < 16 && s_cnt[threadIdx.x]) atomicAdd(&S.W.wide->kcnt[threadIdx.x], s_cnt[threadIdx.x]);
}

// each kind's segment starts on a warp boundary
__global__ void k_w_kind_pos(const DWorld* dw) {
  const DWorld W = *dw;
  DWide* x = W.wide;
  if (!x->run || x->overflow) return;
  int o = 0;
  for (int r = 0; r < 16; r++) {
    x->kpos[r] = o;
    o += (x->kcnt[r] + 31) & ~31;
  }
  x->nh_padded = o;
  x->n_queued2 = 0;
  x->cursor = 0;
}

__global__ void k_w_kind_fill(const DWorld* dw) {
  __shared__ Smem S;
  if (!wide_enter(S, dw)) return;
  WIDE_LOOP(h, S.W.wide->nh_padded) S.W.heavy2[h] = -1;
}

__global__ void k_w_kind_scatter(const DWorld* dw) {
  __shared__ Smem S;
  if (!wide_enter(S, dw)) return;
  const DWorld& W = S.W;
  WIDE_LOOP(h, W.wide->n_queued) {
    const unsigned e = (unsigned)W.heavy[h];
    W.heavy2[atomicAdd(&W.wide->kpos[e >> 28], 1)] = (int)e;
  }
}

template <int THREADS>
__global__ void __launch_bounds__(THREADS) k_w_stage1(const DWorld* dw) {
  __shared__ Smem S;
  if (!wide_enter(S, dw)) return;
  WIDE_LOOP(h, S.W.wide->nh_padded) narrow_stage1(S, h, &S.W.wide->n_queued2);
}

template <int THREADS>
__global__ void __launch_bounds__(THREADS) k_w_stage2(const DWorld* dw) {
  __shared__ Smem S;
  if (!wide_enter(S, dw)) return;
  WIDE_LOOP(h, S.W.wide->n_queued2) narrow_stage2(S, h);
}

__global__ void k_w_contact_counts(const DWorld* dw) {
  __shared__ Smem S;
  if (!wide_enter(S, dw)) return;
  WIDE_LOOP(k, wide_jobs(S.W)) S.W.heavy[k] = S.W.pair_cnt[k];
}

__global__ void k_w_contact_place(const DWorld* dw) {
  __shared__ Smem S;
  if (!wide_enter(S, dw)) return;
  WIDE_LOOP(k, wide_jobs(S.W)) narrow_place(S.W, k);
}

// ---------------------------------------------------------------------------
// rows

__global__ void k_w_fric(const DWorld* dw) {
  __shared__ Smem S;
  if (!wide_enter(S, dw)) return;
  WIDE_LOOP(c, S.W.wide->n_contacts) contact_fric_count(S.W, S.P, c);
}

__global__ void k_w_cands(const DWorld* dw) {
  __shared__ Smem S;
  if (!wide_enter(S, dw)) return;
  const DWorld& W = S.W;
  const int nc = W.wide->n_contacts, nF = W.wide->n_fric;
  WIDE_LOOP(t, nc + S.P.ncons) {
    if (t < nc) contact_cands(W, t, nc, nF);
    else constraint_cands(W, t - nc, nF + nc);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) W.wide->n_cand = nF + nc + S.P.ncon_rows;
}

__global__ void k_w_post(const DWorld* dw) {
  __shared__ Smem S;
  if (!wide_enter(S, dw)) return;
  WIDE_LOOP(c, S.W.wide->n_contacts) contact_post(S.W, c);
}

__global__ void k_w_bodies(const DWorld* dw, int op) {
  __shared__ Smem S;
  if (!wide_enter(S, dw)) return;
  if (op == 0) {
    WIDE_LOOP(i, S.P.nb) wake_body(S.W, i);
    WIDE_LOOP(k, S.P.ncons) constraint_geom(S.W, k);
  } else {
    WIDE_LOOP(i, S.P.nb) solve_prep_body(S.W, S.P, i);
  }
}

__global__ void k_w_assemble(const DWorld* dw, double h) {
  __shared__ Smem S;
  if (!wide_enter(S, dw)) return;
  const DWorld& W = S.W;
  const DWide* x = W.wide;
  const int nc = x->n_contacts, nF = x->n_fric, ncand = x->n_cand, nrows = x->n_rows;
  WIDE_LOOP(t, nc + S.P.ncons) {
    if (t < nc) assemble_contact_rows(W, S.P, t, nF, ncand, nrows, h);
    else assemble_constraint_rows(W, t - nc, nF + nc, ncand, nrows, h);
  }
}

// dependency levels and the level-ordered sweep arrays: one block
__global__ void __launch_bounds__(1024) k_w_levels(const DWorld* dw, int last_cap) {
  __shared__ Smem S;
  extern __shared__ int2 s_dyn[];
  if (!wide_enter(S, dw)) return;
  if (threadIdx.x == 0) S.n_rows = S.W.wide->n_rows;
  __syncthreads();
  if (S.n_rows == 0) return;
  ph_levels(S, (int*)(s_dyn + CP_LEVEL_CHUNK), last_cap, s_dyn);
  if (threadIdx.x == 0) S.W.wide->n_levels = S.n_levels;
}

// ---------------------------------------------------------------------------
// GSSolver sweeps (gs_solver.dart:122-155) of one world on one block.
//
// Thread t takes, in every sweep, the same rows: offset t of each level, or
// with a level of at most half a block, one body's half of a row (side 0:
// bi, side 1: bj, in neighbouring warps; the halves of G*Wlambda meet in
// shared memory).  Its first row record of the next level is loaded during
// the current one, so the level's path holds the binary64 arithmetic, the
// shared-memory vlambda / wlambda and the barriers.

// vlambda (x, y, z), wlambda (x, y, z) of body i at vel[6 i]; the solve
// flag at flg[i]
DI void wv_load(const float* vel, const unsigned char* flg, int i, float4& v, float4& w) {
  const float* p = vel + 6 * i;
  v = make_float4(p[0], p[1], p[2], flg[i] ? 1.f : 0.f);
  w = make_float4(p[3], p[4], p[5], 0.f);
}
DI void wv_store(float* vel, int i, float4 v, float4 w) {
  float* p = vel + 6 * i;
  p[0] = v.x; p[1] = v.y; p[2] = v.z;
  p[3] = w.x; p[4] = w.y; p[5] = w.z;
}
// update_a / update_b of cp_phases.cuh on the packed layout
DI void wv_update_a(float* vel, int i, float4 v, float4 w, const RowRec& R, double dl) {
  wv_store(vel, i, vstep(v, R.im.x * dl, R.j0.x, R.j0.y, R.j0.z), vstep(w, dl, R.j3.x, R.j3.y, R.j3.z));
}
DI void wv_update_b(float* vel, int i, float4 v, float4 w, const RowRec& R, double dl) {
  wv_store(vel, i, vstep(v, R.im.y * dl, R.j1.z, R.j1.w, R.j2.x), vstep(w, dl, R.j3.w, R.j4.x, R.j4.y));
}

DI bool wide_ok(DWide* x, int code, int idx, int bound) {
  if ((unsigned)idx < (unsigned)bound) return true;
  if (atomicCAS(&x->check[0], 0, code) == 0) {
    x->check[1] = idx;
    x->check[2] = bound;
  }
  return false;
}

#define WS_THREADS 256  // 186 registers a thread, no spills
#define WS_LEVELS_SMEM 4096  // level bounds kept in shared memory up to this many levels
#define CP_SCHED_SMEM (200 * 1024)  // dynamic shared memory of k_w_sched

// dynamic shared memory: level bounds (WS_LEVELS_SMEM + 1 ints), then, when
// smem_vel, the packed vlambda / wlambda (6 floats per body) and flags
__global__ void __launch_bounds__(WS_THREADS, 1) k_w_solve(const DWorld* dw, int smem_vel) {
  __shared__ Smem S;
  __shared__ double s_gx[WS_THREADS];
  __shared__ int s_ax[WS_THREADS];
  __shared__ int s_conv;
  extern __shared__ int s_ls[];
  if (!wide_enter(S, dw)) return;
  const DWorld& W = S.W;
  DWide* x = W.wide;
  const int nrows = x->n_rows, nl = x->n_levels, nb = S.P.nb;
  if (nrows == 0 || x->sched) return;  // no rows, or the slot-scheduled sweeps ran
  const bool ls_smem = nl + 1 <= WS_LEVELS_SMEM + 1;
  const int* ls = ls_smem ? s_ls : W.level_start;
  float* vel = smem_vel ? (float*)(s_ls + WS_LEVELS_SMEM + 1) : W.wvel;
  unsigned char* flg = smem_vel ? (unsigned char*)(vel + 6 * nb) : W.wflag;
  if (ls_smem)
    for (int l = threadIdx.x; l <= nl; l += BT) s_ls[l] = W.level_start[l];
  for (int i = threadIdx.x; i < nb; i += BT) {
    const float4 v = *(const float4*)W.bscr[i].vl, w = *(const float4*)W.bscr[i].wl;
    wv_store(vel, i, v, w);
    flg[i] = v.w != 0.f;
  }
  __syncthreads();
  const int half = BT >> 1;
  const int cap = W.sw_cap;
  // a level of at most `half` rows is split: the two sides of a row are in
  // neighbouring warps (side = warp & 1), which the scheduler places on
  // different sub-partitions, so their binary64 instructions issue in
  // parallel; the partner of thread t is t ^ 32
  const int split_side = (threadIdx.x >> 5) & 1;
  const int split_off = (((int)threadIdx.x >> 6) << 5) | ((int)threadIdx.x & 31);
  const int partner = threadIdx.x ^ 32;
  int iters = S.P.iterations;
  for (int sweep = 0; sweep < S.P.iterations; sweep++) {
    double acc = 0.0;
    // this thread's first row of level l
    auto first_row = [&](int l, int& p) {
      const int b = ls[l], cnt = ls[l + 1] - b;
      const int off = cnt <= half ? split_off : (int)threadIdx.x;
      p = off < cnt ? b + off : -1;
    };
    int pn;
    first_row(0, pn);
    RowRec Rn;
    int2 bbn = make_int2(0, 0);
    int rn = -1;
    if (pn >= 0 && wide_ok(x, 1, pn, nrows)) {
      Rn = load_row(W, pn);
      bbn = W.sw_b[pn];
      rn = W.sw_orig[pn];
    } else {
      pn = -1;
    }
    for (int l = 0; l < nl; l++) {
      const int b = ls[l], cnt = ls[l + 1] - b;
      const int pc = pn;
      const RowRec Rc = Rn;
      const int2 bbc = bbn;
      const int rc = rn;
      if (l + 1 < nl) {
        first_row(l + 1, pn);
        if (pn >= 0 && wide_ok(x, 1, pn, nrows)) {
          Rn = load_row(W, pn);
          bbn = W.sw_b[pn];
          rn = W.sw_orig[pn];
        } else {
          pn = -1;
        }
      }
      if (cnt <= half) {
        const int side = split_side;
        const bool mine = pc >= 0 && wide_ok(x, 2, bbc.x, nb) && wide_ok(x, 2, bbc.y, nb);
        const int me = side ? bbc.y : bbc.x;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f), w = v;
        bool act = false;
        double g = 0.0;
        if (mine) {
          wv_load(vel, flg, me, v, w);
          act = v.w != 0.f;
          if (act) g = side ? half_b(Rc, v, w) : half_a(Rc, v, w);
        }
        s_gx[threadIdx.x] = g;
        s_ax[threadIdx.x] = act;
        __syncthreads();
        if (mine) {
          const double go = s_gx[partner];
          const bool ao = s_ax[partner] != 0;
          const double dl = side ? row_dl(Rc, go, ao, g, act) : row_dl(Rc, g, act, go, ao);
          const bool same = bbc.x == bbc.y;
          if (side == 0) {
            W.sw_d[cap + pc].y = Rc.d1.y + dl;
            if (act) wv_update_a(vel, me, v, w, Rc, dl);
            if (same && ao) {  // the same body, after its first update
              float4 v2, w2;
              wv_load(vel, flg, me, v2, w2);
              wv_update_b(vel, me, v2, w2, Rc, dl);
            }
            const int r = rc;
            if (wide_ok(x, 3, r, nrows)) {
              const double a = dl > 0.0 ? dl : -dl;
              W.absdl[r] = a;
              acc += a;
            }
          } else if (act && !same) {
            wv_update_b(vel, me, v, w, Rc, dl);
          }
        }
      } else {
        for (int off = threadIdx.x; off < cnt; off += BT) {
          RowRec R;
          int2 bb;
          int p, r;
          if (off == (int)threadIdx.x) {
            if (pc < 0) continue;
            R = Rc;
            bb = bbc;
            p = pc;
            r = rc;
          } else {
            p = b + off;
            if (!wide_ok(x, 1, p, nrows)) continue;
            R = load_row(W, p);
            bb = W.sw_b[p];
            r = W.sw_orig[p];
          }
          if (!wide_ok(x, 2, bb.x, nb) || !wide_ok(x, 2, bb.y, nb)) continue;
          float4 va, wa, vb, wb;
          wv_load(vel, flg, bb.x, va, wa);
          wv_load(vel, flg, bb.y, vb, wb);
          const bool aa = va.w != 0.f, ab = vb.w != 0.f;
          const double ga = aa ? half_a(R, va, wa) : 0.0;
          const double gb = ab ? half_b(R, vb, wb) : 0.0;
          const double dl = row_dl(R, ga, aa, gb, ab);
          W.sw_d[cap + p].y = R.d1.y + dl;
          if (aa) wv_update_a(vel, bb.x, va, wa, R, dl);
          if (ab) {
            if (bb.x == bb.y) wv_load(vel, flg, bb.y, vb, wb);  // a constraint between a body and itself
            wv_update_b(vel, bb.y, vb, wb, R, dl);
          }
          if (wide_ok(x, 3, r, nrows)) {
            const double a = dl > 0.0 ? dl : -dl;
            W.absdl[r] = a;
            acc += a;
          }
        }
      }
      __syncthreads();
    }
    // (sum of |dlambda| in row order)^2 < tol^2, with the order-free block
    // sum deciding unless it lies within the rounding band of the threshold
    const double sp = block_sum(S, acc);
    if (threadIdx.x == 0) {
      const double tol2 = S.P.tolerance * S.P.tolerance;
      const double band = 2.2 * (double)nrows * 1.1102230246251565e-16;
      const double hi = sp * (1.0 + band), lo = sp * (1.0 - band);
      int conv;
      if (hi * hi * (1.0 + 4.5e-16) < tol2) conv = 1;
      else if (lo * lo * (1.0 - 4.5e-16) >= tol2 && lo >= 0.0) conv = 0;
      else {
        double t = 0.0;
        for (int r = 0; r < nrows; r++) t += W.absdl[r];
        conv = t * t < tol2;
      }
      s_conv = conv;
    }
    __syncthreads();
    if (s_conv) {
      iters = sweep;
      break;
    }
  }
  for (int i = threadIdx.x; i < nb; i += BT) {
    float4 v, w;
    wv_load(vel, flg, i, v, w);
    *(float4*)W.bscr[i].vl = v;
    float4* gw = (float4*)W.bscr[i].wl;
    *gw = make_float4(w.x, w.y, w.z, gw->w);
  }
  if (threadIdx.x == 0) {
    x->iters = iters;
    x->early = iters + 1 < S.P.iterations;
  }
}

// ---------------------------------------------------------------------------
// Slot-scheduled sweeps.  GSSolver.solve runs its rows in order, sweep after
// sweep, and an instance (sweep s, row p) reads only what the instances
// before it that touch one of its active bodies wrote, and its own row's
// lambda from sweep s - 1.  k_w_sched gives every instance the earliest slot
// after those (the rows of sweep 0 fall in their own dependency levels; a
// later sweep starts on a body as soon as that body's rows of the sweep
// before are done) and lists the instances by slot; k_w_solve_sched runs the
// slots in order, one barrier apart, all rows of a slot in parallel.  Each
// body and each row sees its updates in the reference's order, so every
// lambda and vlambda / wlambda is the level-by-level sweeps' bit for bit,
// in fewer barrier-separated steps (a 4,096-box pile: about a quarter).
// Every sweep runs; the exit test of each sweep is evaluated afterwards, in
// order, and when sweep s* passes it before the last sweep, the lambdas and
// the vlambda / wlambda of every touched body are set back to their values
// after s* (lambdas are kept per sweep; a body's vlambda / wlambda are saved
// before its first instance of each sweep).  A world whose last solve
// stopped early keeps the level-by-level sweeps, which stop without the
// extra work.

DI int block_max_int(Smem& S, int v) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
  if (lane == 0) S.warp[wid] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    int m = S.warp[0];
    for (int w = 1; w < (int)NWARP; w++) m = max(m, S.warp[w]);
    S.warp[0] = m;
  }
  __syncthreads();
  const int m = S.warp[0];
  __syncthreads();
  return m;
}

// The slots are found by one warp over shared memory: per row its bodies and
// bits packed in one word and the slot of its instance one sweep earlier (16
// bits), per body the slot and sweep of its last instance, and the level
// bounds; a __syncwarp separates the levels.  A world whose tables do not fit
// (sched_fits) keeps the level-by-level sweeps.  The other warps then sort
// the instances by slot.
DI bool sched_fits(int nb, int nrows, int nl, int iters) {
  return nb < (1 << 14) && (long long)iters * nl < 65535 && nl + 1 <= WS_LEVELS_SMEM + 1 &&
         (size_t)nrows * 6 + (size_t)nb * 8 + sizeof(int) * (WS_LEVELS_SMEM + 1) <= CP_SCHED_SMEM;
}

__global__ void __launch_bounds__(1024, 1) k_w_sched(const DWorld* dw) {
  __shared__ Smem S;
  extern __shared__ int s_sd[];
  if (!wide_enter(S, dw)) return;
  const DWorld& W = S.W;
  DWide* x = W.wide;
  const DSched& D = W.sched;
  const int nrows = x->n_rows, nl = x->n_levels, nb = S.P.nb, iters = S.P.iterations;
  const bool use = nrows > 0 && nl > 0 && iters > 0 && D.rows >= nrows && D.iters == iters && D.nb >= nb &&
                   sched_fits(nb, nrows, nl, iters) && D.mode >= 0 && (D.mode == 1 || (!x->early && x->slow == 0));
  __syncthreads();  // every thread has read x->early and x->slow before they change
  if (threadIdx.x == 0) {
    x->sched = use ? 1 : 0;
    if (x->slow > 0) x->slow--;
  }
  if (!use) return;
  int* ls = s_sd;                                  // level bounds
  int* bt = ls + WS_LEVELS_SMEM + 1;               // per body: slot of its last instance
  int* bs = bt + nb;                               // per body: sweep of its last instance
  unsigned* rp = (unsigned*)(bs + nb);             // per row: bi | bj << 14 | bits << 28
  unsigned short* tp = (unsigned short*)(rp + nrows);  // per row: slot of its last instance
  for (int l = threadIdx.x; l <= nl; l += BT) ls[l] = W.level_start[l];
  for (int b = threadIdx.x; b < nb; b += BT) {
    bt[b] = -1;
    bs[b] = -1;
  }
  // bits: 1 / 2 bi / bj take velocity updates, 4 the bodies pass the index check
  for (int p = threadIdx.x; p < nrows; p += BT) {
    const int2 bb = W.sw_b[p];
    unsigned a = 0;
    if (wide_ok(x, 9, bb.x, nb) && wide_ok(x, 9, bb.y, nb))
      a = ((4u | (W.bscr[bb.x].vl[3] != 0.f ? 1u : 0u) | (W.bscr[bb.y].vl[3] != 0.f ? 2u : 0u)) << 28) | (unsigned)bb.x |
          ((unsigned)bb.y << 14);
    rp[p] = a;
  }
  __syncthreads();
  int tmax = 0;
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    bool ok = true;
    for (int l = 0; l < nl; l++) ok = ok && ls[l] >= 0 && ls[l] <= ls[l + 1] && ls[l + 1] <= nrows;
    for (int s = 0; s < iters && ok; s++) {
      for (int l = 0; l < nl; l++) {
        const int b1 = ls[l + 1];
        for (int p = ls[l] + lane; p < b1; p += 32) {
          const int i = s * nrows + p;
          const unsigned a = rp[p];
          if (!(a & (4u << 28))) {
            D.slot[i] = -1;
            continue;
          }
          const int bx = a & 0x3fff, by = (a >> 14) & 0x3fff;
          const bool fa = a & (1u << 28), fb = a & (2u << 28);
          int t = s > 0 ? (int)tp[p] + 1 : 0;
          if (fa) t = max(t, bt[bx] + 1);
          if (fb) t = max(t, bt[by] + 1);
          const int f = (fa && bs[bx] != s ? 1 : 0) | (fb && bs[by] != s ? 2 : 0);
          D.slot[i] = t;
          D.first[i] = (unsigned char)f;
          tp[p] = (unsigned short)t;
          // the rows of a level share no active body: no two lanes write one
          if (fa) { bt[bx] = t; bs[bx] = s; }
          if (fb) { bt[by] = t; bs[by] = s; }
          tmax = max(tmax, t);
        }
        __syncwarp();
      }
    }
  }
  __syncthreads();
  // which bodies the rows touch (the restore after an early exit reads it)
  for (int b = threadIdx.x; b < nb; b += BT) D.body_s[b] = bs[b];
  const int nslots = block_max_int(S, tmax) + 1;
  const int ninst = iters * nrows;
  if (threadIdx.x == 0) {
    x->n_slots = nslots;
    // a schedule that saves less than two thirds of the level steps costs
    // more than it saves: the next 64 steps take the level-by-level sweeps
    x->slow = 3LL * nslots > (long long)iters * nl ? 64 : 0;
  }
  // counting sort of the instances by slot: ends[t] counts slot t, then
  // holds its start, then (after the scatter) its end
  int* ends = D.ends;
  for (int t = threadIdx.x; t < nslots; t += BT) ends[t] = 0;
  __syncthreads();
  for (int i = threadIdx.x; i < ninst; i += BT) {
    const int t = D.slot[i];
    if (t >= 0 && wide_ok(x, 10, t, nslots)) atomicAdd(&ends[t], 1);
  }
  __syncthreads();
  block_scan_array(S, ends, nslots);
  for (int i = threadIdx.x; i < ninst; i += BT) {
    const int t = D.slot[i];
    if (t >= 0 && t < nslots) D.items[atomicAdd(&ends[t], 1)] = i;
  }
}

DI void ckpt_store(const DSched& D, int s, int b, float4 v, float4 w) {
  float* c = D.ckpt + ((size_t)s * D.nb + b) * 6;
  c[0] = v.x; c[1] = v.y; c[2] = v.z;
  c[3] = w.x; c[4] = w.y; c[5] = w.z;
}

// dynamic shared memory as k_w_solve's (the level bounds' room is unused)
__global__ void __launch_bounds__(WS_THREADS, 1) k_w_solve_sched(const DWorld* dw, int smem_vel) {
  __shared__ Smem S;
  __shared__ int s_conv;
  extern __shared__ int s_ls[];
  if (!wide_enter(S, dw)) return;
  const DWorld& W = S.W;
  DWide* x = W.wide;
  if (!x->sched) return;
  const DSched& D = W.sched;
  const int nrows = x->n_rows, nb = S.P.nb, iters = S.P.iterations, nslots = x->n_slots;
  const int ninst = iters * nrows;
  float* vel = smem_vel ? (float*)(s_ls + WS_LEVELS_SMEM + 1) : W.wvel;
  unsigned char* flg = smem_vel ? (unsigned char*)(vel + 6 * nb) : W.wflag;
  for (int i = threadIdx.x; i < nb; i += BT) {
    const float4 v = *(const float4*)W.bscr[i].vl, w = *(const float4*)W.bscr[i].wl;
    wv_store(vel, i, v, w);
    flg[i] = v.w != 0.f;
  }
  __syncthreads();
  const int cap = W.sw_cap;
  // the thread's first instance of the next slot and its record, loaded
  // while the current slot runs: the instance at the slot's start, the
  // record after the slot's rows.  Its row's lambda from the sweep before
  // is loaded with it when that instance ran two or more slots earlier
  // (its value is final then), else after the barrier.
  auto first_item = [&](int t) -> int {
    if (t >= nslots) return -1;
    const int k = (t > 0 ? D.ends[t - 1] : 0) + (int)threadIdx.x;
    return k < D.ends[t] && k < ninst ? D.items[k] : -1;
  };
  int in_ = first_item(0), fln = 0, rn = 0, tpn = -1;
  double lamn = 0.0;
  RowRec Rn;
  int2 bbn = make_int2(0, 0);
  // t: the slot the fetched instance runs in (loads made during slot t - 1)
  auto fetch = [&](int t) {
    if (in_ < 0 || in_ >= ninst) {
      in_ = -1;
      return;
    }
    const int p = in_ % nrows;
    Rn = load_row(W, p);
    bbn = W.sw_b[p];
    rn = W.sw_orig[p];
    fln = D.first[in_];
    tpn = in_ >= nrows ? D.slot[in_ - nrows] : -1;
    lamn = in_ >= nrows ? D.lam[in_ - nrows] : Rn.d1.y;
    (void)t;
  };
  fetch(0);
  for (int t = 0; t < nslots; t++) {
    const int b = t > 0 ? D.ends[t - 1] : 0, e = D.ends[t];
    const int ic = in_, flc = fln, rc = rn, tpc = tpn;
    const double lamc = lamn;
    const RowRec Rc = Rn;
    const int2 bbc = bbn;
    in_ = first_item(t + 1);
    for (int k = b + (int)threadIdx.x; k < e; k += BT) {
      if (!wide_ok(x, 11, k, ninst)) break;
      const bool first = k == b + (int)threadIdx.x;
      const int i = first ? ic : D.items[k];
      if (!wide_ok(x, 11, i, ninst)) continue;
      const int s = i / nrows, p = i - s * nrows;
      RowRec R = first ? Rc : load_row(W, p);
      const int2 bb = first ? bbc : W.sw_b[p];
      const int r = first ? rc : W.sw_orig[p];
      if (!wide_ok(x, 2, bb.x, nb) || !wide_ok(x, 2, bb.y, nb) || !wide_ok(x, 3, r, nrows)) continue;
      // the prefetched lambda holds when its instance ran before slot t - 1
      const double lam0 = s == 0 ? R.d1.y : (first && tpc >= 0 && tpc + 2 <= t ? lamc : D.lam[i - nrows]);
      R.d1.y = lam0;
      const int fl = first ? flc : D.first[i];
      float4 va, wa, vb, wb;
      wv_load(vel, flg, bb.x, va, wa);
      wv_load(vel, flg, bb.y, vb, wb);
      if (fl & 1) ckpt_store(D, s, bb.x, va, wa);
      if ((fl & 2) && bb.y != bb.x) ckpt_store(D, s, bb.y, vb, wb);
      const bool aa = va.w != 0.f, ab = vb.w != 0.f;
      const double ga = aa ? half_a(R, va, wa) : 0.0;
      const double gb = ab ? half_b(R, vb, wb) : 0.0;
      const double dl = row_dl(R, ga, aa, gb, ab);
      D.lam[i] = lam0 + dl;
      if (aa) wv_update_a(vel, bb.x, va, wa, R, dl);
      if (ab) {
        if (bb.x == bb.y) wv_load(vel, flg, bb.y, vb, wb);  // a constraint between a body and itself
        wv_update_b(vel, bb.y, vb, wb, R, dl);
      }
      D.absdl[(size_t)s * nrows + r] = dl > 0.0 ? dl : -dl;
    }
    fetch(t + 1);
    __syncthreads();
  }
  // the exit test of each sweep, in order: (sum of |dlambda| in row order)^2
  // < tol^2, the order-free sum deciding outside the rounding band
  int sconv = -1;
  for (int s = 0; s < iters; s++) {
    const double* ad = D.absdl + (size_t)s * nrows;
    double part = 0.0;
    for (int r = threadIdx.x; r < nrows; r += BT) part += ad[r];
    const double sp = block_sum(S, part);
    if (threadIdx.x == 0) {
      const double tol2 = S.P.tolerance * S.P.tolerance;
      const double band = 2.2 * (double)nrows * 1.1102230246251565e-16;
      const double hi = sp * (1.0 + band), lo = sp * (1.0 - band);
      int conv;
      if (hi * hi * (1.0 + 4.5e-16) < tol2) conv = 1;
      else if (lo * lo * (1.0 - 4.5e-16) >= tol2 && lo >= 0.0) conv = 0;
      else {
        double tt = 0.0;
        for (int r = 0; r < nrows; r++) tt += ad[r];
        conv = tt * tt < tol2;
      }
      s_conv = conv;
    }
    __syncthreads();
    const int conv = s_conv;
    __syncthreads();
    if (conv) {
      sconv = s;
      break;
    }
  }
  const int sf = sconv >= 0 ? sconv : iters - 1;
  if (sconv >= 0 && sconv + 1 < iters) {
    // back to the state after sweep sconv: a touched body's vlambda /
    // wlambda as saved before its first instance of sweep sconv + 1
    for (int b2 = threadIdx.x; b2 < nb; b2 += BT) {
      if (D.body_s[b2] < 0) continue;
      const float* c = D.ckpt + ((size_t)(sconv + 1) * D.nb + b2) * 6;
      wv_store(vel, b2, make_float4(c[0], c[1], c[2], 0.f), make_float4(c[3], c[4], c[5], 0.f));
    }
  }
  for (int p = threadIdx.x; p < nrows; p += BT) W.sw_d[cap + p].y = D.lam[(size_t)sf * nrows + p];
  for (int r = threadIdx.x; r < nrows; r += BT) W.absdl[r] = D.absdl[(size_t)sf * nrows + r];
  __syncthreads();
  for (int i = threadIdx.x; i < nb; i += BT) {
    float4 v, w;
    wv_load(vel, flg, i, v, w);
    *(float4*)W.bscr[i].vl = v;
    float4* gw = (float4*)W.bscr[i].wl;
    *gw = make_float4(w.x, w.y, w.z, gw->w);
  }
  if (threadIdx.x == 0) {
    x->iters = sconv >= 0 ? sconv : iters;
    x->early = sconv >= 0 && sconv + 1 < iters;
  }
}

// velocity update, multipliers (gs_solver.dart:157-176), then integration
__global__ void k_w_apply(const DWorld* dw, double h) {
  __shared__ Smem S;
  if (!wide_enter(S, dw)) return;
  const int nrows = S.W.wide->n_rows;
  if (nrows == 0) return;
  const double invDt = 1 / h;
  WIDE_LOOP(i, S.P.nb) apply_body(S.W, i);
  WIDE_LOOP(p, nrows) apply_row(S.W, p, invDt);
}

__global__ void k_w_integrate(const DWorld* dw, double dt) {
  __shared__ Smem S;
  if (!wide_enter(S, dw)) return;
  const DWorldParams& P = S.P;
  const bool qn = (P.stepnumber % (long long)(P.qn_skip + 1)) == 0;
  WIDE_LOOP(i, P.nb) integrate_body(S.W, P, i, dt, qn, P.time);
}

// ---------------------------------------------------------------------------
// host side

static int g_wide_grid[CP_MAX_DEVICES];

// grid of the item kernels: every SM busy several times over
static int wide_grid() {
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= CP_MAX_DEVICES) dev = 0;
  if (!g_wide_grid[dev]) {
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    g_wide_grid[dev] = (sms > 0 ? sms : 1) * 8;
  }
  return g_wide_grid[dev];
}

static size_t solve_smem_bytes(int nb, bool vel) {
  return sizeof(int) * (WS_LEVELS_SMEM + 1) + (vel ? (size_t)nb * (6 * sizeof(float) + 1) : 0);
}

// the sweep kernel's own (static) shared memory, as compiled
static int solve_static_smem() {
  cudaFuncAttributes fa;
  if (cudaFuncGetAttributes(&fa, (const void*)k_w_solve) != cudaSuccess) return 1 << 20;
  return (int)fa.sharedSizeBytes;
}

int cpk_wide_smem_vel_max() {
  int dev = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const long long room = (long long)optin - solve_static_smem() - (long long)sizeof(int) * (WS_LEVELS_SMEM + 1);
  return room > 0 ? (int)(room / (6 * sizeof(float) + 1)) : 0;
}

#define WIDE_LAUNCH(k, grid, threads, smem, ...)       \
  do {                                                 \
    k<<<(grid), (threads), (smem), st>>>(__VA_ARGS__); \
    cudaError_t e_ = cudaGetLastError();               \
    if (e_ != cudaSuccess) return e_;                  \
    n++;                                               \
  } while (0)
#define WIDE_SCAN(a, n_ptr, out, out2, cap, bit)                                \
  do {                                                                          \
    cudaError_t e_ = wide_scan(dw, (a), (n_ptr), (out), (out2), (cap), (bit), st); \
    if (e_ != cudaSuccess) return e_;                                           \
    n += 2;                                                                     \
  } while (0)

static cudaError_t wide_step(const DWorld* dw, const DWorld& hw, const WideShape& ws, double dt, double time_inc,
                             cudaStream_t st, long long& n) {
  const int G = wide_grid();
  const int nb = ws.nb;
  const int gb = std::max(1, std::min(G, (nb + WT - 1) / WT));  // grids over bodies
  DWide* x = hw.wide;
  DWorldParams* P = hw.P;
  WIDE_LAUNCH(k_w_begin, 1, 32, 0, dw);
  WIDE_LAUNCH(k_w_prepare, gb, WT, 0, dw);
  // broadphase: n_pairs pairs in pair_a / pair_b
  if (ws.broadphase == CP_BROAD_SAP) {
    WIDE_LAUNCH(k_w_sap_key, gb, WT, 0, dw);
    WIDE_LAUNCH(k_w_sap_rank, gb, WT, 0, dw);
    WIDE_LAUNCH(k_w_sap_copy, gb, WT, 0, dw);
    const int gw = std::max(1, std::min(G, (nb * 32 + WT - 1) / WT));  // one warp per list position
    WIDE_LAUNCH(k_w_sap_pairs, gw, WT, 0, dw, 0);
    WIDE_SCAN(hw.pair_cnt, &P->nb, &x->n_cand_pairs, &x->n_pairs, ws.pairs_cap, ST_PAIRS_OVERFLOW);
    WIDE_LAUNCH(k_w_sap_pairs, gw, WT, 0, dw, 1);
  } else if (ws.broadphase == CP_BROAD_GRID) {
    const int gbin = std::max(1, std::min(G, (ws.nbins + WT - 1) / WT));
    WIDE_LAUNCH(k_w_grid_zero, gbin, WT, 0, dw);
    WIDE_LAUNCH(k_w_grid_bin, gb, WT, 0, dw, 0);
    WIDE_LAUNCH(k_w_grid_planes, 1, 1024, 0, dw, 0);
    WIDE_SCAN(hw.bin_cnt, &P->nbins, &x->total, nullptr, ws.bins_cap, ST_BINS_OVERFLOW);
    WIDE_LAUNCH(k_w_grid_starts, gbin, WT, 0, dw);
    WIDE_LAUNCH(k_w_grid_bin, gb, WT, 0, dw, 1);
    WIDE_LAUNCH(k_w_grid_planes, 1, 1024, 0, dw, 1);
    WIDE_LAUNCH(k_w_grid_sort, gbin, WT, 0, dw);
    WIDE_LAUNCH(k_w_grid_pairs, gbin, WT, 0, dw, 0);
    WIDE_SCAN(hw.bin_cnt, &P->nbins, &x->n_cand_pairs, nullptr, -1, 0);
    WIDE_LAUNCH(k_w_grid_check, 1, 1, 0, dw);
    WIDE_LAUNCH(k_w_grid_pairs, gbin, WT, 0, dw, 1);
    WIDE_LAUNCH(k_w_hash, G, WT, 0, dw, 0);
    WIDE_LAUNCH(k_w_hash, G, WT, 0, dw, 1);
    WIDE_LAUNCH(k_w_hash, G, WT, 0, dw, 2);
    WIDE_SCAN(hw.pair_cnt, &x->n_cand_pairs, &x->n_pairs, nullptr, -1, 0);
    WIDE_LAUNCH(k_w_compact, G, WT, 0, dw);
  } else {
    WIDE_LAUNCH(k_w_naive, CP_WIDE_SCAN_BLOCKS, WT, 0, dw, 0);
    WIDE_LAUNCH(k_w_naive_scan, 1, 1024, 0, dw, CP_WIDE_SCAN_BLOCKS);
    WIDE_LAUNCH(k_w_naive, CP_WIDE_SCAN_BLOCKS, WT, 0, dw, 1);
  }
  if (ws.n_nocollide > 0) {
    WIDE_LAUNCH(k_w_nocollide, G, WT, 0, dw);
    WIDE_SCAN(hw.pair_cnt, &x->n_cand_pairs, &x->n_pairs, nullptr, -1, 0);
    WIDE_LAUNCH(k_w_compact, G, WT, 0, dw);
  }
  // narrowphase: contacts in job order (pair order; shape pairs within a
  // pair for compound bodies)
  if (ws.compound) {
    WIDE_LAUNCH(k_w_jobs, G, WT, 0, dw, 0);
    WIDE_SCAN(hw.pair_cnt, &x->n_pairs, &x->n_jobs, nullptr, ws.jobs_cap, ST_JOBS_OVERFLOW);
    WIDE_LAUNCH(k_w_jobs, G, WT, 0, dw, 1);
  }
  WIDE_LAUNCH(k_w_narrow_first, G, WT, 0, dw);
  WIDE_LAUNCH(k_w_kind_count, G, WT, 0, dw);
  WIDE_LAUNCH(k_w_kind_pos, 1, 1, 0, dw);
  WIDE_LAUNCH(k_w_kind_fill, G, WT, 0, dw);
  WIDE_LAUNCH(k_w_kind_scatter, G, WT, 0, dw);
  WIDE_LAUNCH(k_w_stage1<WT>, G, WT, 0, dw);
  WIDE_LAUNCH(k_w_stage2<WT>, G, WT, 0, dw);
  WIDE_LAUNCH(k_w_contact_counts, G, WT, 0, dw);
  WIDE_SCAN(hw.heavy, ws.compound ? &x->n_jobs : &x->n_pairs, &x->n_contacts, nullptr, ws.contacts_cap,
            ST_CONTACTS_OVERFLOW);
  WIDE_LAUNCH(k_w_contact_place, G, WT, 0, dw);
  // solver rows: friction, contact, constraint candidates and the kept rows
  WIDE_LAUNCH(k_w_fric, G, WT, 0, dw);
  WIDE_SCAN(hw.cscr, &x->n_contacts, &x->n_fric, nullptr, -1, 0);
  WIDE_LAUNCH(k_w_cands, G, WT, 0, dw);
  WIDE_SCAN(hw.cand, &x->n_cand, &x->n_rows, nullptr, ws.rows_cap, ST_ROWS_OVERFLOW);
  // ---- body state changes from here on ----
  WIDE_LAUNCH(k_w_mid, 1, 1, 0, dw);
  WIDE_LAUNCH(k_w_post, G, WT, 0, dw);
  WIDE_LAUNCH(k_w_bodies, gb, WT, 0, dw, 0);
  WIDE_LAUNCH(k_w_bodies, gb, WT, 0, dw, 1);
  WIDE_LAUNCH(k_w_assemble, G, WT, 0, dw, dt);
  const int last_cap = nb < CP_SMEM_LEVEL_MAX ? nb : CP_SMEM_LEVEL_MAX;
  const size_t lsm = sizeof(int2) * CP_LEVEL_CHUNK + sizeof(int) * (size_t)last_cap;
  WIDE_LAUNCH(k_w_levels, 1, 1024, lsm, dw, last_cap);
  WIDE_LAUNCH(k_w_sched, 1, 1024, CP_SCHED_SMEM, dw);
  WIDE_LAUNCH(k_w_solve_sched, 1, WS_THREADS, solve_smem_bytes(nb, ws.smem_vel), dw, ws.smem_vel ? 1 : 0);
  WIDE_LAUNCH(k_w_solve, 1, WS_THREADS, solve_smem_bytes(nb, ws.smem_vel), dw, ws.smem_vel ? 1 : 0);
  WIDE_LAUNCH(k_w_apply, G, WT, 0, dw, dt);
  WIDE_LAUNCH(k_w_integrate, gb, WT, 0, dw, dt);
  WIDE_LAUNCH(k_w_end, 1, 1, 0, dw, time_inc);
  return cudaSuccess;
}

cudaError_t cpk_launch_wide_steps(const DWorld* dw, const DWorld& hw, const WideShape& ws, double dt, double time_inc,
                                  int nsteps, cudaStream_t st, long long* launches) {
  static bool attr_done[CP_MAX_DEVICES];
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev >= 0 && dev < CP_MAX_DEVICES && !attr_done[dev]) {
    int optin = 0;
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaError_t e = cudaFuncSetAttribute((const void*)k_w_solve, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         optin - solve_static_smem());
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute((const void*)k_w_sched, cudaFuncAttributeMaxDynamicSharedMemorySize, CP_SCHED_SMEM);
    if (e == cudaSuccess) {
      cudaFuncAttributes fa;
      e = cudaFuncGetAttributes(&fa, (const void*)k_w_solve_sched);
      if (e == cudaSuccess)
        e = cudaFuncSetAttribute((const void*)k_w_solve_sched, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 optin - (int)fa.sharedSizeBytes);
    }
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute((const void*)k_w_levels, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)(sizeof(int2) * CP_LEVEL_CHUNK + sizeof(int) * CP_SMEM_LEVEL_MAX));
    if (e != cudaSuccess) return e;
    attr_done[dev] = true;
  }
  long long n = 0;
  for (int s = 0; s < nsteps; s++) {
    cudaError_t e = wide_step(dw, hw, ws, dt, time_inc, st, n);
    if (e != cudaSuccess) return e;
  }
  if (launches) *launches += n;
  return cudaSuccess;
}

cudaError_t cpk_wide_filter_check(int on) { return cudaMemcpyToSymbol(g_filter_check, &on, sizeof(int)); }

cudaError_t cpk_wide_filter_counts(unsigned long long out[2], bool reset) {
  cudaError_t e = cudaMemcpyFromSymbol(out, g_filter_count, 2 * sizeof(unsigned long long));
  if (e == cudaSuccess && reset) {
    const unsigned long long z[2] = {0, 0};
    e = cudaMemcpyToSymbol(g_filter_count, z, sizeof(z));
  }
  return e;
}

cudaError_t cpk_wide_check(const DWorld& hw, int out[4], cudaStream_t st) {
  cudaError_t e = cudaMemcpyAsync(out, hw.wide->check, 4 * sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e == cudaSuccess && out[0] != 0) e = cudaMemsetAsync(hw.wide->check, 0, 4 * sizeof(int), st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return e;
}
