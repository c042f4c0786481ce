// cp_phases.cuh -- the phases of one World.step (lib/world/world_class.dart:
// 433-701) as device code: the per-item work (one body, one pair, one
// contact, one row) and the block-wide loops of the one-world-per-block
// kernels (cp_step.cu).  The wide kernels (cp_wide.cu), which spread one
// large world over the whole GPU, run the same per-item functions in
// grid-wide loops, so both produce the same bits.
//
// Phases, each a block-wide loop followed by __syncthreads():
//   prepare      shape world transforms, AABBs the broadphase reads
//   broadphase   Naive / SAP / Grid pair list, in the reference's order
//   narrowphase  contacts per pair (cheap shapes first, then convex-convex),
//                ordered by a scan over per-pair counts
//   rows         friction rows, contact rows, constraint rows (solver.dart
//                addEquation order and filter), wake-ups
//   solve        GSSolver: rows grouped into dependency levels so that rows of
//                one level touch disjoint dynamic bodies; each level runs in
//                parallel and the per-body update sequence is the reference's
//   integrate    damping, Body.integrate, clearForces, sleepTick
// A capacity overflow is detected before the first write to body state; the
// step then returns with a status bit set and the state untouched.
#pragma once
#include <cuda_runtime.h>

#include "cp_narrow.cuh"
#include "cp_cc.cuh"
#include "cp_types.h"

#define BT blockDim.x
#define NWARP (blockDim.x >> 5)

struct __align__(16) Smem {
  long long t_last;
  long long t_acc[CP_NUM_PHASES];
  unsigned long long r_cyc[16];
  unsigned int r_cnt[16];
  DWorld W;
  DWorldParams P;
  int warp[32];
  double dwarp[32];
  int rprof;  // g_res_profile at kernel start
  int n_pairs, n_contacts, n_queued, n_rows;
  int n_fric, n_cand, n_levels, cursor;
  int overflow, converged, wi, n_jobs;  // n_jobs: narrowphase jobs (shape pairs)
  int kcnt[16], kpos[16];  // narrowphase: heavy pairs per resolver kind, segment cursors
  int cursor2, split_e, pad2[2];  // split_e: contact equation objects the narrowphase took
  int bcnt[2][16 * 8 + 4];        // naive broadphase: per (sub-round, warp) counts, then offsets; [128]: total
  // where the narrowphase's contact cursor and overflow flag live: this
  // record's cursor / overflow for a one-block world, device memory for a
  // world spread over the grid
  int* cursor_p;
  int* overflow_p;
};

// ---------------------------------------------------------------------------
// block utilities

DI int block_excl_scan(Smem& S, int v, int& total) {
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) S.warp[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int w = lane < NWARP ? S.warp[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < NWARP) S.warp[lane] = w;
  }
  __syncthreads();
  int pre = (wid > 0 ? S.warp[wid - 1] : 0) + x - v;
  total = S.warp[NWARP - 1];
  __syncthreads();
  return pre;
}

// in-place exclusive scan of a[0..n); returns the total
DI int block_scan_array(Smem& S, int* a, int n) {
  int carry = 0;
  for (int base = 0; base < n; base += BT * 4) {
    int i0 = base + threadIdx.x * 4;
    int v[4], s = 0;
#pragma unroll
    for (int m = 0; m < 4; m++) {
      v[m] = i0 + m < n ? a[i0 + m] : 0;
      s += v[m];
    }
    int tot;
    int pre = block_excl_scan(S, s, tot);
    int run = carry + pre;
#pragma unroll
    for (int m = 0; m < 4; m++)
      if (i0 + m < n) {
        a[i0 + m] = run;
        run += v[m];
      }
    carry += tot;
  }
  // every caller reads elements written by other threads
  __syncthreads();
  return carry;
}

DI double block_sum(Smem& S, double v) {
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if (lane == 0) S.dwarp[wid] = v;
  __syncthreads();
  double t = 0;
  if (threadIdx.x == 0) {
    for (int w = 0; w < NWARP; w++) t += S.dwarp[w];
    S.dwarp[0] = t;
  }
  __syncthreads();
  t = S.dwarp[0];
  __syncthreads();
  return t;
}

// ---------------------------------------------------------------------------
// prepare

// Shape.calculateWorldAABB (sphere.dart:146-156, plane.dart:201-226,
// box.dart:149-192, convex_polyhedron.dart:663-703)
DI void shape_world_aabb(const DWorld& W, const DShape& s, f3 pos, q4 q, f3& mn, f3& mx) {
  const float INF = __int_as_float(0x7f800000);
  if (s.type == CP_SHAPE_SPHERE) {
    double r = s.radius;
    mn = mkf3(pos.x - r, pos.y - r, pos.z - r);
    mx = mkf3(pos.x + r, pos.y + r, pos.z + r);
  } else if (s.type == CP_SHAPE_PLANE) {
    f3 n = vmult(q, f3{0.f, 0.f, 1.f});
    mn = f3{-INF, -INF, -INF};
    mx = f3{INF, INF, INF};
    if (n.x == 1) mx.x = pos.x; else if (n.x == -1) mn.x = pos.x;
    if (n.y == 1) mx.y = pos.y; else if (n.y == -1) mn.y = pos.y;
    if (n.z == 1) mx.z = pos.z; else if (n.z == -1) mn.z = pos.z;
  } else if (s.type == CP_SHAPE_BOX) {
    float ex = s.he[0], ey = s.he[1], ez = s.he[2];
    const f3 c[8] = {{ex, ey, ez}, {-ex, ey, ez}, {-ex, -ey, ez}, {-ex, -ey, -ez},
                     {ex, -ey, -ez}, {ex, ey, -ez}, {-ex, ey, -ez}, {ex, -ey, ez}};
    f3 w = add(vmult(q, c[0]), pos);
    mx = w; mn = w;
    for (int i = 1; i < 8; i++) {
      w = add(vmult(q, c[i]), pos);
      if (w.x > mx.x) mx.x = w.x;
      if (w.y > mx.y) mx.y = w.y;
      if (w.z > mx.z) mx.z = w.z;
      if (w.x < mn.x) mn.x = w.x;
      if (w.y < mn.y) mn.y = w.y;
      if (w.z < mn.z) mn.z = w.z;
    }
  } else {
    const DHull H = W.hulls[s.hull];
    f3 w = add(vmult(q, hv(W, H.v0)), pos);
    mn = w; mx = w;
    for (int i = 1; i < H.nv; i++) {
      w = add(vmult(q, hv(W, H.v0 + i)), pos);
      if (w.x < mn.x) mn.x = w.x;
      if (w.x > mx.x) mx.x = w.x;
      if (w.y < mn.y) mn.y = w.y;
      if (w.y > mx.y) mx.y = w.y;
      if (w.z < mn.z) mn.z = w.z;
      if (w.z > mx.z) mx.z = w.z;
    }
  }
}

// shape world transform of body i and, where the broadphase reads it, its
// world AABB
// dart:math min / max of two doubles, here of binary32 values: a NaN
// operand wins, and -0.0 is below 0.0
DI float dart_min(float a, float b) {
  if (a > b) return b;
  if (a < b) return a;
  if (a != a || b != b) return __int_as_float(0x7fc00000);
  return (signbit(a) || signbit(b)) ? -0.0f : a;
}
DI float dart_max(float a, float b) {
  if (a < b) return b;
  if (a > b) return a;
  if (a != a || b != b) return __int_as_float(0x7fc00000);
  return (signbit(a) && signbit(b)) ? -0.0f : (a == 0.0f ? 0.0f : a);
}

DI void prepare_body(const DWorld& W, const DWorldParams& P, int i) {
  const int bp = P.broadphase;
  const bool aabb_all = bp == CP_BROAD_SAP || (bp == CP_BROAD_NAIVE && P.use_bb);
  const bool aabb_grid = bp == CP_BROAD_GRID;
  DBody& B = W.bodies[i];
  q4 q = ld4q(B.quat);
  f3 p = ld3(B.pos);
  f3 xs = add(vmult(q, ld3(B.shape_off)), p);  // getContacts :671-680, updateAABB :430-434
  q4 qs = qmul(q, ld4q(B.shape_quat));
  st3(W.bscr[i].xs, xs);
  st4q(W.bscr[i].qs, qs);
  {
    const bool ss = B.type == CP_BODY_STATIC || B.sleep_state == CP_SLEEPING;
    W.brec[i] = make_float4(p.x, p.y, p.z, ss ? -fabsf(B.brad32) : fabsf(B.brad32));
    W.bgm[i] = make_int2(B.group, B.mask);
  }
  if ((B.flags & BF_AABB_DIRTY) && B.shape >= 0) {
    const DShape s = W.shapes[B.shape];
    if (aabb_all || (aabb_grid && s.type != CP_SHAPE_SPHERE && s.type != CP_SHAPE_PLANE)) {
      f3 mn, mx;
      shape_world_aabb(W, s, xs, qs, mn, mx);
      // a compound body's AABB extends over each further shape's
      // (rigid_body.dart:415-447, AABB.extend in aabb.dart:121-128)
      for (int e = 0; e < B.nxs; e++) {
        const DBodyShape& X = W.bshapes[B.xs0 + e];
        f3 lo, hi;
        shape_world_aabb(W, W.shapes[X.shape], add(vmult(q, ld3(X.off)), p), qmul(q, ld4q(X.quat)), lo, hi);
        mn = f3{dart_min(mn.x, lo.x), dart_min(mn.y, lo.y), dart_min(mn.z, lo.z)};
        mx = f3{dart_max(mx.x, hi.x), dart_max(mx.y, hi.y), dart_max(mx.z, hi.z)};
      }
      st3(B.aabb_lo, mn);
      st3(B.aabb_hi, mx);
      B.flags &= ~BF_AABB_DIRTY;
    }
  }
}

DI void ph_prepare(Smem& S) {
  for (int i = threadIdx.x; i < S.P.nb; i += BT) prepare_body(S.W, S.P, i);
  __syncthreads();
}

// ---------------------------------------------------------------------------
// broadphase

// Broadphase.needBroadphaseCollision (broadphase.dart:44-63)
DI bool need_pair(const DBody& A, const DBody& B) {
  if ((A.group & B.mask) == 0 || (B.group & A.mask) == 0) return false;
  bool sa = A.type == CP_BODY_STATIC || A.sleep_state == CP_SLEEPING;
  bool sb = B.type == CP_BODY_STATIC || B.sleep_state == CP_SLEEPING;
  return !(sa && sb);
}

// doBoundingSphereBroadphase (broadphase.dart:77-86): |xB - xA|^2 < (rA+rB)^2
// in binary64.  A binary32 evaluation with a relative margin settles almost
// every pair; only pairs within the margin are evaluated in binary64.
DI bool sphere_overlap(const DBody& A, const DBody& B) {
  f3 r = sub(ld3(B.pos), ld3(A.pos));
  float sf = A.brad32 + B.brad32;
  float bf = sf * sf;
  if (bf < 1e30f) {
    float n2f = r.x * r.x + r.y * r.y + r.z * r.z;
    if (n2f < bf * 0.999996f) return true;
    if (n2f > bf * 1.000004f) return false;
  }
  double s = A.bounding_radius + B.bounding_radius;
  return length2(r) < s * s;
}

// AABB.overlaps (aabb.dart:131-147)
DI bool aabb_overlap(const DBody& A, const DBody& B) {
  const float *l1 = A.aabb_lo, *u1 = A.aabb_hi, *l2 = B.aabb_lo, *u2 = B.aabb_hi;
  bool ox = (l2[0] <= u1[0] && u1[0] <= u2[0]) || (l1[0] <= u2[0] && u2[0] <= u1[0]);
  bool oy = (l2[1] <= u1[1] && u1[1] <= u2[1]) || (l1[1] <= u2[1] && u2[1] <= u1[1]);
  bool oz = (l2[2] <= u1[2] && u1[2] <= u2[2]) || (l1[2] <= u2[2] && u2[2] <= u1[2]);
  return ox && oy && oz;
}

DI bool intersection_test(const DWorldParams& P, const DBody& A, const DBody& B) {
  return P.use_bb ? aabb_overlap(A, B) : sphere_overlap(A, B);
}
DI bool intersection_test(const Smem& S, const DBody& A, const DBody& B) { return intersection_test(S.P, A, B); }

// NaiveBroadphase.collisionPairs with the bounding-sphere test
// (naive_broadphase.dart:14-33, broadphase.dart:44-86) over the records of
// the prepare phase: the pair (bodies[i], bodies[j]) at flattened index
// k = i (i - 1) / 2 + j, j < i.  needBroadphaseCollision first (filter
// groups, not both static or sleeping), then |xB - xA|^2 < (rA + rB)^2 in
// binary64, settled in binary32 outside a relative band as sphere_overlap
// does.  `cur` caches body i's record between calls; `check` is the filter
// check switch, read once per phase.
struct NaiveRow {
  int cur;
  bool check;
  float4 a;
  int2 ga;
  DI void init() {
    cur = -1;
    check = g_filter_check != 0;
  }
};

DI bool naive_rec_test(const DWorld& W, int i, int j, NaiveRow& R) {
  if (i != R.cur) {
    R.a = W.brec[i];
    R.ga = W.bgm[i];
    R.cur = i;
  }
  const float4 b = W.brec[j];
  const int2 gb = W.bgm[j];
  if ((R.ga.x & gb.y) == 0 || (gb.x & R.ga.y) == 0) return false;
  if (__float_as_int(R.a.w) < 0 && __float_as_int(b.w) < 0) return false;
  const f3 r = sub(f3{b.x, b.y, b.z}, f3{R.a.x, R.a.y, R.a.z});
  const float sf = fabsf(R.a.w) + fabsf(b.w);
  const float bf = sf * sf;
  int dec = -1;  // the binary32 verdict, -1 inside the band
  if (bf < 1e30f) {
    const float n2f = r.x * r.x + r.y * r.y + r.z * r.z;
    if (n2f < bf * 0.999996f) dec = 1;
    else if (n2f > bf * 1.000004f) dec = 0;
  }
  if (dec >= 0 && !R.check) return dec;
  const double s = W.bodies[i].bounding_radius + W.bodies[j].bounding_radius;
  const bool exact = length2(r) < s * s;
  if (dec >= 0) {  // filter check: the binary32 verdict against binary64
    atomicAdd(&g_filter_count[0], 1ull);
    if ((dec == 1) != exact) atomicAdd(&g_filter_count[1], 1ull);
  }
  return exact;
}

// (i, j) of flattened index k
DI void naive_from_flat(long long k, int& i, int& j) {
  i = (int)((1.0f + sqrtf(1.0f + 8.0f * (float)k)) * 0.5f);
  while ((long long)i * (i - 1) / 2 > k) i--;
  while ((long long)(i + 1) * i / 2 <= k) i++;
  j = (int)(k - (long long)i * (i - 1) / 2);
}

// (i, j) advanced by `by` flattened positions
DI void naive_advance(int& i, int& j, int by) {
  j += by;
  while (j >= i) {
    j -= i;
    i++;
  }
}

// One block-wide tile of the triangle: thread t tests items
// k0 + m * BT + t, m < NAIVE_SUB, below kend, so that a warp reads
// consecutive records.  (i, j) is the thread's item k0 + t on entry and
// k0 + NAIVE_SUB * BT + t on return.  Returns the tile's pairs; with
// `write`, stores them in flattened order from `out` (below `cap`).  The
// offsets come from per-warp ballots and one scan of NAIVE_SUB * NWARP
// counts; two count buffers alternate, so a tile needs two barriers.
// Blocks of at most 256 threads (NAIVE_SUB * 8 warps counts).
#define NAIVE_SUB 16
DI int naive_tile(Smem& S, long long k0, long long kend, bool write, int out, int cap, int& i, int& j, NaiveRow& R,
                  int& buf) {
  const DWorld& W = S.W;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int* cnt = S.bcnt[buf];
  buf ^= 1;
  unsigned bal[NAIVE_SUB];
  int pi[NAIVE_SUB], pj[NAIVE_SUB];
#pragma unroll
  for (int m = 0; m < NAIVE_SUB; m++) {
    const long long k = k0 + (long long)m * BT + threadIdx.x;
    const bool h = k < kend && naive_rec_test(W, i, j, R);
    bal[m] = __ballot_sync(0xffffffffu, h);
    pi[m] = i;
    pj[m] = j;
    if (lane == 0) cnt[m * NWARP + wid] = __popc(bal[m]);
    naive_advance(i, j, BT);
  }
  __syncthreads();
  if (wid == 0) {  // exclusive scan of the counts in (m, warp) order: the flattened order
    const int n = NAIVE_SUB * NWARP;
    int v[4], sum = 0;
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int e = lane * 4 + q;
      v[q] = e < n ? cnt[e] : 0;
      sum += v[q];
    }
    int x = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    int ex = x - sum;
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int e = lane * 4 + q;
      if (e < n) cnt[e] = ex;
      ex += v[q];
    }
    if (lane == 31) cnt[NAIVE_SUB * 8] = x;
  }
  __syncthreads();
  if (write) {
    const unsigned below = (1u << lane) - 1u;
#pragma unroll
    for (int m = 0; m < NAIVE_SUB; m++) {
      if ((bal[m] >> lane) & 1u) {
        const int o = out + cnt[m * NWARP + wid] + __popc(bal[m] & below);
        if (o < cap) {
          W.pair_a[o] = pi[m];
          W.pair_b[o] = pj[m];
        }
      }
    }
  }
  return cnt[NAIVE_SUB * 8];
}

// The one-block form walks the triangle row by row, a warp per row i, 32
// candidates j at a time, and skips the chunks of 32 consecutive bodies
// whose sphere box lies clear of body i's sphere on some axis by a relative
// margin (bodies are usually created in spatial order, so most chunks are
// clear of a given body).  A skipped chunk holds no pair: on that axis
// xj - xi exceeds ri + rj for every body j of it by far more than the
// rounding of the binary32 difference and of the radii.  Pass 0 counts each
// row's pairs, a scan gives each row its offset, pass 1 writes them: row
// order, then j ascending, is the flattened order.

// chunk boxes (warp per chunk); a NaN coordinate or radius drops out of the
// box, which is sound because such a body never passes the sphere test
DI void naive_chunk_boxes(const DWorld& W, int nb) {
  const int lane = threadIdx.x & 31;
  const int nch = (nb + 31) >> 5;
  for (int c = threadIdx.x >> 5; c < nch; c += NWARP) {
    const int j = c * 32 + lane;
    float lx = INFINITY, ly = INFINITY, lz = INFINITY, hx = -INFINITY, hy = -INFINITY, hz = -INFINITY, rm = 0.0f;
    if (j < nb) {
      const float4 b = W.brec[j];
      const float r = fabsf(b.w);
      lx = __fsub_rd(b.x, r);
      ly = __fsub_rd(b.y, r);
      lz = __fsub_rd(b.z, r);
      hx = __fadd_ru(b.x, r);
      hy = __fadd_ru(b.y, r);
      hz = __fadd_ru(b.z, r);
      rm = r;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      lx = fminf(lx, __shfl_xor_sync(0xffffffffu, lx, o));
      ly = fminf(ly, __shfl_xor_sync(0xffffffffu, ly, o));
      lz = fminf(lz, __shfl_xor_sync(0xffffffffu, lz, o));
      hx = fmaxf(hx, __shfl_xor_sync(0xffffffffu, hx, o));
      hy = fmaxf(hy, __shfl_xor_sync(0xffffffffu, hy, o));
      hz = fmaxf(hz, __shfl_xor_sync(0xffffffffu, hz, o));
      rm = fmaxf(rm, __shfl_xor_sync(0xffffffffu, rm, o));
    }
    if (lane == 0) {
      W.cbox[2 * c] = make_float4(lx, ly, lz, 0.0f);
      W.cbox[2 * c + 1] = make_float4(hx, hy, hz, rm);
    }
  }
}

// true when body (a, |a.w|) is clear of the chunk box: on some axis the gap
// g (rounded down) beyond the box exceeds r by 1e-6 of (|g| + r + the
// chunk's largest radius), about 17 binary32 roundings
DI bool naive_chunk_clear(float4 a, float4 lo, float4 hi) {
  const float r = fabsf(a.w);
  const float m = hi.w;
  float g = __fsub_rd(lo.x, a.x);
  if (__fsub_rd(g, r) > 1e-6f * (fabsf(g) + r + m)) return true;
  g = __fsub_rd(a.x, hi.x);
  if (__fsub_rd(g, r) > 1e-6f * (fabsf(g) + r + m)) return true;
  g = __fsub_rd(lo.y, a.y);
  if (__fsub_rd(g, r) > 1e-6f * (fabsf(g) + r + m)) return true;
  g = __fsub_rd(a.y, hi.y);
  if (__fsub_rd(g, r) > 1e-6f * (fabsf(g) + r + m)) return true;
  g = __fsub_rd(lo.z, a.z);
  if (__fsub_rd(g, r) > 1e-6f * (fabsf(g) + r + m)) return true;
  g = __fsub_rd(a.z, hi.z);
  return __fsub_rd(g, r) > 1e-6f * (fabsf(g) + r + m);
}

// Row i (warp-wide): its pairs in j order; counts them, and with `write`
// stores them from `off`.  With the filter check on, skipped chunks are
// tested too: g_filter_count[0] counts them, [1] those holding a pair.
DI int naive_row(const DWorld& W, int i, NaiveRow& R, bool write, int off, int cap) {
  const int lane = threadIdx.x & 31;
  const unsigned below = (1u << lane) - 1u;
  R.a = W.brec[i];
  R.ga = W.bgm[i];
  R.cur = i;
  const int nch = (i + 31) >> 5;  // chunks holding some j < i
  int cnt = 0;
  for (int c0 = 0; c0 < nch; c0 += 32) {
    const int c = c0 + lane;
    const bool clear = c < nch && naive_chunk_clear(R.a, W.cbox[2 * c], W.cbox[2 * c + 1]);
    const unsigned skip = __ballot_sync(0xffffffffu, clear);
    unsigned todo = __ballot_sync(0xffffffffu, c < nch && (!clear || R.check));
    while (todo) {
      const int cc = __ffs(todo) - 1;
      todo &= todo - 1;
      const int j = (c0 + cc) * 32 + lane;
      const bool hit = j < i && naive_rec_test(W, i, j, R);
      const unsigned hb = __ballot_sync(0xffffffffu, hit);
      if ((skip >> cc) & 1u) {  // filter check of a skipped chunk
        if (lane == 0) {
          atomicAdd(&g_filter_count[0], 1ull);
          if (hb) atomicAdd(&g_filter_count[1], 1ull);
        }
      }
      if (write && hit) {
        const int o = off + cnt + __popc(hb & below);
        if (o < cap) {
          W.pair_a[o] = i;
          W.pair_b[o] = j;
        }
      }
      cnt += __popc(hb);
    }
  }
  return cnt;
}

DI void ph_broad_naive_spheres(Smem& S) {
  const DWorld& W = S.W;
  const int nb = S.P.nb;
  const int cap = S.P.pairs_cap;
  const int lane = threadIdx.x & 31;
  int* rows = W.sap_tmp;  // per row: pairs, then offsets (SAP's scratch; free here)
  NaiveRow R;
  R.init();
  naive_chunk_boxes(W, nb);
  __syncthreads();
  for (int i = threadIdx.x >> 5; i < nb; i += NWARP) {
    const int n = i > 0 ? naive_row(W, i, R, false, 0, 0) : 0;
    if (lane == 0) rows[i] = n;
  }
  __syncthreads();
  const int total = nb > 0 ? block_scan_array(S, rows, nb) : 0;
  if (total <= cap) {
    for (int i = 1 + (threadIdx.x >> 5); i < nb; i += NWARP) {
      const int end = i + 1 < nb ? rows[i + 1] : total;
      if (end > rows[i]) naive_row(W, i, R, true, rows[i], cap);
    }
  }
  if (threadIdx.x == 0) {
    S.n_pairs = total;
    if (total > cap) S.overflow |= ST_PAIRS_OVERFLOW;
  }
  __syncthreads();
}

// NaiveBroadphase.collisionPairs (naive_broadphase.dart:14-33): i ascending,
// j < i ascending, pair (bodies[i], bodies[j]).  With useBoundingBoxes the
// test is AABB.overlaps on the bodies' own records.
DI void ph_broad_naive(Smem& S) {
  if (!S.P.use_bb) {
    ph_broad_naive_spheres(S);
    return;
  }
  const DWorld& W = S.W;
  const int nb = S.P.nb;
  const long long T = (long long)nb * (nb - 1) / 2;
  const int cap = S.P.pairs_cap;
  int out = 0;
  for (long long tile = 0; tile < T; tile += BT * 4) {
    long long k0 = tile + (long long)threadIdx.x * 4;
    int bits = 0, cnt = 0;
    int i = 0, j = 0;
    if (k0 < T) {
      i = (int)((1.0f + sqrtf(1.0f + 8.0f * (float)k0)) * 0.5f);
      while ((long long)i * (i - 1) / 2 > k0) i--;
      while ((long long)(i + 1) * i / 2 <= k0) i++;
      j = (int)(k0 - (long long)i * (i - 1) / 2);
      int ii = i, jj = j;
      for (int m = 0; m < 4 && k0 + m < T; m++) {
        const DBody& A = W.bodies[ii];
        const DBody& B = W.bodies[jj];
        if (need_pair(A, B) && intersection_test(S, A, B)) {
          bits |= 1 << m;
          cnt++;
        }
        if (++jj == ii) { ii++; jj = 0; }
      }
    }
    int tot;
    int pre = block_excl_scan(S, cnt, tot);
    if (cnt) {
      int o = out + pre;
      int ii = i, jj = j;
      for (int m = 0; m < 4; m++) {
        if (bits & (1 << m)) {
          if (o < cap) { W.pair_a[o] = ii; W.pair_b[o] = jj; }
          o++;
        }
        if (++jj == ii) { ii++; jj = 0; }
      }
    }
    out += tot;
  }
  if (threadIdx.x == 0) {
    S.n_pairs = out;
    if (out > cap) S.overflow |= ST_PAIRS_OVERFLOW;
  }
  __syncthreads();
}

DI float axis_f(const float* v, int a) { return v[a]; }

// SAPBroadphase.checkBounds (sap_broadphase.dart:41-62) in binary64, with a
// binary32 pre-test whose error bound decides almost every call.
DI bool check_bounds(const DBody& bi, const DBody& bj, int axis) {
  float pi = bi.pos[axis], pj = bj.pos[axis];
  float ri = bi.brad32, rj = bj.brad32;
  if (fabsf(ri) < 1e30f && fabsf(rj) < 1e30f) {
    float a2 = pi + ri, b1 = pj - rj;
    float tol = 3.0e-7f * (fabsf(pi) + fabsf(ri) + fabsf(pj) + fabsf(rj)) + 1e-30f;
    if (b1 < a2 - tol) return true;
    if (b1 > a2 + tol) return false;
  }
  double boundA2 = (double)pi + bi.bounding_radius;
  double boundB1 = (double)pj - bj.bounding_radius;
  return boundB1 < boundA2;
}

// SAPBroadphase.collisionPairs' scan from list position i
// (sap_broadphase.dart:149-165): counts the pairs, or writes them from
// pair_cnt[i] on
DI int sap_scan(const DWorld& W, const DWorldParams& P, int i, bool write) {
  const int nb = P.nb, axis = P.sap_axis;
  const int ai = W.sap_order[i];
  const DBody& bi = W.bodies[ai];
  int c = 0, o = write ? W.pair_cnt[i] : 0;
  for (int j = i + 1; j < nb; j++) {
    const int aj = W.sap_order[j];
    const DBody& bj = W.bodies[aj];
    if (!need_pair(bi, bj)) continue;
    if (!check_bounds(bi, bj, axis)) break;
    if (intersection_test(P, bi, bj)) {
      if (write) {
        W.pair_a[o] = ai;
        W.pair_b[o] = aj;
        o++;
      }
      c++;
    }
  }
  return c;
}

// SAPBroadphase.sortList + collisionPairs (sap_broadphase.dart:66-79,138-189).
// The persistent axisList is re-sorted stably by aabb.lowerBound[axis]: the
// new rank of the entry at position p is #{keys < key_p} + #{q < p, key_q ==
// key_p}, which is exactly where insertion sort leaves it.
DI void ph_broad_sap(Smem& S) {
  const DWorld& W = S.W;
  const int nb = S.P.nb;
  const int axis = S.P.sap_axis;
  float* key = W.sap_key;
  for (int p = threadIdx.x; p < nb; p += BT) key[p] = W.bodies[W.sap_order[p]].aabb_lo[axis];
  __syncthreads();
  for (int p = threadIdx.x; p < nb; p += BT) {
    float kp = key[p];
    int r = 0;
    for (int q = 0; q < nb; q++) {
      float kq = key[q];
      r += (kq < kp) || (kq == kp && q < p);
    }
    W.sap_tmp[r] = W.sap_order[p];
  }
  __syncthreads();
  for (int p = threadIdx.x; p < nb; p += BT) W.sap_order[p] = W.sap_tmp[p];
  __syncthreads();
  // pass 1: pair count per list position
  for (int i = threadIdx.x; i < nb; i += BT) W.pair_cnt[i] = sap_scan(W, S.P, i, false);
  __syncthreads();
  int total = block_scan_array(S, W.pair_cnt, nb);
  const int cap = S.P.pairs_cap;
  if (total <= cap)
    for (int i = threadIdx.x; i < nb; i += BT) sap_scan(W, S.P, i, true);
  if (threadIdx.x == 0) {
    S.n_pairs = total;
    if (total > cap) S.overflow |= ST_PAIRS_OVERFLOW;
  }
  __syncthreads();
}

DI void grid_consts(const DWorldParams& P, double* c) {
  // c: xmin ymin zmin xmult ymult zmult bsx bsy bsz binRadius
  double xmax = P.grid_max[0], ymax = P.grid_max[1], zmax = P.grid_max[2];
  double xmin = P.grid_min[0], ymin = P.grid_min[1], zmin = P.grid_min[2];
  c[0] = xmin; c[1] = ymin; c[2] = zmin;
  c[3] = P.grid_nx / (xmax - xmin); c[4] = P.grid_ny / (ymax - ymin); c[5] = P.grid_nz / (zmax - zmin);
  c[6] = (xmax - xmin) / P.grid_nx; c[7] = (ymax - ymin) / P.grid_ny; c[8] = (zmax - zmin) / P.grid_nz;
  c[9] = sqrt(c[6] * c[6] + c[7] * c[7] + c[8] * c[8]) * 0.5;
}

// bin box of a non-plane body (addBoxToBins arguments); false for planes
DI bool grid_box(const DWorld& W, const DWorldParams& P, const double* c, int i, int* lo, int* hi) {
  const DBody& b = W.bodies[i];
  if (b.shape < 0) return false;
  const DShape& s = W.shapes[b.shape];
  if (s.type == CP_SHAPE_PLANE) return false;
  double a0[3], a1[3];
  if (s.type == CP_SHAPE_SPHERE) {
    double r = s.radius;
    for (int d = 0; d < 3; d++) { a0[d] = (double)b.pos[d] - r; a1[d] = (double)b.pos[d] + r; }
  } else {
    for (int d = 0; d < 3; d++) { a0[d] = b.aabb_lo[d]; a1[d] = b.aabb_hi[d]; }
  }
  const int n[3] = {P.grid_nx, P.grid_ny, P.grid_nz};
  for (int d = 0; d < 3; d++) {
    double f0 = floor((a0[d] - c[d]) * c[3 + d]);
    double f1 = ceil((a1[d] - c[d]) * c[3 + d]);
    lo[d] = f0 < 0 ? 0 : (f0 >= n[d] ? n[d] - 1 : (int)f0);
    hi[d] = f1 < 0 ? 0 : (f1 >= n[d] ? n[d] - 1 : (int)f1);
  }
  return true;
}

DI bool is_plane_body(const DWorld& W, int i) {
  int sh = W.bodies[i].shape;
  return sh >= 0 && W.shapes[sh].type == CP_SHAPE_PLANE;
}

// Bin-centre offsets d = centre - plane position for a plane body, with d
// accumulated in binary32 along the reference's loop order
// (grid_broadphase.dart:169-198): one sequence per axis.
DI void grid_plane_acc(Smem& S, const double* c, int i) {
  const DWorld& W = S.W;
  const DWorldParams& P = S.P;
  const DBody& b = W.bodies[i];
  DShape& sh = W.shapes[b.shape];
  if (threadIdx.x == 0) {
    if (!sh.plane_done) {  // Plane.computeWorldNormal runs once (plane.dart:182-187)
      st3(sh.plane_n, vmult(ld4q(b.quat), f3{0.f, 0.f, 1.f}));
      sh.plane_done = 1;
    }
    const int n[3] = {P.grid_nx, P.grid_ny, P.grid_nz};
    int off = 0;
    for (int d = 0; d < 3; d++) {
      double reset = c[d] + c[6 + d] * 0.5 - b.pos[d];
      float v = (float)reset;
      for (int k = 0; k < n[d]; k++) {
        W.bin_acc[off + k] = v;
        v = (float)(v + c[6 + d]);
      }
      off += n[d];
    }
  }
  __syncthreads();
}

DI bool grid_plane_hit(const DWorld& W, const DWorldParams& P, const double* c, int shape, int bin) {
  int xi = bin / (P.grid_ny * P.grid_nz), yi = (bin / P.grid_nz) % P.grid_ny, zi = bin % P.grid_nz;
  f3 d{W.bin_acc[xi], W.bin_acc[P.grid_nx + yi], W.bin_acc[P.grid_nx + P.grid_ny + zi]};
  return dot(d, ld3(W.shapes[shape].plane_n)) < c[9];
}

DI unsigned long long mix64(unsigned long long z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

// One body's bin memberships (addBoxToBins / addSphereToBins): pass 0
// counts them, pass 1 places the body at the bins' cursors.
DI void grid_bin_body(const DWorld& W, const DWorldParams& P, const double* c, int i, int pass) {
  int lo[3], hi[3];
  if (!grid_box(W, P, c, i, lo, hi)) return;
  const int yz = P.grid_ny * P.grid_nz;
  for (int x = lo[0]; x <= hi[0]; x++)
    for (int y = lo[1]; y <= hi[1]; y++)
      for (int z = lo[2]; z <= hi[2]; z++) {
        int bin = x * yz + y * P.grid_nz + z;
        int pos = atomicAdd(&W.bin_cnt[bin], 1);
        if (pass == 1 && pos < P.bins_cap) W.bin_body[pos] = i;
      }
}

// The plane bodies' bin memberships (the half-space test per bin), plane by
// plane in body order: the bin-centre offsets of a plane are accumulated in
// binary32 along the reference's loop order.  Block-wide; bodies are scanned
// a block at a time, so the search costs nb / blockDim loads per thread.
DI void grid_bin_planes(Smem& S, const double* c, int pass) {
  const DWorld& W = S.W;
  const DWorldParams& P = S.P;
  const int nBins = P.grid_nx * P.grid_ny * P.grid_nz;
  for (int base = 0; base < P.nb; base += BT) {
    const int i = base + threadIdx.x;
    const bool mine = i < P.nb && is_plane_body(W, i);
    if (!__syncthreads_or(mine)) continue;
    for (int t = 0; t < (int)BT && base + t < P.nb; t++) {
      if (!__syncthreads_or(mine && (int)threadIdx.x == t)) continue;
      const int pi = base + t;
      grid_plane_acc(S, c, pi);
      for (int b = threadIdx.x; b < nBins; b += BT)
        if (grid_plane_hit(W, P, c, W.bodies[pi].shape, b)) {
          int pos = atomicAdd(&W.bin_cnt[b], 1);
          if (pass == 1 && pos < P.bins_cap) W.bin_body[pos] = pi;
        }
      __syncthreads();
    }
  }
}

// bin b's bodies in body order (an insertion sort of the placed entries)
DI void grid_sort_bin(const DWorld& W, int b) {
  int s0 = W.bin_start[b], s1 = W.bin_start[b + 1];
  for (int x = s0 + 1; x < s1; x++) {
    int v = W.bin_body[x];
    int y = x - 1;
    while (y >= s0 && W.bin_body[y] > v) { W.bin_body[y + 1] = W.bin_body[y]; y--; }
    W.bin_body[y + 1] = v;
  }
}

// candidate pairs of bin b, (bin[xi], bin[yi]) for yi < xi: counted, or
// written from bin_cnt[b] on
DI int grid_bin_pairs(const DWorld& W, const DWorldParams& P, int b, bool write) {
  int s0 = W.bin_start[b], len = W.bin_start[b + 1] - s0;
  int o = write ? W.bin_cnt[b] : 0;
  int cnt = 0;
  if (len > 1)
    for (int xi = 0; xi < len; xi++) {
      int ia = W.bin_body[s0 + xi];
      for (int yi = 0; yi < xi; yi++) {
        int ib = W.bin_body[s0 + yi];
        const DBody& A = W.bodies[ia];
        const DBody& B = W.bodies[ib];
        if (need_pair(A, B) && intersection_test(P, A, B)) {
          if (write) { W.pair_a[o + cnt] = ia; W.pair_b[o + cnt] = ib; }
          cnt++;
        }
      }
    }
  return cnt;
}

// first appearance of each unordered pair: hash slot -> smallest candidate index
DI void grid_hash_clear(const DWorld& W, int h) { W.hkeys[h] = -1; W.hvals[h] = 0x7fffffff; }
DI void grid_hash_insert(const DWorld& W, int k) {
  const int hmask = W.hash_cap - 1;
  int a = W.pair_a[k], b = W.pair_b[k];
  long long key = ((long long)min(a, b) << 32) | (unsigned)max(a, b);
  int h = (int)(mix64((unsigned long long)key) & hmask);
  for (int probe = 0; probe < W.hash_cap; probe++) {
    unsigned long long prev = atomicCAS((unsigned long long*)&W.hkeys[h], 0xffffffffffffffffULL, (unsigned long long)key);
    if (prev == 0xffffffffffffffffULL || prev == (unsigned long long)key) { atomicMin(&W.hvals[h], k); break; }
    h = (h + 1) & hmask;
  }
}
// candidate k kept (its first appearance): pair_cnt[k] = 1 / 0, the pair
// saved in pair_tstart / heavy for the compaction
DI void grid_hash_keep(const DWorld& W, int k) {
  const int hmask = W.hash_cap - 1;
  int a = W.pair_a[k], b = W.pair_b[k];
  long long key = ((long long)min(a, b) << 32) | (unsigned)max(a, b);
  int h = (int)(mix64((unsigned long long)key) & hmask);
  int keep = 0;
  for (int probe = 0; probe < W.hash_cap; probe++) {
    if (W.hkeys[h] == key) { keep = W.hvals[h] == k; break; }
    h = (h + 1) & hmask;
  }
  W.pair_cnt[k] = keep;
  W.pair_tstart[k] = a;
  W.heavy[k] = b;
}
// stable compaction of the kept pairs (pair_cnt holds their exclusive scan)
DI void compact_pair(const DWorld& W, int k, int n, int kept) {
  int nxt = k + 1 < n ? W.pair_cnt[k + 1] : kept;
  if (nxt > W.pair_cnt[k]) {
    W.pair_a[W.pair_cnt[k]] = W.pair_tstart[k];
    W.pair_b[W.pair_cnt[k]] = W.heavy[k];
  }
}

// GridBroadphase.collisionPairs (grid_broadphase.dart:59-239) with per-bin
// lists, then the de-duplication broadphase.dart:105-134 intends: unique
// unordered pairs in order of first appearance.  Bins list their bodies in
// body order, so every appearance of a pair has the same orientation.
DI void ph_broad_grid(Smem& S) {
  const DWorld& W = S.W;
  const DWorldParams& P = S.P;
  const int nb = P.nb;
  const int nBins = P.grid_nx * P.grid_ny * P.grid_nz;
  double c[10];
  grid_consts(P, c);
  for (int pass = 0; pass < 2; pass++) {
    // pass 0 counts bin memberships, pass 1 places them
    if (pass == 0)
      for (int b = threadIdx.x; b < nBins; b += BT) W.bin_cnt[b] = 0;
    __syncthreads();
    for (int i = threadIdx.x; i < nb; i += BT) grid_bin_body(W, P, c, i, pass);
    grid_bin_planes(S, c, pass);
    __syncthreads();
    if (pass == 0) {
      int total = block_scan_array(S, W.bin_cnt, nBins);
      for (int b = threadIdx.x; b < nBins; b += BT) W.bin_start[b] = W.bin_cnt[b];
      if (threadIdx.x == 0) {
        W.bin_start[nBins] = total;
        if (total > P.bins_cap) S.overflow |= ST_BINS_OVERFLOW;
      }
      __syncthreads();
      if (S.overflow) return;
    }
  }
  for (int b = threadIdx.x; b < nBins; b += BT) grid_sort_bin(W, b);
  __syncthreads();
  for (int pass = 0; pass < 2; pass++) {
    for (int b = threadIdx.x; b < nBins; b += BT) {
      const int cnt = grid_bin_pairs(W, P, b, pass == 1);
      if (pass == 0) W.bin_cnt[b] = cnt;
    }
    __syncthreads();
    if (pass == 0) {
      int total = block_scan_array(S, W.bin_cnt, nBins);
      if (threadIdx.x == 0) {
        S.n_pairs = total;
        if (total > P.pairs_cap || 2 * total > W.hash_cap) S.overflow |= ST_PAIRS_OVERFLOW;
      }
      __syncthreads();
      if (S.overflow) return;
    }
  }
  const int ncand = S.n_pairs;
  for (int h = threadIdx.x; h < W.hash_cap; h += BT) grid_hash_clear(W, h);
  __syncthreads();
  for (int k = threadIdx.x; k < ncand; k += BT) grid_hash_insert(W, k);
  __syncthreads();
  for (int k = threadIdx.x; k < ncand; k += BT) grid_hash_keep(W, k);
  __syncthreads();
  int kept = block_scan_array(S, W.pair_cnt, ncand);
  for (int k = threadIdx.x; k < ncand; k += BT) compact_pair(W, k, ncand, kept);
  __syncthreads();
  if (threadIdx.x == 0) S.n_pairs = kept;
  __syncthreads();
}

// World.internalStep removes the pairs of constraints with
// collideConnected == false (world_class.dart:487-499); a stable filter.
DI void ph_nocollide(Smem& S) {
  const DWorld& W = S.W;
  const int nn = S.P.n_nocollide;
  const int np = S.n_pairs;
  for (int k = threadIdx.x; k < np; k += BT) {
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
  __syncthreads();
  int kept = block_scan_array(S, W.pair_cnt, np);
  for (int k = threadIdx.x; k < np; k += BT) {
    int nxt = k + 1 < np ? W.pair_cnt[k + 1] : kept;
    if (nxt > W.pair_cnt[k]) {
      W.pair_a[W.pair_cnt[k]] = W.pair_tstart[k];
      W.pair_b[W.pair_cnt[k]] = W.heavy[k];
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) S.n_pairs = kept;
  __syncthreads();
}

// ---------------------------------------------------------------------------
// narrowphase (narrow_phase.dart:634-721)

DI int contact_material(const DWorld& W, const DWorldParams& P, int ma, int mb) {
  if (ma < 0 || mb < 0) return -1;
  return W.cm_table[ma * P.nmat + mb];
}

// A pair with both shapes in place: the bodies, shapes and poses a resolver
// takes, in the order narrow_phase.dart:706-710 calls it.
struct PairJob {
  NarrowCtx C;
  int rsi, rsj, bA, bB, shA, shB;
  f3 xA, xB;
  q4 qA, qB;
  float U1;  // hull pairs: stage 1's bound U, or NaN
};

struct PairJob;
DI void certificate_check(Smem& S, int k, int rk, PairJob& X);
DI void just_test_overlap(Smem& S, int k, int rk, PairJob& X);

// Resolver kind of pair k and its job; RK_NONE when the pair makes no
// contact for a reason that needs no resolver (no shape, a kinematic/static
// pair, no resolver for the shape types, the collision filter, the bounding
// spheres, or a binary32 no-contact certificate).  With tests == false the
// pair is known to have passed them and only the job is filled.
// Narrowphase job `job` of a world: its broadphase pair k and the shape
// slots of the pair's two bodies (slot 0: a body's first shape); in a world
// without compound bodies the job is pair k with both first shapes.
DI void job_slots(const DWorld& W, const DWorldParams& P, int job, int& k, int& sa, int& sb) {
  if (!P.compound) {
    k = job; sa = 0; sb = 0;
    return;
  }
  k = W.job_pair[job];
  const int sh = W.job_sh[job];
  sa = sh >> 16;
  sb = sh & 0xffff;
}

// Shape `slot` of body i: its index and world pose (getContacts,
// narrow_phase.dart:671-680; slot 0's pose is the one prepare stored)
DI void slot_pose(const DWorld& W, int i, int slot, int& shape, f3& xs, q4& qs) {
  const DBody& B = W.bodies[i];
  if (slot == 0) {
    shape = B.shape;
    xs = ld3(W.bscr[i].xs);
    qs = ld4q(W.bscr[i].qs);
    return;
  }
  const DBodyShape& e = W.bshapes[B.xs0 + slot - 1];
  const q4 q = ld4q(B.quat);
  shape = e.shape;
  xs = add(vmult(q, ld3(e.off)), ld3(B.pos));
  qs = qmul(q, ld4q(e.quat));
}

DI int pair_job(Smem& S, int job, PairJob& X, bool tests) {
  const DWorld& W = S.W;
  const DWorldParams& P = S.P;
  int k, sa, sb;
  job_slots(W, P, job, k, sa, sb);
  const int i = W.pair_a[k], j = W.pair_b[k];
  const DBody& bi = W.bodies[i];
  const DBody& bj = W.bodies[j];
  bool just_test = false;
  if (tests) {
    just_test = (bi.type == CP_BODY_KINEMATIC && bj.type == CP_BODY_STATIC) ||
                (bi.type == CP_BODY_STATIC && bj.type == CP_BODY_KINEMATIC) ||
                (bi.type == CP_BODY_KINEMATIC && bj.type == CP_BODY_KINEMATIC);
    if (P.events) W.pair_flag[job] = 0;
    if (P.split) W.job_att[job] = 0;
    // a justTest pair only registers an overlap for the event feed (and, with
    // the SplitSolver, may still take an equation object, below)
    if (bi.shape < 0 || bj.shape < 0 || (just_test && !P.events && !P.split)) return RK_NONE;
  }
  int shi, shj;
  f3 xi, xj;
  q4 qi, qj;
  slot_pose(W, i, sa, shi, xi, qi);
  slot_pose(W, j, sb, shj, xj, qj);
  const DShape& si = W.shapes[shi];
  const DShape& sj = W.shapes[shj];
  const bool swap = !(si.type < sj.type);
  const int rk = swap ? resolver_kind(sj.type, si.type) : resolver_kind(si.type, sj.type);
  if (tests && rk == RK_NONE) return RK_NONE;
  if (tests && !((si.mask & sj.group) != 0 && (sj.mask & si.group) != 0)) return RK_NONE;
  if (tests && distance_to(xi, xj) > si.bsr + sj.bsr) return RK_NONE;
  // spherePlane takes its equation object before its depth test and its
  // justTest return (narrow_phase.dart:781-799): the SplitSolver's equation
  // ids count it, contact or not
  if (tests && P.split && rk == RK_SP) W.job_att[job] = 1;
  if (tests && just_test && !P.events) return RK_NONE;
  X.xA = swap ? xj : xi;
  X.xB = swap ? xi : xj;
  X.qA = swap ? qj : qi;
  X.qB = swap ? qi : qj;
  X.shA = swap ? shj : shi;
  X.shB = swap ? shi : shj;
  X.rsi = shi;
  X.rsj = shj;
  X.bA = swap ? j : i;
  X.bB = swap ? i : j;
  if (tests && just_test) {
    just_test_overlap(S, job, rk, X);
    return RK_NONE;
  }
  if (tests) {
    // binary32 no-contact certificates (see cp_narrow.cuh)
    const long long t_res = S.rprof ? clock64() : 0;
    if ((rk == RK_SP && plane_far(X.xB, X.qB, X.xA, (float)W.shapes[X.shA].radius)) ||
        ((rk == RK_PB || rk == RK_PC) && plane_far(X.xA, X.qA, X.xB, (float)W.shapes[X.shB].bsr)) ||
        (rk == RK_SB && sphere_box_far(X.xA, (float)W.shapes[X.shA].radius, X.xB, X.qB, W.shapes[X.shB].he))) {
      if (S.rprof) {
        atomicAdd(&S.r_cyc[10 + (rk == RK_SB ? 2 : (rk == RK_SP ? 0 : 1))], (unsigned long long)(clock64() - t_res));
        atomicAdd(&S.r_cnt[10 + (rk == RK_SB ? 2 : (rk == RK_SP ? 0 : 1))], 1u);
      }
      if (g_filter_check) certificate_check(S, job, rk, X);
      return RK_NONE;
    }
  }
  int cm = contact_material(W, P, si.material, sj.material);
  if (cm < 0) cm = contact_material(W, P, bi.material, bj.material);
  if (cm < 0) cm = 0;
  X.C.W = &W; X.C.cursor = S.cursor_p; X.C.cap = P.contacts_cap; X.C.overflow = S.overflow_p; X.C.cm = cm; X.C.pair = job;
  X.U1 = __int_as_float(0x7fc00000);
  return rk;
}

DI int run_resolver(Smem& S, int rk, const PairJob& X, int& start, bool prof);

// The resolver of pair k run into nothing: its contact count (it counts the
// contacts it finds and writes none)
DI int count_contacts(Smem& S, int k, int rk, PairJob& X) {
  const DWorld& W = S.W;
  X.C.W = &W; X.C.cursor = &g_filter_sink[0]; X.C.cap = 0; X.C.overflow = &g_filter_sink[1]; X.C.cm = 0; X.C.pair = k;
  X.U1 = __int_as_float(0x7fc00000);
  int start = 0;
  return run_resolver(S, rk, X, start, false);
}

// getContacts' justTest call (narrow_phase.dart:665-716): a kinematic /
// static pair makes no contact, but when its shapes overlap (the resolver
// would find a contact) the pair enters the overlap keepers that feed the
// begin / end contact events
DI void just_test_overlap(Smem& S, int k, int rk, PairJob& X) {
  S.W.pair_flag[k] = count_contacts(S, k, rk, X) > 0;
}

// Filter check of a binary32 no-contact certificate: the resolver runs with
// room for no contact (it counts them and writes none); a nonzero count
// means the reference would have found a contact.
DI void certificate_check(Smem& S, int k, int rk, PairJob& X) {
  const int n = count_contacts(S, k, rk, X);
  atomicAdd(&g_filter_count[0], 1ull);
  if (n != 0) atomicAdd(&g_filter_count[1], 1ull);
}

DI int run_resolver(Smem& S, int rk, const PairJob& X, int& start, bool prof) {
  const NarrowCtx& C = X.C;
  const long long t_res = prof ? clock64() : 0;
  int cnt;
  switch (rk) {
    case RK_SS: cnt = sphere_sphere(C, X.bA, X.bB, X.shA, X.shB, X.rsi, X.rsj, X.xA, X.xB, start); break;
    case RK_SP: cnt = sphere_plane(C, X.bA, X.bB, X.shA, X.shB, X.rsi, X.rsj, X.xA, X.xB, X.qB, start); break;
    case RK_SB: cnt = sphere_box(C, X.bA, X.bB, X.shA, X.shB, X.rsi, X.rsj, X.xA, X.xB, X.qB, start); break;
    case RK_SC: cnt = sphere_convex(C, X.bA, X.bB, X.shA, X.shB, X.rsi, X.rsj, X.xA, X.xB, X.qB, start); break;
    case RK_PB: cnt = plane_convex(C, X.bA, X.bB, X.shA, X.shB, X.shA, X.shB, X.xA, X.xB, X.qA, X.qB, start); break;
    case RK_PC: cnt = plane_convex(C, X.bA, X.bB, X.shA, X.shB, X.rsi, X.rsj, X.xA, X.xB, X.qA, X.qB, start); break;
    case RK_BB: cnt = convex_convex(C, X.bA, X.bB, X.shA, X.shB, X.shA, X.shB, X.xA, X.xB, X.qA, X.qB, start, X.U1); break;
    case RK_BC: cnt = convex_convex(C, X.bA, X.bB, X.shA, X.shB, X.shA, X.shB, X.xA, X.xB, X.qA, X.qB, start, X.U1); break;
    default: cnt = convex_convex(C, X.bA, X.bB, X.shA, X.shB, X.rsi, X.rsj, X.xA, X.xB, X.qA, X.qB, start, X.U1); break;
  }
  if (prof) {
    atomicAdd(&S.r_cyc[rk], (unsigned long long)(clock64() - t_res));
    atomicAdd(&S.r_cnt[rk], 1u);
  }
  return cnt;
}

// First pass over pair k: settles it without a resolver, or queues it under
// its resolver kind.  Queued pairs run grouped by kind, each kind's segment
// starting on a warp boundary, so a warp runs one resolver with all its lanes
// instead of interleaving several with a few lanes each (a binary64 warp
// instruction costs the same with one active lane or 32); settling first
// keeps the pairs that need no resolver out of those warps.
DI void narrow_first(Smem& S, int k, int* nq) {
  const DWorld& W = S.W;
  PairJob X;
  const int rk = pair_job(S, k, X, true);
  if (rk != RK_NONE) {
    W.heavy[atomicAdd(nq, 1)] = (int)(((unsigned)rk << 28) | (unsigned)k);  // k < 2^28
    return;
  }
  W.pair_cnt[k] = 0;
  W.pair_tstart[k] = 0;
}

// Queued pair k of kind rk (its tests passed in the first pass); U1: stage
// 1's bound for a hull pair, or NaN.
DI void narrow_queued(Smem& S, int k, int rk, float U1) {
  const DWorld& W = S.W;
  PairJob X;
  pair_job(S, k, X, false);
  X.U1 = U1;
  int start = 0;
  const int cnt = run_resolver(S, rk, X, start, S.rprof != 0);
  W.pair_cnt[k] = cnt;
  W.pair_tstart[k] = start;
}

// Entry h of the kind-sorted queue: hull pairs (kinds RK_BB and up) take
// convex_convex's cheap stage 1 and the survivors are queued again (into
// W.heavy at nq2) for the binary64 stage; other kinds run their resolver.
DI void narrow_stage1(Smem& S, int h, int* nq2) {
  const DWorld& W = S.W;
  const unsigned e = (unsigned)W.heavy2[h];  // 0xffffffff: padding (no kind 15)
  if (e == 0xffffffffu) return;
  const int k = (int)(e & 0x0FFFFFFFu), rk = (int)(e >> 28);
  if (rk >= RK_BB) {
    PairJob X;
    pair_job(S, k, X, false);
    Sat32 S32;
    float U;
    if (cc_stage1(W, X.shA, X.shB, X.xA, X.xB, X.qA, X.qB, S32, U)) {
      W.pair_tstart[k] = __float_as_int(U);  // until the binary64 stage sets it
      W.heavy[atomicAdd(nq2, 1)] = (int)e;
    } else {
      if (g_filter_check &&
          !(distance_to(X.xA, X.xB) > W.shapes[X.shA].bsr + W.shapes[X.shB].bsr))
        cc_filter_check(W, X.shA, X.shB, X.xA, X.xB, X.qA, X.qB, false, d3{0.0, 0.0, 0.0});
      W.pair_cnt[k] = 0;
      W.pair_tstart[k] = 0;
    }
  } else {
    narrow_queued(S, k, rk, __int_as_float(0x7fc00000));
  }
}

// Entry h of the binary64-stage queue
DI void narrow_stage2(Smem& S, int h) {
  const DWorld& W = S.W;
  const unsigned e = (unsigned)W.heavy[h];
  const int k = (int)(e & 0x0FFFFFFFu);
  narrow_queued(S, k, (int)(e >> 28), __int_as_float(W.pair_tstart[k]));
}

// pair k's contacts from the staging area to their place in pair order
// (heavy holds the exclusive scan of the per-pair counts)
DI void narrow_place(const DWorld& W, int k) {
  int c = W.pair_cnt[k], t = W.pair_tstart[k], o = W.heavy[k];
  for (int m = 0; m < c; m++) W.contacts[o + m] = W.ctmp[t + m];
}

// shape slots of a body (0 for a body without shapes)
DI int body_slots(const DBody& B) { return B.shape < 0 ? 0 : 1 + B.nxs; }

// jobs of broadphase pair k: one per shape of its first body times one per
// shape of its second (getContacts' two shape loops, narrow_phase.dart:654-676)
DI int pair_jobs(const DWorld& W, int k) {
  return body_slots(W.bodies[W.pair_a[k]]) * body_slots(W.bodies[W.pair_b[k]]);
}

// pair k's jobs from job o on, pair-major, first body's slot outer
DI void pair_jobs_fill(const DWorld& W, int k, int o) {
  const int na = body_slots(W.bodies[W.pair_a[k]]), nb = body_slots(W.bodies[W.pair_b[k]]);
  for (int a = 0; a < na; a++)
    for (int b = 0; b < nb; b++, o++) {
      W.job_pair[o] = k;
      W.job_sh[o] = (a << 16) | b;
    }
}

// The narrowphase's jobs: the broadphase pairs themselves, or in a world
// with compound bodies their shape pairs (job_pair / job_sh).  Returns the
// job count; sets ST_JOBS_OVERFLOW when they outgrow the job list.
DI int ph_jobs(Smem& S) {
  const DWorld& W = S.W;
  const int np = S.n_pairs;
  if (!S.P.compound) return np;
  for (int k = threadIdx.x; k < np; k += BT) W.pair_cnt[k] = pair_jobs(W, k);
  __syncthreads();
  const int total = block_scan_array(S, W.pair_cnt, np);
  if (total > S.P.jobs_cap) {
    if (threadIdx.x == 0) S.overflow |= ST_JOBS_OVERFLOW;
    __syncthreads();
    return 0;
  }
  for (int k = threadIdx.x; k < np; k += BT) pair_jobs_fill(W, k, W.pair_cnt[k]);
  __syncthreads();
  return total;
}

DI void ph_narrow(Smem& S) {
  const DWorld& W = S.W;
  const int np = ph_jobs(S);
  if (S.overflow) return;
  if (threadIdx.x == 0) { S.n_queued = 0; S.cursor = 0; S.n_jobs = np; }
  __syncthreads();
  for (int k = threadIdx.x; k < np; k += BT) narrow_first(S, k, &S.n_queued);
  __syncthreads();
  // queued pairs by resolver kind, each kind's segment starting on a warp
  // boundary
  const int nh = S.n_queued;
  if (threadIdx.x < 16) S.kcnt[threadIdx.x] = 0;
  __syncthreads();
  for (int h = threadIdx.x; h < nh; h += BT) atomicAdd(&S.kcnt[(unsigned)W.heavy[h] >> 28], 1);
  __syncthreads();
  if (threadIdx.x == 0) {
    int o = 0;
    for (int r = 0; r < 16; r++) {
      S.kpos[r] = o;
      o += (S.kcnt[r] + 31) & ~31;
    }
    S.cursor2 = o;
  }
  __syncthreads();
  const int nhp = S.cursor2;
  for (int h = threadIdx.x; h < nhp; h += BT) W.heavy2[h] = -1;
  __syncthreads();
  for (int h = threadIdx.x; h < nh; h += BT) {
    const unsigned e = (unsigned)W.heavy[h];
    W.heavy2[atomicAdd(&S.kpos[e >> 28], 1)] = (int)e;
  }
  __syncthreads();
  if (threadIdx.x == 0) S.n_queued = 0;
  __syncthreads();
  // hull pairs (kinds RK_BB and up) first take convex_convex's cheap stage 1;
  // the survivors are queued again (into W.heavy, free once sorted) and take
  // the binary64 stage together, in full warps
  for (int h = threadIdx.x; h < nhp; h += BT) narrow_stage1(S, h, &S.n_queued);
  __syncthreads();
  const int nh2 = S.n_queued;
  for (int h = threadIdx.x; h < nh2; h += BT) narrow_stage2(S, h);
  __syncthreads();
  // order: contacts of pair k follow those of pairs < k
  for (int k = threadIdx.x; k < np; k += BT) W.heavy[k] = W.pair_cnt[k];
  __syncthreads();
  int total = block_scan_array(S, W.heavy, np);
  if (threadIdx.x == 0) {
    S.n_contacts = total;
    if (total > S.P.contacts_cap) S.overflow |= ST_CONTACTS_OVERFLOW;
  }
  __syncthreads();
  if (S.overflow) return;
  for (int k = threadIdx.x; k < np; k += BT) narrow_place(W, k);
  __syncthreads();
}

// ---------------------------------------------------------------------------
// rows

// friction of a contact: createFrictionEquationsFromContact (narrow_phase.dart:530-586)
DI double contact_friction(const DWorld& W, const DContact& c) {
  double friction = W.cms[c.cm].friction;
  int ma = W.shapes[c.si].material >= 0 ? W.shapes[c.si].material : W.bodies[c.bi].material;
  int mb = W.shapes[c.sj].material >= 0 ? W.shapes[c.sj].material : W.bodies[c.bj].material;
  if (ma >= 0 && mb >= 0 && W.mats[ma].friction >= 0 && W.mats[mb].friction >= 0)
    friction = W.mats[ma].friction * W.mats[mb].friction;
  return friction;
}

DI bool row_kept(const DWorld& W, int bi, int bj, bool enabled) {  // Solver.addEquation (solver.dart:30-34)
  return enabled && !(W.bodies[bi].flags & BF_TRIGGER) && !(W.bodies[bj].flags & BF_TRIGGER);
}

// Candidates, in World.internalStep order (world_class.dart:539-635):
//   [0, nF)          friction rows, two per contact with friction > 0
//   [nF, nF+nC)      contact rows
//   [nF+nC, ...)     constraint rows (constraint order, equation order)
// Narrowphase.enableFrictionReduction (narrow_phase.dart:114): planeConvex
// and convexConvex (:1904-1911, :2033-2038) create no friction equations per
// contact but one pair of them per shape pair, from its last contact, with
// the pair's contacts averaged (createFrictionFromAverage, :589-627).  The
// other resolvers create theirs per contact as always.
DI bool fric_reduced(const DWorld& W, const DWorldParams& P, const DContact& ct) {
  if (!P.fric_reduction) return false;
  const int ta = W.shapes[ct.si].type, tb = W.shapes[ct.sj].type;
  return resolver_kind(min(ta, tb), max(ta, tb)) >= RK_PB;
}

// friction rows of contact c (cscr[c] = 2 or 0) and its slip force
DI void contact_fric_count(const DWorld& W, const DWorldParams& P, int c) {
  DContact& ct = W.contacts[c];
  // with friction reduction only the last contact of a plane-hull or
  // hull-hull shape pair carries friction rows (the pair's contacts are
  // W.contacts[heavy[k] .. heavy[k] + pair_cnt[k]))
  if (fric_reduced(W, P, ct) && c != W.heavy[ct.pair] + W.pair_cnt[ct.pair] - 1) {
    W.cscr[c] = 0;
    return;
  }
  double fr = contact_friction(W, ct);
  W.cscr[c] = fr > 0 ? 2 : 0;
  if (fr > 0) {
    double mug = fr * length(P.has_fgrav ? ld3(P.fgrav) : ld3(P.gravity));
    double red = W.bodies[ct.bi].inv_mass + W.bodies[ct.bj].inv_mass;
    if (red > 0) red = 1 / red;
    ct.slip = mug * red;
  }
}
// the row candidates of contact c (cscr holds the friction-row scan, nF its
// total)
DI void contact_cands(const DWorld& W, int c, int nc, int nF) {
  DContact& ct = W.contacts[c];
  int f0 = W.cscr[c];
  int has = (c + 1 < nc ? W.cscr[c + 1] : nF) - f0;
  ct.frow = has ? f0 : -1;
  bool keep = row_kept(W, ct.bi, ct.bj, ct.enabled);
  if (has) { W.cand[f0] = keep; W.cand[f0 + 1] = keep; }
  W.cand[nF + c] = keep;
}
// the row candidates of constraint k, after the nF + nc contact candidates
DI void constraint_cands(const DWorld& W, int k, int base0) {
  const DConstraint& cn = W.cons[k];
  int base = base0 + cn.row0;
  for (int r = 0; r < cn.nrows; r++) {
    bool enabled = !(cn.type == CP_CON_HINGE && r == 5 && !cn.motor);
    W.cand[base + r] = row_kept(W, cn.a, cn.b, enabled);
  }
}

DI void ph_rows_list(Smem& S) {
  const DWorld& W = S.W;
  const DWorldParams& P = S.P;
  const int nc = S.n_contacts;
  for (int c = threadIdx.x; c < nc; c += BT) contact_fric_count(W, P, c);
  __syncthreads();
  int nF = block_scan_array(S, W.cscr, nc);
  for (int c = threadIdx.x; c < nc; c += BT) contact_cands(W, c, nc, nF);
  for (int k = threadIdx.x; k < P.ncons; k += BT) constraint_cands(W, k, nF + nc);
  __syncthreads();
  const int ncand = nF + nc + P.ncon_rows;
  int nrows = block_scan_array(S, W.cand, ncand);
  if (threadIdx.x == 0) {
    S.n_fric = nF;
    S.n_cand = ncand;
    S.n_rows = nrows;
    if (nrows > P.rows_cap) S.overflow |= ST_ROWS_OVERFLOW;
  }
  __syncthreads();
}

DI bool cand_kept(const DWorld& W, int c, int ncand, int nrows) {
  int nxt = c + 1 < ncand ? W.cand[c + 1] : nrows;
  return nxt > W.cand[c];
}

// restitution override, wake-up tests (world_class.dart:544-624) and
// constraint geometry (Constraint.update)
// restitution override and wake-up tests of contact c (world_class.dart:
// 544-590)
DI void contact_post(const DWorld& W, int c) {
  DContact& ct = W.contacts[c];
  const DBody& bi = W.bodies[ct.bi];
  const DBody& bj = W.bodies[ct.bj];
  if (bi.material >= 0 && bj.material >= 0) {
    double ra = W.mats[bi.material].restitution, rb = W.mats[bj.material].restitution;
    if (ra >= 0 && rb >= 0) ct.restitution = ra * rb;
  }
  if ((bi.flags & BF_ALLOW_SLEEP) && bi.type == CP_BODY_DYNAMIC && bi.sleep_state == CP_SLEEPING &&
      bj.sleep_state == CP_AWAKE && bj.type != CP_BODY_STATIC) {
    double s2 = length2(ld3(bj.vel)) + length2(ld3(bj.avel));
    double l2 = bj.sleep_speed_limit * bj.sleep_speed_limit;
    if (s2 >= l2 * 2) atomicOr(&W.bodies[ct.bi].flags, BF_WAKE);
  }
  if ((bj.flags & BF_ALLOW_SLEEP) && bj.type == CP_BODY_DYNAMIC && bj.sleep_state == CP_SLEEPING &&
      bi.sleep_state == CP_AWAKE && bi.type != CP_BODY_STATIC) {
    double s2 = length2(ld3(bi.vel)) + length2(ld3(bi.avel));
    double l2 = bi.sleep_speed_limit * bi.sleep_speed_limit;
    if (s2 >= l2 * 2) atomicOr(&W.bodies[ct.bj].flags, BF_WAKE);
  }
}

// wakeUp of the flagged bodies (world_class.dart:618-624)
DI void wake_body(const DWorld& W, int i) {
  DBody& b = W.bodies[i];
  if (b.flags & BF_WAKE) {
    b.sleep_state = CP_AWAKE;
    b.flags &= ~BF_WAKE;
  }
}

// Constraint.update of constraint k: the per-step geometry of its rows
DI void constraint_geom(const DWorld& W, int k) {
  DConstraint& cn = W.cons[k];
  const DBody& A = W.bodies[cn.a];
  const DBody& B = W.bodies[cn.b];
  if (cn.type == CP_CON_DISTANCE || cn.type == CP_CON_SPRING) {
    // distance_constraint.dart:269-280, spring_constraint.dart:45-57
    double half = cn.distance * 0.5;
    f3 n = normalized(sub(ld3(B.pos), ld3(A.pos)));
    st3(cn.n, n);
    st3(cn.ri, scale(n, half));
    st3(cn.rj, scale(n, -half));
  } else {  // point_to_point_constraint.dart:122-137 and the subclasses' update()
    q4 qa = ld4q(A.quat), qb = ld4q(B.quat);
    st3(cn.ri, vmult(qa, ld3(cn.piv_a)));
    st3(cn.rj, vmult(qb, ld3(cn.piv_b)));
    if (cn.type == CP_CON_HINGE) {  // hinge_constraint.dart:217-242
      f3 wa = vmult(qa, ld3(cn.axis_a));
      f3 wb = vmult(qb, ld3(cn.axis_b));
      f3 t1, t2;
      tangents(wa, t1, t2);
      st3(cn.rot_a[0], t1);
      st3(cn.rot_a[1], t2);
      st3(cn.rot_b[0], wb);
      st3(cn.rot_b[1], wb);
      if (cn.motor) {
        st3(cn.ma, vmult(qa, ld3(cn.axis_a)));
        st3(cn.mb, vmult(qb, ld3(cn.axis_b)));
      }
    } else if (cn.type == CP_CON_LOCK) {  // lock_constraint.dart:86-103: (xA, yB), (yA, zB), (zA, xB)
#pragma unroll
      for (int r = 0; r < 3; r++) {
        st3(cn.rot_a[r], vmult(qa, ld3(cn.loc[2 * r])));
        st3(cn.rot_b[r], vmult(qb, ld3(cn.loc[(2 * r + 3) % 6])));
      }
    } else if (cn.type == CP_CON_CONE_TWIST) {  // cone_twist_constraint.dart:77-96
      st3(cn.rot_a[0], vmult(qa, ld3(cn.axis_a)));
      st3(cn.rot_b[0], vmult(qb, ld3(cn.axis_b)));
      // axis.tangents(t, t) leaves the second tangent in t
      f3 t1, t2a, t2b;
      tangents(ld3(cn.axis_a), t1, t2a);
      tangents(ld3(cn.axis_b), t1, t2b);
      st3(cn.rot_a[1], vmult(qa, t2a));
      st3(cn.rot_b[1], vmult(qb, t2b));
    }
  }
}

DI void ph_contacts_post(Smem& S) {
  const DWorld& W = S.W;
  const DWorldParams& P = S.P;
  for (int c = threadIdx.x; c < S.n_contacts; c += BT) contact_post(W, c);
  __syncthreads();
  for (int i = threadIdx.x; i < P.nb; i += BT) wake_body(W, i);
  __syncthreads();
  for (int k = threadIdx.x; k < P.ncons; k += BT) constraint_geom(W, k);
  __syncthreads();
}

// Body solve state: gravity (world_class.dart:460-471, applied here because
// nothing between it and the solver reads Body.force), updateSolveMassProperties
// (rigid_body.dart:303-314), vlambda/wlambda reset and the per-body parts of
// computeGiMf.
DI void solve_prep_body(const DWorld& W, const DWorldParams& P, int i) {
  const double gx = P.gravity[0], gy = P.gravity[1], gz = P.gravity[2];
  DBody& b = W.bodies[i];
  DBodyScr& s = W.bscr[i];
  if (b.type == CP_BODY_DYNAMIC) {
    double m = b.mass;
    b.force[0] = (float)(b.force[0] + m * gx);
    b.force[1] = (float)(b.force[1] + m * gy);
    b.force[2] = (float)(b.force[2] + m * gz);
  }
  bool zero = b.sleep_state == CP_SLEEPING || b.type == CP_BODY_KINEMATIC;
  double im = zero ? 0.0 : b.inv_mass;
  bool any_iw = false;
  float iw[9];
#pragma unroll
  for (int e = 0; e < 9; e++) {
    iw[e] = zero ? 0.f : b.iw[e];
    any_iw |= iw[e] != 0.f;
  }
  s.im_solve = im;
  s.active = (im != 0.0) || any_iw;
  *(float4*)s.vl = make_float4(0.f, 0.f, 0.f, s.active ? 1.f : 0.f);  // w: solve flag
  *(float4*)s.wl = make_float4(0.f, 0.f, 0.f, 0.f);
  st3(s.imf, scale(ld3(b.force), im));
  st3(s.iit, mvmult(iw, ld3(b.torque)));
}

DI void ph_solve_prep(Smem& S) {
  for (int i = threadIdx.x; i < S.P.nb; i += BT) solve_prep_body(S.W, S.P, i);
  __syncthreads();
}

// Row assembly: Jacobians and computeB (contact_equation.dart:34-77,
// friction_equation.dart:19-47, rotational_equation.dart:34-58,
// rotational_motor_equation.dart:17-33), computeC (equation_class.dart:129-174)
struct RowGeom {
  int kind, bi, bj;
  f3 ri, rj, n;       // contact: ni; friction: t
  f3 axA, axB;        // rotational / motor axes
  double restitution, a, b, eps, minF, maxF, cos_max, target;
};

DI void assemble_row(const DWorld& W, const RowGeom& G, DRow& R, double h) {
  const DBody& bi = W.bodies[G.bi];
  const DBody& bj = W.bodies[G.bj];
  const DBodyScr& si = W.bscr[G.bi];
  const DBodyScr& sj = W.bscr[G.bj];
  f3 gaS{0, 0, 0}, gaR{0, 0, 0}, gbS{0, 0, 0}, gbR{0, 0, 0};
  double B;
  if (G.kind == CP_ROW_CONTACT) {
    f3 rixn = cross(G.ri, G.n), rjxn = cross(G.rj, G.n);
    gaS = neg(G.n); gaR = neg(rixn); gbS = G.n; gbR = rjxn;
    f3 pen = ld3(bj.pos);
    pen = add(pen, G.rj);
    pen = sub(pen, ld3(bi.pos));
    pen = sub(pen, G.ri);
    double g = dot(G.n, pen);
    double e1 = G.restitution + 1;
    double gw = e1 * dot(ld3(bj.vel), G.n) - e1 * dot(ld3(bi.vel), G.n) + dot(ld3(bj.avel), rjxn) - dot(ld3(bi.avel), rixn);
    double giMf = (dot(ld3(si.imf), gaS) + dot(ld3(si.iit), gaR)) + (dot(ld3(sj.imf), gbS) + dot(ld3(sj.iit), gbR));
    B = -g * G.a - gw * G.b - h * giMf;
  } else if (G.kind == CP_ROW_FRICTION) {
    f3 rixt = cross(G.ri, G.n), rjxt = cross(G.rj, G.n);
    gaS = neg(G.n); gaR = neg(rixt); gbS = G.n; gbR = rjxt;
    double gw = (dot(ld3(bi.vel), gaS) + dot(ld3(bi.avel), gaR)) + (dot(ld3(bj.vel), gbS) + dot(ld3(bj.avel), gbR));
    double giMf = (dot(ld3(si.imf), gaS) + dot(ld3(si.iit), gaR)) + (dot(ld3(sj.imf), gbS) + dot(ld3(sj.iit), gbR));
    B = -gw * G.b - h * giMf;
  } else if (G.kind == CP_ROW_ROTATIONAL) {
    f3 nixnj = cross(G.axA, G.axB), njxni = cross(G.axB, G.axA);
    gaR = njxni; gbR = nixnj;
    double g = G.cos_max - dot(G.axA, G.axB);
    double gW = (dot(ld3(bi.vel), gaS) + dot(ld3(bi.avel), gaR)) + (dot(ld3(bj.vel), gbS) + dot(ld3(bj.avel), gbR));
    double giMf = (dot(ld3(si.imf), gaS) + dot(ld3(si.iit), gaR)) + (dot(ld3(sj.imf), gbS) + dot(ld3(sj.iit), gbR));
    B = -g * G.a - gW * G.b - h * giMf;
  } else {
    gaR = G.axA; gbR = neg(G.axB);
    double gw = (dot(ld3(bi.vel), gaS) + dot(ld3(bi.avel), gaR)) + (dot(ld3(bj.vel), gbS) + dot(ld3(bj.avel), gbR)) - G.target;
    double giMf = (dot(ld3(si.imf), gaS) + dot(ld3(si.iit), gaR)) + (dot(ld3(sj.imf), gbS) + dot(ld3(sj.iit), gbR));
    B = -gw * G.b - h * giMf;
  }
  float iwa[9], iwb[9];
  bool za = bi.sleep_state == CP_SLEEPING || bi.type == CP_BODY_KINEMATIC;
  bool zb = bj.sleep_state == CP_SLEEPING || bj.type == CP_BODY_KINEMATIC;
#pragma unroll
  for (int e = 0; e < 9; e++) {
    iwa[e] = za ? 0.f : bi.iw[e];
    iwb[e] = zb ? 0.f : bj.iw[e];
  }
  f3 iMaR = mvmult(iwa, gaR), iMbR = mvmult(iwb, gbR);
  double C = si.im_solve + sj.im_solve;
  C += dot(iMaR, gaR);
  C += dot(iMbR, gbR);
  C = C + G.eps;
  st3(R.gaS, gaS); st3(R.gaR, gaR); st3(R.gbS, gbS); st3(R.gbR, gbR);
  st3(R.iMaR, iMaR); st3(R.iMbR, iMbR);
  R.B = B;
  R.invC = 1.0 / C;
  R.eps = G.eps;
  R.minF = G.minF;
  R.maxF = G.maxF;
  R.lambda = 0.0;
  R.imA = si.im_solve;
  R.imB = sj.im_solve;
  R.bi = G.bi;
  R.bj = G.bj;
  R.kind = G.kind;
}

// createFrictionFromAverage (narrow_phase.dart:589-627): the friction rows
// of the last contact `last` of a shape pair with n >= 2 contacts take the
// pair's averaged contact points and the tangents of its averaged normal
DI void fric_average(const DWorld& W, int last, int n, f3& ri, f3& rj, f3& t1, f3& t2) {
  f3 avgN{0.f, 0.f, 0.f}, avgA{0.f, 0.f, 0.f}, avgB{0.f, 0.f, 0.f};
  const int bodyA = W.contacts[last].bi;
  for (int i = 0; i != n; i++) {
    const DContact& c = W.contacts[last - i];
    if (c.bi != bodyA) {
      avgN = add(avgN, ld3(c.ni));
      avgA = add(avgA, ld3(c.ri));
      avgB = add(avgB, ld3(c.rj));
    } else {
      avgN = sub(avgN, ld3(c.ni));
      avgA = add(avgA, ld3(c.rj));
      avgB = add(avgB, ld3(c.ri));
    }
  }
  const double inv = 1.0 / n;
  ri = scale(avgA, inv);
  rj = scale(avgB, inv);
  tangents(normalized(avgN), t1, t2);
}

// the friction and contact rows of contact c
DI void assemble_contact_rows(const DWorld& W, const DWorldParams& P, int c, int nF, int ncand, int nrows, double h) {
  const DContact& ct = W.contacts[c];
  const DContactMaterial& cm = W.cms[ct.cm];
  RowGeom G;
  G.bi = ct.bi; G.bj = ct.bj;
  G.ri = ld3(ct.ri); G.rj = ld3(ct.rj);
  f3 ni = ld3(ct.ni);
  if (ct.frow >= 0) {
    f3 t1, t2;
    const int np = fric_reduced(W, P, ct) ? W.pair_cnt[ct.pair] : 1;
    if (np > 1) fric_average(W, c, np, G.ri, G.rj, t1, t2);
    else tangents(ni, t1, t2);
    G.kind = CP_ROW_FRICTION;
    G.a = cm.fa; G.b = cm.fb; G.eps = cm.feps;
    G.minF = -ct.slip; G.maxF = ct.slip;
    for (int m = 0; m < 2; m++) {
      int cd = ct.frow + m;
      if (cand_kept(W, cd, ncand, nrows)) {
        G.n = m == 0 ? t1 : t2;
        DRow& R = W.rows[W.cand[cd]];
        assemble_row(W, G, R, h);
        R.src = cd;
      }
    }
  }
  int cd = nF + c;
  if (cand_kept(W, cd, ncand, nrows)) {
    G.kind = CP_ROW_CONTACT;
    G.ri = ld3(ct.ri); G.rj = ld3(ct.rj);
    G.n = ni;
    G.restitution = ct.restitution;
    G.a = cm.ca; G.b = cm.cb; G.eps = cm.ceps;
    G.minF = 0.0; G.maxF = 1e6;
    DRow& R = W.rows[W.cand[cd]];
    assemble_row(W, G, R, h);
    R.src = cd;
  }
}

// the rows of constraint k (its candidates start at base0 + row0)
DI void assemble_constraint_rows(const DWorld& W, int k, int base0, int ncand, int nrows, double h) {
  const DConstraint& cn = W.cons[k];
  int base = base0 + cn.row0;
  RowGeom G;
  G.bi = cn.a; G.bj = cn.b;
  G.a = cn.sa; G.b = cn.sb; G.eps = cn.seps;
  G.restitution = 0.0;
  G.target = cn.motor_target;
  for (int r = 0; r < cn.nrows; r++) {
    int cd = base + r;
    if (!cand_kept(W, cd, ncand, nrows)) continue;
    G.minF = -cn.max_force; G.maxF = cn.max_force;
    G.cos_max = cn.cos_rot[0];
    if (cn.type == CP_CON_DISTANCE || cn.type == CP_CON_SPRING) {
      G.kind = CP_ROW_CONTACT;
      G.ri = ld3(cn.ri); G.rj = ld3(cn.rj); G.n = ld3(cn.n);
    } else if (r < 3) {
      G.kind = CP_ROW_CONTACT;
      G.ri = ld3(cn.ri); G.rj = ld3(cn.rj);
      G.n = r == 0 ? f3{1.f, 0.f, 0.f} : (r == 1 ? f3{0.f, 1.f, 0.f} : f3{0.f, 0.f, 1.f});
    } else if (cn.type == CP_CON_HINGE && r == 5) {
      G.kind = CP_ROW_MOTOR;
      G.axA = ld3(cn.ma);
      G.axB = ld3(cn.mb);
      G.minF = -cn.motor_max_force; G.maxF = cn.motor_max_force;
    } else {
      G.kind = CP_ROW_ROTATIONAL;
      G.axA = ld3(cn.rot_a[r - 3]);
      G.axB = ld3(cn.rot_b[r - 3]);
      if (cn.type == CP_CON_CONE_TWIST) {  // both rows push one way: [-maxForce, 0]
        G.maxF = 0.0;
        if (r == 4) G.cos_max = cn.cos_rot[1];
      }
    }
    DRow& R = W.rows[W.cand[cd]];
    assemble_row(W, G, R, h);
    R.src = cd;
  }
}

DI void ph_rows_assemble(Smem& S, double h) {
  const DWorld& W = S.W;
  const int nc = S.n_contacts, nF = S.n_fric, ncand = S.n_cand, nrows = S.n_rows;
  for (int c = threadIdx.x; c < nc; c += BT) assemble_contact_rows(W, S.P, c, nF, ncand, nrows, h);
  for (int k = threadIdx.x; k < S.P.ncons; k += BT) assemble_constraint_rows(W, k, nF + nc, ncand, nrows, h);
  __syncthreads();
}

// ---------------------------------------------------------------------------
// GSSolver.solve (gs_solver.dart:74-180)

// Dependency levels: a row waits for the latest earlier row that shares a
// dynamic body with it.  Bodies with zero solve mass and inertia
// (static, sleeping, kinematic) keep vlambda = wlambda = +0 exactly, so they
// order nothing.
// Rows are walked in order by one thread (the level of a row depends on
// every earlier row on its bodies), from shared memory: all threads stage the
// (bi, bj) pairs of a chunk of rows, thread 0 assigns their levels against a
// per-body table in shared memory (worlds of up to last_cap bodies; larger
// worlds keep the table in global scratch), and all threads write the levels
// back.
#define CP_LEVEL_CHUNK 512
// largest per-body level table kept in shared memory (33 KB; with the row
// chunk the dynamic shared memory stays under the 48 KB default limit)
#define CP_SMEM_LEVEL_MAX 8448

// order: the rows in the order the solver takes them (null: row order)
DI void ph_levels(Smem& S, int* s_last, int last_cap, int2* s_pairs, const int* order = nullptr) {
  const DWorld& W = S.W;
  const int nrows = S.n_rows;
  const int nb = S.P.nb;
  // last[b] = level of the latest row on dynamic body b, or -2 for bodies with
  // zero solve mass and inertia (they order nothing)
  int* last = nb <= last_cap ? s_last : W.level_cursor;
  for (int i = threadIdx.x; i < nb; i += BT) last[i] = W.bscr[i].active ? -1 : -2;
  int nlev = 0;  // thread 0
  for (int c0 = 0; c0 < nrows; c0 += CP_LEVEL_CHUNK) {
    const int n = min(CP_LEVEL_CHUNK, nrows - c0);
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += BT) {
      const int r = order ? order[c0 + i] : c0 + i;
      s_pairs[i] = make_int2(W.rows[r].bi, W.rows[r].bj);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int i = 0; i < n; i++) {
        const int2 p = s_pairs[i];
        const int la = last[p.x], lb = last[p.y];
        int l = (la > lb ? la : lb) + 1;
        if (l < 0) l = 0;
        if (la != -2) last[p.x] = l;
        if (lb != -2) last[p.y] = l;
        s_pairs[i].x = l;
        if (l + 1 > nlev) nlev = l + 1;
      }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += BT) W.level_of[order ? order[c0 + i] : c0 + i] = s_pairs[i].x;
  }
  if (threadIdx.x == 0) S.n_levels = nlev;
  __syncthreads();
  const int nl = S.n_levels;
  for (int l = threadIdx.x; l <= nl; l += BT) W.level_start[l] = 0;
  __syncthreads();
  for (int r = threadIdx.x; r < nrows; r += BT) atomicAdd(&W.level_start[W.level_of[r]], 1);
  __syncthreads();
  block_scan_array(S, W.level_start, nl + 1);
  for (int l = threadIdx.x; l < nl; l += BT) W.level_cursor[l] = W.level_start[l];
  __syncthreads();
  for (int r = threadIdx.x; r < nrows; r += BT) W.level_rows[atomicAdd(&W.level_cursor[W.level_of[r]], 1)] = r;
  __syncthreads();
  // the rows in level order for the sweeps
  const int cap = W.sw_cap;
  for (int p = threadIdx.x; p < nrows; p += BT) {
    const int r = W.level_rows[p];
    const DRow& R = W.rows[r];
    W.sw_j[p] = make_float4(R.gaS[0], R.gaS[1], R.gaS[2], R.gaR[0]);
    W.sw_j[cap + p] = make_float4(R.gaR[1], R.gaR[2], R.gbS[0], R.gbS[1]);
    W.sw_j[2 * cap + p] = make_float4(R.gbS[2], R.gbR[0], R.gbR[1], R.gbR[2]);
    W.sw_j[3 * cap + p] = make_float4(R.iMaR[0], R.iMaR[1], R.iMaR[2], R.iMbR[0]);
    W.sw_j[4 * cap + p] = make_float4(R.iMbR[1], R.iMbR[2], 0.f, 0.f);
    W.sw_d[p] = make_double2(R.B, R.invC);
    W.sw_d[cap + p] = make_double2(R.eps, R.lambda);
    W.sw_d[2 * cap + p] = make_double2(R.imA, R.imB);
    W.sw_d[3 * cap + p] = make_double2(R.minF, R.maxF);
    W.sw_b[p] = make_int2(R.bi, R.bj);
    W.sw_orig[p] = r;
  }
  __syncthreads();
}

// One row of one sweep (gs_solver.dart:127-148 with Equation.computeGWlambda
// and addToWlambda, equation_class.dart:95-169)
// binary32 value to binary64 on the integer pipe: exact, and free of the
// F2F conversion that occupies the binary64 pipe on GB300.  Normal numbers
// and zeros take the integer path; subnormals and non-finite values convert
// the ordinary way.
DI double f2d(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xffu;
  const unsigned long long sign = (unsigned long long)(u & 0x80000000u) << 32;
  if (e - 1u < 254u)
    return __longlong_as_double((long long)(sign | ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)(u & 0x7fffffu) << 29)));
  if ((u << 1) == 0u) return __longlong_as_double((long long)sign);
  return (double)f;
}
DI d3 f2d3(float x, float y, float z) { return d3{f2d(x), f2d(y), f2d(z)}; }

// dot product of two vectors of binary32 values in the reference's order
// ((x + y) + z): every product is exact in binary64, so a fused multiply-add
// rounds each partial sum exactly as the separate multiply and add do
DI double ddot_f(d3 a, d3 b) { return __fma_rn(a.z, b.z, __fma_rn(a.y, b.y, a.x * b.x)); }

// One row of a GSSolver sweep (gs_solver.dart:122-155) at level position p.
// A body with zero solve mass and inertia keeps vlambda = wlambda = +0, so
// its half of G*Wlambda is a signed zero and adding it changes no nonzero
// sum; a zero sum can only change sign, which no later store observes.
DI d3 f2d3v(float4 v) { return f2d3(v.x, v.y, v.z); }
// vlambda / wlambda update: addScaledVector with the binary32 store (w kept)
DI float4 vstep(float4 v, double s, float gx, float gy, float gz) {
  return make_float4(r32f(f2d(v.x) + s * f2d(gx)), r32f(f2d(v.y) + s * f2d(gy)), r32f(f2d(v.z) + s * f2d(gz)), v.w);
}

// Where a world's vlambda / wlambda live during its sweeps: vlambda of body
// i at base[i * stride], wlambda at the next float4; vlambda.w is the body's
// solve flag (1: it takes velocity updates).  Shared memory for a group that
// fits, else the body scratch records in global memory.
struct VelRef {
  float4* base;
  int stride;
};
DI float4* vl_of(VelRef V, int i) { return V.base + (size_t)i * V.stride; }
DI VelRef vel_global(const DWorld& W) { return VelRef{(float4*)W.bscr[0].vl, (int)(sizeof(DBodyScr) / sizeof(float4))}; }

// One row's record, loaded at once so that its loads share one latency.
struct RowRec {
  float4 j0, j1, j2, j3, j4;
  double2 d0, d1, im, d3b;
};
DI RowRec load_row(const DWorld& W, int p) {
  const int cap = W.sw_cap;
  RowRec R;
  R.j0 = W.sw_j[p];
  R.j1 = W.sw_j[cap + p];
  R.j2 = W.sw_j[2 * cap + p];
  R.j3 = W.sw_j[3 * cap + p];
  R.j4 = W.sw_j[4 * cap + p];
  R.d0 = W.sw_d[p];
  R.d1 = W.sw_d[cap + p];
  R.im = W.sw_d[2 * cap + p];
  R.d3b = W.sw_d[3 * cap + p];
  return R;
}

// dlambda of a row from its two halves of G*Wlambda (gs_solver.dart:138-150)
DI double row_dl(const RowRec& R, double ga, bool aa, double gb, bool ab) {
  const double gwl = aa && ab ? ga + gb : (aa ? ga : gb);
  const double lj = R.d1.y;
  double dl = R.d0.y * (R.d0.x - gwl - R.d1.x * lj);
  if (lj + dl < R.d3b.x) dl = R.d3b.x - lj;
  else if (lj + dl > R.d3b.y) dl = R.d3b.y - lj;
  return dl;
}
DI double half_a(const RowRec& R, float4 v, float4 w) {
  return ddot_f(f2d3v(v), f2d3(R.j0.x, R.j0.y, R.j0.z)) + ddot_f(f2d3v(w), f2d3(R.j0.w, R.j1.x, R.j1.y));
}
DI double half_b(const RowRec& R, float4 v, float4 w) {
  return ddot_f(f2d3v(v), f2d3(R.j1.z, R.j1.w, R.j2.x)) + ddot_f(f2d3v(w), f2d3(R.j2.y, R.j2.z, R.j2.w));
}
DI void update_a(float4* pa, float4 v, float4 w, const RowRec& R, double dl) {
  pa[0] = vstep(v, R.im.x * dl, R.j0.x, R.j0.y, R.j0.z);
  pa[1] = vstep(w, dl, R.j3.x, R.j3.y, R.j3.z);
}
DI void update_b(float4* pb, float4 v, float4 w, const RowRec& R, double dl) {
  pb[0] = vstep(v, R.im.y * dl, R.j1.z, R.j1.w, R.j2.x);
  pb[1] = vstep(w, dl, R.j3.w, R.j4.x, R.j4.y);
}

// One row of a GSSolver sweep (gs_solver.dart:122-155) at level position p.
// A body with zero solve mass and inertia keeps vlambda = wlambda = +0, so
// its half of G*Wlambda is a signed zero and adding it changes no nonzero
// sum; a zero sum can only change sign, which no later store observes.
DI double gs_row_sw(const DWorld& W, VelRef V, int p, int2 bb) {
  const RowRec R = load_row(W, p);
  float4* pa = vl_of(V, bb.x);
  float4* pb = vl_of(V, bb.y);
  const float4 vla = pa[0], wla = pa[1], vlb = pb[0], wlb = pb[1];
  const bool aa = vla.w != 0.f, ab = vlb.w != 0.f;
  const double ga = aa ? half_a(R, vla, wla) : 0.0;
  const double gb = ab ? half_b(R, vlb, wlb) : 0.0;
  const double dl = row_dl(R, ga, aa, gb, ab);
  W.sw_d[W.sw_cap + p].y = R.d1.y + dl;
  if (aa) update_a(pa, vla, wla, R, dl);
  if (ab) {
    // re-read: bi == bj is possible for a constraint between a body and itself
    const bool same = bb.x == bb.y;
    update_b(pb, same ? pb[0] : vlb, same ? pb[1] : wlb, R, dl);
  }
  return dl > 0.0 ? dl : -dl;
}

// Add result to velocity; multipliers (gs_solver.dart:157-176)
// binary64 holding a binary32 value -> binary32, on the integer pipe (the
// reverse of f2d); other values convert the ordinary way
DI float d2f(double x) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const unsigned e = (unsigned)(u >> 52) & 0x7ffu;
  const unsigned sign = (unsigned)(u >> 32) & 0x80000000u;
  if (e - 897u < 254u && (u & 0x1fffffffull) == 0)
    return __uint_as_float(sign | ((e - 896u) << 23) | (unsigned)((u >> 29) & 0x7fffffu));
  if ((u << 1) == 0) return __uint_as_float(sign);
  return (float)x;
}

DI void apply_body(const DWorld& W, int i) {
  DBody& b = W.bodies[i];
  DBodyScr& s = W.bscr[i];
  f3 vl = mul(ld3(s.vl), ld3(b.lin_factor));
  st3(b.vel, add(ld3(b.vel), vl));
  f3 wl = mul(ld3(s.wl), ld3(b.ang_factor));
  st3(b.avel, add(ld3(b.avel), wl));
}

DI void apply_row(const DWorld& W, int p, double invDt) {
  DRow& R = W.rows[W.sw_orig[p]];
  const double lam = W.sw_d[W.sw_cap + p].y;
  R.lambda = lam;
  R.mult = lam * invDt;
}

DI void ph_solve_apply(Smem& S, double h) {
  const DWorld& W = S.W;
  for (int i = threadIdx.x; i < S.P.nb; i += BT) apply_body(W, i);
  const double invDt = 1 / h;
  for (int p = threadIdx.x; p < S.n_rows; p += BT) apply_row(W, p, invDt);
  __syncthreads();
}

// ---------------------------------------------------------------------------
// SplitSolver (split_solver.dart:53-126) over the GSSolver.
//
// Its islands are the connected groups of non-static bodies (getUnvisitedNode
// skips static ones), each solved on its own: equations sorted by
// Equation.id, highest first, and its own convergence test.  Islands share
// no body that moves, so they are swept together here: the rows go through
// the dependency levels in descending id order (within an island that is its
// order), a row is skipped once its island has converged, and only the
// bodies of islands with equations take the velocity update.  Ids: the
// constraints' from their constructors, the contact and friction equations'
// from the narrowphase's object pools (last step's equations pushed in order,
// popped from the end; new objects take Equation.idCounter in creation
// order), world_class.dart:506-527, narrow_phase.dart:492-586.

DI bool split_moves(const DBody& b) { return b.type != CP_BODY_STATIC; }

// equation ids of the step's contacts and friction candidates: contact c is
// created after the cscr[c] friction objects of the contacts before it, the
// two of its own right after it
// Contact equation objects are taken in job order: one per contact, and
// one per spherePlane job whether it makes a contact or not; contact c is
// object e(c) of the step.
DI void split_ids(Smem& S) {
  const DWorld& W = S.W;
  const DWorldParams& P = S.P;
  const int Pc = P.pool_c, Pf = P.pool_f;
  const long long idc = P.id_counter;
  const int nj = S.n_jobs;
  for (int j = threadIdx.x; j < nj; j += BT) W.job_base[j] = W.job_att[j] ? 1 : W.pair_cnt[j];
  __syncthreads();
  const int E = block_scan_array(S, W.job_base, nj);
  if (threadIdx.x == 0) S.split_e = E;
  for (int c = threadIdx.x; c < S.n_contacts; c += BT) {
    const int job = W.contacts[c].pair;
    const int e = W.job_base[job] + (c - W.heavy[job]);
    const int F = W.cscr[c];
    W.ct_id[c] = e < Pc ? W.pool_c[Pc - 1 - e] : idc + (e - Pc) + max(0, F - Pf);
    const int f0 = W.contacts[c].frow;
    if (f0 >= 0)
      for (int j = 0; j < 2; j++) {
        const int m = f0 + j;
        W.fr_id[m] = m < Pf ? W.pool_f[Pf - 1 - m] : idc + max(0, e + 1 - Pc) + (m - Pf);
      }
  }
  __syncthreads();
}

// id of the equation behind row candidate cd (friction, contact, then
// constraint candidates)
DI long long split_row_id(const DWorld& W, const DWorldParams& P, int cd, int nF, int nc) {
  if (cd < nF) return W.fr_id[cd];
  if (cd < nF + nc) return W.ct_id[cd - nF];
  const int x = cd - nF - nc;
  int lo = 0, hi = P.ncons - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (W.cons[mid].row0 <= x) lo = mid;
    else hi = mid - 1;
  }
  return W.cons[lo].first_id + (x - W.cons[lo].row0);
}

DI int uf_root(const int* par, int x) {
  int p = *(volatile const int*)&par[x];
  while (p != x) {
    x = p;
    p = *(volatile const int*)&par[x];
  }
  return x;
}
// union by the smaller root: every island ends rooted at its smallest body
DI void uf_union(int* par, int a, int b) {
  for (;;) {
    a = uf_root(par, a);
    b = uf_root(par, b);
    if (a == b) return;
    if (a > b) { const int t = a; a = b; b = t; }
    if (atomicCAS(&par[b], b, a) == b) return;
  }
}

// row ids, islands and the rows in descending id order (sort_val)
DI void split_prepare(Smem& S) {
  const DWorld& W = S.W;
  const DWorldParams& P = S.P;
  const int nb = P.nb, nrows = S.n_rows;
  for (int i = threadIdx.x; i < nb; i += BT) {
    W.isl_par[i] = split_moves(W.bodies[i]) ? i : -1;
    W.isl_rows[i] = 0;
  }
  const int N = W.sort_n;
  for (int r = threadIdx.x; r < N; r += BT) {
    W.sort_key[r] = r < nrows ? split_row_id(W, P, W.rows[r].src, S.n_fric, S.n_contacts) : LLONG_MIN;
    W.sort_val[r] = r;
  }
  __syncthreads();
  for (int r = threadIdx.x; r < nrows; r += BT) {
    const int a = W.rows[r].bi, b = W.rows[r].bj;
    if (W.isl_par[a] >= 0 && W.isl_par[b] >= 0) uf_union(W.isl_par, a, b);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nb; i += BT)
    if (W.isl_par[i] >= 0) W.isl_par[i] = uf_root(W.isl_par, i);
  __syncthreads();
  for (int r = threadIdx.x; r < nrows; r += BT) {
    W.row_id[r] = W.sort_key[r];
    const int a = W.rows[r].bi, b = W.rows[r].bj;
    const int isl = W.isl_par[a] >= 0 ? W.isl_par[a] : W.isl_par[b];
    W.row_isl[r] = isl;
    if (isl >= 0) atomicAdd(&W.isl_rows[isl], 1);
  }
  // bitonic sort of (id, row), highest id first; ids are distinct
  for (int k = 2; k <= N; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      __syncthreads();
      for (int i = threadIdx.x; i < N; i += BT) {
        const int l = i ^ j;
        if (l <= i) continue;
        const long long ki = W.sort_key[i], kl = W.sort_key[l];
        const bool up = (i & k) == 0;  // this run ends up highest first
        if (up ? ki < kl : ki > kl) {
          W.sort_key[i] = kl;
          W.sort_key[l] = ki;
          const int t = W.sort_val[i];
          W.sort_val[i] = W.sort_val[l];
          W.sort_val[l] = t;
        }
      }
    }
  __syncthreads();
}

// GSSolver.solve's sweeps for every island at once; returns the most
// iterations any island took
DI int split_sweeps(Smem& S) {
  const DWorld& W = S.W;
  const DWorldParams& P = S.P;
  const int nb = P.nb, nrows = S.n_rows, nl = S.n_levels;
  const VelRef V = vel_global(W);
  const double tol2 = P.tolerance * P.tolerance;
  for (int i = threadIdx.x; i < nb; i += BT) W.isl_iter[i] = W.isl_rows[i] > 0 ? -1 : 0;
  if (threadIdx.x == 0) S.converged = 0;
  __syncthreads();
  int sweep = 0;
  for (; sweep < P.iterations; sweep++) {
    for (int i = threadIdx.x; i < nb; i += BT) W.isl_sum[i] = 0.0;
    __syncthreads();
    for (int l = 0; l < nl; l++) {
      const int b = W.level_start[l], e = W.level_start[l + 1];
      for (int p = b + threadIdx.x; p < e; p += BT) {
        const int r = W.sw_orig[p];
        const int isl = W.row_isl[r];
        if (isl < 0 || W.isl_iter[isl] >= 0) continue;
        const double a = gs_row_sw(W, V, p, W.sw_b[p]);
        W.absdl[r] = a;
        atomicAdd(&W.isl_sum[isl], a);
      }
      __syncthreads();
    }
    // per island: (sum of |dlambda| in its row order)^2 < tol^2, the
    // order-free sum deciding unless it lies within the rounding band
    int left = 0;
    for (int i = threadIdx.x; i < nb; i += BT) {
      if (W.isl_iter[i] >= 0) continue;
      const double sp = W.isl_sum[i];
      const double band = 2.2 * (double)W.isl_rows[i] * 1.1102230246251565e-16;
      const double hi = sp * (1.0 + band), lo = sp * (1.0 - band);
      int conv;
      if (hi * hi * (1.0 + 4.5e-16) < tol2) conv = 1;
      else if (lo * lo * (1.0 - 4.5e-16) >= tol2 && lo >= 0.0) conv = 0;
      else {
        double t = 0.0;
        for (int q = 0; q < nrows; q++) {
          const int r = W.sort_val[q];
          if (W.row_isl[r] == i) t += W.absdl[r];
        }
        conv = t * t < tol2;
      }
      if (conv) W.isl_iter[i] = sweep;
      else left = 1;
    }
    S.warp[threadIdx.x >> 5] = __any_sync(0xffffffffu, left);
    __syncthreads();
    int any = 0;
    for (int w = 0; w < NWARP; w++) any |= S.warp[w];
    __syncthreads();
    if (!any) { sweep++; break; }
  }
  // islands still sweeping took every iteration
  int most = 0;
  for (int i = threadIdx.x; i < nb; i += BT) {
    if (W.isl_rows[i] == 0) continue;
    const int it = W.isl_iter[i] >= 0 ? W.isl_iter[i] : P.iterations;
    most = max(most, it);
  }
  for (int o = 16; o > 0; o >>= 1) most = max(most, __shfl_xor_sync(0xffffffffu, most, o));
  if ((threadIdx.x & 31) == 0) S.warp[threadIdx.x >> 5] = most;
  __syncthreads();
  int m = 0;
  for (int w = 0; w < NWARP; w++) m = max(m, S.warp[w]);
  __syncthreads();
  (void)sweep;
  return m;
}

// velocity update of the bodies of islands with equations; multipliers
DI void split_apply(Smem& S, double h) {
  const DWorld& W = S.W;
  for (int i = threadIdx.x; i < S.P.nb; i += BT) {
    const int isl = W.isl_par[i];
    if (isl >= 0 && W.isl_rows[isl] > 0) apply_body(W, i);
  }
  const double invDt = 1 / h;
  for (int p = threadIdx.x; p < S.n_rows; p += BT) apply_row(W, p, invDt);
  __syncthreads();
}

// the step's equations back into the pools (world_class.dart:506-517): the
// objects it did not pop stay at the bottom, its own go on top in creation
// order
DI void split_pools(Smem& S) {
  const DWorld& W = S.W;
  const DWorldParams& P = S.P;
  const int nc = S.n_contacts, nF = S.n_fric, E = S.split_e;
  const int bc = P.pool_c - min(P.pool_c, E), bf = P.pool_f - min(P.pool_f, nF);
  __syncthreads();
  for (int c = threadIdx.x; c < nc; c += BT) W.pool_c[bc + c] = W.ct_id[c];
  for (int m = threadIdx.x; m < nF; m += BT) W.pool_f[bf + m] = W.fr_id[m];
  if (threadIdx.x == 0) {
    DWorldParams* gp = W.P;
    gp->pool_c = bc + nc;
    gp->pool_f = bf + nF;
    gp->id_counter = P.id_counter + max(0, E - P.pool_c) + max(0, nF - P.pool_f);
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// damping, integrate, clearForces, sleepTick (world_class.dart:647-700,
// rigid_body.dart:263-300,627-680)
DI void integrate_body(const DWorld& W, const DWorldParams& P, int i, double dt, bool qn, double time) {
  DBody& b = W.bodies[i];
  f3 v = ld3(b.vel), w = ld3(b.avel);
  if (b.type == CP_BODY_DYNAMIC) {
    v = scale(v, W.dpow[2 * i]);
    w = scale(w, W.dpow[2 * i + 1]);
  }
  f3 p = ld3(b.pos);
  q4 q = ld4q(b.quat);
  st3(b.prev_pos, p);
  st4q(b.prev_quat, q);
  if ((b.type == CP_BODY_DYNAMIC || b.type == CP_BODY_KINEMATIC) && b.sleep_state != CP_SLEEPING) {
    double iMdt = b.inv_mass * dt;
    f3 lf = ld3(b.lin_factor), af = ld3(b.ang_factor);
    f3 f = ld3(b.force), t = ld3(b.torque);
    v.x = (float)(v.x + f.x * iMdt * lf.x);
    v.y = (float)(v.y + f.y * iMdt * lf.y);
    v.z = (float)(v.z + f.z * iMdt * lf.z);
    const float* e = b.iw;
    double tx = (double)t.x * af.x, ty = (double)t.y * af.y, tz = (double)t.z * af.z;
    w.x = (float)(w.x + dt * (e[0] * tx + e[1] * ty + e[2] * tz));
    w.y = (float)(w.y + dt * (e[3] * tx + e[4] * ty + e[5] * tz));
    w.z = (float)(w.z + dt * (e[6] * tx + e[7] * ty + e[8] * tz));
    p.x = (float)(p.x + v.x * dt);
    p.y = (float)(p.y + v.y * dt);
    p.z = (float)(p.z + v.z * dt);
    q = qintegrate(q, w, dt, af);
    if (qn) q = P.qn_fast ? qnormalize_fast(q) : qnormalize(q);
    st3(b.pos, p);
    st4q(b.quat, q);
    b.flags |= BF_AABB_DIRTY;
    f3 I = ld3(b.inv_inertia);
    if (!(I.x == I.y && I.y == I.z)) inertia_world(q, I, b.iw);
  }
  st3(b.force, f3{0.f, 0.f, 0.f});
  st3(b.torque, f3{0.f, 0.f, 0.f});
  if (P.allow_sleep && (b.flags & BF_ALLOW_SLEEP)) {
    int st = b.sleep_state;
    double s2 = length2(v) + length2(w);
    double lim2 = b.sleep_speed_limit * b.sleep_speed_limit;
    if (st == CP_AWAKE && s2 < lim2) {
      b.sleep_state = CP_SLEEPY;
      b.time_last_sleepy = time;
    } else if (st == CP_SLEEPY && s2 > lim2) {
      b.sleep_state = CP_AWAKE;
      b.flags &= ~BF_WAKE;
    } else if (st == CP_SLEEPY && time - b.time_last_sleepy > b.sleep_time_limit) {
      b.sleep_state = CP_SLEEPING;
      v = f3{0.f, 0.f, 0.f};
      w = f3{0.f, 0.f, 0.f};
      b.flags &= ~BF_WAKE;
    }
  }
  st3(b.vel, v);
  st3(b.avel, w);

}

DI void ph_integrate(Smem& S, double dt) {
  const DWorldParams& P = S.P;
  const bool qn = (P.stepnumber % (long long)(P.qn_skip + 1)) == 0;
  for (int i = threadIdx.x; i < P.nb; i += BT) integrate_body(S.W, P, i, dt, qn, P.time);
  __syncthreads();
}

// ---------------------------------------------------------------------------

DI void tick(Smem& S, int phase) {
  if (threadIdx.x == 0) {
    long long t = clock64();
    S.t_acc[phase] += t - S.t_last;
    S.t_last = t;
  }
}

// Everything of World.internalStep up to the solver's sweeps; returns false
// when a capacity overflow stopped the step before any body state changed.
DI bool step_pre(Smem& S, int* s_last, int last_cap, int2* s_pairs, double dt) {
  if (threadIdx.x == 0) {
    S.overflow = 0;
    S.n_pairs = S.n_contacts = S.n_rows = S.n_levels = 0;
    S.n_fric = S.n_cand = S.n_jobs = 0;
    S.t_last = clock64();
  }
  __syncthreads();
  ph_prepare(S);
  tick(S, 0);
  if (S.P.broadphase == CP_BROAD_SAP) ph_broad_sap(S);
  else if (S.P.broadphase == CP_BROAD_GRID) ph_broad_grid(S);
  else ph_broad_naive(S);
  if (S.overflow) return false;
  if (S.P.n_nocollide > 0) ph_nocollide(S);
  tick(S, 1);
  ph_narrow(S);
  tick(S, 2);
  if (S.overflow) return false;
  ph_rows_list(S);
  if (S.overflow) return false;
  // ---- body state changes from here on ----
  ph_contacts_post(S);
  ph_solve_prep(S);
  tick(S, 3);
  ph_rows_assemble(S, dt);
  tick(S, 4);
  if (S.P.split) {
    split_ids(S);
    if (S.n_rows > 0) split_prepare(S);
  }
  if (S.n_rows > 0) ph_levels(S, s_last, last_cap, s_pairs, S.P.split ? S.W.sort_val : nullptr);
  tick(S, 5);
  return true;
}

// The rest of a step of a SplitSolver world, in the pre-step kernel's block:
// island sweeps, velocity update, integration, the pools
DI void step_split_rest(Smem& S, double dt, double time_inc) {
  int iters = 0;
  if (S.n_rows > 0) {
    iters = split_sweeps(S);
    split_apply(S, dt);
  }
  ph_integrate(S, dt);
  split_pools(S);
  if (threadIdx.x == 0) {
    DWorldParams* gp = S.W.P;
    gp->last_iterations = iters;
    gp->stepnumber = S.P.stepnumber + 1;
    gp->time = S.P.time + time_inc;
    gp->presolved = 1;
  }
  __syncthreads();
}
