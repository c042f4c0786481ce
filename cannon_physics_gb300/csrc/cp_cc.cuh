// cp_cc.cuh -- convex-convex contacts (narrow_phase.dart:1981-2043 with
// ConvexPolyhedron.findSeparatingAxis / clipAgainstHull,
// convex_polyhedron.dart:189-587,843-883) in binary64 registers holding the
// reference's binary32 values, rounded by r32 where the reference stores.
//
// Three exact shortcuts, each giving the reference's result bit for bit:
//  * Canonical axes.  A face normal or unique edge whose exact negation
//    appears earlier in its hull's list yields the same depth as that earlier
//    entry (every operation of project/testSepAxis is odd in the axis and
//    round-to-nearest is symmetric), and it comes later in the loop order, so
//    under "first strict minimum wins" it can never be chosen, and if it
//    separates the hulls the earlier entry already did.  The same holds for
//    edge pairs built from such edges.  Only canonical entries are tested.
//  * Negated faces in clipping.  The world normal of a non-canonical face is
//    the exact negation of its canonical twin's, and so is its dot product.
//  * Box projection.  A box hull's vertices are all sign combinations of
//    (sx, sy, sz), each v.x*a.x is exact in binary64, and rounding is
//    monotonic, so the largest vertex projection is fl(fl(|sx ax| +
//    |sy ay|) + |sz az|) and the smallest is its negation.
#pragma once
#include "cp_math.cuh"
#include "cp_types.h"

struct d4 { double x, y, z, w; };

DI d4 d4of(q4 q) { return d4{F(q.x), F(q.y), F(q.z), F(q.w)}; }

DI d3 dvmult(d4 q, d3 v) {  // Quat.vmult with the Vector3 store (q, v binary32 values)
  double x = v.x, y = v.y, z = v.z;
  double qx = q.x, qy = q.y, qz = q.z, qw = q.w;
  double ix = fma_ff(-qz, y, fma_ff(qy, z, qw * x));
  double iy = fma_ff(-qx, z, fma_ff(qz, x, qw * y));
  double iz = fma_ff(-qy, x, fma_ff(qx, y, qw * z));
  double iw = fma_ff(-qz, z, fma_ff(-qy, y, -qx * x));
  return d3{r32(ix * qw + iw * -qx + iy * -qz - iz * -qy), r32(iy * qw + iw * -qy + iz * -qx - ix * -qz),
            r32(iz * qw + iw * -qz + ix * -qy - iy * -qx)};
}
DI d3 dneg(d3 v) { return d3{-v.x, -v.y, -v.z}; }
DI d3 dadd(d3 a, d3 b) { return d3{r32(a.x + b.x), r32(a.y + b.y), r32(a.z + b.z)}; }
DI d3 dsub(d3 a, d3 b) { return d3{r32(a.x - b.x), r32(a.y - b.y), r32(a.z - b.z)}; }
DI d3 dscale(d3 a, double s) { return d3{r32(s * a.x), r32(s * a.y), r32(s * a.z)}; }
DI d3 dcross(d3 a, d3 v) {  // binary32 values: each difference of exact products rounds once
  return d3{r32(fma_ff(a.y, v.z, -(a.z * v.y))), r32(fma_ff(a.z, v.x, -(a.x * v.z))), r32(fma_ff(a.x, v.y, -(a.y * v.x)))};
}
DI d3 dnormalized(d3 v) {
  double l = sqrt(ddot(v, v));
  if (l == 0.0) return v;
  double d = 1.0 / l;
  return d3{r32(v.x * d), r32(v.y * d), r32(v.z * d)};
}
DI bool dalmost_zero(d3 a) { return !(fabs(a.x) > 1e-6 || fabs(a.y) > 1e-6 || fabs(a.z) > 1e-6); }
DI d3 dlerp(d3 a, d3 v, double t) { return d3{r32(a.x + (v.x - a.x) * t), r32(a.y + (v.y - a.y) * t), r32(a.z + (v.z - a.z) * t)}; }
DI d3 hvd(const DWorld& W, int i) { return ldd3(W.hvd + 4 * i); }

struct DHullPose {
  DHull H;
  d3 x;
  d4 q;
  d3 origin;  // Transform.pointToLocalFrame(pos, quat, 0)
};

// ConvexPolyhedron.project
DI void dproject(const DWorld& W, const DHullPose& h, d3 axis, double& mx, double& mn) {
  d3 la = dvmult(d4{h.q.x, h.q.y, h.q.z, -h.q.w}, axis);
  double addv = ddot(h.origin, la);
  double max, min;
  if (h.H.is_box) {
    double a = fabs(h.H.he[0] * la.x), b = fabs(h.H.he[1] * la.y), c = fabs(h.H.he[2] * la.z);
    max = (a + b) + c;
    min = -max;
  } else {
    max = ddot(hvd(W, h.H.v0), la);
    min = max;
    for (int i = 1; i < h.H.nv; i++) {
      double v = ddot(hvd(W, h.H.v0 + i), la);
      if (v > max) max = v;
      if (v < min) min = v;
    }
  }
  min -= addv;
  max -= addv;
  if (min > max) { double t = min; min = max; max = t; }
  mx = max;
  mn = min;
}

DI bool dtest_sep_axis(const DWorld& W, const DHullPose& A, const DHullPose& B, d3 axis, double& depth) {
  double maxA, minA, maxB, minB;
  dproject(W, A, axis, maxA, minA);
  dproject(W, B, axis, maxB, minB);
  if (maxA < minB || maxB < minA) return false;
  double d0 = maxA - minB, d1 = maxB - minA;
  depth = d0 < d1 ? d0 : d1;
  return true;
}

// world normal of face f given the canonical world normals wn[] (indexed by face)
DI d3 face_wn(const DWorld& W, const DHull& H, const d3* wn, int f) {
  int c = W.faces[H.f0 + f].canon;
  return c == f ? wn[f] : dneg(wn[c]);
}

DI bool dfind_separating_axis(const DWorld& W, const DHullPose& A, const DHullPose& B, const d3* wnA, const d3* wnB, d3& target) {
  double dmin = __longlong_as_double(0x7ff0000000000000LL);
  double d;
  if (A.H.has_axes)
    for (int k = 0; k < A.H.ncf; k++) {
      int f = W.hcanon[A.H.cf0 + k];
      if (!dtest_sep_axis(W, A, B, wnA[f], d)) return false;
      if (d < dmin) { dmin = d; target = wnA[f]; }
    }
  if (B.H.has_axes)
    for (int k = 0; k < B.H.ncf; k++) {
      int f = W.hcanon[B.H.cf0 + k];
      if (!dtest_sep_axis(W, A, B, wnB[f], d)) return false;
      if (d < dmin) { dmin = d; target = wnB[f]; }
    }
  d3 weB[CP_MAX_HULL_VERTS];
  for (int k = 0; k < B.H.nce; k++) weB[k] = dvmult(B.q, ldd3(W.hed + 4 * (B.H.e0 + W.hcanon[B.H.ce0 + k])));
  for (int k0 = 0; k0 < A.H.nce; k0++) {
    d3 we0 = dvmult(A.q, ldd3(W.hed + 4 * (A.H.e0 + W.hcanon[A.H.ce0 + k0])));
    for (int k1 = 0; k1 < B.H.nce; k1++) {
      d3 cr = dcross(we0, weB[k1]);
      if (!dalmost_zero(cr)) {
        cr = dnormalized(cr);
        if (!dtest_sep_axis(W, A, B, cr, d)) return false;
        if (d < dmin) { dmin = d; target = cr; }
      }
    }
  }
  d3 deltaC = dsub(B.x, A.x);
  if (ddot(deltaC, target) > 0.0) target = dneg(target);
  return true;
}

DI int dclip_face_against_plane(const d3* in, int nin, d3* out, d3 n, double c) {
  if (nin < 2) return 0;
  int nout = 0;
  d3 first = in[nin - 1];
  double nDotFirst = ddot(n, first) + c;
  for (int vi = 0; vi < nin; vi++) {
    d3 last = in[vi];
    double nDotLast = ddot(n, last) + c;
    // the reference's four cases (first/last behind the plane or not) emit
    // the crossing point when exactly one is behind, then `last` when it is
    // behind; one code path for the crossing keeps the division out of two
    // divergent branches
    if ((nDotFirst < 0) != (nDotLast < 0)) {
      if (nout < CP_MAX_CLIP) out[nout] = dlerp(first, last, nDotFirst / (nDotFirst - nDotLast));
      nout++;
    }
    if (nDotLast < 0) {
      if (nout < CP_MAX_CLIP) out[nout] = last;
      nout++;
    }
    first = last;
    nDotFirst = nDotLast;
  }
  return nout;
}

// ---------------------------------------------------------------------------
// findSeparatingAxis with a binary32 filter.
//
// Pass 1 estimates, in binary32, the depth testSepAxis would return on every
// axis of the reference's list (canonical face normals of A, of B, then the
// edge crosses), with an absolute error bound E.  An axis estimated below -E
// separates the hulls for certain: the reference returns false too (at that
// axis or an earlier one).  Otherwise U = min(estimate + E) bounds the
// smallest true depth from above, and U >= 0.
// Pass 2 walks the list again in the reference's order and evaluates in
// binary64, exactly as the reference does, only the axes whose estimate is
// within E of U from below (d - E <= U: candidates for the first strict
// minimum; this includes every axis that might separate, since U >= 0) and
// the edge pairs whose binary32 cross product is too short for a reliable
// direction (near-parallel edges, where the reference's almostZero test
// decides).  An axis left out has a true depth above the true minimum and
// above zero, so it neither separates the hulls nor is chosen; the chosen
// axis and the separation verdict are the reference's, bit for bit.
//
// E: both evaluations round binary32 inputs.  The binary32 projections of
// the two centres each carry a few ulps of |x|, about 3e-7 |x|1; the axis
// direction errs by at most ~1.2e-5 (an edge axis from a cross product of
// length >= SAT_EDGE_MIN; face axes far less), which moves a depth by that
// times the centres' offset and the extents; the hull projections add a few
// ulps of the extents.  E = 4e-6 (|xA|1 + |xB|1) + 4e-5 (|xA - xB|1 + rA +
// rB) + 1e-6 covers these about tenfold; the largest binary32 depth error
// measured over 3 M hull pairs of contact-heavy scenes was a tenth of it.
#define SAT_EDGE_MIN 0.05f

// binary32 [lo, hi] of a hull's projection on unit world axis a
DI void proj32(const DWorld& W, const DHull& H, f3 x, q4 q, const f3* ax, f3 a, float& lo, float& hi) {
  const float c = dot32(a, x);
  if (H.is_box) {
    const float r = fabsf(dot32(a, ax[0])) * (float)H.he[0] + fabsf(dot32(a, ax[1])) * (float)H.he[1] +
                    fabsf(dot32(a, ax[2])) * (float)H.he[2];
    lo = c - r;
    hi = c + r;
    return;
  }
  const f3 la = rot32(q4{-q.x, -q.y, -q.z, q.w}, a);
  float mn = __int_as_float(0x7f800000), mx = -mn;
  for (int i = 0; i < H.nv; i++) {
    const float* v = W.hverts + 4 * (H.v0 + i);
    const float p = la.x * v[0] + la.y * v[1] + la.z * v[2];
    mn = fminf(mn, p);
    mx = fmaxf(mx, p);
  }
  lo = c + mn;
  hi = c + mx;
}

struct Sat32 {
  const DWorld* W;
  const DHull *A, *B;
  f3 xA, xB;
  q4 qA, qB;
  f3 axA[3], axB[3];  // box axes in the world frame
  float E;
  DI float depth(f3 a) const {
    float loA, hiA, loB, hiB;
    proj32(*W, *A, xA, qA, axA, a, loA, hiA);
    proj32(*W, *B, xB, qB, axB, a, loB, hiB);
    return fminf(hiA - loB, hiB - loA);
  }
  DI f3 face(const DHull& H, q4 q, int k) const {
    const float* n = W->faces[H.f0 + W->hcanon[H.cf0 + k]].normal;
    return rot32(q, f3{n[0], n[1], n[2]});
  }
  DI f3 edge(const DHull& H, q4 q, int k) const {
    const float* e = W->hedges + 4 * (H.e0 + W->hcanon[H.ce0 + k]);
    return rot32(q, f3{e[0], e[1], e[2]});
  }
};

DI f3 cross32(f3 a, f3 b) { return f3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
DI float maxabs32(f3 a) { return fmaxf(fabsf(a.x), fmaxf(fabsf(a.y), fabsf(a.z))); }

// Pass 1; returns false when an axis separates the hulls for certain.
DI bool sat32_bound(const Sat32& S, float& U) {
  U = __int_as_float(0x7f800000);
  const DHull& A = *S.A;
  const DHull& B = *S.B;
  if (A.has_axes)
    for (int k = 0; k < A.ncf; k++) {
      float d = S.depth(S.face(A, S.qA, k));
      if (d < -S.E) return false;
      U = fminf(U, d + S.E);
    }
  if (B.has_axes)
    for (int k = 0; k < B.ncf; k++) {
      float d = S.depth(S.face(B, S.qB, k));
      if (d < -S.E) return false;
      U = fminf(U, d + S.E);
    }
  for (int k0 = 0; k0 < A.nce; k0++) {
    const f3 e0 = S.edge(A, S.qA, k0);
    for (int k1 = 0; k1 < B.nce; k1++) {
      const f3 cr = cross32(e0, S.edge(B, S.qB, k1));
      if (maxabs32(cr) < SAT_EDGE_MIN) continue;  // decided exactly in pass 2
      const float l = len32(cr);
      float d = S.depth(f3{cr.x / l, cr.y / l, cr.z / l});
      if (d < -S.E) return false;
      U = fminf(U, d + S.E);
    }
  }
  return true;
}

// Pass 2: the reference's loop over the candidate axes only.
DI bool sat64_candidates(const DWorld& W, const DHullPose& A, const DHullPose& B, const d3* wnA, const d3* wnB,
                         const Sat32& S, float U, d3& target) {
  double dmin = __longlong_as_double(0x7ff0000000000000LL);
  double d;
  if (A.H.has_axes)
    for (int k = 0; k < A.H.ncf; k++) {
      if (S.depth(S.face(A.H, S.qA, k)) - S.E > U) continue;
      const d3 ax = wnA[W.hcanon[A.H.cf0 + k]];
      if (!dtest_sep_axis(W, A, B, ax, d)) return false;
      if (d < dmin) { dmin = d; target = ax; }
    }
  if (B.H.has_axes)
    for (int k = 0; k < B.H.ncf; k++) {
      if (S.depth(S.face(B.H, S.qB, k)) - S.E > U) continue;
      const d3 ax = wnB[W.hcanon[B.H.cf0 + k]];
      if (!dtest_sep_axis(W, A, B, ax, d)) return false;
      if (d < dmin) { dmin = d; target = ax; }
    }
  for (int k0 = 0; k0 < A.H.nce; k0++) {
    const f3 e0 = S.edge(A.H, S.qA, k0);
    bool have0 = false;
    d3 we0;
    for (int k1 = 0; k1 < B.H.nce; k1++) {
      const f3 cr32 = cross32(e0, S.edge(B.H, S.qB, k1));
      if (maxabs32(cr32) >= SAT_EDGE_MIN) {
        const float l = len32(cr32);
        if (S.depth(f3{cr32.x / l, cr32.y / l, cr32.z / l}) - S.E > U) continue;
      }
      if (!have0) {
        we0 = dvmult(A.q, ldd3(W.hed + 4 * (A.H.e0 + W.hcanon[A.H.ce0 + k0])));
        have0 = true;
      }
      d3 cr = dcross(we0, dvmult(B.q, ldd3(W.hed + 4 * (B.H.e0 + W.hcanon[B.H.ce0 + k1]))));
      if (dalmost_zero(cr)) continue;
      cr = dnormalized(cr);
      if (!dtest_sep_axis(W, A, B, cr, d)) return false;
      if (d < dmin) { dmin = d; target = cr; }
    }
  }
  d3 deltaC = dsub(B.x, A.x);
  if (ddot(deltaC, target) > 0.0) target = dneg(target);
  return true;
}

// Pass 2 with the candidates first gathered into a short list (indices into
// the reference's axis order: A faces, B faces, then edge pairs k0-major).
// Lanes of a warp hold different candidates; walking each lane's list in
// rounds runs the binary64 axis test of all lanes together instead of once
// per distinct list position.  More than SAT_MAXC candidates: the walk of
// the whole list (sat64_candidates) decides.
#define SAT_MAXC 8
DI bool sat64_compact(const DWorld& W, const DHullPose& A, const DHullPose& B, const d3* wnA, const d3* wnB,
                      const Sat32& S, float U, d3& target) {
  int cand[SAT_MAXC];
  int nc = 0;
  bool over = false;
  const int nfa = A.H.has_axes ? A.H.ncf : 0, nfb = B.H.has_axes ? B.H.ncf : 0;
  for (int k = 0; k < nfa; k++)
    if (!(S.depth(S.face(A.H, S.qA, k)) - S.E > U)) { if (nc < SAT_MAXC) cand[nc++] = k; else over = true; }
  for (int k = 0; k < nfb; k++)
    if (!(S.depth(S.face(B.H, S.qB, k)) - S.E > U)) { if (nc < SAT_MAXC) cand[nc++] = nfa + k; else over = true; }
  for (int k0 = 0; k0 < A.H.nce; k0++) {
    const f3 e0 = S.edge(A.H, S.qA, k0);
    for (int k1 = 0; k1 < B.H.nce; k1++) {
      const f3 cr32 = cross32(e0, S.edge(B.H, S.qB, k1));
      if (maxabs32(cr32) >= SAT_EDGE_MIN) {
        const float l = len32(cr32);
        if (S.depth(f3{cr32.x / l, cr32.y / l, cr32.z / l}) - S.E > U) continue;
      }
      if (nc < SAT_MAXC) cand[nc++] = nfa + nfb + k0 * B.H.nce + k1; else over = true;
    }
  }
  if (over) return sat64_candidates(W, A, B, wnA, wnB, S, U, target);
  double dmin = __longlong_as_double(0x7ff0000000000000LL);
  double d;
  for (int j = 0; j < nc; j++) {
    const int idx = cand[j];
    d3 ax;
    if (idx < nfa) {
      ax = wnA[W.hcanon[A.H.cf0 + idx]];
    } else if (idx < nfa + nfb) {
      ax = wnB[W.hcanon[B.H.cf0 + idx - nfa]];
    } else {
      const int e = idx - nfa - nfb, k0 = e / B.H.nce, k1 = e - k0 * B.H.nce;
      const d3 we0 = dvmult(A.q, ldd3(W.hed + 4 * (A.H.e0 + W.hcanon[A.H.ce0 + k0])));
      const d3 cr = dcross(we0, dvmult(B.q, ldd3(W.hed + 4 * (B.H.e0 + W.hcanon[B.H.ce0 + k1]))));
      if (dalmost_zero(cr)) continue;
      ax = dnormalized(cr);
    }
    if (!dtest_sep_axis(W, A, B, ax, d)) return false;
    if (d < dmin) { dmin = d; target = ax; }
  }
  d3 deltaC = dsub(B.x, A.x);
  if (ddot(deltaC, target) > 0.0) target = dneg(target);
  return true;
}

// Stage 1 of convexConvex: the bounding spheres (narrow_phase.dart:1994) and
// the binary32 bound of findSeparatingAxis.  False: the reference finds no
// contact for certain.  Cheap and run for every queued hull pair first, so
// that the binary64 stage runs on the survivors in full warps.
// The binary32 SAT context of a pair (world axes, error margin E); false
// when the bounding spheres are apart.
DI bool cc_setup32(const DWorld& W, int shA, int shB, f3 xAf, f3 xBf, q4 qAf, q4 qBf, Sat32& S32) {
  const DShape& SA = W.shapes[shA];
  const DShape& SB = W.shapes[shB];
  if (distance_to(xAf, xBf) > SA.bsr + SB.bsr) return false;
  S32.W = &W;
  S32.A = &W.hulls[SA.hull];
  S32.B = &W.hulls[SB.hull];
  S32.xA = xAf; S32.xB = xBf; S32.qA = qAf; S32.qB = qBf;
  S32.axA[0] = rot32(qAf, f3{1.f, 0.f, 0.f}); S32.axA[1] = rot32(qAf, f3{0.f, 1.f, 0.f}); S32.axA[2] = rot32(qAf, f3{0.f, 0.f, 1.f});
  S32.axB[0] = rot32(qBf, f3{1.f, 0.f, 0.f}); S32.axB[1] = rot32(qBf, f3{0.f, 1.f, 0.f}); S32.axB[2] = rot32(qBf, f3{0.f, 0.f, 1.f});
  S32.E = 4e-6f * (fabsf(xAf.x) + fabsf(xAf.y) + fabsf(xAf.z) + fabsf(xBf.x) + fabsf(xBf.y) + fabsf(xBf.z)) +
          4e-5f * (fabsf(xAf.x - xBf.x) + fabsf(xAf.y - xBf.y) + fabsf(xAf.z - xBf.z) + (float)(SA.bsr + SB.bsr)) + 1e-6f;
  return true;
}
DI bool cc_stage1(const DWorld& W, int shA, int shB, f3 xAf, f3 xBf, q4 qAf, q4 qBf, Sat32& S32, float& U) {
  return cc_setup32(W, shA, shB, xAf, xBf, qAf, qBf, S32) && sat32_bound(S32, U);
}

// ---------------------------------------------------------------------------
// Filter check (a test switch, off by default).  With g_filter_check set,
// every decision a binary32 filter takes for a hull pair is compared with the
// reference's unfiltered binary64 walk (dfind_separating_axis: every axis in
// the reference's order): the separation verdict and, for touching hulls,
// the chosen axis bit for bit.  g_filter_count: {pairs checked, pairs that
// disagree}.  Per translation unit (the one-block and the wide kernels each
// keep their own).
static __device__ int g_filter_check;
static __device__ unsigned long long g_filter_count[2];
static __device__ int g_filter_sink[2];  // cursor and overflow flag of a count-only resolver context

DI bool same_bits(d3 a, d3 b) {
  return __double_as_longlong(a.x) == __double_as_longlong(b.x) && __double_as_longlong(a.y) == __double_as_longlong(b.y) &&
         __double_as_longlong(a.z) == __double_as_longlong(b.z);
}

// touch / sep: what the filtered path decided for the pair (sep: the axis
// after the flip toward A, when touching)
static __device__ __noinline__ void cc_filter_check(const DWorld& W, int shA, int shB, f3 xAf, f3 xBf, q4 qAf, q4 qBf,
                                                    bool touch, d3 sep) {
  const DShape& SA = W.shapes[shA];
  const DShape& SB = W.shapes[shB];
  DHullPose A, B;
  A.H = W.hulls[SA.hull]; A.x = d3of(xAf); A.q = d4of(qAf);
  B.H = W.hulls[SB.hull]; B.x = d3of(xBf); B.q = d4of(qBf);
  if (A.H.nf > CP_MAX_HULL_VERTS || B.H.nf > CP_MAX_HULL_VERTS || B.H.nce > CP_MAX_HULL_VERTS) return;
  A.origin = dvmult(d4{-A.q.x, -A.q.y, -A.q.z, A.q.w}, dsub(d3{0.0, 0.0, 0.0}, A.x));
  B.origin = dvmult(d4{-B.q.x, -B.q.y, -B.q.z, B.q.w}, dsub(d3{0.0, 0.0, 0.0}, B.x));
  d3 wnA[CP_MAX_HULL_VERTS], wnB[CP_MAX_HULL_VERTS];
  for (int k = 0; k < A.H.ncf; k++) {
    int f = W.hcanon[A.H.cf0 + k];
    wnA[f] = dvmult(A.q, ldd3(W.faces[A.H.f0 + f].dnormal));
  }
  for (int k = 0; k < B.H.ncf; k++) {
    int f = W.hcanon[B.H.cf0 + k];
    wnB[f] = dvmult(B.q, ldd3(W.faces[B.H.f0 + f].dnormal));
  }
  d3 t = d3{0.0, 0.0, 0.0};
  const bool ref = dfind_separating_axis(W, A, B, wnA, wnB, t);
  const bool same = ref == touch && (!ref || same_bits(t, sep));
  atomicAdd(&g_filter_count[0], 1ull);
  if (!same) atomicAdd(&g_filter_count[1], 1ull);
}

// Narrowphase.convexConvex (narrow_phase.dart:1981-2043).  Lanes leave at
// data-dependent points (the stage-1 test, the binary64 separating-axis
// walk); a ballot over the lanes that entered together at each such point
// regroups the survivors, so the clipping that follows issues its binary64
// instructions once for all of them instead of once per group of lanes
// that happened to leave a loop together.  Past the last ballot no lane
// returns early (failures set a flag), so the survivors stay together.
// One out-of-line copy: the resolver is large and is reached from several
// dispatch cases; inlining it at each bloats the step kernel's instruction footprint.
// U1: the bound U that stage 1 already found for this pair, or NaN.
static __device__ __noinline__ int convex_convex(const NarrowCtx& C, int bA, int bB, int shA, int shB, int rsi, int rsj, f3 xAf, f3 xBf, q4 qAf, q4 qBf, int& start, float U1) {
  const DWorld& W = *C.W;
  const DShape& SA = W.shapes[shA];
  const DShape& SB = W.shapes[shB];
  unsigned lanes = __activemask();
  Sat32 S32;
  float U = U1;
  const bool near = U1 == U1 ? cc_setup32(W, shA, shB, xAf, xBf, qAf, qBf, S32) : cc_stage1(W, shA, shB, xAf, xBf, qAf, qBf, S32, U);
  lanes = __ballot_sync(lanes, near);
  if (!near) {
    // a binary32 separation certificate (not the bounding spheres, which are
    // the reference's own test) is checked against the full walk
    if (g_filter_check && !(distance_to(xAf, xBf) > SA.bsr + SB.bsr))
      cc_filter_check(W, shA, shB, xAf, xBf, qAf, qBf, false, d3{0.0, 0.0, 0.0});
    return 0;
  }
  DHullPose A, B;
  A.H = W.hulls[SA.hull]; A.x = d3of(xAf); A.q = d4of(qAf);
  B.H = W.hulls[SB.hull]; B.x = d3of(xBf); B.q = d4of(qBf);
  A.origin = dvmult(d4{-A.q.x, -A.q.y, -A.q.z, A.q.w}, dsub(d3{0.0, 0.0, 0.0}, A.x));
  B.origin = dvmult(d4{-B.q.x, -B.q.y, -B.q.z, B.q.w}, dsub(d3{0.0, 0.0, 0.0}, B.x));
  const bool fits = !(A.H.nf > CP_MAX_HULL_VERTS || B.H.nf > CP_MAX_HULL_VERTS || B.H.nce > CP_MAX_HULL_VERTS);
  if (!fits) atomicOr(C.overflow, ST_HULL_OVERFLOW);
  d3 wnA[CP_MAX_HULL_VERTS], wnB[CP_MAX_HULL_VERTS];
  d3 sep = d3{0.0, 0.0, 0.0};
  bool touch = false;
  if (fits) {
    for (int k = 0; k < A.H.ncf; k++) {
      int f = W.hcanon[A.H.cf0 + k];
      wnA[f] = dvmult(A.q, ldd3(W.faces[A.H.f0 + f].dnormal));
    }
    for (int k = 0; k < B.H.ncf; k++) {
      int f = W.hcanon[B.H.cf0 + k];
      wnB[f] = dvmult(B.q, ldd3(W.faces[B.H.f0 + f].dnormal));
    }
    touch = sat64_compact(W, A, B, wnA, wnB, S32, U, sep);
    if (g_filter_check) cc_filter_check(W, shA, shB, xAf, xBf, qAf, qBf, touch, sep);
  }
  lanes = __ballot_sync(lanes, touch);
  if (!touch) return 0;
  bool fail = false;
  // clipAgainstHull: face of B most aligned with the axis
  int cfb = -1;
  double dmax = __longlong_as_double(0xfff0000000000000LL);
  for (int f = 0; f < B.H.nf; f++) {
    double d = ddot(face_wn(W, B.H, wnB, f), sep);
    if (d > dmax) { dmax = d; cfb = f; }
  }
  fail = cfb < 0;
  d3 bufA[CP_MAX_CLIP], bufB[CP_MAX_CLIP];
  const DFace FB = W.faces[B.H.f0 + (fail ? 0 : cfb)];
  if (!fail && FB.n > CP_MAX_CLIP) {
    atomicOr(C.overflow, ST_HULL_OVERFLOW);
    fail = true;
  }
  int nin = fail ? 0 : FB.n;
  for (int i = 0; i < nin; i++) bufA[i] = dadd(dvmult(B.q, hvd(W, B.H.v0 + W.hfi[FB.i0 + i])), B.x);
  // clipFaceAgainstHull: face of A most anti-aligned with the axis
  int cfa = -1;
  double dmin = __longlong_as_double(0x7ff0000000000000LL);
  for (int f = 0; f < A.H.nf; f++) {
    double d = ddot(face_wn(W, A.H, wnA, f), sep);
    if (d < dmin) { dmin = d; cfa = f; }
  }
  fail = fail || cfa < 0;
  const DFace FA = W.faces[A.H.f0 + (cfa < 0 ? 0 : cfa)];
  d3* pin = bufA;
  d3* pout = bufB;
  const int nplanes = fail ? 0 : FA.n;
  for (int i = 0; i < nplanes && !fail; i++) {
    int other = FA.nc > i ? W.hconn[FA.c0 + i] : 0;
    d3 pn = face_wn(W, A.H, wnA, other);
    double planeEqWS = W.faces[A.H.f0 + other].plane_const - ddot(pn, A.x);
    int nout = dclip_face_against_plane(pin, nin, pout, pn, planeEqWS);
    if (nout > CP_MAX_CLIP) {
      atomicOr(C.overflow, ST_HULL_OVERFLOW);
      fail = true;
    }
    d3* t = pin; pin = pout; pout = t;
    nin = nout;
  }
  __syncwarp(lanes);
  if (fail) nin = 0;
  d3 pn = face_wn(W, A.H, wnA, cfa < 0 ? 0 : cfa);
  double planeEqWS = FA.plane_const - ddot(pn, A.x);
  double depth[CP_MAX_CLIP];
  int n = 0;
  for (int i = 0; i < nin; i++) {
    double dd = ddot(pn, pin[i]) + planeEqWS;
    if (dd <= -100.0) dd = -100.0;
    depth[i] = dd;
    if (dd <= 100.0 && dd <= 1e-6) n++;
  }
  if (n == 0) return 0;
  start = reserve(C, n);
  if (start < 0) return n;
  const DBody& BA = W.bodies[bA];
  const DBody& BB = W.bodies[bB];
  d3 ni = dneg(sep);
  d3 pa = d3of(ld3(BA.pos)), pb = d3of(ld3(BB.pos));
  const ContactHead head = contact_head(C, bA, bB, shA, shB, rsi, rsj);
  int k = 0;
  for (int i = 0; i < nin; i++) {
    double dd = depth[i];
    if (dd <= 100.0 && dd <= 1e-6) {
      d3 q = dscale(dneg(pn), dd);
      d3 ri = dadd(pin[i], q);
      d3 rj = pin[i];
      ri = dsub(ri, A.x);
      rj = dsub(rj, B.x);
      ri = dsub(dadd(ri, A.x), pa);
      rj = dsub(dadd(rj, B.x), pb);
      ContactOut g;
      g.ni = f3{(float)ni.x, (float)ni.y, (float)ni.z};
      g.ri = f3{(float)ri.x, (float)ri.y, (float)ri.z};
      g.rj = f3{(float)rj.x, (float)rj.y, (float)rj.z};
      put_contact(W.ctmp[start + k], head, g);
      k++;
    }
  }
  return n;
}
