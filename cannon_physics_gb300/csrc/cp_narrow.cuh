// cp_narrow.cuh -- narrowphase resolvers (lib/world/narrow_phase.dart and
// lib/rigid_body_shapes/convex_polyhedron.dart), one thread per body pair.
//
// A resolver computes the contacts of one pair into registers / local memory,
// counts them, reserves that many slots in the world's contact staging area
// with one shared-memory atomic, and writes them.  The caller records
// (count, first slot) per pair; a block scan over the counts then puts every
// contact at the place the reference appends it (pair order, then resolver
// order).
#pragma once
#include "cp_math.cuh"
#include "cp_types.h"

struct NarrowCtx {
  const DWorld* W;
  int* cursor;     // shared-memory slot cursor of the staging area
  int cap;
  int* overflow;   // shared flag
  int cm;          // contact material index (currentContactMaterial)
  int pair;
};

struct ContactOut {
  f3 ni, ri, rj;
};

// narrow_phase.dart:492-528 createContactEquation: everything except the
// geometry.  shA/shB are the shapes handed to the resolver (type order),
// rsi/rsj the shapes ContactEquation.si/.sj end up holding.
// The fields a pair's contacts share (Narrowphase.createContactEquation,
// narrow_phase.dart:489-528): bodies, shapes, response flag, material and
// restitution; computed once per pair, not once per contact.
struct ContactHead {
  int bi, bj, si, sj, enabled, pair, cm;
  double restitution;
};
DI ContactHead contact_head(const NarrowCtx& C, int bA, int bB, int shA, int shB, int rsi, int rsj) {
  const DWorld& W = *C.W;
  const DBody& A = W.bodies[bA];
  const DBody& B = W.bodies[bB];
  const DShape& SA = W.shapes[shA];
  const DShape& SB = W.shapes[shB];
  ContactHead h;
  h.bi = bA; h.bj = bB; h.si = rsi; h.sj = rsj;
  h.enabled = (A.flags & BF_RESPONSE) && (B.flags & BF_RESPONSE) && SA.response && SB.response;
  h.pair = C.pair;
  h.cm = C.cm;
  double rest = W.cms[C.cm].restitution;
  int ma = SA.material >= 0 ? SA.material : A.material;
  int mb = SB.material >= 0 ? SB.material : B.material;
  if (ma >= 0 && mb >= 0 && W.mats[ma].restitution >= 0 && W.mats[mb].restitution >= 0)
    rest = W.mats[ma].restitution * W.mats[mb].restitution;
  h.restitution = rest;
  return h;
}
DI void put_contact(DContact& c, const ContactHead& h, const ContactOut& g) {
  c.bi = h.bi; c.bj = h.bj; c.si = h.si; c.sj = h.sj;
  st3(c.ni, g.ni); st3(c.ri, g.ri); st3(c.rj, g.rj);
  c.enabled = h.enabled;
  c.pair = h.pair;
  c.cm = h.cm;
  c.frow = -1;
  c.slip = 0.0;
  c.restitution = h.restitution;
}
DI void fill_contact(const NarrowCtx& C, DContact& c, int bA, int bB, int shA, int shB, int rsi, int rsj, const ContactOut& g) {
  put_contact(c, contact_head(C, bA, bB, shA, shB, rsi, rsj), g);
}

// cap == 0: a context that only counts contacts (the filter check), never
// writes them
DI int reserve(const NarrowCtx& C, int n) {
  if (n == 0) return 0;
  if (C.cap <= 0) return -1;
  int s = atomicAdd(C.cursor, n);
  if (s + n > C.cap) { atomicOr(C.overflow, ST_CONTACTS_OVERFLOW); return -1; }
  return s;
}

// "Make it relative to the body": r += x - body.position
DI f3 rel(f3 r, f3 x, const DBody& b) { return sub(add(r, x), ld3(b.pos)); }

// narrow_phase.dart:723-765
DI int sphere_sphere(const NarrowCtx& C, int bA, int bB, int shA, int shB, int rsi, int rsj, f3 xA, f3 xB, int& start) {
  const DWorld& W = *C.W;
  ContactOut g;
  g.ni = normalized(sub(xB, xA));
  g.ri = scale(g.ni, W.shapes[shA].radius);
  g.rj = scale(g.ni, -W.shapes[shB].radius);
  g.ri = rel(g.ri, xA, W.bodies[bA]);
  g.rj = rel(g.rj, xB, W.bodies[bB]);
  start = reserve(C, 1);
  if (start >= 0) fill_contact(C, W.ctmp[start], bA, bB, shA, shB, rsi, rsj, g);
  return 1;
}

// narrow_phase.dart:766-815
DI int sphere_plane(const NarrowCtx& C, int bA, int bB, int shA, int shB, int rsi, int rsj, f3 xA, f3 xB, q4 qB, int& start) {
  const DWorld& W = *C.W;
  double R = W.shapes[shA].radius;
  ContactOut g;
  g.ni = normalized(neg(vmult(qB, f3{0.f, 0.f, 1.f})));
  g.ri = scale(g.ni, R);
  f3 pops = sub(xA, xB);
  f3 ortho = scale(g.ni, dot(g.ni, pops));
  g.rj = sub(pops, ortho);
  if (!(-dot(pops, g.ni) <= R)) return 0;
  g.ri = rel(g.ri, xA, W.bodies[bA]);
  g.rj = rel(g.rj, xB, W.bodies[bB]);
  start = reserve(C, 1);
  if (start >= 0) fill_contact(C, W.ctmp[start], bA, bB, shA, shB, rsi, rsj, g);
  return 1;
}

// binary32 helpers of the no-contact tests and plans (approximate: every
// use carries an error margin)
DI f3 rot32(q4 q, f3 v) {  // binary32 rotation (approximate)
  float ix = q.w * v.x + q.y * v.z - q.z * v.y;
  float iy = q.w * v.y + q.z * v.x - q.x * v.z;
  float iz = q.w * v.z + q.x * v.y - q.y * v.x;
  float iw = -q.x * v.x - q.y * v.y - q.z * v.z;
  return f3{ix * q.w - iw * q.x - iy * q.z + iz * q.y, iy * q.w - iw * q.y - iz * q.x + ix * q.z,
            iz * q.w - iw * q.z - ix * q.y + iy * q.x};
}
DI float dot32(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
DI float len32(f3 a) { return sqrtf(dot32(a, a)); }

// True when the sphere clearly misses the box, decided in binary32.  Every
// branch of the reference's sphereBox that makes a contact puts a point of the
// box (a side point with |d1| < h1, |d2| < h2, a corner, or an edge point with
// |t| < h) within R of the sphere centre, so a centre farther than R + E from
// the box makes none.  The binary32 distance differs from the exact one by a
// few ulps of the box size, of |b2s| and of the positions; E is a wide margin
// over all three.
DI bool sphere_box_far(f3 xA, float R, f3 xB, q4 qB, const float* he) {
  const f3 b2s = f3{xA.x - xB.x, xA.y - xB.y, xA.z - xB.z};
  const f3 p = rot32(q4{-qB.x, -qB.y, -qB.z, qB.w}, b2s);  // centre in the box frame
  const float E = 1e-4f * (R + he[0] + he[1] + he[2] + fabsf(b2s.x) + fabsf(b2s.y) + fabsf(b2s.z)) +
                  4e-7f * (fabsf(xA.x) + fabsf(xA.y) + fabsf(xA.z) + fabsf(xB.x) + fabsf(xB.y) + fabsf(xB.z)) + 1e-6f;
  const float ox = fmaxf(fabsf(p.x) - he[0], 0.f), oy = fmaxf(fabsf(p.y) - he[1], 0.f), oz = fmaxf(fabsf(p.z) - he[2], 0.f);
  const float lim = R + E;
  return ox * ox + oy * oy + oz * oz > lim * lim;
}

DI f3 sb_side(const DShape& sb, q4 qB, int idx) {
  const int a = idx % 3;
  const float s = idx < 3 ? 1.f : -1.f;
  return vmult(qB, f3{a == 0 ? s * sb.he[0] : 0.f, a == 1 ? s * sb.he[1] : 0.f, a == 2 ? s * sb.he[2] : 0.f});
}

// Narrowphase.sphereBox (narrow_phase.dart:816-1038), reached for pairs that
// sphere_box_far does not settle: the reference's binary64 evaluation, with
// one exact shortcut in the side test: side 3 + a is side a
// negated (vmult is odd in its vector and round-to-nearest is symmetric) up to
// the signs of zero components, so its length is that of side a and its dot
// product with b2s is the negated one (or a zero, which the test treats alike);
// the test needs three rotations, three lengths, three normals and three dot
// products (which are also the reference's d1, d2).
// one out-of-line copy: the resolver is large and is reached from several
// dispatch cases; inlining it at each bloats the step kernel's instruction footprint
static __device__ __noinline__ int sphere_box(const NarrowCtx& C, int bA, int bB, int shA, int shB, int rsi, int rsj, f3 xA, f3 xB, q4 qB, int& start) {
  const DWorld& W = *C.W;
  const DShape& sb = W.shapes[shB];
  const double R = W.shapes[shA].radius;
  const f3 b2s = sub(xA, xB);
  f3 sd[3], nrm[3];
  double hl[3], pd[3];
#pragma unroll
  for (int a = 0; a < 3; a++) {
    sd[a] = sb_side(sb, qB, a);
    hl[a] = length(sd[a]);
    nrm[a] = normalized(sd[a]);
    pd[a] = dot(b2s, nrm[a]);
  }
  // sides: the penetrating side of smallest |d - h - R|, the first on ties
  int best = -1;
  double bestDist = 0;
  for (int idx = 0; idx < 6; idx++) {
    const int ax = idx % 3;
    const double h = hl[ax], d = idx < 3 ? pd[ax] : -pd[ax];
    if (!(d < h + R && d > 0)) continue;
    const int i1 = (idx + 1) % 3, i2 = (idx + 2) % 3;
    const double d1 = pd[i1], d2 = pd[i2], h1 = hl[i1], h2 = hl[i2];
    if (d1 < h1 && d1 > -h1 && d2 < h2 && d2 > -h2) {
      const double dist = fabs(d - h - R);
      if (best < 0 || dist < bestDist) {
        best = idx;
        bestDist = dist;
      }
    }
  }
  ContactOut g;
  bool found = false;
  if (best >= 0) {
    found = true;
    const int ax = best % 3, i1 = (best + 1) % 3, i2 = (best + 2) % 3;
    // side 3 + a is rotated from (-h, +0, +0) etc.: its zero components
    // need not be the negated ones of side a, so it is formed as the
    // reference forms it
    const f3 ns = best < 3 ? nrm[ax] : normalized(sb_side(sb, qB, best));
    g.ri = scale(ns, -R);
    g.ni = neg(ns);
    f3 t = scale(ns, hl[ax]);
    t = add(t, scale(nrm[i1], pd[i1]));
    g.rj = add(t, scale(nrm[i2], pd[i2]));
  }
  for (int j = 0; j != 2 && !found; j++)
    for (int k = 0; k != 2 && !found; k++)
      for (int l = 0; l != 2 && !found; l++) {
        f3 rj{0.f, 0.f, 0.f};
        rj = j != 0 ? add(rj, sd[0]) : sub(rj, sd[0]);
        rj = k != 0 ? add(rj, sd[1]) : sub(rj, sd[1]);
        rj = l != 0 ? add(rj, sd[2]) : sub(rj, sd[2]);
        const f3 s2c = sub(add(xB, rj), xA);
        if (length2(s2c) < R * R) {
          found = true;
          g.ri = normalized(s2c);
          g.ni = g.ri;
          g.ri = scale(g.ri, R);
          g.rj = rj;
        }
      }
  f3 sdn[3];
  if (!found)
    for (int a = 0; a < 3; a++) sdn[a] = sb_side(sb, qB, 3 + a);
  for (int j = 0; j != 6 && !found; j++)
    for (int k = 0; k != 6 && !found; k++) {
      if (j % 3 != k % 3) {
        const f3 sj = j < 3 ? sd[j] : sdn[j - 3], sk = k < 3 ? sd[k] : sdn[k - 3];
        const f3 edgeTangent = normalized(cross(sk, sj));
        const f3 edgeCenter = add(sj, sk);
        const f3 r = sub(sub(xA, edgeCenter), xB);
        const double orthonorm = dot(r, edgeTangent);
        const f3 orthogonal = scale(edgeTangent, orthonorm);
        int l = 0;
        while (l == j % 3 || l == k % 3) l++;
        const f3 dist = sub(sub(sub(xA, orthogonal), edgeCenter), xB);
        const double tdist = fabs(orthonorm);
        const double ndist = length(dist);
        if (tdist < hl[l] && ndist < R) {
          found = true;
          g.rj = add(edgeCenter, orthogonal);
          g.ni = normalized(neg(dist));
          const f3 ri = sub(add(g.rj, xB), xA);
          g.ri = scale(normalized(ri), R);
        }
      }
    }
  if (!found) return 0;
  g.ri = rel(g.ri, xA, W.bodies[bA]);
  g.rj = rel(g.rj, xB, W.bodies[bB]);
  start = reserve(C, 1);
  if (start >= 0) fill_contact(C, W.ctmp[start], bA, bB, shA, shB, rsi, rsj, g);
  return 1;
}

// narrow_phase.dart:2584-2617
DI bool point_in_polygon(const f3* verts, int N, f3 normal, f3 p) {
  int state = -1;
  for (int i = 0; i != N; i++) {
    f3 v = verts[i];
    f3 edge = sub(verts[(i + 1) % N], v);
    f3 exn = cross(edge, normal);
    f3 vtp = sub(p, v);
    double r = dot(exn, vtp);
    if (state == -1 || (r > 0 && state == 1) || (r <= 0 && state == 0)) {
      if (state == -1) state = r > 0 ? 1 : 0;
      continue;
    }
    return false;
  }
  return true;
}

DI f3 hv(const DWorld& W, int i) { return ld3(W.hverts + 4 * i); }

// narrow_phase.dart:1039-1257
// one out-of-line copy: the resolver is large and is reached from several
// dispatch cases; inlining it at each bloats the step kernel's instruction footprint
static __device__ __noinline__ int sphere_convex(const NarrowCtx& C, int bA, int bB, int shA, int shB, int rsi, int rsj, f3 xA, f3 xB, q4 qB, int& start) {
  const DWorld& W = *C.W;
  const DHull H = W.hulls[W.shapes[shB].hull];
  double R = W.shapes[shA].radius;
  ContactOut g;
  bool got = false;
  // World vertices, each formed once: the reference forms a vertex's world
  // position anew wherever it uses it (vertex, face and edge tests), with
  // the same operations on the same values, so one copy gives the same bits.
  // The vertex loop fills all of them unless it finds a contact.
  f3 wv[CP_MAX_HULL_VERTS];
  if (H.nv > CP_MAX_HULL_VERTS) { atomicOr(C.overflow, ST_HULL_OVERFLOW); return 0; }
  for (int i = 0; i < H.nv && !got; i++) {
    f3 wc = add(vmult(qB, hv(W, H.v0 + i)), xB);
    wv[i] = wc;
    f3 s2c = sub(wc, xA);
    if (length2(s2c) < R * R) {
      g.ri = normalized(s2c);
      g.ni = g.ri;
      g.ri = scale(g.ri, R);
      g.rj = sub(wc, xB);
      got = true;
    }
  }
  for (int i = 0; i < H.nf && !got; i++) {
    const DFace F = W.faces[H.f0 + i];
    f3 wn = vmult(qB, ld3(F.normal));
    f3 wp = wv[W.hfi[F.i0]];
    f3 wsp = add(xA, scale(wn, -R));
    f3 pv = sub(wsp, wp);
    double pen = dot(pv, wn);
    f3 wp2s = sub(xA, wp);
    if (pen < 0 && dot(wp2s, wn) > 0) {
      f3 fv[CP_MAX_FACE_VERTS];
      if (F.n > CP_MAX_FACE_VERTS) { atomicOr(C.overflow, ST_HULL_OVERFLOW); return 0; }
      int nfv = F.n;
      for (int j = 0; j < nfv; j++) fv[j] = wv[W.hfi[F.i0 + j]];
      if (point_in_polygon(fv, nfv, wn, xA)) {
        g.ri = scale(wn, -R);
        g.ni = neg(wn);
        f3 pv2 = scale(wn, -pen);
        f3 psp = scale(wn, -R);
        f3 rj = sub(xA, xB);
        rj = add(rj, psp);
        rj = add(rj, pv2);
        g.rj = rj;
        got = true;
      } else {
        for (int j = 0; j < nfv && !got; j++) {
          f3 v1 = fv[(j + 1) % nfv];
          f3 v2 = fv[(j + 2) % nfv];
          f3 edge = sub(v2, v1);
          f3 eu = unit(edge);
          f3 v1x = sub(xA, v1);
          double d = dot(v1x, eu);
          f3 p = add(scale(eu, d), v1);
          f3 x2p = sub(p, xA);
          if (d > 0 && d * d < length2(edge) && length2(x2p) < R * R) {
            g.rj = sub(p, xB);
            g.ni = normalized(sub(p, xA));
            g.ri = scale(g.ni, R);
            got = true;
          }
        }
      }
    }
  }
  if (!got) return 0;
  g.ri = rel(g.ri, xA, W.bodies[bA]);
  g.rj = rel(g.rj, xB, W.bodies[bB]);
  start = reserve(C, 1);
  if (start >= 0) fill_contact(C, W.ctmp[start], bA, bB, shA, shB, rsi, rsj, g);
  return 1;
}

// narrow_phase.dart:1847-1915 (planeBox forwards here with its own shapes)
// one out-of-line copy: the resolver is large and is reached from several
// dispatch cases; inlining it at each bloats the step kernel's instruction footprint
static __device__ __noinline__ int plane_convex(const NarrowCtx& C, int bA, int bB, int shA, int shB, int rsi, int rsj, f3 xA, f3 xB, q4 qA, q4 qB, int& start) {
  const DWorld& W = *C.W;
  const DHull H = W.hulls[W.shapes[shB].hull];
  f3 wn = vmult(qA, f3{0.f, 0.f, 1.f});
  f3 wv[CP_MAX_HULL_VERTS];
  double dv[CP_MAX_HULL_VERTS];
  int n = 0;
  if (H.nv > CP_MAX_HULL_VERTS) { atomicOr(C.overflow, ST_HULL_OVERFLOW); return 0; }
  int nv = H.nv;
  for (int i = 0; i < nv; i++) {
    wv[i] = add(vmult(qB, hv(W, H.v0 + i)), xB);
    f3 relpos = sub(wv[i], xA);
    dv[i] = dot(wn, relpos);
    if (dv[i] <= 0.0) n++;
  }
  if (n == 0) return 0;
  start = reserve(C, n);
  if (start < 0) return n;
  const DBody& BA = W.bodies[bA];
  const DBody& BB = W.bodies[bB];
  const f3 pA = ld3(BA.pos), pB = ld3(BB.pos);
  const ContactHead head = contact_head(C, bA, bB, shA, shB, rsi, rsj);
  int k = 0;
  for (int i = 0; i < nv; i++) {
    if (dv[i] <= 0.0) {
      ContactOut g;
      f3 proj = sub(wv[i], scale(wn, dv[i]));
      g.ri = sub(proj, xA);
      g.ni = wn;
      g.rj = sub(wv[i], xB);
      g.ri = sub(add(g.ri, xA), pA);  // rel(): r + x - body.position
      g.rj = sub(add(g.rj, xB), pB);
      put_contact(W.ctmp[start + k], head, g);
      k++;
    }
  }
  return n;
}

// ---- binary32 "no contact" certificates --------------------------------
// Each test below returns true only when the pair certainly produces no
// contact in the reference's binary64 arithmetic: it evaluates a necessary
// condition for a contact in binary32 and demands a relative margin of
// 1e-4 (the binary32 estimate is within ~1e-6 of the binary64 values), so the
// exact resolver, which would return no contacts, can be skipped.


// plane (xP, qP) vs a body whose shape lies within distance rB of xB: a
// contact needs a point of the shape on or behind the plane
// (spherePlane :797, planeConvex :1877)
DI bool plane_far(f3 xP, q4 qP, f3 xB, float rB) {
  f3 n = rot32(qP, f3{0.f, 0.f, 1.f});
  f3 d = f3{xB.x - xP.x, xB.y - xP.y, xB.z - xP.z};
  float h = dot32(n, d);
  float margin = 1e-4f * (rB + fabsf(d.x) + fabsf(d.y) + fabsf(d.z)) + 1e-6f;
  return h > rB + margin;
}

// Resolver choice of narrow_phase.dart:116-238,476-489,706-710.  The shape
// with the lower ShapeType index goes first (for equal types the call is the
// swapped one); (rsi, rsj) stay in getContacts order.
enum ResolverKind { RK_NONE = 0, RK_SS, RK_SP, RK_SB, RK_SC, RK_PB, RK_PC, RK_BB, RK_BC, RK_CC };

DI int resolver_kind(int ta, int tb) {  // ta <= tb
  if (ta == 0) {
    if (tb == 0) return RK_SS;
    if (tb == 1) return RK_SP;
    if (tb == 2) return RK_SB;
    return RK_SC;
  }
  if (ta == 1) {
    if (tb == 1) return RK_NONE;
    if (tb == 2) return RK_PB;
    return RK_PC;
  }
  if (ta == 2) return tb == 2 ? RK_BB : RK_BC;
  // convex + sizedPlane: the reference finds no resolver (its table key is
  // spelled "convexSizedPlane" but looked up lower-cased,
  // narrow_phase.dart:444,476-479)
  if (ta == CP_SHAPE_CONVEX && tb == CP_SHAPE_SIZED_PLANE) return RK_NONE;
  return RK_CC;
}
