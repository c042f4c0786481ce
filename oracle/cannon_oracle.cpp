// cannon_oracle.cpp -- CPU oracle for cannon_physics World.step.
//
// TEST INFRASTRUCTURE ONLY (see cannon_oracle.h).  A sequential restatement
// of the Dart reference, written to follow its operation order exactly:
// binary64 arithmetic, binary32 storage wherever the reference stores into a
// vector_math Vector3 / Quaternion / Matrix3 component.  Every function cites
// the reference file:line it restates (paths relative to the reference repo).
//
// package:vector_math ^2.1.4 is a third-party dependency that is not vendored
// in the reference; its storage (Float32List) and the operations used here
// (dot, length2, length, normalize, negate, conjugate, transpose, setFrom,
// setValues) are restated from its published behaviour.
//
// Build: g++ -O2 -std=c++17 -ffp-contract=off -fno-fast-math -fPIC -shared

#include "cannon_oracle.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <map>
#include <thread>
#include <atomic>
#include <utility>
#include <vector>

namespace orc {

static const double INF = std::numeric_limits<double>::infinity();

// ---------------------------------------------------------------------------
// vector_math storage types
struct V3 { float x = 0.f, y = 0.f, z = 0.f; };
struct Q4 { float x = 0.f, y = 0.f, z = 0.f, w = 1.f; };
struct M3 { float e[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}; };

static inline V3 mk(double x, double y, double z) { V3 v; v.x = (float)x; v.y = (float)y; v.z = (float)z; return v; }
static inline void setValues(V3& v, double x, double y, double z) { v.x = (float)x; v.y = (float)y; v.z = (float)z; }
static inline bool isZero(const V3& v) { return v.x == 0 && v.y == 0 && v.z == 0; }

// Vector3.dot / length2 / length / normalize / negate (vector_math)
static inline double dot(const V3& a, const V3& b) {
  double s = (double)a.x * (double)b.x;
  s += (double)a.y * (double)b.y;
  s += (double)a.z * (double)b.z;
  return s;
}
static inline double length2(const V3& a) { return dot(a, a); }
static inline double length(const V3& a) { return std::sqrt(length2(a)); }
static inline void normalize(V3& v) {
  double l = length(v);
  if (l == 0.0) return;
  double d = 1.0 / l;
  v.x = (float)(v.x * d); v.y = (float)(v.y * d); v.z = (float)(v.z * d);
}
static inline void negate(V3& v) { v.x = -v.x; v.y = -v.y; v.z = -v.z; }

// lib/math/vec3.dart:18-164
static inline void add2(const V3& a, const V3& v, V3& t) {
  t.x = (float)((double)v.x + (double)a.x);
  t.y = (float)((double)v.y + (double)a.y);
  t.z = (float)((double)v.z + (double)a.z);
}
static inline void sub2(const V3& a, const V3& v, V3& t) {
  t.x = (float)((double)a.x - (double)v.x);
  t.y = (float)((double)a.y - (double)v.y);
  t.z = (float)((double)a.z - (double)v.z);
}
static inline void scale2(const V3& a, double s, V3& t) {
  t.x = (float)(s * (double)a.x);
  t.y = (float)(s * (double)a.y);
  t.z = (float)(s * (double)a.z);
}
static inline void cross2(const V3& a, const V3& v, V3& t) {
  double vx = v.x, vy = v.y, vz = v.z;
  t.x = (float)((double)a.y * vz - (double)a.z * vy);
  t.y = (float)((double)a.z * vx - (double)a.x * vz);
  t.z = (float)((double)a.x * vy - (double)a.y * vx);
}
static inline void multiply2(const V3& a, const V3& v, V3& t) {
  t.x = (float)((double)v.x * (double)a.x);
  t.y = (float)((double)v.y * (double)a.y);
  t.z = (float)((double)v.z * (double)a.z);
}
static inline void addScaledVector(const V3& a, double s, const V3& v, V3& t) {
  t.x = (float)((double)a.x + s * (double)v.x);
  t.y = (float)((double)a.y + s * (double)v.y);
  t.z = (float)((double)a.z + s * (double)v.z);
}
static inline void lerp(const V3& a, const V3& v, double tt, V3& t) {
  t.x = (float)((double)a.x + ((double)v.x - (double)a.x) * tt);
  t.y = (float)((double)a.y + ((double)v.y - (double)a.y) * tt);
  t.z = (float)((double)a.z + ((double)v.z - (double)a.z) * tt);
}
static inline double distanceTo(const V3& a, const V3& p) {
  double px = p.x, py = p.y, pz = p.z;
  return std::sqrt((px - a.x) * (px - a.x) + (py - a.y) * (py - a.y) + (pz - a.z) * (pz - a.z));
}
static inline void tangents(const V3& a, V3& t1, V3& t2) {  // vec3.dart:97-117
  double norm = length(a);
  if (norm > 0.0) {
    V3 n;
    double inorm = 1 / norm;
    setValues(n, a.x * inorm, a.y * inorm, a.z * inorm);
    V3 rv;
    if (std::fabs((double)n.x) < 0.9) setValues(rv, 1, 0, 0);
    else setValues(rv, 0, 1, 0);
    cross2(n, rv, t1);
    cross2(n, t1, t2);
  } else {
    setValues(t1, 1, 0, 0);
    setValues(t2, 0, 1, 0);
  }
}
static inline void unit(const V3& a, V3& t) {  // vec3.dart:121-135
  double ninv = std::sqrt((double)a.x * a.x + (double)a.y * a.y + (double)a.z * a.z);
  if (ninv > 0.0) {
    ninv = 1.0 / ninv;
    t.x = (float)(a.x * ninv); t.y = (float)(a.y * ninv); t.z = (float)(a.z * ninv);
  } else {
    t.x = 1; t.y = 0; t.z = 0;
  }
}
static inline bool almostEquals(const V3& a, const V3& v, double p = 1e-6) {
  if (std::fabs((double)a.x - v.x) > p || std::fabs((double)a.y - v.y) > p || std::fabs((double)a.z - v.z) > p) return false;
  return true;
}
static inline bool almostZero(const V3& a, double p = 1e-6) {
  if (std::fabs((double)a.x) > p || std::fabs((double)a.y) > p || std::fabs((double)a.z) > p) return false;
  return true;
}

// lib/math/quaternion.dart:21-111,171-185 and vector_math Quaternion
static inline void vmult(const Q4& q, const V3& v, V3& t) {
  double x = v.x, y = v.y, z = v.z;
  double qx = q.x, qy = q.y, qz = q.z, qw = q.w;
  double ix = qw * x + qy * z - qz * y;
  double iy = qw * y + qz * x - qx * z;
  double iz = qw * z + qx * y - qy * x;
  double iw = -qx * x - qy * y - qz * z;
  t.x = (float)(ix * qw + iw * -qx + iy * -qz - iz * -qy);
  t.y = (float)(iy * qw + iw * -qy + iz * -qx - ix * -qz);
  t.z = (float)(iz * qw + iw * -qz + ix * -qy - iy * -qx);
}
static inline void qmultiply2(const Q4& a, const Q4& b, Q4& t) {
  double ax = a.x, ay = a.y, az = a.z, aw = a.w;
  double bx = b.x, by = b.y, bz = b.z, bw = b.w;
  t.x = (float)(ax * bw + aw * bx + ay * bz - az * by);
  t.y = (float)(ay * bw + aw * by + az * bx - ax * bz);
  t.z = (float)(az * bw + aw * bz + ax * by - ay * bx);
  t.w = (float)(aw * bw - ax * bx - ay * by - az * bz);
}
static inline void qintegrate(const Q4& q, const V3& av, double dt, const V3& af, Q4& t) {
  double ax = (double)av.x * af.x, ay = (double)av.y * af.y, az = (double)av.z * af.z;
  double bx = q.x, by = q.y, bz = q.z, bw = q.w;
  double halfDt = dt * 0.5;
  t.x = (float)(t.x + halfDt * (ax * bw + ay * bz - az * by));
  t.y = (float)(t.y + halfDt * (ay * bw + az * bx - ax * bz));
  t.z = (float)(t.z + halfDt * (az * bw + ax * by - ay * bx));
  t.w = (float)(t.w + halfDt * (-ax * bx - ay * by - az * bz));
}
static inline void qnormalize(Q4& q) {
  double x = q.x, y = q.y, z = q.z, w = q.w;
  double l = std::sqrt((x * x) + (y * y) + (z * z) + (w * w));
  if (l == 0.0) return;
  double d = 1.0 / l;
  q.x = (float)(q.x * d); q.y = (float)(q.y * d); q.z = (float)(q.z * d); q.w = (float)(q.w * d);
}
static inline void qnormalizeFast(Q4& q) {
  double f = (3.0 - ((double)q.x * q.x + (double)q.y * q.y + (double)q.z * q.z + (double)q.w * q.w)) / 2.0;
  if (f == 0) { q.x = 0; q.y = 0; q.z = 0; q.w = 0; }
  else { q.x = (float)(q.x * f); q.y = (float)(q.y * f); q.z = (float)(q.z * f); q.w = (float)(q.w * f); }
}
static inline void conjugate(Q4& q) { q.z = -q.z; q.y = -q.y; q.x = -q.x; }
// Quaternion.slerp (quaternion.dart:118-168): binary64 arithmetic, libm's
// acos and sin, each target component stored to binary32
static inline void slerp(const Q4& a, const Q4& to, double t, Q4& target) {
  const double ax = a.x, ay = a.y, az = a.z, aw = a.w;
  double bx = to.x, by = to.y, bz = to.z, bw = to.w;
  double cosom = ax * bx + ay * by + az * bz + aw * bw;
  if (cosom < 0.0) {
    cosom = -cosom;
    bx = -bx; by = -by; bz = -bz; bw = -bw;
  }
  double scale0, scale1;
  if (1.0 - cosom > 0.000001) {
    double omega = std::acos(cosom);
    double sinom = std::sin(omega);
    scale0 = std::sin((1.0 - t) * omega) / sinom;
    scale1 = std::sin(t * omega) / sinom;
  } else {
    scale0 = 1.0 - t;
    scale1 = t;
  }
  target.x = (float)(scale0 * ax + scale1 * bx);
  target.y = (float)(scale0 * ay + scale1 * by);
  target.z = (float)(scale0 * az + scale1 * bz);
  target.w = (float)(scale0 * aw + scale1 * bw);
}

// lib/math/mat3.dart:9-108 (storage indexed e[3*row+col])
static inline void mvmult(const M3& m, const V3& v, V3& t) {
  const float* e = m.e;
  double x = v.x, y = v.y, z = v.z;
  t.x = (float)(e[0] * x + e[1] * y + e[2] * z);
  t.y = (float)(e[3] * x + e[4] * y + e[5] * z);
  t.z = (float)(e[6] * x + e[7] * y + e[8] * z);
}
static inline void setRotationFromQuaternion(M3& m, const Q4& q) {
  double x = q.x, y = q.y, z = q.z, w = q.w;
  double x2 = x + x, y2 = y + y, z2 = z + z;
  double xx = x * x2, xy = x * y2, xz = x * z2, yy = y * y2, yz = y * z2, zz = z * z2;
  double wx = w * x2, wy = w * y2, wz = w * z2;
  float* e = m.e;
  e[0] = (float)(1 - (yy + zz)); e[1] = (float)(xy - wz); e[2] = (float)(xz + wy);
  e[3] = (float)(xy + wz); e[4] = (float)(1 - (xx + zz)); e[5] = (float)(yz - wx);
  e[6] = (float)(xz - wy); e[7] = (float)(yz + wx); e[8] = (float)(1 - (xx + yy));
}
static inline void mmultiply2(const M3& A, const M3& B, M3& T) {
  double a11 = A.e[0], a12 = A.e[1], a13 = A.e[2], a21 = A.e[3], a22 = A.e[4], a23 = A.e[5], a31 = A.e[6], a32 = A.e[7], a33 = A.e[8];
  double b11 = B.e[0], b12 = B.e[1], b13 = B.e[2], b21 = B.e[3], b22 = B.e[4], b23 = B.e[5], b31 = B.e[6], b32 = B.e[7], b33 = B.e[8];
  T.e[0] = (float)(a11 * b11 + a12 * b21 + a13 * b31);
  T.e[1] = (float)(a11 * b12 + a12 * b22 + a13 * b32);
  T.e[2] = (float)(a11 * b13 + a12 * b23 + a13 * b33);
  T.e[3] = (float)(a21 * b11 + a22 * b21 + a23 * b31);
  T.e[4] = (float)(a21 * b12 + a22 * b22 + a23 * b32);
  T.e[5] = (float)(a21 * b13 + a22 * b23 + a23 * b33);
  T.e[6] = (float)(a31 * b11 + a32 * b21 + a33 * b31);
  T.e[7] = (float)(a31 * b12 + a32 * b22 + a33 * b32);
  T.e[8] = (float)(a31 * b13 + a32 * b23 + a33 * b33);
}
static inline void vscale(const M3& m, const V3& v, M3& t) {
  for (int i = 0; i != 3; i++) {
    t.e[3 * i + 0] = (float)((double)v.x * m.e[3 * i + 0]);
    t.e[3 * i + 1] = (float)((double)v.y * m.e[3 * i + 1]);
    t.e[3 * i + 2] = (float)((double)v.z * m.e[3 * i + 2]);
  }
}
static inline void transpose(M3& m) {
  std::swap(m.e[1], m.e[3]); std::swap(m.e[2], m.e[6]); std::swap(m.e[5], m.e[7]);
}

// lib/math/transform.dart:152-180
static inline void pointToLocalFrame(const V3& pos, const Q4& q, const V3& wp, V3& res) {
  sub2(wp, pos, res);
  Q4 t = q;
  conjugate(t);
  vmult(t, res, res);
}
static inline void vectorToLocalFrame(const Q4& q, const V3& wv, V3& res) {
  Q4 t = q;
  t.w = (float)(t.w * -1.0);
  vmult(t, wv, res);
}

// ---------------------------------------------------------------------------
// Shapes

struct Hull {
  std::vector<V3> vertices;
  std::vector<std::vector<int>> faces;
  std::vector<V3> faceNormals;
  std::vector<V3> uniqueEdges;
  bool hasAxes = false;
  std::vector<V3> uniqueAxes;
};

// convex_polyhedron.dart:174-185
static void computeNormal(const V3& va, const V3& vb, const V3& vc, V3& target) {
  V3 cb, ab;
  sub2(vb, va, ab);
  sub2(vc, vb, cb);
  cross2(cb, ab, target);
  if (!isZero(target)) normalize(target);
}
// convex_polyhedron.dart:80-162 (init: computeNormals, computeEdges)
static void hullInit(Hull& h) {
  h.faceNormals.assign(h.faces.size(), V3());
  for (size_t i = 0; i < h.faces.size(); i++) {
    V3 n;
    const std::vector<int>& f = h.faces[i];
    computeNormal(h.vertices[f[0]], h.vertices[f[1]], h.vertices[f[2]], n);
    negate(n);
    h.faceNormals[i] = n;
  }
  h.uniqueEdges.clear();
  V3 edge;
  for (size_t i = 0; i != h.faces.size(); i++) {
    const std::vector<int>& face = h.faces[i];
    int nv = (int)face.size();
    for (int j = 0; j != nv; j++) {
      int k = (j + 1) % nv;
      sub2(h.vertices[face[j]], h.vertices[face[k]], edge);
      normalize(edge);
      bool found = false;
      for (size_t p = 0; p != h.uniqueEdges.size(); p++) {
        if (almostEquals(h.uniqueEdges[p], edge)) { found = true; break; }
      }
      if (!found) h.uniqueEdges.push_back(edge);
    }
  }
}

struct Shape {
  int type = CP_SHAPE_SPHERE;
  double radius = 1.0;
  V3 halfExtents;
  Hull hull;  // box: convexPolyhedronRepresentation; convex/cylinder: itself
  double bsr = 0;
  int group = -1, mask = -1;
  bool response = true;
  int material = -1;
};

static int buildShape(const cp_shape_desc& d, Shape& s) {
  s.type = d.type;
  s.group = d.collision_filter_group;
  s.mask = d.collision_filter_mask;
  s.response = d.collision_response != 0;
  s.material = d.material;
  Hull& h = s.hull;
  switch (d.type) {
    case CP_SHAPE_SPHERE:
      s.radius = d.radius;
      s.bsr = d.radius;  // sphere.dart:142-144
      break;
    case CP_SHAPE_PLANE:
      s.bsr = INF;  // plane.dart:177,229-231
      break;
    case CP_SHAPE_BOX: {  // box.dart:41-78,124-126
      s.halfExtents.x = d.half_extents[0]; s.halfExtents.y = d.half_extents[1]; s.halfExtents.z = d.half_extents[2];
      double sx = s.halfExtents.x, sy = s.halfExtents.y, sz = s.halfExtents.z;
      h.vertices = {mk(-sx, -sy, -sz), mk(sx, -sy, -sz), mk(sx, sy, -sz), mk(-sx, sy, -sz),
                    mk(-sx, -sy, sz), mk(sx, -sy, sz), mk(sx, sy, sz), mk(-sx, sy, sz)};
      h.faces = {{3, 2, 1, 0}, {4, 5, 6, 7}, {5, 4, 0, 1}, {2, 3, 7, 6}, {0, 4, 7, 3}, {1, 2, 6, 5}};
      h.hasAxes = true;
      h.uniqueAxes = {mk(0, 0, 1), mk(0, 1, 0), mk(1, 0, 0)};
      hullInit(h);
      s.bsr = length(s.halfExtents);
      break;
    }
    case CP_SHAPE_CYLINDER: {  // cylinder.dart:222-294
      const int N = d.num_segments;
      if (d.radius_top < 0 || d.radius_bottom < 0 || N < 3) return CP_ERR_ARG;
      double rt = d.radius_top, rb = d.radius_bottom, ht = d.height;
      std::vector<int> bottom, top;
      h.vertices.push_back(mk(-rb * std::sin(0.0), -ht * 0.5, rb * std::cos(0.0)));
      bottom.push_back(0);
      h.vertices.push_back(mk(-rt * std::sin(0.0), ht * 0.5, rt * std::cos(0.0)));
      top.push_back(1);
      for (int i = 0; i < N; i++) {
        double theta = ((2 * M_PI) / N) * (i + 1);
        double thetaN = ((2 * M_PI) / N) * (i + 0.5);
        if (i < N - 1) {
          h.vertices.push_back(mk(-rb * std::sin(theta), -ht * 0.5, rb * std::cos(theta)));
          bottom.push_back(2 * i + 2);
          h.vertices.push_back(mk(-rt * std::sin(theta), ht * 0.5, rt * std::cos(theta)));
          top.push_back(2 * i + 3);
          h.faces.push_back({2 * i, 2 * i + 1, 2 * i + 3, 2 * i + 2});
        } else {
          h.faces.push_back({2 * i, 2 * i + 1, 1, 0});
        }
        if (N % 2 == 1 || i < N / 2.0) h.uniqueAxes.push_back(mk(-std::sin(thetaN), 0, std::cos(thetaN)));
      }
      h.faces.push_back(bottom);
      h.uniqueAxes.push_back(mk(0, 1, 0));
      std::vector<int> temp;
      for (size_t i = 0; i < top.size(); i++) temp.push_back(top[top.size() - i - 1]);
      h.faces.push_back(temp);
      h.hasAxes = true;
      hullInit(h);
      double max2 = 0;  // convex_polyhedron.dart:648-660 (run again by Body.addShape)
      for (auto& v : h.vertices) { double n2 = length2(v); if (n2 > max2) max2 = n2; }
      s.bsr = std::sqrt(max2);
      break;
    }
    case CP_SHAPE_CONVEX:
    case CP_SHAPE_CAPSULE:       // capsule.dart, cone.dart, sized_plane.dart: their
    case CP_SHAPE_CONE:          // constructors build the vertices and faces, then
    case CP_SHAPE_SIZED_PLANE: {  // ConvexPolyhedron.init as for any hull
      const bool conv = d.type == CP_SHAPE_CONVEX;
      if (d.num_vertices < (conv ? 4 : 3) || d.num_faces < (conv ? 4 : 1) || !d.vertices || !d.face_sizes || !d.face_indices)
        return CP_ERR_ARG;
      for (int i = 0; i < d.num_vertices; i++) h.vertices.push_back(mk(d.vertices[3 * i], d.vertices[3 * i + 1], d.vertices[3 * i + 2]));
      int off = 0;
      for (int f = 0; f < d.num_faces; f++) {
        std::vector<int> face;
        for (int k = 0; k < d.face_sizes[f]; k++) {
          int vi = d.face_indices[off + k];
          if (vi < 0 || vi >= d.num_vertices) return CP_ERR_ARG;
          face.push_back(vi);
        }
        if (face.size() < 3) return CP_ERR_ARG;
        off += d.face_sizes[f];
        h.faces.push_back(face);
      }
      h.hasAxes = d.has_axes != 0;
      if (h.hasAxes)
        for (int i = 0; i < d.num_axes; i++) h.uniqueAxes.push_back(mk(d.axes[3 * i], d.axes[3 * i + 1], d.axes[3 * i + 2]));
      hullInit(h);
      double max2 = 0;
      for (auto& v : h.vertices) { double n2 = length2(v); if (n2 > max2) max2 = n2; }
      s.bsr = std::sqrt(max2);
      break;
    }
    default:
      return CP_ERR_UNSUPPORTED;
  }
  return CP_OK;
}

// Shape.calculateWorldAABB: sphere.dart:146-156, plane.dart:201-226,
// box.dart:149-192, convex_polyhedron.dart:663-703
static void shapeWorldAABB(const Shape& s, const V3& pos, const Q4& quat, V3& mn, V3& mx) {
  switch (s.type) {
    case CP_SHAPE_SPHERE: {
      double r = s.radius;
      mn.x = (float)(pos.x - r); mx.x = (float)(pos.x + r);
      mn.y = (float)(pos.y - r); mx.y = (float)(pos.y + r);
      mn.z = (float)(pos.z - r); mx.z = (float)(pos.z + r);
      break;
    }
    case CP_SHAPE_PLANE: {
      V3 n; setValues(n, 0, 0, 1);
      vmult(quat, n, n);
      setValues(mn, -INF, -INF, -INF);
      setValues(mx, INF, INF, INF);
      if (n.x == 1) mx.x = pos.x; else if (n.x == -1) mn.x = pos.x;
      if (n.y == 1) mx.y = pos.y; else if (n.y == -1) mn.y = pos.y;
      if (n.z == 1) mx.z = pos.z; else if (n.z == -1) mn.z = pos.z;
      break;
    }
    case CP_SHAPE_BOX: {
      const V3& e = s.halfExtents;
      V3 c[8];
      setValues(c[0], e.x, e.y, e.z); setValues(c[1], -e.x, e.y, e.z);
      setValues(c[2], -e.x, -e.y, e.z); setValues(c[3], -e.x, -e.y, -e.z);
      setValues(c[4], e.x, -e.y, -e.z); setValues(c[5], e.x, e.y, -e.z);
      setValues(c[6], -e.x, e.y, -e.z); setValues(c[7], e.x, -e.y, e.z);
      vmult(quat, c[0], c[0]);
      add2(pos, c[0], c[0]);
      mx = c[0]; mn = c[0];
      for (int i = 1; i < 8; i++) {
        vmult(quat, c[i], c[i]);
        add2(pos, c[i], c[i]);
        double x = c[i].x, y = c[i].y, z = c[i].z;
        if (x > mx.x) mx.x = (float)x;
        if (y > mx.y) mx.y = (float)y;
        if (z > mx.z) mx.z = (float)z;
        if (x < mn.x) mn.x = (float)x;
        if (y < mn.y) mn.y = (float)y;
        if (z < mn.z) mn.z = (float)z;
      }
      break;
    }
    default: {  // convex, cylinder
      bool first = true;
      double minx = 0, miny = 0, minz = 0, maxx = 0, maxy = 0, maxz = 0;
      V3 t;
      for (const V3& v : s.hull.vertices) {
        t = v;
        vmult(quat, t, t);
        add2(pos, t, t);
        if (first || t.x < minx) minx = t.x;
        if (first || t.x > maxx) maxx = t.x;
        if (first || t.y < miny) miny = t.y;
        if (first || t.y > maxy) maxy = t.y;
        if (first || t.z < minz) minz = t.z;
        if (first || t.z > maxz) maxz = t.z;
        first = false;
      }
      setValues(mn, minx, miny, minz);
      setValues(mx, maxx, maxy, maxz);
      break;
    }
  }
}

// ---------------------------------------------------------------------------
// Bodies

struct Body {
  V3 position, previousPosition, velocity, force, torque, angularVelocity;
  Q4 quaternion, previousQuaternion;
  V3 linearFactor, angularFactor, inertia, invInertia, invInertiaSolve;
  M3 invInertiaWorld, invInertiaWorldSolve;
  V3 aabbLo, aabbHi;
  V3 shapeOffset; Q4 shapeOrientation;
  V3 vlambda, wlambda;
  V3 interpolatedPosition; Q4 interpolatedQuaternion;  // rigid_body.dart:135,190
  double mass = 0, invMass = 0, invMassSolve = 0;
  double linearDamping = 0.01, angularDamping = 0.01;
  double sleepSpeedLimit = 0.1, sleepTimeLimit = 1, timeLastSleepy = 0;
  double boundingRadius = 0;
  int type = CP_BODY_DYNAMIC, sleepState = CP_AWAKE;
  bool allowSleep = true, wakeUpAfterNarrowphase = false;
  int group = 1, mask = -1;
  bool response = true, isTrigger = false, fixedRotation = false, aabbNeedsUpdate = true;
  int material = -1;
  int shape = -1;  // Body.shapes[0] (at shapeOffset / shapeOrientation)
  // Body.shapes[1..] of a compound body, with their offsets and orientations
  struct Extra { int shape; V3 offset; Q4 orientation; };
  std::vector<Extra> extra;
  int extraFirst = 0;  // where they came from in the world's body_shapes table
  int numShapes() const { return shape < 0 ? 0 : 1 + (int)extra.size(); }
  int shapeAt(int k) const { return k == 0 ? shape : extra[k - 1].shape; }
  const V3& offsetAt(int k) const { return k == 0 ? shapeOffset : extra[k - 1].offset; }
  const Q4& orientationAt(int k) const { return k == 0 ? shapeOrientation : extra[k - 1].orientation; }
};

// dart:math min / max on doubles: NaN wins, and -0.0 is below 0.0
static inline double dartMin(double a, double b) {
  if (a > b) return b;
  if (a < b) return a;
  if (std::isnan(a) || std::isnan(b)) return std::numeric_limits<double>::quiet_NaN();
  return (std::signbit(a) || std::signbit(b)) ? -0.0 : a;
}
static inline double dartMax(double a, double b) {
  if (a < b) return b;
  if (a > b) return a;
  if (std::isnan(a) || std::isnan(b)) return std::numeric_limits<double>::quiet_NaN();
  return (std::signbit(a) && std::signbit(b)) ? -0.0 : (a == 0 ? 0.0 : a);
}

// rigid_body.dart:415-447: each shape's world AABB, the first copied, the
// others extended in (AABB.extend, aabb.dart:121-128)
static void updateAABB(Body& b, const std::vector<Shape>& shapes) {
  const int N = b.numShapes();
  for (int i = 0; i != N; i++) {
    V3 offset, lo, hi; Q4 orientation;
    vmult(b.quaternion, b.offsetAt(i), offset);
    add2(offset, b.position, offset);
    qmultiply2(b.quaternion, b.orientationAt(i), orientation);
    shapeWorldAABB(shapes[b.shapeAt(i)], offset, orientation, lo, hi);
    if (i == 0) {
      b.aabbLo = lo; b.aabbHi = hi;
    } else {
      b.aabbLo.x = (float)dartMin(b.aabbLo.x, lo.x); b.aabbHi.x = (float)dartMax(b.aabbHi.x, hi.x);
      b.aabbLo.y = (float)dartMin(b.aabbLo.y, lo.y); b.aabbHi.y = (float)dartMax(b.aabbHi.y, hi.y);
      b.aabbLo.z = (float)dartMin(b.aabbLo.z, lo.z); b.aabbHi.z = (float)dartMax(b.aabbHi.z, hi.z);
    }
  }
  b.aabbNeedsUpdate = false;
}

// rigid_body.dart:450-466
static void updateInertiaWorld(Body& b, bool force) {
  const V3& I = b.invInertia;
  if (I.x == I.y && I.y == I.z && !force) return;
  M3 m1, m2;
  setRotationFromQuaternion(m1, b.quaternion);
  m2 = m1;
  transpose(m2);
  vscale(m1, I, m1);
  mmultiply2(m1, m2, b.invInertiaWorld);
}

// box.dart:88-94
static void calculateInertia(const V3& e, double mass, V3& t) {
  t.x = (float)(1.0 / 12.0 * mass * (2 * (double)e.y * 2 * e.y + 2 * (double)e.z * 2 * e.z));
  t.y = (float)(1.0 / 12.0 * mass * (2 * (double)e.x * 2 * e.x + 2 * (double)e.z * 2 * e.z));
  t.z = (float)(1.0 / 12.0 * mass * (2 * (double)e.y * 2 * e.y + 2 * (double)e.x * 2 * e.x));
}

// rigid_body.dart:587-609
static void updateMassProperties(Body& b, const std::vector<Shape>& shapes) {
  b.invMass = b.mass > 0 ? 1.0 / b.mass : 0;
  if (b.shape >= 0) updateAABB(b, shapes);
  V3 he;
  setValues(he, ((double)b.aabbHi.x - b.aabbLo.x) / 2, ((double)b.aabbHi.y - b.aabbLo.y) / 2, ((double)b.aabbHi.z - b.aabbLo.z) / 2);
  calculateInertia(he, b.mass, b.inertia);
  const V3& I = b.inertia;
  bool fixed = b.fixedRotation;
  setValues(b.invInertia, I.x > 0 && !fixed ? 1.0 / I.x : 0, I.y > 0 && !fixed ? 1.0 / I.y : 0, I.z > 0 && !fixed ? 1.0 / I.z : 0);
  updateInertiaWorld(b, true);
}

// a body's extra shapes lie inside the table and name existing shapes, only
// a body with a first shape has any, and a body has at most
// CP_MAX_BODY_SHAPES shapes (the ABI's limit)
static bool extrasValid(const cp_body_desc& d, int num_shapes, const cp_body_shape* table, int ntable) {
  if (d.extra_shapes_count == 0) return true;
  if (d.extra_shapes_count < 0 || d.extra_shapes_count >= CP_MAX_BODY_SHAPES || d.shape < 0 || !table ||
      d.extra_shapes_first < 0 || (long long)d.extra_shapes_first + d.extra_shapes_count > ntable)
    return false;
  for (int k = 0; k < d.extra_shapes_count; k++) {
    const int sh = table[d.extra_shapes_first + k].shape;
    if (sh < 0 || sh >= num_shapes) return false;
  }
  return true;
}

static void bodyFromDesc(const cp_body_desc& d, Body& b, const cp_body_shape* table) {
  auto v3 = [](const float* f) { V3 v; v.x = f[0]; v.y = f[1]; v.z = f[2]; return v; };
  auto q4 = [](const float* f) { Q4 q; q.x = f[0]; q.y = f[1]; q.z = f[2]; q.w = f[3]; return q; };
  b.position = v3(d.position); b.quaternion = q4(d.quaternion);
  b.velocity = v3(d.velocity); b.angularVelocity = v3(d.angular_velocity);
  b.force = v3(d.force); b.torque = v3(d.torque);
  b.linearFactor = v3(d.linear_factor); b.angularFactor = v3(d.angular_factor);
  b.invInertia = v3(d.inv_inertia);
  for (int i = 0; i < 9; i++) b.invInertiaWorld.e[i] = d.inv_inertia_world[i];
  b.aabbLo = v3(d.aabb_lower); b.aabbHi = v3(d.aabb_upper);
  b.shapeOffset = v3(d.shape_offset); b.shapeOrientation = q4(d.shape_orientation);
  b.previousPosition = v3(d.previous_position); b.previousQuaternion = q4(d.previous_quaternion);
  b.interpolatedPosition = v3(d.interpolated_position); b.interpolatedQuaternion = q4(d.interpolated_quaternion);
  b.mass = d.mass; b.invMass = d.inv_mass;
  b.linearDamping = d.linear_damping; b.angularDamping = d.angular_damping;
  b.sleepSpeedLimit = d.sleep_speed_limit; b.sleepTimeLimit = d.sleep_time_limit; b.timeLastSleepy = d.time_last_sleepy;
  b.boundingRadius = d.bounding_radius;
  b.type = d.type; b.sleepState = d.sleep_state; b.allowSleep = d.allow_sleep != 0;
  b.wakeUpAfterNarrowphase = d.wake_up_after_narrowphase != 0;
  b.group = d.collision_filter_group; b.mask = d.collision_filter_mask;
  b.response = d.collision_response != 0; b.isTrigger = d.is_trigger != 0;
  b.material = d.material; b.shape = d.shape;
  b.fixedRotation = d.fixed_rotation != 0; b.aabbNeedsUpdate = d.aabb_needs_update != 0;
  b.extra.clear();
  b.extraFirst = d.extra_shapes_first;
  for (int k = 0; k < d.extra_shapes_count; k++) {
    const cp_body_shape& e = table[d.extra_shapes_first + k];
    b.extra.push_back(Body::Extra{e.shape, v3(e.offset), q4(e.orientation)});
  }
}

static void bodyToDesc(const Body& b, cp_body_desc& d) {
  auto v3 = [](float* f, const V3& v) { f[0] = v.x; f[1] = v.y; f[2] = v.z; };
  auto q4 = [](float* f, const Q4& q) { f[0] = q.x; f[1] = q.y; f[2] = q.z; f[3] = q.w; };
  v3(d.position, b.position); q4(d.quaternion, b.quaternion);
  v3(d.velocity, b.velocity); v3(d.angular_velocity, b.angularVelocity);
  v3(d.force, b.force); v3(d.torque, b.torque);
  v3(d.linear_factor, b.linearFactor); v3(d.angular_factor, b.angularFactor);
  v3(d.inv_inertia, b.invInertia);
  for (int i = 0; i < 9; i++) d.inv_inertia_world[i] = b.invInertiaWorld.e[i];
  v3(d.aabb_lower, b.aabbLo); v3(d.aabb_upper, b.aabbHi);
  v3(d.shape_offset, b.shapeOffset); q4(d.shape_orientation, b.shapeOrientation);
  v3(d.previous_position, b.previousPosition); q4(d.previous_quaternion, b.previousQuaternion);
  v3(d.interpolated_position, b.interpolatedPosition); q4(d.interpolated_quaternion, b.interpolatedQuaternion);
  d.mass = b.mass; d.inv_mass = b.invMass;
  d.linear_damping = b.linearDamping; d.angular_damping = b.angularDamping;
  d.sleep_speed_limit = b.sleepSpeedLimit; d.sleep_time_limit = b.sleepTimeLimit; d.time_last_sleepy = b.timeLastSleepy;
  d.bounding_radius = b.boundingRadius;
  d.type = b.type; d.sleep_state = b.sleepState; d.allow_sleep = b.allowSleep;
  d.wake_up_after_narrowphase = b.wakeUpAfterNarrowphase;
  d.collision_filter_group = b.group; d.collision_filter_mask = b.mask;
  d.collision_response = b.response; d.is_trigger = b.isTrigger;
  d.material = b.material; d.shape = b.shape;
  d.fixed_rotation = b.fixedRotation; d.aabb_needs_update = b.aabbNeedsUpdate;
  d.extra_shapes_first = b.extraFirst;
  d.extra_shapes_count = (int32_t)b.extra.size();
}

// ---------------------------------------------------------------------------
// Equations (lib/equations/*.dart)

struct Eq {
  int kind = CP_ROW_CONTACT;
  int bi = 0, bj = 0, si = -1, sj = -1;
  double minForce = -1e6, maxForce = 1e6;
  double a = 0, b = 0, eps = 0;
  V3 gaS, gaR, gbS, gbR;
  bool enabled = true;
  double multiplier = 0;
  double restitution = 0;
  V3 ri, rj, ni;  // contact
  V3 t;           // friction tangent
  V3 axisA, axisB;
  double cosMaxAngle = 0;  // rotational: cos(maxAngle), computed with libm at construction
  double targetVelocity = 0;
  int pair = -1;
  double B = 0, invC = 0, lambda = 0;
  long long id = -1;  // Equation.id (equation_class.dart:34-37), kept under the SplitSolver

  // equation_class.dart:53-60
  void setSpookParams(double stiffness, double relaxation, double timeStep) {
    double d = relaxation, k = stiffness, h = timeStep;
    a = 4.0 / (h * (1 + 4 * d));
    b = 4.0 * d / (1 + 4 * d);
    eps = 4.0 / (h * h * k * (1 + 4 * d));
  }
};

struct ContactMat { double friction = 0.3, restitution = 0.3, cs = 1e7, cr = 3, fs = 1e7, fr = 3; };
struct Material { double friction = -1, restitution = -1; };

struct Constraint {
  int type = CP_CON_POINT_TO_POINT;
  int bodyA = 0, bodyB = 0;
  bool collideConnected = true;
  V3 pivotA, pivotB, axisA, axisB;
  V3 xA, xB, yA, yB, zA, zB;  // LockConstraint's local axes (lock_constraint.dart:41-46)
  double distance = 0;
  // p2p: x,y,z; hinge: x,y,z,rot1,rot2,motor; lock: x,y,z,rot1,rot2,rot3;
  // cone-twist: x,y,z,cone,twist; distance / spring: one contact
  std::vector<Eq> eqs;
};

// OverlapKeeper (lib/collision/overlap_keeper.dart): a sorted list of pair
// keys built by insertion, swapped out every step, and a merge-style diff
struct OverlapKeeper {
  std::vector<long long> current, previous;
  static long long getKey(long long i, long long j) {
    if (j < i) std::swap(i, j);
    return (i << 16) | j;
  }
  void set(int i, int j) {  // overlap_keeper.dart:22-38
    const long long key = getKey(i, j);
    size_t index = 0;
    while (index < current.size() && key > current[index]) index++;
    if (index < current.size() && key == current[index]) return;
    current.insert(current.begin() + index, key);
  }
  void tick() {  // :41-46
    std::swap(current, previous);
    current.clear();
  }
  void getDiff(std::vector<int>& additions, std::vector<int>& removals) const {  // :49-85
    const std::vector<long long>& a = current;
    const std::vector<long long>& b = previous;
    size_t j = 0;
    for (size_t i = 0; i < a.size(); i++) {
      const long long keyA = a[i];
      while (j < b.size() && keyA > b[j]) j++;
      const bool found = j < b.size() && keyA == b[j];
      if (!found) { additions.push_back((int)((keyA & 0xffff0000LL) >> 16)); additions.push_back((int)(keyA & 0xffff)); }
    }
    j = 0;
    for (size_t i = 0; i < b.size(); i++) {
      const long long keyB = b[i];
      while (j < a.size() && keyB > a[j]) j++;
      const bool found = j < a.size() && a[j] == keyB;
      if (!found) { removals.push_back((int)((keyB & 0xffff0000LL) >> 16)); removals.push_back((int)(keyB & 0xffff)); }
    }
  }
};

struct World {
  std::vector<Body> bodies;
  std::vector<Shape> shapes;
  std::vector<Material> materials;
  std::map<std::pair<int, int>, ContactMat> cmTable;
  ContactMat defaultCM;
  std::vector<Constraint> constraints;
  V3 gravity, frictionGravity;
  bool hasFrictionGravity = false;
  bool allowSleep = false;
  int quatNormalizeSkip = 0;
  bool quatNormalizeFast = false;
  int iterations = 10;
  double tolerance = 1e-7;
  int broadphase = CP_BROAD_NAIVE;
  bool useBoundingBoxes = false;
  int sapAxis = 0;
  std::vector<int> axisList;
  bool dirty = true;
  int gridN[3] = {10, 10, 10};
  V3 gridMin, gridMax;
  std::vector<char> planeNormalDone;
  std::vector<V3> planeWorldNormal;
  bool enableFrictionReduction = false;
  std::vector<cp_body_shape> bodyShapeTable;  // the compound bodies' extra shapes
  // events (world_class.dart:213-221,593-610,703-770), when recorded
  bool events = false;
  // SplitSolver (split_solver.dart) and the equation ids it sorts by: the
  // global Equation.idCounter and the narrowphase's reuse pools of contact
  // and friction equation objects, as stacks of ids (world_class.dart:506-527)
  bool split = false;
  long long idCounter = 0;
  std::vector<long long> contactPool, frictionPool;
  long long takeId(std::vector<long long>& pool) {  // pool.removeLast() or a new object
    if (pool.empty()) return idCounter++;
    const long long id = pool.back();
    pool.pop_back();
    return id;
  }
  std::vector<int> bodyIds, shapeIds;
  OverlapKeeper bodyOverlapKeeper, shapeOverlapKeeper;
  std::vector<cp_event> eventQueue;
  int bodyId(int i) const { return bodyIds.empty() ? i : bodyIds[i]; }
  int shapeId(int i) const { return shapeIds.empty() ? i : shapeIds[i]; }
  int bodyIndex(int id) const {
    if (bodyIds.empty()) return id;
    for (size_t i = 0; i < bodyIds.size(); i++) if (bodyIds[i] == id) return (int)i;
    return -1;
  }
  int shapeIndex(int id) const {
    if (shapeIds.empty()) return id;
    for (size_t i = 0; i < shapeIds.size(); i++) if (shapeIds[i] == id) return (int)i;
    return -1;
  }
  double time = 0;
  long long stepnumber = 0;
  double dt = -1;
  // per-step outputs
  std::vector<int> p1, p2;
  std::vector<Eq> contacts;
  std::vector<Eq> frictionEqs;
  std::vector<Eq> solverRows;  // copy of the solved equations in solver order
  int lastIterations = 0;
  // narrowphase state
  ContactMat current;
  V3 sepAxisPersist;  // _convexConvexSepAxis persists across calls
  int curPair = -1;

  const ContactMat* getCM(int m1, int m2) const {
    auto it = cmTable.find(std::make_pair(std::min(m1, m2), std::max(m1, m2)));
    return it == cmTable.end() ? nullptr : &it->second;
  }

  // ---------------------------------------------------------------- broadphase
  // broadphase.dart:44-63
  bool needBroadphaseCollision(const Body& A, const Body& B) const {
    if ((A.group & B.mask) == 0 || (B.group & A.mask) == 0) return false;
    if ((A.type == CP_BODY_STATIC || A.sleepState == CP_SLEEPING) && (B.type == CP_BODY_STATIC || B.sleepState == CP_SLEEPING)) return false;
    return true;
  }
  // aabb.dart:131-147
  static bool overlaps(const Body& A, const Body& B) {
    const V3 &l1 = A.aabbLo, &u1 = A.aabbHi, &l2 = B.aabbLo, &u2 = B.aabbHi;
    bool ox = (l2.x <= u1.x && u1.x <= u2.x) || (l1.x <= u2.x && u2.x <= u1.x);
    bool oy = (l2.y <= u1.y && u1.y <= u2.y) || (l1.y <= u2.y && u2.y <= u1.y);
    bool oz = (l2.z <= u1.z && u1.z <= u2.z) || (l1.z <= u2.z && u2.z <= u1.z);
    return ox && oy && oz;
  }
  // broadphase.dart:66-102
  void intersectionTest(int ia, int ib) {
    Body& A = bodies[ia];
    Body& B = bodies[ib];
    if (useBoundingBoxes) {
      if (A.aabbNeedsUpdate) updateAABB(A, shapes);
      if (B.aabbNeedsUpdate) updateAABB(B, shapes);
      if (overlaps(A, B)) { p1.push_back(ia); p2.push_back(ib); }
    } else {
      V3 r;
      sub2(B.position, A.position, r);
      double s = A.boundingRadius + B.boundingRadius;
      double bound2 = s * s;
      double norm2 = length2(r);
      if (norm2 < bound2) { p1.push_back(ia); p2.push_back(ib); }
    }
  }
  // naive_broadphase.dart:14-33
  void naivePairs() {
    int n = (int)bodies.size();
    for (int i = 0; i != n; i++)
      for (int j = 0; j != i; j++) {
        if (!needBroadphaseCollision(bodies[i], bodies[j])) continue;
        intersectionTest(i, j);
      }
  }
  static double axisComp(const V3& v, int axis) { return axis == 0 ? v.x : (axis == 1 ? v.y : v.z); }
  // sap_broadphase.dart:41-62
  bool checkBounds(const Body& bi, const Body& bj) const {
    double biPos = axisComp(bi.position, sapAxis), bjPos = axisComp(bj.position, sapAxis);
    double boundA2 = biPos + bi.boundingRadius;
    double boundB1 = bjPos - bj.boundingRadius;
    return boundB1 < boundA2;
  }
  // sap_broadphase.dart:66-111,138-189
  // sortList (sap_broadphase.dart:168-189) with the insertion sorts (:66-111)
  void sapSort() {
    for (int bi : axisList) if (bodies[bi].aabbNeedsUpdate) updateAABB(bodies[bi], shapes);
    for (size_t i = 1, l = axisList.size(); i < l; i++) {
      int v = axisList[i];
      double vk = axisComp(bodies[v].aabbLo, sapAxis);
      long j;
      for (j = (long)i - 1; j >= 0; j--) {
        if (axisComp(bodies[axisList[j]].aabbLo, sapAxis) <= vk) break;
        axisList[j + 1] = axisList[j];
      }
      axisList[j + 1] = v;
    }
  }
  void sapPairs() {
    if (dirty) {
      sapSort();
      dirty = false;
    }
    int N = (int)axisList.size();
    for (int i = 0; i != N; i++) {
      int bi = axisList[i];
      for (int j = i + 1; j < N; j++) {
        int bj = axisList[j];
        if (!needBroadphaseCollision(bodies[bi], bodies[bj])) continue;
        if (!checkBounds(bodies[bi], bodies[bj])) break;
        intersectionTest(bi, bj);
      }
    }
  }
  // grid_broadphase.dart:59-239 with per-bin lists, and broadphase.dart:105-134
  // with its intended meaning: unique unordered pairs in order of first
  // appearance, each taking the body order of its last appearance.
  void gridPairs() {
    const int nx = gridN[0], ny = gridN[1], nz = gridN[2];
    const int xstep = ny * nz, ystep = nz, zstep = 1;
    double xmax = gridMax.x, ymax = gridMax.y, zmax = gridMax.z;
    double xmin = gridMin.x, ymin = gridMin.y, zmin = gridMin.z;
    double xmult = nx / (xmax - xmin), ymult = ny / (ymax - ymin), zmult = nz / (zmax - zmin);
    double binsizeX = (xmax - xmin) / nx, binsizeY = (ymax - ymin) / ny, binsizeZ = (zmax - zmin) / nz;
    double binRadius = std::sqrt(binsizeX * binsizeX + binsizeY * binsizeY + binsizeZ * binsizeZ) * 0.5;
    const int nBins = nx * ny * nz;
    std::vector<std::vector<int>> bins(nBins);
    auto addBoxToBins = [&](double x0, double y0, double z0, double x1, double y1, double z1, int bi) {
      long xoff0 = (long)std::floor((x0 - xmin) * xmult), yoff0 = (long)std::floor((y0 - ymin) * ymult), zoff0 = (long)std::floor((z0 - zmin) * zmult);
      long xoff1 = (long)std::ceil((x1 - xmin) * xmult), yoff1 = (long)std::ceil((y1 - ymin) * ymult), zoff1 = (long)std::ceil((z1 - zmin) * zmult);
      auto clampi = [](long v, int n) { return v < 0 ? 0L : (v >= n ? (long)n - 1 : v); };
      xoff0 = clampi(xoff0, nx); yoff0 = clampi(yoff0, ny); zoff0 = clampi(zoff0, nz);
      xoff1 = clampi(xoff1, nx); yoff1 = clampi(yoff1, ny); zoff1 = clampi(zoff1, nz);
      xoff0 *= xstep; yoff0 *= ystep; zoff0 *= zstep;
      xoff1 *= xstep; yoff1 *= ystep; zoff1 *= zstep;
      for (long xoff = xoff0; xoff <= xoff1; xoff += xstep)
        for (long yoff = yoff0; yoff <= yoff1; yoff += ystep)
          for (long zoff = zoff0; zoff <= zoff1; zoff += zstep) bins[xoff + yoff + zoff].push_back(bi);
    };
    const int N = (int)bodies.size();
    for (int i = 0; i != N; i++) {
      Body& b = bodies[i];
      if (b.shape < 0) continue;
      const Shape& s = shapes[b.shape];
      if (s.type == CP_SHAPE_SPHERE) {
        double x = b.position.x, y = b.position.y, z = b.position.z, r = s.radius;
        addBoxToBins(x - r, y - r, z - r, x + r, y + r, z + r, i);
      } else if (s.type == CP_SHAPE_PLANE) {
        if (!planeNormalDone[b.shape]) {  // plane.dart:182-187, cached once
          V3 n; setValues(n, 0, 0, 1);
          vmult(b.quaternion, n, n);
          planeWorldNormal[b.shape] = n;
          planeNormalDone[b.shape] = 1;
        }
        const V3& pn = planeWorldNormal[b.shape];
        double xreset = xmin + binsizeX * 0.5 - b.position.x;
        double yreset = ymin + binsizeY * 0.5 - b.position.y;
        double zreset = zmin + binsizeZ * 0.5 - b.position.z;
        V3 d; setValues(d, xreset, yreset, zreset);
        for (int xi = 0, xoff = 0; xi != nx; xi++, xoff += xstep, d.y = (float)yreset, d.x = (float)(d.x + binsizeX)) {
          for (int yi = 0, yoff = 0; yi != ny; yi++, yoff += ystep, d.z = (float)zreset, d.y = (float)(d.y + binsizeY)) {
            for (int zi = 0, zoff = 0; zi != nz; zi++, zoff += zstep, d.z = (float)(d.z + binsizeZ)) {
              if (dot(d, pn) < binRadius) bins[xoff + yoff + zoff].push_back(i);
            }
          }
        }
      } else {
        if (b.aabbNeedsUpdate) updateAABB(b, shapes);
        addBoxToBins(b.aabbLo.x, b.aabbLo.y, b.aabbLo.z, b.aabbHi.x, b.aabbHi.y, b.aabbHi.z, i);
      }
    }
    for (int i = 0; i != nBins; i++) {
      const std::vector<int>& bin = bins[i];
      int len = (int)bin.size();
      if (len > 1) {
        for (int xi = 0; xi != len; xi++)
          for (int yi = 0; yi != xi; yi++)
            if (needBroadphaseCollision(bodies[bin[xi]], bodies[bin[yi]])) intersectionTest(bin[xi], bin[yi]);
      }
    }
    // makePairsUnique (repaired)
    std::vector<int> q1 = p1, q2 = p2;
    std::map<std::pair<int, int>, int> lastIndex;
    std::vector<std::pair<int, int>> order;
    for (size_t i = 0; i < q1.size(); i++) {
      std::pair<int, int> key(std::min(q1[i], q2[i]), std::max(q1[i], q2[i]));
      auto it = lastIndex.find(key);
      if (it == lastIndex.end()) { lastIndex[key] = (int)i; order.push_back(key); }
      else it->second = (int)i;
    }
    p1.clear(); p2.clear();
    for (auto& k : order) { int idx = lastIndex[k]; p1.push_back(q1[idx]); p2.push_back(q2[idx]); }
  }

  // ---------------------------------------------------------------- narrowphase
  // narrow_phase.dart:492-528
  Eq& createContactEquation(int bi, int bj, const Shape& si, const Shape& sj, int rsi, int rsj) {
    contacts.emplace_back();
    Eq& c = contacts.back();
    c.kind = CP_ROW_CONTACT;
    c.bi = bi; c.bj = bj;
    c.minForce = 0; c.maxForce = 1e6;
    c.enabled = bodies[bi].response && bodies[bj].response && si.response && sj.response;
    const ContactMat& cm = current;
    c.restitution = cm.restitution;
    c.setSpookParams(cm.cs, cm.cr, dt);
    int matA = si.material >= 0 ? si.material : bodies[bi].material;
    int matB = sj.material >= 0 ? sj.material : bodies[bj].material;
    if (matA >= 0 && matB >= 0 && materials[matA].restitution >= 0 && materials[matB].restitution >= 0)
      c.restitution = materials[matA].restitution * materials[matB].restitution;
    c.si = rsi; c.sj = rsj;
    c.pair = curPair;
    if (split) c.id = takeId(contactPool);
    return c;
  }
  // narrow_phase.dart:530-586
  bool createFrictionEquationsFromContact(const Eq& ce) {
    const Body& A = bodies[ce.bi];
    const Body& B = bodies[ce.bj];
    const ContactMat& cm = current;
    double friction = cm.friction;
    int matA = shapes[ce.si].material >= 0 ? shapes[ce.si].material : A.material;
    int matB = shapes[ce.sj].material >= 0 ? shapes[ce.sj].material : B.material;
    if (matA >= 0 && matB >= 0 && materials[matA].friction >= 0 && materials[matB].friction >= 0)
      friction = materials[matA].friction * materials[matB].friction;
    if (friction > 0) {
      double mug = friction * length(hasFrictionGravity ? frictionGravity : gravity);
      double reducedMass = A.invMass + B.invMass;
      if (reducedMass > 0) reducedMass = 1 / reducedMass;
      Eq c1, c2;
      c1.kind = c2.kind = CP_ROW_FRICTION;
      c1.bi = c2.bi = ce.bi;
      c1.bj = c2.bj = ce.bj;
      c1.minForce = c2.minForce = -mug * reducedMass;
      c1.maxForce = c2.maxForce = mug * reducedMass;
      c1.ri = ce.ri; c1.rj = ce.rj; c2.ri = ce.ri; c2.rj = ce.rj;
      tangents(ce.ni, c1.t, c2.t);
      c1.setSpookParams(cm.fs, cm.fr, dt);
      c2.setSpookParams(cm.fs, cm.fr, dt);
      c1.enabled = ce.enabled; c2.enabled = ce.enabled;
      c1.si = c2.si = ce.si; c1.sj = c2.sj = ce.sj;
      c1.pair = c2.pair = ce.pair;
      if (split) {  // c1 then c2 (narrow_phase.dart:556-557)
        c1.id = takeId(frictionPool);
        c2.id = takeId(frictionPool);
      }
      frictionEqs.push_back(c1);
      frictionEqs.push_back(c2);
      return true;
    }
    return false;
  }
  // narrow_phase.dart:589-627
  void createFrictionFromAverage(int numContacts) {
    Eq c = contacts.back();
    if (!createFrictionEquationsFromContact(c) || numContacts == 1) return;
    Eq& f1 = frictionEqs[frictionEqs.size() - 2];
    Eq& f2 = frictionEqs[frictionEqs.size() - 1];
    V3 avgN, avgA, avgB;
    int bodyA = c.bi;
    for (int i = 0; i != numContacts; i++) {
      const Eq& ci = contacts[contacts.size() - 1 - i];
      if (ci.bi != bodyA) {
        add2(avgN, ci.ni, avgN); add2(avgA, ci.ri, avgA); add2(avgB, ci.rj, avgB);
      } else {
        sub2(avgN, ci.ni, avgN); add2(avgA, ci.rj, avgA); add2(avgB, ci.ri, avgB);
      }
    }
    double inv = 1.0 / numContacts;
    scale2(avgA, inv, f1.ri);
    scale2(avgB, inv, f1.rj);
    f2.ri = f1.ri; f2.rj = f1.rj;
    normalize(avgN);
    tangents(avgN, f1.t, f2.t);
  }
  void finishContact(Eq& r, const V3& xi, const V3& xj) {
    // "Make relative to bodies": ri += xi - bi.position; rj += xj - bj.position
    add2(r.ri, xi, r.ri); sub2(r.ri, bodies[r.bi].position, r.ri);
    add2(r.rj, xj, r.rj); sub2(r.rj, bodies[r.bj].position, r.rj);
  }

  // narrow_phase.dart:723-765
  void sphereSphere(const Shape& si, const Shape& sj, const V3& xi, const V3& xj, int bi, int bj, int rsi, int rsj) {
    Eq& c = createContactEquation(bi, bj, si, sj, rsi, rsj);
    sub2(xj, xi, c.ni);
    normalize(c.ni);
    c.ri = c.ni; c.rj = c.ni;
    scale2(c.ri, si.radius, c.ri);
    scale2(c.rj, -sj.radius, c.rj);
    finishContact(c, xi, xj);
    createFrictionEquationsFromContact(c);
  }
  // narrow_phase.dart:766-815
  void spherePlane(const Shape& si, const Shape& sj, const V3& xi, const V3& xj, const Q4& qj, int bi, int bj, int rsi, int rsj) {
    Eq c = createContactEquation(bi, bj, si, sj, rsi, rsj);
    contacts.pop_back();
    setValues(c.ni, 0, 0, 1);
    vmult(qj, c.ni, c.ni);
    negate(c.ni);
    normalize(c.ni);
    scale2(c.ni, si.radius, c.ri);
    V3 pops, ortho;
    sub2(xi, xj, pops);
    scale2(c.ni, dot(c.ni, pops), ortho);
    sub2(pops, ortho, c.rj);
    if (-dot(pops, c.ni) <= si.radius) {
      finishContact(c, xi, xj);
      contacts.push_back(c);
      createFrictionEquationsFromContact(contacts.back());
    }
  }
  // box.dart:99-115
  static void getSideNormals(const Shape& s, V3* sides, const Q4& q) {
    const V3& ex = s.halfExtents;
    setValues(sides[0], ex.x, 0, 0); setValues(sides[1], 0, ex.y, 0); setValues(sides[2], 0, 0, ex.z);
    setValues(sides[3], -ex.x, 0, 0); setValues(sides[4], 0, -ex.y, 0); setValues(sides[5], 0, 0, -ex.z);
    for (int i = 0; i != 6; i++) vmult(q, sides[i], sides[i]);
  }
  // narrow_phase.dart:816-1038
  void sphereBox(const Shape& si, const Shape& sj, const V3& xi, const V3& xj, const Q4& qj, int bi, int bj, int rsi, int rsj) {
    V3 sides[6];
    V3 boxToSphere;
    sub2(xi, xj, boxToSphere);
    getSideNormals(sj, sides, qj);
    double R = si.radius;
    bool found = false;
    V3 sideNs, sideNs1, sideNs2;
    double sideH = 0, sidePenetrations = 0, sideDot1 = 0, sideDot2 = 0, sideDistance = 0;
    bool haveSideDistance = false;
    for (int idx = 0; idx != 6 && !found; idx++) {
      V3 ns = sides[idx];
      double h = length(ns);
      normalize(ns);
      double dotv = dot(boxToSphere, ns);
      if (dotv < h + R && dotv > 0) {
        V3 ns1 = sides[(idx + 1) % 3], ns2 = sides[(idx + 2) % 3];
        double h1 = length(ns1), h2 = length(ns2);
        normalize(ns1); normalize(ns2);
        double dot1 = dot(boxToSphere, ns1), dot2 = dot(boxToSphere, ns2);
        if (dot1 < h1 && dot1 > -h1 && dot2 < h2 && dot2 > -h2) {
          double dist = std::fabs(dotv - h - R);
          if (!haveSideDistance || dist < sideDistance) {
            haveSideDistance = true;
            sideDistance = dist; sideDot1 = dot1; sideDot2 = dot2; sideH = h;
            sideNs = ns; sideNs1 = ns1; sideNs2 = ns2;
            sidePenetrations++;
          }
        }
      }
    }
    if (sidePenetrations != 0) {
      found = true;
      Eq& r = createContactEquation(bi, bj, si, sj, rsi, rsj);
      scale2(sideNs, -R, r.ri);
      r.ni = sideNs;
      negate(r.ni);
      scale2(sideNs, sideH, sideNs);
      scale2(sideNs1, sideDot1, sideNs1);
      add2(sideNs, sideNs1, sideNs);
      scale2(sideNs2, sideDot2, sideNs2);
      add2(sideNs, sideNs2, r.rj);
      finishContact(r, xi, xj);
      createFrictionEquationsFromContact(r);
    }
    V3 rj, sphereToCorner;
    for (int j = 0; j != 2 && !found; j++)
      for (int k = 0; k != 2 && !found; k++)
        for (int l = 0; l != 2 && !found; l++) {
          setValues(rj, 0, 0, 0);
          if (j != 0) add2(rj, sides[0], rj); else sub2(rj, sides[0], rj);
          if (k != 0) add2(rj, sides[1], rj); else sub2(rj, sides[1], rj);
          if (l != 0) add2(rj, sides[2], rj); else sub2(rj, sides[2], rj);
          add2(xj, rj, sphereToCorner);
          sub2(sphereToCorner, xi, sphereToCorner);
          if (length2(sphereToCorner) < R * R) {
            found = true;
            Eq& r = createContactEquation(bi, bj, si, sj, rsi, rsj);
            r.ri = sphereToCorner;
            normalize(r.ri);
            r.ni = r.ri;
            scale2(r.ri, R, r.ri);
            r.rj = rj;
            finishContact(r, xi, xj);
            createFrictionEquationsFromContact(r);
          }
        }
    V3 edgeTangent, edgeCenter, rr, orthogonal, dist;
    for (int j = 0; j != 6 && !found; j++)
      for (int k = 0; k != 6 && !found; k++) {
        if (j % 3 != k % 3) {
          cross2(sides[k], sides[j], edgeTangent);
          normalize(edgeTangent);
          add2(sides[j], sides[k], edgeCenter);
          rr = xi;
          sub2(rr, edgeCenter, rr);
          sub2(rr, xj, rr);
          double orthonorm = dot(rr, edgeTangent);
          scale2(edgeTangent, orthonorm, orthogonal);
          int l = 0;
          while (l == j % 3 || l == k % 3) l++;
          dist = xi;
          sub2(dist, orthogonal, dist);
          sub2(dist, edgeCenter, dist);
          sub2(dist, xj, dist);
          double tdist = std::fabs(orthonorm);
          double ndist = length(dist);
          if (tdist < length(sides[l]) && ndist < R) {
            found = true;
            Eq& res = createContactEquation(bi, bj, si, sj, rsi, rsj);
            add2(edgeCenter, orthogonal, res.rj);
            res.ni = dist;
            negate(res.ni);
            normalize(res.ni);
            res.ri = res.rj;
            add2(res.ri, xj, res.ri);
            sub2(res.ri, xi, res.ri);
            normalize(res.ri);
            scale2(res.ri, R, res.ri);
            finishContact(res, xi, xj);
            createFrictionEquationsFromContact(res);
          }
        }
      }
  }
  // narrow_phase.dart:2584-2617
  static bool pointInPolygon(const std::vector<V3>& verts, const V3& normal, const V3& p) {
    int state = -1;  // -1 unset, 1 positive, 0 non-positive
    const int N = (int)verts.size();
    for (int i = 0; i != N; i++) {
      const V3& v = verts[i];
      V3 edge, exn, vtp;
      sub2(verts[(i + 1) % N], v, edge);
      cross2(edge, normal, exn);
      sub2(p, v, vtp);
      double r = dot(exn, vtp);
      if (state == -1 || (r > 0 && state == 1) || (r <= 0 && state == 0)) {
        if (state == -1) state = r > 0 ? 1 : 0;
        continue;
      }
      return false;
    }
    return true;
  }
  // narrow_phase.dart:1039-1257
  void sphereConvex(const Shape& si, const Shape& sj, const V3& xi, const V3& xj, const Q4& qj, int bi, int bj, int rsi, int rsj) {
    const Hull& H = sj.hull;
    double R = si.radius;
    bool found = false;
    for (size_t i = 0; i != H.vertices.size(); i++) {
      V3 worldCorner, s2c;
      vmult(qj, H.vertices[i], worldCorner);
      add2(xj, worldCorner, worldCorner);
      sub2(worldCorner, xi, s2c);
      if (length2(s2c) < R * R) {
        Eq& r = createContactEquation(bi, bj, si, sj, rsi, rsj);
        r.ri = s2c;
        normalize(r.ri);
        r.ni = r.ri;
        scale2(r.ri, R, r.ri);
        sub2(worldCorner, xj, r.rj);
        add2(r.ri, xi, r.ri); sub2(r.ri, bodies[bi].position, r.ri);
        add2(r.rj, xj, r.rj); sub2(r.rj, bodies[bj].position, r.rj);
        createFrictionEquationsFromContact(r);
        return;
      }
    }
    for (size_t i = 0, nf = H.faces.size(); i != nf && !found; i++) {
      const std::vector<int>& face = H.faces[i];
      V3 worldNormal, worldPoint, wsp, penVec, wp2s;
      vmult(qj, H.faceNormals[i], worldNormal);
      vmult(qj, H.vertices[face[0]], worldPoint);
      add2(worldPoint, xj, worldPoint);
      scale2(worldNormal, -R, wsp);
      add2(xi, wsp, wsp);
      sub2(wsp, worldPoint, penVec);
      double penetration = dot(penVec, worldNormal);
      sub2(xi, worldPoint, wp2s);
      if (penetration < 0 && dot(wp2s, worldNormal) > 0) {
        std::vector<V3> faceVerts(face.size());
        for (size_t j = 0; j != face.size(); j++) {
          vmult(qj, H.vertices[face[j]], faceVerts[j]);
          add2(xj, faceVerts[j], faceVerts[j]);
        }
        if (pointInPolygon(faceVerts, worldNormal, xi)) {
          found = true;
          Eq& r = createContactEquation(bi, bj, si, sj, rsi, rsj);
          scale2(worldNormal, -R, r.ri);
          r.ni = worldNormal;
          negate(r.ni);
          V3 pv2, psp;
          scale2(worldNormal, -penetration, pv2);
          scale2(worldNormal, -R, psp);
          sub2(xi, xj, r.rj);
          add2(r.rj, psp, r.rj);
          add2(r.rj, pv2, r.rj);
          add2(r.rj, xj, r.rj); sub2(r.rj, bodies[bj].position, r.rj);
          add2(r.ri, xi, r.ri); sub2(r.ri, bodies[bi].position, r.ri);
          createFrictionEquationsFromContact(r);
          return;
        } else {
          const int fl = (int)face.size();
          for (int j = 0; j != fl; j++) {
            V3 v1, v2, edge, edgeUnit, p, v1ToXi, xiToP;
            vmult(qj, H.vertices[face[(j + 1) % fl]], v1);
            vmult(qj, H.vertices[face[(j + 2) % fl]], v2);
            add2(xj, v1, v1);
            add2(xj, v2, v2);
            sub2(v2, v1, edge);
            unit(edge, edgeUnit);
            sub2(xi, v1, v1ToXi);
            double dotv = dot(v1ToXi, edgeUnit);
            scale2(edgeUnit, dotv, p);
            add2(p, v1, p);
            sub2(p, xi, xiToP);
            if (dotv > 0 && dotv * dotv < length2(edge) && length2(xiToP) < R * R) {
              Eq& r = createContactEquation(bi, bj, si, sj, rsi, rsj);
              sub2(p, xj, r.rj);
              sub2(p, xi, r.ni);
              normalize(r.ni);
              scale2(r.ni, R, r.ri);
              add2(r.rj, xj, r.rj); sub2(r.rj, bodies[bj].position, r.rj);
              add2(r.ri, xi, r.ri); sub2(r.ri, bodies[bi].position, r.ri);
              createFrictionEquationsFromContact(r);
              return;
            }
          }
        }
      }
    }
  }
  // narrow_phase.dart:1847-1915 (planeBox :1786-1804 forwards here)
  void planeConvex(const Shape& si, const Shape& sj, const V3& xi, const V3& xj, const Q4& qi, const Q4& qj, int bi, int bj, int rsi, int rsj) {
    V3 worldNormal, worldVertex, relpos, projected;
    setValues(worldNormal, 0, 0, 1);
    vmult(qi, worldNormal, worldNormal);
    int numContacts = 0;
    const Hull& H = sj.hull;
    for (size_t i = 0; i != H.vertices.size(); i++) {
      worldVertex = H.vertices[i];
      vmult(qj, worldVertex, worldVertex);
      add2(xj, worldVertex, worldVertex);
      sub2(worldVertex, xi, relpos);
      double dotv = dot(worldNormal, relpos);
      if (dotv <= 0.0) {
        Eq& r = createContactEquation(bi, bj, si, sj, rsi, rsj);
        scale2(worldNormal, dot(worldNormal, relpos), projected);
        sub2(worldVertex, projected, projected);
        sub2(projected, xi, r.ri);
        r.ni = worldNormal;
        sub2(worldVertex, xj, r.rj);
        finishContact(r, xi, xj);
        numContacts++;
        if (!enableFrictionReduction) createFrictionEquationsFromContact(r);
      }
    }
    if (enableFrictionReduction && numContacts != 0) createFrictionFromAverage(numContacts);
  }
  // convex_polyhedron.dart:843-883
  static void project(const Hull& h, const V3& axis, const V3& pos, const Q4& quat, double& mx, double& mn) {
    V3 localAxis, localOrigin;
    vectorToLocalFrame(quat, axis, localAxis);
    pointToLocalFrame(pos, quat, localOrigin, localOrigin);
    double add = dot(localOrigin, localAxis);
    double max = dot(h.vertices[0], localAxis), min = max;
    for (size_t i = 1; i < h.vertices.size(); i++) {
      double val = dot(h.vertices[i], localAxis);
      if (val > max) max = val;
      if (val < min) min = val;
    }
    min -= add;
    max -= add;
    if (min > max) std::swap(min, max);
    mx = max; mn = min;
  }
  // convex_polyhedron.dart:360-384; returns false when separated
  static bool testSepAxis(const Hull& A, const Hull& B, const V3& axis, const V3& posA, const Q4& quatA, const V3& posB, const Q4& quatB, double& depth) {
    double maxA, minA, maxB, minB;
    project(A, axis, posA, quatA, maxA, minA);
    project(B, axis, posB, quatB, maxB, minB);
    if (maxA < minB || maxB < minA) return false;
    double d0 = maxA - minB, d1 = maxB - minA;
    depth = d0 < d1 ? d0 : d1;
    return true;
  }
  // convex_polyhedron.dart:232-356
  static bool findSeparatingAxis(const Hull& A, const Hull& B, const V3& posA, const Q4& quatA, const V3& posB, const Q4& quatB, V3& target) {
    double dmin = INF;
    double d;
    if (A.hasAxes) {
      for (size_t i = 0; i < A.faces.size(); i++) {
        V3 n;
        vmult(quatA, A.faceNormals[i], n);
        if (!testSepAxis(A, B, n, posA, quatA, posB, quatB, d)) return false;
        if (d < dmin) { dmin = d; target = n; }
      }
    }
    if (B.hasAxes) {
      for (size_t i = 0; i < B.faces.size(); i++) {
        V3 n;
        vmult(quatB, B.faceNormals[i], n);
        if (!testSepAxis(A, B, n, posA, quatA, posB, quatB, d)) return false;
        if (d < dmin) { dmin = d; target = n; }
      }
    }
    for (size_t e0 = 0; e0 != A.uniqueEdges.size(); e0++) {
      V3 we0;
      vmult(quatA, A.uniqueEdges[e0], we0);
      for (size_t e1 = 0; e1 != B.uniqueEdges.size(); e1++) {
        V3 we1, cr;
        vmult(quatB, B.uniqueEdges[e1], we1);
        cross2(we0, we1, cr);
        if (!almostZero(cr)) {
          normalize(cr);
          if (!testSepAxis(A, B, cr, posA, quatA, posB, quatB, d)) return false;
          if (d < dmin) { dmin = d; target = cr; }
        }
      }
    }
    V3 deltaC;
    sub2(posB, posA, deltaC);
    if (dot(deltaC, target) > 0.0) negate(target);
    return true;
  }
  struct ClipPoint { V3 point; V3 normal; double depth; };
  // convex_polyhedron.dart:545-587
  static void clipFaceAgainstPlane(const std::vector<V3>& in, std::vector<V3>& out, const V3& n, double c) {
    const int numVerts = (int)in.size();
    if (numVerts < 2) return;
    V3 first = in[numVerts - 1];
    double nDotFirst = dot(n, first) + c;
    for (int vi = 0; vi < numVerts; vi++) {
      const V3& last = in[vi];
      double nDotLast = dot(n, last) + c;
      if (nDotFirst < 0) {
        if (nDotLast < 0) out.push_back(last);
        else { V3 nv; lerp(first, last, nDotFirst / (nDotFirst - nDotLast), nv); out.push_back(nv); }
      } else if (nDotLast < 0) {
        V3 nv; lerp(first, last, nDotFirst / (nDotFirst - nDotLast), nv);
        out.push_back(nv);
        out.push_back(last);
      }
      first = last;
      nDotFirst = nDotLast;
    }
  }
  static double planeConstantOfFace(const Hull& h, int f) { return -dot(h.faceNormals[f], h.vertices[h.faces[f][0]]); }
  // convex_polyhedron.dart:417-541
  static void clipFaceAgainstHull(const Hull& A, const V3& sepNormal, const V3& posA, const Q4& quatA, std::vector<V3>& pIn, double minDist, double maxDist, std::vector<ClipPoint>& result) {
    int closestFaceA = -1;
    double dmin = INF;
    for (size_t face = 0; face < A.faces.size(); face++) {
      V3 n;
      vmult(quatA, A.faceNormals[face], n);
      double d = dot(n, sepNormal);
      if (d < dmin) { dmin = d; closestFaceA = (int)face; }
    }
    if (closestFaceA < 0) return;
    const std::vector<int>& polyA = A.faces[closestFaceA];
    std::vector<int> connected;
    for (size_t i = 0; i < A.faces.size(); i++)
      for (size_t j = 0; j < A.faces[i].size(); j++)
        if (std::find(polyA.begin(), polyA.end(), A.faces[i][j]) != polyA.end() && (int)i != closestFaceA &&
            std::find(connected.begin(), connected.end(), (int)i) == connected.end())
          connected.push_back((int)i);
    std::vector<V3> pOut;
    const int numVerticesA = (int)polyA.size();
    for (int i = 0; i < numVerticesA; i++) {
      int otherFace = (!connected.empty() && (int)connected.size() > i) ? connected[i] : 0;
      double localPlaneEq = planeConstantOfFace(A, otherFace);
      V3 pn;
      vmult(quatA, A.faceNormals[otherFace], pn);
      double planeEqWS = localPlaneEq - dot(pn, posA);
      clipFaceAgainstPlane(pIn, pOut, pn, planeEqWS);
      pIn.swap(pOut);
      pOut.clear();
    }
    double localPlaneEq = planeConstantOfFace(A, closestFaceA);
    V3 pn;
    vmult(quatA, A.faceNormals[closestFaceA], pn);
    double planeEqWS = localPlaneEq - dot(pn, posA);
    for (size_t i = 0; i < pIn.size(); i++) {
      double depth = dot(pn, pIn[i]) + planeEqWS;
      if (depth <= minDist) depth = minDist;
      if (depth <= maxDist) {
        if (depth <= 1e-6) result.push_back({pIn[i], pn, depth});
      }
    }
  }
  // convex_polyhedron.dart:189-227
  static void clipAgainstHull(const Hull& A, const V3& posA, const Q4& quatA, const Hull& B, const V3& posB, const Q4& quatB, const V3& sepNormal, double minDist, double maxDist, std::vector<ClipPoint>& result) {
    int closestFaceB = -1;
    double dmax = -INF;
    for (size_t face = 0; face < B.faces.size(); face++) {
      V3 n;
      vmult(quatB, B.faceNormals[face], n);
      double d = dot(n, sepNormal);
      if (d > dmax) { dmax = d; closestFaceB = (int)face; }
    }
    if (closestFaceB < 0) return;
    std::vector<V3> worldVertsB1;
    for (int vi : B.faces[closestFaceB]) {
      V3 w = B.vertices[vi];
      vmult(quatB, w, w);
      add2(posB, w, w);
      worldVertsB1.push_back(w);
    }
    clipFaceAgainstHull(A, sepNormal, posA, quatA, worldVertsB1, minDist, maxDist, result);
  }
  // narrow_phase.dart:1981-2043 (boxBox :1693, boxConvex :1713 forward here)
  void convexConvex(const Shape& si, const Shape& sj, const V3& xi, const V3& xj, const Q4& qi, const Q4& qj, int bi, int bj, int rsi, int rsj) {
    if (distanceTo(xi, xj) > si.bsr + sj.bsr) return;
    V3& sepAxis = sepAxisPersist;
    if (findSeparatingAxis(si.hull, sj.hull, xi, qi, xj, qj, sepAxis)) {
      std::vector<ClipPoint> res;
      clipAgainstHull(si.hull, xi, qi, sj.hull, xj, qj, sepAxis, -100, 100, res);
      int numContacts = 0;
      for (size_t j = 0; j != res.size(); j++) {
        Eq& r = createContactEquation(bi, bj, si, sj, rsi, rsj);
        r.ni = sepAxis;
        negate(r.ni);
        V3 q = res[j].normal;
        negate(q);
        scale2(q, res[j].depth, q);
        add2(res[j].point, q, r.ri);
        r.rj = res[j].point;
        sub2(r.ri, xi, r.ri);
        sub2(r.rj, xj, r.rj);
        finishContact(r, xi, xj);
        numContacts++;
        if (!enableFrictionReduction) createFrictionEquationsFromContact(r);
      }
      if (enableFrictionReduction && numContacts != 0) createFrictionFromAverage(numContacts);
    }
  }

  // narrow_phase.dart:634-721
  void getContacts() {  // narrow_phase.dart:634-721
    contacts.clear();
    frictionEqs.clear();
    const int NP = (int)p1.size();
    for (int k = 0; k != NP; k++) {
      int ibi = p1[k], ibj = p2[k];
      Body& bi = bodies[ibi];
      Body& bj = bodies[ibj];
      const ContactMat* bodyCM = nullptr;
      if (bi.material >= 0 && bj.material >= 0) bodyCM = getCM(bi.material, bj.material);
      bool justTest = (bi.type == CP_BODY_KINEMATIC && bj.type == CP_BODY_STATIC) ||
                      (bi.type == CP_BODY_STATIC && bj.type == CP_BODY_KINEMATIC) ||
                      (bi.type == CP_BODY_KINEMATIC && bj.type == CP_BODY_KINEMATIC);
      for (int a = 0; a < bi.numShapes(); a++) {
        Q4 qi; V3 xi;
        qmultiply2(bi.quaternion, bi.orientationAt(a), qi);
        vmult(bi.quaternion, bi.offsetAt(a), xi);
        add2(xi, bi.position, xi);
        const int isi = bi.shapeAt(a);
        const Shape& si = shapes[isi];
        for (int b = 0; b < bj.numShapes(); b++) {
          Q4 qj; V3 xj;
          qmultiply2(bj.quaternion, bj.orientationAt(b), qj);
          vmult(bj.quaternion, bj.offsetAt(b), xj);
          add2(xj, bj.position, xj);
          const int isj = bj.shapeAt(b);
          const Shape& sj = shapes[isj];
          if (!((si.mask & sj.group) != 0 && (sj.mask & si.group) != 0)) continue;
          if (distanceTo(xi, xj) > si.bsr + sj.bsr) continue;
          const ContactMat* shapeCM = nullptr;
          if (si.material >= 0 && sj.material >= 0) shapeCM = getCM(si.material, sj.material);
          current = shapeCM ? *shapeCM : (bodyCM ? *bodyCM : defaultCM);
          curPair = k;
          if (justTest) {
            // a justTest resolver adds no contacts; where it would find one it
            // registers the overlap (narrow_phase.dart:712-715).  spherePlane
            // takes its equation object before the justTest return
            // (:781-799), and the object is lost to the pool
            const bool spherePlane = (si.type == CP_SHAPE_SPHERE && sj.type == CP_SHAPE_PLANE) ||
                                     (sj.type == CP_SHAPE_SPHERE && si.type == CP_SHAPE_PLANE);
            if (split && spherePlane) takeId(contactPool);
            if (events) {
              // the reference's resolvers return before creating equations:
              // the trial leaves the pools and the id counter as they were
              const size_t nc = contacts.size(), nf = frictionEqs.size();
              const std::vector<long long> keepC = split ? contactPool : std::vector<long long>();
              const std::vector<long long> keepF = split ? frictionPool : std::vector<long long>();
              const long long keepId = idCounter;
              if (si.type < sj.type) dispatch(si, sj, xi, xj, qi, qj, ibi, ibj, isi, isj, isi, isj);
              else dispatch(sj, si, xj, xi, qj, qi, ibj, ibi, isj, isi, isi, isj);
              if (contacts.size() > nc) {
                shapeOverlapKeeper.set(shapeId(isi), shapeId(isj));
                bodyOverlapKeeper.set(bodyId(ibi), bodyId(ibj));
              }
              contacts.resize(nc);
              frictionEqs.resize(nf);
              if (split) {
                contactPool = keepC;
                frictionPool = keepF;
                idCounter = keepId;
              }
            }
            continue;
          }
          if (si.type < sj.type) dispatch(si, sj, xi, xj, qi, qj, ibi, ibj, isi, isj, isi, isj);
          else dispatch(sj, si, xj, xi, qj, qi, ibj, ibi, isj, isi, isi, isj);
        }
      }
    }
  }
  // a ConvexPolyhedron with a resolver row of its own type: Convex, Cylinder,
  // Capsule, Cone, SizedPlane (narrow_phase.dart:130-168)
  static bool isHull(int t) { return t >= CP_SHAPE_CONVEX && t <= CP_SHAPE_SIZED_PLANE; }
  // narrow_phase.dart:116-238 (resolver table); rsi/rsj are the shapes in
  // getContacts order, passed through unchanged as in :707-709.
  // shA / shB: the indices of shapes a / b (type order)
  void dispatch(const Shape& a, const Shape& b, const V3& xa, const V3& xb, const Q4& qa, const Q4& qb, int ba, int bb, int shA,
                int shB, int rsi, int rsj) {
    int ta = a.type, tb = b.type;
    if (ta == CP_SHAPE_SPHERE && tb == CP_SHAPE_SPHERE) sphereSphere(a, b, xa, xb, ba, bb, rsi, rsj);
    else if (ta == CP_SHAPE_SPHERE && tb == CP_SHAPE_PLANE) spherePlane(a, b, xa, xb, qb, ba, bb, rsi, rsj);
    else if (ta == CP_SHAPE_SPHERE && tb == CP_SHAPE_BOX) sphereBox(a, b, xa, xb, qb, ba, bb, rsi, rsj);
    else if (ta == CP_SHAPE_SPHERE && isHull(tb)) sphereConvex(a, b, xa, xb, qb, ba, bb, rsi, rsj);
    // planeBox / boxBox / boxConvex pass their own (type-ordered) shapes on
    else if (ta == CP_SHAPE_PLANE && tb == CP_SHAPE_BOX) planeConvex(a, b, xa, xb, qa, qb, ba, bb, shA, shB);
    else if (ta == CP_SHAPE_PLANE && isHull(tb)) planeConvex(a, b, xa, xb, qa, qb, ba, bb, rsi, rsj);
    else if (ta == CP_SHAPE_BOX && tb == CP_SHAPE_BOX) convexConvex(a, b, xa, xb, qa, qb, ba, bb, shA, shB);
    else if (ta == CP_SHAPE_BOX && isHull(tb)) convexConvex(a, b, xa, xb, qa, qb, ba, bb, shA, shB);
    // convex + sizedPlane finds no resolver: its table key is spelled
    // "convexSizedPlane" but looked up lower-cased (narrow_phase.dart:444,476-479)
    else if (isHull(ta) && isHull(tb) && !(ta == CP_SHAPE_CONVEX && tb == CP_SHAPE_SIZED_PLANE))
      convexConvex(a, b, xa, xb, qa, qb, ba, bb, rsi, rsj);
    // plane-plane: no resolver
  }

  // ---------------------------------------------------------------- equations
  void computeGiMf(const Eq& e, double& out) const {
    const Body& bi = bodies[e.bi];
    const Body& bj = bodies[e.bj];
    V3 iMfi, iMfj, ti, tj;
    scale2(bi.force, bi.invMassSolve, iMfi);
    scale2(bj.force, bj.invMassSolve, iMfj);
    mvmult(bi.invInertiaWorldSolve, bi.torque, ti);
    mvmult(bj.invInertiaWorldSolve, bj.torque, tj);
    out = (dot(iMfi, e.gaS) + dot(ti, e.gaR)) + (dot(iMfj, e.gbS) + dot(tj, e.gbR));
  }
  double computeGW(const Eq& e) const {
    const Body& bi = bodies[e.bi];
    const Body& bj = bodies[e.bj];
    return (dot(bi.velocity, e.gaS) + dot(bi.angularVelocity, e.gaR)) + (dot(bj.velocity, e.gbS) + dot(bj.angularVelocity, e.gbR));
  }
  double computeGWlambda(const Eq& e) const {
    const Body& bi = bodies[e.bi];
    const Body& bj = bodies[e.bj];
    return (dot(bi.vlambda, e.gaS) + dot(bi.wlambda, e.gaR)) + (dot(bj.vlambda, e.gbS) + dot(bj.wlambda, e.gbR));
  }
  double computeC(const Eq& e) const {
    const Body& bi = bodies[e.bi];
    const Body& bj = bodies[e.bj];
    double result = bi.invMassSolve + bj.invMassSolve;
    V3 tmp;
    mvmult(bi.invInertiaWorldSolve, e.gaR, tmp);
    result += dot(tmp, e.gaR);
    mvmult(bj.invInertiaWorldSolve, e.gbR, tmp);
    result += dot(tmp, e.gbR);
    return result + e.eps;
  }
  void addToWlambda(const Eq& e, double dl) {
    Body& bi = bodies[e.bi];
    Body& bj = bodies[e.bj];
    addScaledVector(bi.vlambda, bi.invMassSolve * dl, e.gaS, bi.vlambda);
    addScaledVector(bj.vlambda, bj.invMassSolve * dl, e.gbS, bj.vlambda);
    V3 temp;
    mvmult(bi.invInertiaWorldSolve, e.gaR, temp);
    addScaledVector(bi.wlambda, dl, temp, bi.wlambda);
    mvmult(bj.invInertiaWorldSolve, e.gbR, temp);
    addScaledVector(bj.wlambda, dl, temp, bj.wlambda);
  }
  double computeB(Eq& e, double h) {
    const Body& bi = bodies[e.bi];
    const Body& bj = bodies[e.bj];
    double giMf;
    switch (e.kind) {
      case CP_ROW_CONTACT: {  // contact_equation.dart:34-77
        V3 rixn, rjxn, pen;
        cross2(e.ri, e.ni, rixn);
        cross2(e.rj, e.ni, rjxn);
        e.gaS = e.ni; negate(e.gaS);
        e.gaR = rixn; negate(e.gaR);
        e.gbS = e.ni;
        e.gbR = rjxn;
        pen = bj.position;
        add2(pen, e.rj, pen);
        sub2(pen, bi.position, pen);
        sub2(pen, e.ri, pen);
        double g = dot(e.ni, pen);
        double ePlusOne = e.restitution + 1;
        double gw = ePlusOne * dot(bj.velocity, e.ni) - ePlusOne * dot(bi.velocity, e.ni) + dot(bj.angularVelocity, rjxn) - dot(bi.angularVelocity, rixn);
        computeGiMf(e, giMf);
        return -g * e.a - gw * e.b - h * giMf;
      }
      case CP_ROW_FRICTION: {  // friction_equation.dart:19-47
        V3 rixt, rjxt;
        cross2(e.ri, e.t, rixt);
        cross2(e.rj, e.t, rjxt);
        e.gaS = e.t; negate(e.gaS);
        e.gaR = rixt; negate(e.gaR);
        e.gbS = e.t;
        e.gbR = rjxt;
        double gw = computeGW(e);
        computeGiMf(e, giMf);
        return -gw * e.b - h * giMf;
      }
      case CP_ROW_ROTATIONAL: {  // rotational_equation.dart:34-58
        V3 nixnj, njxni;
        cross2(e.axisA, e.axisB, nixnj);
        cross2(e.axisB, e.axisA, njxni);
        e.gaR = njxni;
        e.gbR = nixnj;
        double g = e.cosMaxAngle - dot(e.axisA, e.axisB);
        double gW = computeGW(e);
        computeGiMf(e, giMf);
        return -g * e.a - gW * e.b - h * giMf;
      }
      default: {  // rotational_motor_equation.dart:17-33
        e.gaR = e.axisA;
        e.gbR = e.axisB; negate(e.gbR);
        double gw = computeGW(e) - e.targetVelocity;
        computeGiMf(e, giMf);
        return -gw * e.b - h * giMf;
      }
    }
  }
  // rigid_body.dart:303-314
  static void updateSolveMassProperties(Body& b) {
    if (b.sleepState == CP_SLEEPING || b.type == CP_BODY_KINEMATIC) {
      b.invMassSolve = 0;
      b.invInertiaSolve = V3();
      b.invInertiaWorldSolve = M3();
    } else {
      b.invMassSolve = b.invMass;
      b.invInertiaSolve = b.invInertia;
      b.invInertiaWorldSolve = b.invInertiaWorld;
    }
  }
  // gs_solver.dart:74-180
  int solve(std::vector<Eq*>& eqs, double dt) {
    std::vector<int> all(bodies.size());
    for (size_t i = 0; i < all.size(); i++) all[i] = (int)i;
    return gsSolve(eqs, all, dt);
  }
  // SplitSolver.solve (split_solver.dart:53-126): islands of non-static bodies
  // in body order (getUnvisitedNode), each gathered by the node walk of bfs /
  // visitFunc (:134-166), its equations sorted by id, highest first
  // (sortById, :168-170), and solved by the GSSolver over the island's bodies.
  // Returns the most iterations any island took.
  int splitSolve(std::vector<Eq*>& eqs, double dt) {
    const int N = (int)bodies.size();
    std::vector<std::vector<int>> children(N);
    std::vector<std::vector<Eq*>> nodeEqs(N);
    for (Eq* e : eqs) {
      children[e->bi].push_back(e->bj);
      nodeEqs[e->bi].push_back(e);
      children[e->bj].push_back(e->bi);
      nodeEqs[e->bj].push_back(e);
    }
    std::vector<char> visited(N, 0);
    auto unvisited = [&](const std::vector<int>& list) {
      for (int i : list)
        if (!visited[i] && bodies[i].type != CP_BODY_STATIC) return i;
      return -1;
    };
    std::vector<int> all(N);
    for (int i = 0; i < N; i++) all[i] = i;
    int most = 0;
    for (;;) {
      const int root = unvisited(all);
      if (root < 0) break;
      std::vector<int> island;
      std::vector<Eq*> ieqs;
      auto visit = [&](int node) {
        island.push_back(node);
        for (Eq* e : nodeEqs[node])
          if (std::find(ieqs.begin(), ieqs.end(), e) == ieqs.end()) ieqs.push_back(e);
      };
      std::vector<int> queue{root};
      visited[root] = 1;
      visit(root);
      while (!queue.empty()) {
        const int node = queue.back();
        queue.pop_back();
        for (;;) {
          const int child = unvisited(children[node]);
          if (child < 0) break;
          visited[child] = 1;
          visit(child);
          queue.push_back(child);
        }
      }
      std::sort(ieqs.begin(), ieqs.end(), [](const Eq* a, const Eq* b) { return a->id > b->id; });
      most = std::max(most, gsSolve(ieqs, island, dt));
    }
    return most;
  }
  // GSSolver.solve (gs_solver.dart:27-133) over the given bodies
  int gsSolve(std::vector<Eq*>& eqs, const std::vector<int>& bodyList, double dt) {
    int iter = 0;
    const int maxIter = iterations;
    const double tolSquared = tolerance * tolerance;
    const int nEq = (int)eqs.size();
    const int nBodies = (int)bodyList.size();
    const double h = dt;
    if (nEq != 0) for (int bi : bodyList) updateSolveMassProperties(bodies[bi]);
    for (int i = 0; i != nEq; i++) {
      Eq& c = *eqs[i];
      c.lambda = 0.0;
      c.B = computeB(c, h);
      c.invC = 1.0 / computeC(c);
    }
    if (nEq != 0) {
      for (int i = 0; i != nBodies; i++) {
        Body& b = bodies[bodyList[i]];
        setValues(b.vlambda, 0, 0, 0);
        setValues(b.wlambda, 0, 0, 0);
      }
      for (iter = 0; iter != maxIter; iter++) {
        double deltalambdaTot = 0.0;
        for (int j = 0; j != nEq; j++) {
          Eq& c = *eqs[j];
          double B = c.B, invC = c.invC, lambdaj = c.lambda;
          double gwlambda = computeGWlambda(c);
          double deltalambda = invC * (B - gwlambda - c.eps * lambdaj);
          if (lambdaj + deltalambda < c.minForce) deltalambda = c.minForce - lambdaj;
          else if (lambdaj + deltalambda > c.maxForce) deltalambda = c.maxForce - lambdaj;
          c.lambda = c.lambda + deltalambda;
          deltalambdaTot += deltalambda > 0.0 ? deltalambda : -deltalambda;
          addToWlambda(c, deltalambda);
        }
        if (deltalambdaTot * deltalambdaTot < tolSquared) break;
      }
      for (int i = 0; i != nBodies; i++) {
        Body& b = bodies[bodyList[i]];
        multiply2(b.vlambda, b.linearFactor, b.vlambda);
        add2(b.velocity, b.vlambda, b.velocity);
        multiply2(b.wlambda, b.angularFactor, b.wlambda);
        add2(b.angularVelocity, b.wlambda, b.angularVelocity);
      }
      double invDt = 1 / h;
      for (int l = nEq - 1; l > -1; l--) eqs[l]->multiplier = eqs[l]->lambda * invDt;
    }
    return iter;
  }

  // ---------------------------------------------------------------- raycast
  // Ray (lib/collision/ray_class.dart) as World.raycastClosest / Any / All
  // drive it (world_class.dart:248-278): one ray's state and result.
  struct RayRun {
    V3 from, to, direction;
    int mode = CP_RAY_ANY;
    bool skipBackfaces = true, checkResponse = true;
    int group = -1, mask = -1;
    cp_ray_hit result;
    bool shouldStop = false;
    cp_ray_hit* all = nullptr;  // RayMode.all: every hit, in report order
    int cap = 0, count = 0;
  };
  // raycast_result.dart:38-50
  static void rayReset(cp_ray_hit& r) {
    std::memset(&r, 0, sizeof(r));
    r.body = r.shape = r.hit_face_index = -1;
    r.distance = -1;
  }
  // ray_class.dart:669-678
  static bool pointInTriangle(const V3& p, const V3& a, const V3& b, const V3& c) {
    V3 v0, v1, v2;
    sub2(c, a, v0);
    sub2(b, a, v1);
    sub2(p, a, v2);
    double dot00 = dot(v0, v0), dot01 = dot(v0, v1), dot02 = dot(v0, v2), dot11 = dot(v1, v1), dot12 = dot(v1, v2);
    double u = dot11 * dot02 - dot01 * dot12;
    double v = dot00 * dot12 - dot01 * dot02;
    return u >= 0 && v >= 0 && (u + v) < (dot00 * dot11 - dot01 * dot01);
  }
  // ray_class.dart:679-691
  static double distanceFromIntersection(const V3& from, const V3& direction, const V3& position) {
    V3 v0, is;
    sub2(position, from, v0);
    double d = dot(v0, direction);
    scale2(direction, d, is);
    add2(is, from, is);
    return distanceTo(position, is);
  }
  // ray_class.dart:617-664 (_reportIntersection; the face index is stored
  // before the mode decides whether the hit is kept)
  void rayReport(RayRun& R, const V3& normal, const V3& hit, int shape, int body, int faceIndex) {
    const double distance = distanceTo(R.from, hit);
    if (R.skipBackfaces && dot(normal, R.direction) > 0) return;
    R.result.hit_face_index = faceIndex;
    auto set = [&]() {
      R.result.hit_point[0] = hit.x; R.result.hit_point[1] = hit.y; R.result.hit_point[2] = hit.z;
      R.result.hit_normal[0] = normal.x; R.result.hit_normal[1] = normal.y; R.result.hit_normal[2] = normal.z;
      R.result.shape = shape;
      R.result.body = body;
      R.result.distance = distance;
    };
    if (R.mode == CP_RAY_ALL) {
      set();
      R.result.has_hit = 1;
      if (R.count < R.cap) R.all[R.count] = R.result;
      R.count++;
    } else if (R.mode == CP_RAY_CLOSEST) {
      if (distance < R.result.distance || !R.result.has_hit) {
        R.result.has_hit = 1;
        set();
      }
    } else {
      R.result.has_hit = 1;
      set();
      R.shouldStop = true;
    }
  }
  // ray_class.dart:387-438 (the pow(x, 2) terms as x * x)
  void raySphere(RayRun& R, double r, const V3& position, int shape, int body) {
    const V3 &from = R.from, &to = R.to;
    double dx = (double)to.x - from.x, dy = (double)to.y - from.y, dz = (double)to.z - from.z;
    double fx = (double)from.x - position.x, fy = (double)from.y - position.y, fz = (double)from.z - position.z;
    double a = dx * dx + dy * dy + dz * dz;
    double b = 2 * (dx * fx + dy * fy + dz * fz);
    double c = fx * fx + fy * fy + fz * fz - r * r;
    double delta = b * b - 4 * a * c;
    V3 ip, normal;
    if (delta < 0) return;
    if (delta == 0) {
      lerp(from, to, delta, ip);
      sub2(ip, position, normal);
      normalize(normal);
      rayReport(R, normal, ip, shape, body, -1);
      return;
    }
    double d1 = (-b - std::sqrt(delta)) / (2 * a);
    double d2 = (-b + std::sqrt(delta)) / (2 * a);
    if (d1 >= 0 && d1 <= 1) {
      lerp(from, to, d1, ip);
      sub2(ip, position, normal);
      normalize(normal);
      rayReport(R, normal, ip, shape, body, -1);
    }
    if (R.shouldStop) return;
    if (d2 >= 0 && d2 <= 1) {
      lerp(from, to, d2, ip);
      sub2(ip, position, normal);
      normalize(normal);
      rayReport(R, normal, ip, shape, body, -1);
    }
  }
  // ray_class.dart:290-334
  void rayPlane(RayRun& R, const Q4& quat, const V3& position, int shape, int body) {
    const V3 &from = R.from, &to = R.to;
    V3 n = mk(0, 0, 1), len;
    vmult(quat, n, n);
    sub2(from, position, len);
    double planeToFrom = dot(len, n);
    sub2(to, position, len);
    double planeToTo = dot(len, n);
    if (planeToFrom * planeToTo > 0) return;
    if (distanceTo(from, to) < planeToFrom) return;
    double nDotDir = dot(n, R.direction);
    if (std::fabs(nDotDir) < 0.0001) return;
    V3 pp, ds, hit;
    sub2(from, position, pp);
    double t = -dot(n, pp) / nDotDir;
    scale2(R.direction, t, ds);
    add2(from, ds, hit);
    rayReport(R, n, hit, shape, body, -1);
  }
  // ray_class.dart:440-530
  void rayConvex(RayRun& R, const Hull& h, const Q4& q, const V3& x, int shape, int body) {
    const V3 &from = R.from, &to = R.to;
    const double fromToDistance = distanceTo(from, to);
    for (size_t j = 0; !R.shouldStop && j < h.faces.size(); j++) {
      const std::vector<int>& face = h.faces[j];
      V3 vector, normal;
      vmult(q, h.vertices[face[0]], vector);
      add2(vector, x, vector);
      sub2(vector, from, vector);
      vmult(q, h.faceNormals[j], normal);
      double d = dot(R.direction, normal);
      double scalar = dot(normal, vector) / d;
      if (scalar < 0) continue;
      V3 ip, a;
      scale2(R.direction, scalar, ip);
      add2(ip, from, ip);
      vmult(q, h.vertices[face[0]], a);
      add2(x, a, a);
      for (size_t i = 1; !R.shouldStop && i + 1 < face.size(); i++) {
        V3 b, c;
        vmult(q, h.vertices[face[i]], b);
        vmult(q, h.vertices[face[i + 1]], c);
        add2(x, b, b);
        add2(x, c, c);
        double distance = distanceTo(ip, from);
        if (!(pointInTriangle(ip, a, b, c) || pointInTriangle(ip, b, a, c)) || distance > fromToDistance) continue;
        rayReport(R, normal, ip, shape, body, (int)j);
      }
    }
  }
  // ray_class.dart:270-288 (the type table of :104-127 has no entry for
  // Capsule, Cone or SizedPlane)
  void rayShape(RayRun& R, int shapeIndex, const Q4& q, const V3& x, int body) {
    const Shape& s = shapes[shapeIndex];
    if (distanceFromIntersection(R.from, R.direction, x) > s.bsr) return;
    if (s.type == CP_SHAPE_SPHERE) raySphere(R, s.radius, x, shapeIndex, body);
    else if (s.type == CP_SHAPE_PLANE) rayPlane(R, q, x, shapeIndex, body);
    else if (s.type == CP_SHAPE_BOX || s.type == CP_SHAPE_CONVEX || s.type == CP_SHAPE_CYLINDER)
      rayConvex(R, s.hull, q, x, shapeIndex, body);
  }
  // ray_class.dart:201-244
  void rayBody(RayRun& R, int i) {
    const Body& b = bodies[i];
    if (R.checkResponse && !b.response) return;
    if ((R.group & b.mask) == 0 || (b.group & R.mask) == 0) return;
    for (int k = 0; k < b.numShapes(); k++) {
      const int si = b.shapeAt(k);
      if (R.checkResponse && !shapes[si].response) continue;
      Q4 qi;
      V3 xi;
      qmultiply2(b.quaternion, b.orientationAt(k), qi);
      vmult(b.quaternion, b.offsetAt(k), xi);
      add2(xi, b.position, xi);
      rayShape(R, si, qi, xi, i);
      if (R.shouldStop) break;
    }
  }
  // Broadphase.aabbQuery: naive_broadphase.dart:39-56, sap_broadphase.dart:
  // 240-261 (sorting first when the list is dirty, as after every step);
  // GridBroadphase has none (broadphase.dart:151-154: no bodies)
  void aabbQuery(const V3& lo, const V3& hi, std::vector<int>& out) {
    out.clear();
    auto overlapsQuery = [&](const Body& b) {
      bool ox = (lo.x <= b.aabbHi.x && b.aabbHi.x <= hi.x) || (b.aabbLo.x <= hi.x && hi.x <= b.aabbHi.x);
      bool oy = (lo.y <= b.aabbHi.y && b.aabbHi.y <= hi.y) || (b.aabbLo.y <= hi.y && hi.y <= b.aabbHi.y);
      bool oz = (lo.z <= b.aabbHi.z && b.aabbHi.z <= hi.z) || (b.aabbLo.z <= hi.z && hi.z <= b.aabbHi.z);
      return ox && oy && oz;
    };
    if (broadphase == CP_BROAD_NAIVE) {
      for (int i = 0; i < (int)bodies.size(); i++) {
        if (bodies[i].aabbNeedsUpdate) updateAABB(bodies[i], shapes);
        if (overlapsQuery(bodies[i])) out.push_back(i);
      }
    } else if (broadphase == CP_BROAD_SAP) {
      if (dirty) {
        sapSort();
        dirty = false;
      }
      for (int i : axisList) {
        if (bodies[i].aabbNeedsUpdate) updateAABB(bodies[i], shapes);
        if (overlapsQuery(bodies[i])) out.push_back(i);
      }
    }
  }
  // ray_class.dart:163-199
  void raycast(const cp_ray& ray, int mode, cp_ray_hit& result, cp_ray_hit* all, int cap, int& count) {
    RayRun R;
    R.mode = mode;
    R.skipBackfaces = ray.skip_backfaces != 0;
    R.group = ray.collision_filter_group;
    R.mask = ray.collision_filter_mask;
    R.checkResponse = ray.check_collision_response != 0;
    R.from = mk(ray.from[0], ray.from[1], ray.from[2]);
    R.to = mk(ray.to[0], ray.to[1], ray.to[2]);
    R.all = all;
    R.cap = cap;
    rayReset(R.result);
    sub2(R.to, R.from, R.direction);
    normalize(R.direction);
    V3 lo, hi;  // Ray.getAABB (:337-349)
    lo.x = (float)dartMin(R.to.x, R.from.x); lo.y = (float)dartMin(R.to.y, R.from.y); lo.z = (float)dartMin(R.to.z, R.from.z);
    hi.x = (float)dartMax(R.to.x, R.from.x); hi.y = (float)dartMax(R.to.y, R.from.y); hi.z = (float)dartMax(R.to.z, R.from.z);
    std::vector<int> cand;
    aabbQuery(lo, hi, cand);
    for (size_t k = 0; !R.shouldStop && k < cand.size(); k++) rayBody(R, cand[k]);
    result = R.result;
    count = R.count;
  }

  // ---------------------------------------------------------------- constraints
  // point_to_point_constraint.dart:122-137, hinge_constraint.dart:217-242,
  // distance_constraint.dart:269-280
  void updateConstraint(Constraint& c) {
    Body& A = bodies[c.bodyA];
    Body& B = bodies[c.bodyB];
    if (c.type == CP_CON_DISTANCE || c.type == CP_CON_SPRING) {  // spring_constraint.dart:45-57 is the same
      Eq& eq = c.eqs[0];
      double halfDist = c.distance * 0.5;
      sub2(B.position, A.position, eq.ni);
      normalize(eq.ni);
      scale2(eq.ni, halfDist, eq.ri);
      scale2(eq.ni, -halfDist, eq.rj);
      return;
    }
    Eq &x = c.eqs[0], &y = c.eqs[1], &z = c.eqs[2];
    vmult(A.quaternion, c.pivotA, x.ri);
    vmult(B.quaternion, c.pivotB, x.rj);
    y.ri = x.ri; y.rj = x.rj; z.ri = x.ri; z.rj = x.rj;
    if (c.type == CP_CON_HINGE) {
      Eq &r1 = c.eqs[3], &r2 = c.eqs[4], &motor = c.eqs[5];
      V3 wa, wb;
      vmult(A.quaternion, c.axisA, wa);
      vmult(B.quaternion, c.axisB, wb);
      tangents(wa, r1.axisA, r2.axisA);
      r1.axisB = wb; r2.axisB = wb;
      if (motor.enabled) {
        vmult(A.quaternion, c.axisA, motor.axisA);
        vmult(B.quaternion, c.axisB, motor.axisB);
      }
    } else if (c.type == CP_CON_LOCK) {  // lock_constraint.dart:86-103
      Eq &r1 = c.eqs[3], &r2 = c.eqs[4], &r3 = c.eqs[5];
      vmult(A.quaternion, c.xA, r1.axisA);
      vmult(B.quaternion, c.yB, r1.axisB);
      vmult(A.quaternion, c.yA, r2.axisA);
      vmult(B.quaternion, c.zB, r2.axisB);
      vmult(A.quaternion, c.zA, r3.axisA);
      vmult(B.quaternion, c.xB, r3.axisB);
    } else if (c.type == CP_CON_CONE_TWIST) {  // cone_twist_constraint.dart:77-96
      Eq &cone = c.eqs[3], &twist = c.eqs[4];
      vmult(A.quaternion, c.axisA, cone.axisA);
      vmult(B.quaternion, c.axisB, cone.axisB);
      // axisA.tangents(twist.axisA, twist.axisA): both tangents land in one
      // vector, the second (cross2 reads its argument before writing)
      tangents(c.axisA, twist.axisA, twist.axisA);
      vmult(A.quaternion, twist.axisA, twist.axisA);
      tangents(c.axisB, twist.axisB, twist.axisB);
      vmult(B.quaternion, twist.axisB, twist.axisB);
    }
  }

  // ---------------------------------------------------------------- step
  // world_class.dart:433-701 (physics only: collision matrices, overlap
  // keepers and events do not change the state and are left out)
  void internalStep(double dtv) {
    dt = dtv;
    const int N = (int)bodies.size();
    double gx = gravity.x, gy = gravity.y, gz = gravity.z;
    for (int i = 0; i != N; i++) {
      Body& b = bodies[i];
      if (b.type == CP_BODY_DYNAMIC) {
        double m = b.mass;
        b.force.x = (float)(b.force.x + m * gx);
        b.force.y = (float)(b.force.y + m * gy);
        b.force.z = (float)(b.force.z + m * gz);
      }
    }
    p1.clear(); p2.clear();
    if (broadphase == CP_BROAD_NAIVE) naivePairs();
    else if (broadphase == CP_BROAD_SAP) sapPairs();
    else gridPairs();
    for (auto& c : constraints) {
      if (!c.collideConnected) {
        for (int j = (int)p1.size() - 1; j >= 0; j -= 1) {
          if ((c.bodyA == p1[j] && c.bodyB == p2[j]) || (c.bodyB == p1[j] && c.bodyA == p2[j])) {
            p1.erase(p1.begin() + j);
            p2.erase(p2.begin() + j);
          }
        }
      }
    }
    if (events) {  // collisionMatrixTick (world_class.dart:213-221)
      bodyOverlapKeeper.tick();
      shapeOverlapKeeper.tick();
    }
    if (split) {  // last step's equations back into the pools, in order (world_class.dart:506-517)
      for (const Eq& c : contacts) contactPool.push_back(c.id);
      for (const Eq& f : frictionEqs) frictionPool.push_back(f.id);
    }
    getContacts();
    std::vector<Eq*> eqs;
    for (auto& f : frictionEqs) addEquation(eqs, f);
    for (auto& c : contacts) {
      Body& bi = bodies[c.bi];
      Body& bj = bodies[c.bj];
      if (bi.material >= 0 && bj.material >= 0) {
        if (materials[bi.material].restitution >= 0 && materials[bj.material].restitution >= 0)
          c.restitution = materials[bi.material].restitution * materials[bj.material].restitution;
      }
      addEquation(eqs, c);
      if (bi.allowSleep && bi.type == CP_BODY_DYNAMIC && bi.sleepState == CP_SLEEPING && bj.sleepState == CP_AWAKE && bj.type != CP_BODY_STATIC) {
        double s2 = length2(bj.velocity) + length2(bj.angularVelocity);
        double l2 = bj.sleepSpeedLimit * bj.sleepSpeedLimit;
        if (s2 >= l2 * 2) bi.wakeUpAfterNarrowphase = true;
      }
      if (bj.allowSleep && bj.type == CP_BODY_DYNAMIC && bj.sleepState == CP_SLEEPING && bi.sleepState == CP_AWAKE && bi.type != CP_BODY_STATIC) {
        double s2 = length2(bi.velocity) + length2(bi.angularVelocity);
        double l2 = bi.sleepSpeedLimit * bi.sleepSpeedLimit;
        if (s2 >= l2 * 2) bj.wakeUpAfterNarrowphase = true;
      }
      if (events) {
        // the collision matrices alias, so every contact is a "first" one
        // and dispatches collide to both bodies (world_class.dart:593-604)
        eventQueue.push_back(cp_event{CP_EV_COLLIDE, c.bi, c.bj, (int32_t)(&c - &contacts[0]), stepnumber + 1});
        bodyOverlapKeeper.set(bodyId(c.bi), bodyId(c.bj));
        shapeOverlapKeeper.set(shapeId(c.si), shapeId(c.sj));
      }
    }
    if (events) emitContactEvents();
    for (int i = 0; i != N; i++) {
      Body& b = bodies[i];
      if (b.wakeUpAfterNarrowphase) { wakeUp(b); b.wakeUpAfterNarrowphase = false; }
    }
    for (auto& c : constraints) {
      updateConstraint(c);
      for (auto& e : c.eqs) addEquation(eqs, e);
    }
    lastIterations = split ? splitSolve(eqs, dt) : solve(eqs, dt);
    solverRows.clear();
    for (Eq* e : eqs) solverRows.push_back(*e);
    for (int i = 0; i != N; i++) {  // damping
      Body& b = bodies[i];
      if (b.type == CP_BODY_DYNAMIC) {
        double ld = std::pow(1.0 - b.linearDamping, dt);
        scale2(b.velocity, ld, b.velocity);
        double ad = std::pow(1.0 - b.angularDamping, dt);
        scale2(b.angularVelocity, ad, b.angularVelocity);
      }
    }
    bool quatNormalize = stepnumber % (quatNormalizeSkip + 1) == 0;
    for (int i = 0; i != N; i++) integrate(bodies[i], dt, quatNormalize, quatNormalizeFast);
    for (int i = 0; i != N; i++) { setValues(bodies[i].force, 0, 0, 0); setValues(bodies[i].torque, 0, 0, 0); }
    dirty = true;
    stepnumber += 1;
    if (allowSleep) for (int i = 0; i != N; i++) sleepTick(bodies[i], time);
  }
  // world_class.dart:703-770
  void emitContactEvents() {
    std::vector<int> additions, removals;
    bodyOverlapKeeper.getDiff(additions, removals);
    for (size_t i = 0; i < additions.size(); i += 2)
      eventQueue.push_back(cp_event{CP_EV_BEGIN_CONTACT, bodyIndex(additions[i]), bodyIndex(additions[i + 1]), -1, stepnumber + 1});
    for (size_t i = 0; i < removals.size(); i += 2)
      eventQueue.push_back(cp_event{CP_EV_END_CONTACT, bodyIndex(removals[i]), bodyIndex(removals[i + 1]), -1, stepnumber + 1});
    additions.clear();
    removals.clear();
    shapeOverlapKeeper.getDiff(additions, removals);
    for (size_t i = 0; i < additions.size(); i += 2)
      eventQueue.push_back(
          cp_event{CP_EV_BEGIN_SHAPE_CONTACT, shapeIndex(additions[i]), shapeIndex(additions[i + 1]), -1, stepnumber + 1});
    for (size_t i = 0; i < removals.size(); i += 2)
      eventQueue.push_back(
          cp_event{CP_EV_END_SHAPE_CONTACT, shapeIndex(removals[i]), shapeIndex(removals[i + 1]), -1, stepnumber + 1});
  }
  // solver.dart:30-34
  void addEquation(std::vector<Eq*>& eqs, Eq& e) {
    if (e.enabled && !bodies[e.bi].isTrigger && !bodies[e.bj].isTrigger) eqs.push_back(&e);
  }
  static void wakeUp(Body& b) { b.sleepState = CP_AWAKE; b.wakeUpAfterNarrowphase = false; }
  // rigid_body.dart:282-300
  static void sleepTick(Body& b, double time) {
    if (!b.allowSleep) return;
    int st = b.sleepState;
    double speedSquared = length2(b.velocity) + length2(b.angularVelocity);
    double lim2 = b.sleepSpeedLimit * b.sleepSpeedLimit;
    if (st == CP_AWAKE && speedSquared < lim2) { b.sleepState = CP_SLEEPY; b.timeLastSleepy = time; }
    else if (st == CP_SLEEPY && speedSquared > lim2) wakeUp(b);
    else if (st == CP_SLEEPY && time - b.timeLastSleepy > b.sleepTimeLimit) {
      b.sleepState = CP_SLEEPING;
      setValues(b.velocity, 0, 0, 0);
      setValues(b.angularVelocity, 0, 0, 0);
      b.wakeUpAfterNarrowphase = false;
    }
  }
  // rigid_body.dart:627-680
  static void integrate(Body& b, double dt, bool quatNormalize, bool quatNormalizeFast) {
    b.previousPosition = b.position;
    b.previousQuaternion = b.quaternion;
    if (!(b.type == CP_BODY_DYNAMIC || b.type == CP_BODY_KINEMATIC) || b.sleepState == CP_SLEEPING) return;
    double iMdt = b.invMass * dt;
    b.velocity.x = (float)(b.velocity.x + b.force.x * iMdt * b.linearFactor.x);
    b.velocity.y = (float)(b.velocity.y + b.force.y * iMdt * b.linearFactor.y);
    b.velocity.z = (float)(b.velocity.z + b.force.z * iMdt * b.linearFactor.z);
    const float* e = b.invInertiaWorld.e;
    double tx = (double)b.torque.x * b.angularFactor.x;
    double ty = (double)b.torque.y * b.angularFactor.y;
    double tz = (double)b.torque.z * b.angularFactor.z;
    b.angularVelocity.x = (float)(b.angularVelocity.x + dt * (e[0] * tx + e[1] * ty + e[2] * tz));
    b.angularVelocity.y = (float)(b.angularVelocity.y + dt * (e[3] * tx + e[4] * ty + e[5] * tz));
    b.angularVelocity.z = (float)(b.angularVelocity.z + dt * (e[6] * tx + e[7] * ty + e[8] * tz));
    b.position.x = (float)(b.position.x + b.velocity.x * dt);
    b.position.y = (float)(b.position.y + b.velocity.y * dt);
    b.position.z = (float)(b.position.z + b.velocity.z * dt);
    qintegrate(b.quaternion, b.angularVelocity, dt, b.angularFactor, b.quaternion);
    if (quatNormalize) {
      if (quatNormalizeFast) qnormalizeFast(b.quaternion);
      else qnormalize(b.quaternion);
    }
    b.aabbNeedsUpdate = true;
    updateInertiaWorld(b, false);
  }
  void step(double dtv) {  // world_class.dart:392-399 (fixed stepping)
    internalStep(dtv);
    time += dtv;
  }
  double accumulator = 0;  // world_class.dart:119
  int lastSubsteps = 0;
  // world_class.dart:400-430 (interpolated stepping)
  void stepInterpolated(double dtv, double timeSinceLastCalled, int maxSubSteps) {
    accumulator += timeSinceLastCalled;
    const auto t0 = std::chrono::steady_clock::now();
    int substeps = 0;
    while (accumulator >= dtv && substeps < maxSubSteps) {
      internalStep(dtv);
      accumulator -= dtv;
      substeps++;
      const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
      if (ms > dtv * 1000) break;
    }
    // Dart's double % is never negative
    double r = std::fmod(accumulator, dtv);
    if (r < 0) r += dtv;
    if (r == 0) r = 0.0;
    accumulator = r;
    lastSubsteps = substeps;
    const double t = accumulator / dtv;
    for (Body& b : bodies) {
      lerp(b.previousPosition, b.position, t, b.interpolatedPosition);
      slerp(b.previousQuaternion, b.quaternion, t, b.interpolatedQuaternion);
      qnormalize(b.previousQuaternion);
    }
    time += timeSinceLastCalled;
  }
};

static int buildWorld(const cp_world_desc& d, World& w) {
  if (d.num_bodies < 0 || d.num_shapes < 0) return CP_ERR_ARG;
  w.shapes.resize(d.num_shapes);
  for (int i = 0; i < d.num_shapes; i++) {
    int st = buildShape(d.shapes[i], w.shapes[i]);
    if (st) return st;
  }
  w.planeNormalDone.assign(d.num_shapes, 0);
  w.planeWorldNormal.assign(d.num_shapes, V3());
  w.bodies.resize(d.num_bodies);
  w.bodyShapeTable.assign(d.body_shapes, d.body_shapes ? d.body_shapes + d.num_body_shapes : d.body_shapes);
  for (int i = 0; i < d.num_bodies; i++) {
    if (!extrasValid(d.bodies[i], d.num_shapes, d.body_shapes, d.num_body_shapes)) return CP_ERR_ARG;
    bodyFromDesc(d.bodies[i], w.bodies[i], d.body_shapes);
    if (w.bodies[i].shape >= d.num_shapes) return CP_ERR_ARG;
  }
  w.materials.resize(d.num_materials);
  for (int i = 0; i < d.num_materials; i++) { w.materials[i].friction = d.materials[i].friction; w.materials[i].restitution = d.materials[i].restitution; }
  auto cmOf = [](const cp_contact_material& c) {
    ContactMat m;
    m.friction = c.friction; m.restitution = c.restitution;
    m.cs = c.contact_stiffness; m.cr = c.contact_relaxation; m.fs = c.friction_stiffness; m.fr = c.friction_relaxation;
    return m;
  };
  w.defaultCM = cmOf(d.default_contact_material);
  for (int i = 0; i < d.num_contact_materials; i++) {
    const cp_contact_material& c = d.contact_materials[i];
    w.cmTable[std::make_pair(std::min(c.material_a, c.material_b), std::max(c.material_a, c.material_b))] = cmOf(c);
  }
  w.gravity.x = d.gravity[0]; w.gravity.y = d.gravity[1]; w.gravity.z = d.gravity[2];
  w.hasFrictionGravity = d.has_friction_gravity != 0;
  w.frictionGravity.x = d.friction_gravity[0]; w.frictionGravity.y = d.friction_gravity[1]; w.frictionGravity.z = d.friction_gravity[2];
  w.allowSleep = d.allow_sleep != 0;
  w.quatNormalizeSkip = d.quat_normalize_skip;
  w.quatNormalizeFast = d.quat_normalize_fast != 0;
  w.iterations = d.solver_iterations;
  w.tolerance = d.solver_tolerance;
  w.broadphase = d.broadphase;
  w.useBoundingBoxes = d.use_bounding_boxes != 0;
  w.sapAxis = d.sap_axis;
  for (int k = 0; k < 3; k++) w.gridN[k] = d.grid_n[k];
  w.gridMin.x = d.grid_aabb_min[0]; w.gridMin.y = d.grid_aabb_min[1]; w.gridMin.z = d.grid_aabb_min[2];
  w.gridMax.x = d.grid_aabb_max[0]; w.gridMax.y = d.grid_aabb_max[1]; w.gridMax.z = d.grid_aabb_max[2];
  if (w.broadphase == CP_BROAD_GRID && (w.gridN[0] <= 0 || w.gridN[1] <= 0 || w.gridN[2] <= 0)) return CP_ERR_ARG;
  w.enableFrictionReduction = d.enable_friction_reduction != 0;
  w.time = d.time;
  if (d.solver < CP_SOLVER_GS || d.solver > CP_SOLVER_SPLIT) return CP_ERR_ARG;
  w.split = d.solver == CP_SOLVER_SPLIT;
  w.idCounter = d.equation_id_counter;
  w.stepnumber = d.stepnumber;
  w.axisList.resize(d.num_bodies);
  for (int i = 0; i < d.num_bodies; i++) w.axisList[i] = d.sap_axis_list ? d.sap_axis_list[i] : i;
  const double cosHalfPi = std::cos(M_PI / 2);  // RotationalEquation default maxAngle
  for (int i = 0; i < d.num_constraints; i++) {
    const cp_constraint_desc& cd = d.constraints[i];
    if (cd.body_a < 0 || cd.body_a >= d.num_bodies || cd.body_b < 0 || cd.body_b >= d.num_bodies) return CP_ERR_ARG;
    Constraint c;
    c.type = cd.type; c.bodyA = cd.body_a; c.bodyB = cd.body_b;
    c.collideConnected = cd.collide_connected != 0;
    c.pivotA = mk(cd.pivot_a[0], cd.pivot_a[1], cd.pivot_a[2]);
    c.pivotB = mk(cd.pivot_b[0], cd.pivot_b[1], cd.pivot_b[2]);
    long long nextId = cd.first_equation_id;
    auto newEq = [&](int kind, double minF, double maxF) {
      Eq e;
      e.kind = kind; e.bi = cd.body_a; e.bj = cd.body_b;
      e.minForce = minF; e.maxForce = maxF;
      e.setSpookParams(cd.spook_stiffness, cd.spook_relaxation, cd.spook_time_step);
      e.id = w.split ? nextId++ : -1;  // the constructor's equations, in equations-list order
      return e;
    };
    double mf = cd.max_force;
    if (cd.type < CP_CON_POINT_TO_POINT || cd.type > CP_CON_SPRING) return CP_ERR_ARG;
    if (cd.type == CP_CON_DISTANCE || cd.type == CP_CON_SPRING) {
      // DistanceConstraint (distance_constraint.dart); SpringConstraint
      // (spring_constraint.dart:26-42): rest length, one ContactEquation
      // bounded by +-stiffness
      V3 pa = w.bodies[cd.body_a].position, pb = w.bodies[cd.body_b].position;
      c.distance = cd.distance >= 0 ? cd.distance : distanceTo(pa, pb);
      c.eqs.push_back(newEq(CP_ROW_CONTACT, -mf, mf));
    } else {
      for (int k = 0; k < 3; k++) c.eqs.push_back(newEq(CP_ROW_CONTACT, -mf, mf));
      setValues(c.eqs[0].ni, 1, 0, 0); setValues(c.eqs[1].ni, 0, 1, 0); setValues(c.eqs[2].ni, 0, 0, 1);
      if (cd.type == CP_CON_HINGE) {
        c.axisA = mk(cd.axis_a[0], cd.axis_a[1], cd.axis_a[2]); normalize(c.axisA);
        c.axisB = mk(cd.axis_b[0], cd.axis_b[1], cd.axis_b[2]); normalize(c.axisB);
        Eq r1 = newEq(CP_ROW_ROTATIONAL, -mf, mf), r2 = newEq(CP_ROW_ROTATIONAL, -mf, mf);
        r1.axisA = c.axisA; r1.axisB = c.axisB; r1.cosMaxAngle = cosHalfPi;
        r2.axisA = c.axisA; r2.axisB = c.axisB; r2.cosMaxAngle = cosHalfPi;
        Eq motor = newEq(CP_ROW_MOTOR, -mf, mf);
        motor.enabled = cd.motor_enabled != 0;
        motor.targetVelocity = cd.motor_target_velocity;
        if (cd.motor_max_force > 0) { motor.maxForce = cd.motor_max_force; motor.minForce = -cd.motor_max_force; }
        c.eqs.push_back(r1); c.eqs.push_back(r2); c.eqs.push_back(motor);
      } else if (cd.type == CP_CON_LOCK) {  // lock_constraint.dart:26-76
        V3* loc[6] = {&c.xA, &c.xB, &c.yA, &c.yB, &c.zA, &c.zB};
        for (int v = 0; v < 6; v++) *loc[v] = mk(cd.lock_axes[v][0], cd.lock_axes[v][1], cd.lock_axes[v][2]);
        for (int r = 0; r < 3; r++) {
          Eq e = newEq(CP_ROW_ROTATIONAL, -mf, mf);
          e.cosMaxAngle = cosHalfPi;
          c.eqs.push_back(e);
        }
      } else if (cd.type == CP_CON_CONE_TWIST) {  // cone_twist_constraint.dart:26-73
        c.axisA = mk(cd.axis_a[0], cd.axis_a[1], cd.axis_a[2]);
        c.axisB = mk(cd.axis_b[0], cd.axis_b[1], cd.axis_b[2]);
        // ConeEquation / RotationalEquation built with maxForce 0 (bounds
        // [-0, 0]), then minForce = -maxForce
        Eq cone = newEq(CP_ROW_ROTATIONAL, -mf, 0.0);
        cone.cosMaxAngle = std::cos(cd.angle);
        Eq twist = newEq(CP_ROW_ROTATIONAL, -mf, 0.0);
        twist.cosMaxAngle = std::cos(cd.twist_angle);
        c.eqs.push_back(cone); c.eqs.push_back(twist);
      }
    }
    w.constraints.push_back(c);
  }
  return CP_OK;
}

}  // namespace orc

using namespace orc;

struct orc_world { World w; };

extern "C" {

int orc_shape_setup(cp_shape_desc* shape) {
  if (!shape) return CP_ERR_ARG;
  Shape s;
  int st = buildShape(*shape, s);
  if (st) return st;
  shape->bounding_sphere_radius = s.bsr;
  return CP_OK;
}

// rigid_body.dart:27-86 (constructor) then addShape :348-369
int orc_body_setup(const cp_shape_desc* shapes, int32_t num_shapes, const cp_body_shape* body_shapes, int32_t num_body_shapes,
                   cp_body_desc* bodies, int32_t num_bodies) {
  if ((!bodies && num_bodies > 0) || num_bodies < 0 || num_shapes < 0 || num_body_shapes < 0) return CP_ERR_ARG;
  std::vector<Shape> sh(num_shapes);
  for (int i = 0; i < num_shapes; i++) { int st = buildShape(shapes[i], sh[i]); if (st) return st; }
  for (int k = 0; k < num_bodies; k++) {
    cp_body_desc* d = &bodies[k];
    if (d->shape >= num_shapes || !extrasValid(*d, num_shapes, body_shapes, num_body_shapes)) return CP_ERR_ARG;
    Body b;
    bodyFromDesc(*d, b, body_shapes);
    b.previousPosition = b.position;
    b.previousQuaternion = b.quaternion;
    b.interpolatedPosition = b.position;
    b.interpolatedQuaternion = b.quaternion;
    b.invMass = b.mass > 0 ? 1.0 / b.mass : 0;
    if (d->type < 0) b.type = b.mass <= 0.0 ? CP_BODY_STATIC : CP_BODY_DYNAMIC;
    int shapeIdx = b.shape;
    std::vector<Body::Extra> extra;
    extra.swap(b.extra);
    b.shape = -1;
    setValues(b.aabbLo, 0, 0, 0); setValues(b.aabbHi, 0, 0, 0);
    updateMassProperties(b, sh);  // constructor, before the shape is added
    b.boundingRadius = 0;
    if (shapeIdx >= 0) {
      // addShape for the first shape, then for each further one: the last
      // updateMassProperties / updateBoundingRadius see them all
      b.shape = shapeIdx;
      b.extra.swap(extra);
      updateMassProperties(b, sh);
      double radius = 0;  // updateBoundingRadius (rigid_body.dart:395-412)
      for (int i = 0; i != b.numShapes(); i++) {
        double offset = length(b.offsetAt(i));
        double r = sh[b.shapeAt(i)].bsr;
        if (offset + r > radius) radius = offset + r;
      }
      b.boundingRadius = radius;
    }
    b.aabbNeedsUpdate = true;
    bodyToDesc(b, *d);
  }
  return CP_OK;
}

orc_world* orc_world_create(const cp_world_desc* desc) {
  if (!desc) return nullptr;
  orc_world* o = new orc_world();
  if (buildWorld(*desc, o->w) != CP_OK) { delete o; return nullptr; }
  return o;
}

void orc_world_destroy(orc_world* w) { delete w; }

int orc_world_step(orc_world* o, double dt, int32_t nsteps) {
  if (!o || nsteps < 0) return CP_ERR_ARG;
  for (int s = 0; s < nsteps; s++) o->w.step(dt);
  return CP_OK;
}

int orc_world_internal_step(orc_world* o, double dt, int32_t nsteps) {
  if (!o || nsteps < 0) return CP_ERR_ARG;
  for (int s = 0; s < nsteps; s++) o->w.internalStep(dt);
  return CP_OK;
}

int orc_world_step_interpolated(orc_world* o, double dt, double since, int32_t max_sub_steps, int32_t* substeps) {
  if (!o || !(dt > 0) || max_sub_steps < 0) return CP_ERR_ARG;
  o->w.stepInterpolated(dt, since, max_sub_steps);
  if (substeps) *substeps = o->w.lastSubsteps;
  return CP_OK;
}

int orc_world_set_events(orc_world* o, int32_t on, const int32_t* body_ids, const int32_t* shape_ids) {
  if (!o) return CP_ERR_ARG;
  World& w = o->w;
  w.events = on != 0;
  w.bodyIds.assign(on && body_ids ? body_ids : nullptr, on && body_ids ? body_ids + w.bodies.size() : nullptr);
  w.shapeIds.assign(on && shape_ids ? shape_ids : nullptr, on && shape_ids ? shape_ids + w.shapes.size() : nullptr);
  w.bodyOverlapKeeper = OverlapKeeper();
  w.shapeOverlapKeeper = OverlapKeeper();
  w.eventQueue.clear();
  return CP_OK;
}

int orc_world_get_events(orc_world* o, cp_event* out, int32_t cap, int32_t* count) {
  if (!o || !count) return CP_ERR_ARG;
  World& w = o->w;
  *count = (int32_t)w.eventQueue.size();
  if ((int)w.eventQueue.size() > cap || (!out && !w.eventQueue.empty())) return CP_ERR_CAPACITY;
  std::copy(w.eventQueue.begin(), w.eventQueue.end(), out);
  w.eventQueue.clear();
  return CP_OK;
}

int orc_world_set_bodies(orc_world* o, const cp_body_desc* in, int32_t n) {
  if (!o || (!in && n > 0) || n != (int32_t)o->w.bodies.size()) return CP_ERR_ARG;
  for (int i = 0; i < n; i++) {
    const World& w = o->w;
    if (in[i].shape >= (int32_t)w.shapes.size() ||
        !extrasValid(in[i], (int)w.shapes.size(), w.bodyShapeTable.data(), (int)w.bodyShapeTable.size()))
      return CP_ERR_ARG;
    bodyFromDesc(in[i], o->w.bodies[i], w.bodyShapeTable.data());
  }
  return CP_OK;
}

int orc_world_set_sap_order(orc_world* o, const int32_t* in, int32_t n) {
  if (!o || (!in && n > 0) || n != (int32_t)o->w.axisList.size()) return CP_ERR_ARG;
  for (int i = 0; i < n; i++) o->w.axisList[i] = in[i];
  return CP_OK;
}

int orc_world_set_time(orc_world* o, double time, int64_t stepnumber, double accumulator) {
  if (!o || stepnumber < 0) return CP_ERR_ARG;
  o->w.time = time;
  o->w.stepnumber = stepnumber;
  o->w.accumulator = accumulator;
  return CP_OK;
}

int orc_world_get_bodies(orc_world* o, cp_body_desc* out, int32_t n) {
  if (!o || (!out && n > 0) || n != (int32_t)o->w.bodies.size()) return CP_ERR_ARG;
  for (int i = 0; i < n; i++) bodyToDesc(o->w.bodies[i], out[i]);
  return CP_OK;
}

int orc_world_get_pairs(orc_world* o, int32_t* p1, int32_t* p2, int32_t cap, int32_t* count) {
  if (!o || !count) return CP_ERR_ARG;
  int n = (int)o->w.p1.size();
  *count = n;
  if (n > cap) return CP_ERR_CAPACITY;
  for (int i = 0; i < n; i++) { p1[i] = o->w.p1[i]; p2[i] = o->w.p2[i]; }
  return CP_OK;
}

int orc_world_get_contacts(orc_world* o, cp_contact* out, int32_t cap, int32_t* count) {
  if (!o || !count) return CP_ERR_ARG;
  int n = (int)o->w.contacts.size();
  *count = n;
  if (n > cap) return CP_ERR_CAPACITY;
  for (int i = 0; i < n; i++) {
    const Eq& c = o->w.contacts[i];
    cp_contact& r = out[i];
    r.bi = c.bi; r.bj = c.bj; r.si = c.si; r.sj = c.sj;
    r.ni[0] = c.ni.x; r.ni[1] = c.ni.y; r.ni[2] = c.ni.z;
    r.ri[0] = c.ri.x; r.ri[1] = c.ri.y; r.ri[2] = c.ri.z;
    r.rj[0] = c.rj.x; r.rj[1] = c.rj.y; r.rj[2] = c.rj.z;
    r.enabled = c.enabled; r.pair = c.pair; r.restitution = c.restitution;
  }
  return CP_OK;
}

int orc_world_get_rows(orc_world* o, cp_row* out, int32_t cap, int32_t* count) {
  if (!o || !count) return CP_ERR_ARG;
  int n = (int)o->w.solverRows.size();
  *count = n;
  if (n > cap) return CP_ERR_CAPACITY;
  for (int i = 0; i < n; i++) {
    const Eq& e = o->w.solverRows[i];
    cp_row& r = out[i];
    r.kind = e.kind; r.bi = e.bi; r.bj = e.bj; r.pad = 0;
    r.B = e.B; r.inv_c = e.invC; r.lambda = e.lambda; r.multiplier = e.multiplier;
    r.min_force = e.minForce; r.max_force = e.maxForce; r.eps = e.eps;
    r.id = e.id;
  }
  return CP_OK;
}

int orc_world_get_info(orc_world* o, cp_step_info* out) {
  if (!o || !out) return CP_ERR_ARG;
  std::memset(out, 0, sizeof(*out));
  out->stepnumber = o->w.stepnumber;
  out->time = o->w.time;
  out->substeps = o->w.lastSubsteps;
  out->accumulator = o->w.accumulator;
  out->num_pairs = (int)o->w.p1.size();
  out->num_contacts = (int)o->w.contacts.size();
  out->num_rows = (int)o->w.solverRows.size();
  out->iterations = o->w.lastIterations;
  out->num_bodies = (int)o->w.bodies.size();
  return CP_OK;
}

int orc_world_raycast(orc_world* o, const cp_ray* rays, int32_t n, int32_t mode, cp_ray_hit* hits, int32_t max_hits,
                      int32_t* counts) {
  if (!o || n < 0 || (n > 0 && (!rays || !hits)) || mode < CP_RAY_CLOSEST || mode > CP_RAY_ALL) return CP_ERR_ARG;
  if (mode == CP_RAY_ALL && (max_hits < 0 || (n > 0 && !counts))) return CP_ERR_ARG;
  for (int r = 0; r < n; r++) {
    cp_ray_hit res;
    int count = 0;
    if (mode == CP_RAY_ALL) {
      o->w.raycast(rays[r], mode, res, hits + (size_t)r * max_hits, max_hits, count);
      counts[r] = count;
    } else {
      o->w.raycast(rays[r], mode, res, nullptr, 0, count);
      hits[r] = res;
    }
  }
  return CP_OK;
}

int orc_world_get_sap_order(orc_world* o, int32_t* out, int32_t n) {
  if (!o || (!out && n > 0) || n != (int32_t)o->w.axisList.size()) return CP_ERR_ARG;
  for (int i = 0; i < n; i++) out[i] = o->w.axisList[i];
  return CP_OK;
}

int orc_worlds_step_parallel(orc_world** worlds, int32_t n, double dt, int32_t nsteps, int32_t threads) {
  if (!worlds || n < 0 || threads < 1) return CP_ERR_ARG;
  std::atomic<int> next(0);
  auto work = [&]() {
    for (;;) {
      int i = next.fetch_add(1);
      if (i >= n) break;
      for (int s = 0; s < nsteps; s++) worlds[i]->w.step(dt);
    }
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < threads; t++) pool.emplace_back(work);
  work();
  for (auto& t : pool) t.join();
  return CP_OK;
}

int orc_shape_hull(const cp_shape_desc* shape, float* verts, int32_t vcap, int32_t* nv, float* normals, int32_t ncap, int32_t* nf, float* edges, int32_t ecap, int32_t* ne) {
  if (!shape || !nv || !nf || !ne) return CP_ERR_ARG;
  Shape s;
  int st = buildShape(*shape, s);
  if (st) return st;
  *nv = (int)s.hull.vertices.size(); *nf = (int)s.hull.faceNormals.size(); *ne = (int)s.hull.uniqueEdges.size();
  if (*nv > vcap || *nf > ncap || *ne > ecap) return CP_ERR_CAPACITY;
  for (int i = 0; i < *nv; i++) { verts[3 * i] = s.hull.vertices[i].x; verts[3 * i + 1] = s.hull.vertices[i].y; verts[3 * i + 2] = s.hull.vertices[i].z; }
  for (int i = 0; i < *nf; i++) { normals[3 * i] = s.hull.faceNormals[i].x; normals[3 * i + 1] = s.hull.faceNormals[i].y; normals[3 * i + 2] = s.hull.faceNormals[i].z; }
  for (int i = 0; i < *ne; i++) { edges[3 * i] = s.hull.uniqueEdges[i].x; edges[3 * i + 1] = s.hull.uniqueEdges[i].y; edges[3 * i + 2] = s.hull.uniqueEdges[i].z; }
  return CP_OK;
}

}  // extern "C"
