// cp_math.cuh -- device arithmetic with the reference's rounding points.
//
// The reference computes in Dart doubles (binary64) and stores Vector3,
// Quaternion and Matrix3 components in Float32List (package:vector_math), so
// every value below is computed in double and rounded to float exactly where
// the reference stores it.  Compile with -fmad=false: Dart never fuses a
// multiply and an add.
//
// A single +, -, * on two binary32 operands whose binary64 result is then
// stored to binary32 equals the binary32 operation itself (53 >= 2*24+2, so
// the double rounding is innocuous); those operations (Vec3.add2, sub2,
// multiply2, Vector3.negate) run on the FP32 pipe here, which matters on a
// part whose FP64 rate is a small fraction of its FP32 rate.
#pragma once
#include <cstdint>

#define DI __device__ __forceinline__

struct f3 { float x, y, z; };
struct q4 { float x, y, z, w; };
struct d3 { double x, y, z; };  // a Vector3 held as binary64 (each value exactly a binary32)

// (double)(float)x without the F2F conversions: for results in binary32's
// normal range the 29 low mantissa bits are rounded off on the integer pipe
// (round to nearest, ties to even; a carry into the exponent is the correct
// next binade).  Zeros, subnormals, values that could overflow, infinities
// and NaNs take the conversion path.  GB300 issues F2F.F32.F64 at its
// binary64 rate, about 1/60 of the integer rate.
DI double r32(double x) {
  unsigned long long u = (unsigned long long)__double_as_longlong(x);
  unsigned e = (unsigned)(u >> 52) & 0x7ffu;
  if (e - 897u < 253u) {  // 2^-126 <= |x| < 2^127
    u += 0x0FFFFFFFull + ((u >> 29) & 1ull);
    u &= ~0x1FFFFFFFull;
    return __longlong_as_double((long long)u);
  }
  if ((u << 1) == 0) return x;  // +-0
  return (double)__double2float_rn(x);
}
DI d3 d3of(f3 v) { return d3{(double)v.x, (double)v.y, (double)v.z}; }
DI d3 ldd3(const double* p) { return d3{p[0], p[1], p[2]}; }
DI void std3(double* p, d3 v) { p[0] = v.x; p[1] = v.y; p[2] = v.z; }
DI double ddot(d3 a, d3 b) {
  double s = a.x * b.x;
  s = s + a.y * b.y;
  s = s + a.z * b.z;
  return s;
}
// addScaledVector with the binary32 store: a + s * v, rounded
DI d3 dadd_scaled(d3 a, double s, d3 v) { return d3{r32(a.x + s * v.x), r32(a.y + s * v.y), r32(a.z + s * v.z)}; }

DI f3 mkf3(double x, double y, double z) { return f3{(float)x, (float)y, (float)z}; }
DI f3 ld3(const float* p) { return f3{p[0], p[1], p[2]}; }
DI void st3(float* p, f3 v) { p[0] = v.x; p[1] = v.y; p[2] = v.z; }
DI q4 ld4q(const float* p) { return q4{p[0], p[1], p[2], p[3]}; }
DI void st4q(float* p, q4 q) { p[0] = q.x; p[1] = q.y; p[2] = q.z; p[3] = q.w; }

// ---- Vector3 (vector_math) ----
DI double dot(f3 a, f3 b) {
  double s = (double)a.x * (double)b.x;
  s = s + (double)a.y * (double)b.y;
  s = s + (double)a.z * (double)b.z;
  return s;
}
DI double length2(f3 a) { return dot(a, a); }
DI double length(f3 a) { return sqrt(length2(a)); }
DI f3 normalized(f3 v) {  // Vector3.normalize()
  double l = length(v);
  if (l == 0.0) return v;
  double d = 1.0 / l;
  return f3{(float)(v.x * d), (float)(v.y * d), (float)(v.z * d)};
}
DI f3 neg(f3 v) { return f3{-v.x, -v.y, -v.z}; }
DI bool is_zero(f3 v) { return v.x == 0.f && v.y == 0.f && v.z == 0.f; }

// ---- lib/math/vec3.dart ----
// add2: target = vector + this (one binary32 add per component, see header)
DI f3 add(f3 a, f3 b) { return f3{__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z)}; }
DI f3 sub(f3 a, f3 b) { return f3{__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z)}; }
DI f3 mul(f3 a, f3 b) { return f3{__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y), __fmul_rn(a.z, b.z)}; }
DI f3 scale(f3 a, double s) {  // scale2(s): target = s * this
  return f3{(float)(s * (double)a.x), (float)(s * (double)a.y), (float)(s * (double)a.z)};
}
DI f3 cross(f3 a, f3 v) {  // cross2 (target distinct from this)
  double vx = v.x, vy = v.y, vz = v.z;
  return f3{(float)((double)a.y * vz - (double)a.z * vy), (float)((double)a.z * vx - (double)a.x * vz),
            (float)((double)a.x * vy - (double)a.y * vx)};
}
DI f3 add_scaled(f3 a, double s, f3 v) {  // addScaledVector
  return f3{(float)((double)a.x + s * (double)v.x), (float)((double)a.y + s * (double)v.y),
            (float)((double)a.z + s * (double)v.z)};
}
DI f3 lerp(f3 a, f3 v, double t) {
  return f3{(float)((double)a.x + ((double)v.x - (double)a.x) * t), (float)((double)a.y + ((double)v.y - (double)a.y) * t),
            (float)((double)a.z + ((double)v.z - (double)a.z) * t)};
}
DI double distance_to(f3 a, f3 p) {
  double px = p.x, py = p.y, pz = p.z;
  return sqrt((px - a.x) * (px - a.x) + (py - a.y) * (py - a.y) + (pz - a.z) * (pz - a.z));
}
DI void tangents(f3 a, f3& t1, f3& t2) {
  double norm = length(a);
  if (norm > 0.0) {
    double inorm = 1 / norm;
    f3 n = mkf3(a.x * inorm, a.y * inorm, a.z * inorm);
    f3 rv = fabs((double)n.x) < 0.9 ? f3{1.f, 0.f, 0.f} : f3{0.f, 1.f, 0.f};
    t1 = cross(n, rv);
    t2 = cross(n, t1);
  } else {
    t1 = f3{1.f, 0.f, 0.f};
    t2 = f3{0.f, 1.f, 0.f};
  }
}
DI f3 unit(f3 a) {
  double ninv = sqrt((double)a.x * a.x + (double)a.y * a.y + (double)a.z * a.z);
  if (ninv > 0.0) {
    ninv = 1.0 / ninv;
    return f3{(float)(a.x * ninv), (float)(a.y * ninv), (float)(a.z * ninv)};
  }
  return f3{1.f, 0.f, 0.f};
}
DI bool almost_zero(f3 a) {
  return !(fabs((double)a.x) > 1e-6 || fabs((double)a.y) > 1e-6 || fabs((double)a.z) > 1e-6);
}

// ---- lib/math/quaternion.dart ----
DI f3 vmult(q4 q, f3 v) {
  double x = v.x, y = v.y, z = v.z;
  double qx = q.x, qy = q.y, qz = q.z, qw = q.w;
  double ix = qw * x + qy * z - qz * y;
  double iy = qw * y + qz * x - qx * z;
  double iz = qw * z + qx * y - qy * x;
  double iw = -qx * x - qy * y - qz * z;
  return f3{(float)(ix * qw + iw * -qx + iy * -qz - iz * -qy), (float)(iy * qw + iw * -qy + iz * -qx - ix * -qz),
            (float)(iz * qw + iw * -qz + ix * -qy - iy * -qx)};
}
DI q4 qmul(q4 a, q4 b) {  // multiply2
  double ax = a.x, ay = a.y, az = a.z, aw = a.w;
  double bx = b.x, by = b.y, bz = b.z, bw = b.w;
  return q4{(float)(ax * bw + aw * bx + ay * bz - az * by), (float)(ay * bw + aw * by + az * bx - ax * bz),
            (float)(az * bw + aw * bz + ax * by - ay * bx), (float)(aw * bw - ax * bx - ay * by - az * bz)};
}
DI q4 qconj(q4 q) { return q4{-q.x, -q.y, -q.z, q.w}; }
DI q4 qnegw(q4 q) { return q4{q.x, q.y, q.z, -q.w}; }  // Transform.vectorToLocalFrame's w *= -1
DI q4 qintegrate(q4 q, f3 av, double dt, f3 af) {
  double ax = (double)av.x * af.x, ay = (double)av.y * af.y, az = (double)av.z * af.z;
  double bx = q.x, by = q.y, bz = q.z, bw = q.w;
  double h = dt * 0.5;
  return q4{(float)(q.x + h * (ax * bw + ay * bz - az * by)), (float)(q.y + h * (ay * bw + az * bx - ax * bz)),
            (float)(q.z + h * (az * bw + ax * by - ay * bx)), (float)(q.w + h * (-ax * bx - ay * by - az * bz))};
}
DI q4 qnormalize(q4 q) {  // vector_math Quaternion.normalize
  double x = q.x, y = q.y, z = q.z, w = q.w;
  double l = sqrt((x * x) + (y * y) + (z * z) + (w * w));
  if (l == 0.0) return q;
  double d = 1.0 / l;
  return q4{(float)(q.x * d), (float)(q.y * d), (float)(q.z * d), (float)(q.w * d)};
}
DI q4 qnormalize_fast(q4 q) {
  double f = (3.0 - ((double)q.x * q.x + (double)q.y * q.y + (double)q.z * q.z + (double)q.w * q.w)) / 2.0;
  if (f == 0) return q4{0.f, 0.f, 0.f, 0.f};
  return q4{(float)(q.x * f), (float)(q.y * f), (float)(q.z * f), (float)(q.w * f)};
}

// ---- lib/math/mat3.dart (storage e[3*row+col]) ----
DI f3 mvmult(const float* e, f3 v) {
  double x = v.x, y = v.y, z = v.z;
  return f3{(float)(e[0] * x + e[1] * y + e[2] * z), (float)(e[3] * x + e[4] * y + e[5] * z),
            (float)(e[6] * x + e[7] * y + e[8] * z)};
}
// rigid_body.dart:459-464: m1 = R(q); m2 = m1^T; m1 = vscale(I, m1); out = m1 * m2
DI void inertia_world(q4 q, f3 I, float* out) {
  double x = q.x, y = q.y, z = q.z, w = q.w;
  double x2 = x + x, y2 = y + y, z2 = z + z;
  double xx = x * x2, xy = x * y2, xz = x * z2, yy = y * y2, yz = y * z2, zz = z * z2;
  double wx = w * x2, wy = w * y2, wz = w * z2;
  float m[9];
  m[0] = (float)(1 - (yy + zz)); m[1] = (float)(xy - wz); m[2] = (float)(xz + wy);
  m[3] = (float)(xy + wz); m[4] = (float)(1 - (xx + zz)); m[5] = (float)(yz - wx);
  m[6] = (float)(xz - wy); m[7] = (float)(yz + wx); m[8] = (float)(1 - (xx + yy));
  float t[9] = {m[0], m[3], m[6], m[1], m[4], m[7], m[2], m[5], m[8]};  // transpose
  float a[9];
#pragma unroll
  for (int i = 0; i < 3; i++) {
    a[3 * i + 0] = (float)((double)I.x * m[3 * i + 0]);
    a[3 * i + 1] = (float)((double)I.y * m[3 * i + 1]);
    a[3 * i + 2] = (float)((double)I.z * m[3 * i + 2]);
  }
#pragma unroll
  for (int r = 0; r < 3; r++) {
    double a1 = a[3 * r], a2 = a[3 * r + 1], a3 = a[3 * r + 2];
#pragma unroll
    for (int c = 0; c < 3; c++) out[3 * r + c] = (float)(a1 * t[c] + a2 * t[3 + c] + a3 * t[6 + c]);
  }
}

// ---- lib/math/transform.dart ----
DI f3 point_to_local(f3 pos, q4 q, f3 wp) { return vmult(qconj(q), sub(wp, pos)); }
DI f3 vector_to_local(q4 q, f3 wv) { return vmult(qnegw(q), wv); }
