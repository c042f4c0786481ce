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
// binary64 -> nearest binary32 (ties to even) on the integer pipe, for the
// same range as r32; other values convert the ordinary way
DI float r32f(double x) {
  unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const unsigned e = (unsigned)(u >> 52) & 0x7ffu;
  if (e - 897u < 253u) {
    u += 0x0FFFFFFFull + ((u >> 29) & 1ull);
    const unsigned e2 = (unsigned)(u >> 52) & 0x7ffu;  // a carry moves to the next binade
    return __uint_as_float((unsigned)(u >> 32) & 0x80000000u | ((e2 - 896u) << 23) | ((unsigned)(u >> 29) & 0x7fffffu));
  }
  return (float)x;
}
// binary32 -> binary64 (exact) and binary64 -> nearest binary32.  Plain
// conversions: on GB300 they issue on the binary64 pipe, which these kernels
// do not saturate, and every integer-pipe replacement measured slower.
DI double F(float f) { return (double)f; }
DI float rf(double x) { return (float)x; }
// The product of two binary32 values is exact in binary64 (24 + 24 bits), so
// p*q + s rounded once (a fused multiply-add) equals the reference's
// separately rounded multiply and add.  fma_ff is used only where both
// factors are binary32 values.
DI double fma_ff(double p, double q, double s) { return __fma_rn(p, q, s); }

DI d3 d3of(f3 v) { return d3{F(v.x), F(v.y), F(v.z)}; }
DI d3 ldd3(const double* p) { return d3{p[0], p[1], p[2]}; }
DI void std3(double* p, d3 v) { p[0] = v.x; p[1] = v.y; p[2] = v.z; }
// ((x*x' + y*y') + z*z') of vectors of binary32 values (every d3 in these
// kernels holds binary32 values), fused: see fma_ff
DI double ddot(d3 a, d3 b) { return fma_ff(a.z, b.z, fma_ff(a.y, b.y, a.x * b.x)); }
// addScaledVector with the binary32 store: a + s * v, rounded
DI d3 dadd_scaled(d3 a, double s, d3 v) { return d3{r32(a.x + s * v.x), r32(a.y + s * v.y), r32(a.z + s * v.z)}; }

DI f3 mkf3(double x, double y, double z) { return f3{rf(x), rf(y), rf(z)}; }
DI f3 ld3(const float* p) { return f3{p[0], p[1], p[2]}; }
DI void st3(float* p, f3 v) { p[0] = v.x; p[1] = v.y; p[2] = v.z; }
DI q4 ld4q(const float* p) { return q4{p[0], p[1], p[2], p[3]}; }
DI void st4q(float* p, q4 q) { p[0] = q.x; p[1] = q.y; p[2] = q.z; p[3] = q.w; }

// ---- Vector3 (vector_math) ----
DI double dot(f3 a, f3 b) {  // ((x*x' + y*y') + z*z')
  return fma_ff(F(a.z), F(b.z), fma_ff(F(a.y), F(b.y), F(a.x) * F(b.x)));
}
DI double length2(f3 a) { return dot(a, a); }
DI double length(f3 a) { return sqrt(length2(a)); }
DI f3 normalized(f3 v) {  // Vector3.normalize()
  double l = length(v);
  if (l == 0.0) return v;
  double d = 1.0 / l;
  return f3{rf(F(v.x) * d), rf(F(v.y) * d), rf(F(v.z) * d)};
}
DI f3 neg(f3 v) { return f3{-v.x, -v.y, -v.z}; }
DI bool is_zero(f3 v) { return v.x == 0.f && v.y == 0.f && v.z == 0.f; }

// ---- lib/math/vec3.dart ----
// add2: target = vector + this (one binary32 add per component, see header)
DI f3 add(f3 a, f3 b) { return f3{__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z)}; }
DI f3 sub(f3 a, f3 b) { return f3{__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z)}; }
DI f3 mul(f3 a, f3 b) { return f3{__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y), __fmul_rn(a.z, b.z)}; }
DI f3 scale(f3 a, double s) {  // scale2(s): target = s * this
  return f3{rf(s * F(a.x)), rf(s * F(a.y)), rf(s * F(a.z))};
}
DI f3 cross(f3 a, f3 v) {  // cross2 (target distinct from this): y*z' - z*y' ...
  const double ax = F(a.x), ay = F(a.y), az = F(a.z), vx = F(v.x), vy = F(v.y), vz = F(v.z);
  return f3{rf(fma_ff(ay, vz, -(az * vy))), rf(fma_ff(az, vx, -(ax * vz))), rf(fma_ff(ax, vy, -(ay * vx)))};
}
DI f3 add_scaled(f3 a, double s, f3 v) {  // addScaledVector
  return f3{rf(F(a.x) + s * F(v.x)), rf(F(a.y) + s * F(v.y)), rf(F(a.z) + s * F(v.z))};
}
DI f3 lerp(f3 a, f3 v, double t) {
  const double ax = F(a.x), ay = F(a.y), az = F(a.z);
  return f3{rf(ax + (F(v.x) - ax) * t), rf(ay + (F(v.y) - ay) * t), rf(az + (F(v.z) - az) * t)};
}
DI double distance_to(f3 a, f3 p) {
  const double dx = F(p.x) - F(a.x), dy = F(p.y) - F(a.y), dz = F(p.z) - F(a.z);
  return sqrt(dx * dx + dy * dy + dz * dz);
}
DI void tangents(f3 a, f3& t1, f3& t2) {
  double norm = length(a);
  if (norm > 0.0) {
    double inorm = 1 / norm;
    f3 n = mkf3(a.x * inorm, a.y * inorm, a.z * inorm);
    f3 rv = fabs(F(n.x)) < 0.9 ? f3{1.f, 0.f, 0.f} : f3{0.f, 1.f, 0.f};
    t1 = cross(n, rv);
    t2 = cross(n, t1);
  } else {
    t1 = f3{1.f, 0.f, 0.f};
    t2 = f3{0.f, 1.f, 0.f};
  }
}
DI f3 unit(f3 a) {
  double ninv = sqrt(dot(a, a));
  if (ninv > 0.0) {
    ninv = 1.0 / ninv;
    return f3{rf(F(a.x) * ninv), rf(F(a.y) * ninv), rf(F(a.z) * ninv)};
  }
  return f3{1.f, 0.f, 0.f};
}
DI bool almost_zero(f3 a) {
  return !(fabs(F(a.x)) > 1e-6 || fabs(F(a.y)) > 1e-6 || fabs(F(a.z)) > 1e-6);
}

// ---- lib/math/quaternion.dart ----
DI f3 vmult(q4 q, f3 v) {
  const double x = F(v.x), y = F(v.y), z = F(v.z);
  const double qx = F(q.x), qy = F(q.y), qz = F(q.z), qw = F(q.w);
  // (qw*x + qy*z) - qz*y etc.: products of binary32 values, see fma_ff
  const double ix = fma_ff(-qz, y, fma_ff(qy, z, qw * x));
  const double iy = fma_ff(-qx, z, fma_ff(qz, x, qw * y));
  const double iz = fma_ff(-qy, x, fma_ff(qx, y, qw * z));
  const double iw = fma_ff(-qz, z, fma_ff(-qy, y, -qx * x));
  return f3{rf(ix * qw + iw * -qx + iy * -qz - iz * -qy), rf(iy * qw + iw * -qy + iz * -qx - ix * -qz),
            rf(iz * qw + iw * -qz + ix * -qy - iy * -qx)};
}
DI q4 qmul(q4 a, q4 b) {  // multiply2: ((ax*bw + aw*bx) + ay*bz) - az*by etc.
  const double ax = F(a.x), ay = F(a.y), az = F(a.z), aw = F(a.w);
  const double bx = F(b.x), by = F(b.y), bz = F(b.z), bw = F(b.w);
  return q4{rf(fma_ff(-az, by, fma_ff(ay, bz, fma_ff(aw, bx, ax * bw)))), rf(fma_ff(-ax, bz, fma_ff(az, bx, fma_ff(aw, by, ay * bw)))),
            rf(fma_ff(-ay, bx, fma_ff(ax, by, fma_ff(aw, bz, az * bw)))), rf(fma_ff(-az, bz, fma_ff(-ay, by, fma_ff(-ax, bx, aw * bw))))};
}
DI q4 qconj(q4 q) { return q4{-q.x, -q.y, -q.z, q.w}; }
DI q4 qnegw(q4 q) { return q4{q.x, q.y, q.z, -q.w}; }  // Transform.vectorToLocalFrame's w *= -1
DI q4 qintegrate(q4 q, f3 av, double dt, f3 af) {
  const double ax = F(av.x) * F(af.x), ay = F(av.y) * F(af.y), az = F(av.z) * F(af.z);
  const double bx = F(q.x), by = F(q.y), bz = F(q.z), bw = F(q.w);
  const double h = dt * 0.5;
  return q4{rf(bx + h * (ax * bw + ay * bz - az * by)), rf(by + h * (ay * bw + az * bx - ax * bz)),
            rf(bz + h * (az * bw + ax * by - ay * bx)), rf(bw + h * (-ax * bx - ay * by - az * bz))};
}
DI q4 qnormalize(q4 q) {  // vector_math Quaternion.normalize: ((x*x + y*y) + z*z) + w*w
  const double x = F(q.x), y = F(q.y), z = F(q.z), w = F(q.w);
  const double l = sqrt(fma_ff(w, w, fma_ff(z, z, fma_ff(y, y, x * x))));
  if (l == 0.0) return q;
  const double d = 1.0 / l;
  return q4{rf(x * d), rf(y * d), rf(z * d), rf(w * d)};
}
DI q4 qnormalize_fast(q4 q) {
  const double x = F(q.x), y = F(q.y), z = F(q.z), w = F(q.w);
  const double f = (3.0 - fma_ff(w, w, fma_ff(z, z, fma_ff(y, y, x * x)))) / 2.0;
  if (f == 0) return q4{0.f, 0.f, 0.f, 0.f};
  return q4{rf(x * f), rf(y * f), rf(z * f), rf(w * f)};
}

// ---- lib/math/mat3.dart (storage e[3*row+col]) ----
DI f3 mvmult(const float* e, f3 v) {  // (e0*x + e1*y) + e2*z per row
  const double x = F(v.x), y = F(v.y), z = F(v.z);
  return f3{rf(fma_ff(F(e[2]), z, fma_ff(F(e[1]), y, F(e[0]) * x))), rf(fma_ff(F(e[5]), z, fma_ff(F(e[4]), y, F(e[3]) * x))),
            rf(fma_ff(F(e[8]), z, fma_ff(F(e[7]), y, F(e[6]) * x)))};
}
// rigid_body.dart:459-464: m1 = R(q); m2 = m1^T; m1 = vscale(I, m1); out = m1 * m2
DI void inertia_world(q4 q, f3 I, float* out) {
  const double x = F(q.x), y = F(q.y), z = F(q.z), w = F(q.w);
  // x2 = x + x is exact, and x * x2 is a product of binary32 values times 2,
  // exact too: the sums below fuse like products of binary32 values
  const double x2 = x + x, y2 = y + y, z2 = z + z;
  const double xx = x * x2, xy = x * y2, xz = x * z2, yy = y * y2, yz = y * z2;  // z*z2 enters through the fused forms
  float m[9];
  m[0] = rf(1 - fma_ff(z, z2, yy)); m[1] = rf(fma_ff(-w, z2, xy)); m[2] = rf(fma_ff(w, y2, xz));
  m[3] = rf(fma_ff(w, z2, xy)); m[4] = rf(1 - fma_ff(z, z2, xx)); m[5] = rf(fma_ff(-w, x2, yz));
  m[6] = rf(fma_ff(-w, y2, xz)); m[7] = rf(fma_ff(w, x2, yz)); m[8] = rf(1 - fma_ff(y, y2, xx));
  float t[9] = {m[0], m[3], m[6], m[1], m[4], m[7], m[2], m[5], m[8]};  // transpose
  float a[9];
#pragma unroll
  for (int i = 0; i < 3; i++) {  // one binary32 product each, rounded: the binary32 multiply
    a[3 * i + 0] = __fmul_rn(I.x, m[3 * i + 0]);
    a[3 * i + 1] = __fmul_rn(I.y, m[3 * i + 1]);
    a[3 * i + 2] = __fmul_rn(I.z, m[3 * i + 2]);
  }
#pragma unroll
  for (int r = 0; r < 3; r++) {
    const double a1 = F(a[3 * r]), a2 = F(a[3 * r + 1]), a3 = F(a[3 * r + 2]);
#pragma unroll
    for (int c = 0; c < 3; c++) out[3 * r + c] = rf(fma_ff(a3, F(t[6 + c]), fma_ff(a2, F(t[3 + c]), a1 * F(t[c]))));
  }
}

// ---- lib/math/transform.dart ----
DI f3 point_to_local(f3 pos, q4 q, f3 wp) { return vmult(qconj(q), sub(wp, pos)); }
DI f3 vector_to_local(q4 q, f3 wv) { return vmult(qnegw(q), wv); }
