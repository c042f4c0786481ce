// cp_ray.cu -- raycasts over a world's resident state: World.raycastClosest /
// raycastAny / raycastAll (lib/world/world_class.dart:248-278) through
// Ray.intersectWorld (lib/collision/ray_class.dart:163-199).
//
// k_ray_prep (one block) does what the broadphase's aabbQuery does to the
// world before any ray is cast: it refreshes the AABBs of the bodies that
// need it and, for a SAPBroadphase, re-sorts the axis list.  k_ray_cast then
// takes one ray per thread; the rays only read the world.  Arithmetic follows
// the same binary64-compute / binary32-store contract as the step kernels.
#include <cuda_runtime.h>

#include "cp_kernels.h"
#include "cp_narrow.cuh"
#include "cp_cc.cuh"
#include "cp_types.h"
#include "cp_phases.cuh"

namespace {

// Body.updateAABB (rigid_body.dart:415-447) at the body's current pose: each
// shape's world AABB, the first copied, the others extended in
DI void body_aabb(const DWorld& W, const DBody& B, f3& mn, f3& mx) {
  const q4 q = ld4q(B.quat);
  const f3 p = ld3(B.pos);
  shape_world_aabb(W, W.shapes[B.shape], add(vmult(q, ld3(B.shape_off)), p), qmul(q, ld4q(B.shape_quat)), mn, mx);
  for (int e = 0; e < B.nxs; e++) {
    const DBodyShape& X = W.bshapes[B.xs0 + e];
    f3 lo, hi;
    shape_world_aabb(W, W.shapes[X.shape], add(vmult(q, ld3(X.off)), p), qmul(q, ld4q(X.quat)), lo, hi);
    mn = f3{dart_min(mn.x, lo.x), dart_min(mn.y, lo.y), dart_min(mn.z, lo.z)};
    mx = f3{dart_max(mx.x, hi.x), dart_max(mx.y, hi.y), dart_max(mx.z, hi.z)};
  }
}

__global__ void k_ray_prep(const DWorld* dw) {
  __shared__ Smem S;
  if (threadIdx.x == 0) {
    S.W = *dw;
    S.P = *S.W.P;
  }
  __syncthreads();
  const DWorld& W = S.W;
  const int nb = S.P.nb;
  // GridBroadphase has no aabbQuery: the world is left as it is
  if (S.P.broadphase == CP_BROAD_GRID) return;
  for (int i = threadIdx.x; i < nb; i += BT) {
    DBody& B = W.bodies[i];
    if (!(B.flags & BF_AABB_DIRTY)) continue;
    if (B.shape >= 0) {
      f3 mn, mx;
      body_aabb(W, B, mn, mx);
      st3(B.aabb_lo, mn);
      st3(B.aabb_hi, mx);
    }
    B.flags &= ~BF_AABB_DIRTY;
  }
  __syncthreads();
  if (S.P.broadphase != CP_BROAD_SAP) return;
  // SAPBroadphase.sortList (sap_broadphase.dart:168-189): the stable
  // insertion sort on the lower bounds, as a rank sort
  const int axis = S.P.sap_axis;
  float* key = W.sap_key;
  for (int p = threadIdx.x; p < nb; p += BT) key[p] = W.bodies[W.sap_order[p]].aabb_lo[axis];
  __syncthreads();
  for (int p = threadIdx.x; p < nb; p += BT) {
    const float kp = key[p];
    int r = 0;
    for (int q = 0; q < nb; q++) {
      const float kq = key[q];
      r += (kq < kp) || (kq == kp && q < p);
    }
    W.sap_tmp[r] = W.sap_order[p];
  }
  __syncthreads();
  for (int p = threadIdx.x; p < nb; p += BT) W.sap_order[p] = W.sap_tmp[p];
}

// one ray's state (Ray) and result (RaycastResult)
struct RayRun {
  f3 from, to, dir;
  int mode, group, mask;
  bool skip_back, check_resp, stop;
  cp_ray_hit res;
  cp_ray_hit* all;
  int cap, count;
};

// Ray.pointInTriangle (ray_class.dart:669-678)
DI bool point_in_triangle(f3 p, f3 a, f3 b, f3 c) {
  const f3 v0 = sub(c, a), v1 = sub(b, a), v2 = sub(p, a);
  const double dot00 = dot(v0, v0), dot01 = dot(v0, v1), dot02 = dot(v0, v2), dot11 = dot(v1, v1), dot12 = dot(v1, v2);
  const double u = dot11 * dot02 - dot01 * dot12;
  const double v = dot00 * dot12 - dot01 * dot02;
  return u >= 0 && v >= 0 && (u + v) < (dot00 * dot11 - dot01 * dot01);
}

// Ray.distanceFromIntersection (ray_class.dart:679-691)
DI double distance_from_intersection(f3 from, f3 dir, f3 pos) {
  const f3 v0 = sub(pos, from);
  const double d = dot(v0, dir);
  return distance_to(pos, add(scale(dir, d), from));
}

// _reportIntersection (ray_class.dart:617-664): the face index is stored
// before the mode decides whether the hit is kept
DI void report(RayRun& R, f3 normal, f3 hit, int shape, int body, int face) {
  const double distance = distance_to(R.from, hit);
  if (R.skip_back && dot(normal, R.dir) > 0) return;
  R.res.hit_face_index = face;
  bool set = true;
  if (R.mode == CP_RAY_CLOSEST) set = distance < R.res.distance || !R.res.has_hit;
  if (!set) return;
  R.res.has_hit = 1;
  st3(R.res.hit_point, hit);
  st3(R.res.hit_normal, normal);
  R.res.shape = shape;
  R.res.body = body;
  R.res.distance = distance;
  if (R.mode == CP_RAY_ALL) {
    if (R.count < R.cap) R.all[R.count] = R.res;
    R.count++;
  } else if (R.mode == CP_RAY_ANY) {
    R.stop = true;
  }
}

// _intersectSphere (ray_class.dart:387-438); pow(x, 2) as x * x
DI void ray_sphere(RayRun& R, double r, f3 pos, int shape, int body) {
  const double dx = F(R.to.x) - F(R.from.x), dy = F(R.to.y) - F(R.from.y), dz = F(R.to.z) - F(R.from.z);
  const double fx = F(R.from.x) - F(pos.x), fy = F(R.from.y) - F(pos.y), fz = F(R.from.z) - F(pos.z);
  const double a = dx * dx + dy * dy + dz * dz;
  const double b = 2 * (dx * fx + dy * fy + dz * fz);
  const double c = fx * fx + fy * fy + fz * fz - r * r;
  const double delta = b * b - 4 * a * c;
  if (delta < 0) return;
  if (delta == 0) {
    const f3 ip = lerp(R.from, R.to, delta);
    report(R, normalized(sub(ip, pos)), ip, shape, body, -1);
    return;
  }
  const double d1 = (-b - sqrt(delta)) / (2 * a);
  const double d2 = (-b + sqrt(delta)) / (2 * a);
  if (d1 >= 0 && d1 <= 1) {
    const f3 ip = lerp(R.from, R.to, d1);
    report(R, normalized(sub(ip, pos)), ip, shape, body, -1);
  }
  if (R.stop) return;
  if (d2 >= 0 && d2 <= 1) {
    const f3 ip = lerp(R.from, R.to, d2);
    report(R, normalized(sub(ip, pos)), ip, shape, body, -1);
  }
}

// _intersectPlane (ray_class.dart:290-334)
DI void ray_plane(RayRun& R, q4 q, f3 pos, int shape, int body) {
  const f3 n = vmult(q, f3{0.f, 0.f, 1.f});
  const double to_from = dot(sub(R.from, pos), n);
  const double to_to = dot(sub(R.to, pos), n);
  if (to_from * to_to > 0) return;
  if (distance_to(R.from, R.to) < to_from) return;
  const double ndd = dot(n, R.dir);
  if (fabs(ndd) < 0.0001) return;
  const double t = -dot(n, sub(R.from, pos)) / ndd;
  report(R, n, add(R.from, scale(R.dir, t)), shape, body, -1);
}

// _intersectConvex (ray_class.dart:440-530) over hull h
DI void ray_convex(RayRun& R, const DWorld& W, const DHull& H, q4 q, f3 x, int shape, int body) {
  const double from_to = distance_to(R.from, R.to);
  for (int j = 0; !R.stop && j < H.nf; j++) {
    const DFace F = W.faces[H.f0 + j];
    const f3 v0 = hv(W, H.v0 + W.hfi[F.i0]);
    const f3 vec = sub(add(vmult(q, v0), x), R.from);
    const f3 normal = vmult(q, ld3(F.normal));
    const double d = dot(R.dir, normal);
    const double scalar = dot(normal, vec) / d;
    if (scalar < 0) continue;
    const f3 ip = add(scale(R.dir, scalar), R.from);
    const f3 a = add(x, vmult(q, v0));
    for (int i = 1; !R.stop && i + 1 < F.n; i++) {
      const f3 b = add(x, vmult(q, hv(W, H.v0 + W.hfi[F.i0 + i])));
      const f3 c = add(x, vmult(q, hv(W, H.v0 + W.hfi[F.i0 + i + 1])));
      const double distance = distance_to(ip, R.from);
      if (!(point_in_triangle(ip, a, b, c) || point_in_triangle(ip, b, a, c)) || distance > from_to) continue;
      report(R, normal, ip, shape, body, j);
    }
  }
}

// _intersectShape (ray_class.dart:270-288) with the type table of :104-127
// (no entry for Capsule, Cone or SizedPlane)
DI void ray_shape(RayRun& R, const DWorld& W, int si, q4 q, f3 x, int body) {
  const DShape& s = W.shapes[si];
  if (distance_from_intersection(R.from, R.dir, x) > s.bsr) return;
  if (s.type == CP_SHAPE_SPHERE) ray_sphere(R, s.radius, x, si, body);
  else if (s.type == CP_SHAPE_PLANE) ray_plane(R, q, x, si, body);
  else if (s.type == CP_SHAPE_BOX || s.type == CP_SHAPE_CONVEX || s.type == CP_SHAPE_CYLINDER)
    ray_convex(R, W, W.hulls[s.hull], q, x, si, body);
}

// intersectBody (ray_class.dart:201-244)
DI void ray_body(RayRun& R, const DWorld& W, int i) {
  const DBody& B = W.bodies[i];
  if (R.check_resp && !(B.flags & BF_RESPONSE)) return;
  if ((R.group & B.mask) == 0 || (B.group & R.mask) == 0) return;
  if (B.shape < 0) return;
  const q4 q = ld4q(B.quat);
  const f3 p = ld3(B.pos);
  for (int k = 0; k <= B.nxs && !R.stop; k++) {
    int si;
    f3 off;
    q4 orient;
    if (k == 0) {
      si = B.shape;
      off = ld3(B.shape_off);
      orient = ld4q(B.shape_quat);
    } else {
      const DBodyShape& X = W.bshapes[B.xs0 + k - 1];
      si = X.shape;
      off = ld3(X.off);
      orient = ld4q(X.quat);
    }
    if (R.check_resp && !W.shapes[si].response) continue;
    ray_shape(R, W, si, qmul(q, orient), add(vmult(q, off), p), i);
  }
}

// AABB.overlaps (aabb.dart:131-147): body box against the ray's box
DI bool overlaps_query(const DBody& B, f3 lo, f3 hi) {
  const float *l1 = B.aabb_lo, *u1 = B.aabb_hi;
  const bool ox = (lo.x <= u1[0] && u1[0] <= hi.x) || (l1[0] <= hi.x && hi.x <= u1[0]);
  const bool oy = (lo.y <= u1[1] && u1[1] <= hi.y) || (l1[1] <= hi.y && hi.y <= u1[1]);
  const bool oz = (lo.z <= u1[2] && u1[2] <= hi.z) || (l1[2] <= hi.z && hi.z <= u1[2]);
  return ox && oy && oz;
}

__global__ void k_ray_cast(const DWorld* dw, const cp_ray* rays, int n, int mode, cp_ray_hit* hits, int max_hits,
                           int* counts) {
  __shared__ DWorld sW;
  __shared__ DWorldParams sP;
  if (threadIdx.x == 0) {
    sW = *dw;
    sP = *sW.P;
  }
  __syncthreads();
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const DWorld& W = sW;
  const cp_ray ray = rays[r];
  RayRun R;
  R.mode = mode;
  R.group = ray.collision_filter_group;
  R.mask = ray.collision_filter_mask;
  R.skip_back = ray.skip_backfaces != 0;
  R.check_resp = ray.check_collision_response != 0;
  R.stop = false;
  R.from = ld3(ray.from);
  R.to = ld3(ray.to);
  R.dir = normalized(sub(R.to, R.from));
  R.res.has_hit = 0;
  R.res.body = R.res.shape = R.res.hit_face_index = -1;
  R.res.hit_point[0] = R.res.hit_point[1] = R.res.hit_point[2] = 0.f;
  R.res.hit_normal[0] = R.res.hit_normal[1] = R.res.hit_normal[2] = 0.f;
  R.res.distance = -1.0;
  R.all = mode == CP_RAY_ALL ? hits + (size_t)r * max_hits : nullptr;
  R.cap = mode == CP_RAY_ALL ? max_hits : 0;
  R.count = 0;
  // Ray.getAABB (ray_class.dart:337-349)
  const f3 lo{dart_min(R.to.x, R.from.x), dart_min(R.to.y, R.from.y), dart_min(R.to.z, R.from.z)};
  const f3 hi{dart_max(R.to.x, R.from.x), dart_max(R.to.y, R.from.y), dart_max(R.to.z, R.from.z)};
  const int nb = sP.nb;
  if (sP.broadphase != CP_BROAD_GRID) {
    const bool sap = sP.broadphase == CP_BROAD_SAP;
    for (int k = 0; k < nb && !R.stop; k++) {
      const int i = sap ? W.sap_order[k] : k;
      if (overlaps_query(W.bodies[i], lo, hi)) ray_body(R, W, i);
    }
  }
  if (mode == CP_RAY_ALL) counts[r] = R.count;
  else hits[r] = R.res;
}

}  // namespace

cudaError_t cpk_raycast(const DWorld* d_world, const cp_ray* d_rays, int n, int mode, cp_ray_hit* d_hits, int max_hits,
                        int* d_counts, cudaStream_t stream) {
  k_ray_prep<<<1, 256, 0, stream>>>(d_world);
  if (n > 0) k_ray_cast<<<(n + 127) / 128, 128, 0, stream>>>(d_world, d_rays, n, mode, d_hits, max_hits, d_counts);
  return cudaGetLastError();
}
