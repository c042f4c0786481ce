// cp_host.cpp -- host runtime behind include/cannon_gpu.h.
//
//  * setup: the Body / Shape constructor arithmetic (inertia from the body
//    AABB, bounding radii, convex hull tables) restated on the host, because
//    a caller that has no Dart objects still needs the state they would hold;
//  * worlds: one device allocation for the persistent state of a world and
//    one for its step scratch (regrown when a step reports an overflow);
//  * stepping: cp_world_step launches the persistent step kernel on one world;
//    cp_batch_step launches it on many, with the nsteps sequence captured in
//    a CUDA graph that is replayed while the world set and dt stay the same.
//
// Built with -ffp-contract=off: the host arithmetic must round like Dart's.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <iterator>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/cannon_gpu.h"
#include "cp_internal.h"
#include "cp_kernels.h"
#include "cp_types.h"

namespace cpi {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

}  // namespace cpi

using namespace cpi;

namespace {

#define CUDA_TRY(x)                                                                         \
  do {                                                                                      \
    cudaError_t e_ = (x);                                                                   \
    if (e_ != cudaSuccess) return fail(CP_ERR_CUDA, "%s: %s", #x, cudaGetErrorString(e_)); \
  } while (0)

// ---------------------------------------------------------------------------
// host arithmetic (binary64 compute, binary32 store), vector_math semantics

struct h3 { float x = 0.f, y = 0.f, z = 0.f; };
struct hq { float x = 0.f, y = 0.f, z = 0.f, w = 1.f; };

h3 mk3(double x, double y, double z) { h3 v; v.x = (float)x; v.y = (float)y; v.z = (float)z; return v; }
double dot3(const h3& a, const h3& b) {
  double s = (double)a.x * (double)b.x;
  s += (double)a.y * (double)b.y;
  s += (double)a.z * (double)b.z;
  return s;
}
double len3(const h3& a) { return std::sqrt(dot3(a, a)); }
h3 norm3(h3 v) {
  double l = len3(v);
  if (l == 0.0) return v;
  double d = 1.0 / l;
  return mk3(v.x * d, v.y * d, v.z * d);
}
h3 sub3(const h3& a, const h3& b) { return mk3((double)a.x - (double)b.x, (double)a.y - (double)b.y, (double)a.z - (double)b.z); }
h3 add3(const h3& a, const h3& b) { return mk3((double)a.x + (double)b.x, (double)a.y + (double)b.y, (double)a.z + (double)b.z); }
h3 cross3(const h3& a, const h3& v) {
  double vx = v.x, vy = v.y, vz = v.z;
  return mk3((double)a.y * vz - (double)a.z * vy, (double)a.z * vx - (double)a.x * vz, (double)a.x * vy - (double)a.y * vx);
}
bool near3(const h3& a, const h3& v) {
  return !(std::fabs((double)a.x - v.x) > 1e-6 || std::fabs((double)a.y - v.y) > 1e-6 || std::fabs((double)a.z - v.z) > 1e-6);
}
h3 qrot(const hq& q, const h3& v) {
  double x = v.x, y = v.y, z = v.z, qx = q.x, qy = q.y, qz = q.z, qw = q.w;
  double ix = qw * x + qy * z - qz * y;
  double iy = qw * y + qz * x - qx * z;
  double iz = qw * z + qx * y - qy * x;
  double iw = -qx * x - qy * y - qz * z;
  return mk3(ix * qw + iw * -qx + iy * -qz - iz * -qy, iy * qw + iw * -qy + iz * -qx - ix * -qz,
             iz * qw + iw * -qz + ix * -qy - iy * -qx);
}
hq qmul(const hq& a, const hq& b) {
  double ax = a.x, ay = a.y, az = a.z, aw = a.w, bx = b.x, by = b.y, bz = b.z, bw = b.w;
  hq t;
  t.x = (float)(ax * bw + aw * bx + ay * bz - az * by);
  t.y = (float)(ay * bw + aw * by + az * bx - ax * bz);
  t.z = (float)(az * bw + aw * bz + ax * by - ay * bx);
  t.w = (float)(aw * bw - ax * bx - ay * by - az * bz);
  return t;
}
// Body.updateInertiaWorld(force = true) (rigid_body.dart:459-464)
void inertia_world(const hq& q, const h3& I, float* out) {
  double x = q.x, y = q.y, z = q.z, w = q.w;
  double x2 = x + x, y2 = y + y, z2 = z + z;
  double xx = x * x2, xy = x * y2, xz = x * z2, yy = y * y2, yz = y * z2, zz = z * z2;
  double wx = w * x2, wy = w * y2, wz = w * z2;
  float m[9];
  m[0] = (float)(1 - (yy + zz)); m[1] = (float)(xy - wz); m[2] = (float)(xz + wy);
  m[3] = (float)(xy + wz); m[4] = (float)(1 - (xx + zz)); m[5] = (float)(yz - wx);
  m[6] = (float)(xz - wy); m[7] = (float)(yz + wx); m[8] = (float)(1 - (xx + yy));
  float t[9] = {m[0], m[3], m[6], m[1], m[4], m[7], m[2], m[5], m[8]};
  float a[9];
  for (int i = 0; i < 3; i++) {
    a[3 * i + 0] = (float)((double)I.x * m[3 * i + 0]);
    a[3 * i + 1] = (float)((double)I.y * m[3 * i + 1]);
    a[3 * i + 2] = (float)((double)I.z * m[3 * i + 2]);
  }
  for (int r = 0; r < 3; r++) {
    double a1 = a[3 * r], a2 = a[3 * r + 1], a3 = a[3 * r + 2];
    for (int c = 0; c < 3; c++) out[3 * r + c] = (float)(a1 * t[c] + a2 * t[3 + c] + a3 * t[6 + c]);
  }
}

// ---------------------------------------------------------------------------
// convex hulls (convex_polyhedron.dart:80-185, box.dart:41-78, cylinder.dart:222-294)

struct Hull {
  std::vector<h3> verts;
  std::vector<std::vector<int>> faces;
  std::vector<h3> normals;
  std::vector<h3> edges;
  bool has_axes = false;
};

void hull_finish(Hull& h) {
  h.normals.clear();
  for (auto& f : h.faces) {
    const h3 &va = h.verts[f[0]], &vb = h.verts[f[1]], &vc = h.verts[f[2]];
    h3 ab = sub3(vb, va), cb = sub3(vc, vb);
    h3 n = cross3(cb, ab);
    if (!(n.x == 0 && n.y == 0 && n.z == 0)) n = norm3(n);
    n.x = -n.x; n.y = -n.y; n.z = -n.z;
    h.normals.push_back(n);
  }
  h.edges.clear();
  for (auto& f : h.faces) {
    int nv = (int)f.size();
    for (int j = 0; j < nv; j++) {
      h3 e = norm3(sub3(h.verts[f[j]], h.verts[f[(j + 1) % nv]]));
      bool found = false;
      for (auto& u : h.edges)
        if (near3(u, e)) { found = true; break; }
      if (!found) h.edges.push_back(e);
    }
  }
}

int build_hull(const cp_shape_desc& d, Hull& h) {
  if (d.type == CP_SHAPE_BOX) {
    double sx = d.half_extents[0], sy = d.half_extents[1], sz = d.half_extents[2];
    h.verts = {mk3(-sx, -sy, -sz), mk3(sx, -sy, -sz), mk3(sx, sy, -sz), mk3(-sx, sy, -sz),
               mk3(-sx, -sy, sz), mk3(sx, -sy, sz), mk3(sx, sy, sz), mk3(-sx, sy, sz)};
    h.faces = {{3, 2, 1, 0}, {4, 5, 6, 7}, {5, 4, 0, 1}, {2, 3, 7, 6}, {0, 4, 7, 3}, {1, 2, 6, 5}};
    h.has_axes = true;
  } else if (d.type == CP_SHAPE_CYLINDER) {
    const int N = d.num_segments;
    if (d.radius_top < 0 || d.radius_bottom < 0 || N < 3) return fail(CP_ERR_ARG, "invalid cylinder");
    double rt = d.radius_top, rb = d.radius_bottom, ht = d.height;
    std::vector<int> bottom, top;
    h.verts.push_back(mk3(-rb * std::sin(0.0), -ht * 0.5, rb * std::cos(0.0)));
    bottom.push_back(0);
    h.verts.push_back(mk3(-rt * std::sin(0.0), ht * 0.5, rt * std::cos(0.0)));
    top.push_back(1);
    for (int i = 0; i < N; i++) {
      double theta = ((2 * M_PI) / N) * (i + 1);
      if (i < N - 1) {
        h.verts.push_back(mk3(-rb * std::sin(theta), -ht * 0.5, rb * std::cos(theta)));
        bottom.push_back(2 * i + 2);
        h.verts.push_back(mk3(-rt * std::sin(theta), ht * 0.5, rt * std::cos(theta)));
        top.push_back(2 * i + 3);
        h.faces.push_back({2 * i, 2 * i + 1, 2 * i + 3, 2 * i + 2});
      } else {
        h.faces.push_back({2 * i, 2 * i + 1, 1, 0});
      }
    }
    h.faces.push_back(bottom);
    std::vector<int> rev(top.rbegin(), top.rend());
    h.faces.push_back(rev);
    h.has_axes = true;
  } else if (d.type == CP_SHAPE_CONVEX || d.type == CP_SHAPE_CAPSULE || d.type == CP_SHAPE_CONE || d.type == CP_SHAPE_SIZED_PLANE) {
    // Capsule, Cone and SizedPlane: hulls as their constructors built them
    const bool conv = d.type == CP_SHAPE_CONVEX;
    if (d.num_vertices < (conv ? 4 : 3) || d.num_faces < (conv ? 4 : 1) || !d.vertices || !d.face_sizes || !d.face_indices)
      return fail(CP_ERR_ARG, conv ? "convex shape needs >= 4 vertices and faces" : "hull shape needs >= 3 vertices and a face");
    for (int i = 0; i < d.num_vertices; i++) h.verts.push_back(mk3(d.vertices[3 * i], d.vertices[3 * i + 1], d.vertices[3 * i + 2]));
    int off = 0;
    for (int f = 0; f < d.num_faces; f++) {
      std::vector<int> face;
      if (d.face_sizes[f] < 3) return fail(CP_ERR_ARG, "convex face %d has < 3 vertices", f);
      for (int k = 0; k < d.face_sizes[f]; k++) {
        int vi = d.face_indices[off + k];
        if (vi < 0 || vi >= d.num_vertices) return fail(CP_ERR_ARG, "convex face index out of range");
        face.push_back(vi);
      }
      off += d.face_sizes[f];
      h.faces.push_back(face);
    }
    h.has_axes = d.has_axes != 0;
  } else {
    return fail(CP_ERR_ARG, "shape type %d has no hull", d.type);
  }
  hull_finish(h);
  if ((int)h.verts.size() > CP_MAX_HULL_VERTS || (int)h.faces.size() > CP_MAX_HULL_VERTS || (int)h.edges.size() > CP_MAX_HULL_VERTS)
    return fail(CP_ERR_UNSUPPORTED, "hull larger than %d vertices / faces / edges", CP_MAX_HULL_VERTS);
  for (auto& f : h.faces)
    if ((int)f.size() > CP_MAX_FACE_VERTS) return fail(CP_ERR_UNSUPPORTED, "hull face larger than %d vertices", CP_MAX_FACE_VERTS);
  return CP_OK;
}

double shape_bsr(const cp_shape_desc& d, const Hull* h) {
  switch (d.type) {
    case CP_SHAPE_SPHERE: return d.radius;
    case CP_SHAPE_PLANE: return INFINITY;
    case CP_SHAPE_BOX: return len3(mk3(d.half_extents[0], d.half_extents[1], d.half_extents[2]));
    default: {
      double m2 = 0;
      for (auto& v : h->verts) { double n2 = dot3(v, v); if (n2 > m2) m2 = n2; }
      return std::sqrt(m2);
    }
  }
}

// Shape.calculateWorldAABB
// dart:math min / max on doubles: NaN wins, and -0.0 is below 0.0
double dart_min(double a, double b) {
  if (a > b) return b;
  if (a < b) return a;
  if (std::isnan(a) || std::isnan(b)) return NAN;
  return (std::signbit(a) || std::signbit(b)) ? -0.0 : a;
}
double dart_max(double a, double b) {
  if (a < b) return b;
  if (a > b) return a;
  if (std::isnan(a) || std::isnan(b)) return NAN;
  return (std::signbit(a) && std::signbit(b)) ? -0.0 : (a == 0 ? 0.0 : a);
}

// a body's extra shapes lie inside the table and name existing shapes, only
// a body with a first shape has any, and a body has at most CP_MAX_BODY_SHAPES
// shapes
bool extras_valid(const cp_body_desc& d, int num_shapes, const cp_body_shape* table, int ntable) {
  if (d.extra_shapes_count == 0) return true;
  if (d.extra_shapes_count < 0 || d.extra_shapes_count >= CP_MAX_BODY_SHAPES || d.shape < 0 || !table || d.extra_shapes_first < 0 ||
      (long long)d.extra_shapes_first + d.extra_shapes_count > ntable)
    return false;
  for (int k = 0; k < d.extra_shapes_count; k++) {
    const int sh = table[d.extra_shapes_first + k].shape;
    if (sh < 0 || sh >= num_shapes) return false;
  }
  return true;
}

void shape_aabb(const cp_shape_desc& d, const Hull* h, const h3& pos, const hq& q, h3& mn, h3& mx) {
  if (d.type == CP_SHAPE_SPHERE) {
    double r = d.radius;
    mn = mk3(pos.x - r, pos.y - r, pos.z - r);
    mx = mk3(pos.x + r, pos.y + r, pos.z + r);
  } else if (d.type == CP_SHAPE_PLANE) {
    h3 n = qrot(q, mk3(0, 0, 1));
    mn = mk3(-INFINITY, -INFINITY, -INFINITY);
    mx = mk3(INFINITY, INFINITY, INFINITY);
    if (n.x == 1) mx.x = pos.x; else if (n.x == -1) mn.x = pos.x;
    if (n.y == 1) mx.y = pos.y; else if (n.y == -1) mn.y = pos.y;
    if (n.z == 1) mx.z = pos.z; else if (n.z == -1) mn.z = pos.z;
  } else if (d.type == CP_SHAPE_BOX) {
    float ex = d.half_extents[0], ey = d.half_extents[1], ez = d.half_extents[2];
    const float c[8][3] = {{ex, ey, ez}, {-ex, ey, ez}, {-ex, -ey, ez}, {-ex, -ey, -ez},
                           {ex, -ey, -ez}, {ex, ey, -ez}, {-ex, ey, -ez}, {ex, -ey, ez}};
    for (int i = 0; i < 8; i++) {
      h3 w = add3(qrot(q, mk3(c[i][0], c[i][1], c[i][2])), pos);
      if (i == 0) { mn = w; mx = w; continue; }
      if (w.x > mx.x) mx.x = w.x;
      if (w.y > mx.y) mx.y = w.y;
      if (w.z > mx.z) mx.z = w.z;
      if (w.x < mn.x) mn.x = w.x;
      if (w.y < mn.y) mn.y = w.y;
      if (w.z < mn.z) mn.z = w.z;
    }
  } else {
    for (size_t i = 0; i < h->verts.size(); i++) {
      h3 w = add3(qrot(q, h->verts[i]), pos);
      if (i == 0) { mn = w; mx = w; continue; }
      if (w.x < mn.x) mn.x = w.x;
      if (w.x > mx.x) mx.x = w.x;
      if (w.y < mn.y) mn.y = w.y;
      if (w.y > mx.y) mx.y = w.y;
      if (w.z < mn.z) mn.z = w.z;
      if (w.z > mx.z) mx.z = w.z;
    }
  }
}

}  // namespace

namespace {

int upload_world_entry(cp_ctx* c, int id) {
  if (id >= c->d_worlds_cap) {
    int nc = std::max(64, 2 * (id + 1));
    DWorld* nw = nullptr;
    CUDA_TRY(cudaMalloc(&nw, sizeof(DWorld) * nc));
    if (c->d_worlds) {
      CUDA_TRY(cudaMemcpy(nw, c->d_worlds, sizeof(DWorld) * c->d_worlds_cap, cudaMemcpyDeviceToDevice));
      cudaFree(c->d_worlds);
    }
    c->d_worlds = nw;
    c->d_worlds_cap = nc;
    if (c->graph) { cudaGraphExecDestroy(c->graph); c->graph = nullptr; }
  }
  CUDA_TRY(cudaMemcpy(c->d_worlds + id, &c->worlds[id].dw, sizeof(DWorld), cudaMemcpyHostToDevice));
  return CP_OK;
}

int pow2_at_least(int v) {
  int p = 1;
  while (p < v) p <<= 1;
  return p;
}

// Layout of a world's scratch for its current capacities; returns its size
// and, when `base` is given, points the scratch arrays of `d` into it.
size_t scratch_layout_into(const WorldRec& w, DWorld& d, char* base) {
  const int nb = w.nb, cc = w.contacts_cap, rc = w.rows_cap;
  const int pc0 = std::max(w.pairs_cap, nb);  // SAP also keeps one count per list position in the pair arrays
  const int pc = std::max(pc0, w.jobs_cap);   // arrays indexed by narrowphase job
  const int cand_cap = 3 * cc + w.ncon_rows + 1;
  const int hash_cap = w.broadphase == CP_BROAD_GRID ? pow2_at_least(2 * pc0 + 2) : 2;
  Layout L;
  size_t o_bscr = L.take(sizeof(DBodyScr) * (nb + 1));
  size_t o_brec = L.take(sizeof(float4) * (nb + 1));
  size_t o_bgm = L.take(sizeof(int2) * (nb + 1));
  size_t o_cbox = L.take(sizeof(float4) * 2 * ((size_t)nb / 32 + 2));
  size_t o_tmp = L.take(sizeof(int) * (nb + 1));
  size_t o_pa = L.take(sizeof(int) * (pc0 + 1));
  size_t o_pb = L.take(sizeof(int) * (pc0 + 1));
  size_t o_jp = L.take(sizeof(int) * (w.jobs_cap + 1));
  size_t o_js = L.take(sizeof(int) * (w.jobs_cap + 1));
  size_t o_pc = L.take(sizeof(int) * (pc + 1));
  size_t o_pt = L.take(sizeof(int) * (pc + 1));
  size_t o_pf = L.take(sizeof(int) * (pc + 1));
  size_t o_hv = L.take(sizeof(int) * (pc + 1));
  size_t o_hv2 = L.take(sizeof(int) * (pc + 16 * 32 + 1));
  size_t o_ct = L.take(sizeof(DContact) * (cc + 1));
  size_t o_co = L.take(sizeof(DContact) * (cc + 1));
  size_t o_cs = L.take(sizeof(int) * (cc + 1));
  size_t o_cd = L.take(sizeof(int) * (cand_cap + 1));
  size_t o_rw = L.take(sizeof(DRow) * (rc + 1));
  size_t o_ab = L.take(sizeof(double) * (rc + 1));
  size_t o_lo = L.take(sizeof(int) * (rc + 1));
  size_t o_lr = L.take(sizeof(int) * (rc + 1));
  size_t o_ls = L.take(sizeof(int) * (rc + 2));
  size_t o_lc = L.take(sizeof(int) * (rc + 2));
  const int swc = rc + 1;
  size_t o_swj = L.take(sizeof(float) * 4 * 5 * (size_t)swc);
  size_t o_swd = L.take(sizeof(double) * 2 * 4 * (size_t)swc);
  size_t o_swb = L.take(sizeof(int) * 2 * (size_t)swc);
  size_t o_swo = L.take(sizeof(int) * (size_t)swc);
  size_t o_sk = L.take(sizeof(float) * (nb + 1));
  const int nbins = w.broadphase == CP_BROAD_GRID ? w.nbins : 0;
  size_t o_bc = L.take(sizeof(int) * (nbins + 2));
  size_t o_bs = L.take(sizeof(int) * (nbins + 2));
  size_t o_bb = L.take(sizeof(int) * (w.bins_cap + 1));
  size_t o_ba = L.take(sizeof(float) * (w.broadphase == CP_BROAD_GRID ? 3 * 4096 : 1));
  size_t o_hk = L.take(sizeof(long long) * hash_cap);
  size_t o_hw = L.take(sizeof(int) * hash_cap);
  // SplitSolver arrays (one element each without it)
  const bool sp = w.split;
  const int sort_n = sp ? pow2_at_least(rc + 1) : 1;
  size_t o_sct = L.take(sizeof(long long) * (sp ? cc + 1 : 1));
  size_t o_sfr = L.take(sizeof(long long) * (sp ? 2 * (size_t)cc + 1 : 1));
  size_t o_srw = L.take(sizeof(long long) * (sp ? rc + 1 : 1));
  size_t o_skey = L.take(sizeof(long long) * sort_n);
  size_t o_sval = L.take(sizeof(int) * sort_n);
  size_t o_ipar = L.take(sizeof(int) * (sp ? nb + 1 : 1));
  size_t o_irow = L.take(sizeof(int) * (sp ? nb + 1 : 1));
  size_t o_iit = L.take(sizeof(int) * (sp ? nb + 1 : 1));
  size_t o_isum = L.take(sizeof(double) * (sp ? nb + 1 : 1));
  size_t o_risl = L.take(sizeof(int) * (sp ? rc + 1 : 1));
  size_t o_jatt = L.take(sizeof(int) * (sp ? pc + 1 : 1));
  size_t o_jbase = L.take(sizeof(int) * (sp ? pc + 1 : 1));
  size_t o_wd = L.take(sizeof(DWide));
  size_t o_wp = L.take(sizeof(int) * (CP_WIDE_SCAN_BLOCKS + 1));
  size_t o_wv = L.take(sizeof(float) * 6 * (size_t)(nb + 1));
  size_t o_wf = L.take((size_t)nb + 1);
  if (!base) return L.off;
  d.bscr = (DBodyScr*)(base + o_bscr);
  d.brec = (float4*)(base + o_brec);
  d.bgm = (int2*)(base + o_bgm);
  d.cbox = (float4*)(base + o_cbox);
  d.sap_tmp = (int*)(base + o_tmp);
  d.pair_a = (int*)(base + o_pa);
  d.pair_b = (int*)(base + o_pb);
  d.job_pair = (int*)(base + o_jp);
  d.ct_id = (long long*)(base + o_sct);
  d.fr_id = (long long*)(base + o_sfr);
  d.row_id = (long long*)(base + o_srw);
  d.sort_key = (long long*)(base + o_skey);
  d.sort_val = (int*)(base + o_sval);
  d.sort_n = sort_n;
  d.isl_par = (int*)(base + o_ipar);
  d.isl_rows = (int*)(base + o_irow);
  d.isl_iter = (int*)(base + o_iit);
  d.isl_sum = (double*)(base + o_isum);
  d.row_isl = (int*)(base + o_risl);
  d.job_att = (int*)(base + o_jatt);
  d.job_base = (int*)(base + o_jbase);
  d.job_sh = (int*)(base + o_js);
  d.pair_cnt = (int*)(base + o_pc);
  d.pair_tstart = (int*)(base + o_pt);
  d.pair_flag = (int*)(base + o_pf);
  d.heavy = (int*)(base + o_hv);
  d.heavy2 = (int*)(base + o_hv2);
  d.ctmp = (DContact*)(base + o_ct);
  d.contacts = (DContact*)(base + o_co);
  d.cscr = (int*)(base + o_cs);
  d.cand = (int*)(base + o_cd);
  d.rows = (DRow*)(base + o_rw);
  d.absdl = (double*)(base + o_ab);
  d.level_of = (int*)(base + o_lo);
  d.level_rows = (int*)(base + o_lr);
  d.level_start = (int*)(base + o_ls);
  d.level_cursor = (int*)(base + o_lc);
  d.sap_key = (float*)(base + o_sk);
  d.bin_cnt = (int*)(base + o_bc);
  d.bin_start = (int*)(base + o_bs);
  d.bin_body = (int*)(base + o_bb);
  d.bin_acc = (float*)(base + o_ba);
  d.hkeys = (long long*)(base + o_hk);
  d.hvals = (int*)(base + o_hw);
  d.hash_cap = hash_cap;
  d.sw_j = (float4*)(base + o_swj);
  d.sw_d = (double2*)(base + o_swd);
  d.sw_b = (int2*)(base + o_swb);
  d.sw_orig = (int*)(base + o_swo);
  d.sw_cap = swc;
  d.wide = (DWide*)(base + o_wd);
  d.wpart = (int*)(base + o_wp);
  d.wvel = (float*)(base + o_wv);
  d.wflag = (unsigned char*)(base + o_wf);
  return L.off;
}

size_t scratch_layout(WorldRec& w, char* base) { return scratch_layout_into(w, w.dw, base); }

// Device memory of a world: from the context's pool when it has one (stream
// ordered on the context's stream), else cudaMalloc.
int dev_alloc(cp_ctx* c, void** p, size_t bytes, const char* what) {
  *p = nullptr;
  cudaError_t e = c->pool ? cudaMallocFromPoolAsync(p, bytes, c->pool, c->stream) : cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    *p = nullptr;
    cudaGetLastError();
    return fail(CP_ERR_OOM, "%s: allocation of %zu bytes failed: %s", what, bytes, cudaGetErrorString(e));
  }
  return CP_OK;
}

void dev_free(cp_ctx* c, void* p, bool pooled) {
  if (!p) return;
  if (pooled) cudaFreeAsync(p, c->stream);
  else cudaFree(p);
}

// (re)allocate the scratch of a world for its current capacities
int alloc_scratch(cp_ctx* c, WorldRec& w) {
  if (w.scratch) { dev_free(c, w.scratch, w.pooled); w.scratch = nullptr; }
  w.scratch_bytes = scratch_layout(w, nullptr);
  char* base = nullptr;
  int st = dev_alloc(c, (void**)&base, w.scratch_bytes, "world scratch");
  if (st) return st;
  w.scratch = base;
  scratch_layout(w, base);
  // the wide path's index-check record must start clear
  CUDA_TRY(cudaMemsetAsync(w.dw.wide, 0, sizeof(DWide), c->stream));
  // SplitSolver: the equation pools outlive the scratch; they hold at most
  // the most contacts (friction objects: twice that) of any step, so they
  // grow with the contact list, keeping what they hold
  if (w.split && w.pool_cap < w.contacts_cap) {
    const int cap = w.contacts_cap;
    long long* np = nullptr;
    CUDA_TRY(cudaMalloc(&np, sizeof(long long) * 3 * ((size_t)cap + 1)));
    if (w.pool) {
      const int old = w.pool_cap;
      CUDA_TRY(cudaMemcpyAsync(np, w.pool, sizeof(long long) * old, cudaMemcpyDeviceToDevice, c->stream));
      CUDA_TRY(cudaMemcpyAsync(np + cap + 1, w.pool + old + 1, sizeof(long long) * 2 * old, cudaMemcpyDeviceToDevice, c->stream));
      CUDA_TRY(cudaStreamSynchronize(c->stream));
      cudaFree(w.pool);
    }
    w.pool = np;
    w.pool_cap = cap;
  }
  w.dw.pool_c = w.pool;
  w.dw.pool_f = w.pool ? w.pool + w.pool_cap + 1 : nullptr;
  return CP_OK;
}


void body_to_device(const cp_body_desc& s, DBody& b) {
  std::memset(&b, 0, sizeof(b));
  std::memcpy(b.pos, s.position, 12);
  std::memcpy(b.quat, s.quaternion, 16);
  std::memcpy(b.vel, s.velocity, 12);
  std::memcpy(b.avel, s.angular_velocity, 12);
  std::memcpy(b.force, s.force, 12);
  std::memcpy(b.torque, s.torque, 12);
  std::memcpy(b.iw, s.inv_inertia_world, 36);
  std::memcpy(b.inv_inertia, s.inv_inertia, 12);
  std::memcpy(b.lin_factor, s.linear_factor, 12);
  std::memcpy(b.ang_factor, s.angular_factor, 12);
  std::memcpy(b.aabb_lo, s.aabb_lower, 12);
  std::memcpy(b.aabb_hi, s.aabb_upper, 12);
  std::memcpy(b.shape_off, s.shape_offset, 12);
  std::memcpy(b.shape_quat, s.shape_orientation, 16);
  std::memcpy(b.prev_pos, s.previous_position, 12);
  std::memcpy(b.prev_quat, s.previous_quaternion, 16);
  std::memcpy(b.interp_pos, s.interpolated_position, 12);
  std::memcpy(b.interp_quat, s.interpolated_quaternion, 16);
  b.mass = s.mass; b.inv_mass = s.inv_mass;
  b.lin_damp = s.linear_damping; b.ang_damp = s.angular_damping;
  b.sleep_speed_limit = s.sleep_speed_limit; b.sleep_time_limit = s.sleep_time_limit;
  b.time_last_sleepy = s.time_last_sleepy; b.bounding_radius = s.bounding_radius;
  b.type = s.type; b.sleep_state = s.sleep_state;
  b.flags = (s.allow_sleep ? BF_ALLOW_SLEEP : 0) | (s.wake_up_after_narrowphase ? BF_WAKE : 0) |
            (s.collision_response ? BF_RESPONSE : 0) | (s.is_trigger ? BF_TRIGGER : 0) |
            (s.fixed_rotation ? BF_FIXED_ROT : 0) | (s.aabb_needs_update ? BF_AABB_DIRTY : 0);
  b.group = s.collision_filter_group; b.mask = s.collision_filter_mask;
  b.material = s.material; b.shape = s.shape;
  b.brad32 = (float)s.bounding_radius;
  b.xs0 = s.extra_shapes_first;
  b.nxs = s.extra_shapes_count;
}

void body_from_device(const DBody& b, cp_body_desc& s) {
  std::memset(&s, 0, sizeof(s));
  std::memcpy(s.position, b.pos, 12);
  std::memcpy(s.quaternion, b.quat, 16);
  std::memcpy(s.velocity, b.vel, 12);
  std::memcpy(s.angular_velocity, b.avel, 12);
  std::memcpy(s.force, b.force, 12);
  std::memcpy(s.torque, b.torque, 12);
  std::memcpy(s.inv_inertia_world, b.iw, 36);
  std::memcpy(s.inv_inertia, b.inv_inertia, 12);
  std::memcpy(s.linear_factor, b.lin_factor, 12);
  std::memcpy(s.angular_factor, b.ang_factor, 12);
  std::memcpy(s.aabb_lower, b.aabb_lo, 12);
  std::memcpy(s.aabb_upper, b.aabb_hi, 12);
  std::memcpy(s.shape_offset, b.shape_off, 12);
  std::memcpy(s.shape_orientation, b.shape_quat, 16);
  std::memcpy(s.previous_position, b.prev_pos, 12);
  std::memcpy(s.previous_quaternion, b.prev_quat, 16);
  std::memcpy(s.interpolated_position, b.interp_pos, 12);
  std::memcpy(s.interpolated_quaternion, b.interp_quat, 16);
  s.mass = b.mass; s.inv_mass = b.inv_mass;
  s.linear_damping = b.lin_damp; s.angular_damping = b.ang_damp;
  s.sleep_speed_limit = b.sleep_speed_limit; s.sleep_time_limit = b.sleep_time_limit;
  s.time_last_sleepy = b.time_last_sleepy; s.bounding_radius = b.bounding_radius;
  s.type = b.type; s.sleep_state = b.sleep_state;
  s.allow_sleep = (b.flags & BF_ALLOW_SLEEP) != 0;
  s.wake_up_after_narrowphase = (b.flags & BF_WAKE) != 0;
  s.collision_response = (b.flags & BF_RESPONSE) != 0;
  s.is_trigger = (b.flags & BF_TRIGGER) != 0;
  s.fixed_rotation = (b.flags & BF_FIXED_ROT) != 0;
  s.aabb_needs_update = (b.flags & BF_AABB_DIRTY) != 0;
  s.collision_filter_group = b.group; s.collision_filter_mask = b.mask;
  s.material = b.material; s.shape = b.shape;
  s.extra_shapes_first = b.xs0;
  s.extra_shapes_count = b.nxs;
}

// Equation.setSpookParams (equation_class.dart:53-60)
void spook(double stiffness, double relaxation, double h, double& a, double& b, double& eps) {
  double d = relaxation, k = stiffness;
  a = 4.0 / (h * (1 + 4 * d));
  b = 4.0 * d / (1 + 4 * d);
  eps = 4.0 / (h * h * k * (1 + 4 * d));
}

// dt-dependent tables: damping powers (libm pow, as Dart's math.pow) and the
// contact materials' SPOOK parameters (createContactEquation uses world.dt)
int ensure_dt(cp_ctx* c, WorldRec& w, double dt) {
  if (w.dt_cached == dt) return CP_OK;
  std::vector<double> p(2 * (size_t)w.nb);
  for (int i = 0; i < w.nb; i++) {
    p[2 * i] = std::pow(1.0 - w.lin_damp[i], dt);
    p[2 * i + 1] = std::pow(1.0 - w.ang_damp[i], dt);
  }
  for (auto& m : w.cms) {
    spook(m.cs, m.cr, dt, m.ca, m.cb, m.ceps);
    spook(m.fs, m.fr, dt, m.fa, m.fb, m.feps);
  }
  CUDA_TRY(cudaMemcpyAsync(w.dw.dpow, p.data(), sizeof(double) * p.size(), cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(cudaMemcpyAsync(w.dw.cms, w.cms.data(), sizeof(DContactMaterial) * w.cms.size(), cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  w.dt_cached = dt;
  return CP_OK;
}

int check_world(cp_ctx* c, int id) {
  if (!c) return fail(CP_ERR_ARG, "null context");
  if (id < 0 || id >= (int)c->worlds.size() || !c->worlds[id].live) return fail(CP_ERR_ARG, "no world %d", id);
  return CP_OK;
}

int read_params(cp_ctx* c, WorldRec& w, DWorldParams& p) {
  CUDA_TRY(cudaMemcpyAsync(&p, w.dw.P, sizeof(p), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  return CP_OK;
}

// grow the capacities a failed step reported and clear the status
int grow(cp_ctx* c, int id, int status) {
  WorldRec& w = c->worlds[id];
  if (status & ST_HULL_OVERFLOW) return fail(CP_ERR_CAPACITY, "a clipped polygon exceeded %d vertices", CP_MAX_CLIP);
  if (status & ST_PAIRS_OVERFLOW) w.pairs_cap *= 2;
  if (status & ST_CONTACTS_OVERFLOW) w.contacts_cap *= 2;
  if (status & ST_ROWS_OVERFLOW) w.rows_cap *= 2;
  if (status & ST_BINS_OVERFLOW) w.bins_cap *= 2;
  if (status & ST_JOBS_OVERFLOW) w.jobs_cap *= 2;
  if (w.pairs_cap > (1 << 28) || w.contacts_cap > (1 << 28) || w.rows_cap > (1 << 28) || w.jobs_cap > (1 << 28))
    return fail(CP_ERR_CAPACITY, "capacity limit");
  const long long lim = c->list_cap_limit;
  if (lim > 0 && (w.pairs_cap > lim || w.contacts_cap > lim || w.rows_cap > lim || w.bins_cap > lim))
    return fail(CP_ERR_CAPACITY, "world %d: its pair, contact or row list would grow beyond %lld entries", id, lim);
  int st = alloc_scratch(c, w);
  if (st) return st;
  DWorldParams p;
  st = read_params(c, w, p);
  if (st) return st;
  p.status = 0;
  p.pairs_cap = w.pairs_cap;
  p.contacts_cap = w.contacts_cap;
  p.rows_cap = w.rows_cap;
  p.bins_cap = w.bins_cap;
  p.jobs_cap = w.jobs_cap;
  CUDA_TRY(cudaMemcpy(w.dw.P, &p, sizeof(p), cudaMemcpyHostToDevice));
  return upload_world_entry(c, id);
}

int ensure_ids(cp_ctx* c, int n) {
  if (n > c->d_ids_cap) {
    if (c->d_ids) cudaFree(c->d_ids);
    if (c->d_status) cudaFree(c->d_status);
    int cap = std::max(256, 2 * n);
    CUDA_TRY(cudaMalloc(&c->d_ids, sizeof(int) * cap));
    CUDA_TRY(cudaMalloc(&c->d_status, sizeof(long long) * 8 * cap));
    if (c->d_gstart) cudaFree(c->d_gstart);
    CUDA_TRY(cudaMalloc(&c->d_gstart, sizeof(int) * (cap + 1)));
    c->d_ids_cap = cap;
    c->d_status_cap = cap;
    c->dev_order.clear();
    c->dev_gstart.clear();
    if (c->graph) { cudaGraphExecDestroy(c->graph); c->graph = nullptr; }
  }
  return CP_OK;
}

// Reports a failed index check of the solve kernel (the kernel skipped the
// access) as an error of the call that launched it.
int kernel_check() {
  int chk[4];
  CUDA_TRY(cpk_read_check(chk));
  if (chk[0] != 0)
    return fail(CP_ERR_CUDA, "solve kernel index check %d failed: world %d, index %d, bound %d", chk[0], chk[1], chk[2], chk[3]);
  return CP_OK;
}

// a SplitSolver world steps on the one-block path, whatever its size
bool is_wide(const cp_ctx* c, const WorldRec& w) { return !w.split && c->wide_bodies > 0 && w.nb >= c->wide_bodies; }

WideShape wide_shape(const WorldRec& w) {
  WideShape s;
  s.nb = w.nb;
  s.nbins = w.broadphase == CP_BROAD_GRID ? w.nbins : 0;
  s.broadphase = w.broadphase;
  s.n_nocollide = w.n_nocollide;
  s.pairs_cap = w.pairs_cap;
  s.contacts_cap = w.contacts_cap;
  s.rows_cap = w.rows_cap;
  s.bins_cap = w.bins_cap;
  s.smem_vel = w.nb <= cpk_wide_smem_vel_max();
  s.compound = w.compound;
  s.jobs_cap = w.jobs_cap;
  return s;
}

// Reports a failed index check of the wide sweep kernel (the kernel skipped
// the access) as an error of the call that launched it.
int wide_check(cp_ctx* c, const WorldRec& w, int id) {
  int chk[4] = {0, 0, 0, 0};
  CUDA_TRY(cpk_wide_check(w.dw, chk, c->stream));
  if (chk[0] != 0)
    return fail(CP_ERR_CUDA, "wide sweep kernel index check %d failed: world %d, index %d, bound %d", chk[0], id, chk[1], chk[2]);
  return CP_OK;
}

// The slot-scheduled sweeps' buffers of a wide world (DSched), sized for its
// row capacity, iteration count and bodies; remade when the row capacity has
// grown.  Above kSchedMaxBytes the world keeps the level-by-level sweeps
// (the device sees a zero-sized DSched).
const size_t kSchedMaxBytes = (size_t)1 << 30;
int ensure_sched(cp_ctx* c, int id) {
  WorldRec& w = c->worlds[id];
  DSched& D = w.dw.sched;
  const long long R = w.rows_cap, S = w.iterations, N = w.nb;
  if (D.rows >= R && D.iters == S && D.nb >= N && w.sched_mem) {
    if (D.mode == c->sched_mode) return CP_OK;
    D.mode = c->sched_mode;
    return upload_world_entry(c, id);
  }
  if (S <= 0 || R <= 0 || w.sched_skip_rows >= R) return CP_OK;
  Layout L;
  const size_t o_lam = L.take(sizeof(double) * S * R), o_abs = L.take(sizeof(double) * S * R);
  const size_t o_slot = L.take(sizeof(int) * S * R), o_first = L.take((size_t)(S * R));
  const size_t o_items = L.take(sizeof(int) * S * R), o_ends = L.take(sizeof(int) * (S * R + 1));
  const size_t o_bt = L.take(sizeof(int) * N), o_bs = L.take(sizeof(int) * N), o_act = L.take((size_t)R);
  const size_t o_ck = L.take(sizeof(float) * 6 * S * N);
  if (w.sched_mem) {
    dev_free(c, w.sched_mem, w.pooled);
    w.sched_mem = nullptr;
    w.sched_bytes = 0;
  }
  std::memset(&D, 0, sizeof(D));
  if (L.off <= kSchedMaxBytes) {
    char* base = nullptr;
    if (dev_alloc(c, (void**)&base, L.off, "sweep schedule") == CP_OK) {
      w.sched_mem = base;
      w.sched_bytes = L.off;
      D.lam = (double*)(base + o_lam);
      D.absdl = (double*)(base + o_abs);
      D.slot = (int*)(base + o_slot);
      D.first = (unsigned char*)(base + o_first);
      D.items = (int*)(base + o_items);
      D.ends = (int*)(base + o_ends);
      D.body_t = (int*)(base + o_bt);
      D.body_s = (int*)(base + o_bs);
      D.act = (unsigned char*)(base + o_act);
      D.ckpt = (float*)(base + o_ck);
      D.rows = (int)R;
      D.iters = (int)S;
      D.nb = (int)N;
      D.mode = c->sched_mode;
    } else {
      g_err.clear();  // no room: the level-by-level sweeps need none of it
    }
  }
  if (!w.sched_mem) w.sched_skip_rows = R;
  return upload_world_entry(c, id);
}

// nsteps internal steps of one world; its time advances by time_inc per step.
// One-block worlds: the world's parameters before the launches, after them
// and the index check record come back in one copy sequence with a single
// stream synchronisation; a step that overflowed a capacity (rare) then
// takes the retry loop below, which reads as it goes.
int plain_steps(cp_ctx* c, int id, double dt, int nsteps, double time_inc) {
  WorldRec& w = c->worlds[id];
  int st = ensure_dt(c, w, dt);
  if (st) return st;
  const bool wide = is_wide(c, w);
  cp_ctx::PlainStage* hs = c->h_plain;
  if (c->plain_id != id) {
    hs->id = id;  // pinned: the copy reads it when it runs, and nothing rewrites it before the synchronisation below
    CUDA_TRY(cudaMemcpyAsync(c->d_one, &hs->id, sizeof(int), cudaMemcpyHostToDevice, c->stream));
    c->plain_id = id;
  }
  DWorldParams p;
  long long target;
  if (!wide) {
    CUDA_TRY(cudaMemcpyAsync(&hs->before, w.dw.P, sizeof(DWorldParams), cudaMemcpyDeviceToHost, c->stream));
    for (int s = 0; s < nsteps; s++) {
      CUDA_TRY(cpk_launch_step(c->d_worlds, c->d_one, c->d_one_group, 1, dt, time_inc, c->d_queue, 1, 1, c->stream,
                               w.nb > 512 ? 0 : c->plain_variant, 1, w.nb));
      c->launches += 2;  // the two step kernels (the queue reset is a memset)
    }
    CUDA_TRY(cudaMemcpyAsync(&hs->after, w.dw.P, sizeof(DWorldParams), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cpk_read_check_async(hs->chk, c->stream));
    const cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) {
      c->plain_id = -1;
      return fail(CP_ERR_CUDA, "%s", cudaGetErrorString(e));
    }
    if (hs->chk[0] != 0) return kernel_check();  // reads the record again, clears it and reports it
    p = hs->after;
    target = hs->before.stepnumber + nsteps;
    if (p.status == 0 && p.stepnumber == target) return CP_OK;
  } else {
    st = read_params(c, w, p);
    if (st) return st;
    target = p.stepnumber + nsteps;
  }
  for (int guard = 0; guard < 64; guard++) {
    long long done = p.stepnumber;
    if (wide) {
      st = ensure_sched(c, id);
      if (st) return st;
    }
    if (wide && target > done)
      CUDA_TRY(cpk_launch_wide_steps(c->d_worlds + id, w.dw, wide_shape(w), dt, time_inc, (int)(target - done), c->stream,
                                     &c->launches));
    for (long long s = done; s < target && !wide; s++) {
      CUDA_TRY(cpk_launch_step(c->d_worlds, c->d_one, c->d_one_group, 1, dt, time_inc, c->d_queue, 1, 1, c->stream,
                               w.nb > 512 ? 0 : c->plain_variant, 1, w.nb));
      c->launches += 2;  // the two step kernels (the queue reset is a memset)
    }
    st = read_params(c, w, p);
    if (st) return st;
    if (p.status == 0) break;
    st = grow(c, id, p.status);
    if (st) return st;
    st = read_params(c, w, p);
    if (st) return st;
  }
  st = wide ? wide_check(c, w, id) : kernel_check();
  if (st) return st;
  if (p.status != 0 || p.stepnumber != target) return fail(CP_ERR_CAPACITY, "world %d could not complete its steps", id);
  return CP_OK;
}

}  // namespace

// ===========================================================================
extern "C" {

const char* cp_last_error(void) { return g_err.c_str(); }
int cp_abi_version(void) { return CP_ABI_VERSION; }

int cp_shape_setup(cp_shape_desc* s) {
  if (!s) return fail(CP_ERR_ARG, "null shape");
  Hull h;
  if (s->type == CP_SHAPE_SPHERE) {
    if (s->radius < 0) return fail(CP_ERR_ARG, "The sphere radius cannot be negative.");
  } else if (s->type != CP_SHAPE_PLANE) {
    int st = build_hull(*s, h);
    if (st) return st;
  }
  s->bounding_sphere_radius = shape_bsr(*s, &h);
  return CP_OK;
}

int cp_body_setup(const cp_shape_desc* shapes, int32_t num_shapes, const cp_body_shape* body_shapes, int32_t num_body_shapes,
                  cp_body_desc* bodies, int32_t num_bodies) {
  if ((!bodies && num_bodies > 0) || num_bodies < 0 || num_shapes < 0 || (num_shapes > 0 && !shapes) || num_body_shapes < 0)
    return fail(CP_ERR_ARG, "bad arguments");
  std::vector<Hull> hulls(num_shapes);
  std::vector<char> has_hull(num_shapes, 0);
  for (int k = 0; k < num_bodies; k++) {
    cp_body_desc& b = bodies[k];
    if (b.shape >= num_shapes) return fail(CP_ERR_ARG, "body %d: shape %d out of range", k, b.shape);
    if (!extras_valid(b, num_shapes, body_shapes, num_body_shapes))
      return fail(CP_ERR_ARG, "body %d: extra shapes [%d, %d) outside the table of %d, or naming a missing shape", k,
                  b.extra_shapes_first, b.extra_shapes_first + b.extra_shapes_count, num_body_shapes);
    std::memcpy(b.previous_position, b.position, 12);
    std::memcpy(b.previous_quaternion, b.quaternion, 16);
    std::memcpy(b.interpolated_position, b.position, 12);
    std::memcpy(b.interpolated_quaternion, b.quaternion, 16);
    b.inv_mass = b.mass > 0 ? 1.0 / b.mass : 0;
    if (b.type < 0) b.type = b.mass <= 0.0 ? CP_BODY_STATIC : CP_BODY_DYNAMIC;
    h3 he = mk3(0, 0, 0);
    hq q; q.x = b.quaternion[0]; q.y = b.quaternion[1]; q.z = b.quaternion[2]; q.w = b.quaternion[3];
    h3 mn = mk3(0, 0, 0), mx = mk3(0, 0, 0);
    // addShape for each shape in Body.shapes order; the last
    // updateMassProperties (AABB of all shapes, the first copied and the
    // others extended in, rigid_body.dart:415-447) and updateBoundingRadius
    // see them all
    const int nsh = b.shape >= 0 ? 1 + b.extra_shapes_count : 0;
    double radius = 0;
    for (int sl = 0; sl < nsh; sl++) {
      const int si = sl == 0 ? b.shape : body_shapes[b.extra_shapes_first + sl - 1].shape;
      const float* offp = sl == 0 ? b.shape_offset : body_shapes[b.extra_shapes_first + sl - 1].offset;
      const float* orp = sl == 0 ? b.shape_orientation : body_shapes[b.extra_shapes_first + sl - 1].orientation;
      const cp_shape_desc& sd = shapes[si];
      if (sd.type != CP_SHAPE_SPHERE && sd.type != CP_SHAPE_PLANE && !has_hull[si]) {
        int st = build_hull(sd, hulls[si]);
        if (st) return st;
        has_hull[si] = 1;
      }
      h3 off = mk3(offp[0], offp[1], offp[2]);
      h3 pos = mk3(b.position[0], b.position[1], b.position[2]);
      hq so; so.x = orp[0]; so.y = orp[1]; so.z = orp[2]; so.w = orp[3];
      h3 wpos = add3(qrot(q, off), pos);
      hq wq = qmul(q, so);
      h3 smn, smx;
      shape_aabb(sd, &hulls[si], wpos, wq, smn, smx);
      if (sl == 0) {
        mn = smn;
        mx = smx;
      } else {  // AABB.extend (aabb.dart:121-128)
        mn = mk3(dart_min(mn.x, smn.x), dart_min(mn.y, smn.y), dart_min(mn.z, smn.z));
        mx = mk3(dart_max(mx.x, smx.x), dart_max(mx.y, smx.y), dart_max(mx.z, smx.z));
      }
      double r = shape_bsr(sd, &hulls[si]);
      double o = len3(off);
      if (o + r > radius) radius = o + r;
    }
    if (nsh) he = mk3(((double)mx.x - mn.x) / 2, ((double)mx.y - mn.y) / 2, ((double)mx.z - mn.z) / 2);
    b.bounding_radius = radius;
    b.aabb_lower[0] = mn.x; b.aabb_lower[1] = mn.y; b.aabb_lower[2] = mn.z;
    b.aabb_upper[0] = mx.x; b.aabb_upper[1] = mx.y; b.aabb_upper[2] = mx.z;
    // Box.calculateInertia (box.dart:88-94)
    double m = b.mass;
    float Ix = (float)(1.0 / 12.0 * m * (2 * (double)he.y * 2 * he.y + 2 * (double)he.z * 2 * he.z));
    float Iy = (float)(1.0 / 12.0 * m * (2 * (double)he.x * 2 * he.x + 2 * (double)he.z * 2 * he.z));
    float Iz = (float)(1.0 / 12.0 * m * (2 * (double)he.y * 2 * he.y + 2 * (double)he.x * 2 * he.x));
    bool fixed = b.fixed_rotation != 0;
    h3 inv = mk3(Ix > 0 && !fixed ? 1.0 / Ix : 0, Iy > 0 && !fixed ? 1.0 / Iy : 0, Iz > 0 && !fixed ? 1.0 / Iz : 0);
    b.inv_inertia[0] = inv.x; b.inv_inertia[1] = inv.y; b.inv_inertia[2] = inv.z;
    inertia_world(q, inv, b.inv_inertia_world);
    b.aabb_needs_update = 1;
  }
  return CP_OK;
}

int cp_create(const cp_config* cfg, cp_ctx** out) {
  if (!out) return fail(CP_ERR_ARG, "null out");
  *out = nullptr;
  int dev = cfg ? cfg->device : 0;
  int ndev = 0;
  CUDA_TRY(cudaGetDeviceCount(&ndev));
  if (dev < 0 || dev >= ndev) return fail(CP_ERR_ARG, "no CUDA device %d (%d present)", dev, ndev);
  CUDA_TRY(cudaSetDevice(dev));
  cp_ctx* c = new cp_ctx();
  c->device = dev;
  cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&c->d_queue, 2 * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&c->d_one, sizeof(int));
  if (e == cudaSuccess) e = cudaHostAlloc((void**)&c->h_plain, sizeof(cp_ctx::PlainStage), cudaHostAllocDefault);
  if (e == cudaSuccess) e = cudaMalloc(&c->d_one_group, 2 * sizeof(int));
  if (e == cudaSuccess) {
    int og[2] = {0, 1};
    e = cudaMemcpy(c->d_one_group, og, sizeof(og), cudaMemcpyHostToDevice);
  }
  if (e == cudaSuccess) e = cudaEventCreate(&c->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&c->ev1);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) {
    delete c;
    return fail(CP_ERR_CUDA, "context setup: %s", cudaGetErrorString(e));
  }
  for (int v = 0; v < cpk_num_variants(); v++) {
    int bp = 0, bs = 0;
    cpk_max_resident_blocks(v, &bp, &bs);
    c->blocks_pre.push_back(std::max(1, bp));
    c->blocks_solve.push_back(std::max(1, bs));
  }
  *out = c;
  return CP_OK;
}

int cp_destroy(cp_ctx* c) {
  if (!c) return CP_OK;
  cudaSetDevice(c->device);
  if (c->graph) cudaGraphExecDestroy(c->graph);
  for (auto& w : c->worlds) {
    if (w.state) dev_free(c, w.state, w.pooled);
    if (w.scratch) dev_free(c, w.scratch, w.pooled);
    if (w.pool) cudaFree(w.pool);
  }
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->pool) cudaMemPoolDestroy(c->pool);
  if (c->d_worlds) cudaFree(c->d_worlds);
  if (c->d_ids) cudaFree(c->d_ids);
  if (c->d_status) cudaFree(c->d_status);
  if (c->d_queue) cudaFree(c->d_queue);
  if (c->d_one) cudaFree(c->d_one);
  if (c->h_plain) cudaFreeHost(c->h_plain);
  if (c->d_one_group) cudaFree(c->d_one_group);
  if (c->d_gstart) cudaFree(c->d_gstart);
  if (c->d_io_ids) cudaFree(c->d_io_ids);
  if (c->d_io_first) cudaFree(c->d_io_first);
  if (c->d_io) cudaFree(c->d_io);
  if (c->d_states) cudaFree(c->d_states);
  if (c->d_rays) cudaFree(c->d_rays);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return CP_OK;
}

}  // extern "C"

namespace cpi {

int prepare_world(const cp_world_desc* d, PreparedWorld& out) {
  if (!d) return fail(CP_ERR_ARG, "null world descriptor");
  if (d->num_bodies < 0 || d->num_shapes < 0 || d->num_materials < 0 || d->num_contact_materials < 0 || d->num_constraints < 0)
    return fail(CP_ERR_ARG, "negative count");
  if ((d->num_bodies && !d->bodies) || (d->num_shapes && !d->shapes) || (d->num_materials && !d->materials) ||
      (d->num_contact_materials && !d->contact_materials) || (d->num_constraints && !d->constraints))
    return fail(CP_ERR_ARG, "null array");
  if (d->broadphase < CP_BROAD_NAIVE || d->broadphase > CP_BROAD_GRID) return fail(CP_ERR_ARG, "unknown broadphase %d", d->broadphase);
  if (d->solver_iterations < 0) return fail(CP_ERR_ARG, "negative solver iterations");
  const int nb = d->num_bodies, ns = d->num_shapes, nm = d->num_materials;
  for (int i = 0; i < nb; i++) {
    const cp_body_desc& b = d->bodies[i];
    if (b.shape < -1 || b.shape >= ns) return fail(CP_ERR_ARG, "body %d: shape %d out of range", i, b.shape);
    if (b.material < -1 || b.material >= nm) return fail(CP_ERR_ARG, "body %d: material out of range", i);
    if (b.type < 0 || b.type > 2) return fail(CP_ERR_ARG, "body %d: type %d (run cp_body_setup first)", i, b.type);
    if (!extras_valid(b, ns, d->body_shapes, d->num_body_shapes))
      return fail(CP_ERR_ARG, "body %d: extra shapes outside the body_shapes table or naming a missing shape", i);
  }
  if (d->num_body_shapes < 0 || (d->num_body_shapes > 0 && !d->body_shapes)) return fail(CP_ERR_ARG, "bad body_shapes table");
  // shapes and hulls
  std::vector<DShape> shapes(ns);
  std::vector<DHull> hulls;
  std::vector<DFace> faces;
  std::vector<float> hverts, hedges;
  std::vector<double> hvd, hed;
  std::vector<int> hfi, hconn, hcanon;
  std::vector<char> on_f;
  for (int s = 0; s < ns; s++) {
    const cp_shape_desc& sd = d->shapes[s];
    if (sd.material < -1 || sd.material >= nm) return fail(CP_ERR_ARG, "shape %d: material out of range", s);
    DShape& o = shapes[s];
    std::memset(&o, 0, sizeof(o));
    o.type = sd.type; o.group = sd.collision_filter_group; o.mask = sd.collision_filter_mask;
    o.response = sd.collision_response != 0; o.material = sd.material; o.hull = -1;
    o.radius = sd.radius;
    o.he[0] = sd.half_extents[0]; o.he[1] = sd.half_extents[1]; o.he[2] = sd.half_extents[2];
    Hull h;
    if (sd.type == CP_SHAPE_SPHERE || sd.type == CP_SHAPE_PLANE) {
      if (sd.type == CP_SHAPE_SPHERE && sd.radius < 0) return fail(CP_ERR_ARG, "The sphere radius cannot be negative.");
      o.bsr = shape_bsr(sd, nullptr);
      continue;
    }
    if (sd.type < CP_SHAPE_BOX || sd.type > CP_SHAPE_SIZED_PLANE) return fail(CP_ERR_UNSUPPORTED, "shape type %d", sd.type);
    int st = build_hull(sd, h);
    if (st) return st;
    o.bsr = shape_bsr(sd, &h);
    DHull dh;
    std::memset(&dh, 0, sizeof(dh));
    dh.v0 = (int)hverts.size() / 4; dh.nv = (int)h.verts.size();
    dh.f0 = (int)faces.size(); dh.nf = (int)h.faces.size();
    dh.e0 = (int)hedges.size() / 4; dh.ne = (int)h.edges.size();
    dh.has_axes = h.has_axes;
    dh.is_box = sd.type == CP_SHAPE_BOX;
    dh.he[0] = sd.half_extents[0]; dh.he[1] = sd.half_extents[1]; dh.he[2] = sd.half_extents[2];
    for (auto& v : h.verts) {
      hverts.push_back(v.x); hverts.push_back(v.y); hverts.push_back(v.z); hverts.push_back(0.f);
      hvd.push_back(v.x); hvd.push_back(v.y); hvd.push_back(v.z); hvd.push_back(0.0);
    }
    for (auto& e : h.edges) {
      hedges.push_back(e.x); hedges.push_back(e.y); hedges.push_back(e.z); hedges.push_back(0.f);
      hed.push_back(e.x); hed.push_back(e.y); hed.push_back(e.z); hed.push_back(0.0);
    }
    // canonical entries: those whose exact negation does not occur earlier
    auto negated = [](const h3& a, const h3& b) { return a.x == -b.x && a.y == -b.y && a.z == -b.z; };
    std::vector<int> fcanon(h.faces.size());
    dh.cf0 = (int)hcanon.size();
    for (size_t f = 0; f < h.faces.size(); f++) {
      fcanon[f] = (int)f;
      for (size_t g = 0; g < f; g++)
        if (fcanon[g] == (int)g && negated(h.normals[f], h.normals[g])) { fcanon[f] = (int)g; break; }
      if (fcanon[f] == (int)f) hcanon.push_back((int)f);
    }
    dh.ncf = (int)hcanon.size() - dh.cf0;
    dh.ce0 = (int)hcanon.size();
    for (size_t e = 0; e < h.edges.size(); e++) {
      bool dup = false;
      for (size_t g = 0; g < e && !dup; g++) dup = negated(h.edges[e], h.edges[g]);
      if (!dup) hcanon.push_back((int)e);
    }
    dh.nce = (int)hcanon.size() - dh.ce0;
    for (size_t f = 0; f < h.faces.size(); f++) {
      DFace F;
      std::memset(&F, 0, sizeof(F));
      F.i0 = (int)hfi.size(); F.n = (int)h.faces[f].size();
      for (int vi : h.faces[f]) hfi.push_back(vi);
      // connected faces of face f in the order clipFaceAgainstHull builds them
      // (convex_polyhedron.dart:457-473): every other face sharing a vertex
      // with f, ascending (each joins at its first shared vertex)
      F.c0 = (int)hconn.size();
      on_f.assign(h.verts.size(), 0);
      for (int vi : h.faces[f]) on_f[vi] = 1;
      for (size_t i = 0; i < h.faces.size(); i++) {
        if (i == f) continue;
        for (int vj : h.faces[i])
          if (on_f[vj]) {
            hconn.push_back((int)i);
            break;
          }
      }
      F.nc = (int)hconn.size() - F.c0;
      F.normal[0] = h.normals[f].x; F.normal[1] = h.normals[f].y; F.normal[2] = h.normals[f].z;
      F.dnormal[0] = h.normals[f].x; F.dnormal[1] = h.normals[f].y; F.dnormal[2] = h.normals[f].z;
      F.plane_const = -dot3(h.normals[f], h.verts[h.faces[f][0]]);  // getPlaneConstantOfFace
      F.canon = fcanon[f];
      faces.push_back(F);
    }
    o.hull = (int)hulls.size();
    hulls.push_back(dh);
  }
  // materials and contact material table ([0] = world default)
  std::vector<DMaterial> mats(nm);
  for (int i = 0; i < nm; i++) { mats[i].friction = d->materials[i].friction; mats[i].restitution = d->materials[i].restitution; }
  std::vector<DContactMaterial> cms(1 + d->num_contact_materials);
  auto cmOf = [](const cp_contact_material& m) {
    DContactMaterial o;
    std::memset(&o, 0, sizeof(o));
    o.friction = m.friction; o.restitution = m.restitution;
    o.cs = m.contact_stiffness; o.cr = m.contact_relaxation; o.fs = m.friction_stiffness; o.fr = m.friction_relaxation;
    return o;
  };
  cms[0] = cmOf(d->default_contact_material);
  std::vector<int> cmt((size_t)std::max(1, nm * nm), -1);
  for (int i = 0; i < d->num_contact_materials; i++) {
    const cp_contact_material& m = d->contact_materials[i];
    if (m.material_a < 0 || m.material_a >= nm || m.material_b < 0 || m.material_b >= nm) return fail(CP_ERR_ARG, "contact material %d: bad materials", i);
    cms[1 + i] = cmOf(m);
    cmt[m.material_a * nm + m.material_b] = 1 + i;  // TupleDictionary: last set wins
    cmt[m.material_b * nm + m.material_a] = 1 + i;
  }
  // constraints
  std::vector<DConstraint> cons(d->num_constraints);
  std::vector<int> nocollide;
  int con_rows = 0;
  const double cos_max = std::cos(M_PI / 2);  // RotationalEquation default maxAngle (rotational_equation.dart:203)
  for (int k = 0; k < d->num_constraints; k++) {
    const cp_constraint_desc& cd = d->constraints[k];
    if (cd.body_a < 0 || cd.body_a >= nb || cd.body_b < 0 || cd.body_b >= nb) return fail(CP_ERR_ARG, "constraint %d: bad bodies", k);
    if (cd.type < CP_CON_POINT_TO_POINT || cd.type > CP_CON_SPRING) return fail(CP_ERR_ARG, "constraint %d: type", k);
    DConstraint& o = cons[k];
    std::memset(&o, 0, sizeof(o));
    o.type = cd.type; o.a = cd.body_a; o.b = cd.body_b; o.collide = cd.collide_connected != 0;
    o.row0 = con_rows;
    static const int kRows[] = {3, 6, 1, 6, 5, 1};  // equations per constraint type
    o.nrows = kRows[cd.type];
    o.motor = cd.motor_enabled != 0;
    con_rows += o.nrows;
    h3 pa = mk3(cd.pivot_a[0], cd.pivot_a[1], cd.pivot_a[2]), pb = mk3(cd.pivot_b[0], cd.pivot_b[1], cd.pivot_b[2]);
    o.piv_a[0] = pa.x; o.piv_a[1] = pa.y; o.piv_a[2] = pa.z;
    o.piv_b[0] = pb.x; o.piv_b[1] = pb.y; o.piv_b[2] = pb.z;
    if (cd.type == CP_CON_HINGE) {  // HingeConstraint normalizes its axes (hinge_constraint.dart:172-176)
      h3 aa = norm3(mk3(cd.axis_a[0], cd.axis_a[1], cd.axis_a[2])), ab = norm3(mk3(cd.axis_b[0], cd.axis_b[1], cd.axis_b[2]));
      o.axis_a[0] = aa.x; o.axis_a[1] = aa.y; o.axis_a[2] = aa.z;
      o.axis_b[0] = ab.x; o.axis_b[1] = ab.y; o.axis_b[2] = ab.z;
    }
    if (cd.type == CP_CON_CONE_TWIST) {  // the axes are cloned as given (cone_twist_constraint.dart:44-45)
      for (int e = 0; e < 3; e++) { o.axis_a[e] = cd.axis_a[e]; o.axis_b[e] = cd.axis_b[e]; }
    }
    if (cd.type == CP_CON_LOCK)
      for (int v = 0; v < 6; v++)
        for (int e = 0; e < 3; e++) o.loc[v][e] = cd.lock_axes[v][e];
    if (cd.type == CP_CON_DISTANCE || cd.type == CP_CON_SPRING) {
      const float* A = d->bodies[cd.body_a].position;
      const float* B = d->bodies[cd.body_b].position;
      double px = B[0], py = B[1], pz = B[2];
      o.distance = cd.distance >= 0 ? cd.distance
                                     : std::sqrt((px - A[0]) * (px - A[0]) + (py - A[1]) * (py - A[1]) + (pz - A[2]) * (pz - A[2]));
    }
    o.max_force = cd.max_force;
    o.motor_target = cd.motor_target_velocity;
    o.motor_max_force = cd.motor_max_force > 0 ? cd.motor_max_force : cd.max_force;
    spook(cd.spook_stiffness, cd.spook_relaxation, cd.spook_time_step, o.sa, o.sb, o.seps);
    // RotationalEquation / ConeEquation: cos(maxAngle) (rotational_equation.dart:51,
    // cone_equation.dart:46); a cone-twist's cone and twist rows take its angles
    o.cos_rot[0] = cd.type == CP_CON_CONE_TWIST ? std::cos(cd.angle) : cos_max;
    o.cos_rot[1] = cd.type == CP_CON_CONE_TWIST ? std::cos(cd.twist_angle) : cos_max;
    o.first_id = cd.first_equation_id;
    // SplitSolver: the equations of a constraint between two static bodies
    // belong to no island; the reference never solves them and leaves their
    // rows as they were, which this library does not keep
    if (d->solver == CP_SOLVER_SPLIT && d->bodies[cd.body_a].type == CP_BODY_STATIC && d->bodies[cd.body_b].type == CP_BODY_STATIC)
      return fail(CP_ERR_UNSUPPORTED, "constraint %d joins two static bodies under the SplitSolver", k);
    if (!o.collide) { nocollide.push_back(cd.body_a); nocollide.push_back(cd.body_b); }
  }
  // bodies
  std::vector<DBody> bodies(nb);
  WorldRec w;
  w.nb = nb; w.nshapes = ns; w.nmat = nm; w.ncm = (int)cms.size(); w.ncons = d->num_constraints; w.ncon_rows = con_rows;
  w.broadphase = d->broadphase;
  w.lin_damp.resize(nb); w.ang_damp.resize(nb); w.body_shape.resize(nb); w.body_xs0.resize(nb);
  for (int i = 0; i < nb; i++) {
    body_to_device(d->bodies[i], bodies[i]);
    w.lin_damp[i] = d->bodies[i].linear_damping;
    w.ang_damp[i] = d->bodies[i].angular_damping;
    w.body_shape[i] = d->bodies[i].shape;
    w.body_xs0[i] = d->bodies[i].extra_shapes_first;
    w.compound = w.compound || d->bodies[i].extra_shapes_count > 0;
  }
  w.body_shapes.assign(d->body_shapes, d->body_shapes ? d->body_shapes + d->num_body_shapes : d->body_shapes);
  std::vector<DBodyShape> bshapes(w.body_shapes.size());
  for (size_t k = 0; k < bshapes.size(); k++) {
    std::memset(&bshapes[k], 0, sizeof(DBodyShape));
    bshapes[k].shape = w.body_shapes[k].shape;
    std::memcpy(bshapes[k].off, w.body_shapes[k].offset, 12);
    std::memcpy(bshapes[k].quat, w.body_shapes[k].orientation, 16);
  }
  w.cms = cms;
  // params
  DWorldParams P;
  std::memset(&P, 0, sizeof(P));
  P.time = d->time; P.tolerance = d->solver_tolerance; P.dt_cached = -1; P.stepnumber = d->stepnumber;
  P.step_limit = LLONG_MAX;
  for (int k = 0; k < 3; k++) {
    P.gravity[k] = d->gravity[k]; P.fgrav[k] = d->friction_gravity[k];
    P.grid_min[k] = d->grid_aabb_min[k]; P.grid_max[k] = d->grid_aabb_max[k];
  }
  P.nb = nb; P.nshapes = ns; P.nmat = nm; P.ncm = (int)cms.size();
  P.ncons = d->num_constraints; P.ncon_rows = con_rows; P.iterations = d->solver_iterations; P.broadphase = d->broadphase;
  P.sap_axis = d->sap_axis; P.use_bb = d->use_bounding_boxes != 0; P.allow_sleep = d->allow_sleep != 0; P.qn_skip = d->quat_normalize_skip;
  P.qn_fast = d->quat_normalize_fast != 0; P.has_fgrav = d->has_friction_gravity != 0;
  P.grid_nx = d->grid_n[0]; P.grid_ny = d->grid_n[1]; P.grid_nz = d->grid_n[2];
  P.n_nocollide = (int)nocollide.size() / 2;
  P.fric_reduction = d->enable_friction_reduction != 0;
  w.n_nocollide = P.n_nocollide;
  if (d->sap_axis < 0 || d->sap_axis > 2) return fail(CP_ERR_ARG, "sap_axis %d", d->sap_axis);
  if (d->broadphase == CP_BROAD_GRID) {
    if (P.grid_nx <= 0 || P.grid_ny <= 0 || P.grid_nz <= 0) return fail(CP_ERR_ARG, "GridBroadphase: Each dimension's n must be >0");
    if (P.grid_nx + P.grid_ny + P.grid_nz > 3 * 4096 || (long long)P.grid_nx * P.grid_ny * P.grid_nz > (1 << 26))
      return fail(CP_ERR_UNSUPPORTED, "grid too large");
    w.nbins = P.grid_nx * P.grid_ny * P.grid_nz;
  }
  P.nbins = w.nbins;
  // capacities (grown on overflow)
  long long allpairs = (long long)nb * (nb - 1) / 2;
  w.pairs_cap = (int)std::max<long long>(16, std::min<long long>(allpairs, 4LL * nb + 64));
  w.contacts_cap = 2 * w.pairs_cap + 64;
  w.rows_cap = 3 * w.contacts_cap + con_rows + 64;
  w.bins_cap = 4 * nb + (d->broadphase == CP_BROAD_GRID ? w.nbins : 0) + 64;
  w.jobs_cap = w.compound ? 4 * w.pairs_cap : 0;
  P.pairs_cap = w.pairs_cap; P.contacts_cap = w.contacts_cap; P.rows_cap = w.rows_cap; P.bins_cap = w.bins_cap;
  P.compound = w.compound;
  P.jobs_cap = w.jobs_cap;
  if (d->solver != CP_SOLVER_GS && d->solver != CP_SOLVER_SPLIT) return fail(CP_ERR_ARG, "solver %d", d->solver);
  w.split = d->solver == CP_SOLVER_SPLIT;
  w.iterations = d->solver_iterations;
  P.split = w.split;
  P.id_counter = d->equation_id_counter;
  P.pool_c = P.pool_f = 0;
  // state allocation
  Layout L;
  size_t o_P = L.take(sizeof(DWorldParams));
  size_t o_b = L.take(sizeof(DBody) * (nb + 1));
  size_t o_s = L.take(sizeof(DShape) * (ns + 1));
  size_t o_h = L.take(sizeof(DHull) * (hulls.size() + 1));
  size_t o_f = L.take(sizeof(DFace) * (faces.size() + 1));
  size_t o_hv = L.take(sizeof(float) * (hverts.size() + 4));
  size_t o_he = L.take(sizeof(float) * (hedges.size() + 4));
  size_t o_hfi = L.take(sizeof(int) * (hfi.size() + 1));
  size_t o_hvd = L.take(sizeof(double) * (hvd.size() + 4));
  size_t o_hed = L.take(sizeof(double) * (hed.size() + 4));
  size_t o_hcn = L.take(sizeof(int) * (hcanon.size() + 1));
  size_t o_hc = L.take(sizeof(int) * (hconn.size() + 1));
  size_t o_m = L.take(sizeof(DMaterial) * (nm + 1));
  size_t o_ct = L.take(sizeof(int) * cmt.size());
  size_t o_cm = L.take(sizeof(DContactMaterial) * cms.size());
  size_t o_cn = L.take(sizeof(DConstraint) * (cons.size() + 1));
  size_t o_nc = L.take(sizeof(int) * (nocollide.size() + 2));
  size_t o_dp = L.take(sizeof(double) * (2 * nb + 2));
  size_t o_so = L.take(sizeof(int) * (nb + 1));
  size_t o_bsh = L.take(sizeof(DBodyShape) * (bshapes.size() + 1));
  std::vector<char> host(L.off, 0);
  std::memcpy(&host[o_P], &P, sizeof(P));
  if (nb) std::memcpy(&host[o_b], bodies.data(), sizeof(DBody) * nb);
  if (ns) std::memcpy(&host[o_s], shapes.data(), sizeof(DShape) * ns);
  if (!hulls.empty()) std::memcpy(&host[o_h], hulls.data(), sizeof(DHull) * hulls.size());
  if (!faces.empty()) std::memcpy(&host[o_f], faces.data(), sizeof(DFace) * faces.size());
  if (!hverts.empty()) std::memcpy(&host[o_hv], hverts.data(), sizeof(float) * hverts.size());
  if (!hedges.empty()) std::memcpy(&host[o_he], hedges.data(), sizeof(float) * hedges.size());
  if (!hfi.empty()) std::memcpy(&host[o_hfi], hfi.data(), sizeof(int) * hfi.size());
  if (!hvd.empty()) std::memcpy(&host[o_hvd], hvd.data(), sizeof(double) * hvd.size());
  if (!hed.empty()) std::memcpy(&host[o_hed], hed.data(), sizeof(double) * hed.size());
  if (!hcanon.empty()) std::memcpy(&host[o_hcn], hcanon.data(), sizeof(int) * hcanon.size());
  if (!hconn.empty()) std::memcpy(&host[o_hc], hconn.data(), sizeof(int) * hconn.size());
  if (nm) std::memcpy(&host[o_m], mats.data(), sizeof(DMaterial) * nm);
  std::memcpy(&host[o_ct], cmt.data(), sizeof(int) * cmt.size());
  std::memcpy(&host[o_cm], cms.data(), sizeof(DContactMaterial) * cms.size());
  if (!cons.empty()) std::memcpy(&host[o_cn], cons.data(), sizeof(DConstraint) * cons.size());
  if (!nocollide.empty()) std::memcpy(&host[o_nc], nocollide.data(), sizeof(int) * nocollide.size());
  std::vector<int> order(nb);
  for (int i = 0; i < nb; i++) {
    order[i] = d->sap_axis_list ? d->sap_axis_list[i] : i;
    if (order[i] < 0 || order[i] >= nb) return fail(CP_ERR_ARG, "sap_axis_list[%d] out of range", i);
  }
  if (nb) std::memcpy(&host[o_so], order.data(), sizeof(int) * nb);
  if (!bshapes.empty()) std::memcpy(&host[o_bsh], bshapes.data(), sizeof(DBodyShape) * bshapes.size());
  w.state_bytes = L.off;
  w.scratch_bytes = scratch_layout(w, nullptr);
  out.off = StateOffsets{o_P, o_b, o_s, o_h, o_f, o_hv, o_he, o_hfi, o_hvd, o_hed, o_hcn, o_hc,
                         o_m, o_ct, o_cm, o_cn, o_nc, o_dp, o_so, o_bsh};
  out.w = std::move(w);
  out.host = std::move(host);
  return CP_OK;
}

int commit_world(cp_ctx* c, PreparedWorld& p, int* world_id) {
  WorldRec& w = p.w;
  const StateOffsets& o = p.off;
  int st = dev_alloc(c, (void**)&w.state, w.state_bytes, "world state");
  if (st) return st;
  w.pooled = c->pool != nullptr;
  cudaError_t e = cudaMemcpyAsync(w.state, p.host.data(), w.state_bytes, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) {
    dev_free(c, w.state, w.pooled);
    return fail(CP_ERR_CUDA, "world upload: %s", cudaGetErrorString(e));
  }
  char* base = w.state;
  DWorld& dw = w.dw;
  std::memset(&dw, 0, sizeof(dw));
  dw.P = (DWorldParams*)(base + o.P);
  dw.bodies = (DBody*)(base + o.bodies);
  dw.shapes = (DShape*)(base + o.shapes);
  dw.hulls = (DHull*)(base + o.hulls);
  dw.faces = (DFace*)(base + o.faces);
  dw.hverts = (float*)(base + o.hverts);
  dw.hedges = (float*)(base + o.hedges);
  dw.haxes = nullptr;
  dw.hfi = (int*)(base + o.hfi);
  dw.hvd = (double*)(base + o.hvd);
  dw.hed = (double*)(base + o.hed);
  dw.hcanon = (int*)(base + o.hcanon);
  dw.hconn = (int*)(base + o.hconn);
  dw.mats = (DMaterial*)(base + o.mats);
  dw.cm_table = (int*)(base + o.cm_table);
  dw.cms = (DContactMaterial*)(base + o.cms);
  dw.cons = (DConstraint*)(base + o.cons);
  dw.nocollide = (int*)(base + o.nocollide);
  dw.dpow = (double*)(base + o.dpow);
  dw.sap_order = (int*)(base + o.sap_order);
  dw.bshapes = (DBodyShape*)(base + o.bshapes);
  st = alloc_scratch(c, w);
  if (st) { dev_free(c, w.state, w.pooled); w.state = nullptr; return st; }
  w.live = true;
  int id = -1;
  for (size_t i = 0; i < c->worlds.size(); i++)
    if (!c->worlds[i].live) { id = (int)i; break; }
  if (id < 0) { id = (int)c->worlds.size(); c->worlds.emplace_back(); }
  c->worlds[id] = std::move(w);
  p.host.clear();
  st = upload_world_entry(c, id);
  if (st) return st;
  *world_id = id;
  return CP_OK;
}

int destroy_world(cp_ctx* c, int id) {
  WorldRec& w = c->worlds[id];
  if (!w.pooled) cudaStreamSynchronize(c->stream);
  if (w.state) dev_free(c, w.state, w.pooled);
  if (w.scratch) dev_free(c, w.scratch, w.pooled);
  if (w.pool) cudaFree(w.pool);
  if (w.sched_mem) dev_free(c, w.sched_mem, w.pooled);
  w = WorldRec();
  if (c->graph) { cudaGraphExecDestroy(c->graph); c->graph = nullptr; }
  return CP_OK;
}



int read_bodies(cp_ctx* c, int id, cp_body_desc* out) {
  WorldRec& w = c->worlds[id];
  if (w.nb == 0) return CP_OK;
  std::vector<DBody> b(w.nb);
  CUDA_TRY(cudaMemcpyAsync(b.data(), w.dw.bodies, sizeof(DBody) * w.nb, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  for (int i = 0; i < w.nb; i++) body_from_device(b[i], out[i]);
  return CP_OK;
}

int read_info(cp_ctx* c, int id, cp_step_info* out) {
  DWorldParams p;
  int st = read_params(c, c->worlds[id], p);
  if (st) return st;
  std::memset(out, 0, sizeof(*out));
  out->stepnumber = p.stepnumber;
  out->time = p.time;
  out->num_pairs = p.num_pairs;
  out->num_contacts = p.num_contacts;
  out->num_rows = p.num_rows;
  out->iterations = p.last_iterations;
  out->status = p.status;
  out->num_bodies = p.nb;
  out->num_levels = p.num_levels;
  out->substeps = c->worlds[id].last_substeps;
  out->accumulator = c->worlds[id].accumulator;
  return CP_OK;
}

int enable_pool(cp_ctx* c) {
  if (c->pool) return CP_OK;
  cudaMemPoolProps props;
  std::memset(&props, 0, sizeof(props));
  props.allocType = cudaMemAllocationTypePinned;
  props.handleTypes = cudaMemHandleTypeNone;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = c->device;
  CUDA_TRY(cudaMemPoolCreate(&c->pool, &props));
  // keep freed blocks for reuse instead of returning them at each synchronisation
  unsigned long long keep = ~0ull;
  CUDA_TRY(cudaMemPoolSetAttribute(c->pool, cudaMemPoolAttrReleaseThreshold, &keep));
  return CP_OK;
}

const char* last_error() { return g_err.c_str(); }

}  // namespace cpi

extern "C" {

int cp_world_create(cp_ctx* c, const cp_world_desc* d, int32_t* world_id) {
  if (!c || !d || !world_id) return fail(CP_ERR_ARG, "null argument");
  PreparedWorld p;
  int st = prepare_world(d, p);
  if (st) return st;
  std::lock_guard<std::mutex> lock(c->mu);
  cudaSetDevice(c->device);
  return commit_world(c, p, world_id);
}

int cp_world_destroy(cp_ctx* c, int32_t id) {
  int st = check_world(c, id);
  if (st) return st;
  std::lock_guard<std::mutex> lock(c->mu);
  cudaSetDevice(c->device);
  return destroy_world(c, id);
}

}  // extern "C"

namespace {

unsigned long long overlap_key(int a, int b) {
  const unsigned lo = (unsigned)std::min(a, b), hi = (unsigned)std::max(a, b);
  return ((unsigned long long)lo << 32) | hi;
}

// The events of the step just taken (World.internalStep's collide loop,
// world_class.dart:593-608, and emitContactEvents, :703-770): collide per
// contact in contact order, then the overlap keepers' diffs in key order.
int collect_events(cp_ctx* c, int id) {
  WorldRec& w = c->worlds[id];
  DWorldParams p;
  int st = read_params(c, w, p);
  if (st) return st;
  std::vector<DContact> ct(p.num_contacts);
  std::vector<int> pa(p.num_pairs), pb(p.num_pairs), pf(p.num_jobs);
  std::vector<int> jp(w.compound ? p.num_jobs : 0), js(jp.size());
  if (p.num_contacts)
    CUDA_TRY(cudaMemcpyAsync(ct.data(), w.dw.contacts, sizeof(DContact) * ct.size(), cudaMemcpyDeviceToHost, c->stream));
  if (p.num_pairs) {
    CUDA_TRY(cudaMemcpyAsync(pa.data(), w.dw.pair_a, sizeof(int) * pa.size(), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaMemcpyAsync(pb.data(), w.dw.pair_b, sizeof(int) * pb.size(), cudaMemcpyDeviceToHost, c->stream));
  }
  if (p.num_jobs) CUDA_TRY(cudaMemcpyAsync(pf.data(), w.dw.pair_flag, sizeof(int) * pf.size(), cudaMemcpyDeviceToHost, c->stream));
  if (!jp.empty()) {
    CUDA_TRY(cudaMemcpyAsync(jp.data(), w.dw.job_pair, sizeof(int) * jp.size(), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaMemcpyAsync(js.data(), w.dw.job_sh, sizeof(int) * js.size(), cudaMemcpyDeviceToHost, c->stream));
  }
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  const auto bid = [&](int i) { return w.body_ids.empty() ? i : w.body_ids[i]; };
  const auto sid = [&](int i) { return w.shape_ids.empty() ? i : w.shape_ids[i]; };
  std::vector<unsigned long long> bk, sk;
  for (size_t k = 0; k < ct.size(); k++) {
    w.event_queue.push_back(cp_event{CP_EV_COLLIDE, ct[k].bi, ct[k].bj, (int32_t)k, p.stepnumber});
    bk.push_back(overlap_key(bid(ct[k].bi), bid(ct[k].bj)));
    sk.push_back(overlap_key(sid(ct[k].si), sid(ct[k].sj)));
  }
  // shape `slot` of body i (slot 0: its first shape)
  const auto slot_shape = [&](int i, int slot) {
    return slot == 0 ? w.body_shape[i] : w.body_shapes[w.body_xs0[i] + slot - 1].shape;
  };
  for (size_t k = 0; k < pf.size(); k++)
    if (pf[k]) {  // a justTest job whose shapes overlap
      const int q = w.compound ? jp[k] : (int)k;
      const int sa = w.compound ? js[k] >> 16 : 0, sb = w.compound ? js[k] & 0xffff : 0;
      bk.push_back(overlap_key(bid(pa[q]), bid(pb[q])));
      sk.push_back(overlap_key(sid(slot_shape(pa[q], sa)), sid(slot_shape(pb[q], sb))));
    }
  // the index whose id is `v` (ids are unique)
  const auto index_of = [](const std::vector<int>& ids, unsigned v) {
    if (ids.empty()) return (int)v;
    for (size_t i = 0; i < ids.size(); i++)
      if ((unsigned)ids[i] == v) return (int)i;
    return -1;
  };
  const auto diff = [&](std::vector<unsigned long long>& now, std::vector<unsigned long long>& prev, int ev_add, int ev_rem,
                        const std::vector<int>& ids) {
    std::sort(now.begin(), now.end());
    now.erase(std::unique(now.begin(), now.end()), now.end());
    std::vector<unsigned long long> add, rem;
    std::set_difference(now.begin(), now.end(), prev.begin(), prev.end(), std::back_inserter(add));
    std::set_difference(prev.begin(), prev.end(), now.begin(), now.end(), std::back_inserter(rem));
    for (unsigned long long key : add)
      w.event_queue.push_back(cp_event{ev_add, index_of(ids, (unsigned)(key >> 32)), index_of(ids, (unsigned)key), -1, p.stepnumber});
    for (unsigned long long key : rem)
      w.event_queue.push_back(cp_event{ev_rem, index_of(ids, (unsigned)(key >> 32)), index_of(ids, (unsigned)key), -1, p.stepnumber});
    prev.swap(now);
  };
  // emitContactEvents: body pairs (begin, then end), then shape pairs
  diff(bk, w.body_keys, CP_EV_BEGIN_CONTACT, CP_EV_END_CONTACT, w.body_ids);
  diff(sk, w.shape_keys, CP_EV_BEGIN_SHAPE_CONTACT, CP_EV_END_SHAPE_CONTACT, w.shape_ids);
  return CP_OK;
}

// plain_steps, with the event feed collected after every step when it is on
int world_steps(cp_ctx* c, int id, double dt, int nsteps, double time_inc) {
  if (!c->worlds[id].events) return plain_steps(c, id, dt, nsteps, time_inc);
  for (int s = 0; s < nsteps; s++) {
    int st = plain_steps(c, id, dt, 1, time_inc);
    if (!st) st = collect_events(c, id);
    if (st) return st;
  }
  return CP_OK;
}

}  // namespace

namespace cpi {
int world_step_plain(cp_ctx* c, int id, double dt, int nsteps) { return world_steps(c, id, dt, nsteps, dt); }
}  // namespace cpi

extern "C" {

int cp_world_set_events(cp_ctx* c, int32_t id, int32_t on, const int32_t* body_ids, const int32_t* shape_ids) {
  int st = check_world(c, id);
  if (st) return st;
  std::lock_guard<std::mutex> lock(c->mu);
  cudaSetDevice(c->device);
  WorldRec& w = c->worlds[id];
  const auto check_ids = [](const int32_t* ids, int n) {
    std::vector<int> v(ids, ids + n);
    std::sort(v.begin(), v.end());
    for (int i = 0; i < n; i++)
      if (v[i] < 0 || v[i] > 0xffff || (i && v[i] == v[i - 1])) return false;
    return true;
  };
  if (on && body_ids && !check_ids(body_ids, w.nb)) return fail(CP_ERR_ARG, "body ids must be distinct and in [0, 65535]");
  if (on && shape_ids && !check_ids(shape_ids, w.nshapes)) return fail(CP_ERR_ARG, "shape ids must be distinct and in [0, 65535]");
  if (on && !body_ids && w.nb > 0x10000) return fail(CP_ERR_ARG, "more than 65536 bodies need explicit ids");
  w.events = on != 0;
  w.body_ids.assign(on && body_ids ? body_ids : nullptr, on && body_ids ? body_ids + w.nb : nullptr);
  w.shape_ids.assign(on && shape_ids ? shape_ids : nullptr, on && shape_ids ? shape_ids + w.nshapes : nullptr);
  w.body_keys.clear();
  w.shape_keys.clear();
  w.event_queue.clear();
  const int flag = w.events ? 1 : 0;
  CUDA_TRY(cudaMemcpyAsync(&w.dw.P->events, &flag, sizeof(int), cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  return CP_OK;
}

int cp_world_get_events(cp_ctx* c, int32_t id, cp_event* out, int32_t cap, int32_t* count) {
  int st = check_world(c, id);
  if (st) return st;
  if (!count) return fail(CP_ERR_ARG, "null count");
  std::lock_guard<std::mutex> lock(c->mu);
  WorldRec& w = c->worlds[id];
  *count = (int32_t)w.event_queue.size();
  if ((int)w.event_queue.size() > cap || (!out && !w.event_queue.empty()))
    return fail(CP_ERR_CAPACITY, "need room for %zu events", w.event_queue.size());
  std::copy(w.event_queue.begin(), w.event_queue.end(), out);
  w.event_queue.clear();
  return CP_OK;
}

int cp_world_step(cp_ctx* c, int32_t id, double dt, int32_t nsteps) {
  int st = check_world(c, id);
  if (st) return st;
  if (nsteps < 0 || !(dt > 0)) return fail(CP_ERR_ARG, "need dt > 0 and nsteps >= 0");
  std::lock_guard<std::mutex> lock(c->mu);
  cudaSetDevice(c->device);
  return world_steps(c, id, dt, nsteps, dt);
}

int cp_world_internal_step(cp_ctx* c, int32_t id, double dt, int32_t nsteps) {
  int st = check_world(c, id);
  if (st) return st;
  if (nsteps < 0 || !(dt > 0)) return fail(CP_ERR_ARG, "need dt > 0 and nsteps >= 0");
  std::lock_guard<std::mutex> lock(c->mu);
  cudaSetDevice(c->device);
  return world_steps(c, id, dt, nsteps, 0.0);
}

int cp_world_set_time(cp_ctx* c, int32_t id, double time, int64_t stepnumber, double accumulator) {
  int st = check_world(c, id);
  if (st) return st;
  if (stepnumber < 0 || !std::isfinite(time) || !std::isfinite(accumulator))
    return fail(CP_ERR_ARG, "need a finite time and accumulator and stepnumber >= 0");
  std::lock_guard<std::mutex> lock(c->mu);
  cudaSetDevice(c->device);
  WorldRec& w = c->worlds[id];
  const long long sn = stepnumber;
  CUDA_TRY(cudaMemcpyAsync(&w.dw.P->time, &time, sizeof(double), cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(cudaMemcpyAsync(&w.dw.P->stepnumber, &sn, sizeof(long long), cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  w.accumulator = accumulator;
  return CP_OK;
}

// World.step(dt, timeSinceLastCalled, maxSubSteps), world_class.dart:400-430
int cp_world_step_interpolated(cp_ctx* c, int32_t id, double dt, double since, int32_t max_sub_steps, int32_t* substeps) {
  int st = check_world(c, id);
  if (st) return st;
  if (!(dt > 0) || max_sub_steps < 0 || !std::isfinite(since))
    return fail(CP_ERR_ARG, "need dt > 0, a finite timeSinceLastCalled and maxSubSteps >= 0");
  std::lock_guard<std::mutex> lock(c->mu);
  cudaSetDevice(c->device);
  WorldRec& w = c->worlds[id];
  w.accumulator += since;
  const auto t0 = std::chrono::steady_clock::now();
  int n = 0;
  while (w.accumulator >= dt && n < max_sub_steps) {
    st = world_steps(c, id, dt, 1, 0.0);  // returns with the stream synchronised
    if (st) return st;
    w.accumulator -= dt;
    n++;
    // the reference bails out once the sub-steps took longer than dt (its
    // performance.now() is in milliseconds)
    const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (ms > dt * 1000) break;
  }
  // Dart's double %: the remainder with the divisor's magnitude, never negative
  double r = std::fmod(w.accumulator, dt);
  if (r < 0) r += dt;
  if (r == 0) r = 0.0;
  w.accumulator = r;
  w.last_substeps = n;
  if (substeps) *substeps = n;
  CUDA_TRY(cpk_interpolate(c->d_worlds + id, w.nb, w.accumulator / dt, c->stream));
  c->launches += 1;
  DWorldParams p;
  st = read_params(c, w, p);
  if (st) return st;
  const double t1 = p.time + since;
  CUDA_TRY(cudaMemcpyAsync(&w.dw.P->time, &t1, sizeof(double), cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  return CP_OK;
}

}  // extern "C"

namespace {

// ensure_dt without a host allocation: the damping powers go up in chunks
// through a stack buffer (each chunk copy is synchronous, so the buffer can
// be reused), and the contact materials are updated in place.
int ensure_dt_static(cp_ctx* c, WorldRec& w, double dt) {
  if (w.dt_cached == dt) return CP_OK;
  double buf[512];
  for (int i0 = 0; i0 < w.nb; i0 += 256) {
    const int n = std::min(256, w.nb - i0);
    for (int i = 0; i < n; i++) {
      buf[2 * i] = std::pow(1.0 - w.lin_damp[i0 + i], dt);
      buf[2 * i + 1] = std::pow(1.0 - w.ang_damp[i0 + i], dt);
    }
    CUDA_TRY(cudaMemcpyAsync(w.dw.dpow + 2 * i0, buf, sizeof(double) * 2 * n, cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
  }
  for (auto& m : w.cms) {
    spook(m.cs, m.cr, dt, m.ca, m.cb, m.ceps);
    spook(m.fs, m.fr, dt, m.fa, m.fb, m.feps);
  }
  CUDA_TRY(cudaMemcpyAsync(w.dw.cms, w.cms.data(), sizeof(DContactMaterial) * w.cms.size(), cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  w.dt_cached = dt;
  return CP_OK;
}

}  // namespace

extern "C" {

// Steps a world with the static step scratch of cp_step.cu in place of the
// world's own scratch.  The static array holds, from its start: a one-entry
// world table (this world's descriptor with its scratch pointers moved into
// the array), the work list {0} and group bounds {0, 1}, then the scratch.
int cp_world_step_static(cp_ctx* c, int32_t id, double dt, int32_t nsteps) {
  int st = check_world(c, id);
  if (st) return st;
  if (nsteps < 0 || !(dt > 0)) return fail(CP_ERR_ARG, "need dt > 0 and nsteps >= 0");
  std::lock_guard<std::mutex> lock(c->mu);
  cudaSetDevice(c->device);
  void* arena = nullptr;
  size_t arena_bytes = 0;
  CUDA_TRY(cpk_static_scratch(c->device, &arena, &arena_bytes));
  WorldRec& w = c->worlds[id];
  Layout L;
  const size_t o_rec = L.take(sizeof(DWorld));
  const size_t o_ids = L.take(3 * sizeof(int));
  const size_t o_scr = L.take(0);
  DWorld dw = w.dw;
  const size_t need = o_scr + scratch_layout_into(w, dw, nullptr);
  if (need > arena_bytes)
    return fail(CP_ERR_CAPACITY, "world %d needs %zu bytes of step scratch; the static scratch holds %zu (use cp_world_step)",
                id, need, arena_bytes);
  if (nsteps == 0) return CP_OK;
  char* base = (char*)arena;
  scratch_layout_into(w, dw, base + o_scr);
  const int hdr[3] = {0, 0, 1};  // work list {world 0}, group bounds {0, 1}
  st = ensure_dt_static(c, w, dt);
  if (st) return st;
  CUDA_TRY(cudaMemcpyAsync(base + o_rec, &dw, sizeof(DWorld), cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(cudaMemcpyAsync(base + o_ids, hdr, sizeof(hdr), cudaMemcpyHostToDevice, c->stream));
  const DWorld* d_world = (const DWorld*)(base + o_rec);
  const int* d_list = (const int*)(base + o_ids);
  const int variant = w.nb > 512 ? 0 : c->plain_variant;
  for (int s = 0; s < nsteps; s++) {
    CUDA_TRY(cpk_launch_step(d_world, d_list, d_list + 1, 1, dt, dt, c->d_queue, 1, 1, c->stream, variant, 1, w.nb));
    c->launches += 2;  // the two step kernels (the queue reset is a memset)
  }
  DWorldParams p;
  st = read_params(c, w, p);  // synchronises the stream: the host buffers above are no longer in use
  if (st) return st;
  st = kernel_check();
  if (st) return st;
  if (p.status != 0) {
    // The failed step's lists are partial: clear the status and report empty
    // lists (num_pairs, num_contacts, num_rows and num_levels are consecutive
    // ints of the parameter record).
    static_assert(offsetof(DWorldParams, num_levels) == offsetof(DWorldParams, num_pairs) + 3 * sizeof(int), "layout");
    CUDA_TRY(cudaMemsetAsync(&w.dw.P->status, 0, sizeof(int), c->stream));
    CUDA_TRY(cudaMemsetAsync(&w.dw.P->num_pairs, 0, 4 * sizeof(int), c->stream));
    CUDA_TRY(cudaMemsetAsync(&w.dw.P->num_jobs, 0, sizeof(int), c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    return fail(CP_ERR_CAPACITY, "world %d: step %lld overflowed a capacity (status %d); the world is left before that step",
                id, p.stepnumber + 1, p.status);
  }
  // The last step's pairs, contacts and rows (with their lambdas and
  // multipliers) into the world's own scratch, where cp_world_get_pairs /
  // get_contacts / get_rows read them.  Both layouts come from the same
  // capacities, and every count is within them after a step without overflow.
  if (nsteps > 0) {
    if (p.num_pairs > 0) {
      CUDA_TRY(cudaMemcpyAsync(w.dw.pair_a, dw.pair_a, sizeof(int) * p.num_pairs, cudaMemcpyDeviceToDevice, c->stream));
      CUDA_TRY(cudaMemcpyAsync(w.dw.pair_b, dw.pair_b, sizeof(int) * p.num_pairs, cudaMemcpyDeviceToDevice, c->stream));
    }
    if (p.num_contacts > 0)
      CUDA_TRY(cudaMemcpyAsync(w.dw.contacts, dw.contacts, sizeof(DContact) * p.num_contacts, cudaMemcpyDeviceToDevice, c->stream));
    if (w.compound && p.num_jobs > 0) {  // contacts name their job; the job list maps them to pairs
      CUDA_TRY(cudaMemcpyAsync(w.dw.job_pair, dw.job_pair, sizeof(int) * p.num_jobs, cudaMemcpyDeviceToDevice, c->stream));
      CUDA_TRY(cudaMemcpyAsync(w.dw.job_sh, dw.job_sh, sizeof(int) * p.num_jobs, cudaMemcpyDeviceToDevice, c->stream));
    }
    if (p.num_rows > 0)
      CUDA_TRY(cudaMemcpyAsync(w.dw.rows, dw.rows, sizeof(DRow) * p.num_rows, cudaMemcpyDeviceToDevice, c->stream));
    if (w.split && p.num_rows > 0)
      CUDA_TRY(cudaMemcpyAsync(w.dw.row_id, dw.row_id, sizeof(long long) * p.num_rows, cudaMemcpyDeviceToDevice, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
  }
  return CP_OK;
}

int cp_world_get_bodies(cp_ctx* c, int32_t id, cp_body_desc* out, int32_t n) {
  int st = check_world(c, id);
  if (st) return st;
  std::lock_guard<std::mutex> lock(c->mu);
  WorldRec& w = c->worlds[id];
  if ((!out && n > 0) || n != w.nb) return fail(CP_ERR_ARG, "expected %d bodies", w.nb);
  return read_bodies(c, id, out);
}

int cp_world_set_bodies(cp_ctx* c, int32_t id, const cp_body_desc* in, int32_t n) {
  int st = check_world(c, id);
  if (st) return st;
  std::lock_guard<std::mutex> lock(c->mu);
  WorldRec& w = c->worlds[id];
  if ((!in && n > 0) || n != w.nb) return fail(CP_ERR_ARG, "expected %d bodies", w.nb);
  if (w.nb == 0) return CP_OK;
  std::vector<DBody> b(w.nb);
  for (int i = 0; i < w.nb; i++) {
    if (in[i].shape < -1 || in[i].shape >= w.nshapes) return fail(CP_ERR_ARG, "body %d: shape out of range", i);
    if (!extras_valid(in[i], w.nshapes, w.body_shapes.data(), (int)w.body_shapes.size()))
      return fail(CP_ERR_ARG, "body %d: extra shapes outside the world's body_shapes table", i);
    if (in[i].extra_shapes_count > 0 && !w.compound)
      return fail(CP_ERR_ARG, "body %d: a world created without compound bodies cannot take one (create it again)", i);
    body_to_device(in[i], b[i]);
    w.lin_damp[i] = in[i].linear_damping;
    w.ang_damp[i] = in[i].angular_damping;
    w.body_shape[i] = in[i].shape;
    w.body_xs0[i] = in[i].extra_shapes_first;
  }
  CUDA_TRY(cudaMemcpyAsync(w.dw.bodies, b.data(), sizeof(DBody) * w.nb, cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  w.dt_cached = -1.0;
  return CP_OK;
}

}  // extern "C"

namespace {

int ensure_states(cp_ctx* c, int n) {
  if (n <= c->states_cap) return CP_OK;
  const int cap = std::max(n, 2 * c->states_cap);
  if (c->d_states) cudaFree(c->d_states);
  c->d_states = nullptr;
  c->states_cap = 0;
  CUDA_TRY(cudaMalloc(&c->d_states, sizeof(cp_body_state) * (size_t)cap));
  c->states_cap = cap;
  return CP_OK;
}

}  // namespace

extern "C" {

int cp_world_raycast(cp_ctx* c, int32_t id, const cp_ray* rays, int32_t n, int32_t mode, cp_ray_hit* hits, int32_t max_hits,
                     int32_t* counts) {
  int st = check_world(c, id);
  if (st) return st;
  if (n < 0 || (n > 0 && (!rays || !hits)) || mode < CP_RAY_CLOSEST || mode > CP_RAY_ALL)
    return fail(CP_ERR_ARG, "bad raycast arguments");
  if (mode == CP_RAY_ALL && (max_hits < 0 || (n > 0 && !counts))) return fail(CP_ERR_ARG, "RAY_ALL needs max_hits >= 0 and counts");
  std::lock_guard<std::mutex> lock(c->mu);
  cudaSetDevice(c->device);
  const size_t per = mode == CP_RAY_ALL ? (size_t)max_hits : 1;
  Layout L;
  const size_t o_r = L.take(sizeof(cp_ray) * (size_t)n);
  const size_t o_h = L.take(sizeof(cp_ray_hit) * per * (size_t)n);
  const size_t o_c = L.take(sizeof(int32_t) * (size_t)n);
  if (L.off > c->rays_bytes) {
    const size_t cap = std::max(L.off, 2 * c->rays_bytes);
    if (c->d_rays) cudaFree(c->d_rays);
    c->d_rays = nullptr;
    c->rays_bytes = 0;
    CUDA_TRY(cudaMalloc(&c->d_rays, cap));
    c->rays_bytes = cap;
  }
  char* base = (char*)c->d_rays;
  if (n > 0) CUDA_TRY(cudaMemcpyAsync(base + o_r, rays, sizeof(cp_ray) * n, cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(cpk_raycast(c->d_worlds + id, (const cp_ray*)(base + o_r), n, mode, (cp_ray_hit*)(base + o_h), (int)per,
                       (int*)(base + o_c), c->stream));
  c->launches += n > 0 ? 2 : 1;
  if (n > 0) {
    CUDA_TRY(cudaMemcpyAsync(hits, base + o_h, sizeof(cp_ray_hit) * per * n, cudaMemcpyDeviceToHost, c->stream));
    if (mode == CP_RAY_ALL) CUDA_TRY(cudaMemcpyAsync(counts, base + o_c, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, c->stream));
  }
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  return kernel_check();
}

int cp_world_get_states(cp_ctx* c, int32_t id, cp_body_state* out, int32_t n) {
  int st = check_world(c, id);
  if (st) return st;
  std::lock_guard<std::mutex> lock(c->mu);
  cudaSetDevice(c->device);
  WorldRec& w = c->worlds[id];
  if ((!out && n > 0) || n != w.nb) return fail(CP_ERR_ARG, "expected %d bodies", w.nb);
  if (n == 0) return CP_OK;
  st = ensure_states(c, n);
  if (st) return st;
  CUDA_TRY(cpk_states(c->d_worlds + id, n, c->d_states, 0, c->stream));
  c->launches += 1;
  CUDA_TRY(cudaMemcpyAsync(out, c->d_states, sizeof(cp_body_state) * n, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  return CP_OK;
}

int cp_world_set_states(cp_ctx* c, int32_t id, const cp_body_state* in, int32_t n) {
  int st = check_world(c, id);
  if (st) return st;
  std::lock_guard<std::mutex> lock(c->mu);
  cudaSetDevice(c->device);
  WorldRec& w = c->worlds[id];
  if ((!in && n > 0) || n != w.nb) return fail(CP_ERR_ARG, "expected %d bodies", w.nb);
  for (int i = 0; i < n; i++)
    if (in[i].sleep_state < CP_AWAKE || in[i].sleep_state > CP_SLEEPING) return fail(CP_ERR_ARG, "body %d: bad sleep state", i);
  if (n == 0) return CP_OK;
  st = ensure_states(c, n);
  if (st) return st;
  CUDA_TRY(cudaMemcpyAsync(c->d_states, in, sizeof(cp_body_state) * n, cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(cpk_states(c->d_worlds + id, n, c->d_states, 1, c->stream));
  c->launches += 1;
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  return CP_OK;
}

int cp_world_get_info(cp_ctx* c, int32_t id, cp_step_info* out) {
  int st = check_world(c, id);
  if (st) return st;
  if (!out) return fail(CP_ERR_ARG, "null out");
  std::lock_guard<std::mutex> lock(c->mu);
  return read_info(c, id, out);
}

int cp_world_get_pairs(cp_ctx* c, int32_t id, int32_t* p1, int32_t* p2, int32_t cap, int32_t* count) {
  int st = check_world(c, id);
  if (st) return st;
  if (!count) return fail(CP_ERR_ARG, "null count");
  std::lock_guard<std::mutex> lock(c->mu);
  WorldRec& w = c->worlds[id];
  DWorldParams p;
  st = read_params(c, w, p);
  if (st) return st;
  *count = p.num_pairs;
  if (p.num_pairs > cap || (p.num_pairs && (!p1 || !p2))) return fail(CP_ERR_CAPACITY, "need room for %d pairs", p.num_pairs);
  if (p.num_pairs) {
    CUDA_TRY(cudaMemcpy(p1, w.dw.pair_a, sizeof(int) * p.num_pairs, cudaMemcpyDeviceToHost));
    CUDA_TRY(cudaMemcpy(p2, w.dw.pair_b, sizeof(int) * p.num_pairs, cudaMemcpyDeviceToHost));
  }
  return CP_OK;
}

int cp_world_get_contacts(cp_ctx* c, int32_t id, cp_contact* out, int32_t cap, int32_t* count) {
  int st = check_world(c, id);
  if (st) return st;
  if (!count) return fail(CP_ERR_ARG, "null count");
  std::lock_guard<std::mutex> lock(c->mu);
  WorldRec& w = c->worlds[id];
  DWorldParams p;
  st = read_params(c, w, p);
  if (st) return st;
  *count = p.num_contacts;
  if (p.num_contacts > cap || (p.num_contacts && !out)) return fail(CP_ERR_CAPACITY, "need room for %d contacts", p.num_contacts);
  std::vector<DContact> v(p.num_contacts);
  if (p.num_contacts) CUDA_TRY(cudaMemcpy(v.data(), w.dw.contacts, sizeof(DContact) * v.size(), cudaMemcpyDeviceToHost));
  // a contact records its narrowphase job; in a compound world the job's
  // broadphase pair is job_pair[job]
  std::vector<int> jp(w.compound ? p.num_jobs : 0);
  if (!jp.empty()) CUDA_TRY(cudaMemcpy(jp.data(), w.dw.job_pair, sizeof(int) * jp.size(), cudaMemcpyDeviceToHost));
  for (int i = 0; i < p.num_contacts; i++) {
    cp_contact& o = out[i];
    o.bi = v[i].bi; o.bj = v[i].bj; o.si = v[i].si; o.sj = v[i].sj;
    std::memcpy(o.ni, v[i].ni, 12); std::memcpy(o.ri, v[i].ri, 12); std::memcpy(o.rj, v[i].rj, 12);
    o.enabled = v[i].enabled; o.restitution = v[i].restitution;
    o.pair = w.compound ? jp[v[i].pair] : v[i].pair;
  }
  return CP_OK;
}

int cp_world_get_rows(cp_ctx* c, int32_t id, cp_row* out, int32_t cap, int32_t* count) {
  int st = check_world(c, id);
  if (st) return st;
  if (!count) return fail(CP_ERR_ARG, "null count");
  std::lock_guard<std::mutex> lock(c->mu);
  WorldRec& w = c->worlds[id];
  DWorldParams p;
  st = read_params(c, w, p);
  if (st) return st;
  *count = p.num_rows;
  if (p.num_rows > cap || (p.num_rows && !out)) return fail(CP_ERR_CAPACITY, "need room for %d rows", p.num_rows);
  std::vector<DRow> v(p.num_rows);
  if (p.num_rows) CUDA_TRY(cudaMemcpy(v.data(), w.dw.rows, sizeof(DRow) * v.size(), cudaMemcpyDeviceToHost));
  std::vector<long long> ids(w.split ? p.num_rows : 0);
  if (!ids.empty()) CUDA_TRY(cudaMemcpy(ids.data(), w.dw.row_id, sizeof(long long) * ids.size(), cudaMemcpyDeviceToHost));
  for (int i = 0; i < p.num_rows; i++) {
    cp_row& o = out[i];
    o.kind = v[i].kind; o.bi = v[i].bi; o.bj = v[i].bj; o.pad = 0;
    o.B = v[i].B; o.inv_c = v[i].invC; o.lambda = v[i].lambda; o.multiplier = v[i].mult;
    o.min_force = v[i].minF; o.max_force = v[i].maxF; o.eps = v[i].eps;
    o.id = w.split ? ids[i] : -1;
  }
  return CP_OK;
}

int cp_world_get_sap_order(cp_ctx* c, int32_t id, int32_t* out, int32_t n) {
  int st = check_world(c, id);
  if (st) return st;
  std::lock_guard<std::mutex> lock(c->mu);
  WorldRec& w = c->worlds[id];
  if ((!out && n > 0) || n != w.nb) return fail(CP_ERR_ARG, "expected %d entries", w.nb);
  if (n) CUDA_TRY(cudaMemcpy(out, w.dw.sap_order, sizeof(int) * n, cudaMemcpyDeviceToHost));
  return CP_OK;
}

}  // extern "C"

namespace cpi {

int step_worlds(cp_ctx* c, const int* ids, int n, double dt, int nsteps, bool use_graph, std::vector<int>* failed) {
  for (int i = 0; i < n; i++) {
    if (ids[i] < 0 || ids[i] >= (int)c->worlds.size() || !c->worlds[ids[i]].live) return fail(CP_ERR_ARG, "no world %d", ids[i]);
    int st = ensure_dt(c, c->worlds[ids[i]], dt);
    if (st) return st;
  }
  // largest worlds first: the persistent blocks take them from the queue in this order
  std::vector<int> order(ids, ids + n);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return c->worlds[a].nb > c->worlds[b].nb; });
  int st = ensure_ids(c, n);
  if (st) return st;
  // autotuning: while variants are untimed for this world set, each call runs
  // its steps with the next untimed variant (results do not depend on it)
  // A second tuning round once the worlds have settled into contact: early
  // steps (bodies in free fall) favour other variants than contact-heavy ones.
  if (use_graph && c->tune_ids != order) {
    c->tune_ids = order;
    c->tune_calls = 0;
  }
  // A round times every pre-solve kernel variant with solve variant 0, then
  // every solve variant with the fastest pre-solve variant.
  const int npre = cpk_num_pre_variants(), nsol = cpk_num_solve_variants();
  if (use_graph && (c->tune_calls == 0 || c->tune_calls == 48)) {
    c->tune_ms.assign(cpk_num_variants(), 0.0);
    c->tune_plan.clear();
    for (int p = 0; p < npre; p++) c->tune_plan.push_back(p * nsol);
    c->tune_next = 0;
    c->best = -1;
  }
  if (use_graph) c->tune_calls++;
  // Without a graph (world sets that change from call to call) nothing is
  // tuned: the forced variant, else the tuned one, else the default for the
  // set's largest world: a world above 512 bodies gets a 256-thread pre-step
  // block of its own per SM (variant 0, as a single large world does; on
  // served request mixes of 16-4096 bodies 1.5x the throughput of the small
  // worlds' default).
  const bool tuning = use_graph && c->forced < 0 && c->best < 0;
  const int fallback = c->worlds[order[0]].nb > 512 ? 0 : c->plain_variant;
  const int variant = c->forced >= 0 ? c->forced : (tuning ? c->tune_plan[c->tune_next] : (c->best >= 0 ? c->best : fallback));
  // groups of consecutive worlds (the order is by size): up to group_bodies
  // per 128 threads of a block-wide solve kernel (a narrower block takes a
  // smaller group, so its levels still fill its lanes), or up to group_bodies
  // per warp for the warp-centric one
  std::vector<int> gstart(1, 0);
  {
    const long long limit = cpk_solve_group_limit(variant, c->group_bodies);
    int cnt = 0;
    long long bodies = 0;
    for (int i = 0; i < n; i++) {
      int nb = c->worlds[order[i]].nb;
      if (cnt > 0 && (cnt == CP_GROUP_MAX_WORLDS || bodies + nb > limit)) {
        gstart.push_back(i);
        cnt = 0;
        bodies = 0;
      }
      cnt++;
      bodies += nb;
    }
    gstart.push_back(n);
  }
  const int ngroups = (int)gstart.size() - 1;
  const int max_nb = c->worlds[order[0]].nb;  // the order is by size
  const int grid_pre = std::max(1, std::min(n, c->sms * cpk_pre_blocks_per_sm(variant, max_nb)));
  const int grid_solve = std::max(1, std::min(ngroups, c->sms * c->blocks_solve[variant]));
  bool reuse = use_graph && !tuning && c->graph && c->graph_ids == order && c->graph_dt == dt && c->graph_steps == nsteps &&
               c->graph_variant == variant;
  // world list and groups: uploaded when they change (a repeated call on
  // the same worlds reuses them, and its captured graph)
  if (c->dev_order != order) {
    CUDA_TRY(cudaMemcpyAsync(c->d_ids, order.data(), sizeof(int) * n, cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));  // the host vector may change before a pageable copy completes
    c->dev_order = order;
  }
  if (c->dev_gstart != gstart) {
    CUDA_TRY(cudaMemcpyAsync(c->d_gstart, gstart.data(), sizeof(int) * gstart.size(), cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    c->dev_gstart = gstart;
  }
  if (use_graph && !reuse && !tuning) {
    if (c->graph) { cudaGraphExecDestroy(c->graph); c->graph = nullptr; }
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    cudaGraph_t g;
    CUDA_TRY(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    for (int s = 0; s < nsteps; s++) {
      cudaError_t e = cpk_launch_step(c->d_worlds, c->d_ids, c->d_gstart, ngroups, dt, dt, c->d_queue, grid_pre, grid_solve, c->stream,
                                      variant, n, max_nb);
      if (e != cudaSuccess) {
        cudaStreamEndCapture(c->stream, &g);
        return fail(CP_ERR_CUDA, "capture: %s", cudaGetErrorString(e));
      }
    }
    CUDA_TRY(cudaStreamEndCapture(c->stream, &g));
    cudaError_t e = cudaGraphInstantiate(&c->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(CP_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
    c->graph_ids = order;
    c->graph_dt = dt;
    c->graph_steps = nsteps;
    c->graph_variant = variant;
  }
  // step numbers before the launch, to finish worlds whose step overflowed;
  // kept on the device and read only when some world overflowed
  long long* d_before = c->d_status + 4 * (size_t)c->d_status_cap;
  CUDA_TRY(cpk_gather_status(c->d_worlds, c->d_ids, n, d_before, c->stream));
  std::vector<long long> after(4 * (size_t)n);
  CUDA_TRY(cudaEventRecord(c->ev0, c->stream));
  if (tuning || !use_graph) {
    for (int s = 0; s < nsteps; s++)
      CUDA_TRY(cpk_launch_step(c->d_worlds, c->d_ids, c->d_gstart, ngroups, dt, dt, c->d_queue, grid_pre, grid_solve, c->stream,
                               variant, n, max_nb));
  } else {
    CUDA_TRY(cudaGraphLaunch(c->graph, c->stream));
  }
  CUDA_TRY(cudaEventRecord(c->ev1, c->stream));
  c->launches += 2LL * nsteps + 1;  // two step kernels per step and the status gather before them
  CUDA_TRY(cpk_gather_status(c->d_worlds, c->d_ids, n, c->d_status, c->stream));
  CUDA_TRY(cudaMemcpyAsync(after.data(), c->d_status, sizeof(long long) * 4 * n, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  st = kernel_check();
  if (st) return st;
  float gms = 0.f;
  CUDA_TRY(cudaEventElapsedTime(&gms, c->ev0, c->ev1));
  c->graph_ms += gms;
  c->graph_step_launches += nsteps;
  if (tuning) {
    c->tune_ms[variant] = gms / nsteps;
    if (++c->tune_next == (int)c->tune_plan.size()) {
      auto fastest = [&]() {
        int b = c->tune_plan[0];
        for (int v : c->tune_plan)
          if (c->tune_ms[v] < c->tune_ms[b]) b = v;
        return b;
      };
      int b = fastest();
      if ((int)c->tune_plan.size() == npre) {  // first half done: now the solve variants
        c->tune_plan.clear();
        for (int sv = 0; sv < nsol; sv++) c->tune_plan.push_back((b / nsol) * nsol + sv);
        c->tune_next = 1;  // (b, solve 0) is timed already
      } else {
        c->best = b;
      }
    }
  }
  c->launches += 1;
  bool any = false;
  for (int i = 0; i < n && !any; i++) any = after[4 * i] != 0;
  if (!any) return CP_OK;
  std::vector<long long> before(4 * (size_t)n);
  CUDA_TRY(cudaMemcpyAsync(before.data(), d_before, sizeof(long long) * 4 * n, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  for (int i = 0; i < n; i++) {
    if (after[4 * i] != 0) {  // overflowed part way: grow and finish on the plain path
      int id = order[i];
      const long long limit = c->worlds[id].step_limit;
      long long left = std::min(before[4 * i + 1] + nsteps, limit) - after[4 * i + 1];
      st = grow(c, id, (int)after[4 * i]);
      if (!st) st = plain_steps(c, id, dt, (int)left, dt);
      if (st) {
        if (!failed) return st;
        failed->push_back(id);  // this world fails alone; the others go on
      }
    }
  }
  return CP_OK;
}

}  // namespace cpi

extern "C" {

int cp_batch_step(cp_ctx* c, const int32_t* ids, int32_t n, double dt, int32_t nsteps) {
  if (!c || (n > 0 && !ids) || n < 0 || nsteps < 0 || !(dt > 0)) return fail(CP_ERR_ARG, "bad arguments");
  if (n == 0 || nsteps == 0) return CP_OK;
  std::lock_guard<std::mutex> lock(c->mu);
  cudaSetDevice(c->device);
  return step_worlds(c, ids, n, dt, nsteps, true);
}

}  // extern "C"

namespace {
// world list + packed offsets on the device for the batched I/O calls
int prepare_io(cp_ctx* c, const int32_t* ids, int n, int64_t total, int floats_per_body) {
  if (!c || (n > 0 && !ids) || n < 0) return fail(CP_ERR_ARG, "bad arguments");
  std::vector<long long> first(n);
  long long acc = 0;
  for (int i = 0; i < n; i++) {
    if (ids[i] < 0 || ids[i] >= (int)c->worlds.size() || !c->worlds[ids[i]].live) return fail(CP_ERR_ARG, "no world %d", ids[i]);
    first[i] = acc;
    acc += c->worlds[ids[i]].nb;
  }
  if (acc != total) return fail(CP_ERR_ARG, "total_bodies %lld != %lld", (long long)total, acc);
  if (n > c->io_cap) {
    if (c->d_io_ids) cudaFree(c->d_io_ids);
    if (c->d_io_first) cudaFree(c->d_io_first);
    int cap = std::max(256, 2 * n);
    CUDA_TRY(cudaMalloc(&c->d_io_ids, sizeof(int) * cap));
    CUDA_TRY(cudaMalloc(&c->d_io_first, sizeof(long long) * cap));
    c->io_cap = cap;
    c->io_ids.clear();
  }
  long long need = acc * floats_per_body;
  if (need > c->io_floats) {
    if (c->d_io) cudaFree(c->d_io);
    long long cap = std::max<long long>(1 << 16, need + need / 4);
    CUDA_TRY(cudaMalloc(&c->d_io, sizeof(float) * cap));
    c->io_floats = cap;
  }
  if (c->io_ids.size() != (size_t)n || !std::equal(c->io_ids.begin(), c->io_ids.end(), ids)) {
    CUDA_TRY(cudaMemcpyAsync(c->d_io_ids, ids, sizeof(int) * n, cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(cudaMemcpyAsync(c->d_io_first, first.data(), sizeof(long long) * n, cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    c->io_ids.assign(ids, ids + n);
  }
  return CP_OK;
}
}  // namespace

extern "C" {

int cp_batch_set_forces(cp_ctx* c, const int32_t* ids, int32_t n, const float* ft, int64_t total) {
  if (!c) return fail(CP_ERR_ARG, "null context");
  std::lock_guard<std::mutex> lock(c->mu);
  cudaSetDevice(c->device);
  int st = prepare_io(c, ids, n, total, 6);
  if (st) return st;
  if (total == 0) return CP_OK;
  if (!ft) return fail(CP_ERR_ARG, "null buffer");
  CUDA_TRY(cudaMemcpyAsync(c->d_io, ft, sizeof(float) * 6 * total, cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(cpk_scatter_forces(c->d_worlds, c->d_io_ids, c->d_io_first, n, c->d_io, c->stream));
  c->launches += 1;
  return CP_OK;  // ordered before the next step on the context's stream
}

int cp_batch_get_poses(cp_ctx* c, const int32_t* ids, int32_t n, float* out, int64_t total) {
  if (!c) return fail(CP_ERR_ARG, "null context");
  std::lock_guard<std::mutex> lock(c->mu);
  cudaSetDevice(c->device);
  int st = prepare_io(c, ids, n, total, 13);
  if (st) return st;
  if (total == 0) return CP_OK;
  if (!out) return fail(CP_ERR_ARG, "null buffer");
  CUDA_TRY(cpk_gather_poses(c->d_worlds, c->d_io_ids, c->d_io_first, n, c->d_io, c->stream));
  c->launches += 1;
  CUDA_TRY(cudaMemcpyAsync(out, c->d_io, sizeof(float) * 13 * total, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  return CP_OK;
}

int64_t cp_kernel_launches(cp_ctx* c) { return c ? c->launches : 0; }

int cp_get_stream(cp_ctx* c, void** stream) {
  if (!c || !stream) return fail(CP_ERR_ARG, "null argument");
  *stream = (void*)c->stream;
  return CP_OK;
}

int cp_phase_profile(cp_ctx* c, double* cycles, int32_t n) {
  if (!c || !cycles || n < CP_NUM_PHASES) return fail(CP_ERR_ARG, "need room for %d phases", CP_NUM_PHASES);
  std::lock_guard<std::mutex> lock(c->mu);
  cudaSetDevice(c->device);
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  unsigned long long v[CP_PROFILE_SLOTS];
  CUDA_TRY(cpk_phase_cycles(v, true));
  for (int i = 0; i < n && i < CP_PROFILE_SLOTS; i++) cycles[i] = (double)v[i];
  return CP_OK;
}

int cp_set_resolver_profile(cp_ctx* c, int32_t on) {
  if (!c) return fail(CP_ERR_ARG, "null argument");
  std::lock_guard<std::mutex> lock(c->mu);
  cudaSetDevice(c->device);
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  CUDA_TRY(cpk_set_resolver_profile(on));
  return CP_OK;
}

int cp_set_filter_check(cp_ctx* c, int32_t on) {
  if (!c) return fail(CP_ERR_ARG, "null context");
  std::lock_guard<std::mutex> lock(c->mu);
  cudaSetDevice(c->device);
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  CUDA_TRY(cpk_filter_check(on ? 1 : 0));
  CUDA_TRY(cpk_wide_filter_check(on ? 1 : 0));
  return CP_OK;
}

int cp_filter_check_counts(cp_ctx* c, int64_t* checked, int64_t* disagreed, int32_t reset) {
  if (!c || !checked || !disagreed) return fail(CP_ERR_ARG, "null argument");
  std::lock_guard<std::mutex> lock(c->mu);
  cudaSetDevice(c->device);
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  unsigned long long a[2], b[2];
  CUDA_TRY(cpk_filter_counts(a, reset != 0));
  CUDA_TRY(cpk_wide_filter_counts(b, reset != 0));
  *checked = (int64_t)(a[0] + b[0]);
  *disagreed = (int64_t)(a[1] + b[1]);
  return CP_OK;
}

int cp_set_wide_bodies(cp_ctx* c, int32_t bodies) {
  if (!c) return fail(CP_ERR_ARG, "null context");
  if (bodies < 0) return fail(CP_ERR_ARG, "bodies must be >= 0");
  std::lock_guard<std::mutex> lock(c->mu);
  c->wide_bodies = bodies;
  return CP_OK;
}

int cp_set_sweep_schedule(cp_ctx* c, int32_t mode) {
  if (!c) return fail(CP_ERR_ARG, "null context");
  if (mode < -1 || mode > 1) return fail(CP_ERR_ARG, "sweep schedule mode must be -1, 0 or 1");
  std::lock_guard<std::mutex> lock(c->mu);
  c->sched_mode = mode;
  return CP_OK;
}

int cp_set_group_bodies(cp_ctx* c, int32_t bodies) {
  if (!c || bodies < 0) return fail(CP_ERR_ARG, "bad group size");
  std::lock_guard<std::mutex> lock(c->mu);
  c->group_bodies = bodies;
  if (c->graph) { cudaGraphExecDestroy(c->graph); c->graph = nullptr; }
  return CP_OK;
}

int cp_autotune_info(cp_ctx* c, int32_t* variant, int32_t* threads, double* ms, int32_t n) {
  if (!c || !variant || !threads) return fail(CP_ERR_ARG, "null argument");
  std::lock_guard<std::mutex> lock(c->mu);
  *variant = c->best;
  *threads = c->best >= 0 ? cpk_variant_threads(c->best) : 0;
  for (int i = 0; ms && i < n && i < (int)c->tune_ms.size(); i++) ms[i] = c->tune_ms[i];
  return cpk_num_variants();
}

int cp_set_variant(cp_ctx* c, int32_t v) {
  if (!c || v < -1 || v >= cpk_num_variants()) return fail(CP_ERR_ARG, "variant %d out of range", v);
  std::lock_guard<std::mutex> lock(c->mu);
  c->forced = v;
  return CP_OK;
}

int cp_batch_profile(cp_ctx* c, double* graph_ms, int64_t* step_launches) {
  if (!c || !graph_ms || !step_launches) return fail(CP_ERR_ARG, "null argument");
  std::lock_guard<std::mutex> lock(c->mu);
  *graph_ms = c->graph_ms;
  *step_launches = c->graph_step_launches;
  c->graph_ms = 0.0;
  c->graph_step_launches = 0;
  return CP_OK;
}

}  // extern "C"
