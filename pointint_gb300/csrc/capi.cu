// C ABI entry points: device-resident k-grids and object batches, form
// factors, contraction, and the one-shot host-buffer drop-ins that replace the
// reference's compute_intersection_volume*_cuda drivers
// (cpp/src/compute_intersection_volume.cu:172-489,
//  cpp/src/compute_intersection_volume_multi_object.cu:234-713) and its
// per-object registry wrappers (cpp/src/dof/cuda/affine_dof_cuda.cu:855-1321).
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <numeric>
#include <unordered_map>
#include <vector>
#include "pi_internal.h"
#include "group.h"

using namespace pi;

constexpr double INV_8PI3 = 1.0 / (8.0 * 3.14159265358979323846 * 3.14159265358979323846 * 3.14159265358979323846);

namespace {

size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

size_t elem_bytes(int geom_type) { return geom_type == PI_GEOM_TRIANGLE ? sizeof(pi_tri_packed) : sizeof(pi_disk_packed); }

int validate_object(const pi_object& o, int i) {
  char buf[160];
  if (o.geom_type < PI_GEOM_TRIANGLE || o.geom_type > PI_GEOM_GAUSSIAN) {
    snprintf(buf, sizeof buf, "object %d: unknown geometry type %d", i, o.geom_type);
    return fail(PI_ERR_INVALID_ARGUMENT, buf);
  }
  if (o.n_elems < 0 || o.n_elems > 0x7fffffffLL || (o.n_elems > 0 && !o.elems)) {
    snprintf(buf, sizeof buf, "object %d: bad element array", i);
    return fail(PI_ERR_INVALID_ARGUMENT, buf);
  }
  if (o.dof_type == PI_DOF_AFFINE) {
    if (o.n_dofs != 12 || !o.dofs) {
      snprintf(buf, sizeof buf, "object %d: AffineDoF needs 12 DoFs, got %lld", i, (long long)o.n_dofs);
      return fail(PI_ERR_INVALID_ARGUMENT, buf);
    }
  } else if (o.dof_type == PI_DOF_TRIANGLE_MESH) {
    if (o.geom_type != PI_GEOM_TRIANGLE) {
      snprintf(buf, sizeof buf, "object %d: TriangleMeshDoF needs a triangle mesh", i);
      return fail(PI_ERR_UNSUPPORTED, buf);
    }
    if (o.n_dofs <= 0 || o.n_dofs % 3 != 0 || !o.dofs) {
      snprintf(buf, sizeof buf, "object %d: TriangleMeshDoF needs 3V DoFs", i);
      return fail(PI_ERR_INVALID_ARGUMENT, buf);
    }
  } else {
    snprintf(buf, sizeof buf, "object %d: unknown DoF type %d", i, o.dof_type);
    return fail(PI_ERR_INVALID_ARGUMENT, buf);
  }
  return PI_OK;
}

// RAII for temporary device buffers of the host-buffer entry points.
struct DevBuf {
  void* p = nullptr;
  cudaStream_t s = nullptr;
  ~DevBuf() { if (p) cudaFreeAsync(p, s); }
  int alloc(size_t bytes, cudaStream_t st) {
    s = st;
    if (bytes == 0) bytes = 16;
    PI_CUDA(cudaMallocAsync(&p, bytes, st));
    return PI_OK;
  }
};

struct KGridGuard { pi_kgrid k = nullptr; ~KGridGuard() { if (k) pi_kgrid_destroy(k); } };

// G [D][Q] complex64 (the DoF Jacobian's layout) -> out [Q][D] double2 (the
// registry gradient plugin's row-major layout).
__global__ void jacobian_to_qd_kernel(const float2* __restrict__ G, int64_t Q, int64_t D, double2* __restrict__ out) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= Q * D) return;
  const int64_t q = t / D, d = t - q * D;
  const float2 v = G[d * Q + q];
  out[t] = make_double2(v.x, v.y);
}

// Vertex -> (triangle, slot) adjacency of every TriangleMeshDoF object, for
// the deterministic per-vertex gather of the adjoint.  Device-resident
// elements are read back once.
int build_vertex_csr(pi_batch_impl* b, const pi_object* objs, int on_device, cudaStream_t s) {
  int64_t nv = 0, goff = 0;
  std::vector<int64_t> voff(b->n_obj, -1), gofs(b->n_obj);
  for (int i = 0; i < b->n_obj; ++i) {
    gofs[i] = goff;
    goff += b->info[i].n_dofs;
    if (b->info[i].dof_type == PI_DOF_TRIANGLE_MESH) { voff[i] = nv; nv += b->info[i].n_dofs / 3; }
  }
  b->n_mesh_verts = nv;
  if (nv == 0) return PI_OK;
  std::vector<std::vector<int64_t>> adj(nv);
  for (int i = 0; i < b->n_obj; ++i) {
    if (voff[i] < 0) continue;
    const HostObjInfo& in = b->info[i];
    std::vector<pi_tri_packed> tmp;
    const pi_tri_packed* T = static_cast<const pi_tri_packed*>(objs[i].elems);
    if (on_device) {
      tmp.resize(in.n_elems);
      PI_CUDA(cudaMemcpyAsync(tmp.data(), objs[i].elems, in.n_elems * sizeof(pi_tri_packed), cudaMemcpyDeviceToHost, s));
      PI_CUDA(cudaStreamSynchronize(s));
      T = tmp.data();
    }
    const int64_t nvi = in.n_dofs / 3;
    for (int64_t f = 0; f < in.n_elems; ++f) {
      const int32_t v[3] = {T[f].vid0, T[f].vid1, T[f].vid2};
      if (v[0] < 0 || v[1] < 0 || v[2] < 0 || v[0] >= nvi || v[1] >= nvi || v[2] >= nvi) continue;
      for (int sl = 0; sl < 3; ++sl) adj[voff[i] + v[sl]].push_back((in.pool_off + f) * 3 + sl);
    }
  }
  std::vector<int64_t> row(nv + 1, 0), ent, vmap(nv);
  for (int64_t v = 0; v < nv; ++v) row[v + 1] = row[v] + (int64_t)adj[v].size();
  ent.reserve(row[nv]);
  for (auto& a : adj) ent.insert(ent.end(), a.begin(), a.end());
  for (int i = 0; i < b->n_obj; ++i)
    if (voff[i] >= 0)
      for (int64_t v = 0; v < b->info[i].n_dofs / 3; ++v) vmap[voff[i] + v] = gofs[i] + 3 * v;
  PI_CUDA(cudaMalloc((void**)&b->d_vrow, row.size() * sizeof(int64_t)));
  PI_CUDA(cudaMalloc((void**)&b->d_vent, std::max<size_t>(ent.size(), 1) * sizeof(int64_t)));
  PI_CUDA(cudaMalloc((void**)&b->d_vmap, vmap.size() * sizeof(int64_t)));
  PI_CUDA(cudaMemcpy(b->d_vrow, row.data(), row.size() * sizeof(int64_t), cudaMemcpyHostToDevice));
  if (!ent.empty()) PI_CUDA(cudaMemcpy(b->d_vent, ent.data(), ent.size() * sizeof(int64_t), cudaMemcpyHostToDevice));
  PI_CUDA(cudaMemcpy(b->d_vmap, vmap.data(), vmap.size() * sizeof(int64_t), cudaMemcpyHostToDevice));
  return PI_OK;
}
struct BatchGuard { pi_batch b = nullptr; ~BatchGuard() { if (b) pi_batch_destroy(b); } };

// Order `idx` (points p[3 i..3 i + 2]) into groups of `group` consecutive
// entries that are compact in space: recursive bisection at the widest
// coordinate, the lower part taking half the groups (so that every group but
// the last is full).  Ties are broken by index, so the order is deterministic.
void bisect_groups(std::vector<int>& idx, size_t lo, size_t hi, const std::vector<double>& p, size_t group) {
  if (hi - lo <= group) return;
  double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (size_t t = lo; t < hi; ++t)
    for (int c = 0; c < 3; ++c) { mn[c] = std::min(mn[c], p[3 * idx[t] + c]); mx[c] = std::max(mx[c], p[3 * idx[t] + c]); }
  int ax = 0;
  for (int c = 1; c < 3; ++c) if (mx[c] - mn[c] > mx[ax] - mn[ax]) ax = c;
  std::sort(idx.begin() + lo, idx.begin() + hi, [&](int a, int b) {
    return p[3 * a + ax] < p[3 * b + ax] || (p[3 * a + ax] == p[3 * b + ax] && a < b);
  });
  const size_t ng = (hi - lo + group - 1) / group, mid = lo + (ng / 2) * group;
  bisect_groups(idx, lo, mid, p, group);
  bisect_groups(idx, mid, hi, p, group);
}

// The evaluated directions of a k-grid (KGridDev::dpair).  v: the M
// direction vectors (unit directions of a tensor grid, whole k vectors
// otherwise).  Two directions pair when d_j + d_j' vanishes to 1e-10 |d_j|
// (Lebedev tables list exact antipodes, rounded from their angles: 7e-16).
// Each pair is evaluated at the member in the upper half-space (z > 0, then
// y > 0, then x > 0); unpaired directions are evaluated alone.  With pairs
// on a tensor grid the evaluated directions are ordered in compact groups
// of 32 (one warp's lanes), so that a warp's lanes see similar projections
// of an element and take the same branches; without pairs the identity order
// is kept.
std::vector<int2> direction_pairs(const std::vector<double>& v, int64_t M, bool cluster) {
  // candidates by the coordinate with the widest range (a planar set of k
  // vectors would put every point at one value of the others)
  int ax = 0;
  {
    double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int64_t j = 0; j < M; ++j)
      for (int c = 0; c < 3; ++c) { mn[c] = std::min(mn[c], v[3 * j + c]); mx[c] = std::max(mx[c], v[3 * j + c]); }
    for (int c = 1; c < 3; ++c) if (mx[c] - mn[c] > mx[ax] - mn[ax]) ax = c;
  }
  std::vector<int> byx(M), mate(M, -1);
  std::iota(byx.begin(), byx.end(), 0);
  std::sort(byx.begin(), byx.end(),
            [&](int a, int b) { return v[3 * a + ax] < v[3 * b + ax] || (v[3 * a + ax] == v[3 * b + ax] && a < b); });
  std::vector<double> xs(M);
  for (int64_t t = 0; t < M; ++t) xs[t] = v[3 * byx[t] + ax];
  int64_t n_pairs = 0;
  for (int64_t j = 0; j < M; ++j) {
    if (mate[j] >= 0) continue;
    const double* a = &v[3 * j];
    const double nrm = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
    if (!(nrm > 0) || !std::isfinite(nrm)) continue;
    const double tol = 1e-10 * nrm;
    int best = -1;
    double best_d = tol;
    for (auto it = std::lower_bound(xs.begin(), xs.end(), -a[ax] - tol); it != xs.end() && *it <= -a[ax] + tol; ++it) {
      const int i = byx[it - xs.begin()];
      if (i == j || mate[i] >= 0) continue;
      const double* b = &v[3 * i];
      const double d = std::sqrt((a[0] + b[0]) * (a[0] + b[0]) + (a[1] + b[1]) * (a[1] + b[1]) + (a[2] + b[2]) * (a[2] + b[2]));
      if (d <= best_d) { best = i; best_d = d; }
    }
    if (best >= 0) { mate[j] = best; mate[best] = (int)j; ++n_pairs; }
  }
  std::vector<int2> out;
  if (n_pairs == 0) {
    out.resize(M);
    for (int64_t j = 0; j < M; ++j) out[j] = make_int2((int)j, -1);
    return out;
  }
  auto upper = [&](int j) {
    const double* a = &v[3 * j];
    return a[2] > 0 || (a[2] == 0 && (a[1] > 0 || (a[1] == 0 && a[0] > 0)));
  };
  std::vector<int> eval;
  eval.reserve(M - n_pairs);
  for (int64_t j = 0; j < M; ++j) {  // exactly one member of each pair
    const int m = mate[j];
    const bool uj = upper((int)j), um = m >= 0 && upper(m);
    if (m < 0 || (uj != um ? uj : j < m)) eval.push_back((int)j);
  }
  if (cluster) {
    std::vector<double> u(3 * M);
    for (int64_t j = 0; j < M; ++j) {
      const double* a = &v[3 * j];
      const double nrm = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
      for (int c = 0; c < 3; ++c) u[3 * j + c] = nrm > 0 ? a[c] / nrm : 0.0;
    }
    bisect_groups(eval, 0, eval.size(), u, 32);
  }
  out.resize(eval.size());
  for (size_t t = 0; t < eval.size(); ++t) out[t] = make_int2(eval[t], mate[eval[t]]);
  return out;
}

// Detects the reference's tensor order q = r*M + j (kgrid.hpp:33-45); *M is
// the number of directions of a tensor grid, Q otherwise.
bool grid_layout(const double* dirs, const double* kmag, int64_t Q, int64_t* M_out) {
  int64_t M = 1;
  while (M < Q && kmag[M] == kmag[0]) ++M;
  bool tensor = (Q % M == 0);
  if (tensor) {
    for (int64_t q = 0; q < Q && tensor; ++q) {
      const int64_t j = q % M, r0 = q - j;
      tensor = kmag[q] == kmag[r0] && dirs[3 * q] == dirs[3 * j] && dirs[3 * q + 1] == dirs[3 * j + 1] &&
               dirs[3 * q + 2] == dirs[3 * j + 2];
    }
  }
  if (tensor && M > 0x7fffffff) tensor = false;
  *M_out = tensor ? M : Q;
  return tensor;
}

// The stored direction vectors: unit directions of a tensor grid, whole k
// vectors (direction times |k|) otherwise.
std::vector<double> direction_vectors(const double* dirs, const double* kmag, int64_t M, bool tensor) {
  std::vector<double> dv(3 * M);
  for (int64_t j = 0; j < M; ++j)
    for (int c = 0; c < 3; ++c) dv[3 * j + c] = tensor ? dirs[3 * j + c] : dirs[3 * j + c] * kmag[j];
  return dv;
}

}  // namespace

extern "C" {

int pi_kgrid_create(const double* dirs, const double* kmag, const double* w, int64_t Q, pi_kgrid* out) {
  if (!out) return fail(PI_ERR_INVALID_ARGUMENT, "pi_kgrid_create: null output");
  *out = nullptr;
  if (Q <= 0 || !dirs || !kmag) return fail(PI_ERR_INVALID_ARGUMENT, "pi_kgrid_create: empty k-grid");
  if (Q > (int64_t)1 << 31) return fail(PI_ERR_UNSUPPORTED, "pi_kgrid_create: more than 2^31 nodes");
  std::unique_ptr<pi_kgrid_s> kg(new pi_kgrid_s());
  int64_t M = 0;
  const bool tensor = grid_layout(dirs, kmag, Q, &M);
  const int64_t L = tensor ? Q / M : 1;
  std::vector<float4> dh(M), dl(M);
  std::vector<float2> km(L), kt(L), k256(L), tab(256);
  const std::vector<double> dv = direction_vectors(dirs, kmag, M, tensor);
  for (int64_t j = 0; j < M; ++j) {
    double d[3];
    for (int c = 0; c < 3; ++c) d[c] = dv[3 * j + c];
    const double nrm = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    float h[3], l[3];
    for (int c = 0; c < 3; ++c) { h[c] = (float)d[c]; l[c] = (float)(d[c] - (double)h[c]); }
    dh[j] = make_float4(h[0], h[1], h[2], nrm > 0 ? (float)(1.0 / nrm) : 0.f);
    dl[j] = make_float4(l[0], l[1], l[2], (float)nrm);
  }
  for (int64_t r = 0; r < L; ++r) {
    const double k = tensor ? kmag[r * M] : 1.0;
    const float h = (float)k;
    km[r] = make_float2(h, (float)(k - (double)h));
    const double u = k / (2.0 * 3.14159265358979323846);
    const float uh = (float)u;
    kt[r] = make_float2(uh, (float)(u - (double)uh));
    const double v = u * 256.0;
    const float vh = (float)v;
    k256[r] = make_float2(vh, (float)(v - (double)vh));
  }
  for (int j = 0; j < 256; ++j) {
    const double a = 2.0 * 3.14159265358979323846 * j / 256.0;
    tab[j] = make_float2((float)std::cos(a), (float)std::sin(a));
  }
  std::vector<float> sw(Q), sg(Q);
  kg->w.resize(Q);
  bool allpos = true;
  for (int64_t q = 0; q < Q; ++q) {
    const double wq = w ? w[q] : 1.0;
    kg->w[q] = wq;
    sw[q] = (float)std::sqrt(std::fabs(wq));
    sg[q] = wq < 0 ? -1.f : 1.f;
    if (wq < 0) allpos = false;
  }
  const size_t o_dh = 0, o_dl = align16(o_dh + M * sizeof(float4)), o_km = align16(o_dl + M * sizeof(float4)),
               o_sw = align16(o_km + L * sizeof(float2)), o_sg = align16(o_sw + Q * sizeof(float)),
               o_kt = align16(o_sg + Q * sizeof(float)), o_k256 = align16(o_kt + L * sizeof(float2)),
               o_tab = align16(o_k256 + L * sizeof(float2)), o_pair = align16(o_tab + 256 * sizeof(float2));
  const std::vector<int2> pairs = direction_pairs(dv, M, tensor);
  const int64_t Me = (int64_t)pairs.size();
  {  // every direction is written exactly once, as evaluated or as a mirror
    std::vector<char> seen(M, 0);
    bool ok = true;
    for (const int2& pr : pairs) {
      if (pr.x < 0 || pr.x >= M || pr.y < -1 || pr.y >= M || pr.y == pr.x) { ok = false; break; }
      ok = ok && !seen[pr.x]++;
      if (pr.y >= 0) ok = ok && !seen[pr.y]++;
    }
    for (int64_t j = 0; j < M && ok; ++j) ok = seen[j] == 1;
    if (!ok) return fail(PI_ERR_UNSUPPORTED, "pi_kgrid_create: bad direction pairing");
  }
  const size_t total = align16(o_pair + Me * sizeof(int2));
  std::vector<unsigned char> host(total, 0);
  std::memcpy(host.data() + o_dh, dh.data(), M * sizeof(float4));
  std::memcpy(host.data() + o_dl, dl.data(), M * sizeof(float4));
  std::memcpy(host.data() + o_km, km.data(), L * sizeof(float2));
  std::memcpy(host.data() + o_sw, sw.data(), Q * sizeof(float));
  std::memcpy(host.data() + o_sg, sg.data(), Q * sizeof(float));
  std::memcpy(host.data() + o_kt, kt.data(), L * sizeof(float2));
  std::memcpy(host.data() + o_k256, k256.data(), L * sizeof(float2));
  std::memcpy(host.data() + o_tab, tab.data(), 256 * sizeof(float2));
  std::memcpy(host.data() + o_pair, pairs.data(), Me * sizeof(int2));
  PI_CUDA(cudaMalloc(&kg->d_mem, total));
  cudaError_t e = cudaMemcpy(kg->d_mem, host.data(), total, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) { cudaFree(kg->d_mem); return cuda_fail(e, "pi_kgrid_create upload"); }
  unsigned char* base = static_cast<unsigned char*>(kg->d_mem);
  kg->Q = Q; kg->M = (int)M; kg->L = (int)L; kg->tensor = tensor; kg->all_positive = allpos;
  kg->dev.Q = Q; kg->dev.M = (int)M; kg->dev.L = (int)L;
  kg->dev.dir_hi = reinterpret_cast<const float4*>(base + o_dh);
  kg->dev.dir_lo = reinterpret_cast<const float4*>(base + o_dl);
  kg->dev.kmag = reinterpret_cast<const float2*>(base + o_km);
  kg->dev.sqrtw = reinterpret_cast<const float*>(base + o_sw);
  kg->dev.sign = reinterpret_cast<const float*>(base + o_sg);
  kg->dev.kturn = reinterpret_cast<const float2*>(base + o_kt);
  kg->dev.kt256 = reinterpret_cast<const float2*>(base + o_k256);
  kg->dev.cis_tab = reinterpret_cast<const float2*>(base + o_tab);
  kg->dev.dpair = reinterpret_cast<const int2*>(base + o_pair);
  kg->dev.Me = (int)Me;
  kg->Me = (int)Me;
  *out = kg.release();
  return PI_OK;
}

int pi_kgrid_direction_pairs(const double* dirs, const double* kmag, int64_t Q, int32_t* out, int64_t cap,
                             int64_t* n_eval) {
  if (Q <= 0 || !dirs || !kmag || !n_eval || (cap > 0 && !out))
    return fail(PI_ERR_INVALID_ARGUMENT, "pi_kgrid_direction_pairs: bad arguments");
  if (Q > (int64_t)1 << 31) return fail(PI_ERR_UNSUPPORTED, "pi_kgrid_direction_pairs: more than 2^31 nodes");
  int64_t M = 0;
  const bool tensor = grid_layout(dirs, kmag, Q, &M);
  const std::vector<int2> pairs = direction_pairs(direction_vectors(dirs, kmag, M, tensor), M, tensor);
  *n_eval = (int64_t)pairs.size();
  for (int64_t t = 0; t < std::min<int64_t>(cap, *n_eval); ++t) { out[2 * t] = pairs[t].x; out[2 * t + 1] = pairs[t].y; }
  return cap >= *n_eval ? PI_OK : fail(PI_ERR_WORKSPACE_TOO_SMALL, "pi_kgrid_direction_pairs: output too small");
}

int pi_kgrid_destroy(pi_kgrid kg) {
  if (!kg) return PI_OK;
  if (kg->d_mem) cudaFree(kg->d_mem);
  delete kg;
  return PI_OK;
}

int pi_kgrid_info(pi_kgrid kg, int64_t* Q, int64_t* n_dirs, int64_t* n_radial) {
  if (!kg) return fail(PI_ERR_INVALID_ARGUMENT, "pi_kgrid_info: null handle");
  if (Q) *Q = kg->Q;
  if (n_dirs) *n_dirs = kg->M;
  if (n_radial) *n_radial = kg->L;
  return PI_OK;
}

}  // extern "C"

namespace {

// pi_batch_create; with share_sources, objects that name the same element
// array (pointer, count and kind) share one copy of their reference-layout
// source on the device (instances of one mesh under different DoFs upload
// it once).  Only batches whose sources are never replaced share them: the
// host entry points' temporary batches.
int batch_create_impl(const pi_object* objs, int n, int on_device, cudaStream_t s, bool share_sources,
                      pi_batch* out) {
  if (!out) return fail(PI_ERR_INVALID_ARGUMENT, "pi_batch_create: null output");
  *out = nullptr;
  if (n < 0 || (n > 0 && !objs)) return fail(PI_ERR_INVALID_ARGUMENT, "pi_batch_create: bad object array");
  std::unique_ptr<pi_batch_s> b(new pi_batch_s());
  b->n_obj = n;
  b->info.resize(n);
  size_t src_bytes = 0;
  int64_t dof_count = 0;
  std::vector<char> owns_src(n, 1);  // whether object i's source is copied (first of its array)
  std::unordered_map<const void*, int> first_of;  // element array -> first object naming it
  for (int i = 0; i < n; ++i) {
    int rc = validate_object(objs[i], i);
    if (rc) return rc;
    HostObjInfo& in = b->info[i];
    in.geom_type = objs[i].geom_type; in.dof_type = objs[i].dof_type;
    in.n_elems = objs[i].n_elems; in.n_dofs = objs[i].n_dofs;
    int same = -1;
    if (share_sources && in.n_elems > 0) {
      auto it = first_of.find(objs[i].elems);
      if (it == first_of.end()) first_of.emplace(objs[i].elems, i);
      else if (objs[it->second].n_elems == in.n_elems && objs[it->second].geom_type == in.geom_type)
        same = it->second;
    }
    if (same >= 0) {
      in.src_off = b->info[same].src_off;
      owns_src[i] = 0;
    } else {
      in.src_off = (int64_t)src_bytes;
      src_bytes = align16(src_bytes + (size_t)in.n_elems * elem_bytes(in.geom_type));
    }
    in.dof_off = dof_count;
    dof_count += in.n_dofs;
    if (in.geom_type == PI_GEOM_TRIANGLE) { in.pool_off = b->n_tri; b->n_tri += in.n_elems; }
    else { in.pool_off = b->n_surf; b->n_surf += in.n_elems; }
    if (!on_device && in.dof_type == PI_DOF_TRIANGLE_MESH) {
      const pi_tri_packed* T = static_cast<const pi_tri_packed*>(objs[i].elems);
      const int64_t nv = in.n_dofs / 3;
      for (int64_t f = 0; f < in.n_elems; ++f)
        if (T[f].vid0 >= nv || T[f].vid1 >= nv || T[f].vid2 >= nv)
          return fail(PI_ERR_INVALID_ARGUMENT, "TriangleMeshDoF vertex index beyond the DoF vector");
    }
  }
  b->order.resize(n);
  std::iota(b->order.begin(), b->order.end(), 0);
  std::stable_sort(b->order.begin(), b->order.end(),
                   [&](int a, int c) { return b->info[a].n_elems > b->info[c].n_elems; });
  auto cleanup = [&]() {
    cudaFree(b->d_block); cudaFree(b->d_vrow); cudaFree(b->d_vent); cudaFree(b->d_vmap);
  };
  // one device allocation carved into the batch's buffers (256-byte aligned)
  const size_t sizes[9] = {std::max<size_t>(src_bytes, 16),
                           std::max<size_t>(dof_count * sizeof(double), 16),
                           std::max<size_t>(b->n_tri * 3 * sizeof(float4), 16),
                           std::max<size_t>(b->n_surf * 2 * sizeof(float4), 16),
                           std::max<size_t>(b->n_tri * sizeof(float4), 16),
                           std::max<size_t>(b->n_surf * sizeof(float4), 16),
                           std::max<size_t>(b->n_surf * sizeof(float4), 16),
                           std::max<size_t>(n * sizeof(ObjDev), 16),
                           std::max<size_t>(n * sizeof(int32_t), 16)};
  size_t offs[9], total = 0;
  for (int i = 0; i < 9; ++i) {
    offs[i] = total;
    total += (sizes[i] + 255) & ~(size_t)255;
  }
  cudaError_t e = cudaMalloc(&b->d_block, total);
  if (e != cudaSuccess) { cleanup(); return cuda_fail(e, "pi_batch_create allocation"); }
  unsigned char* blk = static_cast<unsigned char*>(b->d_block);
  b->d_src = blk + offs[0];
  b->d_dofs = reinterpret_cast<double*>(blk + offs[1]);
  b->d_tri_pool = reinterpret_cast<float4*>(blk + offs[2]);
  b->d_surf_pool = reinterpret_cast<float4*>(blk + offs[3]);
  b->d_tri_lo = reinterpret_cast<float4*>(blk + offs[4]);
  b->d_surf_lo = reinterpret_cast<float4*>(blk + offs[5]);
  b->d_surf_nref = reinterpret_cast<float4*>(blk + offs[6]);
  b->d_objs = reinterpret_cast<ObjDev*>(blk + offs[7]);
  b->d_order = reinterpret_cast<int32_t*>(blk + offs[8]);
  if (on_device) {
    for (int i = 0; i < n && e == cudaSuccess; ++i) {
      const HostObjInfo& in = b->info[i];
      if (in.n_elems && owns_src[i])
        e = cudaMemcpyAsync(static_cast<unsigned char*>(b->d_src) + in.src_off, objs[i].elems,
                            in.n_elems * elem_bytes(in.geom_type), cudaMemcpyDeviceToDevice, s);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(b->d_dofs + in.dof_off, objs[i].dofs, in.n_dofs * sizeof(double),
                            cudaMemcpyDeviceToDevice, s);
    }
  } else {
    // elements straight from the caller's arrays (one copy per object, no
    // host staging); the DoF vectors are small and go as one copy
    std::vector<double> hd(std::max<int64_t>(dof_count, 1));
    for (int i = 0; i < n && e == cudaSuccess; ++i) {
      const HostObjInfo& in = b->info[i];
      if (in.n_elems && owns_src[i])
        e = cudaMemcpyAsync(static_cast<unsigned char*>(b->d_src) + in.src_off, objs[i].elems,
                            in.n_elems * elem_bytes(in.geom_type), cudaMemcpyHostToDevice, s);
      std::memcpy(hd.data() + in.dof_off, objs[i].dofs, in.n_dofs * sizeof(double));
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(b->d_dofs, hd.data(), dof_count * sizeof(double), cudaMemcpyHostToDevice, s);
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(b->d_order, b->order.data(), n * sizeof(int32_t), cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) { cleanup(); return cuda_fail(e, "pi_batch_create upload"); }
  int rc0 = build_vertex_csr(b.get(), objs, on_device, s);
  if (rc0) { cleanup(); return rc0; }
  int rc = launch_prepare(b.get(), -1, s);
  if (rc) { cleanup(); return rc; }
  *out = b.release();
  return PI_OK;
}

}  // namespace

extern "C" {

int pi_batch_create(const pi_object* objs, int n, int on_device, pi_stream stream, pi_batch* out) {
  return batch_create_impl(objs, n, on_device, reinterpret_cast<cudaStream_t>(stream), false, out);
}

int pi_batch_set_dofs(pi_batch b, int index, const double* d_dofs, pi_stream stream) {
  if (!b || index < 0 || index >= b->n_obj || !d_dofs)
    return fail(PI_ERR_INVALID_ARGUMENT, "pi_batch_set_dofs: bad arguments");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const HostObjInfo& in = b->info[index];
  PI_CUDA(cudaMemcpyAsync(b->d_dofs + in.dof_off, d_dofs, in.n_dofs * sizeof(double), cudaMemcpyDeviceToDevice, s));
  return launch_prepare(b, index, s);
}

int pi_batch_set_all_dofs(pi_batch b, const double* d_dofs, pi_stream stream) {
  if (!b || (!d_dofs && b->n_obj > 0)) return fail(PI_ERR_INVALID_ARGUMENT, "pi_batch_set_all_dofs: bad arguments");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const int64_t nd = dof_gradient_size(b);
  if (nd) PI_CUDA(cudaMemcpyAsync(b->d_dofs, d_dofs, nd * sizeof(double), cudaMemcpyDeviceToDevice, s));
  return launch_prepare(b, -1, s);
}

int pi_batch_prepare(pi_batch b, pi_stream stream) {
  if (!b) return fail(PI_ERR_INVALID_ARGUMENT, "pi_batch_prepare: null batch");
  return launch_prepare(b, -1, reinterpret_cast<cudaStream_t>(stream));
}

int pi_batch_destroy(pi_batch b) {
  if (!b) return PI_OK;
  cudaFree(b->d_block); cudaFree(b->d_vrow); cudaFree(b->d_vent); cudaFree(b->d_vmap);
  delete b;
  return PI_OK;
}

int pi_batch_count(pi_batch b, int* n) {
  if (!b || !n) return fail(PI_ERR_INVALID_ARGUMENT, "pi_batch_count: bad arguments");
  *n = b->n_obj;
  return PI_OK;
}

int pi_form_factors(pi_kgrid kg, pi_batch b, int scale_sqrt_w, void* d_J, pi_stream stream) {
  if (!kg || !b || (!d_J && b->n_obj > 0)) return fail(PI_ERR_INVALID_ARGUMENT, "pi_form_factors: bad arguments");
  return launch_form_factors(kg, b, scale_sqrt_w, static_cast<float2*>(d_J), reinterpret_cast<cudaStream_t>(stream));
}

int pi_form_factors_rowmax(pi_kgrid kg, pi_batch b, int scale_sqrt_w, void* d_J, float* d_row_amax,
                           pi_stream stream) {
  if (!kg || !b || ((!d_J || !d_row_amax) && b->n_obj > 0))
    return fail(PI_ERR_INVALID_ARGUMENT, "pi_form_factors_rowmax: bad arguments");
  return launch_form_factors(kg, b, scale_sqrt_w, static_cast<float2*>(d_J), reinterpret_cast<cudaStream_t>(stream),
                             d_row_amax);
}

int pi_contract_workspace_size(pi_kgrid kg, int n, int precision, size_t* bytes) {
  if (!kg || !bytes || n < 0) return fail(PI_ERR_INVALID_ARGUMENT, "pi_contract_workspace_size: bad arguments");
  if (precision == PI_CONTRACT_FP32) *bytes = contract_fp32_ws_bytes(kg->Q, n);
  else if (precision == PI_CONTRACT_BF16X3) *bytes = group_single_ws_bytes(kg->Q, n, GROUP_OP_BF16);
  else if (precision == PI_CONTRACT_FP16X3) *bytes = group_single_ws_bytes(kg->Q, n, GROUP_OP_F16);
  else if (precision == PI_CONTRACT_TF32X3) *bytes = contract_tc_ws_bytes(kg->Q, n, 1);
  else return fail(PI_ERR_INVALID_ARGUMENT, "unknown contraction precision");
  return PI_OK;
}

int pi_contract_rowmax(pi_kgrid kg, const void* d_Jw, const float* d_row_amax, int n, int precision, double* d_V,
                       void* d_ws, size_t ws_bytes, pi_stream stream) {
  if (!kg || n < 0 || (n > 0 && (!d_Jw || !d_V))) return fail(PI_ERR_INVALID_ARGUMENT, "pi_contract: bad arguments");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const float2* J = static_cast<const float2*>(d_Jw);
  if (precision == PI_CONTRACT_FP32) return launch_contract_fp32(kg, J, n, d_V, d_ws, ws_bytes, s);
  if (precision == PI_CONTRACT_BF16X3 || precision == PI_CONTRACT_TF32X3 || precision == PI_CONTRACT_FP16X3) {
    if (!kg->all_positive)
      return fail(PI_ERR_UNSUPPORTED, "the tensor-core contractions need non-negative quadrature weights");
    if (precision != PI_CONTRACT_TF32X3)
      return launch_group_single(J, kg->Q, n, precision == PI_CONTRACT_FP16X3 ? GROUP_OP_F16 : GROUP_OP_BF16, d_V,
                                 d_ws, ws_bytes, INV_8PI3, s, d_row_amax);
    return launch_contract_tc(kg, J, n, 1, d_V, d_ws, ws_bytes, s);
  }
  return fail(PI_ERR_INVALID_ARGUMENT, "unknown contraction precision");
}

int pi_contract(pi_kgrid kg, const void* d_Jw, int n, int precision, double* d_V, void* d_ws, size_t ws_bytes,
                pi_stream stream) {
  return pi_contract_rowmax(kg, d_Jw, nullptr, n, precision, d_V, d_ws, ws_bytes, stream);
}

int pi_contract_error(int precision, const void* d_ws, pi_stream stream) {
  if (precision == PI_CONTRACT_FP32) return PI_OK;  // no waits, no error word
  if (precision != PI_CONTRACT_BF16X3 && precision != PI_CONTRACT_TF32X3 && precision != PI_CONTRACT_FP16X3)
    return fail(PI_ERR_INVALID_ARGUMENT, "pi_contract_error: unknown contraction precision");
  if (!d_ws) return fail(PI_ERR_INVALID_ARGUMENT, "pi_contract_error: null workspace");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  int code = 0;
  PI_CUDA(cudaMemcpyAsync(&code, d_ws, sizeof(int), cudaMemcpyDeviceToHost, s));
  PI_CUDA(cudaStreamSynchronize(s));
  if (code == 0) return PI_OK;
  static const char* group_roles[] = {"", "loader", "converter", "MMA issuer", "epilogue", "work-item capacity"};
  static const char* tf32_roles[] = {"", "converter", "MMA issuer", "epilogue", "loader"};
  const char* role = precision == PI_CONTRACT_TF32X3 ? (code >= 1 && code <= 4 ? tf32_roles[code] : "unknown role")
                                                     : (code >= 1 && code <= 5 ? group_roles[code] : "unknown role");
  char buf[160];
  snprintf(buf, sizeof buf, "tensor-core contraction: a bounded wait of the %s expired (device code %d); V holds NaN",
           role, code);
  return fail(code == 5 ? PI_ERR_WORKSPACE_TOO_SMALL : PI_ERR_TIMEOUT, buf);
}

int pi_test_set_contract_faults(int64_t wait_cycles, int64_t starve_chunk) {
  group_test_set_faults((long long)wait_cycles, (long long)starve_chunk);
  return PI_OK;
}

int pi_batch_set_elements(pi_batch b, int index, const void* d_elems, pi_stream stream) {
  if (!b || index < 0 || index >= b->n_obj || (!d_elems && b->info[index].n_elems > 0))
    return fail(PI_ERR_INVALID_ARGUMENT, "pi_batch_set_elements: bad arguments");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const HostObjInfo& in = b->info[index];
  if (in.n_elems)
    PI_CUDA(cudaMemcpyAsync(static_cast<unsigned char*>(b->d_src) + in.src_off, d_elems,
                            in.n_elems * elem_bytes(in.geom_type), cudaMemcpyDeviceToDevice, s));
  return launch_prepare(b, index, s);
}

int pi_batch_layout(pi_batch b, int index, int64_t* pool_offset, int64_t* n_elems, int64_t* dof_offset) {
  if (!b || index < 0 || index >= b->n_obj) return fail(PI_ERR_INVALID_ARGUMENT, "pi_batch_layout: bad arguments");
  const HostObjInfo& in = b->info[index];
  int64_t dof = 0;
  for (int i = 0; i < index; ++i) dof += b->info[i].n_dofs;
  if (pool_offset) *pool_offset = in.pool_off;
  if (n_elems) *n_elems = in.n_elems;
  if (dof_offset) *dof_offset = dof;
  return PI_OK;
}

int pi_adjoint_workspace_size(pi_kgrid kg, pi_batch b, size_t* bytes) {
  if (!kg || !b || !bytes) return fail(PI_ERR_INVALID_ARGUMENT, "pi_adjoint_workspace_size: bad arguments");
  *bytes = adjoint_ws_bytes(kg, b);
  return PI_OK;
}

int pi_element_gradients(pi_kgrid kg, pi_batch b, const void* d_Jw, const double* W, float* d_tri_grad,
                         float* d_surf_grad, void* d_ws, size_t ws_bytes, pi_stream stream) {
  if (!kg || !b || !W || (b->n_obj > 0 && !d_Jw)) return fail(PI_ERR_INVALID_ARGUMENT, "pi_element_gradients: bad arguments");
  if (b->n_obj == 0) return PI_OK;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  float *tg = nullptr, *sg = nullptr;
  int rc = launch_adjoint_elements(kg, b, static_cast<const float2*>(d_Jw), W, &tg, &sg, d_ws, ws_bytes, s);
  if (rc) return rc;
  if (d_tri_grad && b->n_tri)
    PI_CUDA(cudaMemcpyAsync(d_tri_grad, tg, b->n_tri * 9 * sizeof(float), cudaMemcpyDeviceToDevice, s));
  if (d_surf_grad && b->n_surf)
    PI_CUDA(cudaMemcpyAsync(d_surf_grad, sg, b->n_surf * 12 * sizeof(float), cudaMemcpyDeviceToDevice, s));
  return PI_OK;
}

int pi_dof_gradients(pi_kgrid kg, pi_batch b, const void* d_Jw, const double* W, double* d_grad, void* d_ws,
                     size_t ws_bytes, pi_stream stream) {
  if (!kg || !b || !W || (b->n_obj > 0 && (!d_Jw || !d_grad)))
    return fail(PI_ERR_INVALID_ARGUMENT, "pi_dof_gradients: bad arguments");
  if (b->n_obj == 0) return PI_OK;
  return launch_dof_gradients(kg, b, static_cast<const float2*>(d_Jw), W, d_grad, d_ws, ws_bytes,
                              reinterpret_cast<cudaStream_t>(stream));
}

int pi_volume_matrix_host(const pi_object* objs, int n, const double* dirs, const double* kmag, const double* w,
                          int64_t Q, int flags, int precision, double* V_out) {
  if (n < 0 || (n > 0 && (!objs || !V_out)) || !dirs || !kmag || !w)
    return fail(PI_ERR_INVALID_ARGUMENT, "pi_volume_matrix_host: bad arguments");
  if (flags & ~PI_VOLUME_ONLY)
    return fail(PI_ERR_UNSUPPORTED, "pi_volume_matrix_host computes volumes only; use the adjoint entry points");
  if (n == 0) return PI_OK;
  cudaStream_t s = cudaStreamPerThread;
  KGridGuard kg;
  int rc = pi_kgrid_create(dirs, kmag, w, Q, &kg.k);
  if (rc) return rc;
  BatchGuard b;
  rc = batch_create_impl(objs, n, 0, s, true, &b.b);
  if (rc) return rc;
  size_t ws_bytes = 0;
  rc = pi_contract_workspace_size(kg.k, n, precision, &ws_bytes);
  if (rc) return rc;
  DevBuf J, ws, V, amax;
  if ((rc = J.alloc((size_t)n * Q * sizeof(float2), s)) || (rc = ws.alloc(ws_bytes, s)) ||
      (rc = V.alloc((size_t)n * n * sizeof(double), s)) || (rc = amax.alloc((size_t)n * sizeof(float), s)))
    return rc;
  float* row_amax = static_cast<float*>(amax.p);
  rc = pi_form_factors_rowmax(kg.k, b.b, 1, J.p, row_amax, reinterpret_cast<pi_stream>(s));
  if (rc) return rc;
  rc = pi_contract_rowmax(kg.k, J.p, row_amax, n, precision, static_cast<double*>(V.p), ws.p, ws_bytes,
                          reinterpret_cast<pi_stream>(s));
  if (rc) return rc;
  PI_CUDA(cudaMemcpyAsync(V_out, V.p, (size_t)n * n * sizeof(double), cudaMemcpyDeviceToHost, s));
  PI_CUDA(cudaStreamSynchronize(s));
  return PI_OK;
}

int pi_pair_volume_host(const pi_object* o1, const pi_object* o2, const double* dirs, const double* kmag,
                        const double* w, int64_t Q, double* volume) {
  if (!o1 || !o2 || !volume) return fail(PI_ERR_INVALID_ARGUMENT, "pi_pair_volume_host: bad arguments");
  pi_object objs[2] = {*o1, *o2};
  double V[4];
  int rc = pi_volume_matrix_host(objs, 2, dirs, kmag, w, Q, PI_VOLUME_ONLY, PI_CONTRACT_FP32, V);
  if (rc) return rc;
  *volume = V[1];
  return PI_OK;
}

// Shared body of the gradient drop-ins: volumes of all pairs plus, for every
// j in `cols`, dV_ij/dtheta_i for all i (one adjoint pass with C = ones in
// column j, i.e. cotangent B_i = A_j for every i).
static int volume_and_grads_host(const pi_object* objs, int n, const double* dirs, const double* kmag,
                                 const double* w, int64_t Q, double* V_out, const std::vector<int>& cols,
                                 std::vector<std::vector<double>>* grads) {
  cudaStream_t s = cudaStreamPerThread;
  KGridGuard kg;
  int rc = pi_kgrid_create(dirs, kmag, w, Q, &kg.k);
  if (rc) return rc;
  BatchGuard b;
  rc = batch_create_impl(objs, n, 0, s, true, &b.b);
  if (rc) return rc;
  size_t ws_c = 0, ws_a = 0;
  if ((rc = pi_contract_workspace_size(kg.k, n, PI_CONTRACT_FP32, &ws_c)) || (rc = pi_adjoint_workspace_size(kg.k, b.b, &ws_a)))
    return rc;
  const int64_t ng = dof_gradient_size(b.b);
  DevBuf J, ws, V, G;
  if ((rc = J.alloc((size_t)n * Q * sizeof(float2), s)) || (rc = ws.alloc(std::max(ws_c, ws_a), s)) ||
      (rc = V.alloc((size_t)n * n * sizeof(double), s)) || (rc = G.alloc((size_t)std::max<int64_t>(ng, 1) * sizeof(double), s)))
    return rc;
  if ((rc = pi_form_factors(kg.k, b.b, 1, J.p, reinterpret_cast<pi_stream>(s)))) return rc;
  if ((rc = pi_contract(kg.k, J.p, n, PI_CONTRACT_FP32, static_cast<double*>(V.p), ws.p, std::max(ws_c, ws_a),
                        reinterpret_cast<pi_stream>(s))))
    return rc;
  PI_CUDA(cudaMemcpyAsync(V_out, V.p, (size_t)n * n * sizeof(double), cudaMemcpyDeviceToHost, s));
  grads->assign(cols.size(), std::vector<double>(ng));
  std::vector<double> C((size_t)n * n);
  for (size_t c = 0; c < cols.size(); ++c) {
    std::fill(C.begin(), C.end(), 0.0);
    for (int i = 0; i < n; ++i) C[(size_t)i * n + cols[c]] = 1.0;  // B_i = A_col for every i
    if ((rc = pi_dof_gradients(kg.k, b.b, J.p, C.data(), static_cast<double*>(G.p), ws.p, std::max(ws_c, ws_a),
                               reinterpret_cast<pi_stream>(s))))
      return rc;
    PI_CUDA(cudaMemcpyAsync((*grads)[c].data(), G.p, ng * sizeof(double), cudaMemcpyDeviceToHost, s));
    PI_CUDA(cudaStreamSynchronize(s));
  }
  PI_CUDA(cudaStreamSynchronize(s));
  return PI_OK;
}

int pi_pair_volume_grad_host(const pi_object* o1, const pi_object* o2, const double* dirs, const double* kmag,
                             const double* w, int64_t Q, double* volume, double* grad1, double* grad2) {
  if (!o1 || !o2 || !volume) return fail(PI_ERR_INVALID_ARGUMENT, "pi_pair_volume_grad_host: bad arguments");
  pi_object objs[2] = {*o1, *o2};
  double V[4];
  std::vector<std::vector<double>> g;
  // column 1: B_0 = A_1 -> dV_01/dtheta_0;  column 0: B_1 = A_0 -> dV_10/dtheta_1
  int rc = volume_and_grads_host(objs, 2, dirs, kmag, w, Q, V, {1, 0}, &g);
  if (rc) return rc;
  *volume = V[1];
  if (grad1) std::copy(g[0].begin(), g[0].begin() + o1->n_dofs, grad1);
  if (grad2) std::copy(g[1].begin() + o1->n_dofs, g[1].begin() + o1->n_dofs + o2->n_dofs, grad2);
  return PI_OK;
}

int pi_volume_matrix_grad_host(const pi_object* objs, int n, const double* dirs, const double* kmag, const double* w,
                               int64_t Q, double* V_out, double* grad_out) {
  if (n <= 0 || !objs || !V_out || !grad_out) return fail(PI_ERR_INVALID_ARGUMENT, "pi_volume_matrix_grad_host: bad arguments");
  std::vector<int> cols(n);
  std::iota(cols.begin(), cols.end(), 0);
  std::vector<std::vector<double>> g;
  int rc = volume_and_grads_host(objs, n, dirs, kmag, w, Q, V_out, cols, &g);
  if (rc) return rc;
  // grad_out block (i, j) = dV_ij/dtheta_i at offset n*goff_i + j*d_i
  int64_t goff = 0;
  for (int i = 0; i < n; ++i) {
    const int64_t d = objs[i].n_dofs;
    for (int j = 0; j < n; ++j) std::copy(g[j].begin() + goff, g[j].begin() + goff + d, grad_out + n * goff + j * d);
    goff += d;
  }
  return PI_OK;
}

int pi_dof_jacobian(pi_kgrid kg, pi_batch b, void* d_G, pi_stream stream) {
  if (!kg || !b || (!d_G && dof_gradient_size(b) > 0)) return fail(PI_ERR_INVALID_ARGUMENT, "pi_dof_jacobian: bad arguments");
  return launch_jacobian(kg, b, static_cast<float2*>(d_G), reinterpret_cast<cudaStream_t>(stream));
}

// Shared body of the Hessian drop-ins.  X = [J; G] (n + D rows of sqrt|w|-scaled
// form factors and DoF Jacobian rows) and one FP32 contraction
// Re(X diag(sign w) X^H)/(8 pi^3) give, in its blocks, V (rows and columns
// < n), dV_ij/dtheta_i (row n + goff_i + a, column j) and the Gauss-Newton
// Hessian (rows and columns >= n).  Returns the full (n + D)^2 matrix on the host.
static int stacked_gram_host(const pi_object* objs, int n, const double* dirs, const double* kmag, const double* w,
                             int64_t Q, std::vector<double>* X, int64_t* D_out) {
  cudaStream_t s = cudaStreamPerThread;
  KGridGuard kg;
  int rc = pi_kgrid_create(dirs, kmag, w, Q, &kg.k);
  if (rc) return rc;
  BatchGuard b;
  rc = batch_create_impl(objs, n, 0, s, true, &b.b);
  if (rc) return rc;
  const int64_t D = dof_gradient_size(b.b), m = n + D;
  if (m > INT32_MAX) return fail(PI_ERR_UNSUPPORTED, "too many DoFs for the Hessian");
  size_t ws_bytes = 0;
  if ((rc = pi_contract_workspace_size(kg.k, (int)m, PI_CONTRACT_FP32, &ws_bytes))) return rc;
  DevBuf J, ws, H;
  if ((rc = J.alloc((size_t)m * Q * sizeof(float2), s)) || (rc = ws.alloc(ws_bytes, s)) ||
      (rc = H.alloc((size_t)m * m * sizeof(double), s)))
    return rc;
  float2* Jp = static_cast<float2*>(J.p);
  if ((rc = pi_form_factors(kg.k, b.b, 1, Jp, reinterpret_cast<pi_stream>(s)))) return rc;
  if ((rc = launch_jacobian(kg.k, b.b, Jp + (size_t)n * Q, s))) return rc;
  if ((rc = pi_contract(kg.k, Jp, (int)m, PI_CONTRACT_FP32, static_cast<double*>(H.p), ws.p, ws_bytes,
                        reinterpret_cast<pi_stream>(s))))
    return rc;
  X->resize((size_t)m * m);
  PI_CUDA(cudaMemcpyAsync(X->data(), H.p, (size_t)m * m * sizeof(double), cudaMemcpyDeviceToHost, s));
  PI_CUDA(cudaStreamSynchronize(s));
  *D_out = D;
  return PI_OK;
}

int pi_volume_matrix_hessian_host(const pi_object* objs, int n, const double* dirs, const double* kmag,
                                  const double* w, int64_t Q, double* V_out, double* grad_out, double* hess_out) {
  if (n <= 0 || !objs || !V_out || !hess_out || !dirs || !kmag || !w)
    return fail(PI_ERR_INVALID_ARGUMENT, "pi_volume_matrix_hessian_host: bad arguments");
  std::vector<double> X;
  int64_t D = 0;
  int rc = stacked_gram_host(objs, n, dirs, kmag, w, Q, &X, &D);
  if (rc) return rc;
  const int64_t m = n + D;
  std::vector<int64_t> goff(n + 1, 0);
  for (int i = 0; i < n; ++i) goff[i + 1] = goff[i] + objs[i].n_dofs;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) V_out[(size_t)i * n + j] = X[(size_t)i * m + j];
  if (grad_out)  // block (i, j) = dV_ij/dtheta_i at n * goff_i + j * d_i
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j)
        for (int64_t a = 0; a < objs[i].n_dofs; ++a)
          grad_out[n * goff[i] + j * objs[i].n_dofs + a] = X[(size_t)(n + goff[i] + a) * m + j];
  // hessian_ij blocks in (i, j) row-major order, each d_i x d_j row-major
  size_t off = 0;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j)
      for (int64_t a = 0; a < objs[i].n_dofs; ++a)
        for (int64_t c = 0; c < objs[j].n_dofs; ++c) hess_out[off++] = X[(size_t)(n + goff[i] + a) * m + n + goff[j] + c];
  return PI_OK;
}

int pi_pair_volume_hessian_host(const pi_object* o1, const pi_object* o2, const double* dirs, const double* kmag,
                                const double* w, int64_t Q, double* volume, double* grad1, double* grad2, double* H11,
                                double* H22, double* H12) {
  if (!o1 || !o2 || !volume || !H11 || !H22 || !H12)
    return fail(PI_ERR_INVALID_ARGUMENT, "pi_pair_volume_hessian_host: bad arguments");
  pi_object objs[2] = {*o1, *o2};
  std::vector<double> X;
  int64_t D = 0;
  int rc = stacked_gram_host(objs, 2, dirs, kmag, w, Q, &X, &D);
  if (rc) return rc;
  const int64_t m = 2 + D, d1 = o1->n_dofs, d2 = o2->n_dofs;
  auto at = [&](int64_t r, int64_t c) { return X[(size_t)r * m + c]; };
  *volume = at(0, 1);
  for (int64_t a = 0; a < d1; ++a) {
    if (grad1) grad1[a] = at(2 + a, 1);  // dV_12/dtheta_1: G_1 rows against A_2
    for (int64_t c = 0; c < d1; ++c) H11[a * d1 + c] = at(2 + a, 2 + c);
    for (int64_t c = 0; c < d2; ++c) H12[a * d2 + c] = at(2 + a, 2 + d1 + c);
  }
  for (int64_t a = 0; a < d2; ++a) {
    if (grad2) grad2[a] = at(2 + d1 + a, 0);
    for (int64_t c = 0; c < d2; ++c) H22[a * d2 + c] = at(2 + d1 + a, 2 + d1 + c);
  }
  return PI_OK;
}

int pi_compute_Ak(const pi_object* obj, const double* dirs, const double* kmag, int64_t Q, double* d_A_out,
                  int block_size) {
  (void)block_size;  // kept for signature parity with CudaComputeAkFunc; the kernel picks its own shape
  if (!obj || !d_A_out) return fail(PI_ERR_INVALID_ARGUMENT, "pi_compute_Ak: bad arguments");
  cudaStream_t s = cudaStreamPerThread;
  KGridGuard kg;
  int rc = pi_kgrid_create(dirs, kmag, nullptr, Q, &kg.k);
  if (rc) return rc;
  BatchGuard b;
  rc = pi_batch_create(obj, 1, 0, reinterpret_cast<pi_stream>(s), &b.b);
  if (rc) return rc;
  DevBuf J;
  if ((rc = J.alloc((size_t)Q * sizeof(float2), s))) return rc;
  rc = pi_form_factors(kg.k, b.b, 0, J.p, reinterpret_cast<pi_stream>(s));
  if (rc) return rc;
  rc = launch_to_double2(static_cast<const float2*>(J.p), Q, d_A_out, s);
  if (rc) return rc;
  // The reference wrapper returned with the result in place (it synchronised the device).
  PI_CUDA(cudaStreamSynchronize(s));
  return PI_OK;
}

int pi_compute_Ak_single(const pi_object* obj, const double* k, double* out) {
  if (!obj || !k || !out) return fail(PI_ERR_INVALID_ARGUMENT, "pi_compute_Ak_single: bad arguments");
  const double km = std::sqrt(k[0] * k[0] + k[1] * k[1] + k[2] * k[2]);
  double dir[3] = {0.0, 0.0, 0.0};
  if (km > 0) for (int c = 0; c < 3; ++c) dir[c] = k[c] / km;
  DevBuf d;
  int rc = d.alloc(2 * sizeof(double), cudaStreamPerThread);
  if (rc) return rc;
  rc = pi_compute_Ak(obj, dir, &km, 1, static_cast<double*>(d.p), 256);
  if (rc) return rc;
  PI_CUDA(cudaMemcpy(out, d.p, 2 * sizeof(double), cudaMemcpyDeviceToHost));
  return PI_OK;
}

int pi_compute_Ak_gradient(const pi_object* obj, const double* dirs, const double* kmag, int64_t Q,
                           double* d_grad_out, int block_size) {
  (void)block_size;  // kept for signature parity with the registry's gradient function
  if (!obj || !d_grad_out || Q <= 0) return fail(PI_ERR_INVALID_ARGUMENT, "pi_compute_Ak_gradient: bad arguments");
  cudaStream_t s = cudaStreamPerThread;
  KGridGuard kg;
  int rc = pi_kgrid_create(dirs, kmag, nullptr, Q, &kg.k);  // unit weights: G = dA/dtheta
  if (rc) return rc;
  BatchGuard b;
  rc = pi_batch_create(obj, 1, 0, reinterpret_cast<pi_stream>(s), &b.b);
  if (rc) return rc;
  const int64_t D = obj->n_dofs;
  DevBuf G;
  if ((rc = G.alloc((size_t)(D * Q) * sizeof(float2), s))) return rc;
  if ((rc = pi_dof_jacobian(kg.k, b.b, G.p, reinterpret_cast<pi_stream>(s)))) return rc;
  const int64_t total = D * Q;
  jacobian_to_qd_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(static_cast<const float2*>(G.p), Q, D,
                                                                        reinterpret_cast<double2*>(d_grad_out));
  PI_LAUNCHED("jacobian_to_qd_kernel");
  // The reference wrapper returned with the result in place (it synchronised the device).
  PI_CUDA(cudaStreamSynchronize(s));
  return PI_OK;
}

int pi_compute_Ak_gradient_single(const pi_object* obj, const double* k, double* out) {
  if (!obj || !k || !out || obj->n_dofs <= 0)
    return fail(PI_ERR_INVALID_ARGUMENT, "pi_compute_Ak_gradient_single: bad arguments");
  const int64_t D = obj->n_dofs;
  const double km = std::sqrt(k[0] * k[0] + k[1] * k[1] + k[2] * k[2]);
  if (km < 1e-10) {  // the reference returns zeros at k = 0 (compute_intersection_volume.cu:586)
    int rc = validate_object(*obj, 0);
    if (rc) return rc;
    std::fill(out, out + 2 * D, 0.0);
    return PI_OK;
  }
  const double dir[3] = {k[0] / km, k[1] / km, k[2] / km};
  DevBuf d;
  int rc = d.alloc((size_t)(2 * D) * sizeof(double), cudaStreamPerThread);
  if (rc) return rc;
  rc = pi_compute_Ak_gradient(obj, dir, &km, 1, static_cast<double*>(d.p), 256);
  if (rc) return rc;
  PI_CUDA(cudaMemcpy(out, d.p, (size_t)(2 * D) * sizeof(double), cudaMemcpyDeviceToHost));
  return PI_OK;
}

}  // extern "C"
