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
#include <vector>
#include "pi_internal.h"

using namespace pi;

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
struct BatchGuard { pi_batch b = nullptr; ~BatchGuard() { if (b) pi_batch_destroy(b); } };

}  // namespace

extern "C" {

int pi_kgrid_create(const double* dirs, const double* kmag, const double* w, int64_t Q, pi_kgrid* out) {
  if (!out) return fail(PI_ERR_INVALID_ARGUMENT, "pi_kgrid_create: null output");
  *out = nullptr;
  if (Q <= 0 || !dirs || !kmag) return fail(PI_ERR_INVALID_ARGUMENT, "pi_kgrid_create: empty k-grid");
  if (Q > (int64_t)1 << 31) return fail(PI_ERR_UNSUPPORTED, "pi_kgrid_create: more than 2^31 nodes");
  std::unique_ptr<pi_kgrid_s> kg(new pi_kgrid_s());
  // Detect the reference's tensor order q = r*M + j (kgrid.hpp:33-45).
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
  const int64_t L = tensor ? Q / M : 1;
  if (!tensor) M = Q;
  std::vector<float4> dh(M), dl(M);
  std::vector<float2> km(L);
  for (int64_t j = 0; j < M; ++j) {
    double d[3];
    for (int c = 0; c < 3; ++c) d[c] = tensor ? dirs[3 * j + c] : dirs[3 * j + c] * kmag[j];
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
               total = align16(o_sg + Q * sizeof(float));
  std::vector<unsigned char> host(total, 0);
  std::memcpy(host.data() + o_dh, dh.data(), M * sizeof(float4));
  std::memcpy(host.data() + o_dl, dl.data(), M * sizeof(float4));
  std::memcpy(host.data() + o_km, km.data(), L * sizeof(float2));
  std::memcpy(host.data() + o_sw, sw.data(), Q * sizeof(float));
  std::memcpy(host.data() + o_sg, sg.data(), Q * sizeof(float));
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
  *out = kg.release();
  return PI_OK;
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

int pi_batch_create(const pi_object* objs, int n, int on_device, pi_stream stream, pi_batch* out) {
  if (!out) return fail(PI_ERR_INVALID_ARGUMENT, "pi_batch_create: null output");
  *out = nullptr;
  if (n < 0 || (n > 0 && !objs)) return fail(PI_ERR_INVALID_ARGUMENT, "pi_batch_create: bad object array");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  std::unique_ptr<pi_batch_s> b(new pi_batch_s());
  b->n_obj = n;
  b->info.resize(n);
  size_t src_bytes = 0;
  int64_t dof_count = 0;
  for (int i = 0; i < n; ++i) {
    int rc = validate_object(objs[i], i);
    if (rc) return rc;
    HostObjInfo& in = b->info[i];
    in.geom_type = objs[i].geom_type; in.dof_type = objs[i].dof_type;
    in.n_elems = objs[i].n_elems; in.n_dofs = objs[i].n_dofs;
    in.src_off = (int64_t)src_bytes;
    src_bytes = align16(src_bytes + (size_t)in.n_elems * elem_bytes(in.geom_type));
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
    cudaFree(b->d_src); cudaFree(b->d_dofs); cudaFree(b->d_tri_pool); cudaFree(b->d_surf_pool);
    cudaFree(b->d_objs); cudaFree(b->d_order);
  };
  cudaError_t e = cudaSuccess;
  if (e == cudaSuccess) e = cudaMalloc(&b->d_src, std::max<size_t>(src_bytes, 16));
  if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_dofs, std::max<size_t>(dof_count * sizeof(double), 16));
  if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_tri_pool, std::max<size_t>(b->n_tri * 3 * sizeof(float4), 16));
  if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_surf_pool, std::max<size_t>(b->n_surf * 2 * sizeof(float4), 16));
  if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_objs, std::max<size_t>(n * sizeof(ObjDev), 16));
  if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_order, std::max<size_t>(n * sizeof(int32_t), 16));
  if (e != cudaSuccess) { cleanup(); return cuda_fail(e, "pi_batch_create allocation"); }
  if (on_device) {
    for (int i = 0; i < n && e == cudaSuccess; ++i) {
      const HostObjInfo& in = b->info[i];
      if (in.n_elems)
        e = cudaMemcpyAsync(static_cast<unsigned char*>(b->d_src) + in.src_off, objs[i].elems,
                            in.n_elems * elem_bytes(in.geom_type), cudaMemcpyDeviceToDevice, s);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(b->d_dofs + in.dof_off, objs[i].dofs, in.n_dofs * sizeof(double),
                            cudaMemcpyDeviceToDevice, s);
    }
  } else {
    std::vector<unsigned char> hs(std::max<size_t>(src_bytes, 16));
    std::vector<double> hd(std::max<int64_t>(dof_count, 1));
    for (int i = 0; i < n; ++i) {
      const HostObjInfo& in = b->info[i];
      if (in.n_elems) std::memcpy(hs.data() + in.src_off, objs[i].elems, in.n_elems * elem_bytes(in.geom_type));
      std::memcpy(hd.data() + in.dof_off, objs[i].dofs, in.n_dofs * sizeof(double));
    }
    e = cudaMemcpyAsync(b->d_src, hs.data(), src_bytes, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(b->d_dofs, hd.data(), dof_count * sizeof(double), cudaMemcpyHostToDevice, s);
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(b->d_order, b->order.data(), n * sizeof(int32_t), cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) { cleanup(); return cuda_fail(e, "pi_batch_create upload"); }
  int rc = launch_prepare(b.get(), -1, s);
  if (rc) { cleanup(); return rc; }
  *out = b.release();
  return PI_OK;
}

int pi_batch_set_dofs(pi_batch b, int index, const double* d_dofs, pi_stream stream) {
  if (!b || index < 0 || index >= b->n_obj || !d_dofs)
    return fail(PI_ERR_INVALID_ARGUMENT, "pi_batch_set_dofs: bad arguments");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const HostObjInfo& in = b->info[index];
  PI_CUDA(cudaMemcpyAsync(b->d_dofs + in.dof_off, d_dofs, in.n_dofs * sizeof(double), cudaMemcpyDeviceToDevice, s));
  return launch_prepare(b, index, s);
}

int pi_batch_prepare(pi_batch b, pi_stream stream) {
  if (!b) return fail(PI_ERR_INVALID_ARGUMENT, "pi_batch_prepare: null batch");
  return launch_prepare(b, -1, reinterpret_cast<cudaStream_t>(stream));
}

int pi_batch_destroy(pi_batch b) {
  if (!b) return PI_OK;
  cudaFree(b->d_src); cudaFree(b->d_dofs); cudaFree(b->d_tri_pool); cudaFree(b->d_surf_pool);
  cudaFree(b->d_objs); cudaFree(b->d_order);
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

int pi_contract_workspace_size(pi_kgrid kg, int n, int precision, size_t* bytes) {
  if (!kg || !bytes || n < 0) return fail(PI_ERR_INVALID_ARGUMENT, "pi_contract_workspace_size: bad arguments");
  if (precision == PI_CONTRACT_FP32) *bytes = contract_fp32_ws_bytes(kg->Q, n);
  else if (precision == PI_CONTRACT_BF16X3) *bytes = contract_tc_ws_bytes(kg->Q, n, 0);
  else if (precision == PI_CONTRACT_TF32X3) *bytes = contract_tc_ws_bytes(kg->Q, n, 1);
  else return fail(PI_ERR_INVALID_ARGUMENT, "unknown contraction precision");
  return PI_OK;
}

int pi_contract(pi_kgrid kg, const void* d_Jw, int n, int precision, double* d_V, void* d_ws, size_t ws_bytes,
                pi_stream stream) {
  if (!kg || n < 0 || (n > 0 && (!d_Jw || !d_V))) return fail(PI_ERR_INVALID_ARGUMENT, "pi_contract: bad arguments");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const float2* J = static_cast<const float2*>(d_Jw);
  if (precision == PI_CONTRACT_FP32) return launch_contract_fp32(kg, J, n, d_V, d_ws, ws_bytes, s);
  if (precision == PI_CONTRACT_BF16X3 || precision == PI_CONTRACT_TF32X3) {
    if (!kg->all_positive)
      return fail(PI_ERR_UNSUPPORTED, "the tensor-core contractions need non-negative quadrature weights");
    return launch_contract_tc(kg, J, n, precision == PI_CONTRACT_BF16X3 ? 0 : 1, d_V, d_ws, ws_bytes, s);
  }
  return fail(PI_ERR_INVALID_ARGUMENT, "unknown contraction precision");
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
  rc = pi_batch_create(objs, n, 0, reinterpret_cast<pi_stream>(s), &b.b);
  if (rc) return rc;
  size_t ws_bytes = 0;
  rc = pi_contract_workspace_size(kg.k, n, precision, &ws_bytes);
  if (rc) return rc;
  DevBuf J, ws, V;
  if ((rc = J.alloc((size_t)n * Q * sizeof(float2), s)) || (rc = ws.alloc(ws_bytes, s)) ||
      (rc = V.alloc((size_t)n * n * sizeof(double), s)))
    return rc;
  rc = pi_form_factors(kg.k, b.b, 1, J.p, reinterpret_cast<pi_stream>(s));
  if (rc) return rc;
  rc = pi_contract(kg.k, J.p, n, precision, static_cast<double*>(V.p), ws.p, ws_bytes, reinterpret_cast<pi_stream>(s));
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

}  // extern "C"
