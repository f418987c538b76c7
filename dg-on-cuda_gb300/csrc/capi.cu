// capi.cu -- C ABI of the GB300 nodal-DG hot path (declared in include/dgc_gb300.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "dgc_gb300.h"
#include "dgc_internal.hpp"
#include "rhs_launch.cuh"

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  return fail(DGC_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define CK(call)                                        \
  do {                                                  \
    cudaError_t e_ = (call);                            \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
  } while (0)

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

// Low-storage RK4 coefficients, Carpenter & Kennedy (1994), NASA TM-109112,
// five-stage fourth-order 2N-storage scheme ("solution 3").
const double kRkA[5] = {0.0, -567301805773.0 / 1357537059087.0, -2404267990393.0 / 2016746695238.0,
                        -3550918686646.0 / 2091501179385.0, -1275806237668.0 / 842570457699.0};
const double kRkB[5] = {1432997174477.0 / 9575080441755.0, 5161836677717.0 / 13612068292357.0,
                        1720146321549.0 / 2090206949498.0, 3134564353537.0 / 4481467310338.0,
                        2277821191437.0 / 14882151754819.0};
const double kRkC[5] = {0.0, 1432997174477.0 / 9575080441755.0, 2526269341429.0 / 6820363962896.0,
                        2006345519317.0 / 3224310063776.0, 2802321613138.0 / 2924317926251.0};

// ------------------------------------------------------------------ small kernels
template <typename R>
__global__ void k_axpy(size_t n, R a, const R* __restrict__ x, const R* __restrict__ y, R* __restrict__ out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = a * x[i] + y[i];
}

// native q[k][f][NpP] <-> reference CPU q[f][k][Np] / GPU q[f][j][k]
template <typename R>
__global__ void k_layout(int K, int Nf, int Np, int NpP, int layout, int to_native, const R* __restrict__ src,
                         R* __restrict__ dst) {
  const size_t n = (size_t)K * Nf * NpP;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
    const int j = (int)(idx % NpP);
    const size_t kf = idx / NpP;
    const int f = (int)(kf % Nf);
    const size_t k = kf / Nf;
    if (j >= Np) {
      if (to_native) dst[idx] = (R)0;
      continue;
    }
    const size_t r = layout == DGC_LAYOUT_REF_CPU ? ((size_t)f * K + k) * Np + j : ((size_t)f * Np + j) * K + k;
    if (to_native) dst[idx] = src[r];
    else dst[r] = src[idx];
  }
}

// the same for DGC_F32C states: FP64 reference arrays <-> native [hi | lo]
// pairs (hi = the FP32 rounding of the value, lo = the FP32 rounding of the
// rest)
__global__ void k_layout_x2(int K, int Nf, int Np, int NpP, int layout, int to_native, const void* src_v,
                            void* dst_v) {
  const size_t n = (size_t)K * Nf * NpP;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
    const int j = (int)(idx % NpP);
    const size_t kf = idx / NpP;
    const int f = (int)(kf % Nf);
    const size_t k = kf / Nf;
    if (j >= Np) {
      if (to_native) {
        static_cast<float*>(dst_v)[idx] = 0.0f;
        static_cast<float*>(dst_v)[n + idx] = 0.0f;
      }
      continue;
    }
    const size_t r = layout == DGC_LAYOUT_REF_CPU ? ((size_t)f * K + k) * Np + j : ((size_t)f * Np + j) * K + k;
    if (to_native) {
      const double v = static_cast<const double*>(src_v)[r];
      const float hi = __double2float_rn(v);
      static_cast<float*>(dst_v)[idx] = hi;
      static_cast<float*>(dst_v)[n + idx] = __double2float_rn(v - (double)hi);
    } else {
      const float* q = static_cast<const float*>(src_v);
      static_cast<double*>(dst_v)[r] = (double)q[idx] + (double)q[n + idx];
    }
  }
}

// launched with programmatic serialization like the stages: it waits for the
// step's last stage, and the next step's first stage waits for it
__global__ void k_clock(double* t, double dt) {
  dgk::grid_dep_launch();
  dgk::grid_dep_wait();
  t[0] += dt;
}

template <typename R>
std::vector<R> pack_mats(const dgc::RefElement& re, const std::vector<double>& Dr, const std::vector<double>& Ds,
                         const std::vector<double>& L) {
  const int Np = re.Np, NF = 3 * re.Nfp;
  const int kD = (Np * Np + 3) / 4 * 4, kL = (NF * Np + 3) / 4 * 4;
  std::vector<R> m((size_t)2 * kD + kL, (R)0);
  for (int i = 0; i < Np; ++i)
    for (int j = 0; j < Np; ++j) {
      m[(size_t)j * Np + i] = (R)Dr[(size_t)i * Np + j];
      m[(size_t)kD + j * Np + i] = (R)Ds[(size_t)i * Np + j];
    }
  for (int i = 0; i < Np; ++i)
    for (int c = 0; c < NF; ++c) m[(size_t)2 * kD + c * Np + i] = (R)L[(size_t)i * NF + c];
  return m;
}

}  // namespace

namespace dgc {

int set_error(int code, const char* msg) {
  g_err = msg;
  return code;
}

int upload_operators(dgc_handle_s* h, int form) {
  const dgc::RefElement& re = h->re;
  const std::vector<double>& Dr = form == 0 ? re.Drw : re.Drs;
  const std::vector<double>& Ds = form == 0 ? re.Dsw : re.Dss;
  const std::vector<double>& L = form == 0 ? re.Lw : re.Ls;
  std::vector<double> m64 = pack_mats<double>(re, Dr, Ds, L);
  std::vector<float> m32 = pack_mats<float>(re, Dr, Ds, L);
  if (!h->d_mats64[form]) CK(cudaMalloc(&h->d_mats64[form], m64.size() * sizeof(double)));
  if (!h->d_mats32[form]) CK(cudaMalloc(&h->d_mats32[form], m32.size() * sizeof(float)));
  CK(cudaMemcpy(h->d_mats64[form], m64.data(), m64.size() * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(h->d_mats32[form], m32.data(), m32.size() * sizeof(float), cudaMemcpyHostToDevice));
  if (form == 0) {
    // register-blocked kernel operand: rows j of Dr^T, Ds^T (j < Np) and m of
    // LIFT^T (m < 3 Nfp), each padded with zeros to NpP columns
    const int Np = re.Np, NF = 3 * re.Nfp, NpP = dgc::padded_nodes(re.N);
    std::vector<float> bk((size_t)(2 * Np + NF) * NpP, 0.0f);
    for (int j = 0; j < Np; ++j)
      for (int i = 0; i < Np; ++i) {
        bk[(size_t)j * NpP + i] = (float)Dr[(size_t)i * Np + j];
        bk[(size_t)(Np + j) * NpP + i] = (float)Ds[(size_t)i * Np + j];
      }
    for (int m = 0; m < NF; ++m)
      for (int i = 0; i < Np; ++i) bk[(size_t)(2 * Np + m) * NpP + i] = (float)L[(size_t)i * NF + m];
    if (!h->d_blk_b) CK(cudaMalloc(&h->d_blk_b, bk.size() * sizeof(float)));
    CK(cudaMemcpy(h->d_blk_b, bk.data(), bk.size() * sizeof(float), cudaMemcpyHostToDevice));
  }
  if (form == 1) {
    // compensated-state kernel operand: rows j of the strong-form Dr^T, Ds^T
    // and m of LIFT^T, each padded with zeros to NpP columns
    const int Np = re.Np, NF = 3 * re.Nfp, NpP = dgc::padded_nodes(re.N);
    std::vector<float> bk((size_t)(2 * Np + NF) * NpP, 0.0f);
    for (int j = 0; j < Np; ++j)
      for (int i = 0; i < Np; ++i) {
        bk[(size_t)j * NpP + i] = (float)Dr[(size_t)i * Np + j];
        bk[(size_t)(Np + j) * NpP + i] = (float)Ds[(size_t)i * Np + j];
      }
    for (int m = 0; m < NF; ++m)
      for (int i = 0; i < Np; ++i) bk[(size_t)(2 * Np + m) * NpP + i] = (float)L[(size_t)i * NF + m];
    if (!h->d_blk_bs) CK(cudaMalloc(&h->d_blk_bs, bk.size() * sizeof(float)));
    CK(cudaMemcpy(h->d_blk_bs, bk.data(), bk.size() * sizeof(float), cudaMemcpyHostToDevice));
  }
  if (form == 1 && re.N <= 6) {
    // tensor-core operand (the FP32 tcgen05 kernel evaluates the strong form):
    // row n = output node, K = [Dr(n,:) pad | Ds(n,:) pad | LIFT(n,:)] with the
    // derivative blocks padded to NpP columns; K-major core matrices (8 rows x
    // 4 floats); hi / lo TF32 split
    const int Np = re.Np, NF = 3 * re.Nfp, NpP = dgc::padded_nodes(re.N);
    const int KP = (2 * NpP + NF + 7) / 8 * 8, NC = Np <= 16 ? 16 : 32, SBO4 = KP / 4 * 32;
    std::vector<float> tc((size_t)2 * NC * KP, 0.0f);
    for (int n = 0; n < Np; ++n)
      for (int k = 0; k < 2 * NpP + NF; ++k) {
        double x = 0.0;
        if (k < NpP) x = k < Np ? Dr[(size_t)n * Np + k] : 0.0;
        else if (k < 2 * NpP) x = (k - NpP) < Np ? Ds[(size_t)n * Np + k - NpP] : 0.0;
        else x = L[(size_t)n * NF + k - 2 * NpP];
        // round to nearest TF32 (10 explicit mantissa bits, ties away from zero)
        auto tf32 = [](float f) {
          uint32_t b;
          std::memcpy(&b, &f, 4);
          b = (b + 0x1000u) & 0xFFFFE000u;
          float r;
          std::memcpy(&r, &b, 4);
          return r;
        };
        const float hi = tf32((float)x);
        const float lo = tf32((float)(x - (double)hi));
        const size_t o = (size_t)(n >> 3) * SBO4 + (k >> 2) * 32 + (n & 7) * 4 + (k & 3);
        tc[o] = hi;
        tc[(size_t)NC * KP + o] = lo;
      }
    if (!h->d_tc_b) CK(cudaMalloc(&h->d_tc_b, tc.size() * sizeof(float)));
    CK(cudaMemcpy(h->d_tc_b, tc.data(), tc.size() * sizeof(float), cudaMemcpyHostToDevice));
  }
  return DGC_OK;
}

}  // namespace dgc


extern "C" const char* dgc_last_error(void) { return g_err.c_str(); }

namespace {

int check_desc(const dgc_problem_desc* desc) {
  if (desc->physics < DGC_ADVECTION || desc->physics > DGC_LAPLACE)
    return fail(DGC_ERR_ARG, "unknown physics %d", desc->physics);
  if (desc->precision != DGC_F64 && desc->precision != DGC_F32 && desc->precision != DGC_F32C)
    return fail(DGC_ERR_ARG, "unknown precision %d", desc->precision);
  if (desc->precision == DGC_F32C && desc->physics == DGC_LAPLACE)
    return fail(DGC_ERR_UNSUPPORTED, "the compensated FP32 state is offered for advection and Maxwell handles");
  if (desc->order < 1 || desc->order > dgc::kMaxOrder)
    return fail(DGC_ERR_ARG, "order %d outside [1, %d]", desc->order, dgc::kMaxOrder);
  if (desc->physics == DGC_ADVECTION && (desc->bc < DGC_BC_SINSIN || desc->bc > DGC_BC_ZERO))
    return fail(DGC_ERR_ARG, "unknown advection boundary kind %d", desc->bc);
  if (desc->physics == DGC_ADVECTION && desc->bc == DGC_BC_GAUSS && !(desc->gw > 0.0))
    return fail(DGC_ERR_ARG, "gaussian width must be positive");
  return DGC_OK;
}

// the device side of a handle whose reference element and mesh are built
int finish_create(dgc_handle_s* h, int K, dgc_handle* out) {
  const dgc_problem_desc* desc = &h->desc;
  h->K = K;
  h->N = desc->order;
  h->Np = h->re.Np;
  h->Nfp = h->re.Nfp;
  h->NpP = dgc::padded_nodes(h->N);
  h->Nf = (desc->physics == DGC_MAXWELL_TM || desc->physics == DGC_MAXWELL_TE) ? 3 : 1;
  h->prec = desc->precision;
  int rc = dgc::device_init(h);
  if (rc != DGC_OK) {
    dgc::device_free(h);
    delete h;
    return rc;
  }
  *out = h;
  return DGC_OK;
}

}  // namespace

extern "C" int dgc_create(int nv, const double* vxy, int K, const int32_t* cells, const dgc_problem_desc* desc,
                          dgc_handle* out) {
  if (!out || !desc) return fail(DGC_ERR_ARG, "null argument");
  *out = nullptr;
  if (int rc = check_desc(desc)) return rc;
  auto* h = new dgc_handle_s();
  h->desc = *desc;
  std::string err;
  if (!dgc::build_ref_element(desc->order, h->re, err)) {
    delete h;
    return fail(DGC_ERR_ARG, "%s", err.c_str());
  }
  // half-edge matching on the GPU from 16384 cells (DGC_GPU_TOPOLOGY_MIN overrides)
  int64_t gpu_topo_min = 16384;
  if (const char* e = std::getenv("DGC_GPU_TOPOLOGY_MIN")) gpu_topo_min = std::atoll(e);
  if (!dgc::build_mesh(vxy, nv, cells, K, h->re, h->mesh, err, (int64_t)K >= gpu_topo_min)) {
    delete h;
    return fail(DGC_ERR_MESH, "%s", err.c_str());
  }
  return finish_create(h, K, out);
}

extern "C" int dgc_create_from_arrays(int K, const double* invJ, const double* J, const double* faceJ,
                                      const int32_t* nb_cell, const int32_t* nb_face, int num_boundary_nodes,
                                      const double* bx, const double* by, const double* nx, const double* ny,
                                      const dgc_problem_desc* desc, dgc_handle* out) {
  if (!out || !desc || !invJ || !J || !faceJ || !nb_cell || !nb_face || !nx || !ny ||
      (num_boundary_nodes > 0 && (!bx || !by)))
    return fail(DGC_ERR_ARG, "null argument");
  *out = nullptr;
  if (int rc = check_desc(desc)) return rc;
  auto* h = new dgc_handle_s();
  h->desc = *desc;
  std::string err;
  if (!dgc::build_ref_element(desc->order, h->re, err)) {
    delete h;
    return fail(DGC_ERR_ARG, "%s", err.c_str());
  }
  if (!dgc::build_mesh_from_arrays(K, h->re, invJ, J, faceJ, nb_cell, nb_face, num_boundary_nodes, bx, by, nx, ny,
                                   h->mesh, err)) {
    delete h;
    return fail(DGC_ERR_MESH, "%s", err.c_str());
  }
  return finish_create(h, K, out);
}

namespace dgc {

// the stage kernel of the handle's precision and variant: launch (info NULL)
// or describe it
cudaError_t rhs_dispatch_any(const dgc_handle_s* h, const dgk::RhsParams& p, cudaStream_t s, dgk::LaunchInfo* info) {
  if (h->prec == DGC_F64) return dgk::rhs_dispatch<double>(h->N, h->desc.physics, h->rhs_variant, p, h->sm_count, s, info);
  if (h->prec == DGC_F32C) return dgk::rhs_x2_dispatch(h->N, h->desc.physics, p, h->sm_count, s, info);
  return dgk::rhs_dispatch<float>(h->N, h->desc.physics, h->rhs_variant, p, h->sm_count, s, info);
}

int device_init(dgc_handle_s* h) {
  CK(cudaGetDevice(&h->device));
  CK(cudaDeviceGetAttribute(&h->sm_count, cudaDevAttrMultiProcessorCount, h->device));
  const MeshData& m = h->mesh;
  CK(cudaMalloc(&h->d_geom, m.geom.size() * sizeof(double)));
  CK(cudaMemcpy(h->d_geom, m.geom.data(), m.geom.size() * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMalloc(&h->d_nbr, (size_t)h->K * sizeof(int4)));
  CK(cudaMemcpy(h->d_nbr, m.nbr.data(), (size_t)h->K * sizeof(int4), cudaMemcpyHostToDevice));
  const size_t nb = m.bxy.size() ? m.bxy.size() : 2;
  CK(cudaMalloc(&h->d_bxy, nb * sizeof(double)));
  if (!m.bxy.empty()) CK(cudaMemcpy(h->d_bxy, m.bxy.data(), m.bxy.size() * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMalloc(&h->d_tau, m.tau.size() * sizeof(double)));
  CK(cudaMemcpy(h->d_tau, m.tau.data(), m.tau.size() * sizeof(double), cudaMemcpyHostToDevice));
  {
    const std::vector<double> g64 = kernel_geometry<double>(m.geom, h->K);
    const std::vector<float> g32 = kernel_geometry<float>(m.geom, h->K);
    const std::vector<float> t32(m.tau.begin(), m.tau.end());
    CK(cudaMalloc(&h->d_kgeom64, g64.size() * sizeof(double)));
    CK(cudaMemcpy(h->d_kgeom64, g64.data(), g64.size() * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMalloc(&h->d_kgeom32, g32.size() * sizeof(float)));
    CK(cudaMemcpy(h->d_kgeom32, g32.data(), g32.size() * sizeof(float), cudaMemcpyHostToDevice));
    CK(cudaMalloc(&h->d_tau32, t32.size() * sizeof(float)));
    CK(cudaMemcpy(h->d_tau32, t32.data(), t32.size() * sizeof(float), cudaMemcpyHostToDevice));
  }
  CK(cudaMalloc(&h->d_status, 64));
  CK(cudaMemset(h->d_status, 0, 64));
  CK(cudaMalloc(&h->d_time, 64));
  CK(cudaMemset(h->d_time, 0, 64));
  int rc = upload_operators(h, 0);
  if (rc != DGC_OK) return rc;
  rc = upload_operators(h, 1);
  if (rc != DGC_OK) return rc;
  if (h->desc.physics != DGC_LAPLACE) {
    dgk::LaunchInfo li;
    const cudaError_t e = rhs_dispatch_any(h, dgk::RhsParams{}, 0, &li);
    if (e != cudaSuccess) return cuda_fail(e, "configure rhs kernel");
    h->rhs_info = li;
  }
  return ipdg_init(h);
}

void device_free(dgc_handle_s* h) {
  if (h->graph_exec) cudaGraphExecDestroy(h->graph_exec);
  cudaFree(h->d_geom);
  cudaFree(h->d_nbr);
  cudaFree(h->d_bxy);
  cudaFree(h->d_tau);
  cudaFree(h->d_kgeom64);
  cudaFree(h->d_kgeom32);
  cudaFree(h->d_tau32);
  cudaFree(h->d_status);
  cudaFree(h->d_time);
  for (int f = 0; f < 2; ++f) {
    cudaFree(h->d_mats64[f]);
    cudaFree(h->d_mats32[f]);
  }
  cudaFree(h->d_tc_b);
  cudaFree(h->d_blk_b);
  cudaFree(h->d_blk_bs);
  ipdg_free(h);
}

}  // namespace dgc

extern "C" int dgc_destroy(dgc_handle h) {
  if (!h) return fail(DGC_ERR_ARG, "null handle");
  dgc::device_free(h);
  delete h;
  return DGC_OK;
}

extern "C" int dgc_get_info(dgc_handle h, dgc_info* o) {
  if (!h || !o) return fail(DGC_ERR_ARG, "null argument");
  std::memset(o, 0, sizeof *o);
  o->num_cells = h->K;
  o->order = h->N;
  o->np = h->Np;
  o->np_padded = h->NpP;
  o->nfp = h->Nfp;
  o->num_fields = h->Nf;
  o->precision = h->prec;
  o->state_len = (int64_t)h->K * h->Nf * h->NpP;
  o->scalar_bytes = h->prec == DGC_F32 ? 4 : 8;
  o->num_boundary_faces = h->mesh.num_bfaces;
  o->min_edge = h->mesh.min_edge;
  o->min_altitude = h->mesh.min_altitude;
  o->rhs_tile = h->rhs_info.tile;
  o->rhs_threads = h->rhs_info.threads;
  o->rhs_smem = h->rhs_info.smem;
  o->rhs_blocks_per_sm = h->rhs_info.blocks_per_sm;
  o->sm_count = h->sm_count;
  return DGC_OK;
}

extern "C" int dgc_node_coordinates(dgc_handle h, double* x, double* y) {
  if (!h || !x || !y) return fail(DGC_ERR_ARG, "null argument");
  const dgc::MeshData& m = h->mesh;
  if (m.cells.empty())
    return fail(DGC_ERR_UNSUPPORTED, "the handle was created from geometry arrays and has no vertex coordinates");
  for (int k = 0; k < h->K; ++k) {
    const int32_t* c = &m.cells[3 * (size_t)k];
    for (int j = 0; j < h->Np; ++j) {
      const double r = h->re.r[j], s = h->re.s[j];
      const double l1 = 0.5 * (s + 1.0), l2 = -0.5 * (r + s), l3 = 0.5 * (r + 1.0);
      x[(size_t)k * h->Np + j] = l2 * m.vx[c[0]] + l3 * m.vx[c[1]] + l1 * m.vx[c[2]];
      y[(size_t)k * h->Np + j] = l2 * m.vy[c[0]] + l3 * m.vy[c[1]] + l1 * m.vy[c[2]];
    }
  }
  return DGC_OK;
}

extern "C" int dgc_get_operator(dgc_handle h, int which, double* out) {
  if (!h || !out) return fail(DGC_ERR_ARG, "null argument");
  const dgc::RefElement& re = h->re;
  const std::vector<double>* src = nullptr;
  switch (which) {
    case DGC_OP_DR_WEAK: src = &re.Drw; break;
    case DGC_OP_DS_WEAK: src = &re.Dsw; break;
    case DGC_OP_LIFT: src = &re.Lw; break;
    case DGC_OP_DR_STRONG: src = &re.Drs; break;
    case DGC_OP_DS_STRONG: src = &re.Dss; break;
    case DGC_OP_MASS: src = &re.M; break;
    case DGC_OP_V: src = &re.V; break;
    default: return fail(DGC_ERR_ARG, "unknown operator %d", which);
  }
  std::memcpy(out, src->data(), src->size() * sizeof(double));
  return DGC_OK;
}

extern "C" int dgc_set_operators(dgc_handle h, int form, const double* Dr, const double* Ds, const double* L) {
  if (!h || !Dr || !Ds || !L) return fail(DGC_ERR_ARG, "null argument");
  if (form != 0 && form != 1) return fail(DGC_ERR_ARG, "form must be 0 (weak) or 1 (strong)");
  const size_t nn = (size_t)h->Np * h->Np, nl = (size_t)h->Np * 3 * h->Nfp;
  dgc::RefElement& re = h->re;
  (form == 0 ? re.Drw : re.Drs).assign(Dr, Dr + nn);
  (form == 0 ? re.Dsw : re.Dss).assign(Ds, Ds + nn);
  (form == 0 ? re.Lw : re.Ls).assign(L, L + nl);
  CK(cudaDeviceSynchronize());
  const int rc = dgc::upload_operators(h, form);
  if (rc == DGC_OK) dgc::ipdg_operators_changed(h);
  return rc;
}

static int layout_convert(dgc_handle h, int layout, const void* src, void* dst, void* stream, int to_native) {
  if (!h || !src || !dst) return fail(DGC_ERR_ARG, "null argument");
  if (src == dst) return fail(DGC_ERR_ARG, "layout conversion cannot run in place");
  if (layout != DGC_LAYOUT_REF_CPU && layout != DGC_LAYOUT_REF_GPU)
    return fail(DGC_ERR_ARG, "unknown layout %d", layout);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t n = (size_t)h->K * h->Nf * h->NpP;
  const int grid = (int)std::min<size_t>((n + 255) / 256, (size_t)h->sm_count * 16);
  if (h->prec == DGC_F32C)
    k_layout_x2<<<grid, 256, 0, s>>>(h->K, h->Nf, h->Np, h->NpP, layout, to_native, src, dst);
  else if (h->prec == DGC_F64)
    k_layout<double><<<grid, 256, 0, s>>>(h->K, h->Nf, h->Np, h->NpP, layout, to_native,
                                          static_cast<const double*>(src), static_cast<double*>(dst));
  else
    k_layout<float><<<grid, 256, 0, s>>>(h->K, h->Nf, h->Np, h->NpP, layout, to_native,
                                         static_cast<const float*>(src), static_cast<float*>(dst));
  CK(cudaGetLastError());
  return DGC_OK;
}

extern "C" int dgc_to_native(dgc_handle h, int layout, const void* src, void* dst, void* stream) {
  return layout_convert(h, layout, src, dst, stream, 1);
}
extern "C" int dgc_from_native(dgc_handle h, int layout, const void* src, void* dst, void* stream) {
  return layout_convert(h, layout, src, dst, stream, 0);
}

extern "C" int dgc_axpy(dgc_handle h, double a, const void* x, const void* y, void* out, void* stream) {
  if (!h || !x || !y || !out) return fail(DGC_ERR_ARG, "null argument");
  if (h->prec == DGC_F32C) return fail(DGC_ERR_UNSUPPORTED, "axpy is not offered for compensated FP32 states");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t n = (size_t)h->K * h->Nf * h->NpP;
  const int grid = (int)std::min<size_t>((n + 255) / 256, (size_t)h->sm_count * 8);
  if (h->prec == DGC_F64)
    k_axpy<double><<<grid, 256, 0, s>>>(n, a, static_cast<const double*>(x), static_cast<const double*>(y),
                                        static_cast<double*>(out));
  else
    k_axpy<float><<<grid, 256, 0, s>>>(n, (float)a, static_cast<const float*>(x), static_cast<const float*>(y),
                                       static_cast<float*>(out));
  CK(cudaGetLastError());
  return DGC_OK;
}

namespace {

dgk::RhsParams base_params(dgc_handle h) {
  dgk::RhsParams p{};
  p.K = h->K;
  p.geom = h->prec == DGC_F64 ? (const void*)h->d_kgeom64 : (const void*)h->d_kgeom32;
  p.nbr = reinterpret_cast<const int4*>(h->d_nbr);
  p.bxy = h->d_bxy;
  p.mats = h->prec == DGC_F64 ? h->d_mats64[0] : h->d_mats32[0];
  p.mats_tc = h->prec == DGC_F32 ? h->d_tc_b : nullptr;
  p.mats_blk = h->prec == DGC_F32 ? h->d_blk_b : (h->prec == DGC_F32C ? h->d_blk_bs : nullptr);
  p.ax = h->desc.ax;
  p.ay = h->desc.ay;
  p.gx0 = h->desc.gx0;
  p.gy0 = h->desc.gy0;
  p.gw = h->desc.gw;
  p.bc = h->desc.bc;
  p.status = h->d_status;
  return p;
}

int launch(dgc_handle h, const dgk::RhsParams& p, cudaStream_t s) {
  const cudaError_t e = dgc::rhs_dispatch_any(h, p, s, nullptr);
  if (e != cudaSuccess) return cuda_fail(e, "rhs kernel launch");
  ++h->launches;
  return DGC_OK;
}

int check_time_dependent(dgc_handle h) {
  if (h->desc.physics == DGC_LAPLACE) return fail(DGC_ERR_UNSUPPORTED, "laplace handle has no time-dependent operator");
  return DGC_OK;
}

}  // namespace

namespace dgc {
dgk::RhsParams rhs_base_params(dgc_handle_s* h) { return base_params(h); }
const double* lserk_coeffs(int which) { return which == 0 ? kRkA : (which == 1 ? kRkB : kRkC); }
}  // namespace dgc

extern "C" int dgc_rhs(dgc_handle h, const void* q, double t, void* out, void* stream) {
  if (!h || !q || !out) return fail(DGC_ERR_ARG, "null argument");
  if (int rc = check_time_dependent(h)) return rc;
  if (q == out) return fail(DGC_ERR_ARG, "q and out must not alias");
  if (!aligned16(q) || !aligned16(out)) return fail(DGC_ERR_ARG, "state buffers must be 16-byte aligned");
  dgk::RhsParams p = base_params(h);
  p.q_in = q;
  p.out = out;
  p.t = t;
  p.mode = dgk::MODE_RHS;
  return launch(h, p, static_cast<cudaStream_t>(stream));
}

extern "C" int dgc_rk4_step(dgc_handle h, void* q, double t, double dt, void* const* work, void* stream) {
  if (!h || !q || !work || !work[0] || !work[1] || !work[2]) return fail(DGC_ERR_ARG, "null argument");
  if (int rc = check_time_dependent(h)) return rc;
  if (h->prec == DGC_F32C)
    return fail(DGC_ERR_UNSUPPORTED, "classical RK4 is not offered for compensated FP32 states (use LSERK4)");
  void* ya = work[0];
  void* yb = work[1];
  void* acc = work[2];
  if (q == ya || q == yb || q == acc || ya == yb || ya == acc || yb == acc)
    return fail(DGC_ERR_ARG, "q and the three work buffers must be distinct");
  for (const void* b : {(const void*)q, (const void*)ya, (const void*)yb, (const void*)acc})
    if (!aligned16(b)) return fail(DGC_ERR_ARG, "state buffers must be 16-byte aligned");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  dgk::RhsParams p = base_params(h);
  p.mode = dgk::MODE_RK4;
  p.aux = acc;
  p.q0 = q;
  const void* in[4] = {q, ya, yb, ya};
  void* outb[4] = {ya, yb, ya, nullptr};
  const double co[4] = {0.5 * dt, 0.5 * dt, dt, dt / 6.0};
  const double wa[4] = {1.0, 2.0, 2.0, 0.0};
  const double ts[4] = {t, t + 0.5 * dt, t + 0.5 * dt, t + dt};
  for (int st = 0; st < 4; ++st) {
    p.stage = st;
    p.q_in = in[st];
    p.out = outb[st];
    p.ca = co[st];
    p.cb = wa[st];
    p.t = ts[st];
    if (int rc = launch(h, p, s)) return rc;
  }
  return DGC_OK;
}

namespace {

int lserk4_launches(dgc_handle h, void* q_in, void* q_out, void* res, double t, double dt, bool dev_time,
                    cudaStream_t s) {
  dgk::RhsParams p = base_params(h);
  p.mode = dgk::MODE_LSERK;
  p.aux = res;
  p.dt = dt;
  p.t_dev = dev_time ? h->d_time : nullptr;
  void* bufs[2] = {q_in, q_out};
  for (int st = 0; st < 5; ++st) {
    p.q_in = bufs[st & 1];
    p.out = bufs[(st + 1) & 1];
    p.ca = kRkA[st];
    p.cb = kRkB[st];
    p.t = dev_time ? kRkC[st] * dt : t + kRkC[st] * dt;
    if (int rc = launch(h, p, s)) return rc;
  }
  if (dev_time) {
    CK(dgk::launch_stage(k_clock, 1, 1, 0, s, h->d_time, dt));
    ++h->launches;
  }
  return DGC_OK;
}

int check_lserk_buffers(dgc_handle h, const void* a, const void* b, const void* r) {
  if (!h || !a || !b || !r) return fail(DGC_ERR_ARG, "null argument");
  if (a == b || a == r || b == r) return fail(DGC_ERR_ARG, "state, scratch and residual buffers must be distinct");
  if (!aligned16(a) || !aligned16(b) || !aligned16(r)) return fail(DGC_ERR_ARG, "state buffers must be 16-byte aligned");
  return check_time_dependent(h);
}

}  // namespace

extern "C" int dgc_lserk4_stage(dgc_handle h, int stage, const void* q_in, void* q_out, void* res, double t,
                                double dt, void* stream) {
  if (int rc = check_lserk_buffers(h, q_in, q_out, res)) return rc;
  if (stage < 0 || stage > 4) return fail(DGC_ERR_ARG, "LSERK4 stage %d outside [0, 4]", stage);
  dgk::RhsParams p = base_params(h);
  p.mode = dgk::MODE_LSERK;
  p.aux = res;
  p.dt = dt;
  p.q_in = q_in;
  p.out = q_out;
  p.ca = kRkA[stage];
  p.cb = kRkB[stage];
  p.t = t + kRkC[stage] * dt;
  return launch(h, p, static_cast<cudaStream_t>(stream));
}

extern "C" int dgc_lserk4_step(dgc_handle h, void* q_in, void* q_out, void* res, double t, double dt, void* stream) {
  if (int rc = check_lserk_buffers(h, q_in, q_out, res)) return rc;
  // 5 stages alternate q_in -> q_out -> q_in ...; the odd count ends in q_out
  return lserk4_launches(h, q_in, q_out, res, t, dt, false, static_cast<cudaStream_t>(stream));
}

extern "C" int dgc_lserk4_run(dgc_handle h, void* qa, void* qb, void* res, double t0, double dt, int nsteps,
                              int use_graph, void** final_state, void* stream) {
  if (int rc = check_lserk_buffers(h, qa, qb, res)) return rc;
  if (nsteps < 0) return fail(DGC_ERR_ARG, "negative step count");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // simulation time lives in device memory so that captured launches stay valid
  CK(cudaMemcpyAsync(h->d_time, &t0, sizeof(double), cudaMemcpyHostToDevice, s));
  int done = 0;
  void* cur = qa;
  void* other = qb;
  if (use_graph && nsteps >= 2) {
    const int gsteps = nsteps >= 20 ? 20 : 2;
    const bool reuse = h->graph_exec && h->graph_key[0] == qa && h->graph_key[1] == qb && h->graph_key[2] == res &&
                       h->graph_dt == dt && h->graph_steps == gsteps;
    if (!reuse) {
      if (h->graph_exec) {
        cudaGraphExecDestroy(h->graph_exec);
        h->graph_exec = nullptr;
      }
      cudaStream_t cs;
      CK(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
      cudaGraph_t g = nullptr;
      cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
      int rc = DGC_OK;
      if (e == cudaSuccess) {
        void* a = qa;
        void* b = qb;
        for (int i = 0; i < gsteps && rc == DGC_OK; ++i) {
          rc = lserk4_launches(h, a, b, res, 0.0, dt, true, cs);
          std::swap(a, b);
        }
        e = cudaStreamEndCapture(cs, &g);
      }
      cudaStreamDestroy(cs);
      if (rc != DGC_OK) {
        if (g) cudaGraphDestroy(g);
        return rc;
      }
      if (e != cudaSuccess) return cuda_fail(e, "capture LSERK4 graph");
      e = cudaGraphInstantiate(&h->graph_exec, g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) return cuda_fail(e, "instantiate LSERK4 graph");
      h->graph_key[0] = qa;
      h->graph_key[1] = qb;
      h->graph_key[2] = res;
      h->graph_dt = dt;
      h->graph_steps = gsteps;
      h->launches -= (int64_t)gsteps * 6;  // captured, not executed
    }
    // gsteps is even, so every replay starts and ends with the state in qa
    while (nsteps - done >= gsteps) {
      CK(cudaGraphLaunch(h->graph_exec, s));
      h->launches += (int64_t)gsteps * 6;
      done += gsteps;
    }
  }
  for (; done < nsteps; ++done) {
    if (int rc = lserk4_launches(h, cur, other, res, 0.0, dt, true, s)) return rc;
    std::swap(cur, other);
  }
  if (final_state) *final_state = cur;
  return DGC_OK;
}

extern "C" int dgc_check_device_status(dgc_handle h, int* code) {
  if (!h) return fail(DGC_ERR_ARG, "null handle");
  int w[16] = {};
  CK(cudaMemcpy(w, h->d_status, sizeof w, cudaMemcpyDeviceToHost));
  const int v = w[0];
  if (code) *code = v;
  if (v != 0) {
    unsigned long long rec[3];
    std::memcpy(rec, w + 2, sizeof rec);
    CK(cudaMemset(h->d_status, 0, 64));
    if (v != 1) return fail(DGC_ERR_DEVICE, "device-side error code %d (singular diagonal block)", v);
    return fail(DGC_ERR_DEVICE,
                "device-side error code %d (bounded wait expired after %llu ns, %llu SM cycles, %llu polls)", v,
                rec[0], rec[1], rec[2]);
  }
  return DGC_OK;
}

extern "C" int64_t dgc_launch_count(dgc_handle h) { return h ? h->launches : -1; }

// ---------------------------------------------------------------- host-only queries
extern "C" int dgc_ref_nodes(int order, double* r, double* s) {
  if (!r || !s) return fail(DGC_ERR_ARG, "null argument");
  if (order < 1 || order > dgc::kMaxOrder) return fail(DGC_ERR_ARG, "order %d outside [1, %d]", order, dgc::kMaxOrder);
  std::vector<double> rr, ss;
  dgc::warp_blend_nodes(order, rr, ss);
  std::memcpy(r, rr.data(), rr.size() * sizeof(double));
  std::memcpy(s, ss.data(), ss.size() * sizeof(double));
  return DGC_OK;
}

extern "C" int dgc_ref_operator(int order, int which, double* out) {
  if (!out) return fail(DGC_ERR_ARG, "null argument");
  dgc::RefElement re;
  std::string err;
  if (!dgc::build_ref_element(order, re, err)) return fail(DGC_ERR_ARG, "%s", err.c_str());
  const std::vector<double>* src = nullptr;
  switch (which) {
    case DGC_OP_DR_WEAK: src = &re.Drw; break;
    case DGC_OP_DS_WEAK: src = &re.Dsw; break;
    case DGC_OP_LIFT: src = &re.Lw; break;
    case DGC_OP_DR_STRONG: src = &re.Drs; break;
    case DGC_OP_DS_STRONG: src = &re.Dss; break;
    case DGC_OP_MASS: src = &re.M; break;
    case DGC_OP_V: src = &re.V; break;
    default: return fail(DGC_ERR_ARG, "unknown operator %d", which);
  }
  std::memcpy(out, src->data(), src->size() * sizeof(double));
  return DGC_OK;
}

extern "C" int dgc_mesh_neighbors(dgc_handle h, int32_t* nbr, int* num_bfaces) {
  if (!h) return fail(DGC_ERR_ARG, "null handle");
  if (nbr) std::memcpy(nbr, h->mesh.nbr.data(), h->mesh.nbr.size() * sizeof(int32_t));
  if (num_bfaces) *num_bfaces = h->mesh.num_bfaces;
  return DGC_OK;
}

extern "C" int dgc_host_mesh(int nv, const double* vxy, int K, const int32_t* cells, int order, double* geom,
                             int32_t* nbr, int* num_bfaces) {
  dgc::RefElement re;
  dgc::MeshData m;
  std::string err;
  if (!dgc::build_ref_element(order, re, err)) return fail(DGC_ERR_ARG, "%s", err.c_str());
  if (!dgc::build_mesh(vxy, nv, cells, K, re, m, err)) return fail(DGC_ERR_MESH, "%s", err.c_str());
  if (geom) std::memcpy(geom, m.geom.data(), m.geom.size() * sizeof(double));
  if (nbr) std::memcpy(nbr, m.nbr.data(), m.nbr.size() * sizeof(int32_t));
  if (num_bfaces) *num_bfaces = m.num_bfaces;
  return DGC_OK;
}

// ---------------------------------------------------------------- autotuning
namespace {

int refresh_rhs_info(dgc_handle h) {
  dgk::LaunchInfo li;
  const cudaError_t e = dgc::rhs_dispatch_any(h, dgk::RhsParams{}, 0, &li);
  if (e != cudaSuccess) return cuda_fail(e, "configure rhs kernel");
  h->rhs_info = li;
  return DGC_OK;
}

std::string tune_key(dgc_handle h) {
  cudaDeviceProp prop{};
  cudaGetDeviceProperties(&prop, h->device);
  int kb = 0;
  while ((1 << (kb + 1)) <= h->K) ++kb;  // K bucket: floor(log2 K)
  char buf[sizeof prop.name + 96];  // the device name can fill its 256 bytes
  std::snprintf(buf, sizeof buf, "%s|sm%d|phys%d|prec%d|N%d|K2^%d", prop.name, prop.multiProcessorCount,
                h->desc.physics, h->prec, h->N, kb);
  for (char* c = buf; *c; ++c)
    if (*c == ' ') *c = '_';
  return buf;
}

int cache_lookup(const std::string& key) {
  const char* path = std::getenv("DGC_TUNE_CACHE");
  if (!path || !*path) return -1;
  FILE* f = std::fopen(path, "r");
  if (!f) return -1;
  char k[300];
  int v, found = -1;
  while (std::fscanf(f, "%299s %d", k, &v) == 2)
    if (key == k) found = v;  // last entry wins
  std::fclose(f);
  return found;
}

void cache_store(const std::string& key, int v) {
  const char* path = std::getenv("DGC_TUNE_CACHE");
  if (!path || !*path) return;
  FILE* f = std::fopen(path, "a");
  if (!f) return;
  std::fprintf(f, "%s %d\n", key.c_str(), v);
  std::fclose(f);
}

}  // namespace

extern "C" int dgc_num_variants(dgc_handle h) {
  if (!h) return fail(DGC_ERR_ARG, "null handle");
  if (h->desc.physics == DGC_LAPLACE || h->prec == DGC_F32C) return 1;
  return dgk::rhs_num_variants(h->prec == DGC_F32, h->N);
}

extern "C" int dgc_set_variant(dgc_handle h, int v) {
  if (!h) return fail(DGC_ERR_ARG, "null handle");
  const int nv = dgc_num_variants(h);
  if (v < 0 || v >= nv) return fail(DGC_ERR_ARG, "variant %d outside [0, %d)", v, nv);
  if (v != h->rhs_variant && h->graph_exec) {
    // the cached LSERK4 graph holds the previous variant's kernel
    cudaGraphExecDestroy(h->graph_exec);
    h->graph_exec = nullptr;
  }
  h->rhs_variant = v;
  return h->desc.physics == DGC_LAPLACE ? DGC_OK : refresh_rhs_info(h);
}

extern "C" int dgc_autotune(dgc_handle h, int reps, double* times_ms, int* chosen, void* stream) {
  if (!h) return fail(DGC_ERR_ARG, "null handle");
  if (int rc = check_time_dependent(h)) return rc;
  const int nv = dgc_num_variants(h);
  const std::string key = tune_key(h);
  if (!times_ms) {
    const int v = cache_lookup(key);
    if (v >= 0 && v < nv) {
      if (chosen) *chosen = v;
      return dgc_set_variant(h, v);
    }
  }
  if (reps <= 0) reps = 10;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t bytes = dgc::state_bytes(h);
  void *qa = nullptr, *qb = nullptr, *res = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  const int keep = h->rhs_variant;
  const int64_t l0 = h->launches;
  int best = 0;
  double best_ms = 1e300;
  int rc = DGC_OK;
  cudaError_t ce = cudaMalloc(&qa, bytes);
  if (ce == cudaSuccess) ce = cudaMalloc(&qb, bytes);
  if (ce == cudaSuccess) ce = cudaMalloc(&res, bytes);
  if (ce == cudaSuccess) ce = cudaMemsetAsync(qa, 0, bytes, s);
  if (ce == cudaSuccess) ce = cudaMemsetAsync(qb, 0, bytes, s);
  if (ce == cudaSuccess) ce = cudaMemsetAsync(res, 0, bytes, s);
  if (ce == cudaSuccess) ce = cudaEventCreate(&e0);
  if (ce == cudaSuccess) ce = cudaEventCreate(&e1);
  if (ce != cudaSuccess) rc = cuda_fail(ce, "autotune scratch set-up");
  for (int v = 0; v < nv && rc == DGC_OK; ++v) {
    h->rhs_variant = v;
    std::vector<float> ms;
    for (int r = 0; r < reps + 2 && rc == DGC_OK; ++r) {
      cudaEventRecord(e0, s);
      rc = dgc_lserk4_stage(h, r % 5, (r & 1) ? qb : qa, (r & 1) ? qa : qb, res, 0.0, 1e-6, s);
      cudaEventRecord(e1, s);
      cudaEventSynchronize(e1);
      float t = 0.0f;
      cudaEventElapsedTime(&t, e0, e1);
      if (r >= 2) ms.push_back(t);
    }
    std::sort(ms.begin(), ms.end());
    const double med = ms.empty() ? 1e300 : ms[ms.size() / 2];
    if (times_ms) times_ms[v] = med;
    if (med < best_ms) {
      best_ms = med;
      best = v;
    }
  }
  // one exit path: the scratch and the events are released whatever failed
  h->launches = l0;
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(qa);
  cudaFree(qb);
  cudaFree(res);
  h->rhs_variant = keep;
  if (rc != DGC_OK) return rc;
  cache_store(key, best);
  if (chosen) *chosen = best;
  return dgc_set_variant(h, best);
}
