// dgc_internal.hpp -- the handle behind the C ABI (include/dgc_gb300.h).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "dgc_gb300.h"
#include "rhs_launch.cuh"
#include "setup.hpp"

namespace dgc {
struct IpdgState;
struct CoarseSpace;
}

// the handle behind the opaque C type
struct dgc_handle_s {
  dgc_problem_desc desc{};
  dgc::RefElement re;
  dgc::MeshData mesh;
  int K = 0, N = 0, Np = 0, NpP = 0, Nfp = 0, Nf = 1, prec = DGC_F64;
  int device = 0, sm_count = 0;
  // device data owned by the handle
  double* d_geom = nullptr;   // [K][16] FP64
  int32_t* d_nbr = nullptr;   // [K][4]
  double* d_bxy = nullptr;    // boundary face node coordinates
  double* d_tau = nullptr;    // [K][4] laplace penalty per face
  double* d_kgeom64 = nullptr;  // [K][16] kernel geometry records (dgc::kernel_geometry), FP64
  float* d_kgeom32 = nullptr;   // [K][16] the same, rounded once to FP32
  float* d_tau32 = nullptr;     // [K][4] laplace penalty, FP32
  void* d_mats64[2] = {nullptr, nullptr};  // weak, strong (transposed, padded)
  void* d_mats32[2] = {nullptr, nullptr};
  void* d_tc_b = nullptr;     // FP32 tensor-core operand [Dr | Ds | LIFT] (strong form, split TF32)
  void* d_blk_b = nullptr;    // FP32 operand of the register-blocked kernel (weak form, rows padded to NpP)
  void* d_blk_bs = nullptr;   // the same rows in the strong form (compensated-state kernel, DGC_F32C)
  int* d_status = nullptr;    // device-side error word
  double* d_time = nullptr;   // simulation time for graph-replayed steps
  dgk::LaunchInfo rhs_info;
  int rhs_variant = 0;        // tile-shape variant of the fused RHS kernel (dgc_autotune)
  int64_t launches = 0;       // kernels launched through this handle
  // cached CUDA graph of LSERK4 steps
  cudaGraphExec_t graph_exec = nullptr;
  void* graph_key[3] = {nullptr, nullptr, nullptr};
  double graph_dt = 0.0;
  int graph_steps = 0;
  dgc::IpdgState* ipdg = nullptr;
  dgc::CoarseSpace* coarse = nullptr;  // two-level preconditioner (dgc_coarse_build)
};

namespace dgc {

// bytes of one state vector of the handle (DGC_F32C: the hi and lo vectors)
inline size_t state_bytes(const dgc_handle_s* h) {
  return (size_t)h->K * h->Nf * h->NpP * (h->prec == DGC_F32 ? 4 : 8);
}

int set_error(int code, const char* msg);
// the stage kernel of the handle's precision and variant (capi.cu)
cudaError_t rhs_dispatch_any(const dgc_handle_s* h, const dgk::RhsParams& p, cudaStream_t s, dgk::LaunchInfo* info);
int upload_operators(dgc_handle_s* h, int form);
int device_init(dgc_handle_s* h);
void device_free(dgc_handle_s* h);
int ipdg_init(dgc_handle_s* h);
void ipdg_free(dgc_handle_s* h);
void ipdg_operators_changed(dgc_handle_s* h);
// block-Jacobi inverse of the SPD laplace form (built once), and z = Binv r
// (FP64 vectors; the blocks and sums in FP32 with fp32)
int ipdg_build_preconditioner(dgc_handle_s* h, cudaStream_t s);
int ipdg_block_jacobi_apply(dgc_handle_s* h, const double* r, double* z, cudaStream_t s);
// z = Binv r with the FP32 blocks, r given in FP64 (r64) or FP32 (r32, used when
// non-null); z32, when non-null, receives an FP32 copy of z
int ipdg_block_jacobi_apply_f32(dgc_handle_s* h, const double* r64, const float* r32, double* z, float* z32,
                                cudaStream_t s);
// the SPD form's shift, and whether the boundary types are the handle's uniform ones
double ipdg_shift(const dgc_handle_s* h);
bool ipdg_uniform_bc(const dgc_handle_s* h);
// coarse space (csrc/coarse.cu): z (+)= P A_c^-1 P^T r (binv_r = Binv r when the
// caller has it, else NULL; fp32: the two smoothing applies of S in FP32, and
// binv_r32, when non-null, an FP32 copy of binv_r the caller already holds in
// the coarse space's first FP32 work vector); freeing
// dots, when non-null (FP32 path with add), makes the last kernel also form
// out = (r.r, z.r, z.q) with the new z, on `grid` blocks
struct CoarseDots {
  double* out;
  const double* r;
  const double* q;
  int grid;
};
int coarse_apply(dgc_handle_s* h, const double* r, const double* binv_r, double* z, bool add, bool fp32,
                 cudaStream_t s, bool binv_r32_ready = false, const CoarseDots* dots = nullptr);
void coarse_free(CoarseSpace* c);
// flexible PCG with M = Binv + coarse term from the residual r (updated) on x, until
// r.r <= tol2 or maxit iterations; op32: S applied through the FP32 kernels
int two_level_pcg(dgc_handle_s* h, double* x, double* r, double tol2, int maxit, int* iterations, bool op32,
                  cudaStream_t s);
// device list of the cells with a boundary face (laplace handles)
int ipdg_boundary_cells(const dgc_handle_s* h, const int** cells, int* n);
// out = S u with the FP32 kernels (any laplace handle; one field, native layout)
int ipdg_spd_apply_f32(dgc_handle_s* h, const float* u, float* out, cudaStream_t s);
// stage-kernel parameters of a handle (geometry, operators, physics; no buffers)
dgk::RhsParams rhs_base_params(dgc_handle_s* h);
// LSERK4 (Carpenter-Kennedy) coefficients: 0 -> a_k, 1 -> b_k, 2 -> c_k (5 each)
const double* lserk_coeffs(int which);

}  // namespace dgc
