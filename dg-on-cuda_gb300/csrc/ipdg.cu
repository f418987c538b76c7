// ipdg.cu -- host side of the matrix-free laplace_2d operator and its solvers:
// block-Jacobi set-up on the GPU, the device-driven PCG loop (scalars stay in
// device memory; three-iteration chunks replayed from a CUDA graph), and mixed
// precision iterative refinement (FP32 inner PCG, FP64 residuals).
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <type_traits>
#include <vector>

#include "dgc_internal.hpp"
#include "ipdg.cuh"
#include "ipdg_blk.cuh"

namespace dgk {

enum IpdgKernel : int { IK_GRAD_PLAIN, IK_GRAD_PCG, IK_DIV_LAPLACE, IK_DIV_SPD, IK_DIV_SPD_DOT, IK_DIV_RESID,
                        IK_UPDATE, IK_START };

template <typename R, int N>
const void* ipdg_fn(int kind) {
  switch (kind) {
    case IK_GRAD_PLAIN: return (const void*)ipdg_grad_kernel<R, N, GRAD_PLAIN>;
    case IK_GRAD_PCG: return (const void*)ipdg_grad_kernel<R, N, GRAD_PCG>;
    case IK_DIV_LAPLACE: return (const void*)ipdg_div_kernel<R, N, DIV_LAPLACE>;
    case IK_DIV_SPD: return (const void*)ipdg_div_kernel<R, N, DIV_SPD>;
    case IK_DIV_SPD_DOT: return (const void*)ipdg_div_kernel<R, N, DIV_SPD_DOT>;
    case IK_DIV_RESID: return (const void*)ipdg_div_kernel<R, N, DIV_RESID>;
    case IK_UPDATE: return (const void*)pcg_update_kernel<R, N>;
    case IK_START: return (const void*)pcg_start_kernel<R, N>;
    default: return nullptr;
  }
}

template <typename R, int N>
cudaError_t ipdg_launch_n(int kind, const IpdgParams& p, int sm, cudaStream_t s) {
  using C = IpdgConfig<R, N>;
  static std::once_flag once[8];
  static int bps[8];
  static cudaError_t st[8];
  const void* fn = ipdg_fn<R, N>(kind);
  if (!fn) return cudaErrorInvalidValue;
  const bool dyn = kind <= IK_DIV_RESID;
  const int smem = dyn ? (int)C::kSmem : 0;
  std::call_once(once[kind], [&] {
    st[kind] = cudaSuccess;
    if (dyn) st[kind] = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (st[kind] == cudaSuccess) st[kind] = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps[kind], fn, 256, smem);
  });
  if (st[kind] != cudaSuccess) return st[kind];
  const int ntiles = (p.K + C::TE - 1) / C::TE;
  int grid = sm * (bps[kind] > 0 ? bps[kind] : 1);
  if (grid > ntiles) grid = ntiles;
  void* args[] = {const_cast<IpdgParams*>(&p)};
  return cudaLaunchKernel(fn, dim3(grid), dim3(256), args, smem, s);
}

// register-blocked FP32 CG kernels
enum IpdgBlkKernel : int { IB_GRAD = 0, IB_DIV = 1, IB_UPDATE = 2 };

template <int N>
cudaError_t ipdg_blk_launch_n(int kind, const IpdgParams& p, int sm, cudaStream_t s) {
  using B = IpdgBlk<N>;
  static std::once_flag once[3];
  static int bps[3];
  static cudaError_t st[3];
  const void* fn = kind == IB_GRAD ? (const void*)ipdg_grad_blk_kernel<N>
                   : kind == IB_DIV ? (const void*)ipdg_div_blk_kernel<N>
                                    : (const void*)pcg_update_blk_kernel<N>;
  const int smem = (int)(kind == IB_GRAD ? B::kSmemGrad : kind == IB_DIV ? B::kSmemDiv : B::kSmemUpd);
  std::call_once(once[kind], [&] {
    st[kind] = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    // all of the unified L1 / shared storage as shared memory, so residency is
    // set by registers (64 per thread: 4 CTAs of 256) rather than the carveout
    if (st[kind] == cudaSuccess)
      st[kind] = cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    if (st[kind] == cudaSuccess)
      st[kind] = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps[kind], fn, 256, smem);
  });
  if (st[kind] != cudaSuccess) return st[kind];
  const int ntiles = (p.K + B::TE - 1) / B::TE;
  int grid = sm * (bps[kind] > 0 ? bps[kind] : 1);
  if (grid > ntiles) grid = ntiles;
  // programmatic dependent launch: the kernels wait (grid_dep_wait) before
  // their first access to the CG scalars and vectors
  void* args[] = {const_cast<IpdgParams*>(&p)};
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(256);
  cfg.dynamicSmemBytes = (size_t)smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = stage_overlap_enabled() ? 1 : 0;
  return cudaLaunchKernelExC(&cfg, fn, args);
}

cudaError_t ipdg_blk_launch(int N, int kind, const IpdgParams& p, int sm, cudaStream_t s) {
  switch (N) {
    case 1: return ipdg_blk_launch_n<1>(kind, p, sm, s);
    case 2: return ipdg_blk_launch_n<2>(kind, p, sm, s);
    case 3: return ipdg_blk_launch_n<3>(kind, p, sm, s);
    case 4: return ipdg_blk_launch_n<4>(kind, p, sm, s);
    case 5: return ipdg_blk_launch_n<5>(kind, p, sm, s);
    case 6: return ipdg_blk_launch_n<6>(kind, p, sm, s);
    case 7: return ipdg_blk_launch_n<7>(kind, p, sm, s);
    case 8: return ipdg_blk_launch_n<8>(kind, p, sm, s);
    default: return cudaErrorInvalidValue;
  }
}

template <typename R>
cudaError_t bc_rhs_launch(int N, int ncells, const IpdgParams& p, const int* cells, const double* g, const double* h,
                          R* out, cudaStream_t s) {
  if (ncells == 0) return cudaSuccess;
#define DGK_BC(n) \
  case n: ipdg_bc_rhs_kernel<R, n><<<ncells, 64, 0, s>>>(p, cells, g, h, out); return cudaGetLastError();
  switch (N) {
    DGK_BC(1) DGK_BC(2) DGK_BC(3) DGK_BC(4) DGK_BC(5) DGK_BC(6) DGK_BC(7) DGK_BC(8)
    default: return cudaErrorInvalidValue;
  }
#undef DGK_BC
}

template <typename R>
cudaError_t bc_jump_launch(int N, int ncells, const IpdgParams& p, const int* cells, R* out, cudaStream_t s) {
  if (ncells == 0) return cudaSuccess;
#define DGK_BJ(n) \
  case n: ipdg_bc_jump_kernel<R, n><<<ncells, 64, 0, s>>>(p, cells, out); return cudaGetLastError();
  switch (N) {
    DGK_BJ(1) DGK_BJ(2) DGK_BJ(3) DGK_BJ(4) DGK_BJ(5) DGK_BJ(6) DGK_BJ(7) DGK_BJ(8)
    default: return cudaErrorInvalidValue;
  }
#undef DGK_BJ
}

// floats per packed block (IpdgBlk<N>::PK) for the allocation on the host
int packed_stride(int N) {
  switch (N) {
    case 1: return IpdgBlk<1>::PK;
    case 2: return IpdgBlk<2>::PK;
    case 3: return IpdgBlk<3>::PK;
    case 4: return IpdgBlk<4>::PK;
    case 5: return IpdgBlk<5>::PK;
    case 6: return IpdgBlk<6>::PK;
    case 7: return IpdgBlk<7>::PK;
    case 8: return IpdgBlk<8>::PK;
    default: return 0;
  }
}

cudaError_t pack_binv(int N, int K, const double* binv, int bstr, float* out, cudaStream_t s) {
  auto go = [&](auto kern, int pk) {
    const int64_t n = (int64_t)K * pk;
    kern<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(K, binv, bstr, out);
    return cudaGetLastError();
  };
  switch (N) {
    case 1: return go(pack_binv_kernel<1>, IpdgBlk<1>::PK);
    case 2: return go(pack_binv_kernel<2>, IpdgBlk<2>::PK);
    case 3: return go(pack_binv_kernel<3>, IpdgBlk<3>::PK);
    case 4: return go(pack_binv_kernel<4>, IpdgBlk<4>::PK);
    case 5: return go(pack_binv_kernel<5>, IpdgBlk<5>::PK);
    case 6: return go(pack_binv_kernel<6>, IpdgBlk<6>::PK);
    case 7: return go(pack_binv_kernel<7>, IpdgBlk<7>::PK);
    case 8: return go(pack_binv_kernel<8>, IpdgBlk<8>::PK);
    default: return cudaErrorInvalidValue;
  }
}

template <typename R>
cudaError_t ipdg_launch(int N, int kind, const IpdgParams& p, int sm, cudaStream_t s) {
  switch (N) {
    case 1: return ipdg_launch_n<R, 1>(kind, p, sm, s);
    case 2: return ipdg_launch_n<R, 2>(kind, p, sm, s);
    case 3: return ipdg_launch_n<R, 3>(kind, p, sm, s);
    case 4: return ipdg_launch_n<R, 4>(kind, p, sm, s);
    case 5: return ipdg_launch_n<R, 5>(kind, p, sm, s);
    case 6: return ipdg_launch_n<R, 6>(kind, p, sm, s);
    case 7: return ipdg_launch_n<R, 7>(kind, p, sm, s);
    case 8: return ipdg_launch_n<R, 8>(kind, p, sm, s);
    default: return cudaErrorInvalidValue;
  }
}

// blocks[k] += shift J_k M (the diagonal blocks of S + shift J M)
__global__ void k_block_shift(int K, int Np, int bstr, const double* __restrict__ geom, const double* __restrict__ M,
                              double shift, double* __restrict__ blocks) {
  const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (g >= (int64_t)K * Np * Np) return;
  const int k = (int)(g / (Np * Np)), q = (int)(g % (Np * Np));
  blocks[(size_t)k * bstr + q] += shift * geom[(size_t)k * 16 + 4] * M[q];  // geom slot 4: J
}

template <int N>
cudaError_t diag_blocks_n(int K, int dirichlet, double shift, const double* geom, const int4* nbr, const double* tau,
                          const double* Dr, const double* Ds, const double* L, const double* M, double* blocks,
                          float* blocks32, int bstr, int* status, cudaStream_t s) {
  using O = Order<N>;
  const int64_t n = (int64_t)K * O::Np;
  ipdg_diag_blocks_kernel<N><<<(unsigned)((n + 127) / 128), 128, 0, s>>>(K, dirichlet, geom, nbr, tau, Dr, Ds, L,
                                                                         M, blocks, bstr);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if (shift != 0.0) {
    const int64_t m = n * O::Np;
    k_block_shift<<<(unsigned)((m + 255) / 256), 256, 0, s>>>(K, O::Np, bstr, geom, M, shift, blocks);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  block_invert_kernel<N><<<K, 128, 0, s>>>(K, blocks, blocks32, bstr, status);
  return cudaGetLastError();
}

cudaError_t diag_blocks(int N, int K, int dirichlet, double shift, const double* geom, const int4* nbr,
                        const double* tau, const double* Dr, const double* Ds, const double* L, const double* M,
                        double* blocks, float* blocks32, int bstr, int* status, cudaStream_t s) {
#define DGK_DB(n) \
  case n:          \
    return diag_blocks_n<n>(K, dirichlet, shift, geom, nbr, tau, Dr, Ds, L, M, blocks, blocks32, bstr, status, s);
  switch (N) {
    DGK_DB(1) DGK_DB(2) DGK_DB(3) DGK_DB(4) DGK_DB(5) DGK_DB(6) DGK_DB(7) DGK_DB(8)
    default: return cudaErrorInvalidValue;
  }
#undef DGK_DB
}

// ---------------------------------------------------------------- vector kernels
// sum of x over valid nodes (padding excluded) into *out
__global__ void k_valid_sum(size_t n, int NpP, int Np, const double* __restrict__ x, double* out) {
  __shared__ double red[16];
  double s = 0.0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    if ((int)(i % NpP) < Np) s += x[i];
  s = block_sum(s, red);
  if (threadIdx.x == 0) atomicAdd(out, s);
}
// x -= *c / count on valid nodes (c read on the device)
__global__ void k_sub_mean(size_t n, int NpP, int Np, const double* __restrict__ c, double count, double* x) {
  const double m = *c / count;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    if ((int)(i % NpP) < Np) x[i] -= m;
}
__global__ void k_r64_to_r32(size_t n, const double* __restrict__ r, double scale, float* __restrict__ out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = (float)(r[i] * scale);
}
__global__ void k_x_update(size_t n, double* __restrict__ x, const float* __restrict__ d, double scale) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    x[i] += scale * (double)d[i];
}
template <typename R>
__global__ void k_dot(size_t n, const R* __restrict__ a, const R* __restrict__ b, double* out) {
  __shared__ double red[16];
  double s = 0.0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    s += (double)a[i] * (double)b[i];
  s = block_sum(s, red);
  if (threadIdx.x == 0) atomicAdd(out, s);
}
__global__ void k_add(size_t n, double* __restrict__ x, const double* __restrict__ d) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    x[i] += d[i];
}
// out = J_k M f_k (mass-weighted right-hand side), one thread per node
__global__ void k_mass(int K, int Np, int NpP, const double* __restrict__ geom, const double* __restrict__ M,
                       const double* __restrict__ f, double* __restrict__ out) {
  const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (g >= (int64_t)K * Np) return;
  const int k = (int)(g / Np), i = (int)(g % Np);
  double s = 0.0;
  for (int j = 0; j < Np; ++j) s += M[i * Np + j] * f[(size_t)k * NpP + j];
  out[(size_t)k * NpP + i] = geom[(size_t)k * 16 + 4] * s;
}
// start of a CG solve: relative tolerance against the initial residual
__global__ void k_cg_start(CgScalars* cg, double tol2, int maxit) {
  cg->bb = cg->rr[0];
  cg->tol2 = tol2;
  cg->maxit = maxit;
  if (cg->rr[0] == 0.0) cg->done = 1;
}
// convergence bookkeeping, one thread: done when rr <= tol2 * bb or iters >= maxit
// a plain launch: it ends the overlap chain of one iteration's launches
__global__ void k_cg_check(CgScalars* cg, int slot) {
  if (cg->done) return;
  cg->iters += 1;
  if (cg->rr[slot] <= cg->tol2 * cg->bb) cg->done = 1;
  else if (cg->iters >= cg->maxit) cg->done = 2;
}

}  // namespace dgk

namespace dgc {

struct IpdgState {
  int bstr = 0;
  bool ready = false;          // preconditioner built
  double* binv64 = nullptr;
  float* binv32 = nullptr;
  float* binv_pk32 = nullptr;  // [K][PK] packed upper triangles (register-blocked FP32 CG)
  float* ops_blk32 = nullptr;  // rows Dr^T | Ds^T | LIFT^T, strong form, padded to NpP columns
  float* mass_blk32 = nullptr; // rows of M padded to NpP columns
  uint8_t* bcdir = nullptr;    // per boundary node condition type (dgc_laplace_set_bc_types), or NULL
  double shift = 0.0;          // S = -J M (A - shift I) (dgc_laplace_set_shift)
  double* bproj = nullptr;     // projected right-hand side of a singular (all-Neumann) solve
  int* bcells = nullptr;       // cells with a boundary face
  int n_bcells = 0;
  int* jcells = nullptr;       // boundary cells and their face neighbours (ipdg_bc_jump_kernel)
  int n_jcells = 0;
  int bc_data_mode = DGC_BC_DATA_REFERENCE;
  void* qd = nullptr;          // lifted Dirichlet data q_d, 2 x K x NpP in the handle's precision
  void* mass64 = nullptr;      // padded M in FP64 / FP32
  void* mass32 = nullptr;
  double* dense64 = nullptr;   // row-major Dr | Ds | L | M (FP64) for the block set-up
  // workspace: FP64 and FP32 vector sets
  double* w64[10] = {};
  float* w32[10] = {};
  dgk::CgScalars* cg = nullptr;   // [3]: fp64 solve, fp32 inner solve, standalone FP32 applies (never done)
  double* dots = nullptr;         // scratch dot products
  dgk::CgScalars* h_cg = nullptr; // pinned host mirror
  double* h_dots = nullptr;
  // graphs of 3-iteration chunks per precision
  cudaGraphExec_t chunk[2] = {nullptr, nullptr};
  const void* chunk_key[2] = {nullptr, nullptr};
};

namespace {

int cuda_err(cudaError_t e, const char* what) {
  std::string m = std::string(what) + ": " + cudaGetErrorString(e);
  return set_error(DGC_ERR_CUDA, m.c_str());
}
#define CKI(call)                                    \
  do {                                               \
    cudaError_t e_ = (call);                         \
    if (e_ != cudaSuccess) return cuda_err(e_, #call); \
  } while (0)

size_t nvec(const dgc_handle_s* h) { return (size_t)h->K * h->NpP; }

// The chunk graphs capture IpdgParams by value (shift, boundary-type array):
// every change of those drops them, and the next graphed solve captures anew.
void drop_chunk_graphs(IpdgState* st) {
  for (int i = 0; i < 2; ++i) {
    if (st->chunk[i]) cudaGraphExecDestroy(st->chunk[i]);
    st->chunk[i] = nullptr;
    st->chunk_key[i] = nullptr;
  }
}

template <typename R>
dgk::IpdgParams base(const dgc_handle_s* h) {
  dgk::IpdgParams p{};
  p.K = h->K;
  p.dirichlet = h->desc.dirichlet;
  p.geom = sizeof(R) == 8 ? (const void*)h->d_kgeom64 : (const void*)h->d_kgeom32;
  p.nbr = reinterpret_cast<const int4*>(h->d_nbr);
  p.tau = sizeof(R) == 8 ? (const void*)h->d_tau : (const void*)h->d_tau32;
  p.mats = sizeof(R) == 8 ? h->d_mats64[1] : h->d_mats32[1];
  p.mass = sizeof(R) == 8 ? h->ipdg->mass64 : h->ipdg->mass32;
  p.binv = sizeof(R) == 8 ? (const void*)h->ipdg->binv64 : (const void*)h->ipdg->binv32;
  p.mats_blk = h->ipdg->ops_blk32;
  p.mass_blk = h->ipdg->mass_blk32;
  p.binv_pk = h->ipdg->binv_pk32;
  p.bcdir = h->ipdg->bcdir;
  p.shift = h->ipdg->shift;
  p.status = h->d_status;
  return p;
}

template <typename R>
int launch(dgc_handle_s* h, int kind, const dgk::IpdgParams& p, cudaStream_t s) {
  cudaError_t e = dgk::ipdg_launch<R>(h->N, kind, p, h->sm_count, s);
  if (e != cudaSuccess) return cuda_err(e, "ipdg kernel launch");
  ++h->launches;
  return DGC_OK;
}

int grid_for(const dgc_handle_s* h, size_t n) {
  return (int)std::min<size_t>((n + 255) / 256, (size_t)h->sm_count * 8);
}

template <typename R>
R* wv(dgc_handle_s* h, int i) {
  if constexpr (sizeof(R) == 8) return h->ipdg->w64[i];
  else return h->ipdg->w32[i];
}

// workspace slots
// (search directions rotate through W_P .. W_P + 2 by iteration slot, so that
// a grad pass never overwrites the direction its neighbours are still reading)
enum { W_X = 0, W_R = 1, W_Z = 2, W_P = 3, W_AP = 6, W_QX = 7, W_QY = 8, W_T = 9, W_COUNT = 10 };

}  // namespace

int ipdg_build_preconditioner(dgc_handle_s* h, cudaStream_t s) {
  IpdgState* st = h->ipdg;
  if (st->ready) return DGC_OK;
  if (st->bcdir)
    return set_error(DGC_ERR_UNSUPPORTED, "block-Jacobi CG needs uniform boundary types (clear the per-node types)");
  cudaError_t e = dgk::diag_blocks(h->N, h->K, h->desc.dirichlet, st->shift, h->d_geom,
                                   reinterpret_cast<const int4*>(h->d_nbr), h->d_tau,
                                   st->dense64, st->dense64 + (size_t)h->Np * h->Np,
                                   st->dense64 + (size_t)2 * h->Np * h->Np,
                                   st->dense64 + (size_t)2 * h->Np * h->Np + (size_t)h->Np * 3 * h->Nfp,
                                   st->binv64, st->binv32, st->bstr, h->d_status, s);
  if (e != cudaSuccess) return cuda_err(e, "block-Jacobi set-up");
  e = dgk::pack_binv(h->N, h->K, st->binv64, st->bstr, st->binv_pk32, s);
  if (e != cudaSuccess) return cuda_err(e, "block-Jacobi packing");
  h->launches += 3;
  st->ready = true;
  return DGC_OK;
}

// z = Binv r elementwise (FP64 vectors, native layout; padding nodes of z set to
// 0), the blocks and the sums in B's type (FP64 here; the FP32 cycle of the
// two-level preconditioner uses the packed blocks below).  A CTA holds whole
// elements (blockDim = E * NpP) and stages r once per node in shared memory, in
// B's type.
// The residual may also come as an FP32 vector (RIn = float: the two-level
// cycle's FP32 operator output, no FP64 round trip), and z32, when given,
// receives an FP32 copy of z (the input of the next FP32 operator apply).
template <typename B, typename RIn = double>
__global__ void k_bj_apply(int K, int Np, int NpP, int bstr, const B* __restrict__ binv,
                           const RIn* __restrict__ r, double* __restrict__ z, float* __restrict__ z32) {
  __shared__ B rs[256];
  const int E = blockDim.x / NpP;
  const int t = threadIdx.x, e = t / NpP, i = t - e * NpP;
  const int64_t k = (int64_t)blockIdx.x * E + e;
  const bool live = k < K;
  rs[t] = live ? (B)r[k * NpP + i] : (B)0;
  __syncthreads();
  if (!live) return;
  B s = 0;
  if (i < Np) {
    const B* Bk = binv + (size_t)k * bstr;
    const B* rk = rs + e * NpP;
    for (int j = 0; j < Np; ++j) s += Bk[j * Np + i] * rk[j];
  }
  z[k * NpP + i] = (double)s;
  if (z32) z32[k * NpP + i] = (float)s;
}

// z = Binv r with the packed FP32 blocks (upper triangles row by row, PK floats
// per element: the layout the register-blocked CG update stages), for the
// two-level cycle: 496 instead of 900 bytes of blocks per element at N = 4.
// A CTA holds whole elements; it copies their packed blocks (contiguous) and
// residuals into shared memory, and thread (element, node i) sums over j with
// B(i, j) = B(min, max) through a per-CTA table of packed indices.
template <int N, typename RIn>
__global__ void k_bj_apply_pk(int K, const float* __restrict__ bpk, const RIn* __restrict__ r,
                              double* __restrict__ z, float* __restrict__ z32) {
  // compile-time sizes: the j loop unrolls, so the block and residual reads of
  // a thread are independent loads issued back to back
  constexpr int Np = dgk::IpdgBlk<N>::Np, NpP = dgk::IpdgBlk<N>::NpP, PK = dgk::IpdgBlk<N>::PK;
  extern __shared__ __align__(16) float sm_pk[];
  const int E = blockDim.x / NpP;
  float* sB = sm_pk;                  // [E][PK]
  float* sR = sB + E * PK;            // [E][NpP]
  uint16_t* tab = reinterpret_cast<uint16_t*>(sR + E * NpP);  // [Np][NpP]
  const int t = threadIdx.x, e = t / NpP, i = t - e * NpP;
  const int64_t k0 = (int64_t)blockIdx.x * E;
  const int ne = (int)min((int64_t)E, (int64_t)K - k0);
  const float4* src = reinterpret_cast<const float4*>(bpk + k0 * PK);
  for (int x = t; x < ne * PK / 4; x += blockDim.x) reinterpret_cast<float4*>(sB)[x] = src[x];
  if (e < ne) sR[t] = (float)r[(k0 + e) * NpP + i];
  for (int q = t; q < Np * NpP; q += blockDim.x) {
    const int j = q / NpP, ii = q - j * NpP;
    const int lo = ii < j ? ii : j, hi = ii < j ? j : ii;
    tab[q] = (uint16_t)(ii >= Np ? 0 : lo * Np - lo * (lo - 1) / 2 + (hi - lo));
  }
  __syncthreads();
  if (e >= ne) return;
  float acc = 0.0f;
  if (i < Np) {
    const float* Bk = sB + e * PK;
    const float* rk = sR + e * NpP;
#pragma unroll
    for (int j = 0; j < Np; ++j) acc += Bk[tab[j * NpP + i]] * rk[j];
  }
  const int64_t o = (k0 + e) * NpP + i;
  z[o] = (double)acc;
  if (z32) z32[o] = acc;
}

int ipdg_block_jacobi_apply(dgc_handle_s* h, const double* r, double* z, cudaStream_t s) {
  if (int rc = ipdg_build_preconditioner(h, s)) return rc;
  const IpdgState* st = h->ipdg;
  const int E = 256 / h->NpP;  // whole elements per CTA (NpP <= 48)
  const unsigned grid = (unsigned)((h->K + E - 1) / E), block = (unsigned)(E * h->NpP);
  k_bj_apply<double><<<grid, block, 0, s>>>(h->K, h->Np, h->NpP, st->bstr, st->binv64, r, z, nullptr);
  CKI(cudaGetLastError());
  ++h->launches;
  return DGC_OK;
}

int ipdg_block_jacobi_apply_f32(dgc_handle_s* h, const double* r64, const float* r32, double* z, float* z32,
                                cudaStream_t s) {
  if (int rc = ipdg_build_preconditioner(h, s)) return rc;
  const IpdgState* st = h->ipdg;
  const int E = 256 / h->NpP;
  const unsigned grid = (unsigned)((h->K + E - 1) / E), block = (unsigned)(E * h->NpP);
  auto go = [&](auto nc) {
    constexpr int N = decltype(nc)::value;
    constexpr int PK = dgk::IpdgBlk<N>::PK, Np = dgk::IpdgBlk<N>::Np, NpP = dgk::IpdgBlk<N>::NpP;
    const size_t smem = (size_t)E * PK * 4 + (size_t)E * NpP * 4 + (size_t)Np * NpP * 2;
    if (r32)
      k_bj_apply_pk<N, float><<<grid, block, smem, s>>>(h->K, st->binv_pk32, r32, z, z32);
    else
      k_bj_apply_pk<N, double><<<grid, block, smem, s>>>(h->K, st->binv_pk32, r64, z, z32);
  };
  switch (h->N) {
    case 1: go(std::integral_constant<int, 1>{}); break;
    case 2: go(std::integral_constant<int, 2>{}); break;
    case 3: go(std::integral_constant<int, 3>{}); break;
    case 4: go(std::integral_constant<int, 4>{}); break;
    case 5: go(std::integral_constant<int, 5>{}); break;
    case 6: go(std::integral_constant<int, 6>{}); break;
    case 7: go(std::integral_constant<int, 7>{}); break;
    case 8: go(std::integral_constant<int, 8>{}); break;
    default: return set_error(DGC_ERR_ARG, "order outside 1..8");
  }
  CKI(cudaGetLastError());
  ++h->launches;
  return DGC_OK;
}

int upload_ipdg_matrices(dgc_handle_s* h) {
  IpdgState* st = h->ipdg;
  const int Np = h->Np, NF = 3 * h->Nfp;
  std::vector<double> m64((size_t)st->bstr, 0.0);
  std::vector<float> m32((size_t)st->bstr, 0.0f);
  for (int i = 0; i < Np * Np; ++i) {
    m64[i] = h->re.M[i];
    m32[i] = (float)h->re.M[i];
  }
  CKI(cudaMemcpy(st->mass64, m64.data(), m64.size() * 8, cudaMemcpyHostToDevice));
  CKI(cudaMemcpy(st->mass32, m32.data(), m32.size() * 4, cudaMemcpyHostToDevice));
  std::vector<double> dense;
  dense.insert(dense.end(), h->re.Drs.begin(), h->re.Drs.end());
  dense.insert(dense.end(), h->re.Dss.begin(), h->re.Dss.end());
  dense.insert(dense.end(), h->re.Ls.begin(), h->re.Ls.end());
  dense.insert(dense.end(), h->re.M.begin(), h->re.M.end());
  (void)NF;
  CKI(cudaMemcpy(st->dense64, dense.data(), dense.size() * 8, cudaMemcpyHostToDevice));
  // register-blocked operands: row j of Dr^T, Ds^T (j < Np), row m of LIFT^T and
  // row j of M, each padded with zeros to NpP columns
  const int NpP = h->NpP;
  std::vector<float> ob((size_t)(2 * Np + NF) * NpP, 0.0f), mb((size_t)Np * NpP, 0.0f);
  for (int j = 0; j < Np; ++j)
    for (int i = 0; i < Np; ++i) {
      ob[(size_t)j * NpP + i] = (float)h->re.Drs[(size_t)i * Np + j];
      ob[(size_t)(Np + j) * NpP + i] = (float)h->re.Dss[(size_t)i * Np + j];
      mb[(size_t)j * NpP + i] = (float)h->re.M[(size_t)j * Np + i];
    }
  for (int m = 0; m < NF; ++m)
    for (int i = 0; i < Np; ++i) ob[(size_t)(2 * Np + m) * NpP + i] = (float)h->re.Ls[(size_t)i * NF + m];
  CKI(cudaMemcpy(st->ops_blk32, ob.data(), ob.size() * 4, cudaMemcpyHostToDevice));
  CKI(cudaMemcpy(st->mass_blk32, mb.data(), mb.size() * 4, cudaMemcpyHostToDevice));
  st->ready = false;
  return DGC_OK;
}

int ipdg_init(dgc_handle_s* h) {
  if (h->desc.physics != DGC_LAPLACE) return DGC_OK;
  if (h->desc.tau != DGC_TAU_ONE && h->desc.tau != DGC_TAU_SCALED)
    return set_error(DGC_ERR_ARG, "unknown tau mode");
  auto* st = new IpdgState();
  h->ipdg = st;
  const int Np = h->Np, NF = 3 * h->Nfp;
  st->bstr = (Np * Np + 3) / 4 * 4;
  if (h->desc.tau == DGC_TAU_ONE) {  // both penalty copies (FP64 and FP32 kernels)
    std::vector<double> ones((size_t)4 * h->K, 1.0);
    std::vector<float> ones32((size_t)4 * h->K, 1.0f);
    CKI(cudaMemcpy(h->d_tau, ones.data(), ones.size() * 8, cudaMemcpyHostToDevice));
    CKI(cudaMemcpy(h->d_tau32, ones32.data(), ones32.size() * 4, cudaMemcpyHostToDevice));
  }
  CKI(cudaMalloc(&st->mass64, (size_t)st->bstr * 8));
  CKI(cudaMalloc(&st->mass32, (size_t)st->bstr * 4));
  CKI(cudaMalloc(&st->dense64, ((size_t)3 * Np * Np + (size_t)Np * NF) * 8));
  CKI(cudaMalloc(&st->binv64, (size_t)h->K * st->bstr * 8));
  CKI(cudaMalloc(&st->binv32, (size_t)h->K * st->bstr * 4));
  CKI(cudaMemset(st->binv64, 0, (size_t)h->K * st->bstr * 8));
  CKI(cudaMemset(st->binv32, 0, (size_t)h->K * st->bstr * 4));
  const size_t pk = (size_t)dgk::packed_stride(h->N);
  CKI(cudaMalloc(&st->binv_pk32, (size_t)h->K * pk * 4));
  CKI(cudaMemset(st->binv_pk32, 0, (size_t)h->K * pk * 4));
  {
    std::vector<int> bc;
    for (int k = 0; k < h->K; ++k)
      if (h->mesh.nbr[4 * (size_t)k] < 0 || h->mesh.nbr[4 * (size_t)k + 1] < 0 || h->mesh.nbr[4 * (size_t)k + 2] < 0)
        bc.push_back(k);
    st->n_bcells = (int)bc.size();
    CKI(cudaMalloc(&st->bcells, std::max<size_t>(bc.size(), 1) * sizeof(int)));
    if (!bc.empty()) CKI(cudaMemcpy(st->bcells, bc.data(), bc.size() * sizeof(int), cudaMemcpyHostToDevice));
    std::vector<char> mark(h->K, 0);
    for (int k : bc) {
      mark[k] = 1;
      for (int f = 0; f < 3; ++f) {
        const int nb = h->mesh.nbr[4 * (size_t)k + f];
        if (nb >= 0) mark[nb >> 2] = 1;
      }
    }
    std::vector<int> jc;
    for (int k = 0; k < h->K; ++k)
      if (mark[k]) jc.push_back(k);
    st->n_jcells = (int)jc.size();
    CKI(cudaMalloc(&st->jcells, std::max<size_t>(jc.size(), 1) * sizeof(int)));
    if (!jc.empty()) CKI(cudaMemcpy(st->jcells, jc.data(), jc.size() * sizeof(int), cudaMemcpyHostToDevice));
  }
  CKI(cudaMalloc(&st->ops_blk32, (size_t)(2 * Np + NF) * h->NpP * 4));
  CKI(cudaMalloc(&st->mass_blk32, (size_t)Np * h->NpP * 4));
  const size_t n = nvec(h);
  for (int i = 0; i < W_COUNT; ++i) {
    CKI(cudaMalloc(&st->w64[i], n * 8));
    CKI(cudaMalloc(&st->w32[i], n * 4));
    CKI(cudaMemset(st->w64[i], 0, n * 8));
    CKI(cudaMemset(st->w32[i], 0, n * 4));
  }
  CKI(cudaMalloc(&st->cg, 3 * sizeof(dgk::CgScalars)));
  CKI(cudaMemset(st->cg, 0, 3 * sizeof(dgk::CgScalars)));
  CKI(cudaMalloc(&st->dots, 64));
  CKI(cudaMallocHost(&st->h_cg, 2 * sizeof(dgk::CgScalars)));
  CKI(cudaMallocHost(&st->h_dots, 64));
  return upload_ipdg_matrices(h);
}

void ipdg_free(dgc_handle_s* h) {
  coarse_free(h->coarse);
  h->coarse = nullptr;
  IpdgState* st = h->ipdg;
  if (!st) return;
  for (int i = 0; i < 2; ++i)
    if (st->chunk[i]) cudaGraphExecDestroy(st->chunk[i]);
  cudaFree(st->binv64);
  cudaFree(st->binv32);
  cudaFree(st->binv_pk32);
  cudaFree(st->ops_blk32);
  cudaFree(st->mass_blk32);
  cudaFree(st->bcdir);
  cudaFree(st->bcells);
  cudaFree(st->jcells);
  cudaFree(st->qd);
  cudaFree(st->bproj);
  cudaFree(st->mass64);
  cudaFree(st->mass32);
  cudaFree(st->dense64);
  for (int i = 0; i < W_COUNT; ++i) {
    cudaFree(st->w64[i]);
    cudaFree(st->w32[i]);
  }
  cudaFree(st->cg);
  cudaFree(st->dots);
  cudaFreeHost(st->h_cg);
  cudaFreeHost(st->h_dots);
  delete st;
  h->ipdg = nullptr;
}

double ipdg_shift(const dgc_handle_s* h) { return h->ipdg ? h->ipdg->shift : 0.0; }

bool ipdg_uniform_bc(const dgc_handle_s* h) { return !h->ipdg || !h->ipdg->bcdir; }

int ipdg_boundary_cells(const dgc_handle_s* h, const int** cells, int* n) {
  if (!h->ipdg) return set_error(DGC_ERR_UNSUPPORTED, "not a laplace handle");
  *cells = h->ipdg->bcells;
  *n = h->ipdg->n_bcells;
  return DGC_OK;
}

void ipdg_operators_changed(dgc_handle_s* h) {
  if (h->ipdg) upload_ipdg_matrices(h);
}

namespace {

int check_laplace(dgc_handle_s* h) {
  if (!h) return set_error(DGC_ERR_ARG, "null handle");
  if (h->desc.physics != DGC_LAPLACE || !h->ipdg)
    return set_error(DGC_ERR_UNSUPPORTED, "operation needs a DGC_LAPLACE handle");
  return DGC_OK;
}

// grad + div of u into out, with the given div mode (and b for residuals)
template <typename R>
int apply(dgc_handle_s* h, int div_kind, const R* u, R* out, const R* b, double* dot, cudaStream_t s) {
  dgk::IpdgParams p = base<R>(h);
  p.u = u;
  p.qx = wv<R>(h, W_QX);
  p.qy = wv<R>(h, W_QY);
  if (int rc = launch<R>(h, dgk::IK_GRAD_PLAIN, p, s)) return rc;
  p.du_src = u;
  p.out = out;
  p.b = b;
  p.dot_out = dot;
  return launch<R>(h, div_kind, p, s);
}

// one CG iteration (three launches) for slot i mod 3
template <typename R>
int cg_iteration(dgc_handle_s* h, int cgi, int slot, int first, cudaStream_t s) {
  dgk::IpdgParams p = base<R>(h);
  p.cg = h->ipdg->cg + cgi;
  p.slot = slot;
  p.first = first;
  p.u = wv<R>(h, W_Z);
  p.p = wv<R>(h, W_P + slot);
  p.p_old = wv<R>(h, W_P + (slot + 2) % 3);
  p.qx = wv<R>(h, W_QX);
  p.qy = wv<R>(h, W_QY);
  // FP32: the register-blocked kernels (ipdg_blk.cuh); FP64: the one-node-per-thread ones
  auto run = [&](int kind_r, int kind_blk) -> int {
    if (sizeof(R) == 4) {
      const cudaError_t e = dgk::ipdg_blk_launch(h->N, kind_blk, p, h->sm_count, s);
      if (e != cudaSuccess) return cuda_err(e, "ipdg blocked kernel launch");
      ++h->launches;
      return DGC_OK;
    }
    return launch<R>(h, kind_r, p, s);
  };
  if (int rc = run(dgk::IK_GRAD_PCG, dgk::IB_GRAD)) return rc;
  p.du_src = wv<R>(h, W_P + slot);
  p.out = wv<R>(h, W_AP);
  if (int rc = run(dgk::IK_DIV_SPD_DOT, dgk::IB_DIV)) return rc;
  p.x = wv<R>(h, W_X);
  p.r = wv<R>(h, W_R);
  p.z = wv<R>(h, W_Z);
  p.Ap = wv<R>(h, W_AP);
  if (int rc = run(dgk::IK_UPDATE, dgk::IB_UPDATE)) return rc;
  dgk::k_cg_check<<<1, 1, 0, s>>>(h->ipdg->cg + cgi, (slot + 1) % 3);
  CKI(cudaGetLastError());
  ++h->launches;
  return DGC_OK;
}

// PCG on S x = r0 with x = 0 initially (x, r in workspace slots W_X, W_R);
// stops at ||r|| <= rtol ||r0|| or maxit.  Returns iterations via *iters.
template <typename R>
int pcg_core(dgc_handle_s* h, double rtol, int maxit, bool use_graph, int* iters, int* converged, cudaStream_t s) {
  IpdgState* st = h->ipdg;
  const int cgi = sizeof(R) == 8 ? 0 : 1;
  dgk::CgScalars init{};
  CKI(cudaMemcpyAsync(st->cg + cgi, &init, sizeof init, cudaMemcpyHostToDevice, s));
  dgk::IpdgParams p = base<R>(h);
  p.cg = st->cg + cgi;
  p.r = wv<R>(h, W_R);
  p.z = wv<R>(h, W_Z);
  CKI(cudaMemsetAsync(wv<R>(h, W_X), 0, nvec(h) * sizeof(R), s));
  for (int i = 0; i < 3; ++i) CKI(cudaMemsetAsync(wv<R>(h, W_P + i), 0, nvec(h) * sizeof(R), s));
  if (int rc = launch<R>(h, dgk::IK_START, p, s)) return rc;
  // bb = rr[0], tol2 = rtol^2 (device side, one thread)
  dgk::k_cg_start<<<1, 1, 0, s>>>(st->cg + cgi, rtol * rtol, maxit);
  CKI(cudaGetLastError());
  if (int rc = cg_iteration<R>(h, cgi, 0, 1, s)) return rc;
  const void* key = wv<R>(h, W_X);
  if (use_graph && (!st->chunk[cgi] || st->chunk_key[cgi] != key)) {
    if (st->chunk[cgi]) cudaGraphExecDestroy(st->chunk[cgi]);
    st->chunk[cgi] = nullptr;
    cudaStream_t cs;
    CKI(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    int rc = DGC_OK;
    const int64_t l0 = h->launches;
    if (e == cudaSuccess) {
      for (int i = 1; i <= 3 && rc == DGC_OK; ++i) rc = cg_iteration<R>(h, cgi, i % 3, 0, cs);
      e = cudaStreamEndCapture(cs, &g);
    }
    h->launches = l0;
    cudaStreamDestroy(cs);
    if (rc != DGC_OK) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (e != cudaSuccess) return cuda_err(e, "capture CG chunk");
    e = cudaGraphInstantiate(&st->chunk[cgi], g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_err(e, "instantiate CG chunk");
    st->chunk_key[cgi] = key;
  }
  int done_it = 1;
  const int chunks_per_check = 4;
  while (true) {
    for (int c = 0; c < chunks_per_check; ++c) {
      if (use_graph) {
        CKI(cudaGraphLaunch(st->chunk[cgi], s));
        h->launches += 12;
      } else {
        for (int i = 1; i <= 3; ++i)
          if (int rc = cg_iteration<R>(h, cgi, i % 3, 0, s)) return rc;
      }
      done_it += 3;
    }
    CKI(cudaMemcpyAsync(st->h_cg + cgi, st->cg + cgi, sizeof(dgk::CgScalars), cudaMemcpyDeviceToHost, s));
    CKI(cudaStreamSynchronize(s));
    if (st->h_cg[cgi].done) break;
    if (done_it > maxit + 12) break;
  }
  *iters = st->h_cg[cgi].iters;
  *converged = st->h_cg[cgi].done == 1;
  return DGC_OK;
}

template <typename R>
int true_residual(dgc_handle_s* h, const double* b64, const double* x64, double* r64, double* rr, cudaStream_t s) {
  IpdgState* st = h->ipdg;
  CKI(cudaMemsetAsync(st->dots, 0, 8, s));
  if (int rc = apply<double>(h, dgk::IK_DIV_RESID, x64, r64, b64, st->dots, s)) return rc;
  CKI(cudaMemcpyAsync(st->h_dots, st->dots, 8, cudaMemcpyDeviceToHost, s));
  CKI(cudaStreamSynchronize(s));
  *rr = st->h_dots[0];
  return DGC_OK;
}

}  // namespace

int ipdg_spd_apply_f32(dgc_handle_s* h, const float* u, float* out, cudaStream_t s) {
  if (int rc = check_laplace(h)) return rc;
  IpdgState* st = h->ipdg;
  if (st->bcdir) return apply<float>(h, dgk::IK_DIV_SPD, u, out, nullptr, nullptr, s);
  // uniform boundary types: the register-blocked passes of the FP32 CG
  // iteration with beta = 0 (the grad pass copies u to the direction slot W_T,
  // the div pass writes S u), on a CG scalar record that never stops
  dgk::IpdgParams p = base<float>(h);
  p.cg = st->cg + 2;
  p.first = 1;
  p.slot = 0;
  p.u = u;
  p.p_old = u;
  p.p = wv<float>(h, W_T);
  p.qx = wv<float>(h, W_QX);
  p.qy = wv<float>(h, W_QY);
  cudaError_t e = dgk::ipdg_blk_launch(h->N, dgk::IB_GRAD, p, h->sm_count, s);
  if (e != cudaSuccess) return cuda_err(e, "ipdg blocked kernel launch");
  p.du_src = wv<float>(h, W_T);
  p.out = out;
  e = dgk::ipdg_blk_launch(h->N, dgk::IB_DIV, p, h->sm_count, s);
  if (e != cudaSuccess) return cuda_err(e, "ipdg blocked kernel launch");
  h->launches += 2;
  return DGC_OK;
}

}  // namespace dgc

using namespace dgc;

extern "C" int dgc_laplace_apply(dgc_handle h, const void* u, void* out, void* stream) {
  if (int rc = check_laplace(h)) return rc;
  if (!u || !out || u == out) return set_error(DGC_ERR_ARG, "u and out must be distinct, non-null buffers");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  return h->prec == DGC_F64
             ? apply<double>(h, dgk::IK_DIV_LAPLACE, (const double*)u, (double*)out, nullptr, nullptr, s)
             : apply<float>(h, dgk::IK_DIV_LAPLACE, (const float*)u, (float*)out, nullptr, nullptr, s);
}

extern "C" int dgc_laplace_spd_apply(dgc_handle h, const void* u, void* out, void* stream) {
  if (int rc = check_laplace(h)) return rc;
  if (!u || !out || u == out) return set_error(DGC_ERR_ARG, "u and out must be distinct, non-null buffers");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  return h->prec == DGC_F64 ? apply<double>(h, dgk::IK_DIV_SPD, (const double*)u, (double*)out, nullptr, nullptr, s)
                            : apply<float>(h, dgk::IK_DIV_SPD, (const float*)u, (float*)out, nullptr, nullptr, s);
}

extern "C" int dgc_pcg_solve(dgc_handle h, const double* b, double* x, const dgc_solve_opts* opts,
                             dgc_solve_stats* stats, void* stream) {
  if (int rc = check_laplace(h)) return rc;
  if (!b || !x || !opts || b == x) return set_error(DGC_ERR_ARG, "b and x must be distinct, non-null buffers");
  if (!(opts->rtol > 0.0) || opts->maxit <= 0) return set_error(DGC_ERR_ARG, "rtol must be > 0 and maxit > 0");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  IpdgState* st = h->ipdg;
  if (int rc = ipdg_build_preconditioner(h, s)) return rc;
  const auto t0 = std::chrono::steady_clock::now();
  const size_t n = nvec(h);
  dgc_solve_stats S{};
  // all-Neumann without shift: S is singular with the constants as null space;
  // solve with the right-hand side projected onto its range (zero sum over the
  // valid nodes) and return the solution with zero mean
  const bool singular = !h->desc.dirichlet && st->shift == 0.0;
  const double count = (double)h->K * h->Np;
  if (singular) {
    if (!st->bproj) CKI(cudaMalloc(&st->bproj, n * 8));
    CKI(cudaMemcpyAsync(st->bproj, b, n * 8, cudaMemcpyDeviceToDevice, s));
    CKI(cudaMemsetAsync(st->dots, 0, 8, s));
    dgk::k_valid_sum<<<grid_for(h, n), 256, 0, s>>>(n, h->NpP, h->Np, b, st->dots);
    dgk::k_sub_mean<<<grid_for(h, n), 256, 0, s>>>(n, h->NpP, h->Np, st->dots, count, st->bproj);
    CKI(cudaGetLastError());
    h->launches += 2;
    b = st->bproj;
  }
  // ||b||^2
  CKI(cudaMemsetAsync(st->dots, 0, 8, s));
  dgk::k_dot<double><<<grid_for(h, n), 256, 0, s>>>(n, b, b, st->dots);
  CKI(cudaGetLastError());
  CKI(cudaMemcpyAsync(st->h_dots, st->dots, 8, cudaMemcpyDeviceToHost, s));
  CKI(cudaStreamSynchronize(s));
  const double bb = st->h_dots[0];
  const double tol2 = opts->rtol * opts->rtol * bb;
  double* r64 = st->w64[W_T];
  double rr = 0.0;
  // r = b - S x (x is the caller's initial guess)
  if (int rc = true_residual<double>(h, b, x, r64, &rr, s)) return rc;
  const bool graph = opts->use_graph != 0;
  const bool two_level = opts->mode == DGC_SOLVE_TWO_LEVEL || opts->mode == DGC_SOLVE_TWO_LEVEL_MIXED;
  if (opts->mode != DGC_SOLVE_FP64_PCG && opts->mode != DGC_SOLVE_MIXED_IR && !two_level)
    return set_error(DGC_ERR_ARG, "unknown solve mode");
  if (two_level && !h->coarse) return set_error(DGC_ERR_ARG, "the two-level modes need dgc_coarse_build first");
  // Refinement loop on the true FP64 residual.  FP64 mode: each pass solves
  // S d = r in FP64 to a little below the remaining target (a second pass
  // mops up the drift between CG's recursive and true residuals).  Mixed
  // mode: each pass solves the normalised residual system in FP32 to
  // inner_rtol and adds the correction in FP64.
  const bool fp64 = opts->mode == DGC_SOLVE_FP64_PCG;
  const double inner = opts->inner_rtol > 0.0 ? opts->inner_rtol : 1e-4;
  const int max_outer = opts->max_outer > 0 ? opts->max_outer : (fp64 ? 4 : 20);
  int outer = 0;
  while (rr > tol2 && outer < max_outer) {
    const int budget = opts->maxit - S.inner_iterations;
    if (budget <= 0) break;
    const double nr = std::sqrt(rr);
    int it = 0, conv = 0;
    if (two_level) {
      // on x and the true residual directly: to a little below the target in FP64,
      // by inner_rtol per pass with the FP32 operator (the true residual is refined here)
      const bool op32 = opts->mode == DGC_SOLVE_TWO_LEVEL_MIXED;
      const double t2 = op32 ? std::max(0.25 * tol2, inner * inner * rr) : 0.25 * tol2;
      if (int rc = two_level_pcg(h, x, r64, t2, budget, &it, op32, s)) return rc;
      S.inner_iterations += it;
      ++outer;
      if (int rc = true_residual<double>(h, b, x, r64, &rr, s)) return rc;
      continue;
    }
    if (fp64) {
      CKI(cudaMemcpyAsync(st->w64[W_R], r64, n * 8, cudaMemcpyDeviceToDevice, s));
      const double rel = std::max(0.5 * std::sqrt(tol2 / rr), 1e-15);
      if (int rc = pcg_core<double>(h, rel, budget, graph, &it, &conv, s)) return rc;
      dgk::k_add<<<grid_for(h, n), 256, 0, s>>>(n, x, st->w64[W_X]);
    } else {
      dgk::k_r64_to_r32<<<grid_for(h, n), 256, 0, s>>>(n, r64, 1.0 / nr, st->w32[W_R]);
      CKI(cudaGetLastError());
      if (int rc = pcg_core<float>(h, inner, budget, graph, &it, &conv, s)) return rc;
      dgk::k_x_update<<<grid_for(h, n), 256, 0, s>>>(n, x, st->w32[W_X], nr);
    }
    CKI(cudaGetLastError());
    h->launches += 2;
    S.inner_iterations += it;
    ++outer;
    if (int rc = true_residual<double>(h, b, x, r64, &rr, s)) return rc;
  }
  S.outer_iterations = outer;
  S.iterations = S.inner_iterations;
  CKI(cudaStreamSynchronize(s));
  if (singular) {  // the null-space component of x: zero mean
    CKI(cudaMemsetAsync(st->dots, 0, 8, s));
    dgk::k_valid_sum<<<grid_for(h, n), 256, 0, s>>>(n, h->NpP, h->Np, x, st->dots);
    dgk::k_sub_mean<<<grid_for(h, n), 256, 0, s>>>(n, h->NpP, h->Np, st->dots, count, x);
    CKI(cudaGetLastError());
    CKI(cudaStreamSynchronize(s));
    h->launches += 2;
  }
  S.final_relres = bb > 0.0 ? std::sqrt(rr / bb) : 0.0;
  S.converged = rr <= tol2 ? 1 : 0;
  S.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (stats) *stats = S;
  if (!S.converged) {
    char msg[160];
    snprintf(msg, sizeof msg, "PCG did not reach the requested tolerance (relative residual %.3e > %.3e after %d iterations)",
             S.final_relres, opts->rtol, S.iterations);
    return set_error(DGC_ERR_NOT_CONVERGED, msg);
  }
  return DGC_OK;
}

extern "C" int dgc_mass_apply(dgc_handle h, const double* f, double* out, void* stream) {
  if (int rc = check_laplace(h)) return rc;
  if (!f || !out || f == out) return set_error(DGC_ERR_ARG, "f and out must be distinct, non-null buffers");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int64_t n = (int64_t)h->K * h->Np;
  CKI(cudaMemsetAsync(out, 0, nvec(h) * 8, s));
  dgk::k_mass<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(h->K, h->Np, h->NpP, h->d_geom, (const double*)h->ipdg->mass64,
                                                      f, out);
  CKI(cudaGetLastError());
  ++h->launches;
  return DGC_OK;
}

extern "C" int dgc_block_jacobi(dgc_handle h, double* blocks, void* stream) {
  if (int rc = check_laplace(h)) return rc;
  if (!blocks) return set_error(DGC_ERR_ARG, "null argument");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (int rc = ipdg_build_preconditioner(h, s)) return rc;
  const int Np = h->Np, bs = h->ipdg->bstr;
  CKI(cudaMemcpy2DAsync(blocks, (size_t)Np * Np * 8, h->ipdg->binv64, (size_t)bs * 8, (size_t)Np * Np * 8, h->K,
                        cudaMemcpyDeviceToDevice, s));
  return DGC_OK;
}

extern "C" int dgc_laplace_set_bc_types(dgc_handle h, const uint8_t* flags) {
  if (int rc = check_laplace(h)) return rc;
  IpdgState* st = h->ipdg;
  const size_t nb = (size_t)h->mesh.num_bfaces * h->Nfp;
  if (!flags) {
    if (st->bcdir) drop_chunk_graphs(st);
    cudaFree(st->bcdir);
    st->bcdir = nullptr;
    return DGC_OK;
  }
  if (nb == 0) return DGC_OK;
  if (!st->bcdir) {
    drop_chunk_graphs(st);
    CKI(cudaMalloc(&st->bcdir, nb));
  }
  CKI(cudaMemcpy(st->bcdir, flags, nb, cudaMemcpyHostToDevice));
  return DGC_OK;
}

extern "C" int dgc_laplace_bc_rhs(dgc_handle h, const double* g, const double* hn, void* out, void* stream) {
  if (int rc = check_laplace(h)) return rc;
  if (!out) return set_error(DGC_ERR_ARG, "null output");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  IpdgState* st = h->ipdg;
  const bool jump = st->bc_data_mode == DGC_BC_DATA_CONSISTENT && g && st->n_bcells;
  const size_t n = nvec(h), esz = h->prec == DGC_F64 ? 8 : 4;
  if (jump && !st->qd) {  // zero off the boundary cells for good: only those are ever written
    CKI(cudaMalloc(&st->qd, 2 * n * esz));
    CKI(cudaMemset(st->qd, 0, 2 * n * esz));
  }
  cudaError_t e;
  auto run = [&](auto zero, void* const* mats) {
    using R = decltype(zero);
    dgk::IpdgParams p = base<R>(h);
    p.mats = mats[1];
    if (jump) {
      p.qx = st->qd;
      p.qy = static_cast<char*>(st->qd) + n * esz;
    }
    e = dgk::bc_rhs_launch<R>(h->N, st->n_bcells, p, st->bcells, g, hn, static_cast<R*>(out), s);
    if (e == cudaSuccess && jump) e = dgk::bc_jump_launch<R>(h->N, st->n_jcells, p, st->jcells, static_cast<R*>(out), s);
  };
  if (h->prec == DGC_F64)
    run(0.0, h->d_mats64);
  else
    run(0.0f, h->d_mats32);
  if (e != cudaSuccess) return cuda_err(e, "boundary-data kernel");
  if (st->n_bcells) ++h->launches;
  if (jump && st->n_jcells) ++h->launches;
  return DGC_OK;
}

extern "C" int dgc_laplace_set_bc_data_mode(dgc_handle h, int mode) {
  if (int rc = check_laplace(h)) return rc;
  if (mode != DGC_BC_DATA_REFERENCE && mode != DGC_BC_DATA_CONSISTENT)
    return set_error(DGC_ERR_ARG, "unknown boundary-data mode");
  h->ipdg->bc_data_mode = mode;
  return DGC_OK;
}

extern "C" int dgc_laplace_set_shift(dgc_handle h, double shift) {
  if (int rc = check_laplace(h)) return rc;
  if (!(shift >= 0.0)) return set_error(DGC_ERR_ARG, "shift must be >= 0");
  IpdgState* st = h->ipdg;
  if (st->shift != shift) {
    st->shift = shift;
    st->ready = false;  // the block-Jacobi blocks depend on the shift
    drop_chunk_graphs(st);
  }
  return DGC_OK;
}
