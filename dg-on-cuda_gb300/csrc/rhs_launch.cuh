// rhs_launch.cuh -- host-side launch of the fused RHS kernel for one
// (precision, order, physics) instantiation.  Persistent grid: as many CTAs as
// fit on the GPU at once (occupancy x SM count), capped by the tile count.
#pragma once

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <utility>

#include "dg_rhs.cuh"

namespace dgk {

struct LaunchInfo {
  int threads = 0, tile = 0, smem = 0, blocks_per_sm = 0;
};

// Launch of a stage kernel that calls grid_dep_wait before it touches the
// previous launch's data (dg_rhs_blk_kernel, dg_rhs_tcp_kernel,
// dg_rhs_x2_kernel, dg_batch_kernel, the FP32 CG kernels): with programmatic stream serialization its CTAs are
// scheduled, and run their set-up (barriers, operator copies, tensor memory),
// while the previous kernel of the stream finishes.  DGC_STAGE_OVERLAP=0 in the
// environment launches them without the attribute.
inline bool stage_overlap_enabled() {
  static const bool on = [] {
    const char* v = std::getenv("DGC_STAGE_OVERLAP");
    return !(v && std::strcmp(v, "0") == 0);
  }();
  return on;
}

template <typename... Args, typename... Act>
cudaError_t launch_stage(void (*kern)(Args...), int grid, int threads, size_t smem, cudaStream_t s, Act&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3((unsigned)threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = stage_overlap_enabled() ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kern, std::forward<Act>(args)...);
}

template <typename R, int N, int P>
cudaError_t rhs_configure(LaunchInfo* info) {
  using C = RhsConfig<R, N, P>;
  static std::once_flag once;
  static cudaError_t st = cudaSuccess;
  static int bps = 0;
  std::call_once(once, [] {
    st = cudaFuncSetAttribute(dg_rhs_kernel<R, N, P>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::kSmem);
    if (st == cudaSuccess)
      st = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, dg_rhs_kernel<R, N, P>, C::kThreads, C::kSmem);
  });
  if (info) {
    info->threads = C::kThreads;
    info->tile = C::TE;
    info->smem = C::kSmem;
    info->blocks_per_sm = bps;
  }
  return st;
}

template <typename R, int N, int P>
cudaError_t rhs_launch(const RhsParams& p, int sm_count, cudaStream_t s) {
  using C = RhsConfig<R, N, P>;
  LaunchInfo li;
  cudaError_t e = rhs_configure<R, N, P>(&li);
  if (e != cudaSuccess) return e;
  const int ntiles = (p.K + C::TE - 1) / C::TE;
  int grid = sm_count * (li.blocks_per_sm > 0 ? li.blocks_per_sm : 1);
  if (grid > ntiles) grid = ntiles;
  dg_rhs_kernel<R, N, P><<<grid, C::kThreads, C::kSmem, s>>>(p);
  return cudaGetLastError();
}

// dispatch over order (1..8) and physics; defined in rhs_f64.cu / rhs_f32.cu
template <typename R>
cudaError_t rhs_dispatch(int N, int P, int variant, const RhsParams& p, int sm_count, cudaStream_t s,
                         LaunchInfo* info);
// number of tile-shape variants compiled for (precision, order)
int rhs_num_variants(int prec_f32, int N);
// the compensated-state stage kernel (dg_rhs_x2.cuh), defined in rhs_x2.cu
cudaError_t rhs_x2_dispatch(int N, int P, const RhsParams& p, int sm_count, cudaStream_t s, LaunchInfo* info);

}  // namespace dgk

#include "dg_rhs_blk.cuh"
#include "dg_rhs_tc.cuh"
#include "dg_rhs_tct.cuh"
#include "dg_rhs_tcp.cuh"
#include "dg_rhs_v2.cuh"
#include "dg_rhs_x2.cuh"

namespace dgk {

template <int N, int P, int G, int EPT>
cudaError_t rhs_v2_shape(const RhsParams* p, int sm_count, cudaStream_t s, LaunchInfo* info) {
  using C = V2Config<N, P, G, EPT>;
  static std::once_flag once;
  static cudaError_t st = cudaSuccess;
  static int bps = 0;
  std::call_once(once, [] {
    st = cudaFuncSetAttribute(dg_rhs_v2_kernel<N, P, G, EPT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              C::kSmem);
    if (st == cudaSuccess)
      st = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, dg_rhs_v2_kernel<N, P, G, EPT>, C::kThreads,
                                                         C::kSmem);
  });
  if (st != cudaSuccess) return st;
  if (info) {
    info->threads = C::kThreads;
    info->tile = C::TE;
    info->smem = C::kSmem;
    info->blocks_per_sm = bps;
    return cudaSuccess;
  }
  const int ntiles = (p->K + C::TE - 1) / C::TE;
  int grid = sm_count * (bps > 0 ? bps : 1);
  if (grid > ntiles) grid = ntiles;
  dg_rhs_v2_kernel<N, P, G, EPT><<<grid, C::kThreads, C::kSmem, s>>>(*p);
  return cudaGetLastError();
}

// launch (p != nullptr) or describe (info != nullptr) tile-shape variant v
template <int N, int P>
cudaError_t rhs_v2(int v, const RhsParams* p, int sm, cudaStream_t s, LaunchInfo* info) {
  using S = V2Shapes<N>;
  switch (v) {
    case 0: return rhs_v2_shape<N, P, S::G[0], S::EPT[0]>(p, sm, s, info);
    case 1: return rhs_v2_shape<N, P, S::G[1], S::EPT[1]>(p, sm, s, info);
    case 2: return rhs_v2_shape<N, P, S::G[2], S::EPT[2]>(p, sm, s, info);
    default: return cudaErrorInvalidValue;
  }
}

template <int N, int P>
cudaError_t rhs_tc(const RhsParams* p, int sm_count, cudaStream_t s, LaunchInfo* info) {
  using C = TcConfig<N, P>;
  static std::once_flag once;
  static cudaError_t st = cudaSuccess;
  static int bps = 0;
  std::call_once(once, [] {
    st = cudaFuncSetAttribute(dg_rhs_tc_kernel<N, P>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::kSmem);
    if (st == cudaSuccess)
      st = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, dg_rhs_tc_kernel<N, P>, C::kThreads, C::kSmem);
  });
  if (st != cudaSuccess) return st;
  if (info) {
    info->threads = C::kThreads;
    info->tile = C::TE;
    info->smem = C::kSmem;
    info->blocks_per_sm = bps;
    return cudaSuccess;
  }
  if (!p->mats_tc) return cudaErrorInvalidValue;
  const int ntiles = (p->K + C::TE - 1) / C::TE;
  int grid = sm_count * (bps > 0 ? bps : 1);
  if (grid > ntiles) grid = ntiles;
  dg_rhs_tc_kernel<N, P><<<grid, C::kThreads, C::kSmem, s>>>(*p);
  return cudaGetLastError();
}

template <int N, int P>
cudaError_t rhs_tct(const RhsParams* p, int sm_count, cudaStream_t s, LaunchInfo* info) {
  using C = TctConfig<N, P>;
  static std::once_flag once;
  static cudaError_t st = cudaSuccess;
  static int bps = 0;
  std::call_once(once, [] {
    const void* fn = (const void*)dg_rhs_tct_kernel<N, P>;
    st = cudaFuncSetAttribute(dg_rhs_tct_kernel<N, P>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::kSmemLaunch);
    if (st == cudaSuccess)
      st = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, dg_rhs_tct_kernel<N, P>, C::kThreads, C::kSmemLaunch);
    // The occupancy query reports one CTA per SM for kernels that allocate
    // tensor memory; the resident count is the smallest of the register,
    // shared-memory, thread and TMEM-column limits (CTAs of this kernel never
    // wait on each other, so an estimate above the true count only queues
    // CTAs).
    cudaFuncAttributes fa{};
    int dev = 0, smem_sm = 0, resv = 0, regs_sm = 0, thr_sm = 0;
    if (st == cudaSuccess) st = cudaFuncGetAttributes(&fa, fn);
    if (st == cudaSuccess) st = cudaGetDevice(&dev);
    if (st == cudaSuccess) st = cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    if (st == cudaSuccess) st = cudaDeviceGetAttribute(&resv, cudaDevAttrReservedSharedMemoryPerBlock, dev);
    if (st == cudaSuccess) st = cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev);
    if (st == cudaSuccess) st = cudaDeviceGetAttribute(&thr_sm, cudaDevAttrMaxThreadsPerMultiProcessor, dev);
    if (st == cudaSuccess) {
      const int regs_warp = (fa.numRegs * 32 + 255) / 256 * 256;
      int n = regs_sm / (regs_warp * (C::kThreads / 32));
      n = std::min(n, smem_sm / ((int)C::kSmemLaunch + (int)fa.sharedSizeBytes + resv));
      n = std::min(n, thr_sm / C::kThreads);
      n = std::min(n, 512 / (int)C::kTmemCols);
      bps = std::max(bps, n);
    }
  });
  if (st != cudaSuccess) return st;
  if (info) {
    info->threads = C::kThreads;
    info->tile = C::TE;
    info->smem = C::kSmemLaunch;
    info->blocks_per_sm = bps;
    return cudaSuccess;
  }
  if (!p->mats_tc) return cudaErrorInvalidValue;
  const int ntiles = (p->K + C::TE - 1) / C::TE;
  int grid = sm_count * (bps > 0 ? bps : 1);
  if (grid > ntiles) grid = ntiles;
  dg_rhs_tct_kernel<N, P><<<grid, C::kThreads, C::kSmemLaunch, s>>>(*p);
  return cudaGetLastError();
}

// warp-specialized pipelined tensor-memory kernel: one 512-thread CTA per SM
// (it owns all 512 TMEM columns); advection runs the tct kernel instead
template <int N, int P>
cudaError_t rhs_tcp(const RhsParams* p, int sm_count, cudaStream_t s, LaunchInfo* info) {
  if constexpr (P == PHYS_ADV) {
    return rhs_tct<N, P>(p, sm_count, s, info);
  } else {
    using C = TcpConfig<N, P>;
    static std::once_flag once;
    static cudaError_t st = cudaSuccess;
    std::call_once(once, [] {
      st = cudaFuncSetAttribute(dg_rhs_tcp_kernel<N, P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                C::kSmemLaunch);
    });
    if (st != cudaSuccess) return st;
    if (info) {
      info->threads = C::kThreads;
      info->tile = C::TE;
      info->smem = C::kSmemLaunch;
      info->blocks_per_sm = 1;
      return cudaSuccess;
    }
    if (!p->mats_tc) return cudaErrorInvalidValue;
    const int ntiles = (p->K + C::TE - 1) / C::TE;
    const int grid = std::min(ntiles, sm_count);
    return launch_stage(dg_rhs_tcp_kernel<N, P>, grid, C::kThreads, C::kSmemLaunch, s, *p);
  }
}

template <int N, int P, int EPT, int MAP>
cudaError_t rhs_blk(const RhsParams* p, int sm_count, cudaStream_t s, LaunchInfo* info) {
  using C = BlkConfig<N, P, EPT, MAP>;
  static std::once_flag once;
  static cudaError_t st = cudaSuccess;
  static int bps = 0;
  std::call_once(once, [] {
    st = cudaFuncSetAttribute(dg_rhs_blk_kernel<N, P, EPT, MAP>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::kSmem);
    if (st == cudaSuccess)
      st = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, dg_rhs_blk_kernel<N, P, EPT, MAP>, C::kThreads,
                                                         C::kSmem);
  });
  if (st != cudaSuccess) return st;
  if (info) {
    info->threads = C::kThreads;
    info->tile = C::TE;
    info->smem = C::kSmem;
    info->blocks_per_sm = bps;
    return cudaSuccess;
  }
  if (!p->mats_blk) return cudaErrorInvalidValue;
  const int ntiles = (p->K + C::TE - 1) / C::TE;
  int grid = sm_count * (bps > 0 ? bps : 1);
  if (grid > ntiles) grid = ntiles;
  return launch_stage(dg_rhs_blk_kernel<N, P, EPT, MAP>, grid, C::kThreads, C::kSmem, s, *p);
}

// FP32 variants at orders 1..6: 0 = one thread per element-node (dg_rhs_kernel),
// 1..3 = register-blocked-by-node tile shapes (dg_rhs_v2_kernel), 4 = tensor
// cores (dg_rhs_tc_kernel), 5, 6 = 4-node x 1 or 2 element blocks
// (dg_rhs_blk_kernel, mapping 0), 7 = 4-node x 1 element blocks with
// warp-uniform operator loads (mapping 1), 8 = tensor cores with the A operand
// in TMEM (dg_rhs_tct_kernel), 9 = its warp-specialized pipelined form
// (dg_rhs_tcp_kernel, Maxwell; advection runs variant 8).  Orders 7, 8: 0 =
// dg_rhs_kernel, 1, 2, 3 = dg_rhs_blk_kernel (EPT 1, EPT 2, mapping 1).
constexpr int kF32Variants = 10;
constexpr int kF32VariantsHigh = 4;

template <int N, int P>
cudaError_t rhs_f32_variant(int v, const RhsParams* p, int sm, cudaStream_t s, LaunchInfo* info) {
  if (v == 0) return info ? rhs_configure<float, N, P>(info) : rhs_launch<float, N, P>(*p, sm, s);
  if constexpr (N <= 6) {
    if (v >= 1 && v <= 3) return rhs_v2<N, P>(v - 1, p, sm, s, info);
    if (v == 4) return rhs_tc<N, P>(p, sm, s, info);
    if (v == 5) return rhs_blk<N, P, 1, 0>(p, sm, s, info);
    if (v == 6) return rhs_blk<N, P, 2, 0>(p, sm, s, info);
    if (v == 7) return rhs_blk<N, P, 1, 1>(p, sm, s, info);
    if (v == 8) return rhs_tct<N, P>(p, sm, s, info);
    if (v == 9) return rhs_tcp<N, P>(p, sm, s, info);
  } else {
    if (v == 1) return rhs_blk<N, P, 1, 0>(p, sm, s, info);
    if (v == 2) return rhs_blk<N, P, 2, 0>(p, sm, s, info);
    if (v == 3) return rhs_blk<N, P, 1, 1>(p, sm, s, info);
  }
  return cudaErrorInvalidValue;
}

// per-order entry points, defined in rhs_f32_n<N>.cu
template <int N>
cudaError_t rhs_v2_order(int P, int v, const RhsParams* p, int sm, cudaStream_t s, LaunchInfo* info);

}  // namespace dgk
