// rhs_x2.cu -- launches of the compensated-state stage kernel
// (dg_rhs_x2_kernel, DGC_F32C handles), orders 1..8, all physics.
#include "rhs_launch.cuh"

namespace dgk {

template <int N, int P>
static cudaError_t rhs_x2(const RhsParams* p, int sm_count, cudaStream_t s, LaunchInfo* info) {
  using C = X2Config<N, P>;
  static std::once_flag once;
  static cudaError_t st = cudaSuccess;
  static int bps = 0;
  std::call_once(once, [] {
    st = cudaFuncSetAttribute(dg_rhs_x2_kernel<N, P>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::kSmem);
    if (st == cudaSuccess)
      st = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, dg_rhs_x2_kernel<N, P>, C::kThreads, C::kSmem);
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
  return launch_stage(dg_rhs_x2_kernel<N, P>, grid, C::kThreads, C::kSmem, s, *p);
}

template <int N>
static cudaError_t x2_by_phys(int P, const RhsParams* p, int sm, cudaStream_t s, LaunchInfo* info) {
  switch (P) {
    case PHYS_ADV: return rhs_x2<N, PHYS_ADV>(p, sm, s, info);
    case PHYS_TM: return rhs_x2<N, PHYS_TM>(p, sm, s, info);
    case PHYS_TE: return rhs_x2<N, PHYS_TE>(p, sm, s, info);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t rhs_x2_dispatch(int N, int P, const RhsParams& p_in, int sm, cudaStream_t s, LaunchInfo* info) {
  const RhsParams p = with_f32_scalars(p_in);
  const RhsParams* pp = info ? nullptr : &p;
  switch (N) {
    case 1: return x2_by_phys<1>(P, pp, sm, s, info);
    case 2: return x2_by_phys<2>(P, pp, sm, s, info);
    case 3: return x2_by_phys<3>(P, pp, sm, s, info);
    case 4: return x2_by_phys<4>(P, pp, sm, s, info);
    case 5: return x2_by_phys<5>(P, pp, sm, s, info);
    case 6: return x2_by_phys<6>(P, pp, sm, s, info);
    case 7: return x2_by_phys<7>(P, pp, sm, s, info);
    case 8: return x2_by_phys<8>(P, pp, sm, s, info);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace dgk
