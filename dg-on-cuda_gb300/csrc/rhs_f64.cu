// rhs_f64.cu -- double instantiations of the fused RHS kernel (orders 1..8,
// advection / Maxwell TM / Maxwell TE).
#include "rhs_launch.cuh"

namespace dgk {

template <int N>
static cudaError_t by_phys(int P, const RhsParams& p, int sm, cudaStream_t s, LaunchInfo* info) {
  if (info) {
    switch (P) {
      case PHYS_ADV: return rhs_configure<double, N, PHYS_ADV>(info);
      case PHYS_TM: return rhs_configure<double, N, PHYS_TM>(info);
      case PHYS_TE: return rhs_configure<double, N, PHYS_TE>(info);
      default: return cudaErrorInvalidValue;
    }
  }
  switch (P) {
    case PHYS_ADV: return rhs_launch<double, N, PHYS_ADV>(p, sm, s);
    case PHYS_TM: return rhs_launch<double, N, PHYS_TM>(p, sm, s);
    case PHYS_TE: return rhs_launch<double, N, PHYS_TE>(p, sm, s);
    default: return cudaErrorInvalidValue;
  }
}

template <>
cudaError_t rhs_dispatch<double>(int N, int P, int v, const RhsParams& p, int sm, cudaStream_t s, LaunchInfo* info) {
  (void)v;
  switch (N) {
    case 1: return by_phys<1>(P, p, sm, s, info);
    case 2: return by_phys<2>(P, p, sm, s, info);
    case 3: return by_phys<3>(P, p, sm, s, info);
    case 4: return by_phys<4>(P, p, sm, s, info);
    case 5: return by_phys<5>(P, p, sm, s, info);
    case 6: return by_phys<6>(P, p, sm, s, info);
    case 7: return by_phys<7>(P, p, sm, s, info);
    case 8: return by_phys<8>(P, p, sm, s, info);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace dgk
