// rhs_f32.cu -- float instantiations of the fused RHS kernel (orders 1..8,
// advection / Maxwell TM / Maxwell TE).
#include "rhs_launch.cuh"

namespace dgk {

// orders 1..6: variant v of rhs_f32_variant (rhs_launch.cuh); orders 7, 8:
// dg_rhs_kernel
template <int N>
static cudaError_t by_phys(int P, int v, const RhsParams& p, int sm, cudaStream_t s, LaunchInfo* info) {
  if constexpr (N <= 6) {
    return rhs_v2_order<N>(P, v, info ? nullptr : &p, sm, s, info);
  } else {
    if (info) {
      switch (P) {
        case PHYS_ADV: return rhs_configure<float, N, PHYS_ADV>(info);
        case PHYS_TM: return rhs_configure<float, N, PHYS_TM>(info);
        case PHYS_TE: return rhs_configure<float, N, PHYS_TE>(info);
        default: return cudaErrorInvalidValue;
      }
    }
    switch (P) {
      case PHYS_ADV: return rhs_launch<float, N, PHYS_ADV>(p, sm, s);
      case PHYS_TM: return rhs_launch<float, N, PHYS_TM>(p, sm, s);
      case PHYS_TE: return rhs_launch<float, N, PHYS_TE>(p, sm, s);
      default: return cudaErrorInvalidValue;
    }
  }
}

template <>
cudaError_t rhs_dispatch<float>(int N, int P, int v, const RhsParams& p, int sm, cudaStream_t s, LaunchInfo* info) {
  switch (N) {
    case 1: return by_phys<1>(P, v, p, sm, s, info);
    case 2: return by_phys<2>(P, v, p, sm, s, info);
    case 3: return by_phys<3>(P, v, p, sm, s, info);
    case 4: return by_phys<4>(P, v, p, sm, s, info);
    case 5: return by_phys<5>(P, v, p, sm, s, info);
    case 6: return by_phys<6>(P, v, p, sm, s, info);
    case 7: return by_phys<7>(P, v, p, sm, s, info);
    case 8: return by_phys<8>(P, v, p, sm, s, info);
    default: return cudaErrorInvalidValue;
  }
}

int rhs_num_variants(int prec_f32, int N) { return (prec_f32 && N <= 6) ? kF32Variants : 1; }

}  // namespace dgk
