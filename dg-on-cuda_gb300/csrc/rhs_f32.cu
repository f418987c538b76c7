// rhs_f32.cu -- float instantiations of the fused RHS kernel (orders 1..8,
// advection / Maxwell TM / Maxwell TE).
#include "rhs_launch.cuh"

namespace dgk {

// orders 1..6: variant v of rhs_f32_variant (rhs_launch.cuh), compiled per
// order in rhs_f32_n<N>.cu; orders 7, 8: dg_rhs_kernel (v = 0) and the
// register-blocked dg_rhs_blk_kernel (v = 1, 2), compiled here
template <int N>
static cudaError_t by_phys(int P, int v, const RhsParams& p, int sm, cudaStream_t s, LaunchInfo* info) {
  const RhsParams* pp = info ? nullptr : &p;
  if constexpr (N <= 6) {
    return rhs_v2_order<N>(P, v, pp, sm, s, info);
  } else {
    switch (P) {
      case PHYS_ADV: return rhs_f32_variant<N, PHYS_ADV>(v, pp, sm, s, info);
      case PHYS_TM: return rhs_f32_variant<N, PHYS_TM>(v, pp, sm, s, info);
      case PHYS_TE: return rhs_f32_variant<N, PHYS_TE>(v, pp, sm, s, info);
      default: return cudaErrorInvalidValue;
    }
  }
}

template <>
cudaError_t rhs_dispatch<float>(int N, int P, int v, const RhsParams& p_in, int sm, cudaStream_t s, LaunchInfo* info) {
  const RhsParams p = with_f32_scalars(p_in);
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

int rhs_num_variants(int prec_f32, int N) {
  return prec_f32 ? (N <= 6 ? kF32Variants : kF32VariantsHigh) : 1;
}

}  // namespace dgk
