// rhs_f32_n6.cu -- FP32 RHS kernels (all variants) of order 6 (all physics and
// tile-shape variants); one translation unit per order so they compile in parallel.
#include "rhs_launch.cuh"

namespace dgk {

template <>
cudaError_t rhs_v2_order<6>(int P, int v, const RhsParams* p, int sm, cudaStream_t s, LaunchInfo* info) {
  switch (P) {
    case PHYS_ADV: return rhs_f32_variant<6, PHYS_ADV>(v, p, sm, s, info);
    case PHYS_TM: return rhs_f32_variant<6, PHYS_TM>(v, p, sm, s, info);
    case PHYS_TE: return rhs_f32_variant<6, PHYS_TE>(v, p, sm, s, info);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace dgk
