// rhs_f32_n5.cu -- FP32 RHS kernels (all variants) of order 5 (all physics and
// tile-shape variants); one translation unit per order so they compile in parallel.
#include "rhs_launch.cuh"

namespace dgk {

template <>
cudaError_t rhs_v2_order<5>(int P, int v, const RhsParams* p, int sm, cudaStream_t s, LaunchInfo* info) {
  switch (P) {
    case PHYS_ADV: return rhs_f32_variant<5, PHYS_ADV>(v, p, sm, s, info);
    case PHYS_TM: return rhs_f32_variant<5, PHYS_TM>(v, p, sm, s, info);
    case PHYS_TE: return rhs_f32_variant<5, PHYS_TE>(v, p, sm, s, info);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace dgk
