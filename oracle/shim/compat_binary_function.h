// Build shim for compiling the reference's CPU path with CUDA 13: CCCL 3 removed
// thrust::binary_function, which the reference's src/axpy.h derives from.
#pragma once
#include <thrust/functional.h>
namespace thrust {
template <class A1, class A2, class R>
struct binary_function {
  using first_argument_type = A1;
  using second_argument_type = A2;
  using result_type = R;
};
}  // namespace thrust
