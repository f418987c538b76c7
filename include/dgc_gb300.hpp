// dgc_gb300.hpp -- header-only C++ adapter that keeps the reference's call
// shapes on top of the C ABI (dgc_gb300.h), so host code written against
// hsongxa/dg-on-cuda keeps working:
//
//   dgc::device_SemiDiscOp_wrapper<Op>   src/device_SemiDiscOp_wrapper.cuh:45-58
//       op(in, size, t, out)  ->  dgc_rhs
//   dgc::kernel_adapter<F>               src/kernel_adapter.cuh:59-83
//       execute_phase(phase_one{}, inout, size) / (phase_two{}, ...)  ->  laplace_2d passes
//   dgc::k_axpy_auto / dgc::axpy_n       src/k_axpy.cuh:47-55, src/axpy.h:112-122
//   dgc::rk4                             src/explicit_runge_kutta.h:33-51
//       (the same template: 4 operator calls + 8 axpy calls), plus the fused
//       dgc::rk4_fused / dgc::lserk4 that run one launch per stage.
//
// Errors become std::runtime_error, as the reference's wrappers throw on
// cudaGetLastError (device_SemiDiscOp_wrapper.cuh:56, kernel_adapter.cuh:74,81).
// Host-only C++17; link against libdgc_gb300.so.
#pragma once

#include <cstddef>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "dgc_gb300.h"

namespace dgc {

inline void check(int rc, const char* what) {
  if (rc != DGC_OK) throw std::runtime_error(std::string(what) + ": " + dgc_last_error());
}

// Owning handle (replaces the create_/destroy_device_object pairs of the
// examples, e.g. examples/advection_2d/k_advection_2d.cu:45-126).
class discretization {
 public:
  discretization(const std::vector<double>& vertex_xy, const std::vector<int32_t>& cells,
                 const dgc_problem_desc& desc) {
    dgc_handle h = nullptr;
    check(dgc_create((int)(vertex_xy.size() / 2), vertex_xy.data(), (int)(cells.size() / 3), cells.data(), &desc, &h),
          "dgc_create");
    h_.reset(h);
    check(dgc_get_info(h, &info_), "dgc_get_info");
  }
  dgc_handle get() const { return h_.get(); }
  const dgc_info& info() const { return info_; }
  std::size_t state_len() const { return (std::size_t)info_.state_len; }

 private:
  struct deleter {
    void operator()(dgc_handle h) const { dgc_destroy(h); }
  };
  std::unique_ptr<dgc_handle_s, deleter> h_;
  dgc_info info_{};
};

// The semi-discrete operator as a callable: op(in, size, t, out).
template <typename DeviceSemiDiscOp = discretization>
struct device_SemiDiscOp_wrapper {
  const discretization* m_Dop = nullptr;
  void* m_Stream = nullptr;  // cudaStream_t

  template <typename T, typename ConstItr, typename Itr>
  void operator()(ConstItr in, std::size_t size, T t, Itr out) const {
    if (size != m_Dop->state_len()) throw std::runtime_error("state size does not match the discretisation");
    check(dgc_rhs(m_Dop->get(), in, (double)t, out, m_Stream), "failed to launch kernel/device code!");
  }
};

// Phases of the two-pass laplace_2d device operator
// (examples/poisson_2d/d_poisson_2d.cuh:38-39).
struct phase_one {};
struct phase_two {};

// kernel_adapter over a DGC_LAPLACE handle: execute_phase(phase_one{}, ...)
// followed by execute_phase(phase_two{}, ...) replaces inout by laplace(inout).
// Both phases run inside phase_two (the grad/div passes are fused in the
// library); phase_one only records the input.
template <typename DeviceFunctor = discretization>
struct kernel_adapter {
  const discretization* Dobj;
  int GridSize, BlockSize;  // kept for source compatibility; the library sizes its own grids
  std::size_t NumExecs;
  void* Stream = nullptr;
  void* Scratch = nullptr;  // one state vector of device scratch, supplied by the caller

  kernel_adapter(const discretization* obj, int grid_size, int block_size, std::size_t num_execs)
      : Dobj(obj), GridSize(grid_size), BlockSize(block_size), NumExecs(num_execs) {}

  template <typename T>
  void execute_phase(phase_one, T* inout, std::size_t size) {
    (void)inout;
    if (size != Dobj->state_len()) throw std::runtime_error("state size does not match the discretisation");
  }
  template <typename T>
  void execute_phase(phase_two, T* inout, std::size_t size) {
    if (!Scratch) throw std::runtime_error("kernel_adapter: set Scratch to one device state vector");
    if (size != Dobj->state_len()) throw std::runtime_error("state size does not match the discretisation");
    check(dgc_laplace_apply(Dobj->get(), inout, Scratch, Stream), "failed to launch kernel of device function phase!");
    check(dgc_axpy(Dobj->get(), 0.0, inout, Scratch, inout, Stream), "failed to launch kernel of device function phase!");
  }
};

// out = a x + y on device state vectors of a handle (k_axpy_auto's signature
// plus the handle).
struct device_axpy {
  const discretization* d;
  void* stream = nullptr;
  template <typename T>
  void operator()(T a, const T* x, std::size_t n, const T* y, T* out) const {
    if (n != d->state_len()) throw std::runtime_error("axpy size does not match the discretisation");
    check(dgc_axpy(d->get(), (double)a, x, y, out, stream), "axpy");
  }
};

// The reference's classical RK4, unchanged in form (explicit_runge_kutta.h:33-51).
template <typename Itr, typename T, typename DiscreteOp, typename Axpy>
void rk4(Itr inout, std::size_t size, T t, T dt, const DiscreteOp& op, const Axpy& axpy, Itr wk0, Itr wk1, Itr wk2,
         Itr wk3, Itr wk4) {
  op(inout, size, t, wk1);
  axpy((T)(0.5L) * dt, wk1, size, inout, wk0);
  op(wk0, size, t + (T)(0.5L) * dt, wk2);
  axpy((T)(0.5L) * dt, wk2, size, inout, wk0);
  op(wk0, size, t + (T)(0.5L) * dt, wk3);
  axpy(dt, wk3, size, inout, wk0);
  op(wk0, size, t + dt, wk4);
  axpy((T)(2.0L), wk2, size, wk1, wk0);
  axpy((T)(2.0L), wk3, size, wk4, wk1);
  axpy(dt / (T)(6.0L), wk0, size, inout, wk2);
  axpy(dt / (T)(6.0L), wk1, size, wk2, inout);
}

// Fused classical RK4: the same step in 4 launches (work: 3 state vectors).
template <typename T>
void rk4_fused(const discretization& d, T* q, double t, double dt, T* w0, T* w1, T* w2, void* stream = nullptr) {
  void* work[3] = {w0, w1, w2};
  check(dgc_rk4_step(d.get(), q, t, dt, work, stream), "rk4_fused");
}

// LSERK4 over nsteps; returns the buffer (qa or qb) that holds the result.
template <typename T>
T* lserk4(const discretization& d, T* qa, T* qb, T* res, double t0, double dt, int nsteps, bool graph = true,
          void* stream = nullptr) {
  void* fin = nullptr;
  check(dgc_lserk4_run(d.get(), qa, qb, res, t0, dt, nsteps, graph ? 1 : 0, &fin, stream), "lserk4");
  return static_cast<T*>(fin);
}

}  // namespace dgc
