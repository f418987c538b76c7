// adv1d.cu -- the 1D advection example on the GPU (C ABI: dgc_adv1d_*):
// u_t + c u_x = 0 on [0, 2 pi], c = 2 pi, K cells of N+1 Gauss-Lobatto nodes,
// strong-form derivative D = Dr 2/h and lift L = V V^T 2/h, upwind flux,
// inflow u(0, t) = -sin(2 pi t), outflow extrapolation
// (examples/advection_1d/advection_1d.h:91-196; its device counterpart
// examples/advection_1d/d_advection_1d.cuh runs one thread per cell).
//
// State layout: [cell][node], the reference's CPU layout.  Kernel: a CTA of
// 256 threads holds 256 / (N+1) cells and the two neighbouring traces in
// shared memory with the operators; one thread per node computes the RHS and,
// in RK4 mode, the classical RK4 stage update (same four-launch scheme as
// dgc_rk4_step).
#include <cuda_runtime.h>

#include <cmath>
#include <string>
#include <vector>

#include "dgc_gb300.h"
#include "dgc_internal.hpp"

struct dgc_adv1d_s {
  int K = 0, N = 0, np = 0, prec = DGC_F64;
  double h = 0.0, c = 0.0;
  std::vector<double> D, L, xr;  // host copies (np x np row-major), reference nodes
  void* d_ops = nullptr;         // [D | L] in the handle's precision
  int64_t launches = 0;
};

namespace dgk {

enum { A1_RHS = 0, A1_RK4 = 1 };

template <typename R, int NP>
__global__ void __launch_bounds__(256) k_adv1d(int K, const R* __restrict__ ops, R c, R inflow, int mode,
                                               int stage, R co, R wa, const R* __restrict__ q_in,
                                               R* __restrict__ out, R* __restrict__ acc, R* __restrict__ q0) {
  constexpr int CPB = 256 / NP;
  __shared__ R sD[NP * NP], sL[NP * NP];
  __shared__ R sU[CPB * NP + 2];
  const int t = threadIdx.x;
  const int k0 = blockIdx.x * CPB;
  const int nc = min(CPB, K - k0);
  for (int q = t; q < NP * NP; q += 256) {
    sD[q] = ops[q];
    sL[q] = ops[NP * NP + q];
  }
  for (int q = t; q < nc * NP; q += 256) sU[1 + q] = q_in[(size_t)k0 * NP + q];
  if (t == 0) sU[0] = k0 > 0 ? q_in[(size_t)k0 * NP - 1] : inflow;  // left trace "a" of the first flux
  if (t == 1) {                                                        // right trace "b" of the last flux
    const size_t e = (size_t)(k0 + nc) * NP;
    sU[1 + nc * NP] = k0 + nc < K ? q_in[e] : q_in[e - 1];
  }
  __syncthreads();
  const int e = t / NP, i = t % NP;
  if (e >= nc) return;
  const R* u = sU + 1 + e * NP;
  R d = R(0);
#pragma unroll
  for (int j = 0; j < NP; ++j) d += sD[i * NP + j] * u[j];
  const R half = R(0.5);
  auto flux = [&](R a, R b) { return c * half * (a + b) + c * half * (a - b); };  // upwind (alpha = 0)
  const R f0 = flux(u[-1], u[0]), f1 = flux(u[NP - 1], u[NP]);
  const R r = -c * d + sL[i * NP] * (f0 - c * u[0]) + sL[i * NP + NP - 1] * (c * u[NP - 1] - f1);
  const size_t o = (size_t)(k0 + e) * NP + i;
  if (mode == A1_RHS) {
    out[o] = r;
  } else if (stage == 0) {
    acc[o] = r;
    out[o] = u[i] + co * r;
  } else if (stage < 3) {
    acc[o] = acc[o] + wa * r;
    out[o] = q0[o] + co * r;
  } else {
    q0[o] = q0[o] + co * (acc[o] + r);
  }
}

template <typename R>
cudaError_t launch_adv1d(int np, int K, const R* ops, R c, R inflow, int mode, int stage, R co, R wa, const R* q_in,
                         R* out, R* acc, R* q0, cudaStream_t s) {
  auto go = [&](auto kern, int NP) {
    const int cpb = 256 / NP;
    kern<<<(K + cpb - 1) / cpb, 256, 0, s>>>(K, ops, c, inflow, mode, stage, co, wa, q_in, out, acc, q0);
    return cudaGetLastError();
  };
  switch (np) {
    case 2: return go(k_adv1d<R, 2>, 2);
    case 3: return go(k_adv1d<R, 3>, 3);
    case 4: return go(k_adv1d<R, 4>, 4);
    case 5: return go(k_adv1d<R, 5>, 5);
    case 6: return go(k_adv1d<R, 6>, 6);
    case 7: return go(k_adv1d<R, 7>, 7);
    case 8: return go(k_adv1d<R, 8>, 8);
    case 9: return go(k_adv1d<R, 9>, 9);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace dgk

using namespace dgc;

namespace {

int a1err(int code, const std::string& msg) { return set_error(code, msg.c_str()); }

template <typename R>
int run(dgc_adv1d a, int mode, int stage, double t, double co, double wa, const void* q_in, void* out, void* acc,
        void* q0, cudaStream_t s) {
  const R inflow = (R)(-std::sin(2.0 * M_PI * t));  // advection_1d.h:163
  cudaError_t e = dgk::launch_adv1d<R>(a->np, a->K, static_cast<const R*>(a->d_ops), (R)a->c, inflow, mode, stage,
                                       (R)co, (R)wa, static_cast<const R*>(q_in), static_cast<R*>(out),
                                       static_cast<R*>(acc), static_cast<R*>(q0), s);
  if (e != cudaSuccess) return a1err(DGC_ERR_CUDA, cudaGetErrorString(e));
  ++a->launches;
  return DGC_OK;
}

int dispatch(dgc_adv1d a, int mode, int stage, double t, double co, double wa, const void* q_in, void* out,
             void* acc, void* q0, cudaStream_t s) {
  return a->prec == DGC_F64 ? run<double>(a, mode, stage, t, co, wa, q_in, out, acc, q0, s)
                            : run<float>(a, mode, stage, t, co, wa, q_in, out, acc, q0, s);
}

}  // namespace

extern "C" int dgc_adv1d_create(int num_cells, int order, int precision, dgc_adv1d* out) {
  if (!out) return a1err(DGC_ERR_ARG, "null argument");
  *out = nullptr;
  if (num_cells < 1 || order < 1 || order > 8) return a1err(DGC_ERR_ARG, "num_cells >= 1 and order in [1, 8]");
  if (precision != DGC_F64 && precision != DGC_F32) return a1err(DGC_ERR_ARG, "unknown precision");
  auto* a = new dgc_adv1d_s();
  a->K = num_cells;
  a->N = order;
  a->np = order + 1;
  a->prec = precision;
  a->c = 2.0 * M_PI;          // advection_1d.h:84-85
  a->h = 2.0 * M_PI / num_cells;
  const int np = a->np;
  // advection_1d.h:91-104: V(i,j) = P_j(r_i), Dr = Vr V^-1, D = Dr 2/h, L = V V^T 2/h
  a->xr = gauss_lobatto(np);
  std::vector<double> V((size_t)np * np), Vr((size_t)np * np), Vi;
  for (int i = 0; i < np; ++i)
    for (int j = 0; j < np; ++j) {
      V[(size_t)i * np + j] = jacobi(0.0, 0.0, j, a->xr[i]);
      Vr[(size_t)i * np + j] = jacobi_grad(0.0, 0.0, j, a->xr[i]);
    }
  if (!invert(V, np, Vi)) {
    delete a;
    return a1err(DGC_ERR_ARG, "singular Vandermonde matrix");
  }
  const std::vector<double> Dr = matmul(Vr, Vi, np, np, np);
  const std::vector<double> Mi = matmul(V, transpose(V, np, np), np, np, np);
  a->D.resize((size_t)np * np);
  a->L.resize((size_t)np * np);
  for (int q = 0; q < np * np; ++q) {
    a->D[q] = Dr[q] * (2.0 / a->h);
    a->L[q] = Mi[q] * (2.0 / a->h);
  }
  const size_t sz = precision == DGC_F64 ? 8 : 4;
  std::vector<unsigned char> ops(2 * (size_t)np * np * sz);
  for (int q = 0; q < np * np; ++q) {
    if (precision == DGC_F64) {
      reinterpret_cast<double*>(ops.data())[q] = a->D[q];
      reinterpret_cast<double*>(ops.data())[np * np + q] = a->L[q];
    } else {
      reinterpret_cast<float*>(ops.data())[q] = (float)a->D[q];
      reinterpret_cast<float*>(ops.data())[np * np + q] = (float)a->L[q];
    }
  }
  cudaError_t e = cudaMalloc(&a->d_ops, ops.size());
  if (e == cudaSuccess) e = cudaMemcpy(a->d_ops, ops.data(), ops.size(), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(a->d_ops);
    delete a;
    return a1err(DGC_ERR_CUDA, cudaGetErrorString(e));
  }
  *out = a;
  return DGC_OK;
}

extern "C" int dgc_adv1d_destroy(dgc_adv1d a) {
  if (!a) return DGC_OK;
  cudaFree(a->d_ops);
  delete a;
  return DGC_OK;
}

extern "C" int dgc_adv1d_info(dgc_adv1d a, double* min_elem_size, double* wave_speed) {
  if (!a) return a1err(DGC_ERR_ARG, "null handle");
  if (min_elem_size) *min_elem_size = a->h;
  if (wave_speed) *wave_speed = a->c;
  return DGC_OK;
}

extern "C" int dgc_adv1d_node_x(dgc_adv1d a, double* x) {
  if (!a || !x) return a1err(DGC_ERR_ARG, "null argument");
  for (int i = 0; i < a->K; ++i)  // advection_1d.h:107-125
    for (int j = 0; j < a->np; ++j) x[(size_t)i * a->np + j] = i * a->h + (1.0 + a->xr[j]) * 0.5 * a->h;
  return DGC_OK;
}

extern "C" int dgc_adv1d_get_operator(dgc_adv1d a, int which, double* out) {
  if (!a || !out || (which != 0 && which != 1)) return a1err(DGC_ERR_ARG, "bad argument");
  const std::vector<double>& m = which == 0 ? a->D : a->L;
  std::copy(m.begin(), m.end(), out);
  return DGC_OK;
}

extern "C" int dgc_adv1d_rhs(dgc_adv1d a, const void* q, double t, void* out, void* stream) {
  if (!a || !q || !out || q == out) return a1err(DGC_ERR_ARG, "null or aliased buffers");
  return dispatch(a, dgk::A1_RHS, 0, t, 0.0, 0.0, q, out, nullptr, nullptr, static_cast<cudaStream_t>(stream));
}

extern "C" int dgc_adv1d_rk4_step(dgc_adv1d a, void* q, double t, double dt, void* const* work, void* stream) {
  if (!a || !q || !work || !work[0] || !work[1] || !work[2]) return a1err(DGC_ERR_ARG, "null argument");
  void* ya = work[0];
  void* yb = work[1];
  void* acc = work[2];
  if (q == ya || q == yb || q == acc || ya == yb || ya == acc || yb == acc)
    return a1err(DGC_ERR_ARG, "q and the three work buffers must be distinct");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const void* in[4] = {q, ya, yb, ya};
  void* outb[4] = {ya, yb, ya, nullptr};
  const double co[4] = {0.5 * dt, 0.5 * dt, dt, dt / 6.0};
  const double wa[4] = {1.0, 2.0, 2.0, 0.0};
  const double ts[4] = {t, t + 0.5 * dt, t + 0.5 * dt, t + dt};
  for (int st = 0; st < 4; ++st)
    if (int rc = dispatch(a, dgk::A1_RK4, st, ts[st], co[st], wa[st], in[st], outb[st], acc, q, s)) return rc;
  return DGC_OK;
}

extern "C" int64_t dgc_adv1d_launch_count(dgc_adv1d a) { return a ? a->launches : -1; }
