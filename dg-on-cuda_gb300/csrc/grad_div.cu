// grad_div.cu -- weak-form gradient and divergence with central fluxes on the
// handle's mesh (C ABI: dgc_grad_apply, dgc_div_apply, dgc_boundary_nodes).
//
// grad_2d::operator() (src/grad_2d.h:141-187), per element k, node i:
//   gx = -(Dx u)_i + (1/J) sum_m LIFT_im faceJ_m nx_m (u- + u+)_m / 2
//   gy = -(Dy u)_i + (1/J) sum_m LIFT_im faceJ_m ny_m (u- + u+)_m / 2
// div_2d::operator() (src/div_2d.h:148-190):
//   d  = -(Dx ux + Dy uy)_i + (1/J) sum_m LIFT_im faceJ_m (n.(u- + u+))_m / 2
// with the weak Dr, Ds, LIFT of the advection operator, Dx = rx Dr + sx Ds,
// Dy = ry Dr + sy Ds, and the exterior trace u+ taken from the face neighbour
// (its face nodes in reverse order) or, on the boundary, from the caller's
// boundary data u+ = g + sign u- (the exterior_val callbacks of the
// reference's boundary-condition objects all have this form).
//
// Kernel: one CTA of 256 threads holds E = 256 / NpP elements; their fields are
// staged in shared memory, one thread per face node computes the central flux
// into shared memory, then one thread per (element, node) applies the
// operators (read from L1-resident global memory) and writes the result.
#include <cuda_runtime.h>

#include <algorithm>

#include "common.cuh"
#include "dgc_gb300.h"
#include "dgc_internal.hpp"

namespace dgk {

template <typename R, int N, bool DIV>
__global__ void __launch_bounds__(256) k_grad_div(int K, const R* __restrict__ geom, const int4* __restrict__ nbr,
                                                  const R* __restrict__ mats, const R* __restrict__ u0,
                                                  const R* __restrict__ u1, const double* __restrict__ g0,
                                                  const double* __restrict__ g1, R sign, R* __restrict__ out0,
                                                  R* __restrict__ out1) {
  constexpr int Np = (N + 1) * (N + 2) / 2, Nfp = N + 1, NF = 3 * Nfp, NpP = (Np + 3) / 4 * 4;
  constexpr int E = 256 / NpP;
  constexpr int kD = (Np * Np + 3) / 4 * 4;
  __shared__ R sU[2][E * NpP];
  __shared__ R sF[E * NF];
  const int t = threadIdx.x;
  const int k0 = blockIdx.x * E;
  const int ne = min(E, K - k0);
  for (int q = t; q < ne * NpP; q += 256) {
    sU[0][q] = u0[(size_t)k0 * NpP + q];
    if (DIV) sU[1][q] = u1[(size_t)k0 * NpP + q];
  }
  __syncthreads();
  // central fluxes, pre-multiplied by faceJ (and by nothing else: grad applies n per component)
  for (int q = t; q < ne * NF; q += 256) {
    const int e = q / NF, m = q % NF, f = m / Nfp, d = m % Nfp;
    const int k = k0 + e;
    const R* G = geom + (size_t)k * 16;
    const int nd = fmask<N>(f, d);
    const R a0 = sU[0][e * NpP + nd];
    const R a1 = DIV ? sU[1][e * NpP + nd] : R(0);
    R b0, b1 = R(0);
    const int nb = (&nbr[k].x)[f];
    if (nb >= 0) {
      const int kn = nb >> 2, nd2 = fmask<N>(nb & 3, Nfp - 1 - d);
      b0 = u0[(size_t)kn * NpP + nd2];
      if (DIV) b1 = u1[(size_t)kn * NpP + nd2];
    } else {
      const size_t bi = (size_t)(-1 - nb) * Nfp + d;
      b0 = (g0 ? (R)g0[bi] : R(0)) + sign * a0;
      if (DIV) b1 = (g1 ? (R)g1[bi] : R(0)) + sign * a1;
    }
    const R fJ = G[5 + f];
    sF[q] = DIV ? (R(0.5) * ((a0 + b0) * G[8 + f] + (a1 + b1) * G[11 + f])) * fJ : (R(0.5) * (a0 + b0)) * fJ;
  }
  __syncthreads();
  const int e = t / NpP, i = t % NpP;
  if (e >= ne || i >= Np) return;
  const int k = k0 + e;
  const R* G = geom + (size_t)k * 16;
  const R rx = G[0], ry = G[1], sx = G[2], sy = G[3], invJ = -G[4];
  const R* DrT = mats;
  const R* DsT = mats + kD;
  const R* LT = mats + 2 * kD;
  const R* ua = sU[0] + e * NpP;
  const R* ub = sU[1] + e * NpP;
  R dr0 = R(0), ds0 = R(0), dr1 = R(0), ds1 = R(0);
#pragma unroll 4
  for (int j = 0; j < Np; ++j) {
    const R dr = __ldg(DrT + j * Np + i), ds = __ldg(DsT + j * Np + i);
    dr0 += dr * ua[j];
    ds0 += ds * ua[j];
    if (DIV) {
      dr1 += dr * ub[j];
      ds1 += ds * ub[j];
    }
  }
  const R* F = sF + e * NF;
  if (DIV) {
    R l = R(0);
#pragma unroll 4
    for (int m = 0; m < NF; ++m) l += __ldg(LT + m * Np + i) * F[m];
    out0[(size_t)k * NpP + i] = -(rx * dr0 + sx * ds0) - (ry * dr1 + sy * ds1) + invJ * l;
  } else {
    R lx = R(0), ly = R(0);
#pragma unroll
    for (int f = 0; f < 3; ++f) {
      R lf = R(0);
      for (int d = 0; d < Nfp; ++d) lf += __ldg(LT + (f * Nfp + d) * Np + i) * F[f * Nfp + d];
      lx += lf * G[8 + f];
      ly += lf * G[11 + f];
    }
    out0[(size_t)k * NpP + i] = -(rx * dr0 + sx * ds0) + invJ * lx;
    out1[(size_t)k * NpP + i] = -(ry * dr0 + sy * ds0) + invJ * ly;
  }
}

template <typename R, bool DIV>
cudaError_t launch_grad_div(int N, int K, const R* geom, const int4* nbr, const R* mats, const R* u0, const R* u1,
                            const double* g0, const double* g1, R sign, R* out0, R* out1, cudaStream_t s) {
  auto go = [&](auto kern, int NpP) {
    const int E = 256 / NpP;
    kern<<<(K + E - 1) / E, 256, 0, s>>>(K, geom, nbr, mats, u0, u1, g0, g1, sign, out0, out1);
    return cudaGetLastError();
  };
  switch (N) {
    case 1: return go(k_grad_div<R, 1, DIV>, 4);
    case 2: return go(k_grad_div<R, 2, DIV>, 8);
    case 3: return go(k_grad_div<R, 3, DIV>, 12);
    case 4: return go(k_grad_div<R, 4, DIV>, 16);
    case 5: return go(k_grad_div<R, 5, DIV>, 24);
    case 6: return go(k_grad_div<R, 6, DIV>, 28);
    case 7: return go(k_grad_div<R, 7, DIV>, 36);
    case 8: return go(k_grad_div<R, 8, DIV>, 48);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace dgk

using namespace dgc;

namespace {

int check_scalar_handle(dgc_handle h) {
  if (!h) return set_error(DGC_ERR_ARG, "null handle");
  if (h->Nf != 1) return set_error(DGC_ERR_UNSUPPORTED, "grad / div act on scalar-field (advection, laplace) handles");
  if (h->prec == DGC_F32C) return set_error(DGC_ERR_UNSUPPORTED, "grad / div are not offered for compensated FP32 handles");
  return DGC_OK;
}

template <typename R, bool DIV>
int grad_div(dgc_handle h, const void* u0, const void* u1, const double* g0, const double* g1, double sign,
             void* out0, void* out1, cudaStream_t s) {
  const bool f64 = sizeof(R) == 8;
  const R* geom = static_cast<const R*>(f64 ? (const void*)h->d_kgeom64 : (const void*)h->d_kgeom32);
  const R* mats = static_cast<const R*>(f64 ? (const void*)h->d_mats64[0] : (const void*)h->d_mats32[0]);
  cudaError_t e = dgk::launch_grad_div<R, DIV>(h->N, h->K, geom, reinterpret_cast<const int4*>(h->d_nbr), mats,
                                               static_cast<const R*>(u0), static_cast<const R*>(u1), g0, g1,
                                               (R)sign, static_cast<R*>(out0), static_cast<R*>(out1), s);
  if (e != cudaSuccess) return set_error(DGC_ERR_CUDA, cudaGetErrorString(e));
  ++h->launches;
  return DGC_OK;
}

}  // namespace

extern "C" int dgc_boundary_nodes(dgc_handle h, double* xy) {
  if (!h || !xy) return set_error(DGC_ERR_ARG, "null argument");
  std::copy(h->mesh.bxy.begin(), h->mesh.bxy.end(), xy);
  return DGC_OK;
}

extern "C" int dgc_grad_apply(dgc_handle h, const void* u, void* gx, void* gy, const double* g, double sign,
                              void* stream) {
  if (int rc = check_scalar_handle(h)) return rc;
  if (!u || !gx || !gy || gx == gy || u == gx || u == gy)
    return set_error(DGC_ERR_ARG, "u, gx, gy must be distinct, non-null buffers");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  return h->prec == DGC_F64 ? grad_div<double, false>(h, u, nullptr, g, nullptr, sign, gx, gy, s)
                            : grad_div<float, false>(h, u, nullptr, g, nullptr, sign, gx, gy, s);
}

extern "C" int dgc_div_apply(dgc_handle h, const void* ux, const void* uy, void* out, const double* gx,
                             const double* gy, double sign, void* stream) {
  if (int rc = check_scalar_handle(h)) return rc;
  if (!ux || !uy || !out || out == ux || out == uy)
    return set_error(DGC_ERR_ARG, "ux, uy, out must be non-null and out distinct from the inputs");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  return h->prec == DGC_F64 ? grad_div<double, true>(h, ux, uy, gx, gy, sign, out, nullptr, s)
                            : grad_div<float, true>(h, ux, uy, gx, gy, sign, out, nullptr, s);
}
