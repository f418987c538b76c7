// mpnn.cu -- learned preconditioner for the IPDG laplace solves: a
// message-passing network over element adjacency (C ABI: dgc_mpnn_*,
// dgc_fpcg_solve in include/dgc_gb300.h).  No reference counterpart.
//
// Network (width W = 64, L layers), per element k with input x_k (NpP values):
//   h0_k = Win x_k + bin
//   h_l,k = h_{l-1},k + relu(Ws_l h_{l-1},k + Wn_l m_{l-1},k + b_l),
//           m_{l-1},k = sum of h_{l-1} over the face neighbours of k
//   y_k = Wout h_L,k + bout
// Weights: FP32 masters (Adam), BF16 copies read by every kernel, FP32
// accumulation.  Training samples are whole fields; a batch of S fields is
// S * K graph nodes (neighbours of sample s offset by s K).
//
// Preconditioner of the SPD laplace form: M(r) = Binv r + (|r|/c) y(c r/|r|),
// c = sqrt(K Np) so that the network input has unit RMS per node; used
// by truncated flexible CG (Notay, SIAM J. Sci. Comput. 22 (2000) 1444-1460:
// each direction S-orthogonalised against the previous m) whose convergence
// test is the FP64 residual, so the solution does not depend on the network.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <initializer_list>
#include <random>
#include <string>
#include <vector>

#include "dgc_gb300.h"
#include "dgc_internal.hpp"
#include "mpnn_tc.cuh"

namespace dgk {

constexpr int kW = 64;  // feature width

struct MpnnLayout {
  int npi = 0, L = 0;
  int64_t oWin = 0, obin = 0, oWout = 0, obout = 0, total = 0;
  int64_t oWs(int l) const { return obin + kW + (int64_t)l * (2 * kW * kW + kW); }
  int64_t oWn(int l) const { return oWs(l) + kW * kW; }
  int64_t ob(int l) const { return oWs(l) + 2 * kW * kW; }
  void init(int npi_, int L_) {
    npi = npi_;
    L = L_;
    oWin = 0;
    obin = (int64_t)kW * npi;
    oWout = oWs(L);
    obout = oWout + (int64_t)npi * kW;
    total = obout + npi;
  }
};

__device__ __forceinline__ float bf(const __nv_bfloat16 v) { return __bfloat162float(v); }

// block sum of a double into *out (atomic)
__device__ __forceinline__ void block_add(double v, double* out) {
  __shared__ double red[32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += red[i];
    atomicAdd(out, s);
  }
}


// h0 = Win x + bin; 4 nodes x 64 channels per 256 threads, groups strided over the grid
__global__ void __launch_bounds__(256) k_fwd_in(int64_t n, int npi, const __nv_bfloat16* __restrict__ Win,
                                                const __nv_bfloat16* __restrict__ bin, const float* __restrict__ x,
                                                float* __restrict__ h0) {
  __shared__ float wT[64][kW];  // [input][channel]
  __shared__ float xs[4][64];
  const int t = threadIdx.x, el = t >> 6, c = t & 63;
  for (int i = t; i < kW * npi; i += 256) wT[i % npi][i / npi] = bf(Win[i]);
  const float b = bf(bin[c]);
  for (int64_t g0 = (int64_t)blockIdx.x * 4; g0 < n; g0 += (int64_t)gridDim.x * 4) {
    __syncthreads();
    for (int i = t; i < 4 * npi; i += 256) {
      const int64_t e = g0 + i / npi;
      xs[i / npi][i % npi] = e < n ? x[e * npi + i % npi] : 0.0f;
    }
    __syncthreads();
    const int64_t e = g0 + el;
    if (e < n) {
      float a = b;
      for (int j = 0; j < npi; ++j) a = fmaf(wT[j][c], xs[el][j], a);
      h0[e * kW + c] = a;
    }
  }
}


// y = Wout h + bout; min(256 / npi, 16) nodes x npi outputs per block
__global__ void __launch_bounds__(256) k_fwd_out(int64_t n, int npi, const __nv_bfloat16* __restrict__ Wout,
                                                 const __nv_bfloat16* __restrict__ bout, const float* __restrict__ h,
                                                 float* __restrict__ y) {
  __shared__ float wT[kW][64];  // [channel][output]
  __shared__ float hs[16][kW];
  const int per = min(256 / npi, 16), t = threadIdx.x, el = t / npi, o = t - el * npi;
  for (int i = t; i < npi * kW; i += 256) wT[i % kW][i / kW] = bf(Wout[i]);
  const float b = o < npi ? bf(bout[o]) : 0.0f;
  for (int64_t g0 = (int64_t)blockIdx.x * per; g0 < n; g0 += (int64_t)gridDim.x * per) {
    __syncthreads();
    for (int i = t; i < per * kW; i += 256) {
      const int64_t e = g0 + i / kW;
      hs[i / kW][i % kW] = e < n ? h[e * kW + i % kW] : 0.0f;
    }
    __syncthreads();
    const int64_t e = g0 + el;
    if (el < per && e < n) {
      float a = b;
#pragma unroll 8
      for (int c = 0; c < kW; ++c) a = fmaf(wT[c][o], hs[el][c], a);
      y[e * npi + o] = a;
    }
  }
}

// per-sample 1 / sum of squared targets over valid nodes
__global__ void k_target_norm(int K, int npi, int np, const float* __restrict__ t, double* __restrict__ acc) {
  const int s = blockIdx.y;
  double v = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (int64_t)K * npi;
       i += (int64_t)gridDim.x * blockDim.x)
    if ((int)(i % npi) < np) {
      const double x = t[(int64_t)s * K * npi + i];
      v += x * x;
    }
  block_add(v, acc + s);
}

// dy = d loss / dy, loss += sum (y - t)^2 / |t_s|^2 / S
__global__ void k_loss(int64_t n, int K, int npi, int np, int S, const float* __restrict__ y,
                       const float* __restrict__ t, const double* __restrict__ tn, float* __restrict__ dy,
                       double* __restrict__ loss) {
  double v = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n * npi; i += (int64_t)gridDim.x * blockDim.x) {
    const int o = (int)(i % npi);
    const int s = (int)(i / ((int64_t)K * npi));
    const double w = tn[s] > 0.0 ? 1.0 / (tn[s] * S) : 0.0;
    const float d = o < np ? y[i] - t[i] : 0.0f;
    dy[i] = (float)(2.0 * d * w);
    v += (double)d * d * w;
  }
  block_add(v, loss);
}

// d = y - t and tm = t on valid nodes, 0 on padding nodes
__global__ void k_mask_diff(int64_t n, int npi, int np, const float* __restrict__ y, const float* __restrict__ t,
                            float* __restrict__ d, float* __restrict__ tm) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const bool ok = (int)(i % npi) < np;
    d[i] = ok ? y[i] - t[i] : 0.0f;
    tm[i] = ok ? t[i] : 0.0f;
  }
}

// per sample s = blockIdx.y: out[2s] += d.Sd, out[2s+1] += t.St (valid nodes)
__global__ void k_energy_dots(int K, int npi, int np, const float* __restrict__ d, const float* __restrict__ Sd,
                              const float* __restrict__ t, const float* __restrict__ St, double* __restrict__ out) {
  const int s = blockIdx.y;
  double a = 0.0, b = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (int64_t)K * npi;
       i += (int64_t)gridDim.x * blockDim.x)
    if ((int)(i % npi) < np) {
      const int64_t g = (int64_t)s * K * npi + i;
      a += (double)d[g] * Sd[g];
      b += (double)t[g] * St[g];
    }
  block_add(a, out + 2 * s);
  block_add(b, out + 2 * s + 1);
}

// energy loss: dy = 2 S d / (t.St S) on valid nodes; *loss = sum_s d.Sd / t.St / S
__global__ void k_energy_grad(int64_t n, int K, int npi, int np, int S, const float* __restrict__ Sd,
                              const double* __restrict__ dots, float* __restrict__ dy, double* __restrict__ loss) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int s = (int)(i / ((int64_t)K * npi));
    const double tst = dots[2 * s + 1];
    const double w = tst > 0.0 ? 2.0 / (tst * S) : 0.0;
    dy[i] = (int)(i % npi) < np ? (float)(w * Sd[i]) : 0.0f;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    double l = 0.0;
    for (int s = 0; s < S; ++s)
      if (dots[2 * s + 1] > 0.0) l += dots[2 * s] / dots[2 * s + 1];
    *loss = l / S;
  }
}

// dh = Wout^T dy
__global__ void __launch_bounds__(256) k_bwd_out(int64_t n, int npi, const __nv_bfloat16* __restrict__ Wout,
                                                 const float* __restrict__ dy, float* __restrict__ dh) {
  __shared__ float w[64][kW];  // [output][channel]
  __shared__ float ds[4][64];
  const int t = threadIdx.x, el = t >> 6, c = t & 63;
  for (int i = t; i < npi * kW; i += 256) w[i / kW][i % kW] = bf(Wout[i]);
  for (int64_t g0 = (int64_t)blockIdx.x * 4; g0 < n; g0 += (int64_t)gridDim.x * 4) {
    __syncthreads();
    for (int i = t; i < 4 * npi; i += 256) {
      const int64_t e = g0 + i / npi;
      ds[i / npi][i % npi] = e < n ? dy[e * npi + i % npi] : 0.0f;
    }
    __syncthreads();
    const int64_t e = g0 + el;
    if (e < n) {
      float a = 0.0f;
      for (int o = 0; o < npi; ++o) a = fmaf(w[o][c], ds[el][o], a);
      dh[e * kW + c] = a;
    }
  }
}

// m = sum of h over the face neighbours
__global__ void k_gather(int64_t n, int K, const int4* __restrict__ nbr, const float* __restrict__ h,
                         float* __restrict__ m) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n * kW; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = i / kW;
    const int c = (int)(i % kW);
    int64_t j[3];
    neighbours(nbr, K, e, j);
    float v = 0.0f;
#pragma unroll
    for (int f = 0; f < 3; ++f)
      if (j[f] >= 0) v += h[j[f] * kW + c];
    m[i] = v;
  }
}

// g = dh * (a > 0), or g = dh for the linear network
__global__ void k_relu_bwd(int64_t n, const float* __restrict__ dh, const float* __restrict__ a,
                           float* __restrict__ g, int linear) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    g[i] = (linear || a[i] > 0.0f) ? dh[i] : 0.0f;
}

// gW[o][i] += sum_e gout[e][o] xin[e][i], gb[o] += sum_e gout[e][o]; nout, nin <= 64.
// A block accumulates 32-node chunks (grid-strided) in registers, then adds atomically.
__global__ void __launch_bounds__(256) k_grad_dense(int64_t n, int nout, int nin, const float* __restrict__ gout,
                                                    const float* __restrict__ xin, float* __restrict__ gW,
                                                    float* __restrict__ gb) {
  __shared__ float go[32][64], xi[32][64];
  const int t = threadIdx.x;
  const int pairs = nout * nin;
  float acc[16];
#pragma unroll
  for (int q = 0; q < 16; ++q) acc[q] = 0.0f;
  float accb = 0.0f;
  for (int64_t g0 = (int64_t)blockIdx.x * 32; g0 < n; g0 += (int64_t)gridDim.x * 32) {
    __syncthreads();
    for (int i = t; i < 32 * 64; i += 256) {
      const int r = i >> 6, c = i & 63;
      const int64_t e = g0 + r;
      go[r][c] = (e < n && c < nout) ? gout[e * nout + c] : 0.0f;
      xi[r][c] = (e < n && c < nin) ? xin[e * nin + c] : 0.0f;
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const int pidx = t + q * 256;
      if (pidx < pairs) {
        const int o = pidx / nin, i = pidx - o * nin;
        float a = acc[q];
        for (int r = 0; r < 32; ++r) a = fmaf(go[r][o], xi[r][i], a);
        acc[q] = a;
      }
    }
    if (t < nout)
      for (int r = 0; r < 32; ++r) accb += go[r][t];
  }
#pragma unroll
  for (int q = 0; q < 16; ++q) {
    const int pidx = t + q * 256;
    if (pidx < pairs) atomicAdd(gW + pidx, acc[q]);
  }
  if (t < nout && gb) atomicAdd(gb + t, accb);
}

// dh_prev = dh + Ws^T g + Wn^T (sum of g over the face neighbours)
__global__ void __launch_bounds__(256) k_bwd_layer_in(int64_t n, int K, const int4* __restrict__ nbr,
                                                      const __nv_bfloat16* __restrict__ Ws,
                                                      const __nv_bfloat16* __restrict__ Wn,
                                                      const float* __restrict__ dh, const float* __restrict__ g,
                                                      float* __restrict__ dhp) {
  __shared__ float ws[kW][kW], wn[kW][kW];  // [channel c][input i]
  __shared__ float gs[4][kW], Gs[4][kW];
  const int t = threadIdx.x, el = t >> 6, i = t & 63;
  for (int q = t; q < kW * kW; q += 256) {
    ws[q / kW][q % kW] = bf(Ws[q]);
    wn[q / kW][q % kW] = bf(Wn[q]);
  }
  for (int64_t g0 = (int64_t)blockIdx.x * 4; g0 < n; g0 += (int64_t)gridDim.x * 4) {
    __syncthreads();
    {
      const int64_t e = g0 + el;
      float gv = 0.0f, Gv = 0.0f;
      if (e < n) {
        gv = g[e * kW + i];
        int64_t j[3];
        neighbours(nbr, K, e, j);
#pragma unroll
        for (int f = 0; f < 3; ++f)
          if (j[f] >= 0) Gv += g[j[f] * kW + i];
      }
      gs[el][i] = gv;
      Gs[el][i] = Gv;
    }
    __syncthreads();
    const int64_t e = g0 + el;
    if (e < n) {
      float a = dh[e * kW + i];
#pragma unroll 8
      for (int c = 0; c < kW; ++c) a = fmaf(ws[c][i], gs[el][c], fmaf(wn[c][i], Gs[el][c], a));
      dhp[e * kW + i] = a;
    }
  }
}

__global__ void k_adam(int64_t P, float* __restrict__ w, __nv_bfloat16* __restrict__ w16,
                       const float* __restrict__ gr, float* __restrict__ m, float* __restrict__ v, float lr,
                       float c1, float c2) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P; i += (int64_t)gridDim.x * blockDim.x) {
    const float gi = gr[i];
    const float mi = 0.9f * m[i] + 0.1f * gi, vi = 0.999f * v[i] + 0.001f * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi * c1) / (sqrtf(vi * c2) + 1e-8f);
    w[i] = wi;
    w16[i] = __float2bfloat16(wi);
  }
}

__global__ void k_to_bf16(int64_t P, const float* __restrict__ w, __nv_bfloat16* __restrict__ w16) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P; i += (int64_t)gridDim.x * blockDim.x)
    w16[i] = __float2bfloat16(w[i]);
}

// x = r * scale (FP32, padding nodes 0)
__global__ void k_scale_to_f32(int64_t n, int npi, int np, const double* __restrict__ r, double scale,
                               float* __restrict__ x) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x[i] = (int)(i % npi) < np ? (float)(r[i] * scale) : 0.0f;
}

// residual-correction form: rp = r - S z0 on valid nodes (FP32; S z0 given in
// FP32), and |rp|^2 accumulated in FP64 into *nrm
__global__ void k_post_residual(int64_t n, int npi, int np, const double* __restrict__ r,
                                const float* __restrict__ sz, float* __restrict__ rp, double* __restrict__ nrm) {
  double acc = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float v = (int)(i % npi) < np ? (float)r[i] - sz[i] : 0.0f;
    rp[i] = v;
    acc += (double)v * (double)v;
  }
  block_add(acc, nrm);
}

// FP64 vector -> FP32 copy (padding nodes 0)
__global__ void k_to_f32_valid(int64_t n, int npi, int np, const double* __restrict__ x, float* __restrict__ y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = (int)(i % npi) < np ? (float)x[i] : 0.0f;
}

// x *= scale in place
__global__ void k_scale_f32(int64_t n, float scale, float* __restrict__ x) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x[i] *= scale;
}

// z = bj + scale * y (padding nodes 0)
__global__ void k_precond_combine(int64_t n, int npi, int np, const double* __restrict__ bj,
                                  const float* __restrict__ y, double scale, double* __restrict__ z) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    z[i] = (int)(i % npi) < np ? bj[i] + scale * (double)y[i] : 0.0;
}

// out[j] += a_j . b_j for j < cnt (FP64); `a` shared by every pair when set
constexpr int kMaxDots = 10;
struct DotList {
  const double* a;
  const double* b[kMaxDots];
  int cnt;
};
__global__ void k_mdot(int64_t n, DotList d, double* __restrict__ out) {
  double s[kMaxDots];
#pragma unroll
  for (int j = 0; j < kMaxDots; ++j) s[j] = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double ai = d.a[i];
#pragma unroll
    for (int j = 0; j < kMaxDots; ++j)
      if (j < d.cnt) s[j] = fma(ai, d.b[j][i], s[j]);
  }
#pragma unroll
  for (int j = 0; j < kMaxDots; ++j)
    if (j < d.cnt) block_add(s[j], out + j);
}

// y = a x + y
__global__ void k_axpy64(int64_t n, double a, const double* __restrict__ x, double* __restrict__ y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] += a * x[i];
}
// x += alpha p, r -= alpha q
__global__ void k_step64(int64_t n, double alpha, const double* __restrict__ p, const double* __restrict__ q,
                         double* __restrict__ x, double* __restrict__ r) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    x[i] = fma(alpha, p[i], x[i]);
    r[i] = fma(-alpha, q[i], r[i]);
  }
}
// p = z + sum_j beta_j p_j (j < cnt)
struct DirList {
  const double* p[kMaxDots];
  double beta[kMaxDots];
  int cnt;
};
__global__ void k_orth64(int64_t n, const double* __restrict__ z, DirList d, double* __restrict__ p) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double v = z[i];
#pragma unroll
    for (int j = 0; j < kMaxDots; ++j)
      if (j < d.cnt) v = fma(d.beta[j], d.p[j][i], v);
    p[i] = v;
  }
}
// r = b - r
__global__ void k_bminus64(int64_t n, const double* __restrict__ b, double* __restrict__ r) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    r[i] = b[i] - r[i];
}

}  // namespace dgk

struct dgc_mpnn_s {
  dgc_handle h = nullptr;
  dgk::MpnnLayout lay;
  int sm_count = 0;
  float* w = nullptr;            // FP32 master weights
  __nv_bfloat16* w16 = nullptr;  // BF16 copies read by the kernels
  float* grad = nullptr;
  float* am = nullptr;           // Adam moments
  float* av = nullptr;
  int64_t step = 0;
  // training activations for `cap` samples
  int cap = 0;
  std::vector<float*> hs;        // h_0 .. h_L  [S K W]
  std::vector<float*> as;        // a_1 .. a_L  [S K W]
  float *y = nullptr, *dy = nullptr, *dh0 = nullptr, *dh1 = nullptr, *g = nullptr, *m = nullptr;
  float *sd = nullptr, *tm = nullptr, *st = nullptr;  // energy loss: S d, masked t, S t
  int loss_kind = DGC_MPNN_LOSS_ENERGY;
  int linear = 0;                // DGC_MPNN_ACT_LINEAR: no ReLU, biases held at zero
  int post = 0;                  // DGC_MPNN_CORR_RESIDUAL: the network acts on r - S z0
  bool coarse = false;           // add the handle's coarse-space correction to Binv r
  double* scal = nullptr;        // training: [0] loss, [1..] per-sample target norms; solver: dot products
  double* h_scal = nullptr;      // pinned
  int scal_cap = 0;
  // preconditioner / flexible CG work (one field)
  float *px = nullptr, *ph0 = nullptr, *ph1 = nullptr, *py = nullptr, *pt = nullptr;
  double *bj = nullptr, *r = nullptr, *z = nullptr;
  static constexpr int kMaxWindow = 8;
  double* pv[kMaxWindow + 1] = {};  // direction ring p_i, i mod (window + 1)
  double* qv[kMaxWindow + 1] = {};  // S p_i
};

namespace {

int merr(int code, const char* msg) {
  dgc::set_error(code, msg);
  return code;
}
int mcuda(cudaError_t e, const char* what) {
  std::string s = std::string(what) + ": " + cudaGetErrorString(e);
  return merr(DGC_ERR_CUDA, s.c_str());
}
#define CKM(call)                                     \
  do {                                                \
    cudaError_t e_ = (call);                          \
    if (e_ != cudaSuccess) return mcuda(e_, #call);   \
  } while (0)

int grid_for(const dgc_mpnn_s* m, int64_t work, int per_block) {
  const int64_t b = (work + per_block - 1) / per_block;
  return (int)std::max<int64_t>(1, std::min<int64_t>(b, (int64_t)m->sm_count * 8));
}

// reductions end in one atomic per block and product on the same few addresses:
// 2 blocks per SM
int dot_grid(const dgc_mpnn_s* m, int64_t n) { return std::min(grid_for(m, n, 256), 2 * std::max(m->sm_count, 1)); }

size_t field_len(const dgc_mpnn_s* m) { return (size_t)m->h->K * m->h->NpP; }

// device allocation cleared to zero: solver vectors are summed whole, padding included
template <typename T>
cudaError_t zalloc(T** p, size_t count) {
  cudaError_t e = cudaMalloc(p, count * sizeof(T));
  return e == cudaSuccess ? cudaMemset(*p, 0, count * sizeof(T)) : e;
}

// device scalars (and their pinned host copy) for at least `count` doubles
int ensure_scal(dgc_mpnn m, int count) {
  if (count <= m->scal_cap) return DGC_OK;
  double* ns = nullptr;
  double* nh = nullptr;
  CKM(cudaMalloc(&ns, count * sizeof(double)));
  if (cudaError_t e = cudaMallocHost(&nh, count * sizeof(double))) {
    cudaFree(ns);
    return mcuda(e, "cudaMallocHost");
  }
  cudaFree(m->scal);
  cudaFreeHost(m->h_scal);
  m->scal = ns;
  m->h_scal = nh;
  m->scal_cap = count;
  return DGC_OK;
}

int ensure_train(dgc_mpnn m, int S) {
  if (S <= m->cap) return DGC_OK;
  auto fr = [](float*& p) { cudaFree(p); p = nullptr; };
  for (auto& p : m->hs) fr(p);
  for (auto& p : m->as) fr(p);
  fr(m->y); fr(m->dy); fr(m->dh0); fr(m->dh1); fr(m->g); fr(m->m);
  fr(m->sd); fr(m->tm); fr(m->st);
  const size_t nW = (size_t)S * m->h->K * dgk::kW, nY = (size_t)S * field_len(m);
  m->hs.assign(m->lay.L + 1, nullptr);
  m->as.assign(m->lay.L, nullptr);
  for (auto& p : m->hs) CKM(zalloc(&p, nW));
  for (auto& p : m->as) CKM(zalloc(&p, nW));
  CKM(zalloc(&m->y, nY));
  CKM(zalloc(&m->dy, nY));
  CKM(zalloc(&m->dh0, nW));
  CKM(zalloc(&m->dh1, nW));
  CKM(zalloc(&m->g, nW));
  CKM(zalloc(&m->m, nW));
  CKM(zalloc(&m->sd, nY));
  CKM(zalloc(&m->tm, nY));
  CKM(zalloc(&m->st, nY));
  m->cap = S;
  // [0] loss, [1..S] target norms (L2 loss), [1+S .. 1+3S) per-sample d.Sd, t.St (energy loss)
  return ensure_scal(m, 1 + 3 * S);
}

int ensure_apply(dgc_mpnn m) {
  if (m->px) return DGC_OK;
  const size_t nW = (size_t)m->h->K * dgk::kW, nY = field_len(m);
  CKM(zalloc(&m->px, nY));
  CKM(zalloc(&m->py, nY));
  CKM(zalloc(&m->pt, nY));
  CKM(zalloc(&m->ph0, nW));
  CKM(zalloc(&m->ph1, nW));
  for (double** p : {&m->bj, &m->r, &m->z}) CKM(zalloc(p, nY));
  return ensure_scal(m, 4);
}

// direction ring of window + 1 slots and a dot-product buffer of kMaxDots
int ensure_fcg(dgc_mpnn m, int window) {
  const size_t nY = field_len(m);
  for (int i = 0; i <= window; ++i) {
    if (!m->pv[i]) CKM(zalloc(&m->pv[i], nY));
    if (!m->qv[i]) CKM(zalloc(&m->qv[i], nY));
  }
  return ensure_scal(m, dgk::kMaxDots);
}

// forward over n graph nodes; h ping-pong through (ha, hb) or the stored layers
int forward(dgc_mpnn m, int64_t n, const float* x, float* y, float* ha, float* hb, bool store, cudaStream_t s) {
  const auto& L = m->lay;
  const int4* nbr = reinterpret_cast<const int4*>(m->h->d_nbr);
  const int K = m->h->K;
  float* cur = store ? m->hs[0] : ha;
  dgk::k_fwd_in<<<grid_for(m, n, 4), 256, 0, s>>>(n, L.npi, m->w16 + L.oWin, m->w16 + L.obin, x, cur);
  CKM(cudaGetLastError());
  for (int l = 0; l < L.L; ++l) {
    float* nxt = store ? m->hs[l + 1] : (cur == ha ? hb : ha);
    // tensor-core layer (mpnn_tc.cuh): persistent CTAs over 128-node tiles, 2 per SM
    const int tiles = (int)std::min<int64_t>((n + dgk::MpnnTc::kRows - 1) / dgk::MpnnTc::kRows,
                                             (int64_t)m->sm_count * 2);
    dgk::k_fwd_layer_tc<<<tiles, dgk::MpnnTc::kThreads, dgk::MpnnTc::kSmem, s>>>(
        n, K, nbr, m->w16 + L.oWs(l), m->w16 + L.oWn(l), m->w16 + L.ob(l), cur, store ? m->as[l] : nullptr, nxt,
        m->linear, m->h->d_status);
    CKM(cudaGetLastError());
    cur = nxt;
  }
  const int per = std::min(256 / L.npi, 16);
  dgk::k_fwd_out<<<grid_for(m, n, per), 256, 0, s>>>(n, L.npi, m->w16 + L.oWout, m->w16 + L.obout, cur, y);
  CKM(cudaGetLastError());
  m->h->launches += L.L + 2;
  return DGC_OK;
}

// FP64 dot products a.b_j (j < cnt) into out, synchronising the stream
int dots(dgc_mpnn m, const double* a, std::initializer_list<const double*> bs, double* out, cudaStream_t s) {
  const int64_t n = (int64_t)field_len(m);
  dgk::DotList d{};
  d.a = a;
  d.cnt = 0;
  for (const double* b : bs) d.b[d.cnt++] = b;
  CKM(cudaMemsetAsync(m->scal, 0, d.cnt * sizeof(double), s));
  dgk::k_mdot<<<dot_grid(m, n), 256, 0, s>>>(n, d, m->scal);
  CKM(cudaGetLastError());
  CKM(cudaMemcpyAsync(m->h_scal, m->scal, d.cnt * sizeof(double), cudaMemcpyDeviceToHost, s));
  CKM(cudaStreamSynchronize(s));
  for (int j = 0; j < d.cnt; ++j) out[j] = m->h_scal[j];
  ++m->h->launches;
  return DGC_OK;
}

// M(r) into z (block-Jacobi part left in m->bj); nr = |r| when known (< 0: computed here)
int precondition(dgc_mpnn m, const double* r, double* z, cudaStream_t s, double nr = -1.0) {
  dgc_handle h = m->h;
  const int64_t n = (int64_t)field_len(m);
  if (nr < 0.0) {
    double rr;
    if (int rc = dots(m, r, {r}, &rr, s)) return rc;
    nr = std::sqrt(rr);
  }
  if (int rc = dgc::ipdg_block_jacobi_apply(h, r, m->bj, s)) return rc;
  if (m->coarse)
    if (int rc = dgc::coarse_apply(h, r, m->bj, m->bj, true, true, s)) return rc;
  if (nr == 0.0) {
    CKM(cudaMemsetAsync(z, 0, n * sizeof(double), s));
    return DGC_OK;
  }
  // network input x c / |x| (unit RMS per valid node, c = sqrt(K Np)), output scaled back by |x| / c;
  // x = r, or in the residual-correction form x = r - S z0 (S applied in FP32)
  const double c = std::sqrt((double)h->K * h->Np);
  if (m->post) {
    dgk::k_to_f32_valid<<<grid_for(m, n, 256), 256, 0, s>>>(n, m->lay.npi, h->Np, m->bj, m->pt);
    CKM(cudaGetLastError());
    if (int rc = dgc::ipdg_spd_apply_f32(h, m->pt, m->py, s)) return rc;
    CKM(cudaMemsetAsync(m->scal, 0, sizeof(double), s));
    dgk::k_post_residual<<<dot_grid(m, n), 256, 0, s>>>(n, m->lay.npi, h->Np, r, m->py, m->px, m->scal);
    CKM(cudaGetLastError());
    CKM(cudaMemcpyAsync(m->h_scal, m->scal, sizeof(double), cudaMemcpyDeviceToHost, s));
    CKM(cudaStreamSynchronize(s));
    nr = std::sqrt(m->h_scal[0]);
    if (nr == 0.0) {
      CKM(cudaMemcpyAsync(z, m->bj, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
      return DGC_OK;
    }
    dgk::k_scale_f32<<<grid_for(m, n, 256), 256, 0, s>>>(n, (float)(c / nr), m->px);
    h->launches += 3;
  } else {
    dgk::k_scale_to_f32<<<grid_for(m, n, 256), 256, 0, s>>>(n, m->lay.npi, h->Np, r, c / nr, m->px);
  }
  CKM(cudaGetLastError());
  if (int rc = forward(m, h->K, m->px, m->py, m->ph0, m->ph1, false, s)) return rc;
  dgk::k_precond_combine<<<grid_for(m, n, 256), 256, 0, s>>>(n, m->lay.npi, h->Np, m->bj, m->py, nr / c, z);
  CKM(cudaGetLastError());
  h->launches += 3;
  return DGC_OK;
}

}  // namespace

extern "C" int dgc_mpnn_create(dgc_handle h, int layers, uint64_t seed, dgc_mpnn* out) {
  if (!h || !out) return merr(DGC_ERR_ARG, "null argument");
  *out = nullptr;
  if (h->desc.physics != DGC_LAPLACE || !h->desc.dirichlet)
    return merr(DGC_ERR_UNSUPPORTED, "the learned preconditioner needs a Dirichlet laplace handle");
  if (layers < 1 || layers > 16) return merr(DGC_ERR_ARG, "layers outside [1, 16]");
  if (h->NpP > 64) return merr(DGC_ERR_UNSUPPORTED, "orders above 9 not supported by the network");
  auto* m = new dgc_mpnn_s();
  m->h = h;
  m->lay.init(h->NpP, layers);
  auto fail = [&](int rc) {
    dgc_mpnn_destroy(m);
    return rc;
  };
  cudaError_t e = cudaDeviceGetAttribute(&m->sm_count, cudaDevAttrMultiProcessorCount, h->device);
  const int64_t P = m->lay.total;
  // Glorot-uniform hidden weights, zero biases and a zero output layer: an
  // untrained network adds nothing, so M starts as block-Jacobi and training
  // can only move it from there
  std::vector<float> w(P, 0.0f);
  std::mt19937_64 rng(seed);
  auto fill = [&](int64_t off, int rows, int cols, float gain) {
    const float a = gain * std::sqrt(6.0f / (rows + cols));
    std::uniform_real_distribution<float> u(-a, a);
    for (int64_t i = 0; i < (int64_t)rows * cols; ++i) w[off + i] = u(rng);
  };
  fill(m->lay.oWin, dgk::kW, m->lay.npi, 1.0f);
  for (int l = 0; l < layers; ++l) {
    fill(m->lay.oWs(l), dgk::kW, dgk::kW, 0.5f);
    fill(m->lay.oWn(l), dgk::kW, dgk::kW, 0.5f);
  }
  if (e == cudaSuccess) e = cudaMalloc(&m->w, P * 4);
  if (e == cudaSuccess) e = cudaMalloc(&m->w16, P * sizeof(__nv_bfloat16));
  if (e == cudaSuccess) e = cudaMalloc(&m->grad, P * 4);
  if (e == cudaSuccess) e = cudaMalloc(&m->am, P * 4);
  if (e == cudaSuccess) e = cudaMalloc(&m->av, P * 4);
  if (e == cudaSuccess) e = cudaMemcpy(m->w, w.data(), P * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(m->am, 0, P * 4);
  if (e == cudaSuccess) e = cudaMemset(m->av, 0, P * 4);
  if (e != cudaSuccess) return fail(mcuda(e, "mpnn set-up"));
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(dgk::k_fwd_layer_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, dgk::MpnnTc::kSmem);
  if (e != cudaSuccess) return fail(mcuda(e, "mpnn set-up"));
  dgk::k_to_bf16<<<grid_for(m, P, 256), 256>>>(P, m->w, m->w16);
  if ((e = cudaGetLastError()) != cudaSuccess) return fail(mcuda(e, "mpnn set-up"));
  *out = m;
  return DGC_OK;
}

extern "C" int dgc_mpnn_destroy(dgc_mpnn m) {
  if (!m) return DGC_OK;
  for (float* p : {m->w, m->grad, m->am, m->av, m->y, m->dy, m->dh0, m->dh1, m->g, m->m, m->sd, m->tm, m->st,
                   m->px, m->ph0, m->ph1,
                   m->py, m->pt})
    cudaFree(p);
  for (auto p : m->hs) cudaFree(p);
  for (auto p : m->as) cudaFree(p);
  cudaFree(m->w16);
  for (double* p : {m->scal, m->bj, m->r, m->z}) cudaFree(p);
  for (int i = 0; i <= dgc_mpnn_s::kMaxWindow; ++i) {
    cudaFree(m->pv[i]);
    cudaFree(m->qv[i]);
  }
  cudaFreeHost(m->h_scal);
  delete m;
  return DGC_OK;
}

extern "C" int64_t dgc_mpnn_num_params(dgc_mpnn m) { return m ? m->lay.total : -1; }

extern "C" int dgc_mpnn_get_weights(dgc_mpnn m, float* out) {
  if (!m || !out) return merr(DGC_ERR_ARG, "null argument");
  CKM(cudaMemcpy(out, m->w, m->lay.total * 4, cudaMemcpyDeviceToHost));
  return DGC_OK;
}

extern "C" int dgc_mpnn_set_weights(dgc_mpnn m, const float* in) {
  if (!m || !in) return merr(DGC_ERR_ARG, "null argument");
  CKM(cudaMemcpy(m->w, in, m->lay.total * 4, cudaMemcpyHostToDevice));
  dgk::k_to_bf16<<<grid_for(m, m->lay.total, 256), 256>>>(m->lay.total, m->w, m->w16);
  CKM(cudaGetLastError());
  CKM(cudaDeviceSynchronize());
  return DGC_OK;
}

extern "C" int dgc_mpnn_set_loss(dgc_mpnn m, int kind) {
  if (!m) return merr(DGC_ERR_ARG, "null argument");
  if (kind != DGC_MPNN_LOSS_L2 && kind != DGC_MPNN_LOSS_ENERGY) return merr(DGC_ERR_ARG, "unknown loss kind");
  m->loss_kind = kind;
  return DGC_OK;
}

extern "C" int dgc_mpnn_set_coarse(dgc_mpnn m, int cells_per_aggregate, void* stream) {
  if (!m) return merr(DGC_ERR_ARG, "null network");
  if (cells_per_aggregate <= 0) {
    m->coarse = false;
    return DGC_OK;
  }
  if (int rc = dgc_coarse_build(m->h, cells_per_aggregate, stream)) return rc;
  m->coarse = true;
  return DGC_OK;
}

extern "C" int dgc_mpnn_forward(dgc_mpnn m, const float* x, float* y, void* stream) {
  if (!m || !x || !y) return merr(DGC_ERR_ARG, "null argument");
  if (int rc = ensure_apply(m)) return rc;
  return forward(m, m->h->K, x, y, m->ph0, m->ph1, false, static_cast<cudaStream_t>(stream));
}

// zero the bias entries of a parameter-sized vector (weights or gradients)
static int zero_biases(dgc_mpnn m, float* v, cudaStream_t s) {
  const auto& L = m->lay;
  CKM(cudaMemsetAsync(v + L.obin, 0, dgk::kW * 4, s));
  for (int l = 0; l < L.L; ++l) CKM(cudaMemsetAsync(v + L.ob(l), 0, dgk::kW * 4, s));
  CKM(cudaMemsetAsync(v + L.obout, 0, (size_t)L.npi * 4, s));
  return DGC_OK;
}

extern "C" int dgc_mpnn_set_activation(dgc_mpnn m, int kind) {
  if (!m) return merr(DGC_ERR_ARG, "null network");
  if (kind != DGC_MPNN_ACT_RELU && kind != DGC_MPNN_ACT_LINEAR) return merr(DGC_ERR_ARG, "unknown activation");
  m->linear = kind == DGC_MPNN_ACT_LINEAR;
  if (m->linear) {
    if (int rc = zero_biases(m, m->w, 0)) return rc;
    const auto& L = m->lay;
    dgk::k_to_bf16<<<grid_for(m, L.total, 256), 256>>>(L.total, m->w, m->w16);
    CKM(cudaGetLastError());
    CKM(cudaDeviceSynchronize());
  }
  return DGC_OK;
}

extern "C" int dgc_mpnn_set_correction(dgc_mpnn m, int kind) {
  if (!m) return merr(DGC_ERR_ARG, "null network");
  if (kind != DGC_MPNN_CORR_ADDITIVE && kind != DGC_MPNN_CORR_RESIDUAL)
    return merr(DGC_ERR_ARG, "unknown correction form");
  m->post = kind == DGC_MPNN_CORR_RESIDUAL;
  return DGC_OK;
}

extern "C" int dgc_mpnn_train_step(dgc_mpnn m, const float* x, const float* t, int S, float lr, float* loss,
                                   float* grad_out, void* stream) {
  if (!m || !x || !t || S <= 0) return merr(DGC_ERR_ARG, "null argument or no samples");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (int rc = ensure_train(m, S)) return rc;
  const auto& L = m->lay;
  const int K = m->h->K, np = m->h->Np, npi = L.npi;
  const int64_t n = (int64_t)S * K;
  const int4* nbr = reinterpret_cast<const int4*>(m->h->d_nbr);
  // forward, keeping activations
  if (int rc = forward(m, n, x, m->y, nullptr, nullptr, true, s)) return rc;
  // loss and dy
  CKM(cudaMemsetAsync(m->scal, 0, (1 + 3 * S) * sizeof(double), s));
  if (m->loss_kind == DGC_MPNN_LOSS_L2) {
    dgk::k_target_norm<<<dim3(grid_for(m, (int64_t)K * npi, 256), S), 256, 0, s>>>(K, npi, np, t, m->scal + 1);
    dgk::k_loss<<<grid_for(m, n * npi, 256), 256, 0, s>>>(n, K, npi, np, S, m->y, t, m->scal + 1, m->dy, m->scal);
    CKM(cudaGetLastError());
    m->h->launches += 2;
  } else {  // energy norm: |y - t|_S^2 / |t|_S^2 with the FP32 SPD apply
    const int64_t f = (int64_t)K * npi;
    dgk::k_mask_diff<<<grid_for(m, n * npi, 256), 256, 0, s>>>(n * npi, npi, np, m->y, t, m->dy, m->tm);
    CKM(cudaGetLastError());
    for (int j = 0; j < S; ++j) {
      if (int rc = dgc::ipdg_spd_apply_f32(m->h, m->dy + j * f, m->sd + j * f, s)) return rc;
      if (int rc = dgc::ipdg_spd_apply_f32(m->h, m->tm + j * f, m->st + j * f, s)) return rc;
    }
    double* dots = m->scal + 1 + S;
    dgk::k_energy_dots<<<dim3(grid_for(m, f, 256), S), 256, 0, s>>>(K, npi, np, m->dy, m->sd, m->tm, m->st, dots);
    dgk::k_energy_grad<<<grid_for(m, n * npi, 256), 256, 0, s>>>(n * npi, K, npi, np, S, m->sd, dots, m->dy,
                                                                 m->scal);
    CKM(cudaGetLastError());
    m->h->launches += 3;
  }
  // backward
  CKM(cudaMemsetAsync(m->grad, 0, L.total * 4, s));
  dgk::k_grad_dense<<<grid_for(m, n, 32), 256, 0, s>>>(n, npi, dgk::kW, m->dy, m->hs[L.L], m->grad + L.oWout,
                                                       m->grad + L.obout);
  dgk::k_bwd_out<<<grid_for(m, n, 4), 256, 0, s>>>(n, npi, m->w16 + L.oWout, m->dy, m->dh0);
  CKM(cudaGetLastError());
  float* dh = m->dh0;
  float* dhp = m->dh1;
  for (int l = L.L - 1; l >= 0; --l) {
    dgk::k_relu_bwd<<<grid_for(m, n * dgk::kW, 256), 256, 0, s>>>(n * dgk::kW, dh, m->as[l], m->g, m->linear);
    dgk::k_grad_dense<<<grid_for(m, n, 32), 256, 0, s>>>(n, dgk::kW, dgk::kW, m->g, m->hs[l], m->grad + L.oWs(l),
                                                         m->grad + L.ob(l));
    dgk::k_gather<<<grid_for(m, n * dgk::kW, 256), 256, 0, s>>>(n, K, nbr, m->hs[l], m->m);
    dgk::k_grad_dense<<<grid_for(m, n, 32), 256, 0, s>>>(n, dgk::kW, dgk::kW, m->g, m->m, m->grad + L.oWn(l),
                                                         nullptr);
    dgk::k_bwd_layer_in<<<grid_for(m, n, 4), 256, 0, s>>>(n, K, nbr, m->w16 + L.oWs(l), m->w16 + L.oWn(l), dh,
                                                          m->g, dhp);
    CKM(cudaGetLastError());
    std::swap(dh, dhp);
  }
  dgk::k_grad_dense<<<grid_for(m, n, 32), 256, 0, s>>>(n, dgk::kW, npi, dh, x, m->grad + L.oWin, m->grad + L.obin);
  CKM(cudaGetLastError());
  m->h->launches += 3 + 5 * L.L;  // output grads, 5 per layer, input grads
  if (m->linear) {  // the biases stay at zero: the network remains a linear map
    if (int rc = zero_biases(m, m->grad, s)) return rc;
  }
  if (grad_out) CKM(cudaMemcpyAsync(grad_out, m->grad, L.total * 4, cudaMemcpyDeviceToDevice, s));
  if (lr > 0.0f) {
    ++m->step;
    const float c1 = 1.0f / (1.0f - std::pow(0.9f, (float)m->step));
    const float c2 = 1.0f / (1.0f - std::pow(0.999f, (float)m->step));
    dgk::k_adam<<<grid_for(m, L.total, 256), 256, 0, s>>>(L.total, m->w, m->w16, m->grad, m->am, m->av, lr, c1, c2);
    CKM(cudaGetLastError());
    ++m->h->launches;
  }
  if (loss) {
    CKM(cudaMemcpyAsync(m->h_scal, m->scal, sizeof(double), cudaMemcpyDeviceToHost, s));
    CKM(cudaStreamSynchronize(s));
    *loss = (float)m->h_scal[0];
  }
  return DGC_OK;
}

extern "C" int dgc_mpnn_precondition(dgc_mpnn m, const double* r, double* z, void* stream) {
  if (!m || !r || !z) return merr(DGC_ERR_ARG, "null argument");
  if (int rc = ensure_apply(m)) return rc;
  return precondition(m, r, z, static_cast<cudaStream_t>(stream));
}

extern "C" int dgc_fpcg_solve(dgc_handle h, dgc_mpnn m, const double* b, double* x, const dgc_solve_opts* opts,
                              dgc_solve_stats* stats, void* stream) {
  if (!h || !m || !b || !x || !opts || b == x) return merr(DGC_ERR_ARG, "null argument or b aliases x");
  if (m->h != h) return merr(DGC_ERR_ARG, "network built for another handle");
  if (!(opts->rtol > 0.0) || opts->maxit <= 0) return merr(DGC_ERR_ARG, "rtol must be > 0 and maxit > 0");
  const int window = opts->max_outer <= 0 ? 4 : opts->max_outer;
  if (window > dgc_mpnn_s::kMaxWindow) return merr(DGC_ERR_ARG, "truncation window above 8");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (int rc = ensure_apply(m)) return rc;
  if (int rc = ensure_fcg(m, window)) return rc;
  const auto t0 = std::chrono::steady_clock::now();
  const int64_t n = (int64_t)field_len(m);
  const int gd = grid_for(m, n, 256);
  auto residual = [&](double* rr) -> int {  // r = b - S x, rr = |r|^2
    if (int rc = dgc_laplace_spd_apply(h, x, m->r, s)) return rc;
    dgk::k_bminus64<<<gd, 256, 0, s>>>(n, b, m->r);
    CKM(cudaGetLastError());
    ++h->launches;
    return dots(m, m->r, {m->r}, rr, s);
  };
  double bb = 0.0;
  if (int rc = dots(m, b, {b}, &bb, s)) return rc;
  const double tol2 = opts->rtol * opts->rtol * bb;
  double rr = 0.0;
  if (int rc = residual(&rr)) return rc;
  double pq[dgc_mpnn_s::kMaxWindow + 1] = {};  // p_i . S p_i per ring slot
  // k counts iterations since the last (re)start; when the recursive residual
  // falls below a quarter of the target the true residual is computed and,
  // if still above it, the iteration restarts from it (drift correction)
  int it = 0, k = 0, passes = 0;
  bool done = rr <= tol2;  // decided on true residuals only
  while (!done && it < opts->maxit) {
    if (int rc = precondition(m, m->r, m->z, s, std::sqrt(rr))) return rc;
    const int nprev = std::min(k, window), slots = window + 1, slot = k % slots;
    // z.r and z.q_j against the previous directions (newest first)
    dgk::DotList dl{};
    double d[dgk::kMaxDots];
    auto zdots = [&]() -> int {
      dl.a = m->z;
      dl.cnt = 1 + nprev;
      dl.b[0] = m->r;
      for (int j = 0; j < nprev; ++j) dl.b[1 + j] = m->qv[(k - 1 - j + slots) % slots];
      CKM(cudaMemsetAsync(m->scal, 0, dl.cnt * sizeof(double), s));
      dgk::k_mdot<<<dot_grid(m, n), 256, 0, s>>>(n, dl, m->scal);
      CKM(cudaGetLastError());
      CKM(cudaMemcpyAsync(m->h_scal, m->scal, dl.cnt * sizeof(double), cudaMemcpyDeviceToHost, s));
      CKM(cudaStreamSynchronize(s));
      for (int j = 0; j < dl.cnt; ++j) d[j] = m->h_scal[j];
      ++h->launches;
      return DGC_OK;
    };
    if (int rc = zdots()) return rc;
    if (!(d[0] > 0.0)) {  // M(r) is no descent direction: take the block-Jacobi one
      CKM(cudaMemcpyAsync(m->z, m->bj, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
      if (int rc = zdots()) return rc;
    }
    dgk::DirList dir{};
    dir.cnt = nprev;
    for (int j = 0; j < nprev; ++j) {
      const int kj = (k - 1 - j + slots) % slots;
      dir.p[j] = m->pv[kj];
      dir.beta[j] = -d[1 + j] / pq[kj];
    }
    double* p = m->pv[slot];
    double* q = m->qv[slot];
    dgk::k_orth64<<<gd, 256, 0, s>>>(n, m->z, dir, p);
    CKM(cudaGetLastError());
    ++h->launches;
    if (int rc = dgc_laplace_spd_apply(h, p, q, s)) return rc;
    double e[2];
    if (int rc = dots(m, p, {q, m->r}, e, s)) return rc;
    if (!(e[0] > 0.0)) return merr(DGC_ERR_NOT_CONVERGED, "flexible CG: direction of non-positive curvature");
    pq[slot] = e[0];
    dgk::k_step64<<<gd, 256, 0, s>>>(n, e[1] / e[0], p, q, x, m->r);
    CKM(cudaGetLastError());
    ++h->launches;
    ++it;
    ++k;
    if (int rc = dots(m, m->r, {m->r}, &rr, s)) return rc;
    if (rr <= 0.25 * tol2 || it == opts->maxit) {
      if (int rc = residual(&rr)) return rc;
      ++passes;
      k = 0;
      done = rr <= tol2;
    }
  }
  // rr is the true residual here: the initial one or that of the last check
  dgc_solve_stats S{};
  S.iterations = S.inner_iterations = it;
  S.outer_iterations = passes;  // true-residual checks (restarts + 1 when converged)
  S.final_relres = bb > 0.0 ? std::sqrt(rr / bb) : 0.0;
  S.converged = rr <= tol2 ? 1 : 0;
  S.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (stats) *stats = S;
  if (!S.converged) return merr(DGC_ERR_NOT_CONVERGED, "flexible CG did not reach the requested tolerance");
  return DGC_OK;
}

extern "C" int dgc_learned_solve(dgc_handle h, dgc_mpnn m, const double* b, double* x, const dgc_solve_opts* opts,
                                 int fcg_maxit, dgc_solve_stats* stats, int* fell_back, void* stream) {
  if (!h || !m || !b || !x || !opts || !fell_back) return merr(DGC_ERR_ARG, "null argument");
  if (fcg_maxit < 0 || opts->maxit <= 0) return merr(DGC_ERR_ARG, "fcg_maxit must be >= 0 and maxit > 0");
  *fell_back = 0;
  dgc_solve_stats fs{};
  int rc = DGC_ERR_NOT_CONVERGED;
  if (fcg_maxit > 0) {
    dgc_solve_opts fo = *opts;
    fo.maxit = std::min(fcg_maxit, opts->maxit);
    rc = dgc_fpcg_solve(h, m, b, x, &fo, &fs, stream);
    if (rc != DGC_OK && rc != DGC_ERR_NOT_CONVERGED) return rc;
  }
  if (rc == DGC_OK) {
    if (stats) *stats = fs;
    return DGC_OK;
  }
  // fallback: block-Jacobi PCG from the current iterate, to the same true residual
  *fell_back = 1;
  dgc_solve_opts po = *opts;
  po.maxit = std::max(1, opts->maxit - fs.iterations);
  po.max_outer = 0;  // opts->max_outer was the flexible-CG window; refinement passes take their default
  dgc_solve_stats ps{};
  rc = dgc_pcg_solve(h, b, x, &po, &ps, stream);
  dgc_solve_stats S = ps;
  S.iterations = fs.iterations + ps.iterations;
  S.inner_iterations = fs.iterations;
  S.seconds = fs.seconds + ps.seconds;
  if (stats) *stats = S;
  return rc;
}
