// coarse.cu -- two-level preconditioning of the SPD laplace form (C ABI:
// dgc_coarse_build / dgc_coarse_apply / dgc_coarse_info): the coarse space, the
// two-level PCG behind dgc_pcg_solve's DGC_SOLVE_TWO_LEVEL(_MIXED) modes, and the
// coarse term of the learned preconditioner (mpnn.cu, dgc_mpnn_set_coarse).  No
// counterpart in the reference, which solves its systems directly.
//
// Block-Jacobi on the element blocks of S = -J M A removes the error inside
// each element, but the smooth, mesh-wide error modes it leaves are what
// make plain PCG need thousands of iterations at K ~ 10^4-10^5, and a
// 4-hop message-passing network cannot see them either.  The coarse space
// takes them out.  P0 is constant on each aggregate of about
// `cells_per_aggregate` face-connected cells; constants that jump between
// aggregates pay the interior-penalty term, so the prolongation is smoothed
// once (smoothed aggregation):
//   P = (I - w Binv S) P0,   w = 4 / (3 lambda_max(Binv S)),
// A_c = P^T S P is the Galerkin coarse matrix, and the additive two-level
// preconditioner is
//   M r = Binv r + P A_c^-1 P^T r   (+ the network's correction).
//
// Set-up (host + GPU, once per handle and shift): greedy breadth-first
// aggregation in cell order (aggregates smaller than a quarter of the
// target merge into a neighbour); lambda_max from 20 power iterations
// (times 1.1); a colouring of the aggregates such that no cell has two
// aggregates of one colour within six faces (the reach of P^T S P: two faces
// per S, laplace_2d's two passes), so one application of P^T S P to the sum
// of a colour's indicator vectors yields all of that colour's columns of
// A_c; A_c inverted in place on the GPU by Gauss-Jordan without pivoting
// (SPD).  Apply: P^T r = P0^T (r - w S Binv r), a deterministic restriction
// (one warp per aggregate over its cells, fixed order), a dense FP64 product
// with A_c^-1 (one warp per row), the prolongation y = P0 x_c and
// z += y - w Binv S y.  All-Neumann handles without shift have the constants as
// null space (P 1 = 1): A_c gets a rank-one term that makes it regular and
// leaves its action on consistent (zero-sum) residuals unchanged, and the
// two-level PCG keeps its preconditioned residual at zero mean.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "dgc_gb300.h"
#include "dgc_internal.hpp"

namespace dgc {

struct CoarseSpace {
  int cells_per_agg = 0, nagg = 0, ncolors = 0;
  double shift = 0.0;                 // the SPD form's shift when A_c was built
  double omega = 0.0;                 // prolongation smoothing weight
  std::vector<int32_t> agg;           // aggregate of each cell (host)
  int32_t* d_ptr = nullptr;           // [nagg + 1] CSR of the cells of each aggregate
  int32_t* d_cells = nullptr;         // [K]
  int32_t* d_agg = nullptr;           // [K]
  double* d_ainv = nullptr;           // [nagg][nagg] A_c^-1
  float* d_ainv32 = nullptr;          // FP32 copy of A_c^-1 (the FP32 coarse cycle)
  double* d_rc = nullptr;             // P^T r
  float* d_rc32 = nullptr;            // FP32 copy of P^T r
  double* d_xc = nullptr;             // A_c^-1 P^T r
  double* d_w[3] = {};                // work vectors (K x NpP)
  float* d_f[2] = {};                 // FP32 work vectors of the FP32 smoothing applies
  double* d_pcg[3] = {};              // two-level PCG: z, p, q = S p (allocated on first use)
  double* d_dots = nullptr;           // [4] dot products of the current kernel pair, [3] a mean
  double* d_sc = nullptr;             // [8] device-resident CG scalars (k_coarse_step_dev)
  double* h_sc = nullptr;             // pinned mirror
};

void coarse_free(CoarseSpace* c) {
  if (!c) return;
  for (void* p : {(void*)c->d_ptr, (void*)c->d_cells, (void*)c->d_agg, (void*)c->d_ainv, (void*)c->d_rc,
                  (void*)c->d_xc, (void*)c->d_w[0], (void*)c->d_w[1], (void*)c->d_w[2], (void*)c->d_f[0],
                  (void*)c->d_f[1], (void*)c->d_pcg[0], (void*)c->d_pcg[1], (void*)c->d_pcg[2],
                  (void*)c->d_dots, (void*)c->d_sc, (void*)c->d_ainv32, (void*)c->d_rc32})
    cudaFree(p);
  cudaFreeHost(c->h_sc);
  delete c;
}

}  // namespace dgc

namespace dgk {

// v = indicator of the aggregates of colour `col` on the valid nodes
__global__ void k_coarse_indicator(int64_t n, int npp, int np, const int32_t* __restrict__ agg,
                                   const int32_t* __restrict__ color, int col, double* __restrict__ v) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = i / npp;
    v[i] = ((int)(i - k * npp) < np && color[agg[k]] == col) ? 1.0 : 0.0;
  }
}

// out = x - w z, or out += x - w z with add (out may alias x)
__global__ void k_coarse_axpy(int64_t n, const double* x, double w, const double* __restrict__ z, double* out,
                              int add) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double v = x[i] - w * z[i];
    out[i] = add ? out[i] + v : v;
  }
}

// out = x - w z with z in FP32 (an FP32 operator's output, no FP64 round trip)
__global__ void k_coarse_axpy_z32(int64_t n, const double* x, double w, const float* __restrict__ z, double* out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = x[i] - w * (double)z[i];
}

// FP32 copy of an FP64 vector, and back
__global__ void k_coarse_to_f32(int64_t n, const double* __restrict__ x, float* __restrict__ y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = (float)x[i];
}
__global__ void k_coarse_to_f64(int64_t n, const float* __restrict__ x, double* __restrict__ y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = (double)x[i];
}

// out[j] += a_j . b_j, j < 3 (FP64; unused pairs have a null a)
struct Dot3 {
  const double* a[3];
  const double* b[3];
};
__global__ void k_coarse_dots(int64_t n, Dot3 d, double* __restrict__ out) {
  double s[3] = {0.0, 0.0, 0.0};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      if (d.a[j]) s[j] += d.a[j][i] * d.b[j][i];
  __shared__ double red[3][8];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    double v = s[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[j][w] = v;
  }
  __syncthreads();
  if (threadIdx.x < 3 && d.a[threadIdx.x]) {
    double v = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) v += red[threadIdx.x][q];
    atomicAdd(&out[threadIdx.x], v);
  }
}
// block sums of up to three partial dot products, one FP64 atomic per block and product
__device__ __forceinline__ void block_dots_add(const double (&s)[3], int used, double* out) {
  __shared__ double red[3][8];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    double v = s[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[j][w] = v;
  }
  __syncthreads();
  if ((int)threadIdx.x < used) {
    double v = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) v += red[threadIdx.x][q];
    atomicAdd(&out[threadIdx.x], v);
  }
}
// q = x32 in FP64 and out[0] += p.q (the FP32 operator output of the two-level
// iteration, and the dot product its step needs)
__global__ void k_coarse_to_f64_dot(int64_t n, const float* __restrict__ x32, double* __restrict__ q,
                                    const double* __restrict__ p, double* out) {
  double s[3] = {0.0, 0.0, 0.0};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double v = (double)x32[i];
    q[i] = v;
    s[0] += p[i] * v;
  }
  block_dots_add(s, 1, out);
}
// z += x - w y, then out += (r.r, z.r, z.q) with the new z (the last kernel of the
// two-level preconditioner and the dot products of the direction update)
__global__ void k_coarse_axpy_dots(int64_t n, const double* __restrict__ x, double w, const double* __restrict__ y,
                                   double* __restrict__ z, const double* __restrict__ r,
                                   const double* __restrict__ q, double* out) {
  double s[3] = {0.0, 0.0, 0.0};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double zi = z[i] + (x[i] - w * y[i]);
    z[i] = zi;
    const double ri = r[i];
    s[0] += ri * ri;
    s[1] += zi * ri;
    s[2] += zi * q[i];
  }
  block_dots_add(s, 3, out);
}

// out += sum of z over the valid nodes; z -= *out / count on the valid nodes
__global__ void k_coarse_valid_sum(int64_t n, int npp, int np, const double* __restrict__ z, double* out) {
  double v = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if ((int)(i % npp) < np) v += z[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(out, v);
}
__global__ void k_coarse_sub_mean(int64_t n, int npp, int np, const double* __restrict__ sum, double count,
                                  double* __restrict__ z) {
  const double m = *sum / count;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if ((int)(i % npp) < np) z[i] -= m;
}

// The two-level PCG keeps its scalars on the device, so that its kernels queue
// back to back: sc[0], sc[1] = z.r by iteration parity, sc[3] = r.r, sc[5] =
// alpha, sc[6] = stop flag (positivity lost); t = the dot products of the kernel
// just before.
// x += alpha p, r -= alpha q with alpha = z.r / p.q (t[0] = p.q)
__global__ void k_coarse_step_dev(int64_t n, const double* __restrict__ p, const double* __restrict__ q,
                                  double* __restrict__ x, double* __restrict__ r, double* sc,
                                  const double* __restrict__ t, int cur) {
  // one FP64 division per block, not per thread (GB300's FP64 rate is low)
  __shared__ double s_alpha;
  __shared__ int s_ok;
  if (threadIdx.x == 0) {
    const double rz = sc[cur], pq = t[0];
    // at the rounding floor p.Sp or z.r can lose their sign: stop, the caller
    // checks the true residual
    const bool ok = pq > 0.0 && rz > 0.0 && sc[6] == 0.0;
    s_alpha = ok ? rz / pq : 0.0;
    s_ok = ok;
    if (blockIdx.x == 0) {
      sc[5] = s_alpha;
      if (!ok) sc[6] = 1.0;
    }
  }
  __syncthreads();
  const double alpha = s_alpha;
  if (!s_ok) return;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    x[i] += alpha * p[i];
    r[i] -= alpha * q[i];
  }
}
// p = z + beta p, beta = -alpha z.q / (z.r)_old (Polak-Ribiere, robust to the FP32
// rounding inside the coarse term); t = (r.r, z.r, z.q) of the new residual.  The
// new z.r goes to the other parity slot: no block reads what another writes.
__global__ void k_coarse_dir_dev(int64_t n, const double* __restrict__ z, double* __restrict__ p, double* sc,
                                 const double* __restrict__ t, int cur, int nxt, int first, float* __restrict__ p32) {
  __shared__ double s_beta;
  if (threadIdx.x == 0) {
    const double rzo = sc[cur];
    s_beta = (first || sc[6] != 0.0 || !(rzo > 0.0)) ? 0.0 : -sc[5] * t[2] / rzo;
  }
  __syncthreads();
  const double beta = s_beta;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double v = first ? z[i] : z[i] + beta * p[i];
    p[i] = v;
    if (p32) p32[i] = (float)v;  // the next FP32 operator apply's input
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    sc[nxt] = t[1];
    sc[3] = t[0];
  }
}

// in-place Gauss-Jordan step i of an SPD matrix: col[r] = A[r][i]
__global__ void k_gj_col(int n, int i, const double* __restrict__ A, double* __restrict__ col) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < n) col[r] = A[(size_t)r * n + i];
}
// row i: A[i][c] = (c == i ? 1 : A[i][c]) / pivot
__global__ void k_gj_row(int n, int i, double* __restrict__ A, const double* __restrict__ col) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < n) A[(size_t)i * n + c] = (c == i ? 1.0 : A[(size_t)i * n + c]) / col[i];
}
// rows r != i: A[r][c] = (c == i ? 0 : A[r][c]) - col[r] A[i][c]
__global__ void k_gj_elim(int n, int i, double* __restrict__ A, const double* __restrict__ col) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  const int r = blockIdx.y;
  if (c >= n || r == i) return;
  const double v = c == i ? 0.0 : A[(size_t)r * n + c];
  A[(size_t)r * n + c] = v - col[r] * A[(size_t)i * n + c];
}

// rc[a] = sum of r over the valid nodes of the cells of aggregate a (fixed order)
__global__ void k_coarse_restrict(int nagg, int npp, int np, const int32_t* __restrict__ ptr,
                                  const int32_t* __restrict__ cells, const double* __restrict__ r,
                                  double* __restrict__ rc, float* __restrict__ rc32) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= nagg) return;
  double s = 0.0;
  for (int q = ptr[warp]; q < ptr[warp + 1]; ++q) {
    const double* rk = r + (size_t)cells[q] * npp;
    for (int j = lane; j < np; j += 32) s += rk[j];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) {
    rc[warp] = s;
    if (rc32) rc32[warp] = (float)s;
  }
}

// xc = Ainv rc, one warp per row
__global__ void k_coarse_gemv(int n, const double* __restrict__ A, const double* __restrict__ x,
                              double* __restrict__ y) {
  const int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (row >= n) return;
  const double* a = A + (size_t)row * n;
  double s = 0.0;
  for (int c = lane; c < n; c += 32) s += a[c] * x[c];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) y[row] = s;
}

// the same product with the FP32 copy of A_c^-1 and of x, FP32 sums (inside the
// FP32 coarse cycle): half the bytes and no FP64 arithmetic
__global__ void k_coarse_gemv32(int n, const float* __restrict__ A, const float* __restrict__ x,
                                double* __restrict__ y) {
  const int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (row >= n) return;
  const float* a = A + (size_t)row * n;
  float s = 0.0f;
  for (int c = lane; c < n; c += 32) s = fmaf(a[c], x[c], s);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) y[row] = (double)s;
}

// z[k][j] (+)= xc[agg[k]] on the valid nodes
__global__ void k_coarse_prolong(int64_t n, int npp, int np, const int32_t* __restrict__ agg,
                                 const double* __restrict__ xc, int add, double* __restrict__ z,
                                 float* __restrict__ z32) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = i / npp;
    const double v = (int)(i - k * npp) < np ? xc[agg[k]] : 0.0;
    const double o = add ? z[i] + v : v;
    z[i] = o;
    if (z32) z32[i] = (float)o;  // the next FP32 operator apply's input
  }
}

}  // namespace dgk

using namespace dgc;

namespace {

int cfail(cudaError_t e, const char* what) {
  const std::string m = std::string("coarse space: ") + what + ": " + cudaGetErrorString(e);
  return set_error(DGC_ERR_CUDA, m.c_str());
}
#define CKC(call, what)                             \
  do {                                              \
    cudaError_t e_ = (call);                        \
    if (e_ != cudaSuccess) return cfail(e_, what);  \
  } while (0)

int grid1(int64_t n) { return (int)std::min<int64_t>((n + 255) / 256, 8192); }

// breadth-first aggregation in cell order; small aggregates merge into a neighbour
int aggregate(const dgc_handle_s* h, int target, std::vector<int32_t>& agg) {
  const int K = h->K;
  const std::vector<int32_t>& nbr = h->mesh.nbr;
  agg.assign(K, -1);
  std::vector<int> size;
  std::vector<int> queue;
  for (int k0 = 0; k0 < K; ++k0) {
    if (agg[k0] >= 0) continue;
    const int a = (int)size.size();
    size.push_back(0);
    queue.assign(1, k0);
    agg[k0] = a;
    for (size_t q = 0; q < queue.size() && size[a] < target; ++q) {
      const int k = queue[q];
      ++size[a];
      for (int f = 0; f < 3; ++f) {
        const int nb = nbr[4 * (size_t)k + f];
        if (nb < 0) continue;
        const int kn = nb >> 2;
        if (agg[kn] < 0 && (int)queue.size() < target) {
          agg[kn] = a;
          queue.push_back(kn);
        }
      }
    }
    // cells queued beyond the ones counted are still members
    size[a] = (int)queue.size();
  }
  // merge aggregates below a quarter of the target into the neighbour they touch first
  const int nagg0 = (int)size.size();
  std::vector<int> into(nagg0);
  for (int a = 0; a < nagg0; ++a) into[a] = a;
  for (int k = 0; k < K; ++k) {
    const int a = agg[k];
    if (4 * size[a] >= target || into[a] != a) continue;
    for (int f = 0; f < 3; ++f) {
      const int nb = nbr[4 * (size_t)k + f];
      if (nb < 0) continue;
      const int b = into[agg[nb >> 2]];
      if (b != a && 4 * size[b] >= target) {
        into[a] = b;
        size[b] += size[a];
        break;
      }
    }
  }
  std::vector<int> id(nagg0, -1);
  int n = 0;
  for (int a = 0; a < nagg0; ++a)
    if (into[a] == a) id[a] = n++;
  for (int k = 0; k < K; ++k) agg[k] = id[into[agg[k]]];
  return n;
}

// multi-source breadth-first search from the cells of each aggregate to depth
// `radius`: calls visit(a, cell) once per (aggregate, cell within reach)
template <typename F>
void aggregate_reach(const dgc_handle_s* h, const std::vector<int32_t>& ptr, const std::vector<int32_t>& cells,
                     int radius, std::vector<int>& mark, F visit) {
  const std::vector<int32_t>& nbr = h->mesh.nbr;
  std::vector<int> frontier, next, seen;
  const int nagg = (int)ptr.size() - 1;
  for (int a = 0; a < nagg; ++a) {
    frontier.assign(cells.begin() + ptr[a], cells.begin() + ptr[a + 1]);
    for (int k : frontier) mark[k] = a;
    seen = frontier;
    for (int d = 0; d < radius && !frontier.empty(); ++d) {
      next.clear();
      for (int k : frontier)
        for (int f = 0; f < 3; ++f) {
          const int nb = nbr[4 * (size_t)k + f];
          if (nb < 0 || mark[nb >> 2] == a) continue;
          mark[nb >> 2] = a;
          next.push_back(nb >> 2);
          seen.push_back(nb >> 2);
        }
      frontier.swap(next);
    }
    for (int k : seen) visit(a, k);
  }
}

}  // namespace

extern "C" int dgc_coarse_build(dgc_handle h, int cells_per_aggregate, void* stream) {
  if (!h) return set_error(DGC_ERR_ARG, "null handle");
  if (h->desc.physics != DGC_LAPLACE || h->prec != DGC_F64)
    return set_error(DGC_ERR_UNSUPPORTED, "the coarse space needs an FP64 laplace handle");
  if (cells_per_aggregate < 1) return set_error(DGC_ERR_ARG, "cells_per_aggregate must be >= 1");
  if (!ipdg_uniform_bc(h)) return set_error(DGC_ERR_UNSUPPORTED, "the coarse space needs uniform boundary types");
  if (h->coarse && h->coarse->cells_per_agg == cells_per_aggregate && h->coarse->shift == ipdg_shift(h))
    return DGC_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  coarse_free(h->coarse);
  h->coarse = nullptr;
  auto* c = new CoarseSpace();
  c->cells_per_agg = cells_per_aggregate;
  c->shift = ipdg_shift(h);
  const int K = h->K, Np = h->Np, NpP = h->NpP;
  const int nagg = aggregate(h, cells_per_aggregate, c->agg);
  if (nagg > 8192) {
    coarse_free(c);
    return set_error(DGC_ERR_ARG, "more than 8192 aggregates: raise cells_per_aggregate");
  }
  c->nagg = nagg;
  // CSR of the cells of each aggregate
  std::vector<int32_t> ptr(nagg + 1, 0), cells(K);
  for (int k = 0; k < K; ++k) ++ptr[c->agg[k] + 1];
  for (int a = 0; a < nagg; ++a) ptr[a + 1] += ptr[a];
  {
    std::vector<int32_t> fill(ptr.begin(), ptr.end() - 1);
    for (int k = 0; k < K; ++k) cells[fill[c->agg[k]]++] = k;
  }
  // colouring.  One S reaches two faces (laplace_2d's two passes), Binv none,
  // so P^T S P 1_a lives within six faces of aggregate a: touch[k] lists the
  // aggregates within six faces of cell k, and aggregates within twelve faces
  // of each other get different colours.
  constexpr int kReach = 6;
  std::vector<std::vector<int>> touch(K);
  std::vector<std::vector<int>> conflict(nagg);
  {
    std::vector<int> mark(K, -1);
    aggregate_reach(h, ptr, cells, kReach, mark, [&](int a, int k) { touch[k].push_back(a); });
    std::fill(mark.begin(), mark.end(), -1);
    aggregate_reach(h, ptr, cells, 2 * kReach, mark, [&](int a, int k) {
      const int b = c->agg[k];
      if (b != a && (conflict[a].empty() || conflict[a].back() != b)) conflict[a].push_back(b);
    });
  }
  std::vector<int32_t> color(nagg, -1);
  int ncol = 0;
  {
    std::vector<int> used;
    for (int a = 0; a < nagg; ++a) {
      used.assign(ncol + 1, 0);
      for (int b : conflict[a])
        if (color[b] >= 0) used[color[b]] = 1;
      int col = 0;
      while (used[col]) ++col;
      color[a] = col;
      ncol = std::max(ncol, col + 1);
    }
  }
  c->ncolors = ncol;
  const int64_t n = (int64_t)K * NpP;
  int32_t* d_color = nullptr;
  auto fail = [&](int rc) {
    cudaFree(d_color);
    coarse_free(c);
    return rc;
  };
  cudaError_t e = cudaSuccess;
  if ((e = cudaMalloc(&c->d_ptr, (nagg + 1) * 4)) != cudaSuccess || (e = cudaMalloc(&c->d_cells, K * 4)) ||
      (e = cudaMalloc(&c->d_agg, K * 4)) || (e = cudaMalloc(&c->d_ainv, (size_t)nagg * nagg * 8)) ||
      (e = cudaMalloc(&c->d_rc, nagg * 8)) || (e = cudaMalloc(&c->d_xc, nagg * 8)) ||
      (e = cudaMalloc(&d_color, nagg * 4)) || (e = cudaMalloc(&c->d_w[0], n * 8)) ||
      (e = cudaMalloc(&c->d_w[1], n * 8)) || (e = cudaMalloc(&c->d_w[2], n * 8)) ||
      (e = cudaMalloc(&c->d_f[0], n * 4)) || (e = cudaMalloc(&c->d_f[1], n * 4)))
    return fail(cfail(e, "allocation"));
  // work vectors are summed whole (padding included): start them at zero
  for (double* w : c->d_w)
    if ((e = cudaMemset(w, 0, n * 8)) != cudaSuccess) return fail(cfail(e, "clear"));
  for (float* f : c->d_f)
    if ((e = cudaMemset(f, 0, n * 4)) != cudaSuccess) return fail(cfail(e, "clear"));
  if ((e = cudaMemcpy(c->d_ptr, ptr.data(), (nagg + 1) * 4, cudaMemcpyHostToDevice)) ||
      (e = cudaMemcpy(c->d_cells, cells.data(), K * 4, cudaMemcpyHostToDevice)) ||
      (e = cudaMemcpy(c->d_agg, c->agg.data(), K * 4, cudaMemcpyHostToDevice)) ||
      (e = cudaMemcpy(d_color, color.data(), nagg * 4, cudaMemcpyHostToDevice)))
    return fail(cfail(e, "upload"));
  double *v = c->d_w[0], *w1 = c->d_w[1], *w2 = c->d_w[2];
  std::vector<double> hv(n);
  auto download = [&](const double* d) {
    if ((e = cudaMemcpyAsync(hv.data(), d, n * 8, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return false;
    return (e = cudaStreamSynchronize(s)) == cudaSuccess;
  };
  // lambda_max(Binv S): power iteration from a fixed pseudo-random start, norms on the host
  double lam = 0.0;
  {
    uint64_t x = 0x9e3779b97f4a7c15ull;
    for (int64_t i = 0; i < n; ++i) {
      x ^= x << 13;
      x ^= x >> 7;
      x ^= x << 17;
      hv[i] = (i % NpP) < Np ? (double)(x >> 11) * (1.0 / 9007199254740992.0) - 0.5 : 0.0;
    }
    double nv = 0.0;
    for (double q : hv) nv += q * q;
    nv = std::sqrt(nv);
    for (double& q : hv) q /= nv;
    if ((e = cudaMemcpyAsync(v, hv.data(), n * 8, cudaMemcpyHostToDevice, s)) != cudaSuccess)
      return fail(cfail(e, "upload"));
    for (int it = 0; it < 20; ++it) {
      if (int rc = dgc_laplace_spd_apply(h, v, w1, s)) return fail(rc);
      if (int rc = ipdg_block_jacobi_apply(h, w1, w2, s)) return fail(rc);
      if (!download(w2)) return fail(cfail(e, "download"));
      double nz = 0.0;
      for (double q : hv) nz += q * q;
      nz = std::sqrt(nz);
      lam = nz;  // |Binv S v| with |v| = 1
      if (!(nz > 0.0)) break;
      for (double& q : hv) q /= nz;
      if ((e = cudaMemcpyAsync(v, hv.data(), n * 8, cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return fail(cfail(e, "upload"));
    }
  }
  if (!(lam > 0.0)) return fail(set_error(DGC_ERR_DEVICE, "coarse space: lambda_max(Binv S) estimate is not positive"));
  c->omega = 4.0 / (3.0 * 1.1 * lam);
  const double om = c->omega;
  // A_c column by colour: v = sum of the colour's indicators, w1 = P v, w2 = S P v,
  // w1 = P^T w2 = w2 - w S Binv w2; cell k of aggregate b adds its node sum to
  // A_c[b][a], a the colour's aggregate within reach of k
  std::vector<double> Ac((size_t)nagg * nagg, 0.0);
  for (int col = 0; col < ncol; ++col) {
    dgk::k_coarse_indicator<<<grid1(n), 256, 0, s>>>(n, NpP, Np, c->d_agg, d_color, col, v);
    if ((e = cudaGetLastError()) != cudaSuccess) return fail(cfail(e, "indicator"));
    if (int rc = dgc_laplace_spd_apply(h, v, w1, s)) return fail(rc);
    if (int rc = ipdg_block_jacobi_apply(h, w1, w2, s)) return fail(rc);
    dgk::k_coarse_axpy<<<grid1(n), 256, 0, s>>>(n, v, om, w2, w1, 0);   // w1 = P v
    if (int rc = dgc_laplace_spd_apply(h, w1, w2, s)) return fail(rc);   // w2 = S P v
    if (int rc = ipdg_block_jacobi_apply(h, w2, v, s)) return fail(rc);  // v = Binv S P v
    if (int rc = dgc_laplace_spd_apply(h, v, w1, s)) return fail(rc);    // w1 = S Binv S P v
    dgk::k_coarse_axpy<<<grid1(n), 256, 0, s>>>(n, w2, om, w1, w1, 0);  // w1 = P^T S P v
    if ((e = cudaGetLastError()) != cudaSuccess) return fail(cfail(e, "probe"));
    if (!download(w1)) return fail(cfail(e, "download"));
    for (int k = 0; k < K; ++k) {
      int a = -1;
      for (int t : touch[k])
        if (color[t] == col) a = t;
      if (a < 0) continue;
      double sk = 0.0;
      for (int j = 0; j < Np; ++j) sk += hv[(size_t)k * NpP + j];
      Ac[(size_t)c->agg[k] * nagg + a] += sk;
    }
  }
  for (int i = 0; i < nagg; ++i)
    for (int j = i + 1; j < nagg; ++j) {
      const double m = 0.5 * (Ac[(size_t)i * nagg + j] + Ac[(size_t)j * nagg + i]);
      Ac[(size_t)i * nagg + j] = Ac[(size_t)j * nagg + i] = m;
    }
  for (int i = 0; i < nagg; ++i)
    if (!(Ac[(size_t)i * nagg + i] > 0.0))
      return fail(set_error(DGC_ERR_DEVICE, "coarse matrix has a non-positive diagonal"));
  // all-Neumann without shift: S 1 = 0, so P 1 = 1 and A_c has the coarse constants
  // as null space.  A_c + a 1 1^T / nagg (a = mean diagonal) is regular and acts as
  // A_c's pseudo-inverse on the zero-sum right-hand sides a consistent residual gives.
  if (!h->desc.dirichlet && c->shift == 0.0) {
    double a = 0.0;
    for (int i = 0; i < nagg; ++i) a += Ac[(size_t)i * nagg + i];
    a /= (double)nagg * nagg;
    for (double& v : Ac) v += a;
  }
  if ((e = cudaMemcpyAsync(c->d_ainv, Ac.data(), Ac.size() * 8, cudaMemcpyHostToDevice, s)) != cudaSuccess)
    return fail(cfail(e, "upload"));
  // Gauss-Jordan in place (SPD: no pivoting); c->d_rc holds the pivot column
  const dim3 eg((nagg + 127) / 128, nagg);
  for (int i = 0; i < nagg; ++i) {
    dgk::k_gj_col<<<(nagg + 127) / 128, 128, 0, s>>>(nagg, i, c->d_ainv, c->d_rc);
    dgk::k_gj_row<<<(nagg + 127) / 128, 128, 0, s>>>(nagg, i, c->d_ainv, c->d_rc);
    dgk::k_gj_elim<<<eg, 128, 0, s>>>(nagg, i, c->d_ainv, c->d_rc);
  }
  if ((e = cudaMalloc(&c->d_ainv32, (size_t)nagg * nagg * 4)) != cudaSuccess ||
      (e = cudaMalloc(&c->d_rc32, (size_t)nagg * 4)) != cudaSuccess)
    return fail(cfail(e, "allocation"));
  dgk::k_coarse_to_f32<<<grid1((int64_t)nagg * nagg), 256, 0, s>>>((int64_t)nagg * nagg, c->d_ainv, c->d_ainv32);
  if ((e = cudaGetLastError()) != cudaSuccess || (e = cudaStreamSynchronize(s)) != cudaSuccess)
    return fail(cfail(e, "inversion"));
  h->launches += 3 * (int64_t)ncol + 3 * (int64_t)nagg + 1;
  cudaFree(d_color);
  h->coarse = c;
  return DGC_OK;
}

int dgc::coarse_apply(dgc_handle_s* h, const double* r, const double* binv_r, double* z, bool add, bool fp32,
                      cudaStream_t s, bool binv_r32_ready, const CoarseDots* dots) {
  CoarseSpace* c = h->coarse;
  if (!c) return set_error(DGC_ERR_ARG, "no coarse space: call dgc_coarse_build first");
  if (c->shift != ipdg_shift(h)) return set_error(DGC_ERR_ARG, "the shift changed since dgc_coarse_build");
  const int64_t n = (int64_t)h->K * h->NpP;
  double *w0 = c->d_w[0], *w1 = c->d_w[1], *w2 = c->d_w[2];
  float *f0 = c->d_f[0], *f1 = c->d_f[1];
  const double om = c->omega;
  if (fp32) {
    // the FP32 path keeps the operator's inputs and outputs in FP32 between
    // kernels: each conversion happens once, inside the kernel that produces
    // or consumes the value (same values as converting through FP64 vectors)
    if (!binv_r) {
      if (int rc = ipdg_block_jacobi_apply_f32(h, r, nullptr, w0, f0, s)) return rc;
      binv_r = w0;
    } else if (!binv_r32_ready) {
      dgk::k_coarse_to_f32<<<grid1(n), 256, 0, s>>>(n, binv_r, f0);
      ++h->launches;
    }
    // P^T r = P0^T (r - w S Binv r)
    if (int rc = ipdg_spd_apply_f32(h, f0, f1, s)) return rc;
    dgk::k_coarse_axpy_z32<<<grid1(n), 256, 0, s>>>(n, r, om, f1, w1);
    dgk::k_coarse_restrict<<<(c->nagg * 32 + 255) / 256, 256, 0, s>>>(c->nagg, h->NpP, h->Np, c->d_ptr, c->d_cells,
                                                                    w1, c->d_rc, c->d_rc32);
    dgk::k_coarse_gemv32<<<(c->nagg * 32 + 255) / 256, 256, 0, s>>>(c->nagg, c->d_ainv32, c->d_rc32, c->d_xc);
    // y = P0 x_c;  z (+)= y - w Binv S y
    dgk::k_coarse_prolong<<<grid1(n), 256, 0, s>>>(n, h->NpP, h->Np, c->d_agg, c->d_xc, 0, w1, f0);
    CKC(cudaGetLastError(), "apply");
    if (int rc = ipdg_spd_apply_f32(h, f0, f1, s)) return rc;
    if (int rc = ipdg_block_jacobi_apply_f32(h, nullptr, f1, w0, nullptr, s)) return rc;
    if (dots && add) {
      CKC(cudaMemsetAsync(dots->out, 0, 3 * 8, s), "dots");
      dgk::k_coarse_axpy_dots<<<dots->grid, 256, 0, s>>>(n, w1, om, w0, z, dots->r, dots->q, dots->out);
    } else {
      dgk::k_coarse_axpy<<<grid1(n), 256, 0, s>>>(n, w1, om, w0, z, add ? 1 : 0);
    }
    CKC(cudaGetLastError(), "apply");
    h->launches += 5;
    return DGC_OK;
  }
  // P^T r = P0^T (r - w S Binv r)
  if (!binv_r) {
    if (int rc = ipdg_block_jacobi_apply(h, r, w0, s)) return rc;
    binv_r = w0;
  }
  if (int rc = dgc_laplace_spd_apply(h, binv_r, w1, s)) return rc;
  dgk::k_coarse_axpy<<<grid1(n), 256, 0, s>>>(n, r, om, w1, w1, 0);
  dgk::k_coarse_restrict<<<(c->nagg * 32 + 255) / 256, 256, 0, s>>>(c->nagg, h->NpP, h->Np, c->d_ptr, c->d_cells, w1,
                                                                  c->d_rc, nullptr);
  dgk::k_coarse_gemv<<<(c->nagg * 32 + 255) / 256, 256, 0, s>>>(c->nagg, c->d_ainv, c->d_rc, c->d_xc);
  // y = P0 x_c;  z (+)= y - w Binv S y
  dgk::k_coarse_prolong<<<grid1(n), 256, 0, s>>>(n, h->NpP, h->Np, c->d_agg, c->d_xc, 0, w1, nullptr);
  CKC(cudaGetLastError(), "apply");
  if (int rc = dgc_laplace_spd_apply(h, w1, w2, s)) return rc;
  if (int rc = ipdg_block_jacobi_apply(h, w2, w0, s)) return rc;
  dgk::k_coarse_axpy<<<grid1(n), 256, 0, s>>>(n, w1, om, w0, z, add ? 1 : 0);
  CKC(cudaGetLastError(), "apply");
  h->launches += 5;
  return DGC_OK;
}

int dgc::two_level_pcg(dgc_handle_s* h, double* x, double* r, double tol2, int maxit, int* iterations, bool op32,
                       cudaStream_t s) {
  CoarseSpace* c = h->coarse;
  if (!c) return set_error(DGC_ERR_ARG, "no coarse space: call dgc_coarse_build first");
  const int64_t n = (int64_t)h->K * h->NpP;
  if (!c->d_pcg[0]) {
    for (double*& v : c->d_pcg) {
      CKC(cudaMalloc(&v, n * 8), "allocation");
      CKC(cudaMemset(v, 0, n * 8), "clear");
    }
    CKC(cudaMalloc(&c->d_dots, 4 * 8), "allocation");
    CKC(cudaMalloc(&c->d_sc, 8 * 8), "allocation");
    CKC(cudaMallocHost(&c->h_sc, 8 * 8), "allocation");
  }
  double *z = c->d_pcg[0], *p = c->d_pcg[1], *q = c->d_pcg[2];
  double *t = c->d_dots, *sc = c->d_sc;
  const int gd = grid1(n);
  // reductions end in one atomic per block on the same few addresses: 2 blocks per SM
  const int gr = std::max(1, std::min(gd, 2 * h->sm_count));
  // dots of up to three pairs into t, left on the device
  auto dots = [&](dgk::Dot3 d) -> int {
    CKC(cudaMemsetAsync(t, 0, 3 * 8, s), "dots");
    dgk::k_coarse_dots<<<gr, 256, 0, s>>>(n, d, t);
    CKC(cudaGetLastError(), "dots");
    ++h->launches;
    return DGC_OK;
  };
  // all-Neumann without shift: the constants are S's null space.  Rounding in the
  // FP32 smoothing leaks a little of them into the coarse term; unchecked, x drifts
  // along them until S x loses its accuracy, so z is kept at zero mean.
  const bool singular = !h->desc.dirichlet && c->shift == 0.0;
  // with `fused`, the preconditioner's last kernel also forms (r.r, z.r, z.q)
  // in t (not for the singular system, whose z changes once more afterwards)
  auto precondition = [&](bool fused) -> int {  // z = Binv r + P A_c^-1 P^T r, Binv and the coarse term in FP32
    if (int rc = ipdg_block_jacobi_apply_f32(h, r, nullptr, z, c->d_f[0], s)) return rc;
    const CoarseDots cd{t, r, q, gr};
    if (int rc = coarse_apply(h, r, z, z, true, true, s, true, fused && !singular ? &cd : nullptr)) return rc;
    if (singular) {
      CKC(cudaMemsetAsync(t + 3, 0, 8, s), "mean");
      dgk::k_coarse_valid_sum<<<gr, 256, 0, s>>>(n, h->NpP, h->Np, z, t + 3);
      dgk::k_coarse_sub_mean<<<gd, 256, 0, s>>>(n, h->NpP, h->Np, t + 3, (double)h->K * h->Np, z);
      CKC(cudaGetLastError(), "mean");
      h->launches += 2;
    }
    return DGC_OK;
  };
  // q = S p in FP64, or through the FP32 kernels (the caller refines on the FP64 residual)
  // (FP32: the direction kernel leaves an FP32 copy of p in the first FP32
  // work vector, which nothing else writes before this apply reads it)
  float* p32 = op32 ? c->d_f[0] : nullptr;
  auto apply = [&]() -> int {
    if (!op32) return dgc_laplace_spd_apply(h, p, q, s);
    if (int rc = ipdg_spd_apply_f32(h, p32, c->d_f[1], s)) return rc;
    // q back in FP64, with t[0] = p.q for the step
    CKC(cudaMemsetAsync(t, 0, 3 * 8, s), "dots");
    dgk::k_coarse_to_f64_dot<<<gr, 256, 0, s>>>(n, c->d_f[1], q, p, t);
    CKC(cudaGetLastError(), "apply");
    h->launches += 1;
    return DGC_OK;
  };
  // read r.r and the stop flag (synchronises the stream)
  auto check = [&](double* rr, bool* stop) -> int {
    CKC(cudaMemcpyAsync(c->h_sc, sc, 8 * 8, cudaMemcpyDeviceToHost, s), "scalars");
    CKC(cudaStreamSynchronize(s), "scalars");
    *rr = c->h_sc[3];
    *stop = c->h_sc[6] != 0.0;
    if (!std::isfinite(*rr)) return set_error(DGC_ERR_NOT_CONVERGED, "two-level PCG: non-finite residual");
    return DGC_OK;
  };
  CKC(cudaMemsetAsync(sc, 0, 8 * 8, s), "scalars");
  if (int rc = precondition(false)) return rc;
  if (int rc = dots({{r, z, nullptr}, {r, r, nullptr}})) return rc;
  dgk::k_coarse_dir_dev<<<gd, 256, 0, s>>>(n, z, p, sc, t, 0, 0, 1, p32);  // p = z, sc[0] = z.r, sc[3] = r.r
  CKC(cudaGetLastError(), "start");
  double rr = 0.0;
  bool stop = false;
  if (int rc = check(&rr, &stop)) return rc;
  // the host looks at r.r every kCheck iterations: the kernels in between queue
  // without a round trip
  constexpr int kCheck = 8;
  int it = 0;
  while (rr > tol2 && !stop && it < maxit) {
    const int cur = it & 1;
    if (int rc = apply()) return rc;
    if (!op32)  // the FP32 apply forms p.q while it converts q
      if (int rc = dots({{p, nullptr, nullptr}, {q, nullptr, nullptr}})) return rc;
    dgk::k_coarse_step_dev<<<gd, 256, 0, s>>>(n, p, q, x, r, sc, t, cur);
    if (int rc = precondition(true)) return rc;
    if (singular)
      if (int rc = dots({{r, z, z}, {r, r, q}})) return rc;
    dgk::k_coarse_dir_dev<<<gd, 256, 0, s>>>(n, z, p, sc, t, cur, cur ^ 1, 0, p32);
    CKC(cudaGetLastError(), "update");
    h->launches += 2;
    ++it;
    if (it % kCheck == 0 || it == maxit)
      if (int rc = check(&rr, &stop)) return rc;
  }
  *iterations = it;
  return DGC_OK;
}

extern "C" int dgc_coarse_apply(dgc_handle h, const double* r, double* z, int precision, void* stream) {
  if (!h || !r || !z || r == z) return set_error(DGC_ERR_ARG, "r and z must be distinct, non-null buffers");
  if (precision != DGC_F64 && precision != DGC_F32) return set_error(DGC_ERR_ARG, "precision must be F64 or F32");
  return coarse_apply(h, r, nullptr, z, false, precision == DGC_F32, static_cast<cudaStream_t>(stream));
}

extern "C" int dgc_coarse_info(dgc_handle h, int32_t* agg, int* num_aggregates, int* num_colors, double* omega) {
  if (!h) return set_error(DGC_ERR_ARG, "null handle");
  if (!h->coarse) return set_error(DGC_ERR_ARG, "no coarse space: call dgc_coarse_build first");
  if (agg) std::copy(h->coarse->agg.begin(), h->coarse->agg.end(), agg);
  if (num_aggregates) *num_aggregates = h->coarse->nagg;
  if (num_colors) *num_colors = h->coarse->ncolors;
  if (omega) *omega = h->coarse->omega;
  return DGC_OK;
}
