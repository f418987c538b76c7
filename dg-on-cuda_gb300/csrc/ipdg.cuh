// ipdg.cuh -- matrix-free laplace_2d (strong-form LDG/IPDG) and the fused
// kernels of the block-Jacobi preconditioned CG that solves with it.
//
// Restates src/laplace_2d.h:130-251 (apply_homogeneous) as two passes over
// element tiles:
//   grad pass: q = (Dx u, Dy u) - LIFT(n du faceJ / 2) / J,
//              du = u- - u+ (interior), 2 u- (Dirichlet face), 0 (Neumann face)
//   div pass:  A u = Dx qx + Dy qy - LIFT((n.[q] + 2 tau du) faceJ / 2) / J,
//              n.[q] = (q- - q+).n (interior), 0 (Dirichlet), 2 q-.n (Neumann)
// The reference penalty is tau = 1 (laplace_2d.h:244); the per-face tau array
// carries either 1 or (N+1)^2 / h_f.  The SPD form used by CG is
// S u = -J_k M (A u)_k (mass-weighted, symmetric positive definite for
// Dirichlet problems).
//
// PCG fusion (one CG iteration = three launches, scalars in device memory):
//   grad  : p = z + beta p_old (beta = rz[i] / rz[i-1]), q = grad(p)
//   div   : Ap = S p, pAp = p.Ap
//   update: alpha = rz[i] / pAp; x += alpha p; r -= alpha Ap;
//           z = Binv r (block Jacobi, symmetric blocks); rz[i+1] = r.z, rr[i+1] = r.r
#pragma once

#include "common.cuh"

namespace dgk {

enum IpdgGradMode : int { GRAD_PLAIN = 0, GRAD_PCG = 1 };
enum IpdgDivMode : int { DIV_LAPLACE = 0, DIV_SPD = 1, DIV_SPD_DOT = 2, DIV_RESID = 3 };

// device-resident CG scalars; slot = iteration mod 3
struct CgScalars {
  double rz[3];
  double rr[3];
  double pAp;
  double bb;        // ||b||^2 (of the system being solved)
  double tol2;      // stop when rr <= tol2 * bb
  int done;         // set once converged (1) or out of iterations (2); later kernels become no-ops
  int iters;        // completed iterations
  int maxit;        // iteration budget of this solve
  int pad;
};

struct IpdgParams {
  int K;
  int dirichlet;
  const void* geom;     // [K][16] kernel geometry records, in R (slot 4 = -1/J, 14 = -J)
  const int4* nbr;      // [K]
  const void* tau;      // [K][4] penalty per face, in R
  const void* mats;     // strong-form DrT | DsT | LT (R)
  const void* mass;     // M (Np x Np, R), symmetric
  // grad pass
  const void* u;        // input u (GRAD_PLAIN) or z (GRAD_PCG)
  void* p;              // GRAD_PCG: new search direction p (written); update: p (read)
  const void* p_old;    // GRAD_PCG: previous search direction (a different buffer)
  void* qx;
  void* qy;
  // div pass
  const void* du_src;   // field whose jumps enter the penalty (u or p)
  void* out;            // A u | S u | residual r
  const void* b;        // DIV_RESID: right-hand side
  // update
  void* x;
  void* r;
  void* z;
  const void* Ap;
  const void* binv;     // [K][BSTR] symmetric block inverses
  // register-blocked FP32 kernels (ipdg_blk.cuh)
  const void* mats_blk; // rows Dr^T | Ds^T | LIFT^T (strong form), padded to NpP columns
  const void* mass_blk; // rows of M, padded to NpP columns
  const void* binv_pk;  // [K][PK] packed upper triangles of the block inverses
  const uint8_t* bcdir; // per boundary node: 1 Dirichlet, 0 Neumann (NULL: `dirichlet` everywhere)
  double shift;         // SPD modes: S = -J M (A - shift I) (Helmholtz-type operators; 0 = laplace)
  CgScalars* cg;
  double* dot_out;      // DIV_SPD_DOT / DIV_RESID: accumulated dot product
  int slot;             // iteration slot (i mod 3)
  int first;            // first iteration: beta = 0
  int* status;
};

template <typename R, int N>
struct IpdgConfig {
  using O = Order<N>;
  static constexpr int kThreads = 256;
  static constexpr int TE = (kThreads / O::Np) > 0 ? (kThreads / O::Np) : 1;
  static constexpr int kD = (O::Np * O::Np + 3) / 4 * 4;
  static constexpr int kL = (O::Nface * O::Np + 3) / 4 * 4;
  static constexpr uint32_t kMatBytes = (2 * kD + kL) * sizeof(R);
  static constexpr uint32_t kMassBytes = kD * sizeof(R);
  static constexpr int BSTR = kD;  // per-element block stride of Binv
  // shared memory layout (bytes)
  static constexpr uint32_t oBar = 0;
  static constexpr uint32_t oMats = 16;
  static constexpr uint32_t oMass = oMats + kMatBytes;
  static constexpr uint32_t oA = oMass + kMassBytes;                 // tile field A (u / qx / x)
  static constexpr uint32_t oB = oA + TE * O::NpP * sizeof(R);       // tile field B (p_old / qy / p)
  static constexpr uint32_t oC = oB + TE * O::NpP * sizeof(R);       // tile field C (u for jumps / r)
  static constexpr uint32_t oD = oC + TE * O::NpP * sizeof(R);       // tile field D (b / Ap)
  static constexpr uint32_t oGeom = oD + TE * O::NpP * sizeof(R);
  static constexpr uint32_t oNbr = oGeom + TE * 16 * sizeof(R);
  static constexpr uint32_t oTau = oNbr + TE * 16;
  static constexpr uint32_t oF = oTau + TE * 4 * sizeof(R);          // face work: 2 x TE x Nface
  static constexpr uint32_t oW = oF + 2 * TE * O::Nface * sizeof(R); // node work: TE x NpP
  static constexpr uint32_t oRed = (oW + TE * O::NpP * sizeof(R) + 15) / 16 * 16;  // 2 x 8 warps doubles
  static constexpr uint32_t kSmem = oRed + 16 * sizeof(double);
};

__device__ __forceinline__ double block_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += red[i];
  return s;  // valid in thread 0
}

template <typename R, int N>
struct IpdgTile {
  using O = Order<N>;
  using C = IpdgConfig<R, N>;
  static constexpr int Np = O::Np, NpP = O::NpP, Nfp = O::Nfp, NFACE = O::Nface, TE = C::TE;
  unsigned char* smem;
  uint64_t* bar;
  uint32_t phase;
  __device__ R* A() const { return reinterpret_cast<R*>(smem + C::oA); }
  __device__ R* B() const { return reinterpret_cast<R*>(smem + C::oB); }
  __device__ R* Cc() const { return reinterpret_cast<R*>(smem + C::oC); }
  __device__ R* Dd() const { return reinterpret_cast<R*>(smem + C::oD); }
  __device__ R* G() const { return reinterpret_cast<R*>(smem + C::oGeom); }
  __device__ int4* Nb() const { return reinterpret_cast<int4*>(smem + C::oNbr); }
  __device__ R* Tau() const { return reinterpret_cast<R*>(smem + C::oTau); }
  __device__ R* F0() const { return reinterpret_cast<R*>(smem + C::oF); }
  __device__ R* F1() const { return reinterpret_cast<R*>(smem + C::oF) + TE * NFACE; }
  __device__ R* W() const { return reinterpret_cast<R*>(smem + C::oW); }
  __device__ double* Red() const { return reinterpret_cast<double*>(smem + C::oRed); }
  __device__ const R* DrT() const { return reinterpret_cast<const R*>(smem + C::oMats); }
  __device__ const R* DsT() const { return DrT() + C::kD; }
  __device__ const R* LT() const { return DrT() + 2 * C::kD; }
  __device__ const R* M() const { return reinterpret_cast<const R*>(smem + C::oMass); }

  // Load matrices (and mass matrix) once per CTA.
  __device__ bool init(const void* mats, const void* mass, int* status) {
    bar = reinterpret_cast<uint64_t*>(smem + C::oBar);
    phase = 0;
    if (threadIdx.x == 0) {
      mbar_init(bar, 1);
      fence_barrier_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      mbar_arrive_expect_tx(bar, C::kMatBytes + (mass ? C::kMassBytes : 0));
      bulk_g2s(smem + C::oMats, mats, C::kMatBytes, bar);
      if (mass) bulk_g2s(smem + C::oMass, mass, C::kMassBytes, bar);
    }
    // the barrier is re-armed by the first load(): every thread must have
    // observed this phase first (a fast tile copy could otherwise complete the
    // next phase before a slow warp polls this one); the AND also makes a
    // timed-out wait exit the whole CTA
    const bool ok = __syncthreads_and(mbar_wait(bar, phase, status));
    phase ^= 1;
    return ok;
  }

  // Bulk-load up to four node fields plus geometry / neighbours / tau of a tile.
  __device__ bool load(int k0, int ne, const R* a, const R* b, const R* c, const R* d, const void* geom,
                       const int4* nbr, const void* tau, int* status) {
    if (threadIdx.x == 0) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      const uint32_t bf = ne * NpP * sizeof(R);
      uint32_t tot = ne * 16 * sizeof(R) + ne * 16 + (tau ? ne * 4 * sizeof(R) : 0);
      tot += (a ? bf : 0) + (b ? bf : 0) + (c ? bf : 0) + (d ? bf : 0);
      mbar_arrive_expect_tx(bar, tot);
      if (a) bulk_g2s(A(), a + (size_t)k0 * NpP, bf, bar);
      if (b) bulk_g2s(B(), b + (size_t)k0 * NpP, bf, bar);
      if (c) bulk_g2s(Cc(), c + (size_t)k0 * NpP, bf, bar);
      if (d) bulk_g2s(Dd(), d + (size_t)k0 * NpP, bf, bar);
      bulk_g2s(G(), static_cast<const R*>(geom) + (size_t)k0 * 16, ne * 16 * sizeof(R), bar);
      bulk_g2s(Nb(), nbr + k0, ne * 16, bar);
      if (tau) bulk_g2s(Tau(), static_cast<const R*>(tau) + (size_t)k0 * 4, ne * 4 * sizeof(R), bar);
    }
    const bool ok = __syncthreads_and(mbar_wait(bar, phase, status));
    phase ^= 1;
    return ok;
  }
};

template <typename R, int N>
__device__ __forceinline__ int nb_of(const int4& n, int f) { return f == 0 ? n.x : (f == 1 ? n.y : n.z); }

// condition type of node d of boundary face `nb` (< 0): the per-node flags when
// given (the reference's is_dirichlet(x, y)), else the handle's uniform type
template <int N>
__device__ __forceinline__ bool bc_dirichlet(const IpdgParams& p, int nb, int d) {
  return p.bcdir ? p.bcdir[(size_t)(-1 - nb) * (N + 1) + d] != 0 : p.dirichlet != 0;
}

// ---------------------------------------------------------------- grad pass
template <typename R, int N, int MODE>
__global__ void __launch_bounds__(256) ipdg_grad_kernel(const IpdgParams p) {
  using T = IpdgTile<R, N>;
  using C = IpdgConfig<R, N>;
  constexpr int Np = T::Np, NpP = T::NpP, Nfp = T::Nfp, NFACE = T::NFACE, TE = T::TE;
  extern __shared__ __align__(128) unsigned char smem[];
  if (MODE == GRAD_PCG && p.cg->done) return;
  T t{smem};
  // beta = rz_new / rz_old: one FP64 division per CTA, broadcast through shared
  // memory (t.init's barrier publishes it)
  __shared__ R s_beta;
  if (threadIdx.x == 0) {
    s_beta = (R)0;
    if (MODE == GRAD_PCG && !p.first) {
      const int s = p.slot, sp = (s + 2) % 3;
      s_beta = (R)(p.cg->rz[s] / p.cg->rz[sp]);
    }
  }
  if (!t.init(p.mats, nullptr, p.status)) return;
  const R* u_in = static_cast<const R*>(p.u);
  R* pv = static_cast<R*>(p.p);
  const R* pold = static_cast<const R*>(p.p_old);
  const R beta = s_beta;
  if (MODE == GRAD_PCG && blockIdx.x == 0 && threadIdx.x == 0) p.cg->pAp = 0.0;
  const int ntiles = (p.K + TE - 1) / TE;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int k0 = tile * TE, ne = min(TE, p.K - k0);
    // A = u (or z), B = p_old
    if (!t.load(k0, ne, u_in, MODE == GRAD_PCG ? pold : nullptr, nullptr, nullptr, p.geom, p.nbr, nullptr, p.status))
      return;
    R* sU = t.A();
    if (MODE == GRAD_PCG) {
      // p = z + beta p_old on the tile; write p
      for (int it = threadIdx.x; it < ne * NpP; it += blockDim.x) {
        const R v = sU[it] + beta * t.B()[it];
        sU[it] = v;
        pv[(size_t)k0 * NpP + it] = v;
      }
      __syncthreads();
    }
    // jumps on face nodes
    for (int it = threadIdx.x; it < ne * NFACE; it += blockDim.x) {
      const int e = it / NFACE, fm = it - e * NFACE, f = fm / Nfp, d = fm - f * Nfp;
      const R* g = t.G() + e * 16;
      const int nb = nb_of<R, N>(t.Nb()[e], f);
      const R um = sU[e * NpP + fmask<N>(f, d)];
      R du;
      if (nb >= 0) {
        const int kn = nb >> 2, nd2 = fmask<N>(nb & 3, Nfp - 1 - d);
        R up;
        if (kn >= k0 && kn < k0 + ne) up = sU[(kn - k0) * NpP + nd2];
        else if (MODE == GRAD_PCG)
          up = __ldg(u_in + (size_t)kn * NpP + nd2) + beta * __ldg(pold + (size_t)kn * NpP + nd2);
        else up = __ldg(u_in + (size_t)kn * NpP + nd2);
        du = um - up;
      } else {
        du = bc_dirichlet<N>(p, nb, d) ? (R)2 * um : (R)0;
      }
      const R tl = du * (R)g[5 + f] / (R)2;
      t.F0()[e * NFACE + fm] = (R)g[8 + f] * tl;
      t.F1()[e * NFACE + fm] = (R)g[11 + f] * tl;
    }
    __syncthreads();
    if (threadIdx.x < ne * Np) {
      const int e = threadIdx.x / Np, i = threadIdx.x - e * Np;
      const R* ue = sU + e * NpP;
      R ur = 0, us = 0, lx = 0, ly = 0;
#pragma unroll 5
      for (int j = 0; j < Np; ++j) {
        const R v = ue[j];
        ur = fma(t.DrT()[j * Np + i], v, ur);
        us = fma(t.DsT()[j * Np + i], v, us);
      }
      const R* fx = t.F0() + e * NFACE;
      const R* fy = t.F1() + e * NFACE;
#pragma unroll 3
      for (int m = 0; m < NFACE; ++m) {
        const R l = t.LT()[m * Np + i];
        lx = fma(l, fx[m], lx);
        ly = fma(l, fy[m], ly);
      }
      const R* g = t.G() + e * 16;
      const R ilJ = g[4];  // -1/J
      const size_t o = (size_t)(k0 + e) * NpP + i;
      static_cast<R*>(p.qx)[o] = (R)g[0] * ur + (R)g[2] * us + ilJ * lx;
      static_cast<R*>(p.qy)[o] = (R)g[1] * ur + (R)g[3] * us + ilJ * ly;
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------- div pass
template <typename R, int N, int MODE>
__global__ void __launch_bounds__(256) ipdg_div_kernel(const IpdgParams p) {
  using T = IpdgTile<R, N>;
  constexpr int Np = T::Np, NpP = T::NpP, Nfp = T::Nfp, NFACE = T::NFACE, TE = T::TE;
  extern __shared__ __align__(128) unsigned char smem[];
  if (MODE == DIV_SPD_DOT && p.cg->done) return;
  T t{smem};
  const bool spd = MODE != DIV_LAPLACE;
  if (!t.init(p.mats, spd ? p.mass : nullptr, p.status)) return;
  if (MODE == DIV_SPD_DOT && blockIdx.x == 0 && threadIdx.x == 0) {
    const int s1 = (p.slot + 1) % 3;
    p.cg->rz[s1] = 0.0;
    p.cg->rr[s1] = 0.0;
  }
  const R* qx = static_cast<const R*>(p.qx);
  const R* qy = static_cast<const R*>(p.qy);
  const R* uj = static_cast<const R*>(p.du_src);
  double dot = 0.0;
  const int ntiles = (p.K + TE - 1) / TE;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int k0 = tile * TE, ne = min(TE, p.K - k0);
    if (!t.load(k0, ne, qx, qy, uj, MODE == DIV_RESID ? static_cast<const R*>(p.b) : nullptr, p.geom, p.nbr,
                p.tau, p.status))
      return;
    for (int it = threadIdx.x; it < ne * NFACE; it += blockDim.x) {
      const int e = it / NFACE, fm = it - e * NFACE, f = fm / Nfp, d = fm - f * Nfp;
      const R* g = t.G() + e * 16;
      const int nb = nb_of<R, N>(t.Nb()[e], f);
      const int nd = fmask<N>(f, d);
      const R nx = (R)g[8 + f], ny = (R)g[11 + f];
      const R qxm = t.A()[e * NpP + nd], qym = t.B()[e * NpP + nd], um = t.Cc()[e * NpP + nd];
      R dqn, du;
      if (nb >= 0) {
        const int kn = nb >> 2, nd2 = fmask<N>(nb & 3, Nfp - 1 - d);
        R qxp, qyp, up;
        if (kn >= k0 && kn < k0 + ne) {
          const int o = (kn - k0) * NpP + nd2;
          qxp = t.A()[o]; qyp = t.B()[o]; up = t.Cc()[o];
        } else {
          const size_t o = (size_t)kn * NpP + nd2;
          qxp = qx[o]; qyp = qy[o]; up = uj[o];
        }
        dqn = (qxm - qxp) * nx + (qym - qyp) * ny;
        du = um - up;
      } else if (bc_dirichlet<N>(p, nb, d)) {
        dqn = (R)0;
        du = (R)2 * um;
      } else {
        dqn = (R)2 * (qxm * nx + qym * ny);
        du = (R)0;
      }
      const R tau = (R)t.Tau()[e * 4 + f];
      t.F0()[e * NFACE + fm] = (dqn + (R)2 * tau * du) * (R)g[5 + f] / (R)2;
    }
    __syncthreads();
    R au = 0;
    int e = 0, i = 0;
    const bool act = threadIdx.x < ne * Np;
    if (act) {
      e = threadIdx.x / Np;
      i = threadIdx.x - e * Np;
      const R* xe = t.A() + e * NpP;
      const R* ye = t.B() + e * NpP;
      R xr = 0, xs = 0, yr = 0, ys = 0, lf = 0;
#pragma unroll 5
      for (int j = 0; j < Np; ++j) {
        const R dr = t.DrT()[j * Np + i], ds = t.DsT()[j * Np + i];
        xr = fma(dr, xe[j], xr);
        xs = fma(ds, xe[j], xs);
        yr = fma(dr, ye[j], yr);
        ys = fma(ds, ye[j], ys);
      }
      const R* fe = t.F0() + e * NFACE;
#pragma unroll 3
      for (int m = 0; m < NFACE; ++m) lf = fma(t.LT()[m * Np + i], fe[m], lf);
      const R* g = t.G() + e * 16;
      au = ((R)g[0] * xr + (R)g[2] * xs) + ((R)g[1] * yr + (R)g[3] * ys) + g[4] * lf;  // g[4] = -1/J
    }
    if (!spd) {
      if (act) static_cast<R*>(p.out)[(size_t)(k0 + e) * NpP + i] = au;
    } else {
      // S u = -J M (A u): the mass matrix mixes the element's nodes
      if (act) t.W()[e * NpP + i] = au - (R)p.shift * t.Cc()[e * NpP + i];  // (A - shift I) u
      __syncthreads();
      if (act) {
        const R* we = t.W() + e * NpP;
        R s = 0;
#pragma unroll 5
        for (int j = 0; j < Np; ++j) s = fma(t.M()[j * Np + i], we[j], s);
        const R* g = t.G() + e * 16;
        s *= g[14];  // -J
        const size_t o = (size_t)(k0 + e) * NpP + i;
        if (MODE == DIV_RESID) {
          const R r = t.Dd()[e * NpP + i] - s;
          static_cast<R*>(p.out)[o] = r;
          dot += (double)r * (double)r;
        } else {
          static_cast<R*>(p.out)[o] = s;
          if (MODE == DIV_SPD_DOT) dot += (double)t.Cc()[e * NpP + i] * (double)s;
        }
      }
    }
    // padded output nodes are written as 0 (callers sum over whole vectors)
    constexpr int kPad = NpP - Np;
    if constexpr (kPad > 0)
      for (int q = threadIdx.x; q < ne * kPad; q += blockDim.x)
        static_cast<R*>(p.out)[(size_t)(k0 + q / kPad) * NpP + Np + q % kPad] = (R)0;
    __syncthreads();
  }
  if (MODE == DIV_SPD_DOT || MODE == DIV_RESID) {
    const double s = block_sum(dot, t.Red());
    if (threadIdx.x == 0) atomicAdd(MODE == DIV_SPD_DOT ? &p.cg->pAp : p.dot_out, s);
  }
}

// ---------------------------------------------------------------- CG update
template <typename R, int N>
__global__ void __launch_bounds__(256) pcg_update_kernel(const IpdgParams p) {
  using O = Order<N>;
  constexpr int Np = O::Np, NpP = O::NpP;
  constexpr int TE = IpdgConfig<R, N>::TE, BSTR = IpdgConfig<R, N>::BSTR;
  __shared__ R sr[TE * NpP];
  __shared__ double red[16];
  __shared__ R s_alpha;
  CgScalars* cg = p.cg;
  if (cg->done) return;
  const int s = p.slot, s1 = (s + 1) % 3;
  if (threadIdx.x == 0) s_alpha = (R)(cg->rz[s] / cg->pAp);  // one FP64 division per CTA
  __syncthreads();
  const R alpha = s_alpha;
  R* x = static_cast<R*>(p.x);
  R* r = static_cast<R*>(p.r);
  R* z = static_cast<R*>(p.z);
  const R* pv = static_cast<const R*>(p.p);
  const R* Ap = static_cast<const R*>(p.Ap);
  const R* binv = static_cast<const R*>(p.binv);
  double rz = 0.0, rr = 0.0;
  const int ntiles = (p.K + TE - 1) / TE;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int k0 = tile * TE, ne = min(TE, p.K - k0);
    const bool act = threadIdx.x < ne * Np;
    int e = 0, i = 0;
    R rv = 0;
    if (act) {
      e = threadIdx.x / Np;
      i = threadIdx.x - e * Np;
      const size_t o = (size_t)(k0 + e) * NpP + i;
      x[o] = x[o] + alpha * pv[o];
      rv = r[o] - alpha * Ap[o];
      r[o] = rv;
      sr[e * NpP + i] = rv;
      rr += (double)rv * (double)rv;
    }
    __syncthreads();
    if (act) {
      const R* be = binv + (size_t)(k0 + e) * BSTR;
      const R* re = sr + e * NpP;
      R zv = 0;
#pragma unroll 5
      for (int j = 0; j < Np; ++j) zv = fma(__ldg(be + j * Np + i), re[j], zv);
      z[(size_t)(k0 + e) * NpP + i] = zv;
      rz += (double)rv * (double)zv;
    }
    __syncthreads();
  }
  const double a = block_sum(rz, red);
  const double b = block_sum(rr, red);
  if (threadIdx.x == 0) {
    atomicAdd(&cg->rz[s1], a);
    atomicAdd(&cg->rr[s1], b);
  }
}

// Block-Jacobi preconditioner application z = Binv r (no scalars): used to
// start CG.  Also accumulates r.z and r.r into slot 0.
template <typename R, int N>
__global__ void __launch_bounds__(256) pcg_start_kernel(const IpdgParams p) {
  using O = Order<N>;
  constexpr int Np = O::Np, NpP = O::NpP;
  constexpr int TE = IpdgConfig<R, N>::TE, BSTR = IpdgConfig<R, N>::BSTR;
  __shared__ R sr[TE * NpP];
  __shared__ double red[16];
  const R* r = static_cast<const R*>(p.r);
  R* z = static_cast<R*>(p.z);
  const R* binv = static_cast<const R*>(p.binv);
  double rz = 0.0, rr = 0.0;
  const int ntiles = (p.K + TE - 1) / TE;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int k0 = tile * TE, ne = min(TE, p.K - k0);
    const bool act = threadIdx.x < ne * Np;
    int e = 0, i = 0;
    R rv = 0;
    if (act) {
      e = threadIdx.x / Np;
      i = threadIdx.x - e * Np;
      rv = r[(size_t)(k0 + e) * NpP + i];
      sr[e * NpP + i] = rv;
      rr += (double)rv * (double)rv;
    }
    __syncthreads();
    if (act) {
      const R* be = binv + (size_t)(k0 + e) * BSTR;
      R zv = 0;
#pragma unroll 5
      for (int j = 0; j < Np; ++j) zv = fma(__ldg(be + j * Np + i), sr[e * NpP + j], zv);
      z[(size_t)(k0 + e) * NpP + i] = zv;
      rz += (double)rv * (double)zv;
    }
    __syncthreads();
  }
  const double a = block_sum(rz, red);
  const double b = block_sum(rr, red);
  if (threadIdx.x == 0) {
    atomicAdd(&p.cg->rz[0], a);
    atomicAdd(&p.cg->rr[0], b);
  }
}

// ---------------------------------------------------------------- boundary data
// apply_inhomogeneous_as_rhs (src/laplace_2d.h:253-348): for each cell with a
// boundary face (one CTA of 64 threads each) adds to out
//   Dx qx + Dy qy - LIFT((hq + 2 tau gu) faceJ / 2) / J,
//   q = -LIFT(n gu faceJ / 2) / J,
// gu = g[b] at Dirichlet nodes (else 0), hq = h[b] at Neumann nodes (else 0).
template <typename R, int N>
__global__ void __launch_bounds__(64) ipdg_bc_rhs_kernel(const IpdgParams p, const int* __restrict__ cells,
                                                         const double* __restrict__ g, const double* __restrict__ h,
                                                         R* __restrict__ out) {
  using O = Order<N>;
  constexpr int Np = O::Np, NpP = O::NpP, Nfp = O::Nfp, NFACE = O::Nface;
  constexpr int kD = IpdgConfig<R, N>::kD;
  __shared__ R tx[NFACE], ty[NFACE], hq[NFACE], qx[Np], qy[Np];
  const int c = cells[blockIdx.x];
  const int t = threadIdx.x;
  const R* G = static_cast<const R*>(p.geom) + (size_t)c * 16;
  const R* tau = static_cast<const R*>(p.tau) + (size_t)c * 4;
  const R* DrT = static_cast<const R*>(p.mats);
  const R* DsT = DrT + kD;
  const R* LT = DrT + 2 * kD;
  const int4 n4 = p.nbr[c];
  for (int m = t; m < NFACE; m += blockDim.x) {
    const int f = m / Nfp, d = m - f * Nfp;
    const int nb = f == 0 ? n4.x : (f == 1 ? n4.y : n4.z);
    R v = 0, w = 0;
    if (nb < 0) {
      const size_t b = (size_t)(-1 - nb) * Nfp + d;
      const bool dir = bc_dirichlet<N>(p, nb, d);
      v = dir && g ? (R)g[b] : (R)0;
      w = !dir && h ? (R)h[b] : (R)0;
    }
    const R hf = G[5 + f] / (R)2;
    hq[m] = (w + (R)2 * tau[f] * v) * hf;
    tx[m] = G[8 + f] * v * hf;
    ty[m] = G[11 + f] * v * hf;
  }
  __syncthreads();
  const R nJ = G[4];  // -1/J
  if (t < Np) {
    R ax = 0, ay = 0;
    for (int m = 0; m < NFACE; ++m) {
      ax += LT[m * Np + t] * tx[m];
      ay += LT[m * Np + t] * ty[m];
    }
    qx[t] = nJ * ax;
    qy[t] = nJ * ay;
    if (p.qx) {  // kept for ipdg_bc_jump_kernel
      static_cast<R*>(p.qx)[(size_t)c * NpP + t] = nJ * ax;
      static_cast<R*>(p.qy)[(size_t)c * NpP + t] = nJ * ay;
    }
  }
  __syncthreads();
  if (t < Np) {
    R xr = 0, xs = 0, yr = 0, ys = 0, lf = 0;
    for (int j = 0; j < Np; ++j) {
      const R dr = DrT[j * Np + t], ds = DsT[j * Np + t];
      xr += dr * qx[j];
      xs += ds * qx[j];
      yr += dr * qy[j];
      ys += ds * qy[j];
    }
    for (int m = 0; m < NFACE; ++m) lf += LT[m * Np + t] * hq[m];
    out[(size_t)c * NpP + t] += (G[0] * xr + G[2] * xs) + (G[1] * yr + G[3] * ys) + nJ * lf;
  }
}

// The jumps of the lifted Dirichlet data q_d that apply_inhomogeneous_as_rhs
// leaves out (its second pass adds only boundary-face terms, laplace_2d.h:
// 310-348, where apply_homogeneous's dqN also holds the jumps of q across
// interior faces and 2 q.n on Neumann faces, :222-242).  q_d as stored by
// ipdg_bc_rhs_kernel in p.qx / p.qy (zero off the boundary cells); on each
// listed cell (a boundary cell or a face neighbour of one), one CTA of 64
// threads adds
//   -LIFT(dqN faceJ / 2) / J,  dqN = (q_d(c) - q_d(nb)).n on interior faces,
//   2 q_d(c).n on Neumann faces, 0 on Dirichlet faces.
template <typename R, int N>
__global__ void __launch_bounds__(64) ipdg_bc_jump_kernel(const IpdgParams p, const int* __restrict__ cells,
                                                          R* __restrict__ out) {
  using O = Order<N>;
  constexpr int Np = O::Np, NpP = O::NpP, Nfp = O::Nfp, NFACE = O::Nface;
  constexpr int kD = IpdgConfig<R, N>::kD;
  __shared__ R tl[NFACE];
  const int c = cells[blockIdx.x];
  const int t = threadIdx.x;
  const R* G = static_cast<const R*>(p.geom) + (size_t)c * 16;
  const R* LT = static_cast<const R*>(p.mats) + 2 * kD;
  const R* qx = static_cast<const R*>(p.qx);
  const R* qy = static_cast<const R*>(p.qy);
  const int4 n4 = p.nbr[c];
  for (int m = t; m < NFACE; m += blockDim.x) {
    const int f = m / Nfp, d = m - f * Nfp;
    const int nb = f == 0 ? n4.x : (f == 1 ? n4.y : n4.z);
    const size_t ia = (size_t)c * NpP + fmask<N>(f, d);
    const R nx = G[8 + f], ny = G[11 + f];
    R dqn;
    if (nb >= 0) {
      const size_t ib = (size_t)(nb >> 2) * NpP + fmask<N>(nb & 3, Nfp - 1 - d);
      dqn = (qx[ia] - qx[ib]) * nx + (qy[ia] - qy[ib]) * ny;
    } else {
      dqn = bc_dirichlet<N>(p, nb, d) ? (R)0 : (R)2 * (qx[ia] * nx + qy[ia] * ny);
    }
    tl[m] = dqn * (G[5 + f] / (R)2);
  }
  __syncthreads();
  if (t < Np) {
    R lf = 0;
    for (int m = 0; m < NFACE; ++m) lf += LT[m * Np + t] * tl[m];
    out[(size_t)c * NpP + t] += G[4] * lf;  // G[4] = -1/J
  }
}

// ---------------------------------------------------------------- diagonal blocks
// Column j of the diagonal block S_kk of the SPD form, one thread per (k, j):
// a unit vector on node j of cell k produces q on cell k (volume + its own
// jumps) and q on each interior neighbour (the neighbour's jump against it);
// the div pass of cell k then sees both.  Written transposed (= the block,
// which is symmetric) as blocks[k][j][i].
template <int N>
__global__ void ipdg_diag_blocks_kernel(int K, int dirichlet, const double* __restrict__ geom,
                                        const int4* __restrict__ nbr, const double* __restrict__ tau,
                                        const double* __restrict__ Dr, const double* __restrict__ Ds,
                                        const double* __restrict__ L, const double* __restrict__ M,
                                        double* __restrict__ blocks, int bstr) {
  using O = Order<N>;
  constexpr int Np = O::Np, Nfp = O::Nfp, NF = O::Nface;
  const int64_t gid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (gid >= (int64_t)K * Np) return;
  const int k = (int)(gid / Np), j = (int)(gid % Np);
  const double* g = geom + (size_t)k * 16;
  const int4 nb4 = nbr[k];
  const int nbv[3] = {nb4.x, nb4.y, nb4.z};
  double qx[Np], qy[Np], out[Np];
  // own q: D e_j - LIFT(n du faceJ/2)/J with du = e_j (x2 on Dirichlet faces)
  double tlx[NF], tly[NF];
  for (int f = 0; f < 3; ++f)
    for (int d = 0; d < Nfp; ++d) {
      const double du = (fmask<N>(f, d) == j) ? ((nbv[f] < 0) ? (dirichlet ? 2.0 : 0.0) : 1.0) : 0.0;
      tlx[f * Nfp + d] = g[8 + f] * du * g[5 + f] / 2.0;
      tly[f * Nfp + d] = g[11 + f] * du * g[5 + f] / 2.0;
    }
  for (int i = 0; i < Np; ++i) {
    double lx = 0.0, ly = 0.0;
    for (int m = 0; m < NF; ++m) {
      lx += L[i * NF + m] * tlx[m];
      ly += L[i * NF + m] * tly[m];
    }
    const double ur = Dr[i * Np + j], us = Ds[i * Np + j];
    qx[i] = g[0] * ur + g[2] * us - lx / g[4];
    qy[i] = g[1] * ur + g[3] * us - ly / g[4];
  }
  // div pass on cell k
  double tl[NF];
  for (int f = 0; f < 3; ++f) {
    const int nb = nbv[f];
    for (int d = 0; d < Nfp; ++d) {
      const int nd = fmask<N>(f, d);
      const double nx = g[8 + f], ny = g[11 + f];
      const double um = (nd == j) ? 1.0 : 0.0;
      double dqn, du;
      if (nb >= 0) {
        // neighbour's q at its face node facing (f, d): only its jump term
        const int kn = nb >> 2, fn = nb & 3;
        const double* gn = geom + (size_t)kn * 16;
        const int ndn = fmask<N>(fn, Nfp - 1 - d);
        double qxp = 0.0, qyp = 0.0;
        for (int dd = 0; dd < Nfp; ++dd) {
          // neighbour jump at its face node dd: 0 - (our value at the facing node)
          const int ours = fmask<N>(f, Nfp - 1 - dd);
          const double dun = (ours == j) ? -1.0 : 0.0;
          if (dun == 0.0) continue;
          const double c = L[ndn * NF + fn * Nfp + dd] * dun * gn[5 + fn] / 2.0;
          qxp -= gn[8 + fn] * c / gn[4];
          qyp -= gn[11 + fn] * c / gn[4];
        }
        dqn = (qx[nd] - qxp) * nx + (qy[nd] - qyp) * ny;
        du = um;
      } else if (dirichlet) {
        dqn = 0.0;
        du = 2.0 * um;
      } else {
        dqn = 2.0 * (qx[nd] * nx + qy[nd] * ny);
        du = 0.0;
      }
      tl[f * Nfp + d] = (dqn + 2.0 * tau[(size_t)k * 4 + f] * du) * g[5 + f] / 2.0;
    }
  }
  for (int i = 0; i < Np; ++i) {
    double xr = 0, xs = 0, yr = 0, ys = 0, lf = 0;
    for (int m = 0; m < Np; ++m) {
      xr += Dr[i * Np + m] * qx[m];
      xs += Ds[i * Np + m] * qx[m];
      yr += Dr[i * Np + m] * qy[m];
      ys += Ds[i * Np + m] * qy[m];
    }
    for (int m = 0; m < NF; ++m) lf += L[i * NF + m] * tl[m];
    out[i] = g[0] * xr + g[2] * xs + g[1] * yr + g[3] * ys - lf / g[4];
  }
  for (int i = 0; i < Np; ++i) {
    double s = 0.0;
    for (int m = 0; m < Np; ++m) s += M[i * Np + m] * out[m];
    blocks[(size_t)k * bstr + (size_t)j * Np + i] = -g[4] * s;
  }
}

// Gauss-Jordan inverse (partial pivoting) of one Np x Np block per CTA, on the
// augmented matrix [B | I] in shared memory.  The block is read row-major
// with stride bstr and replaced by its (symmetrised) inverse in FP64 and FP32.
// Records a singular block in *status.
template <int N>
__global__ void __launch_bounds__(128) block_invert_kernel(int K, double* __restrict__ blocks,
                                                           float* __restrict__ blocks32, int bstr, int* status) {
  using O = Order<N>;
  constexpr int Np = O::Np, W = 2 * Np;
  __shared__ double a[Np * W];
  __shared__ int piv;
  const int k = blockIdx.x;
  if (k >= K) return;
  double* b = blocks + (size_t)k * bstr;
  for (int t = threadIdx.x; t < Np * W; t += blockDim.x) {
    const int r = t / W, c = t % W;
    a[t] = c < Np ? b[r * Np + c] : (c - Np == r ? 1.0 : 0.0);
  }
  __syncthreads();
  for (int c = 0; c < Np; ++c) {
    if (threadIdx.x == 0) {
      int pv = c;
      for (int r = c + 1; r < Np; ++r)
        if (fabs(a[r * W + c]) > fabs(a[pv * W + c])) pv = r;
      piv = (a[pv * W + c] == 0.0) ? -1 : pv;
    }
    __syncthreads();
    const int pv = piv;
    if (pv < 0) {
      if (threadIdx.x == 0) atomicCAS(status, 0, 2);
      return;
    }
    if (pv != c)
      for (int q = threadIdx.x; q < W; q += blockDim.x) {
        const double t = a[c * W + q];
        a[c * W + q] = a[pv * W + q];
        a[pv * W + q] = t;
      }
    __syncthreads();
    const double d = 1.0 / a[c * W + c];
    __syncthreads();
    for (int q = threadIdx.x; q < W; q += blockDim.x) a[c * W + q] *= d;
    __syncthreads();
    for (int t = threadIdx.x; t < Np * W; t += blockDim.x) {
      const int r = t / W, q = t % W;
      if (r != c && q != c) a[t] -= a[r * W + c] * a[c * W + q];
    }
    __syncthreads();
    for (int r = threadIdx.x; r < Np; r += blockDim.x)
      if (r != c) a[r * W + c] = 0.0;
    __syncthreads();
  }
  for (int t = threadIdx.x; t < Np * Np; t += blockDim.x) {
    const int i = t / Np, j = t % Np;
    const double v = 0.5 * (a[i * W + Np + j] + a[j * W + Np + i]);
    b[t] = v;
    blocks32[(size_t)k * bstr + t] = (float)v;
  }
}

}  // namespace dgk
