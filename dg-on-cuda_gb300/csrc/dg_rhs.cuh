// dg_rhs.cuh -- fused nodal-DG right-hand side + time-integrator stage.
//
// One launch evaluates the semi-discrete operator of every element and applies
// the time-stepping update in the same pass:
//   volume term   (Dr, Ds applied to the fields, combined with rx, ry, sx, sy),
//   face gather   (own and neighbour face nodes through the neighbour table),
//   numerical flux (upwind advection, upwind Maxwell TM / TE with PEC walls),
//   LIFT          (surface integral lifted to the volume nodes, scaled by 1/J),
//   epilogue      (plain RHS, LSERK4 stage, or classical-RK4 stage).
// It replaces the reference's per-element device operators
// (examples/advection_2d/d_advection_2d.cuh:45-100,
//  examples/maxwell_2d/d_maxwell_2d.cuh:50-131) launched through
// dgc::opx (src/device_SemiDiscOp_wrapper.cuh:35-43), plus the axpy kernels of
// dgc::rk4 (src/explicit_runge_kutta.h:33-51, src/k_axpy.cuh:38-55).
//
// Layout (HBM): state q[k][field][NpP], NpP = Np padded to a multiple of 4, so
// that every element is a contiguous, 16-byte aligned run.  Geometry records
// are 16 values per element in the kernel's type (rounded once on the host
// from the FP64 set-up, -1/J precomputed); neighbours are one int4 per element.
//
// Execution: persistent CTAs loop over tiles of TE elements.  The operator
// matrices (stored transposed) are copied into shared memory once per CTA and
// each tile's state / geometry / neighbour records are copied in by
// cp.async.bulk with an mbarrier; the neighbour face values that fall outside
// the tile are gathered from global memory (L2).
#pragma once

#include "common.cuh"

namespace dgk {

enum Physics : int { PHYS_ADV = 0, PHYS_TM = 1, PHYS_TE = 2 };
enum Mode : int { MODE_RHS = 0, MODE_LSERK = 1, MODE_RK4 = 2 };
enum BcKind : int { BC_SINSIN = 0, BC_GAUSS = 1, BC_ZERO = 2 };

template <int P>
struct PhysTraits { static constexpr int Nf = (P == PHYS_ADV) ? 1 : 3; };

struct RhsParams {
  int K;
  const void* q_in;   // operator input state
  void* out;          // RHS: rhs | LSERK: next state | RK4: next stage input
  void* aux;          // LSERK: residual | RK4: stage accumulator
  void* q0;           // RK4: base state (updated by the last stage)
  const void* geom;   // [K][16] kernel geometry records in the kernel type (slot 4 = -1/J)
  const int4* nbr;    // [K]
  const double* bxy;  // boundary face nodes [nbf][Nfp][2]
  const void* mats;   // DrT | DsT | LT, each padded to 16 bytes
  const void* mats_tc;// FP32 tensor-core operand [Dr | Ds | LIFT] (split TF32, core-matrix layout)
  const void* mats_blk;// FP32 rows of Dr^T | Ds^T | LIFT^T, each padded to NpP columns (weak form)
  double t, dt;       // time of the operator evaluation (offset when t_dev is set), step size
  const double* t_dev;// optional device-resident base time: operator time = *t_dev + t
  double ca, cb;      // LSERK: a_k, b_k | RK4: output coefficient, accumulator weight
  double ax, ay;      // advection velocity
  double gx0, gy0, gw;
  int bc, mode, stage;
  int* status;
  // FP32 copies of ax, ay, ca, cb, dt, filled by rhs_dispatch<float> so that
  // FP32 kernels convert nothing on the (slow) FP64 pipe
  float fax, fay, fca, fcb, fdt;
};

inline RhsParams with_f32_scalars(RhsParams p) {
  p.fax = (float)p.ax;
  p.fay = (float)p.ay;
  p.fca = (float)p.ca;
  p.fcb = (float)p.cb;
  p.fdt = (float)p.dt;
  return p;
}

template <typename R, int N>
struct MatLayout {
  using O = Order<N>;
  static constexpr int kD = (O::Np * O::Np + 3) / 4 * 4;
  static constexpr int kL = (O::Nface * O::Np + 3) / 4 * 4;
  static constexpr int kTotal = 2 * kD + kL;  // in elements of R
  static constexpr uint32_t kBytes = kTotal * sizeof(R);
};

template <typename R, int N, int P>
struct RhsConfig {
  using O = Order<N>;
  static constexpr int kThreads = 256;
  static constexpr int TE = (kThreads / O::Np) > 0 ? (kThreads / O::Np) : 1;  // elements per tile
  static constexpr int Nf = PhysTraits<P>::Nf;
  static constexpr int ESTR = Nf * O::NpP;                                      // state stride per element
  // dynamic shared memory layout (bytes)
  static constexpr uint32_t oBar = 0;
  static constexpr uint32_t oMats = 32;  // room for the three barriers of the batched kernel's other tile code
  static constexpr uint32_t oQ = oMats + MatLayout<R, N>::kBytes;
  static constexpr uint32_t oGeom = (oQ + TE * ESTR * sizeof(R) + 15) / 16 * 16;
  static constexpr uint32_t oNbr = oGeom + TE * 16 * sizeof(R);
  static constexpr uint32_t oFlux = oNbr + TE * 16;
  static constexpr uint32_t kSmem = (oFlux + TE * Nf * O::Nface * sizeof(R) + 15) / 16 * 16;
};

template <typename R>
__device__ __forceinline__ R ldg(const R* p) { return __ldg(p); }

__device__ __forceinline__ double adv_exact(const RhsParams& p, double t, double x, double y) {
  if (p.bc == BC_SINSIN)
    return sin((x + 1.0 - p.ax * t) * M_PI) * sin((y + 1.0 - p.ay * t) * M_PI);
  if (p.bc == BC_GAUSS) {
    const double dx = x - p.ax * t - p.gx0, dy = y - p.ay * t - p.gy0;
    return exp(-(dx * dx + dy * dy) / p.gw);
  }
  return 0.0;
}

// Shared-memory view of the tile layout of dg_rhs_kernel (RhsConfig).
template <typename R, int N, int P>
struct V1Smem {
  using C = RhsConfig<R, N, P>;
  uint64_t* bar;
  R *sDrT, *sDsT, *sLT, *sQ, *sG, *sF;
  int4* sN;
  __device__ explicit V1Smem(unsigned char* smem) {
    constexpr int kD = MatLayout<R, N>::kD;
    bar = reinterpret_cast<uint64_t*>(smem + C::oBar);
    sDrT = reinterpret_cast<R*>(smem + C::oMats);
    sDsT = sDrT + kD;
    sLT = sDrT + 2 * kD;
    sQ = reinterpret_cast<R*>(smem + C::oQ);
    sG = reinterpret_cast<R*>(smem + C::oGeom);
    sN = reinterpret_cast<int4*>(smem + C::oNbr);
    sF = reinterpret_cast<R*>(smem + C::oFlux);
  }
};

// Bulk-copy the operator matrices of p into shared memory.  Every thread has
// observed the completed phase before the function returns (the caller
// re-arms the same barrier next); false if the wait expired.
template <typename R, int N, int P>
__device__ __forceinline__ bool rhs_v1_load_mats(const RhsParams& p, const V1Smem<R, N, P>& s, uint32_t& phase) {
  if (threadIdx.x == 0) {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_arrive_expect_tx(s.bar, MatLayout<R, N>::kBytes);
    bulk_g2s(s.sDrT, p.mats, MatLayout<R, N>::kBytes, s.bar);
  }
  // All threads must have observed this phase before thread 0 re-arms the
  // barrier for a tile: otherwise a fast tile copy can complete the next
  // phase before a slow warp polls this one, and that warp would then wait
  // for a phase that never comes.  The AND also makes a timed-out wait exit
  // the whole CTA.
  const bool ok = __syncthreads_and(mbar_wait(s.bar, phase, p.status));
  phase ^= 1;
  return ok;
}

// One tile of the stage: the ne (<= TE) elements from k0 -- bulk load of
// state / geometry / neighbours, numerical fluxes on the face nodes, volume
// and lift contractions (one thread per element-node), stage epilogue.
// Ends with a CTA barrier; false if a wait expired.
template <typename R, int N, int P>
__device__ __forceinline__ bool rhs_v1_tile(const RhsParams& p, const V1Smem<R, N, P>& s, uint32_t& phase, int k0,
                                            int ne) {
  using O = Order<N>;
  using C = RhsConfig<R, N, P>;
  constexpr int Np = O::Np, Nfp = O::Nfp, NpP = O::NpP, NFACE = O::Nface;
  constexpr int NF = C::Nf, ESTR = C::ESTR;
  const int tid = threadIdx.x;
  const R* qin = static_cast<const R*>(p.q_in);
  // scalar parameters in the kernel type
  constexpr bool f32 = sizeof(R) == 4;
  const R cax = f32 ? (R)p.fax : (R)p.ax, cay = f32 ? (R)p.fay : (R)p.ay;
  const R cca = f32 ? (R)p.fca : (R)p.ca, ccb = f32 ? (R)p.fcb : (R)p.cb, cdt = f32 ? (R)p.fdt : (R)p.dt;
  R* sQ = s.sQ;
  R* sG = s.sG;
  int4* sN = s.sN;
  R* sF = s.sF;
  const R* sDrT = s.sDrT;
  const R* sDsT = s.sDsT;
  const R* sLT = s.sLT;
  if (tid == 0) {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    const uint32_t bq = ne * ESTR * sizeof(R), bg = ne * 16 * sizeof(R), bn = ne * 16;
    mbar_arrive_expect_tx(s.bar, bq + bg + bn);
    bulk_g2s(sQ, qin + (size_t)k0 * ESTR, bq, s.bar);
    bulk_g2s(sG, static_cast<const R*>(p.geom) + (size_t)k0 * 16, bg, s.bar);
    bulk_g2s(sN, p.nbr + k0, bn, s.bar);
  }
  if (!__syncthreads_and(mbar_wait(s.bar, phase, p.status))) return false;
  phase ^= 1;
  // ---- numerical fluxes on the tile's face nodes, scaled by faceJ
  for (int it = tid; it < ne * NFACE; it += blockDim.x) {
    const int e = it / NFACE, fm = it - e * NFACE, f = fm / Nfp, d = fm - f * Nfp;
    const R* g = sG + e * 16;
    const int nb = f == 0 ? sN[e].x : (f == 1 ? sN[e].y : sN[e].z);
    const int nd = fmask<N>(f, d);
    const R* qa = sQ + e * ESTR;
    const R nx = (R)g[8 + f], ny = (R)g[11 + f], fJ = (R)g[5 + f];
    R a[NF], b[NF];
#pragma unroll
    for (int c = 0; c < NF; ++c) a[c] = qa[c * NpP + nd];
    if (nb >= 0) {
      const int kn = nb >> 2, fn = nb & 3, nd2 = fmask<N>(fn, Nfp - 1 - d);
      if (kn >= k0 && kn < k0 + ne) {
        const R* qb = sQ + (kn - k0) * ESTR;
#pragma unroll
        for (int c = 0; c < NF; ++c) b[c] = qb[c * NpP + nd2];
      } else {
        const R* qb = qin + (size_t)kn * ESTR;
#pragma unroll
        for (int c = 0; c < NF; ++c) b[c] = ldg(qb + c * NpP + nd2);
      }
    } else if (P == PHYS_ADV) {
      const int bf = -1 - nb;
      const double x = p.bxy[((size_t)bf * Nfp + d) * 2], y = p.bxy[((size_t)bf * Nfp + d) * 2 + 1];
      b[0] = (R)adv_exact(p, p.t_dev ? *p.t_dev + p.t : p.t, x, y);
    } else if (P == PHYS_TM) {  // PEC: H+ = H-, Ez+ = -Ez-
      b[0] = a[0]; b[1] = a[1]; b[2] = -a[2];
    } else {                    // PEC: E+ = -E-, Hz+ = Hz-
      b[0] = -a[0]; b[1] = -a[1]; b[2] = a[2];
    }
    R* fo = sF + e * NF * NFACE + fm;
    if (P == PHYS_ADV) {
      const R an = cax * nx + cay * ny;
      fo[0] = ((an >= (R)0) ? a[0] : b[0]) * an * fJ;
    } else if (P == PHYS_TM) {
      const R d0 = a[0] - b[0], d1 = a[1] - b[1], s2 = a[2] + b[2];
      const R w = s2 + ny * d0 - nx * d1;
      fo[0] = (R)0.5 * ny * w * fJ;
      fo[NFACE] = -(R)0.5 * nx * w * fJ;
      fo[2 * NFACE] = (R)0.5 * (ny * (a[0] + b[0]) - nx * (a[1] + b[1]) + a[2] - b[2]) * fJ;
    } else {
      const R d0 = a[0] - b[0], d1 = a[1] - b[1], s2 = a[2] + b[2];
      const R w = s2 - ny * d0 + nx * d1;
      fo[0] = -(R)0.5 * ny * w * fJ;
      fo[NFACE] = (R)0.5 * nx * w * fJ;
      fo[2 * NFACE] = (R)0.5 * (nx * (a[1] + b[1]) - ny * (a[0] + b[0]) + a[2] - b[2]) * fJ;
    }
  }
  __syncthreads();

  // ---- volume + lift + epilogue: one (element, node) per thread
  if (tid < ne * Np) {
    const int e = tid / Np, i = tid - e * Np;
    const R* qe = sQ + e * ESTR;
    R ur[NF], us[NF], lf[NF];
#pragma unroll
    for (int c = 0; c < NF; ++c) ur[c] = us[c] = lf[c] = (R)0;
#pragma unroll 4
    for (int j = 0; j < Np; ++j) {
      const R dr = sDrT[j * Np + i], ds = sDsT[j * Np + i];
#pragma unroll
      for (int c = 0; c < NF; ++c) {
        const R v = qe[c * NpP + j];
        ur[c] = fma(dr, v, ur[c]);
        us[c] = fma(ds, v, us[c]);
      }
    }
    const R* fe = sF + e * NF * NFACE;
#pragma unroll 3
    for (int m = 0; m < NFACE; ++m) {
      const R l = sLT[m * Np + i];
#pragma unroll
      for (int c = 0; c < NF; ++c) lf[c] = fma(l, fe[c * NFACE + m], lf[c]);
    }
    const R* g = sG + e * 16;
    const R rx = (R)g[0], ry = (R)g[1], sx = (R)g[2], sy = (R)g[3];
    const R ilJ = g[4];  // -1/J
    R rhs[NF];
    if (P == PHYS_ADV) {
      const R dx = rx * ur[0] + sx * us[0], dy = ry * ur[0] + sy * us[0];
      rhs[0] = cax * dx + cay * dy + ilJ * lf[0];
    } else if (P == PHYS_TM) {  // Hx' = Dy Ez, Hy' = -Dx Ez, Ez' = -Dx Hy + Dy Hx
      rhs[0] = (ry * ur[2] + sy * us[2]) + ilJ * lf[0];
      rhs[1] = -(rx * ur[2] + sx * us[2]) + ilJ * lf[1];
      rhs[2] = -(rx * ur[1] + sx * us[1]) + (ry * ur[0] + sy * us[0]) + ilJ * lf[2];
    } else {                    // Ex' = -Dy Hz, Ey' = Dx Hz, Hz' = Dx Ey - Dy Ex
      rhs[0] = -(ry * ur[2] + sy * us[2]) + ilJ * lf[0];
      rhs[1] = (rx * ur[2] + sx * us[2]) + ilJ * lf[1];
      rhs[2] = (rx * ur[1] + sx * us[1]) - (ry * ur[0] + sy * us[0]) + ilJ * lf[2];
    }
    const size_t base = (size_t)(k0 + e) * ESTR + i;
    R* out = static_cast<R*>(p.out);
    R* aux = static_cast<R*>(p.aux);
    if (p.mode == MODE_RHS) {
#pragma unroll
      for (int c = 0; c < NF; ++c) out[base + c * NpP] = rhs[c];
    } else if (p.mode == MODE_LSERK) {
#pragma unroll
      for (int c = 0; c < NF; ++c) {
        const size_t o = base + c * NpP;
        const R r = cca * aux[o] + cdt * rhs[c];
        aux[o] = r;
        out[o] = qe[c * NpP + i] + ccb * r;
      }
    } else {  // classical RK4 stage
      R* q0 = static_cast<R*>(p.q0);
      const R co = cca, wa = ccb;
#pragma unroll
      for (int c = 0; c < NF; ++c) {
        const size_t o = base + c * NpP;
        if (p.stage == 0) {
          aux[o] = rhs[c];
          out[o] = qe[c * NpP + i] + co * rhs[c];
        } else if (p.stage < 3) {
          aux[o] = aux[o] + wa * rhs[c];
          out[o] = q0[o] + co * rhs[c];
        } else {
          q0[o] = q0[o] + co * (aux[o] + rhs[c]);
        }
      }
    }
  }
  __syncthreads();
  return true;
}

template <typename R, int N, int P>
__global__ void __launch_bounds__(256) dg_rhs_kernel(const RhsParams p) {
  using C = RhsConfig<R, N, P>;
  extern __shared__ __align__(128) unsigned char smem[];
  const V1Smem<R, N, P> s(smem);
  const int ntiles = (p.K + C::TE - 1) / C::TE;
  if (threadIdx.x == 0) {
    mbar_init(s.bar, 1);
    fence_barrier_init();
  }
  __syncthreads();
  uint32_t phase = 0;
  if (!rhs_v1_load_mats<R, N, P>(p, s, phase)) return;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int k0 = tile * C::TE;
    if (!rhs_v1_tile<R, N, P>(p, s, phase, k0, min(C::TE, p.K - k0))) return;
  }
}

}  // namespace dgk
