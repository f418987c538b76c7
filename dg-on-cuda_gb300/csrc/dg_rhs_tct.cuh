// dg_rhs_tct.cuh -- fused RHS + stage kernel on the tensor cores with the A
// operand staged in Tensor Memory.
//
// Same formulation as dg_rhs_tc.cuh (strong form, one product per element and
// output field of the constant operator [Dr | Ds | LIFT] with a K-vector
// [alpha | beta | gamma] built from the element's state, geometry and face
// flux jumps; FP32 through split TF32, D = A_hi B_hi + A_hi B_lo + A_lo B_hi),
// but the rows of A are written straight into TMEM by the threads that own
// them (tcgen05.st, lane = row) instead of through shared memory.
//
// Rows are field-major, row = field * TE + element, so that a warp (one TMEM
// lane quadrant) holds one field of 32 elements and builds its alpha / beta
// columns without divergence.  With three fields, TE = 32 and rows 96..127 are
// unused: the two warps of that lane quadrant process the face tasks
// (element, face) -- neighbour gathers, numerical-flux jumps, gamma -- while
// the six row-owner warps build alpha (half 0) and beta (half 1).  With one
// field, TE = 128 and all warps do the face tasks first.
//   TMEM per CTA: A_hi [0, KP), A_lo [KP, 2 KP), then D_a (2 NC columns) and
//   D_b (NC columns).  B_lo follows B_hi row for row in shared memory, so one
//   N = 2 NC MMA gives A_hi B_hi | A_hi B_lo in D_a and one N = NC MMA gives
//   A_lo B_hi in D_b: two MMAs per K step (an MMA this small costs the same
//   time at N = 32 and N = 64), summed in the epilogue.
// B = [Dr | Ds | LIFT] (hi and lo) is bulk-copied to shared memory once per
// CTA; tiles (state, LSERK residual, geometry, neighbours) are double-buffered.
#pragma once

#include "dg_rhs_tc.cuh"

namespace dgk {

__device__ __forceinline__ void tmem_alloc_n(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc_n(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
// 4 consecutive TMEM columns of this thread's lane
__device__ __forceinline__ void tmem_st4(uint32_t taddr, float a, float b, float c, float d) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x4.b32 [%0], {%1, %2, %3, %4};" ::"r"(taddr), "r"(__float_as_uint(a)),
               "r"(__float_as_uint(b)), "r"(__float_as_uint(c)), "r"(__float_as_uint(d))
               : "memory");
}
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }
// D (TMEM) [+]= A (TMEM) * B (shared memory descriptor)
__device__ __forceinline__ void tc_mma_tf32_ta(uint32_t d_tmem, uint32_t a_tmem, uint64_t b_desc, uint32_t idesc,
                                               uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n}\n" ::"r"(d_tmem),
      "r"(a_tmem), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}
// split 4 values into TF32 hi / lo parts and store both to TMEM
__device__ __forceinline__ void tmem_st4_split(uint32_t t_hi, uint32_t t_lo, const float* v) {
  float hi[4], lo[4];
#pragma unroll
  for (int l = 0; l < 4; ++l) tf32_split(v[l], hi[l], lo[l]);
  tmem_st4(t_hi, hi[0], hi[1], hi[2], hi[3]);
  tmem_st4(t_lo, lo[0], lo[1], lo[2], lo[3]);
}

template <int N, int P>
struct TctConfig {
  using O = Order<N>;
  static constexpr int Np = O::Np, Nfp = O::Nfp, NpP = O::NpP, NFACE = O::Nface;
  static constexpr int Nf = PhysTraits<P>::Nf;
  static constexpr int kThreads = 256;
  static constexpr int TE = Nf == 3 ? 32 : 128;              // elements per tile
  static constexpr int ROWS = Nf * TE;                        // A / D rows in use
  static constexpr bool kFaceWarps = ROWS <= 96;              // lane quadrant 3 free for the face tasks
  static constexpr int ESTR = Nf * NpP;
  static constexpr int KG = 2 * NpP;                          // first gamma column
  static constexpr int KP = (2 * NpP + NFACE + 7) / 8 * 8;    // contraction length
  static constexpr int GC = KP - KG;                          // gamma columns (multiple of 8)
  static constexpr int NC = Np <= 16 ? 16 : 32;
  static constexpr int SBO = (KP / 4) * 128;
  static constexpr uint32_t kTmemCols = (2 * KP + 3 * NC) <= 32 ? 32 : (2 * KP + 3 * NC) <= 64 ? 64
                                        : (2 * KP + 3 * NC) <= 128 ? 128 : 256;
  static constexpr uint32_t kBBytes = NC * KP * 4;
  static constexpr uint32_t kQ = TE * ESTR * 4, kG = TE * 16 * 4, kN = TE * 16;
  static constexpr uint32_t kBuf = 2 * kQ + kG + kN;          // state | residual | geometry | neighbours
  static constexpr uint32_t oBar = 0;                         // 4 mbarriers + TMEM address
  static constexpr uint32_t oB = 64;
  static constexpr uint32_t oGam = oB + 2 * kBBytes;
  // gamma columns are stored column-major, [GC][ROWS]: the face tasks of a warp
  // (consecutive elements) write consecutive words
  static constexpr uint32_t kGam = GC * ROWS * 4;
  static constexpr uint32_t oBuf = oGam + kGam;
  static constexpr uint32_t kSmem = oBuf + 2 * kBuf;
  // dynamic shared memory requested at launch: at least enough that no more
  // CTAs share an SM than its 512 TMEM columns serve (233472 B of shared
  // memory per SM, 1 KB of it reserved per CTA), so tcgen05.alloc never waits
  static constexpr uint32_t kSmemMinForTmem = 233472u / (512u / kTmemCols + 1u);
  static constexpr uint32_t kSmemLaunch = kSmem > kSmemMinForTmem ? kSmem : kSmemMinForTmem;
  static constexpr int kTasks = 3 * TE;                       // (element, face) tasks per tile
  static constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(NC >> 3) << 17) |
                                     ((uint32_t)(128 >> 4) << 24);
  static constexpr uint32_t kIdesc2 = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)((2 * NC) >> 3) << 17) |
                                      ((uint32_t)(128 >> 4) << 24);  // N = 2 NC: [B_hi | B_lo]
  static_assert(2 * KP + 3 * NC <= 256, "TMEM budget");
  static_assert(GC % 8 == 0 && NpP % 4 == 0, "4-column TMEM stores split over two halves");
  static_assert(ROWS <= 128 && TE % 32 == 0, "one field per lane quadrant");
};

// Face tasks: the Nfp nodes of face f of tile element e, in two steps so that
// a caller can issue the gathers of one tile before computing the fluxes of
// another.
//   face_gather: neighbour traces of an interior face (tile element: shared
//     memory, other elements: global memory) or the prescribed boundary values
//     (advection); returns the neighbour code (kn << 2 | fn, or < 0 on the
//     boundary).
//   face_flux: own traces, PEC reflection on boundary faces (Maxwell), the jump
//     of the upwind flux against the own flux, gamma = -(faceJ / J)
//     (f* - n.F(q-)), written to the element's gamma rows (field-major) of the
//     column-major gamma buffer.
template <int N, int P>
__device__ __forceinline__ int face_gather(const RhsParams& p, int e, int f, int k0, int ne, const float* sQ,
                                           const int4* sN, const float* qin,
                                           float (&b)[Order<N>::Nfp][PhysTraits<P>::Nf]) {
  using C = TctConfig<N, P>;
  constexpr int Nfp = C::Nfp, NpP = C::NpP, NF = C::Nf, ESTR = C::ESTR;
  const int4 n4 = sN[e];
  const int nb = f == 0 ? n4.x : (f == 1 ? n4.y : n4.z);
  if (nb >= 0) {
    const int kn = nb >> 2, fn = nb & 3;
    if (kn >= k0 && kn < k0 + ne) {
      const float* qn = sQ + (kn - k0) * ESTR;
#pragma unroll
      for (int d = 0; d < Nfp; ++d)
#pragma unroll
        for (int c = 0; c < NF; ++c) b[d][c] = qn[c * NpP + fmask<N>(fn, Nfp - 1 - d)];
    } else {
      const float* qn = qin + (size_t)kn * ESTR;
#pragma unroll
      for (int d = 0; d < Nfp; ++d)
#pragma unroll
        for (int c = 0; c < NF; ++c) b[d][c] = __ldg(qn + c * NpP + fmask<N>(fn, Nfp - 1 - d));
    }
  } else if (P == PHYS_ADV) {
    const int bf = -1 - nb;
    const double tnow = p.t_dev ? *p.t_dev + p.t : p.t;
#pragma unroll
    for (int d = 0; d < Nfp; ++d) {
      const double xx = p.bxy[((size_t)bf * Nfp + d) * 2], yy = p.bxy[((size_t)bf * Nfp + d) * 2 + 1];
      b[d][0] = (float)adv_exact(p, tnow, xx, yy);
    }
  }
  return nb;
}

template <int N, int P>
__device__ __forceinline__ void face_flux(int e, int f, int nb, const float* sQ, const float* sG,
                                          float (&b)[Order<N>::Nfp][PhysTraits<P>::Nf], float* sGam, float cax,
                                          float cay) {
  using C = TctConfig<N, P>;
  constexpr int Nfp = C::Nfp, NpP = C::NpP, NF = C::Nf, ESTR = C::ESTR, ROWS = C::ROWS, TE = C::TE;
  const float* g = sG + e * 16;
  const float nx = g[8 + f], ny = g[11 + f];
  const float sc = g[5 + f] * g[4];  // -faceJ / J
  const float* qe = sQ + e * ESTR;
  float a[Nfp][NF];
#pragma unroll
  for (int d = 0; d < Nfp; ++d)
#pragma unroll
    for (int c = 0; c < NF; ++c) a[d][c] = qe[c * NpP + fmask<N>(f, d)];
  if (nb < 0 && P != PHYS_ADV) {
#pragma unroll
    for (int d = 0; d < Nfp; ++d) {
      if (P == PHYS_TM) {  // PEC: H+ = H-, Ez+ = -Ez-
        b[d][0] = a[d][0]; b[d][1] = a[d][1]; b[d][2] = -a[d][2];
      } else {             // PEC: E+ = -E-, Hz+ = Hz-
        b[d][0] = -a[d][0]; b[d][1] = -a[d][1]; b[d][2] = a[d][2];
      }
    }
  }
#pragma unroll
  for (int d = 0; d < Nfp; ++d) {
    float dl[NF];
    if (P == PHYS_ADV) {
      const float an = cax * nx + cay * ny;
      dl[0] = an >= 0.0f ? 0.0f : an * (b[d][0] - a[d][0]);
    } else if (P == PHYS_TM) {
      const float dHx = a[d][0] - b[d][0], dHy = a[d][1] - b[d][1], dEz = a[d][2] - b[d][2];
      const float ez = 0.5f * (-dEz + ny * dHx - nx * dHy);
      dl[0] = ny * ez;
      dl[1] = -nx * ez;
      dl[2] = 0.5f * (-ny * dHx + nx * dHy + dEz);
    } else {
      const float dEx = a[d][0] - b[d][0], dEy = a[d][1] - b[d][1], dHz = a[d][2] - b[d][2];
      const float hz = 0.5f * (-dHz - ny * dEx + nx * dEy);
      dl[0] = -ny * hz;
      dl[1] = nx * hz;
      dl[2] = 0.5f * (-nx * dEy + ny * dEx + dHz);
    }
#pragma unroll
    for (int c = 0; c < NF; ++c) sGam[(f * Nfp + d) * ROWS + c * TE + e] = dl[c] * sc;
  }
}

template <int N, int P>
__device__ __forceinline__ void tct_face_task(const RhsParams& p, int e, int f, int k0, int ne, const float* sQ,
                                              const float* sG, const int4* sN, const float* qin, float* sGam,
                                              float cax, float cay) {
  float b[Order<N>::Nfp][PhysTraits<P>::Nf];
  const int nb = face_gather<N, P>(p, e, f, k0, ne, sQ, sN, qin, b);
  face_flux<N, P>(e, f, nb, sQ, sG, b, sGam, cax, cay);
}

template <int N, int P>
__global__ void __launch_bounds__(256, 2) dg_rhs_tct_kernel(const RhsParams p) {
  using C = TctConfig<N, P>;
  constexpr int Np = C::Np, NpP = C::NpP;
  constexpr int TE = C::TE, ESTR = C::ESTR, KP = C::KP, KG = C::KG, GC = C::GC;
  constexpr int NC = C::NC, SBO = C::SBO, NT = C::kThreads, ROWS = C::ROWS;

  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + C::oBar);  // [0],[1] tiles, [2] operator, [3] MMA
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + C::oBar + 32);
  float* Bhi = reinterpret_cast<float*>(smem + C::oB);
  float* sGam = reinterpret_cast<float*>(smem + C::oGam);  // [column][row] scaled flux jumps
  auto bufQ = [&](int b) { return reinterpret_cast<float*>(smem + C::oBuf + b * C::kBuf); };
  auto bufA = [&](int b) { return reinterpret_cast<float*>(smem + C::oBuf + b * C::kBuf + C::kQ); };
  auto bufG = [&](int b) { return reinterpret_cast<float*>(smem + C::oBuf + b * C::kBuf + 2 * C::kQ); };
  auto bufN = [&](int b) {
    return reinterpret_cast<int4*>(smem + C::oBuf + b * C::kBuf + 2 * C::kQ + C::kG);
  };

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int quad = warp & 3, half = warp >> 2;
  const int row = quad * 32 + lane;                 // this thread's A / D row (TMEM lane)
  const bool owner = row < ROWS;                    // warp-uniform
  const int fo = row / TE, er = row - fo * TE;      // (field, element) of the row
  const int ntiles = (p.K + TE - 1) / TE;
  const float* qin = static_cast<const float*>(p.q_in);
  const float cax = p.fax, cay = p.fay, cca = p.fca, ccb = p.fcb, cdt = p.fdt;
  const bool aux_tile = p.mode == MODE_LSERK;

  if (tid == 0) {
    for (int i = 0; i < 4; ++i) mbar_init(&bar[i], 1);
    fence_barrier_init();
  }
  if (warp == 0) tmem_alloc_n(tmem_slot, C::kTmemCols);
  // gamma padding columns are never written by the face tasks
  for (int x = tid; x < GC * ROWS; x += NT) sGam[x] = 0.0f;
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  const uint32_t lane_base = (uint32_t)(quad * 32) << 16;  // this warp's TMEM lane quadrant
  const uint32_t tA = tmem + lane_base;                     // A_hi column 0 of this thread's row
  const uint32_t tD = tmem + 2 * KP;                        // D column 0 (lane 0)
  // zero every A column of the warp's lanes once (each half takes every other
  // 4-column group), so no row or column ever holds uninitialised contents
  for (int c = 4 * half; c < 2 * KP; c += 8) tmem_st4(tA + c, 0.0f, 0.0f, 0.0f, 0.0f);

  auto issue = [&](int tile, int b) {
    const int k0 = tile * TE, ne = min(TE, p.K - k0);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    const uint32_t bq = ne * ESTR * 4, bg = ne * 16 * 4, bn = ne * 16;
    mbar_arrive_expect_tx(&bar[b], bq + (aux_tile ? bq : 0) + bg + bn);
    bulk_g2s(bufQ(b), qin + (size_t)k0 * ESTR, bq, &bar[b]);
    if (aux_tile) bulk_g2s(bufA(b), static_cast<const float*>(p.aux) + (size_t)k0 * ESTR, bq, &bar[b]);
    bulk_g2s(bufG(b), static_cast<const float*>(p.geom) + (size_t)k0 * 16, bg, &bar[b]);
    bulk_g2s(bufN(b), p.nbr + k0, bn, &bar[b]);
  };
  if (tid == 0) {
    mbar_arrive_expect_tx(&bar[2], 2 * C::kBBytes);
    bulk_g2s(Bhi, p.mats_tc, 2 * C::kBBytes, &bar[2]);
    if ((int)blockIdx.x < ntiles) issue(blockIdx.x, 0);
  }
  tmem_wait_st();
  bool ok = __syncthreads_and(mbar_wait(&bar[2], 0, p.status));

  const uint32_t bH = smem_u32(Bhi);  // B_hi, with B_lo directly after it
  const int j0 = 16 * half;                 // first node of this thread's half row in the epilogue
  const int jn = min(NpP - j0, 16);         // nodes of the half row (multiple of 4; <= 0: none)
  float* out = static_cast<float*>(p.out);
  float* aux = static_cast<float*>(p.aux);
  uint32_t ph[2] = {0, 0}, phm = 0;
  int it = 0;
  for (int tile = blockIdx.x; ok && tile < ntiles; tile += gridDim.x, ++it) {
    const int b = it & 1;
    const int k0 = tile * TE, ne = min(TE, p.K - k0);
    const int nxt = tile + gridDim.x;
    // buffer b^1 and its barrier were released by the CTA barrier that ended the
    // previous iteration
    if (tid == 0 && nxt < ntiles) issue(nxt, b ^ 1);
    ok = __syncthreads_and(mbar_wait(&bar[b], ph[b], p.status));
    if (!ok) break;
    ph[b] ^= 1;
    const float* sQ = bufQ(b);
    const float* sR = bufA(b);
    const float* sG = bufG(b);
    const int4* sN = bufN(b);

    // ---- 1. face tasks (element, face): the free lane quadrant's warps while
    //      the row owners build alpha / beta, or every thread first
    if (C::kFaceWarps ? !owner : true) {
      const int nw = C::kFaceWarps ? 64 : NT;
      const int w0 = C::kFaceWarps ? half * 32 + lane : tid;
      for (int t = w0; t < C::kTasks; t += nw) {
        const int f = t / TE, e = t - f * TE;
        if (e < ne) tct_face_task<N, P>(p, e, f, k0, ne, sQ, sG, sN, qin, sGam, cax, cay);
      }
    }

    // ---- 2. volume columns straight to TMEM: half 0 writes alpha, half 1 beta,
    //      alpha_j = -(rx F_x + ry F_y)_j, beta_j = -(sx F_x + sy F_y)_j of the flux
    //      F of output field fo (strong form); padding nodes and rows without an
    //      element store zeros (tcgen05.st is warp-collective)
    if (owner) {
      const bool valid = er < ne;
      const int erc = valid ? er : 0;
      const float* g = sG + erc * 16;
      const float mx = half == 0 ? g[0] : g[2], my = half == 0 ? g[1] : g[3];
      const float* qe = sQ + erc * ESTR;
      const uint32_t col0 = (uint32_t)(half * NpP);
#pragma unroll
      for (int j = 0; j < NpP; j += 4) {
        float v[4];
        if (P == PHYS_ADV) {
          const float4 u = *reinterpret_cast<const float4*>(qe + j);
          const float cm = -(cax * mx + cay * my);
          v[0] = cm * u.x; v[1] = cm * u.y; v[2] = cm * u.z; v[3] = cm * u.w;
        } else if (fo < 2) {  // Ex, Ey (TE) / Hx, Hy (TM): flux of the third field only
          const float4 q2 = *reinterpret_cast<const float4*>(qe + 2 * NpP + j);
          // TE: F(Ex) = (0, -Hz) -> alpha = my Hz;  F(Ey) = (Hz, 0) -> alpha = -mx Hz
          // TM: F(Hx) = (0, Ez) -> alpha = -my Ez;  F(Hy) = (-Ez, 0) -> alpha = mx Ez
          const float cm = (P == PHYS_TE) ? (fo == 0 ? my : -mx) : (fo == 0 ? -my : mx);
          v[0] = cm * q2.x; v[1] = cm * q2.y; v[2] = cm * q2.z; v[3] = cm * q2.w;
        } else {              // Hz (TE): F = (Ey, -Ex);  Ez (TM): F = (-Hy, Hx)
          const float4 q0 = *reinterpret_cast<const float4*>(qe + j);
          const float4 q1 = *reinterpret_cast<const float4*>(qe + NpP + j);
          const float c0 = (P == PHYS_TE) ? my : -my, c1 = (P == PHYS_TE) ? -mx : mx;
          v[0] = c0 * q0.x + c1 * q1.x; v[1] = c0 * q0.y + c1 * q1.y;
          v[2] = c0 * q0.z + c1 * q1.z; v[3] = c0 * q0.w + c1 * q1.w;
        }
#pragma unroll
        for (int l = 0; l < 4; ++l)
          if (!valid || j + l >= Np) v[l] = 0.0f;
        tmem_st4_split(tA + col0 + j, tA + KP + col0 + j, v);
      }
    }
    __syncthreads();  // gamma rows complete

    // ---- 3. gamma columns of the row to TMEM (the halves take alternate groups)
    if (owner) {
      const float* gr = sGam + row;
#pragma unroll
      for (int c = 4 * half; c < GC; c += 8) {
        const float v[4] = {gr[c * ROWS], gr[(c + 1) * ROWS], gr[(c + 2) * ROWS], gr[(c + 3) * ROWS]};
        tmem_st4_split(tA + KG + c, tA + KP + KG + c, v);
      }
      tmem_wait_st();
    }

    // ---- 4. tensor cores: D = A_hi B_hi + A_hi B_lo + A_lo B_hi
    tc_fence_before();
    __syncthreads();
    if (tid == 0) {
      tc_fence_after();
#pragma unroll
      for (int s = 0; s < KP / 8; ++s) {
        const uint64_t dB = smem_desc(bH + s * 256, 128, SBO);  // rows 0..NC-1: B_hi, NC..2NC-1: B_lo
        tc_mma_tf32_ta(tD, tmem + (uint32_t)(8 * s), dB, C::kIdesc2, s > 0 ? 1u : 0u);
        tc_mma_tf32_ta(tD + 2 * NC, tmem + (uint32_t)(KP + 8 * s), dB, C::kIdesc, s > 0 ? 1u : 0u);
      }
      tc_commit(&bar[3]);
    }
    ok = __syncthreads_and(mbar_wait(&bar[3], phm, p.status));
    phm ^= 1;
    if (!ok) break;
    tc_fence_after();

    // ---- 5. epilogue: this thread's half row (16 nodes) from its warp's TMEM lanes
    if (owner && j0 < NC) {
      float rhs[16], r1[16], r2[16];
      tmem_ld16(tD + lane_base + (uint32_t)j0, rhs);
      tmem_ld16(tD + lane_base + (uint32_t)(NC + j0), r1);
      tmem_ld16(tD + lane_base + (uint32_t)(2 * NC + j0), r2);
#pragma unroll
      for (int j = 0; j < 16; ++j) rhs[j] += r1[j] + r2[j];
      if (er < ne && jn > 0) {
        const size_t base = (size_t)(k0 + er) * ESTR + (size_t)fo * NpP + j0;
        const float* qrow = sQ + er * ESTR + fo * NpP + j0;
        auto rv = [&](int j) { return (j0 + j) < Np ? rhs[j] : 0.0f; };
        if (p.mode == MODE_RHS) {
#pragma unroll
          for (int j = 0; j < 16; j += 4)
            if (j < jn)
              *reinterpret_cast<float4*>(out + base + j) = make_float4(rv(j), rv(j + 1), rv(j + 2), rv(j + 3));
        } else if (p.mode == MODE_LSERK) {
          const float* rrow = sR + er * ESTR + fo * NpP + j0;
#pragma unroll
          for (int j = 0; j < 16; j += 4)
            if (j < jn) {
              const float4 qv = *reinterpret_cast<const float4*>(qrow + j);
              float4 r = *reinterpret_cast<const float4*>(rrow + j);
              r.x = cca * r.x + cdt * rv(j);
              r.y = cca * r.y + cdt * rv(j + 1);
              r.z = cca * r.z + cdt * rv(j + 2);
              r.w = cca * r.w + cdt * rv(j + 3);
              float4 o4 = make_float4(qv.x + ccb * r.x, qv.y + ccb * r.y, qv.z + ccb * r.z, qv.w + ccb * r.w);
              // padding nodes are written as 0
              if (j0 + j + 3 >= Np) { r.w = 0.0f; o4.w = 0.0f; }
              if (j0 + j + 2 >= Np) { r.z = 0.0f; o4.z = 0.0f; }
              if (j0 + j + 1 >= Np) { r.y = 0.0f; o4.y = 0.0f; }
              *reinterpret_cast<float4*>(aux + base + j) = r;
              *reinterpret_cast<float4*>(out + base + j) = o4;
            }
        } else {
          float* q0 = static_cast<float*>(p.q0);
#pragma unroll
          for (int j = 0; j < 16; ++j) {  // constant indices keep rhs[] in registers
            if (j >= jn || j0 + j >= Np) continue;
            const size_t o = base + j;
            if (p.stage == 0) {
              aux[o] = rhs[j];
              out[o] = qrow[j] + cca * rhs[j];
            } else if (p.stage < 3) {
              aux[o] = aux[o] + ccb * rhs[j];
              out[o] = q0[o] + cca * rhs[j];
            } else {
              q0[o] = q0[o] + cca * (aux[o] + rhs[j]);
            }
          }
        }
      }
    }
    tc_fence_before();
    __syncthreads();
  }
  // ---- release TMEM on every exit path
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc_n(tmem, C::kTmemCols);
  }
}

}  // namespace dgk
