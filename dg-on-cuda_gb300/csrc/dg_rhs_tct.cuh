// dg_rhs_tct.cuh -- fused RHS + stage kernel on the tensor cores with the A
// operand staged in Tensor Memory.
//
// Same formulation as dg_rhs_tc.cuh (strong form, one product per element and
// output field of the constant operator [Dr | Ds | LIFT] with a K-vector
// [alpha | beta | gamma] built from the element's state, geometry and face
// flux jumps; FP32 through split TF32, D = A_hi B_hi + A_hi B_lo + A_lo B_hi),
// but the rows of A are written straight into TMEM by the threads that own
// them (tcgen05.st, lane = row) instead of through shared memory:
//   * no shared-memory stores or bank conflicts for A, and 80 KB less shared
//     memory per CTA at order 6, so two CTAs share an SM;
//   * TMEM per CTA: A_hi [0, KP), A_lo [KP, 2 KP), D [2 KP, 2 KP + NC) columns.
// B = [Dr | Ds | LIFT] (hi and lo) is bulk-copied to shared memory once per
// CTA.  Tiles (state, LSERK residual, geometry, neighbours) are
// double-buffered.  Row r = tid % 128 is (element r / Nf, field r % Nf); its
// two threads (half = tid / 128) split the alpha / beta / gamma columns and
// the epilogue's 16-node halves.
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

template <int N, int P>
struct TctConfig {
  using O = Order<N>;
  static constexpr int Np = O::Np, Nfp = O::Nfp, NpP = O::NpP, NFACE = O::Nface;
  static constexpr int Nf = PhysTraits<P>::Nf;
  static constexpr int kThreads = 256;
  static constexpr int TE = 128 / Nf;
  static constexpr int ESTR = Nf * NpP;
  static constexpr int KG = 2 * NpP;                         // first gamma column
  static constexpr int KP = (2 * NpP + NFACE + 7) / 8 * 8;   // contraction length
  static constexpr int GC = KP - KG;                          // gamma columns (multiple of 4)
  static constexpr int GSTR = (GC + 3) / 4 * 4;               // gamma row stride in shared memory
  static constexpr int NC = Np <= 16 ? 16 : 32;
  static constexpr int SBO = (KP / 4) * 128;
  static constexpr uint32_t kTmemCols = (2 * KP + NC) <= 32 ? 32 : (2 * KP + NC) <= 64 ? 64
                                        : (2 * KP + NC) <= 128 ? 128 : 256;
  static constexpr uint32_t kBBytes = NC * KP * 4;
  static constexpr uint32_t kQ = TE * ESTR * 4, kG = TE * 16 * 4, kN = TE * 16;
  static constexpr uint32_t kBuf = 2 * kQ + kG + kN;         // state | residual | geometry | neighbours
  static constexpr uint32_t oBar = 0;                        // 4 mbarriers + TMEM address
  static constexpr uint32_t oB = 64;
  static constexpr uint32_t oGam = oB + 2 * kBBytes;
  static constexpr uint32_t oBuf = oGam + 128 * GSTR * 4;
  static constexpr uint32_t kSmem = oBuf + 2 * kBuf;
  // dynamic shared memory requested at launch: at least enough that no more
  // CTAs share an SM than its 512 TMEM columns serve (233472 B of shared
  // memory per SM, 1 KB of it reserved per CTA), so tcgen05.alloc never waits
  static constexpr uint32_t kSmemMinForTmem = 233472u / (512u / kTmemCols + 1u);
  static constexpr uint32_t kSmemLaunch = kSmem > kSmemMinForTmem ? kSmem : kSmemMinForTmem;
  static constexpr int kItems = (TE * NFACE + kThreads - 1) / kThreads;
  static constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(NC >> 3) << 17) |
                                     ((uint32_t)(128 >> 4) << 24);
  static_assert(2 * KP + NC <= 256, "TMEM budget");
  static_assert(GC % 4 == 0 && NpP % 4 == 0, "4-column TMEM stores");
};

template <int N, int P>
__global__ void __launch_bounds__(256, 2) dg_rhs_tct_kernel(const RhsParams p) {
  using C = TctConfig<N, P>;
  constexpr int Np = C::Np, Nfp = C::Nfp, NpP = C::NpP, NFACE = C::NFACE, NF = C::Nf;
  constexpr int TE = C::TE, ESTR = C::ESTR, KP = C::KP, KG = C::KG, GC = C::GC, GSTR = C::GSTR;
  constexpr int NC = C::NC, SBO = C::SBO, NT = C::kThreads;

  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + C::oBar);  // [0],[1] tiles, [2] operator, [3] MMA
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + C::oBar + 32);
  float* Bhi = reinterpret_cast<float*>(smem + C::oB);
  float* sGam = reinterpret_cast<float*>(smem + C::oGam);  // [row][GSTR] scaled face-flux jumps
  auto bufQ = [&](int b) { return reinterpret_cast<float*>(smem + C::oBuf + b * C::kBuf); };
  auto bufA = [&](int b) { return reinterpret_cast<float*>(smem + C::oBuf + b * C::kBuf + C::kQ); };
  auto bufG = [&](int b) { return reinterpret_cast<float*>(smem + C::oBuf + b * C::kBuf + 2 * C::kQ); };
  auto bufN = [&](int b) {
    return reinterpret_cast<int4*>(smem + C::oBuf + b * C::kBuf + 2 * C::kQ + C::kG);
  };

  const int tid = threadIdx.x, warp = tid >> 5;
  const int row = tid & 127, half = tid >> 7, fo = row % NF, er = row / NF;
  const int ntiles = (p.K + TE - 1) / TE;
  const float* qin = static_cast<const float*>(p.q_in);
  const float cax = p.fax, cay = p.fay, cca = p.fca, ccb = p.fcb, cdt = p.fdt;
  const bool aux_tile = p.mode == MODE_LSERK;

  if (tid == 0) {
    for (int i = 0; i < 4; ++i) mbar_init(&bar[i], 1);
    fence_barrier_init();
  }
  if (warp == 0) tmem_alloc_n(tmem_slot, C::kTmemCols);
  // gamma padding columns are never written by the face phase
  for (int x = tid; x < 128 * GSTR; x += NT) sGam[x] = 0.0f;
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;  // this warp's TMEM lane quadrant
  const uint32_t tA = tmem + lane_base;                           // A_hi column 0 of this thread's row
  const uint32_t tD = tmem + 2 * KP;                              // D column 0 (lane 0)
  // zero this thread's half of its A row once (hi and lo), so that no column
  // or unused row ever holds uninitialised TMEM contents
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

  const uint32_t bH = smem_u32(Bhi), bL = bH + C::kBBytes;
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

    // ---- 1. neighbour gathers of this thread's face items (latency hidden by step 2)
    float av[C::kItems][NF], bv[C::kItems][NF];
#pragma unroll
    for (int s2 = 0; s2 < C::kItems; ++s2) {
      const int x = tid + s2 * NT;
      if (x >= ne * NFACE) continue;
      const int e = x / NFACE, fm = x - e * NFACE, f = fm / Nfp, d = fm - f * Nfp;
      const int nb = f == 0 ? sN[e].x : (f == 1 ? sN[e].y : sN[e].z);
      const int nd = fmask<N>(f, d);
#pragma unroll
      for (int c = 0; c < NF; ++c) av[s2][c] = sQ[e * ESTR + c * NpP + nd];
      if (nb >= 0) {
        const int kn = nb >> 2, nd2 = fmask<N>(nb & 3, Nfp - 1 - d);
        if (kn >= k0 && kn < k0 + ne) {
#pragma unroll
          for (int c = 0; c < NF; ++c) bv[s2][c] = sQ[(kn - k0) * ESTR + c * NpP + nd2];
        } else {
          const float* qb = qin + (size_t)kn * ESTR + nd2;
#pragma unroll
          for (int c = 0; c < NF; ++c) bv[s2][c] = __ldg(qb + c * NpP);
        }
      } else if (P == PHYS_ADV) {
        const int bf = -1 - nb;
        const double xx = p.bxy[((size_t)bf * Nfp + d) * 2], yy = p.bxy[((size_t)bf * Nfp + d) * 2 + 1];
        bv[s2][0] = (float)adv_exact(p, p.t_dev ? *p.t_dev + p.t : p.t, xx, yy);
      } else if (P == PHYS_TM) {  // PEC: H+ = H-, Ez+ = -Ez-
        bv[s2][0] = av[s2][0]; bv[s2][1] = av[s2][1]; bv[s2][2] = -av[s2][2];
      } else {                    // PEC: E+ = -E-, Hz+ = Hz-
        bv[s2][0] = -av[s2][0]; bv[s2][1] = -av[s2][1]; bv[s2][2] = av[s2][2];
      }
    }

    // ---- 2. volume columns straight to TMEM: half 0 writes alpha, half 1 beta,
    //      alpha_j = -(rx F_x + ry F_y)_j, beta_j = -(sx F_x + sy F_y)_j of the flux
    //      F of output field fo (strong form); padding nodes are 0.  tcgen05.st is
    //      warp-collective, so rows without an element (ragged last tile, rows
    //      past TE * Nf) read element 0 and store zeros.
    const bool valid = er < ne;
    const int erc = valid ? er : 0;
    {
      const float* g = sG + erc * 16;
      // this half's metric pair: (rx, ry) for alpha, (sx, sy) for beta
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
        } else {
          const float4 q0 = *reinterpret_cast<const float4*>(qe + j);
          const float4 q1 = *reinterpret_cast<const float4*>(qe + NpP + j);
          const float4 q2 = *reinterpret_cast<const float4*>(qe + 2 * NpP + j);
          const float a0[4] = {q0.x, q0.y, q0.z, q0.w}, a1[4] = {q1.x, q1.y, q1.z, q1.w};
          const float a2[4] = {q2.x, q2.y, q2.z, q2.w};
#pragma unroll
          for (int l = 0; l < 4; ++l) {
            if (P == PHYS_TM) {  // F(Hx) = (0, Ez), F(Hy) = (-Ez, 0), F(Ez) = (-Hy, Hx)
              v[l] = fo == 0 ? -my * a2[l] : (fo == 1 ? mx * a2[l] : mx * a1[l] - my * a0[l]);
            } else {             // F(Ex) = (0, -Hz), F(Ey) = (Hz, 0), F(Hz) = (Ey, -Ex)
              v[l] = fo == 0 ? my * a2[l] : (fo == 1 ? -mx * a2[l] : my * a0[l] - mx * a1[l]);
            }
          }
        }
        float hi[4], lo[4];
#pragma unroll
        for (int l = 0; l < 4; ++l) {
          const float x = (valid && j + l < Np) ? v[l] : 0.0f;
          tf32_split(x, hi[l], lo[l]);
        }
        tmem_st4(tA + col0 + j, hi[0], hi[1], hi[2], hi[3]);
        tmem_st4(tA + KP + col0 + j, lo[0], lo[1], lo[2], lo[3]);
      }
    }

    // ---- 3. face-flux jumps, gamma = -(faceJ / J) (f* - n.F(q-)) per output field
#pragma unroll
    for (int s2 = 0; s2 < C::kItems; ++s2) {
      const int x = tid + s2 * NT;
      if (x >= ne * NFACE) continue;
      const int e = x / NFACE, fm = x - e * NFACE, f = fm / Nfp;
      const float* g = sG + e * 16;
      const float* a = av[s2];
      const float* bb = bv[s2];
      const float nx = g[8 + f], ny = g[11 + f];
      const float sc = g[5 + f] * g[4];  // -faceJ / J
      float dl[NF];
      if (P == PHYS_ADV) {
        const float an = cax * nx + cay * ny;
        dl[0] = an >= 0.0f ? 0.0f : an * (bb[0] - a[0]);
      } else if (P == PHYS_TM) {
        const float dHx = a[0] - bb[0], dHy = a[1] - bb[1], dEz = a[2] - bb[2];
        const float ez = 0.5f * (-dEz + ny * dHx - nx * dHy);
        dl[0] = ny * ez;
        dl[1] = -nx * ez;
        dl[2] = 0.5f * (-ny * dHx + nx * dHy + dEz);
      } else {
        const float dEx = a[0] - bb[0], dEy = a[1] - bb[1], dHz = a[2] - bb[2];
        const float hz = 0.5f * (-dHz - ny * dEx + nx * dEy);
        dl[0] = -ny * hz;
        dl[1] = nx * hz;
        dl[2] = 0.5f * (-nx * dEy + ny * dEx + dHz);
      }
#pragma unroll
      for (int c = 0; c < NF; ++c) sGam[(e * NF + c) * GSTR + fm] = dl[c] * sc;
    }
    __syncthreads();

    // ---- 4. gamma columns of this thread's row to TMEM (the halves split them;
    //      every lane stores, rows without an element hold finite stale values
    //      whose products land only in their own, discarded, D rows)
    {
      const float* gr = sGam + row * GSTR;
#pragma unroll
      for (int c = 4 * half; c < GC; c += 8) {
        const float4 v = *reinterpret_cast<const float4*>(gr + c);
        float hi[4], lo[4];
        tf32_split(v.x, hi[0], lo[0]);
        tf32_split(v.y, hi[1], lo[1]);
        tf32_split(v.z, hi[2], lo[2]);
        tf32_split(v.w, hi[3], lo[3]);
        tmem_st4(tA + KG + c, hi[0], hi[1], hi[2], hi[3]);
        tmem_st4(tA + KP + KG + c, lo[0], lo[1], lo[2], lo[3]);
      }
    }

    // ---- 5. tensor cores: D = A_hi B_hi + A_hi B_lo + A_lo B_hi
    tmem_wait_st();
    tc_fence_before();
    __syncthreads();
    if (tid == 0) {
      tc_fence_after();
#pragma unroll 1
      for (int s = 0; s < KP / 8; ++s) {
        const uint64_t dBh = smem_desc(bH + s * 256, 128, SBO), dBl = smem_desc(bL + s * 256, 128, SBO);
        tc_mma_tf32_ta(tD, tmem + (uint32_t)(8 * s), dBh, C::kIdesc, s > 0 ? 1u : 0u);
        tc_mma_tf32_ta(tD, tmem + (uint32_t)(8 * s), dBl, C::kIdesc, 1u);
        tc_mma_tf32_ta(tD, tmem + (uint32_t)(KP + 8 * s), dBh, C::kIdesc, 1u);
      }
      tc_commit(&bar[3]);
    }
    ok = __syncthreads_and(mbar_wait(&bar[3], phm, p.status));
    phm ^= 1;
    if (!ok) break;
    tc_fence_after();

    // ---- 6. epilogue: this thread's half row (16 nodes) from its warp's TMEM lanes
    if (j0 < NC) {
      float rhs[16];
      tmem_ld16(tD + lane_base + (uint32_t)j0, rhs);
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
          for (int j = 0; j < jn && j0 + j < Np; ++j) {
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
