// dg_rhs_tc.cuh -- fused RHS + time-stage kernel with the element contractions
// on the 5th-generation tensor cores (tcgen05, TMEM accumulators), FP32 via
// split TF32 (x = hi + lo, both rounded to TF32; 3 products hi*hi + hi*lo + lo*hi).
//
// Formulation.  The kernel evaluates the strong form of the same DG operator,
//   q_t = -(Dx F_x + Dy F_y) + LIFT(-(faceJ / J) (f* - n.F(q-))),
// with strong-form Dr, Ds (Vr V^-1, Vs V^-1).  On straight-sided elements with
// exact quadrature this equals the weak form the reference uses
// (Dr_weak u = -Dr_strong u + LIFT(n_r faceJ u-), to rounding), and it suits
// split-TF32 products: the strong derivative annihilates constants and the
// surface term only carries flux jumps, so the summed terms stay small
// (the weak Dr maps a constant to O(Np) values that the lift then cancels).
// Per-element geometric factors are constant on an element, so they scale the
// operator's inputs instead of its outputs: Dx q = Dr (rx q) + Ds (sx q).
// Every output field of an element is therefore one product of the constant
// operator [Dr | Ds | LIFT] (K = 2 NpP + 3 Nfp, padded to 8) with a K-vector
// built from the element's state, geometry and face fluxes:
//   D^T (rows = element x field, cols = nodes) = A (rows x K) * B^T (K x nodes)
// with A built in shared memory per tile and B = [Dr | Ds | LIFT] (one row per
// output node) loaded once per CTA.  One tcgen05.mma kind::tf32 with M = 128,
// N = 16 or 32, K = 8 per instruction; D lives in TMEM (32 columns).  The 256
// threads then read their rows (one element-field, 16 nodes per thread) with
// tcgen05.ld (two threads per row, 16 columns each) and applies the stage
// update with float4 global traffic.
//
// Operand layout: K-major, no swizzle ("canonical" core matrices of 8 rows x
// 16 bytes): element (row, k) at byte (row/8)*SBO + (k/4)*128 + (row%8)*16 +
// (k%4)*4 with LBO = 128, SBO = (K/4)*128.
#pragma once

#include "dg_rhs.cuh"

namespace dgk {

// ---------------------------------------------------------------- tcgen05 wrappers
__device__ __forceinline__ void tmem_alloc32(uint32_t* dst) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 32;" ::"r"(smem_u32(dst)) : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc32(uint32_t taddr) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 32;" ::"r"(taddr) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tc_mma_tf32(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                            uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void tc_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// 16 / 32 consecutive TMEM columns of the warp's 32 lanes (one row per thread)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
  tmem_ld16(taddr, v);
  tmem_ld16(taddr + 16, v + 16);
}

// shared-memory matrix descriptor: K-major, no swizzle, descriptor version 1
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}

// round to the nearest TF32 value (10 explicit mantissa bits, ties away)
__device__ __forceinline__ float tf32_rn(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}
// split x = hi + lo with both parts exact TF32 values; |x - hi - lo| <= 2^-22 |x|
__device__ __forceinline__ void tf32_split(float x, float& hi, float& lo) {
  hi = tf32_rn(x);
  lo = tf32_rn(x - hi);
}

template <int N, int P>
struct TcConfig {
  using O = Order<N>;
  static constexpr int Np = O::Np, Nfp = O::Nfp, NpP = O::NpP, NFACE = O::Nface;
  static constexpr int Nf = PhysTraits<P>::Nf;
  static constexpr int kThreads = 256;                 // two threads per A/D row (row = tid % 128)
  static constexpr int TE = 128 / Nf;                  // elements per tile (rows = TE * Nf <= 128)
  static constexpr int ESTR = Nf * NpP;
  static constexpr int KB = NpP;                       // start of the beta columns
  static constexpr int KG = 2 * NpP;                   // start of the lifted (gamma) columns
  static constexpr int KP = (2 * NpP + NFACE + 7) / 8 * 8;  // contraction length
  static constexpr int NC = Np <= 16 ? 16 : 32;        // MMA N (output nodes, padded)
  static constexpr int SBO = (KP / 4) * 128;           // bytes between 8-row groups
  static constexpr uint32_t kBBytes = NC * KP * 4;     // one split of B
  static constexpr uint32_t kABytes = 128 * KP * 4;    // one split of A
  static constexpr uint32_t kQ = TE * ESTR * 4, kG = TE * 16 * 4, kN = TE * 16;
  static constexpr uint32_t kBuf = kQ + kG + kN;
  static constexpr uint32_t oBar = 0;                  // 4 mbarriers + TMEM address
  static constexpr uint32_t oB = 64;
  static constexpr uint32_t oA = oB + 2 * kBBytes;
  static constexpr uint32_t oBuf = oA + 2 * kABytes;
  static constexpr uint32_t kSmem = oBuf + 2 * kBuf;
  static constexpr int kItems = (TE * NFACE + kThreads - 1) / kThreads;  // face nodes per thread
  static constexpr int kRes = NpP < 16 ? NpP / 4 : 4;  // residual float4s a thread prefetches
  // instruction descriptor: D f32, A/B tf32, both K-major, N >> 3, M >> 4
  static constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(NC >> 3) << 17) |
                                     ((uint32_t)(128 >> 4) << 24);
};

template <int SBO>
__device__ __forceinline__ uint32_t op_off(int row, int k) {  // float offset in an operand
  return (uint32_t)((row >> 3) * (SBO / 4) + (k >> 2) * 32 + (row & 7) * 4 + (k & 3));
}

template <int N, int P>
__global__ void __launch_bounds__(256) dg_rhs_tc_kernel(const RhsParams p) {
  using C = TcConfig<N, P>;
  constexpr int Np = C::Np, Nfp = C::Nfp, NpP = C::NpP, NFACE = C::NFACE, NF = C::Nf;
  constexpr int TE = C::TE, ESTR = C::ESTR, KP = C::KP, NC = C::NC, SBO = C::SBO, NT = C::kThreads;

  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + C::oBar);  // [0],[1] tiles, [2] operator, [3] MMA
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + C::oBar + 32);
  float* Bhi = reinterpret_cast<float*>(smem + C::oB);
  float* Ahi = reinterpret_cast<float*>(smem + C::oA);
  float* Alo = Ahi + C::kABytes / 4;
  auto bufQ = [&](int b) { return reinterpret_cast<float*>(smem + C::oBuf + b * C::kBuf); };
  auto bufG = [&](int b) { return reinterpret_cast<float*>(smem + C::oBuf + b * C::kBuf + C::kQ); };
  auto bufN = [&](int b) { return reinterpret_cast<int4*>(smem + C::oBuf + b * C::kBuf + C::kQ + C::kG); };

  const int tid = threadIdx.x, warp = tid >> 5;
  const int row = tid & 127, half = tid >> 7, fo = row % NF, er = row / NF;  // this thread's A/D row
  const int ntiles = (p.K + TE - 1) / TE;
  const float* qin = static_cast<const float*>(p.q_in);
  const double tnow = p.t_dev ? *p.t_dev + p.t : p.t;
  // FP32 copies of the scalar parameters (rhs_dispatch<float>)
  const float cax = p.fax, cay = p.fay, cca = p.fca, ccb = p.fcb, cdt = p.fdt;

  if (tid == 0) {
    for (int i = 0; i < 4; ++i) mbar_init(&bar[i], 1);
    fence_barrier_init();
  }
  if (warp == 0) tmem_alloc32(tmem_slot);
  // zero A once: padding columns and unused rows are never written again
  for (int x = tid; x < (int)(2 * C::kABytes / 4); x += NT) Ahi[x] = 0.0f;
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  auto issue = [&](int tile, int b) {
    const int k0 = tile * TE, ne = min(TE, p.K - k0);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    const uint32_t bq = ne * ESTR * 4, bg = ne * 16 * 4, bn = ne * 16;
    mbar_arrive_expect_tx(&bar[b], bq + bg + bn);
    bulk_g2s(bufQ(b), qin + (size_t)k0 * ESTR, bq, &bar[b]);
    bulk_g2s(bufG(b), static_cast<const float*>(p.geom) + (size_t)k0 * 16, bg, &bar[b]);
    bulk_g2s(bufN(b), p.nbr + k0, bn, &bar[b]);
  };
  if (tid == 0) {
    mbar_arrive_expect_tx(&bar[2], 2 * C::kBBytes);
    bulk_g2s(Bhi, p.mats_tc, 2 * C::kBBytes, &bar[2]);
    if ((int)blockIdx.x < ntiles) issue(blockIdx.x, 0);
  }
  bool ok = mbar_wait(&bar[2], 0, p.status);
  ok = __syncthreads_and(ok);

  const uint32_t aH = smem_u32(Ahi), aL = smem_u32(Alo), bH = smem_u32(Bhi), bL = bH + C::kBBytes;
  const int j0 = 16 * half;                 // first node of this thread's half row
  const int jn = min(NpP - j0, 16);         // nodes of the half row (multiple of 4; <= 0: none)
  float* out = static_cast<float*>(p.out);
  float* aux = static_cast<float*>(p.aux);
  uint32_t ph[2] = {0, 0}, phm = 0;
  int it = 0;
  for (int tile = blockIdx.x; ok && tile < ntiles; tile += gridDim.x, ++it) {
    const int b = it & 1;
    const int k0 = tile * TE, ne = min(TE, p.K - k0);
    const int nxt = tile + gridDim.x;
    if (tid == 0 && nxt < ntiles) issue(nxt, b ^ 1);
    ok = __syncthreads_and(mbar_wait(&bar[b], ph[b], p.status));
    if (!ok) break;
    ph[b] ^= 1;
    const float* sQ = bufQ(b);
    const float* sG = bufG(b);
    const int4* sN = bufN(b);
    const bool mine = er < ne && j0 < NC && jn > 0;
    const size_t base = (size_t)(k0 + er) * ESTR + (size_t)fo * NpP + j0;

    // ---- 1. issue the loads whose latency the A construction hides: the
    //      residual of this thread's half row and all neighbour gathers
    float4 r4[C::kRes];
    if (p.mode == MODE_LSERK && mine) {
#pragma unroll
      for (int j = 0; j < C::kRes; ++j)
        if (4 * j < jn) r4[j] = *reinterpret_cast<const float4*>(aux + base + 4 * j);
    }
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
        bv[s2][0] = (float)adv_exact(p, tnow, xx, yy);
      } else if (P == PHYS_TM) {  // PEC: H+ = H-, Ez+ = -Ez-
        bv[s2][0] = av[s2][0]; bv[s2][1] = av[s2][1]; bv[s2][2] = -av[s2][2];
      } else {                    // PEC: E+ = -E-, Hz+ = Hz-
        bv[s2][0] = -av[s2][0]; bv[s2][1] = -av[s2][1]; bv[s2][2] = av[s2][2];
      }
    }

    // ---- 2. volume columns of A, strong form: row (e, f) holds
    //      alpha_j = -(rx F_x + ry F_y)_j, beta_j = -(sx F_x + sy F_y)_j of the
    //      flux F of output field f; 4 nodes per 16-byte store
    if (er < ne) {
      const float* g = sG + er * 16;
      const float rx = g[0], ry = g[1], sx = g[2], sy = g[3];
      const float* qe = sQ + er * ESTR;
#pragma unroll 2
      for (int c = half; c < NpP / 4; c += 2) {
        const int j = 4 * c;
        float al[4], be[4];
        if (P == PHYS_ADV) {
          const float4 u = *reinterpret_cast<const float4*>(qe + j);
          const float cr = -(cax * rx + cay * ry), cs = -(cax * sx + cay * sy);
          al[0] = cr * u.x; al[1] = cr * u.y; al[2] = cr * u.z; al[3] = cr * u.w;
          be[0] = cs * u.x; be[1] = cs * u.y; be[2] = cs * u.z; be[3] = cs * u.w;
        } else {
          const float4 q0 = *reinterpret_cast<const float4*>(qe + j);
          const float4 q1 = *reinterpret_cast<const float4*>(qe + NpP + j);
          const float4 q2 = *reinterpret_cast<const float4*>(qe + 2 * NpP + j);
          const float a0[4] = {q0.x, q0.y, q0.z, q0.w}, a1[4] = {q1.x, q1.y, q1.z, q1.w};
          const float a2[4] = {q2.x, q2.y, q2.z, q2.w};
#pragma unroll
          for (int l = 0; l < 4; ++l) {
            if (P == PHYS_TM) {  // F(Hx) = (0, Ez), F(Hy) = (-Ez, 0), F(Ez) = (-Hy, Hx)
              if (fo == 0) { al[l] = -ry * a2[l]; be[l] = -sy * a2[l]; }
              else if (fo == 1) { al[l] = rx * a2[l]; be[l] = sx * a2[l]; }
              else { al[l] = rx * a1[l] - ry * a0[l]; be[l] = sx * a1[l] - sy * a0[l]; }
            } else {             // F(Ex) = (0, -Hz), F(Ey) = (Hz, 0), F(Hz) = (Ey, -Ex)
              if (fo == 0) { al[l] = ry * a2[l]; be[l] = sy * a2[l]; }
              else if (fo == 1) { al[l] = -rx * a2[l]; be[l] = -sx * a2[l]; }
              else { al[l] = ry * a0[l] - rx * a1[l]; be[l] = sy * a0[l] - sx * a1[l]; }
            }
          }
        }
#pragma unroll
        for (int l = 0; l < 4; ++l)
          if (j + l >= Np) al[l] = be[l] = 0.0f;  // padding nodes
        float ah[4], alo[4], bh[4], blo[4];
#pragma unroll
        for (int l = 0; l < 4; ++l) {
          tf32_split(al[l], ah[l], alo[l]);
          tf32_split(be[l], bh[l], blo[l]);
        }
        const uint32_t oa = op_off<SBO>(row, j), ob = op_off<SBO>(row, C::KB + j);
        *reinterpret_cast<float4*>(Ahi + oa) = make_float4(ah[0], ah[1], ah[2], ah[3]);
        *reinterpret_cast<float4*>(Alo + oa) = make_float4(alo[0], alo[1], alo[2], alo[3]);
        *reinterpret_cast<float4*>(Ahi + ob) = make_float4(bh[0], bh[1], bh[2], bh[3]);
        *reinterpret_cast<float4*>(Alo + ob) = make_float4(blo[0], blo[1], blo[2], blo[3]);
      }
    }

    // ---- 3. lifted columns: gamma = -(faceJ / J) (f* - n.F(q-)) per output field
#pragma unroll
    for (int s2 = 0; s2 < C::kItems; ++s2) {
      const int x = tid + s2 * NT;
      if (x >= ne * NFACE) continue;
      const int e = x / NFACE, fm = x - e * NFACE, f = fm / Nfp;
      const float* g = sG + e * 16;
      const float* a = av[s2];
      const float* bb = bv[s2];
      const float nx = g[8 + f], ny = g[11 + f];
      const float sc = g[5 + f] * g[4];  // -faceJ/J
      float dl[NF];
      if (P == PHYS_ADV) {
        const float an = cax * nx + cay * ny;
        dl[0] = an >= 0.0f ? 0.0f : an * (bb[0] - a[0]);
      } else if (P == PHYS_TM) {
        // Ez* - Ez- = (-dEz + ny dHx - nx dHy)/2, n x H* - n x H- = (ny (Hx+ - Hx-) - nx (Hy+ - Hy-) + dEz)/2
        const float dHx = a[0] - bb[0], dHy = a[1] - bb[1], dEz = a[2] - bb[2];
        const float ez = 0.5f * (-dEz + ny * dHx - nx * dHy);
        dl[0] = ny * ez;
        dl[1] = -nx * ez;
        dl[2] = 0.5f * (-ny * dHx + nx * dHy + dEz);
      } else {
        // Hz* - Hz- = (-dHz - ny dEx + nx dEy)/2, (n x E)* - n x E- = (-nx dEy + ny dEx + dHz)/2
        const float dEx = a[0] - bb[0], dEy = a[1] - bb[1], dHz = a[2] - bb[2];
        const float hz = 0.5f * (-dHz - ny * dEx + nx * dEy);
        dl[0] = -ny * hz;
        dl[1] = nx * hz;
        dl[2] = 0.5f * (-nx * dEy + ny * dEx + dHz);
      }
#pragma unroll
      for (int c = 0; c < NF; ++c) {
        const uint32_t o = op_off<SBO>(e * NF + c, C::KG + fm);
        float h, l;
        tf32_split(dl[c] * sc, h, l);
        Ahi[o] = h;
        Alo[o] = l;
      }
    }

    // ---- 4. tensor cores: D = A_hi B_hi + A_hi B_lo + A_lo B_hi
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      tc_fence_after();
#pragma unroll 1
      for (int s = 0; s < KP / 8; ++s) {
        const uint64_t dAh = smem_desc(aH + s * 256, 128, SBO), dAl = smem_desc(aL + s * 256, 128, SBO);
        const uint64_t dBh = smem_desc(bH + s * 256, 128, SBO), dBl = smem_desc(bL + s * 256, 128, SBO);
        tc_mma_tf32(tmem, dAh, dBh, C::kIdesc, s > 0 ? 1u : 0u);
        tc_mma_tf32(tmem, dAh, dBl, C::kIdesc, 1u);
        tc_mma_tf32(tmem, dAl, dBh, C::kIdesc, 1u);
      }
      tc_commit(&bar[3]);
    }
    ok = __syncthreads_and(mbar_wait(&bar[3], phm, p.status));
    phm ^= 1;
    if (!ok) break;
    tc_fence_after();

    // ---- 5. epilogue: this thread's half row (16 nodes) from its warp's TMEM lanes
    if (j0 < NC) {
      float rhs[16];
      tmem_ld16(tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)j0, rhs);
      if (mine) {
        const float* qrow = sQ + er * ESTR + fo * NpP + j0;
        auto rv = [&](int j) { return (j0 + j) < Np ? rhs[j] : 0.0f; };
        if (p.mode == MODE_RHS) {
#pragma unroll
          for (int j = 0; j < 16; j += 4)
            if (j < jn) *reinterpret_cast<float4*>(out + base + j) = make_float4(rv(j), rv(j + 1), rv(j + 2), rv(j + 3));
        } else if (p.mode == MODE_LSERK) {
          const float ca = cca, cb = ccb, dt = cdt;
#pragma unroll
          for (int j = 0; j < 16; j += 4)
            if (j < jn) {
              const float4 qv = *reinterpret_cast<const float4*>(qrow + j);
              float4 r = r4[j / 4];
              r.x = ca * r.x + dt * rv(j);
              r.y = ca * r.y + dt * rv(j + 1);
              r.z = ca * r.z + dt * rv(j + 2);
              r.w = ca * r.w + dt * rv(j + 3);
              *reinterpret_cast<float4*>(aux + base + j) = r;
              *reinterpret_cast<float4*>(out + base + j) =
                  make_float4(qv.x + cb * r.x, qv.y + cb * r.y, qv.z + cb * r.z, qv.w + cb * r.w);
            }
        } else {
          float* q0 = static_cast<float*>(p.q0);
          const float co = cca, wa = ccb;
#pragma unroll
          for (int j = 0; j < 16; ++j) {  // constant indices keep rhs[] in registers
            if (j >= jn || j0 + j >= Np) continue;
            const size_t o = base + j;
            if (p.stage == 0) {
              aux[o] = rhs[j];
              out[o] = qrow[j] + co * rhs[j];
            } else if (p.stage < 3) {
              aux[o] = aux[o] + wa * rhs[j];
              out[o] = q0[o] + co * rhs[j];
            } else {
              q0[o] = q0[o] + co * (aux[o] + rhs[j]);
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
    tmem_dealloc32(tmem);
  }
}

}  // namespace dgk
