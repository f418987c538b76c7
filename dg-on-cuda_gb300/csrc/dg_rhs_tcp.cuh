// dg_rhs_tcp.cuh -- warp-specialized, software-pipelined version of the
// tensor-memory stage kernel (dg_rhs_tct.cuh) for the three-field Maxwell
// systems.  Same operator, formulation (strong form, split TF32, A in TMEM)
// and tile layout (32 elements, field-major rows); the work of a tile is split
// into stages run by different warps on different tiles at the same time:
//
//   MMA   warp 15, lane 0   tcgen05.mma + commit
//   LOAD  warp 15, lane 1   bulk loads of the tiles (NB buffers), as far ahead
//                           as the epilogue releases buffers
//   FACE  warps 3, 7, 11    face tasks (element, face): the neighbour gathers
//                           of tile i + 1 are issued before the flux jumps of
//                           tile i are computed; gamma rows in shared memory
//                           (2 buffers)
//   BUILD warps 0-2, 4-6    alpha / beta / gamma columns of A -> TMEM (2 A buffers)
//   EPI   warps 8-10, 12-14 D -> stage update and global stores (2 D buffers)
//
// BUILD and EPI warps sit on lane quadrants 0..2 (the field of their rows);
// FACE and CTRL use quadrant 3.  Every hand-off is an mbarrier with a bounded
// wait: a wait that expires records the error in the status word and its
// thread stops waiting from then on, so a fault elsewhere cannot hang the
// CTA.  One CTA per SM: the 512 TMEM columns hold A x 2 and D x 2 (each D =
// D_a | D_b of 2 NC + NC columns, two MMAs per K step as in dg_rhs_tct).
//
// Barrier phases (tile i of the CTA, buffers s = i % NB, g = i % 2):
//   dfull[s]  bulk copy of tile i landed            -> FACE (from tile i - 1), BUILD, EPI
//   gfull[g]  gamma rows of tile i written          -> BUILD
//   gempty[g] gamma rows of tile i consumed         -> FACE (tile i + 2)
//   afull[g]  A of tile i complete in TMEM          -> CTRL
//   mdone[g]  MMA of tile i complete (commit)       -> EPI, BUILD (tile i + 2)
//   dempty[g] D of tile i read                      -> CTRL (tile i + 2)
//   dfree[s]  tile buffer of tile i released        -> LOAD (tile i + NB)
// No waiter can fall a whole phase behind: each next completion depends on
// the waiter's own later progress.
#pragma once

#include "dg_rhs_tct.cuh"

namespace dgk {

template <int N, int P>
struct TcpConfig {
  using T = TctConfig<N, P>;
  static constexpr int Np = T::Np, Nfp = T::Nfp, NpP = T::NpP, NFACE = T::NFACE, Nf = T::Nf;
  static constexpr int TE = T::TE, ROWS = T::ROWS, ESTR = T::ESTR, KG = T::KG, KP = T::KP, GC = T::GC;
  static constexpr int NC = T::NC, SBO = T::SBO;
  static constexpr int kThreads = 512;
  static constexpr uint32_t kTmemCols = 512;
  static constexpr uint32_t kBBytes = T::kBBytes;
  static constexpr uint32_t kQ = T::kQ, kG = T::kG, kN = T::kN, kBuf = T::kBuf;
  static constexpr uint32_t kGam = T::kGam;  // column-major [GC][ROWS]
  // tile buffers: a buffer stays in use from its load through the face,
  // build, MMA and epilogue stages, so the ring depth bounds the tile period
  static constexpr int NB = 4;
  static_assert(NB <= 8, "barrier slots");
  // shared memory: 27 mbarriers + TMEM address | B hi, lo | gamma x 2 | tiles x NB
  static constexpr uint32_t oBar = 0;
  static constexpr uint32_t oB = 256;
  static constexpr uint32_t oGam = oB + 2 * kBBytes;
  static constexpr uint32_t oBuf = oGam + 2 * kGam;
  static constexpr uint32_t kSmem = oBuf + NB * kBuf;
  // requested at launch: more than half an SM's 233472 B, so a second CTA
  // (whose 512-column TMEM allocation would have to wait) is never co-resident
  static constexpr uint32_t kSmemLaunch = kSmem > 116800u ? kSmem : 116800u;
  static constexpr uint32_t kIdesc = T::kIdesc, kIdesc2 = T::kIdesc2;
  static_assert(Nf == 3 && ROWS == 96, "three fields on lane quadrants 0..2");
  static_assert(4 * KP + 6 * NC <= 512, "TMEM budget");
};

// mbarrier slots
enum : int { TB_DFULL = 0, TB_GFULL = 8, TB_GEMPTY = 10, TB_AFULL = 12, TB_MDONE = 14, TB_DEMPTY = 16,
             TB_DFREE = 18, TB_BFULL = 26, TB_COUNT = 27 };  // tile-buffer slots sized for up to 8 buffers

template <int N, int P>
__global__ void __launch_bounds__(512, 1) dg_rhs_tcp_kernel(const RhsParams p) {
  using C = TcpConfig<N, P>;
  constexpr int Np = C::Np, NpP = C::NpP, TE = C::TE, ESTR = C::ESTR, NB = C::NB;
  constexpr int KP = C::KP, KG = C::KG, GC = C::GC, NC = C::NC, SBO = C::SBO, ROWS = C::ROWS;

  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + C::oBar);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + C::oBar + 8 * TB_COUNT);
  float* Bhi = reinterpret_cast<float*>(smem + C::oB);
  auto gam = [&](int g) { return reinterpret_cast<float*>(smem + C::oGam + g * C::kGam); };
  auto bufQ = [&](int s) { return reinterpret_cast<float*>(smem + C::oBuf + s * C::kBuf); };
  auto bufR = [&](int s) { return reinterpret_cast<float*>(smem + C::oBuf + s * C::kBuf + C::kQ); };
  auto bufG = [&](int s) { return reinterpret_cast<float*>(smem + C::oBuf + s * C::kBuf + 2 * C::kQ); };
  auto bufN = [&](int s) {
    return reinterpret_cast<int4*>(smem + C::oBuf + s * C::kBuf + 2 * C::kQ + C::kG);
  };

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int quad = warp & 3;
  const int ntiles = (p.K + TE - 1) / TE;
  const int nt = ntiles > (int)blockIdx.x ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
  const float* qin = static_cast<const float*>(p.q_in);
  const float cax = p.fax, cay = p.fay, cca = p.fca, ccb = p.fcb, cdt = p.fdt;
  const bool aux_tile = p.mode == MODE_LSERK;

  grid_dep_launch();  // the next stage may be scheduled; it waits for this grid before its reads
  if (tid == 0) {
    for (int s = 0; s < NB; ++s) {
      mbar_init(&bar[TB_DFULL + s], 1);
      mbar_init(&bar[TB_DFREE + s], 192);
    }
    for (int g = 0; g < 2; ++g) {
      mbar_init(&bar[TB_GFULL + g], 96);
      mbar_init(&bar[TB_GEMPTY + g], 192);
      mbar_init(&bar[TB_AFULL + g], 192);
      mbar_init(&bar[TB_MDONE + g], 1);
      mbar_init(&bar[TB_DEMPTY + g], 192);
    }
    mbar_init(&bar[TB_BFULL], 1);
    fence_barrier_init();
  }
  if (warp == 0) tmem_alloc_n(tmem_slot, C::kTmemCols);
  // gamma padding columns are never written by the face tasks
  for (int x = tid; x < (int)(2 * C::kGam / 4); x += C::kThreads) gam(0)[x] = 0.0f;
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  const uint32_t lane_base = (uint32_t)(quad * 32) << 16;
  auto colA = [&](int g) { return (uint32_t)(g * 2 * KP); };        // A_hi of buffer g (A_lo at + KP)
  auto colD = [&](int g) { return (uint32_t)(4 * KP + g * 3 * NC); };  // 3 accumulators of buffer g

  bool ok = true;  // this thread's waits have all completed (a wait that expires turns it off)
  auto wait = [&](int slot, uint32_t parity) {
    if (ok) ok = mbar_wait_backoff(&bar[slot], parity, p.status);
  };
  auto tile_of = [&](int i) { return (int)blockIdx.x + i * (int)gridDim.x; };

  if (warp == 15) {
    if (lane == 1) {
      // ============================================================== LOAD
      grid_dep_wait();  // the state and the residual are the previous launch's output
      for (int i = 0; i < nt; ++i) {
        const int s = i % NB, k0 = tile_of(i) * TE, ne = min(TE, p.K - k0);
        if (i >= NB) wait(TB_DFREE + s, ((i - NB) / NB) & 1);  // epilogue of tile i - NB done
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        const uint32_t bq = ne * ESTR * 4, bg = ne * 16 * 4, bn = ne * 16;
        mbar_arrive_expect_tx(&bar[TB_DFULL + s], bq + (aux_tile ? bq : 0) + bg + bn);
        bulk_g2s(bufQ(s), qin + (size_t)k0 * ESTR, bq, &bar[TB_DFULL + s]);
        if (aux_tile) bulk_g2s(bufR(s), static_cast<const float*>(p.aux) + (size_t)k0 * ESTR, bq, &bar[TB_DFULL + s]);
        bulk_g2s(bufG(s), static_cast<const float*>(p.geom) + (size_t)k0 * 16, bg, &bar[TB_DFULL + s]);
        bulk_g2s(bufN(s), p.nbr + k0, bn, &bar[TB_DFULL + s]);
      }
    } else if (lane == 0) {
      // ============================================================== MMA
      mbar_arrive_expect_tx(&bar[TB_BFULL], 2 * C::kBBytes);
      bulk_g2s(Bhi, p.mats_tc, 2 * C::kBBytes, &bar[TB_BFULL]);
      wait(TB_BFULL, 0);
      const uint32_t bH = smem_u32(Bhi);  // B_hi, with B_lo directly after it
      for (int i = 0; i < nt; ++i) {
        const int g = i & 1;
        wait(TB_AFULL + g, (i >> 1) & 1);
        if (i >= 2) wait(TB_DEMPTY + g, ((i - 2) >> 1) & 1);
        tc_fence_after();
        const uint32_t tD = tmem + colD(g), tAh = tmem + colA(g), tAl = tAh + KP;
#pragma unroll
        for (int s2 = 0; s2 < KP / 8; ++s2) {
          const uint64_t dB = smem_desc(bH + s2 * 256, 128, SBO);  // rows: B_hi then B_lo
          const uint32_t acc = s2 > 0 ? 1u : 0u;
          tc_mma_tf32_ta(tD, tAh + (uint32_t)(8 * s2), dB, C::kIdesc2, acc);
          tc_mma_tf32_ta(tD + 2 * NC, tAl + (uint32_t)(8 * s2), dB, C::kIdesc, acc);
        }
        tc_commit(&bar[TB_MDONE + g]);
      }
      // the last MMA completes before TMEM is released
      if (nt > 0) wait(TB_MDONE + ((nt - 1) & 1), ((nt - 1) >> 1) & 1);
    }
  } else if (quad == 3) {
    // ================================================================ FACE
    const int fid = (warp >> 2) * 32 + lane;  // 0..95: (face, element) task of each tile
    const int f = fid / TE, e = fid - f * TE;
    constexpr int Nfp = C::Nfp;
    float bc[Nfp][3], bx[Nfp][3];  // neighbour traces of the current / next tile
    int nbc = -1, nbx = -1;
    auto gather = [&](int i, float (&b)[Nfp][3], int& nb) {
      const int s = i % NB, k0 = tile_of(i) * TE, ne = min(TE, p.K - k0);
      wait(TB_DFULL + s, (i / NB) & 1);
      nb = -1;
      if (e < ne) nb = face_gather<N, P>(p, e, f, k0, ne, bufQ(s), bufN(s), qin, b);
    };
    // one step: issue the gathers of tile i + 1 into `nxt`, then compute tile
    // i from `cur` (gathered one step earlier); unrolled by two so that the
    // buffers swap roles without a register copy that would wait for the loads
    auto step = [&](int i, float (&cur)[Nfp][3], int nbcur, float (&nxt)[Nfp][3], int& nbnxt) {
      const int s = i % NB, g = i & 1, k0 = tile_of(i) * TE, ne = min(TE, p.K - k0);
      if (i + 1 < nt) gather(i + 1, nxt, nbnxt);
      if (i >= 2) wait(TB_GEMPTY + g, ((i - 2) >> 1) & 1);
      if (e < ne) face_flux<N, P>(e, f, nbcur, bufQ(s), bufG(s), cur, gam(g), cax, cay);
      mbar_arrive(&bar[TB_GFULL + g]);
    };
    grid_dep_wait();  // neighbour traces are read from the previous launch's output
    if (nt > 0) gather(0, bc, nbc);
    for (int i = 0; i < nt; i += 2) {
      step(i, bc, nbc, bx, nbx);
      if (i + 1 < nt) step(i + 1, bx, nbx, bc, nbc);
    }
  } else if (warp < 8) {
    // ================================================================ BUILD
    const int half = warp >> 2, fo = quad, er = lane;
    const uint32_t tRow = tmem + lane_base;
    // zero both A buffers of this warp's lanes once (padding never rewritten)
    for (int c = 4 * half; c < 4 * KP; c += 8) tmem_st4(tRow + c, 0.0f, 0.0f, 0.0f, 0.0f);
    for (int i = 0; i < nt; ++i) {
      const int s = i % NB, g = i & 1, k0 = tile_of(i) * TE, ne = min(TE, p.K - k0);
      wait(TB_DFULL + s, (i / NB) & 1);
      if (i >= 2) wait(TB_MDONE + g, ((i - 2) >> 1) & 1);  // MMA of tile i - 2 no longer reads A[g]
      tc_fence_after();
      __syncwarp();  // tcgen05.st below is warp-collective
      const float* sQ = bufQ(s);
      const float* sG = bufG(s);
      const uint32_t tA = tRow + colA(g);
      {
        const bool valid = er < ne;
        const int erc = valid ? er : 0;
        const float* gg = sG + erc * 16;
        const float mx = half == 0 ? gg[0] : gg[2], my = half == 0 ? gg[1] : gg[3];
        const float* qe = sQ + erc * ESTR;
        const uint32_t col0 = (uint32_t)(half * NpP);
#pragma unroll
        for (int j = 0; j < NpP; j += 4) {
          float v[4];
          if (fo < 2) {  // Ex, Ey (TE) / Hx, Hy (TM): flux of the third field only
            const float4 q2 = *reinterpret_cast<const float4*>(qe + 2 * NpP + j);
            const float cm = (P == PHYS_TE) ? (fo == 0 ? my : -mx) : (fo == 0 ? -my : mx);
            v[0] = cm * q2.x; v[1] = cm * q2.y; v[2] = cm * q2.z; v[3] = cm * q2.w;
          } else {       // Hz (TE): F = (Ey, -Ex);  Ez (TM): F = (-Hy, Hx)
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
      wait(TB_GFULL + g, (i >> 1) & 1);
      __syncwarp();
      {
        const float* gr = gam(g) + fo * TE + er;
#pragma unroll
        for (int c = 4 * half; c < GC; c += 8) {
          const float v[4] = {gr[c * ROWS], gr[(c + 1) * ROWS], gr[(c + 2) * ROWS], gr[(c + 3) * ROWS]};
          tmem_st4_split(tA + KG + c, tA + KP + KG + c, v);
        }
      }
      tmem_wait_st();
      tc_fence_before();
      mbar_arrive(&bar[TB_GEMPTY + g]);
      mbar_arrive(&bar[TB_AFULL + g]);
    }
  } else {
    // ================================================================ EPI
    const int half = (warp >> 2) & 1, fo = quad, er = lane;
    const int j0 = 16 * half, jn = min(NpP - j0, 16);
    float* out = static_cast<float*>(p.out);
    float* aux = static_cast<float*>(p.aux);
    grid_dep_wait();  // the previous launch reads the buffers written here
    for (int i = 0; i < nt; ++i) {
      const int s = i % NB, g = i & 1, k0 = tile_of(i) * TE, ne = min(TE, p.K - k0);
      wait(TB_DFULL + s, (i / NB) & 1);
      wait(TB_MDONE + g, (i >> 1) & 1);
      tc_fence_after();
      __syncwarp();  // tcgen05.ld below is warp-collective
      if (j0 < NC) {
        float rhs[16], r1[16], r2[16];
        tmem_ld16(tmem + lane_base + colD(g) + (uint32_t)j0, rhs);
        tmem_ld16(tmem + lane_base + colD(g) + (uint32_t)(NC + j0), r1);
        tmem_ld16(tmem + lane_base + colD(g) + (uint32_t)(2 * NC + j0), r2);
#pragma unroll
        for (int j = 0; j < 16; ++j) rhs[j] += r1[j] + r2[j];
        if (er < ne && jn > 0) {
          const size_t base = (size_t)(k0 + er) * ESTR + (size_t)fo * NpP + j0;
          const float* qrow = bufQ(s) + er * ESTR + fo * NpP + j0;
          auto rv = [&](int j) { return (j0 + j) < Np ? rhs[j] : 0.0f; };
          if (p.mode == MODE_RHS) {
#pragma unroll
            for (int j = 0; j < 16; j += 4)
              if (j < jn)
                *reinterpret_cast<float4*>(out + base + j) = make_float4(rv(j), rv(j + 1), rv(j + 2), rv(j + 3));
          } else if (p.mode == MODE_LSERK) {
            const float* rrow = bufR(s) + er * ESTR + fo * NpP + j0;
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
                if (j0 + j + 3 >= Np) { r.w = 0.0f; o4.w = 0.0f; }  // padding nodes are written as 0
                if (j0 + j + 2 >= Np) { r.z = 0.0f; o4.z = 0.0f; }
                if (j0 + j + 1 >= Np) { r.y = 0.0f; o4.y = 0.0f; }
                *reinterpret_cast<float4*>(aux + base + j) = r;
                *reinterpret_cast<float4*>(out + base + j) = o4;
              }
          } else {
            float* q0 = static_cast<float*>(p.q0);
#pragma unroll
            for (int j = 0; j < 16; ++j) {
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
      mbar_arrive(&bar[TB_DEMPTY + g]);
      mbar_arrive(&bar[TB_DFREE + s]);
    }
  }
  // ---- release TMEM once every role is done (the last MMA was waited for)
  __syncwarp();  // warp 15: lanes 1..31 wait for the CTRL lane
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc_n(tmem, C::kTmemCols);
  }
}

}  // namespace dgk
