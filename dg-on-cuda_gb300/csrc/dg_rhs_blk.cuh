// dg_rhs_blk.cuh -- register-blocked FP32 variant of the fused RHS + stage
// kernel (dg_rhs.cuh): same operator, fluxes and epilogues, laid out as a
// small dense product per element so that every shared-memory load feeds many
// FMAs.
//
// Per element and field c the weak-form stage is
//   rhs_c[i] = sum_c' (Gr_cc' ur_c'[i] + Gs_cc' us_c'[i]) + sum_m LIFT[i][m] g_c[m],
//   ur_c' = Dr q_c',  us_c' = Ds q_c',  g_c = -(faceJ / J) f*_c  (face flux),
// with Gr, Gs the physics' combination of rx, ry, sx, sy.  Thread (slot s,
// group g) owns nodes 4g .. 4g+3 of EPT elements of the tile (elements s and
// s + NTE) and all their fields:
//   * the element's field values are read 4 columns at a time (float4), the
//     operators as rows of the transposed matrices padded to NpP columns, so
//     one float4 of Dr^T / Ds^T / LIFT^T row j covers the thread's 4 nodes;
//   * Maxwell: the curl of the first two fields is accumulated as one
//     product pair Dr u + Ds v, u and v their combination with the element's
//     (constant) rx, ry, sx, sy, next to Dr q2 and Ds q2 for the gradient of
//     the third field: 3 x 4 x EPT accumulators and 4 FMAs per node and
//     column instead of 6 (advection: Dr q and Ds q);
//   * the face fluxes are stored already scaled by -faceJ/J so LIFT
//     accumulates straight into rhs;
//   * columns past Np are skipped at compile time (padding never enters a
//     valid output) and padded output nodes are written as 0.
// Two thread mappings (MAP):
//   0: the NG = NpP/4 groups of an element are consecutive threads (a warp
//      covers ~32/NG elements and reads NG different operator chunks);
//   1: a warp holds one node group of 32 consecutive elements, so every
//      operator load is warp-uniform (a broadcast) and the 32 element rows of
//      a state load fall in distinct banks when NG is odd.
// Tiles are double-buffered: the bulk copy of the next tile (state, residual,
// geometry, neighbours) is in flight while the current one is computed.
#pragma once

#include "dg_rhs.cuh"

namespace dgk {

template <int N, int P, int EPT_, int MAP_ = 0>
struct BlkConfig {
  using O = Order<N>;
  static constexpr int Np = O::Np, NpP = O::NpP, NFACE = O::Nface;
  static constexpr int EPT = EPT_, MAP = MAP_;
  static constexpr int NG = NpP / 4;                 // 4-node groups per element
  static constexpr int RW = (8 / NG) > 0 ? 8 / NG : 1;  // MAP 1: rows of 32 elements per CTA
  static constexpr int kThreads = MAP == 0 ? 256 : NG * 32 * RW;
  static constexpr int kMinBlocks = EPT == 2 ? 2 : 3;
  static constexpr int NTE = MAP == 0 ? kThreads / NG : 32 * RW;  // element slots per CTA
  static constexpr int TE = NTE * EPT;               // elements per tile
  static constexpr int Nf = PhysTraits<P>::Nf;
  static constexpr int ESTR = Nf * NpP;              // state stride per element
  static constexpr int FSTR = (NFACE + 3) / 4 * 4;   // padded face-flux row
  static constexpr int kFItems = (TE * O::Nfp + kThreads - 1) / kThreads;  // (element, face-node) items per thread
  static constexpr int KB = 2 * Np + NFACE;          // operator rows: Dr^T | Ds^T | LIFT^T
  static constexpr uint32_t kMat = KB * NpP * 4;
  // the LSERK residual tile is prefetched with the state tile when the extra
  // buffers keep the CTA count per SM (one element per thread)
  static constexpr bool kAuxTile = EPT == 1;
  static constexpr uint32_t kQ = TE * ESTR * 4, kA = kAuxTile ? kQ : 0, kG = TE * 16 * 4, kN = TE * 16;
  static constexpr uint32_t kBuf = kQ + kA + kG + kN;  // one tile buffer: state | residual | geometry | neighbours
  static constexpr uint32_t oBar = 0;
  static constexpr uint32_t oMats = 32;
  static constexpr uint32_t oBuf = oMats + kMat;
  static constexpr uint32_t oFlux = oBuf + 2 * kBuf;
  static constexpr uint32_t kSmem = oFlux + TE * Nf * FSTR * 4;
  static_assert(NpP % 4 == 0 && kMat % 16 == 0, "16-byte operator rows");
};

__device__ __forceinline__ float f4c(const float4& v, int i) {
  return i == 0 ? v.x : (i == 1 ? v.y : (i == 2 ? v.z : v.w));
}

// Tiles t0, t0 + tstep, ... < tend of the stage p: the operator copy, then a
// double-buffered tile loop.  smem holds BlkConfig's layout with its three
// mbarriers (initialised by the caller) at offset 0; ph[0], ph[1] are the
// phases of the tile-buffer barriers, ph[2] that of the operator barrier, kept
// by the caller across calls.  Every thread must have finished with smem
// before the call; the call ends in a CTA barrier.  False if a wait expired
// (uniform across the CTA).
template <int N, int P, int EPT_, int MAP_>
__device__ __forceinline__ bool blk_tiles(const RhsParams& p, unsigned char* smem, uint32_t (&ph)[3], int t0,
                                          int tstep, int tend) {
  using C = BlkConfig<N, P, EPT_, MAP_>;
  constexpr int Np = C::Np, NpP = C::NpP, NFACE = C::NFACE, Nfp = Order<N>::Nfp;
  constexpr int EPT = C::EPT, NG = C::NG, NTE = C::NTE, TE = C::TE, NF = C::Nf, ESTR = C::ESTR;
  constexpr int FSTR = C::FSTR, NT = C::kThreads;

  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + C::oBar);  // [0], [1]: tile buffers, [2]: operators
  const float* sB = reinterpret_cast<const float*>(smem + C::oMats);
  float* sF = reinterpret_cast<float*>(smem + C::oFlux);
  auto bufQ = [&](int b) { return reinterpret_cast<float*>(smem + C::oBuf + b * C::kBuf); };
  auto bufA = [&](int b) { return reinterpret_cast<float*>(smem + C::oBuf + b * C::kBuf + C::kQ); };
  auto bufG = [&](int b) { return reinterpret_cast<float*>(smem + C::oBuf + b * C::kBuf + C::kQ + C::kA); };
  auto bufN = [&](int b) {
    return reinterpret_cast<int4*>(smem + C::oBuf + b * C::kBuf + C::kQ + C::kA + C::kG);
  };
  const bool aux_tile = C::kAuxTile && p.mode == MODE_LSERK;

  const int tid = threadIdx.x;
  // element slot and 4-node group of this thread
  const int slot = C::MAP == 0 ? tid / NG : ((tid >> 5) / NG) * 32 + (tid & 31);
  const int grp = C::MAP == 0 ? tid - (tid / NG) * NG : (tid >> 5) % NG;
  const float* qin = static_cast<const float*>(p.q_in);
  const float cax = p.fax, cay = p.fay, cca = p.fca, ccb = p.fcb, cdt = p.fdt;

  // the padding columns of the flux rows are never written by the face phase
  for (int x = tid; x < TE * NF * FSTR; x += NT) sF[x] = 0.0f;
  __syncthreads();

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
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_arrive_expect_tx(&bar[2], C::kMat);
    bulk_g2s(const_cast<float*>(sB), p.mats_blk, C::kMat, &bar[2]);
  }
  // the operators are set-up data; the state, the residual and the device
  // time are the previous launch's output
  grid_dep_wait();
  const double tnow = p.t_dev ? *p.t_dev + p.t : p.t;
  if (tid == 0 && t0 < tend) issue(t0, 0);
  if (!__syncthreads_and(mbar_wait(&bar[2], ph[2], p.status))) return false;
  ph[2] ^= 1;

  int it = 0;
  for (int tile = t0; tile < tend; tile += tstep, ++it) {
    const int b = it & 1;
    const int k0 = tile * TE, ne = min(TE, p.K - k0);
    const int nxt = tile + tstep;
    // buffer b^1 was last read in the previous iteration, which ended in a
    // CTA barrier, so it (and its mbarrier) can be refilled now
    if (tid == 0 && nxt < tend) issue(nxt, b ^ 1);
    if (!__syncthreads_and(mbar_wait(&bar[b], ph[b], p.status))) return false;
    ph[b] ^= 1;
    const float* sQ = bufQ(b);
    const float* sA = bufA(b);
    const float* sG = bufG(b);
    const int4* sN = bufN(b);

    // ---- volume: nodes 4 grp .. 4 grp + 3 of elements slot, slot + NTE.  It
    //      needs no face data, so it runs first and the face phase's neighbour
    //      gathers of some warps overlap the volume products of others.
    float rh[EPT][NF][4];
    if (slot < NTE) {
      const float* bR = sB + 4 * grp;           // Dr^T row j at bR + j NpP
      const float* bS = bR + Np * NpP;          // Ds^T
      if constexpr (P == PHYS_ADV) {
        float ur[EPT][4], us[EPT][4];
#pragma unroll
        for (int l = 0; l < EPT; ++l)
#pragma unroll
          for (int n = 0; n < 4; ++n) ur[l][n] = us[l][n] = 0.0f;
#pragma unroll
        for (int j0 = 0; j0 < Np; j0 += 4) {
          float4 a[EPT];
#pragma unroll
          for (int l = 0; l < EPT; ++l) a[l] = *reinterpret_cast<const float4*>(sQ + (slot + l * NTE) * ESTR + j0);
#pragma unroll
          for (int jj = 0; jj < 4; ++jj) {
            if (j0 + jj >= Np) break;
            const float4 br = *reinterpret_cast<const float4*>(bR + (j0 + jj) * NpP);
            const float4 bs = *reinterpret_cast<const float4*>(bS + (j0 + jj) * NpP);
#pragma unroll
            for (int l = 0; l < EPT; ++l) {
              const float v = f4c(a[l], jj);
              ur[l][0] = fmaf(br.x, v, ur[l][0]); us[l][0] = fmaf(bs.x, v, us[l][0]);
              ur[l][1] = fmaf(br.y, v, ur[l][1]); us[l][1] = fmaf(bs.y, v, us[l][1]);
              ur[l][2] = fmaf(br.z, v, ur[l][2]); us[l][2] = fmaf(bs.z, v, us[l][2]);
              ur[l][3] = fmaf(br.w, v, ur[l][3]); us[l][3] = fmaf(bs.w, v, us[l][3]);
            }
          }
        }
#pragma unroll
        for (int l = 0; l < EPT; ++l) {
          const float4 g0 = *reinterpret_cast<const float4*>(sG + (slot + l * NTE) * 16);  // rx ry sx sy
#pragma unroll
          for (int n = 0; n < 4; ++n) {
            const float dx = g0.x * ur[l][n] + g0.z * us[l][n], dy = g0.y * ur[l][n] + g0.w * us[l][n];
            rh[l][0][n] = cax * dx + cay * dy;
          }
        }
      } else {
        // Maxwell: the curl term of the third field is one product pair,
        // Dr u + Ds v with u, v the geometric combinations of the first two
        // fields (rx, ry, sx, sy are constant on an element):
        //   TE  Hz' = Dx Ey - Dy Ex = Dr (rx Ey - ry Ex) + Ds (sx Ey - sy Ex),
        //   TM  Ez' = Dy Hx - Dx Hy = Dr (ry Hx - rx Hy) + Ds (sy Hx - sx Hy);
        // the gradient of the third field needs Dr q2 and Ds q2.
        float gr[EPT][4], gs[EPT][4], cu[EPT][4];
        float4 g0[EPT];
#pragma unroll
        for (int l = 0; l < EPT; ++l) {
          g0[l] = *reinterpret_cast<const float4*>(sG + (slot + l * NTE) * 16);  // rx ry sx sy
#pragma unroll
          for (int n = 0; n < 4; ++n) gr[l][n] = gs[l][n] = cu[l][n] = 0.0f;
        }
#pragma unroll
        for (int j0 = 0; j0 < Np; j0 += 4) {
          float4 a[EPT][NF];
#pragma unroll
          for (int l = 0; l < EPT; ++l)
#pragma unroll
            for (int c = 0; c < NF; ++c)
              a[l][c] = *reinterpret_cast<const float4*>(sQ + (slot + l * NTE) * ESTR + c * NpP + j0);
#pragma unroll
          for (int jj = 0; jj < 4; ++jj) {
            if (j0 + jj >= Np) break;
            const float4 br = *reinterpret_cast<const float4*>(bR + (j0 + jj) * NpP);
            const float4 bs = *reinterpret_cast<const float4*>(bS + (j0 + jj) * NpP);
#pragma unroll
            for (int l = 0; l < EPT; ++l) {
              const float q0 = f4c(a[l][0], jj), q1 = f4c(a[l][1], jj), v = f4c(a[l][2], jj);
              const float u = (P == PHYS_TE) ? g0[l].x * q1 - g0[l].y * q0 : g0[l].y * q0 - g0[l].x * q1;
              const float w = (P == PHYS_TE) ? g0[l].z * q1 - g0[l].w * q0 : g0[l].w * q0 - g0[l].z * q1;
              gr[l][0] = fmaf(br.x, v, gr[l][0]); gs[l][0] = fmaf(bs.x, v, gs[l][0]);
              gr[l][1] = fmaf(br.y, v, gr[l][1]); gs[l][1] = fmaf(bs.y, v, gs[l][1]);
              gr[l][2] = fmaf(br.z, v, gr[l][2]); gs[l][2] = fmaf(bs.z, v, gs[l][2]);
              gr[l][3] = fmaf(br.w, v, gr[l][3]); gs[l][3] = fmaf(bs.w, v, gs[l][3]);
              cu[l][0] = fmaf(br.x, u, fmaf(bs.x, w, cu[l][0]));
              cu[l][1] = fmaf(br.y, u, fmaf(bs.y, w, cu[l][1]));
              cu[l][2] = fmaf(br.z, u, fmaf(bs.z, w, cu[l][2]));
              cu[l][3] = fmaf(br.w, u, fmaf(bs.w, w, cu[l][3]));
            }
          }
        }
#pragma unroll
        for (int l = 0; l < EPT; ++l) {
          const float rx = g0[l].x, ry = g0[l].y, sx = g0[l].z, sy = g0[l].w;
#pragma unroll
          for (int n = 0; n < 4; ++n) {
            if (P == PHYS_TM) {  // Hx' = Dy Ez, Hy' = -Dx Ez
              rh[l][0][n] = ry * gr[l][n] + sy * gs[l][n];
              rh[l][1][n] = -(rx * gr[l][n] + sx * gs[l][n]);
            } else {             // Ex' = -Dy Hz, Ey' = Dx Hz
              rh[l][0][n] = -(ry * gr[l][n] + sy * gs[l][n]);
              rh[l][1][n] = rx * gr[l][n] + sx * gs[l][n];
            }
            rh[l][2][n] = cu[l][n];
          }
        }
      }
    }

    // the next stage may be scheduled once every CTA is past the volume term of
    // its last tile: its set-up then overlaps this tile's face, lift and
    // epilogue phases, and the launches ahead never run more than one stage
    // deep (it waits for this grid before its reads)
    if (tile + tstep >= tend) grid_dep_launch();

    // ---- face nodes: item (element e, face-node index d) takes node d of the
    //      three faces of e; the own and neighbour values of all three are
    //      gathered first, then the three fluxes formed
#pragma unroll
    for (int s = 0; s < C::kFItems; ++s) {
      const int x = tid + s * NT;
      if (x >= ne * Nfp) break;
      const int e = x / Nfp, d = x - e * Nfp;
      const int4 nb4 = sN[e];
      float av[3][NF], bv[3][NF];
#pragma unroll
      for (int f = 0; f < 3; ++f) {
        const int nb = f == 0 ? nb4.x : (f == 1 ? nb4.y : nb4.z);
        const int nd = fmask<N>(f, d);
#pragma unroll
        for (int c = 0; c < NF; ++c) av[f][c] = sQ[e * ESTR + c * NpP + nd];
        if (nb >= 0) {
          const int kn = nb >> 2, nd2 = fmask<N>(nb & 3, Nfp - 1 - d);
          if (kn >= k0 && kn < k0 + ne) {
#pragma unroll
            for (int c = 0; c < NF; ++c) bv[f][c] = sQ[(kn - k0) * ESTR + c * NpP + nd2];
          } else {
            const float* qb = qin + (size_t)kn * ESTR + nd2;
#pragma unroll
            for (int c = 0; c < NF; ++c) bv[f][c] = __ldg(qb + c * NpP);
          }
        } else if (P == PHYS_ADV) {
          const int bf = -1 - nb;
          const double xx = p.bxy[((size_t)bf * Nfp + d) * 2], yy = p.bxy[((size_t)bf * Nfp + d) * 2 + 1];
          bv[f][0] = (float)adv_exact(p, tnow, xx, yy);
        } else if (P == PHYS_TM) {  // PEC: H+ = H-, Ez+ = -Ez-
          bv[f][0] = av[f][0]; bv[f][1] = av[f][1]; bv[f][2] = -av[f][2];
        } else {                    // PEC: E+ = -E-, Hz+ = Hz-
          bv[f][0] = -av[f][0]; bv[f][1] = -av[f][1]; bv[f][2] = av[f][2];
        }
      }
      const float* g = sG + e * 16;
      const float mJ = g[4];
#pragma unroll
      for (int f = 0; f < 3; ++f) {
        const float nx = g[8 + f], ny = g[11 + f];
        const float sc = g[5 + f] * mJ;  // -faceJ / J: the lift scale folded into the flux
        const float* a = av[f];
        const float* bb = bv[f];
        float* fo = sF + e * NF * FSTR + f * Nfp + d;
        if (P == PHYS_ADV) {
          const float an = cax * nx + cay * ny;
          fo[0] = ((an >= 0.0f) ? a[0] : bb[0]) * an * sc;
        } else if (P == PHYS_TM) {
          const float w = (a[2] + bb[2]) + ny * (a[0] - bb[0]) - nx * (a[1] - bb[1]);
          fo[0] = 0.5f * ny * w * sc;
          fo[FSTR] = -0.5f * nx * w * sc;
          fo[2 * FSTR] = 0.5f * (ny * (a[0] + bb[0]) - nx * (a[1] + bb[1]) + a[2] - bb[2]) * sc;
        } else {
          const float w = (a[2] + bb[2]) - ny * (a[0] - bb[0]) + nx * (a[1] - bb[1]);
          fo[0] = -0.5f * ny * w * sc;
          fo[FSTR] = 0.5f * nx * w * sc;
          fo[2 * FSTR] = 0.5f * (nx * (a[1] + bb[1]) - ny * (a[0] + bb[0]) + a[2] - bb[2]) * sc;
        }
      }
    }
    __syncthreads();

    // ---- lift + epilogue
    if (slot < NTE) {
      const float* bL = sB + 4 * grp + 2 * Np * NpP;  // LIFT^T row m at bL + m NpP
      // lift of the scaled face fluxes
#pragma unroll
      for (int m0 = 0; m0 < NFACE; m0 += 4) {
        float4 fv[EPT][NF];
#pragma unroll
        for (int l = 0; l < EPT; ++l)
#pragma unroll
          for (int c = 0; c < NF; ++c)
            fv[l][c] = *reinterpret_cast<const float4*>(sF + (slot + l * NTE) * NF * FSTR + c * FSTR + m0);
#pragma unroll
        for (int mm = 0; mm < 4; ++mm) {
          if (m0 + mm >= NFACE) break;
          const float4 bl = *reinterpret_cast<const float4*>(bL + (m0 + mm) * NpP);
#pragma unroll
          for (int l = 0; l < EPT; ++l)
#pragma unroll
            for (int c = 0; c < NF; ++c) {
              const float v = f4c(fv[l][c], mm);
              rh[l][c][0] = fmaf(bl.x, v, rh[l][c][0]);
              rh[l][c][1] = fmaf(bl.y, v, rh[l][c][1]);
              rh[l][c][2] = fmaf(bl.z, v, rh[l][c][2]);
              rh[l][c][3] = fmaf(bl.w, v, rh[l][c][3]);
            }
        }
      }
      // ---- epilogue, 4 nodes of one element-field per float4
      float* out = static_cast<float*>(p.out);
      float* aux = static_cast<float*>(p.aux);
      float* q0 = static_cast<float*>(p.q0);
      // lanes of the last group past Np are padding: written as 0
      const int nvalid = Np - 4 * grp;
#pragma unroll
      for (int l = 0; l < EPT; ++l) {
        const int e = slot + l * NTE;
        if (e >= ne) break;
#pragma unroll
        for (int c = 0; c < NF; ++c) {
          const size_t o = (size_t)(k0 + e) * ESTR + c * NpP + 4 * grp;
          float4 r = make_float4(rh[l][c][0], rh[l][c][1], rh[l][c][2], rh[l][c][3]);
          const float4 qv = *reinterpret_cast<const float4*>(sQ + e * ESTR + c * NpP + 4 * grp);
          float4 w0 = r, w1 = r;  // values for out (w0) and aux / q0 (w1)
          bool wr_aux = true, wr_q0 = false, wr_out = true;
          if (p.mode == MODE_RHS) {
            wr_aux = false;
          } else if (p.mode == MODE_LSERK) {
            const float4 av4 = aux_tile ? *reinterpret_cast<const float4*>(sA + e * ESTR + c * NpP + 4 * grp)
                                        : *reinterpret_cast<const float4*>(aux + o);
            w1 = make_float4(cca * av4.x + cdt * r.x, cca * av4.y + cdt * r.y, cca * av4.z + cdt * r.z,
                             cca * av4.w + cdt * r.w);
            w0 = make_float4(qv.x + ccb * w1.x, qv.y + ccb * w1.y, qv.z + ccb * w1.z, qv.w + ccb * w1.w);
          } else if (p.stage == 0) {  // classical RK4, first stage
            w1 = r;
            w0 = make_float4(qv.x + cca * r.x, qv.y + cca * r.y, qv.z + cca * r.z, qv.w + cca * r.w);
          } else if (p.stage < 3) {
            const float4 av4 = *reinterpret_cast<const float4*>(aux + o);
            const float4 b4 = *reinterpret_cast<const float4*>(q0 + o);
            w1 = make_float4(av4.x + ccb * r.x, av4.y + ccb * r.y, av4.z + ccb * r.z, av4.w + ccb * r.w);
            w0 = make_float4(b4.x + cca * r.x, b4.y + cca * r.y, b4.z + cca * r.z, b4.w + cca * r.w);
          } else {                    // last stage updates the base state only
            const float4 av4 = *reinterpret_cast<const float4*>(aux + o);
            const float4 b4 = *reinterpret_cast<const float4*>(q0 + o);
            w1 = make_float4(b4.x + cca * (av4.x + r.x), b4.y + cca * (av4.y + r.y), b4.z + cca * (av4.z + r.z),
                             b4.w + cca * (av4.w + r.w));
            wr_aux = false;
            wr_q0 = true;
            wr_out = false;
          }
          if (nvalid < 4) { w0.w = 0.0f; w1.w = 0.0f; }
          if (nvalid < 3) { w0.z = 0.0f; w1.z = 0.0f; }
          if (nvalid < 2) { w0.y = 0.0f; w1.y = 0.0f; }
          if (wr_out) *reinterpret_cast<float4*>(out + o) = w0;
          if (wr_aux) *reinterpret_cast<float4*>(aux + o) = w1;
          if (wr_q0) *reinterpret_cast<float4*>(q0 + o) = w1;
        }
      }
    }
    __syncthreads();
  }
  return true;
}

template <int N, int P, int EPT_, int MAP_>
__global__ void __launch_bounds__(BlkConfig<N, P, EPT_, MAP_>::kThreads, BlkConfig<N, P, EPT_, MAP_>::kMinBlocks)
    dg_rhs_blk_kernel(const RhsParams p) {
  using C = BlkConfig<N, P, EPT_, MAP_>;
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + C::oBar);
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_init(&bar[2], 1);
    fence_barrier_init();
  }
  __syncthreads();
  uint32_t ph[3] = {0, 0, 0};
  blk_tiles<N, P, EPT_, MAP_>(p, smem, ph, blockIdx.x, gridDim.x, (p.K + C::TE - 1) / C::TE);
}

}  // namespace dgk
