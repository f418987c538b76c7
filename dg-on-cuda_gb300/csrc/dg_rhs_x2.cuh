// dg_rhs_x2.cuh -- fused RHS + LSERK4 stage for the compensated FP32 state
// (DGC_F32C handles): FP32 arithmetic everywhere, the state carried as an
// unevaluated pair q = hi + lo of FP32 values.
//
// Why a separate kernel.  With a plain FP32 state the relative L2 error of the
// TE cavity run at T = 1 stops near 1e-5 whatever the mesh, while the FP64
// run reaches the discretisation error (1e-9 .. 1e-13).  Two FP32 round-off
// sources set that floor, and they are removed here without FP64 arithmetic
// (which runs at a small fraction of the FP32 rate on this GPU):
//   1. the surface term.  In the weak form the lifted face flux is O(|q|) and
//      is rounded at eps |q| before LIFT (entries ~ (N+1)^2 / h) amplifies
//      it.  This kernel evaluates the strong form, whose surface term depends
//      only on the jumps d = q+ - q- at the face nodes, and forms each jump as
//      (hi+ - hi-) + (lo+ - lo-): the first difference is exact for nearby
//      values, so d keeps its own relative precision;
//   2. the volume term.  The strong-form derivative matrices annihilate
//      constants, so Dr q = Dr (q - c) for any constant c.  Each element-field
//      is contracted as hi - c with c = its first nodal value, a small
//      quantity of size h |grad q|, so the products' rounding shrinks with it.
//   The state update q += b_k res is a compensated sum (Knuth's TwoSum and a
//   Fast2Sum renormalisation, round-to-nearest intrinsics so nothing is
//   contracted or reordered), so the ~10^4 stage updates of a run do not
//   accumulate the state's own rounding.  The residual register res and the
//   geometric factors stay single FP32 values: their rounding enters the
//   solution at O(eps dt |L q|) per stage, below the two terms above.
//
// Strong form per element (Hesthaven & Warburton, ch. 6):
//   rhs = -div F(q) + (1/J) LIFT (faceJ (n.F(q-) - n.F*)),
// with the upwind fluxes of the weak-form kernels (dg_rhs.cuh) rewritten in
// the jumps: for Maxwell TE with d = q+ - q-,
//   w = d_Hz + ny d_Ex - nx d_Ey,
//   g = n.F* - n.F(q-) = (-ny w / 2, nx w / 2, (nx d_Ey - ny d_Ex - d_Hz) / 2),
// TM likewise, advection g = (a.n) d when a.n < 0 (inflow), else 0.
//
// Layout: a DGC_F32C state buffer holds 2 K Nf NpP floats, the hi vector of
// the native layout followed by the lo vector; the residual register is a
// plain FP32 vector of K Nf NpP floats.
//
// Mapping: as dg_rhs_blk_kernel (mapping 0, one element per thread slot):
// thread (slot, group) owns nodes 4g .. 4g+3 of one element and all its
// fields; operator rows are float4 loads of Dr^T | Ds^T | LIFT^T (strong
// form) padded to NpP columns.  Tiles are double-buffered (hi, lo, geometry,
// neighbours); the residual is read from global memory in the epilogue.
#pragma once

#include "dg_rhs_blk.cuh"

namespace dgk {

template <int N, int P>
struct X2Config {
  using O = Order<N>;
  static constexpr int Np = O::Np, NpP = O::NpP, NFACE = O::Nface;
  static constexpr int NG = NpP / 4;            // 4-node groups per element
  static constexpr int kThreads = 256;
  static constexpr int kMinBlocks = 3;
  static constexpr int TE = kThreads / NG;      // elements per tile
  static constexpr int Nf = PhysTraits<P>::Nf;
  static constexpr int ESTR = Nf * NpP;
  static constexpr int FSTR = (NFACE + 3) / 4 * 4;
  static constexpr int kFItems = (TE * O::Nfp + kThreads - 1) / kThreads;  // (element, face-node) items per thread
  static constexpr int KB = 2 * Np + NFACE;
  static constexpr uint32_t kMat = KB * NpP * 4;
  static constexpr uint32_t kQ = TE * ESTR * 4, kG = TE * 16 * 4, kN = TE * 16;
  static constexpr uint32_t kBuf = 2 * kQ + kG + kN;  // hi | lo | geometry | neighbours
  static constexpr uint32_t oBar = 0;
  static constexpr uint32_t oMats = 32;
  static constexpr uint32_t oBuf = oMats + kMat;
  static constexpr uint32_t oFlux = oBuf + 2 * kBuf;
  static constexpr uint32_t kSmem = oFlux + TE * Nf * FSTR * 4;
  static_assert(NpP % 4 == 0 && kMat % 16 == 0 && kQ % 16 == 0 && kG % 16 == 0, "16-byte regions");
};

// q (hi, lo) += d, compensated: TwoSum of hi and d, the error folded into lo,
// then a Fast2Sum renormalisation so that |lo| <= ulp(hi) / 2
__device__ __forceinline__ void x2_add(float& hi, float& lo, float d) {
  const float s = __fadd_rn(hi, d);
  const float bb = __fsub_rn(s, hi);
  const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(d, bb));
  const float l = __fadd_rn(lo, e);
  const float h2 = __fadd_rn(s, l);
  lo = __fsub_rn(l, __fsub_rn(h2, s));
  hi = h2;
}

template <int N, int P>
__global__ void __launch_bounds__(X2Config<N, P>::kThreads, X2Config<N, P>::kMinBlocks)
    dg_rhs_x2_kernel(const RhsParams p) {
  using C = X2Config<N, P>;
  constexpr int Np = C::Np, NpP = C::NpP, NFACE = C::NFACE, Nfp = Order<N>::Nfp;
  constexpr int NG = C::NG, TE = C::TE, NF = C::Nf, ESTR = C::ESTR;
  constexpr int FSTR = C::FSTR, NT = C::kThreads;

  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + C::oBar);  // [0], [1]: tile buffers, [2]: operators
  const float* sB = reinterpret_cast<const float*>(smem + C::oMats);
  float* sF = reinterpret_cast<float*>(smem + C::oFlux);
  auto bufH = [&](int b) { return reinterpret_cast<float*>(smem + C::oBuf + b * C::kBuf); };
  auto bufL = [&](int b) { return reinterpret_cast<float*>(smem + C::oBuf + b * C::kBuf + C::kQ); };
  auto bufG = [&](int b) { return reinterpret_cast<float*>(smem + C::oBuf + b * C::kBuf + 2 * C::kQ); };
  auto bufN = [&](int b) {
    return reinterpret_cast<int4*>(smem + C::oBuf + b * C::kBuf + 2 * C::kQ + C::kG);
  };

  const int tid = threadIdx.x;
  const int slot = tid / NG, grp = tid - (tid / NG) * NG;
  const int ntiles = (p.K + TE - 1) / TE;
  const size_t nvec = (size_t)p.K * ESTR;
  const float* qhi = static_cast<const float*>(p.q_in);
  const float* qlo = qhi + nvec;
  const float cax = p.fax, cay = p.fay, cca = p.fca, ccb = p.fcb, cdt = p.fdt;

  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_init(&bar[2], 1);
    fence_barrier_init();
  }
  for (int x = tid; x < TE * NF * FSTR; x += NT) sF[x] = 0.0f;
  __syncthreads();

  auto issue = [&](int tile, int b) {
    const int k0 = tile * TE, ne = min(TE, p.K - k0);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    const uint32_t bq = ne * ESTR * 4, bg = ne * 16 * 4, bn = ne * 16;
    mbar_arrive_expect_tx(&bar[b], 2 * bq + bg + bn);
    bulk_g2s(bufH(b), qhi + (size_t)k0 * ESTR, bq, &bar[b]);
    bulk_g2s(bufL(b), qlo + (size_t)k0 * ESTR, bq, &bar[b]);
    bulk_g2s(bufG(b), static_cast<const float*>(p.geom) + (size_t)k0 * 16, bg, &bar[b]);
    bulk_g2s(bufN(b), p.nbr + k0, bn, &bar[b]);
  };

  if (tid == 0) {
    mbar_arrive_expect_tx(&bar[2], C::kMat);
    bulk_g2s(const_cast<float*>(sB), p.mats_blk, C::kMat, &bar[2]);
  }
  // the operators are set-up data; the state, the residual and the device
  // time are the previous launch's output
  grid_dep_wait();
  const double tnow = p.t_dev ? *p.t_dev + p.t : p.t;
  if (tid == 0 && (int)blockIdx.x < ntiles) issue(blockIdx.x, 0);
  if (!__syncthreads_and(mbar_wait(&bar[2], 0, p.status))) return;

  uint32_t ph[2] = {0, 0};
  int it = 0;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
    const int b = it & 1;
    const int k0 = tile * TE, ne = min(TE, p.K - k0);
    const int nxt = tile + gridDim.x;
    if (tid == 0 && nxt < ntiles) issue(nxt, b ^ 1);
    if (!__syncthreads_and(mbar_wait(&bar[b], ph[b], p.status))) return;
    ph[b] ^= 1;
    const float* sH = bufH(b);
    const float* sL = bufL(b);
    const float* sG = bufG(b);
    const int4* sN = bufN(b);

    // ---- volume (on hi - c): nodes 4 grp .. 4 grp + 3 of element slot.  It
    //      needs no face data, so it runs first; the residual loads for the
    //      epilogue are issued after it and complete behind the face phase.
    const bool mine = slot < TE && slot < ne;
    float* aux = static_cast<float*>(p.aux);
    float rh[NF][4];
    float4 res4[NF];
    if (mine) {
      const float* bR = sB + 4 * grp;
      const float* bS = bR + Np * NpP;
      const float* qe = sH + slot * ESTR;
      float cm[NF];
#pragma unroll
      for (int c = 0; c < NF; ++c) cm[c] = qe[c * NpP];
      const float4 g0 = *reinterpret_cast<const float4*>(sG + slot * 16);  // rx ry sx sy
      const float rx = g0.x, ry = g0.y, sx = g0.z, sy = g0.w;
      if constexpr (P == PHYS_ADV) {
        float ur[4] = {0.0f, 0.0f, 0.0f, 0.0f}, us[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
        for (int j0 = 0; j0 < Np; j0 += 4) {
          float4 a = *reinterpret_cast<const float4*>(qe + j0);
          a.x -= cm[0]; a.y -= cm[0]; a.z -= cm[0]; a.w -= cm[0];
#pragma unroll
          for (int jj = 0; jj < 4; ++jj) {
            if (j0 + jj >= Np) break;
            const float4 br = *reinterpret_cast<const float4*>(bR + (j0 + jj) * NpP);
            const float4 bs = *reinterpret_cast<const float4*>(bS + (j0 + jj) * NpP);
            const float v = f4c(a, jj);
            ur[0] = fmaf(br.x, v, ur[0]); us[0] = fmaf(bs.x, v, us[0]);
            ur[1] = fmaf(br.y, v, ur[1]); us[1] = fmaf(bs.y, v, us[1]);
            ur[2] = fmaf(br.z, v, ur[2]); us[2] = fmaf(bs.z, v, us[2]);
            ur[3] = fmaf(br.w, v, ur[3]); us[3] = fmaf(bs.w, v, us[3]);
          }
        }
#pragma unroll
        for (int n = 0; n < 4; ++n) {  // -(a.grad u)
          const float dx = rx * ur[n] + sx * us[n], dy = ry * ur[n] + sy * us[n];
          rh[0][n] = -(cax * dx + cay * dy);
        }
      } else {
        // the curl term of the third field is one product pair Dr u + Ds v,
        // u and v the geometric combinations of the first two fields (both
        // taken as hi - c):
        //   TE  Hz' = Dy Ex - Dx Ey = Dr (ry Ex - rx Ey) + Ds (sy Ex - sx Ey),
        //   TM  Ez' = Dx Hy - Dy Hx = Dr (rx Hy - ry Hx) + Ds (sx Hy - sy Hx);
        // the gradient of the third field needs Dr q2 and Ds q2.
        float gr[4] = {0.0f, 0.0f, 0.0f, 0.0f}, gs[4] = {0.0f, 0.0f, 0.0f, 0.0f}, cu[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
        for (int j0 = 0; j0 < Np; j0 += 4) {
          float4 a[NF];
#pragma unroll
          for (int c = 0; c < NF; ++c) {
            a[c] = *reinterpret_cast<const float4*>(qe + c * NpP + j0);
            a[c].x -= cm[c]; a[c].y -= cm[c]; a[c].z -= cm[c]; a[c].w -= cm[c];
          }
#pragma unroll
          for (int jj = 0; jj < 4; ++jj) {
            if (j0 + jj >= Np) break;
            const float4 br = *reinterpret_cast<const float4*>(bR + (j0 + jj) * NpP);
            const float4 bs = *reinterpret_cast<const float4*>(bS + (j0 + jj) * NpP);
            const float q0 = f4c(a[0], jj), q1 = f4c(a[1], jj), v = f4c(a[2], jj);
            const float u = (P == PHYS_TE) ? ry * q0 - rx * q1 : rx * q1 - ry * q0;
            const float w = (P == PHYS_TE) ? sy * q0 - sx * q1 : sx * q1 - sy * q0;
            gr[0] = fmaf(br.x, v, gr[0]); gs[0] = fmaf(bs.x, v, gs[0]);
            gr[1] = fmaf(br.y, v, gr[1]); gs[1] = fmaf(bs.y, v, gs[1]);
            gr[2] = fmaf(br.z, v, gr[2]); gs[2] = fmaf(bs.z, v, gs[2]);
            gr[3] = fmaf(br.w, v, gr[3]); gs[3] = fmaf(bs.w, v, gs[3]);
            cu[0] = fmaf(br.x, u, fmaf(bs.x, w, cu[0]));
            cu[1] = fmaf(br.y, u, fmaf(bs.y, w, cu[1]));
            cu[2] = fmaf(br.z, u, fmaf(bs.z, w, cu[2]));
            cu[3] = fmaf(br.w, u, fmaf(bs.w, w, cu[3]));
          }
        }
#pragma unroll
        for (int n = 0; n < 4; ++n) {
          if (P == PHYS_TM) {  // Hx' = -Dy Ez, Hy' = Dx Ez
            rh[0][n] = -(ry * gr[n] + sy * gs[n]);
            rh[1][n] = rx * gr[n] + sx * gs[n];
          } else {             // Ex' = Dy Hz, Ey' = -Dx Hz
            rh[0][n] = ry * gr[n] + sy * gs[n];
            rh[1][n] = -(rx * gr[n] + sx * gs[n]);
          }
          rh[2][n] = cu[n];
        }
      }
      if (p.mode == MODE_LSERK) {
#pragma unroll
        for (int c = 0; c < NF; ++c)
          res4[c] = *reinterpret_cast<const float4*>(aux + (size_t)(k0 + slot) * ESTR + c * NpP + 4 * grp);
      }
    }

    // the next stage may be scheduled once every CTA is past the volume term of
    // its last tile (see dg_rhs_blk_kernel)
    if (tile + (int)gridDim.x >= ntiles) grid_dep_launch();

    // ---- face nodes: jumps d = q+ - q- from the hi and lo parts, then the
    // strong-form flux differences, pre-scaled by -faceJ / J.  Item (element
    // e, face-node index dd) takes node dd of the three faces of e.
#pragma unroll
    for (int s = 0; s < C::kFItems; ++s) {
      const int x = tid + s * NT;
      if (x >= ne * Nfp) break;
      const int e = x / Nfp, dd = x - e * Nfp;
      const int4 nb4 = sN[e];
      float d[3][NF];
#pragma unroll
      for (int f = 0; f < 3; ++f) {
        const int nb = f == 0 ? nb4.x : (f == 1 ? nb4.y : nb4.z);
        const int nd = fmask<N>(f, dd);
        float ah[NF], al[NF];
#pragma unroll
        for (int c = 0; c < NF; ++c) {
          ah[c] = sH[e * ESTR + c * NpP + nd];
          al[c] = sL[e * ESTR + c * NpP + nd];
        }
        if (nb >= 0) {
          const int kn = nb >> 2, nd2 = fmask<N>(nb & 3, Nfp - 1 - dd);
          float bh[NF], bl[NF];
          if (kn >= k0 && kn < k0 + ne) {
#pragma unroll
            for (int c = 0; c < NF; ++c) {
              bh[c] = sH[(kn - k0) * ESTR + c * NpP + nd2];
              bl[c] = sL[(kn - k0) * ESTR + c * NpP + nd2];
            }
          } else {
            const size_t o = (size_t)kn * ESTR + nd2;
#pragma unroll
            for (int c = 0; c < NF; ++c) {
              bh[c] = __ldg(qhi + o + c * NpP);
              bl[c] = __ldg(qlo + o + c * NpP);
            }
          }
#pragma unroll
          for (int c = 0; c < NF; ++c) d[f][c] = __fadd_rn(__fsub_rn(bh[c], ah[c]), __fsub_rn(bl[c], al[c]));
        } else if (P == PHYS_ADV) {
          const int bf = -1 - nb;
          const double xx = p.bxy[((size_t)bf * Nfp + dd) * 2], yy = p.bxy[((size_t)bf * Nfp + dd) * 2 + 1];
          d[f][0] = (float)((adv_exact(p, tnow, xx, yy) - (double)ah[0]) - (double)al[0]);
        } else if (P == PHYS_TM) {  // PEC: H+ = H-, Ez+ = -Ez-
          d[f][0] = 0.0f; d[f][1] = 0.0f; d[f][2] = -2.0f * ah[2] - 2.0f * al[2];
        } else {                    // PEC: E+ = -E-, Hz+ = Hz-
          d[f][0] = -2.0f * ah[0] - 2.0f * al[0]; d[f][1] = -2.0f * ah[1] - 2.0f * al[1]; d[f][2] = 0.0f;
        }
      }
      const float* g = sG + e * 16;
      const float mJ = g[4];
#pragma unroll
      for (int f = 0; f < 3; ++f) {
        const float nx = g[8 + f], ny = g[11 + f];
        const float sc = g[5 + f] * mJ;  // -faceJ / J
        const float* df = d[f];
        float* fo = sF + e * NF * FSTR + f * Nfp + dd;
        if (P == PHYS_ADV) {
          const float an = cax * nx + cay * ny;
          fo[0] = an < 0.0f ? an * df[0] * sc : 0.0f;
        } else if (P == PHYS_TM) {
          const float w = df[2] - ny * df[0] + nx * df[1];
          fo[0] = 0.5f * ny * w * sc;
          fo[FSTR] = -0.5f * nx * w * sc;
          fo[2 * FSTR] = 0.5f * (ny * df[0] - nx * df[1] - df[2]) * sc;
        } else {
          const float w = df[2] + ny * df[0] - nx * df[1];
          fo[0] = -0.5f * ny * w * sc;
          fo[FSTR] = 0.5f * nx * w * sc;
          fo[2 * FSTR] = 0.5f * (nx * df[1] - ny * df[0] - df[2]) * sc;
        }
      }
    }
    __syncthreads();

    // ---- lift + epilogue
    if (mine) {
      const float* bL = sB + 4 * grp + 2 * Np * NpP;
#pragma unroll
      for (int m0 = 0; m0 < NFACE; m0 += 4) {
        float4 fv[NF];
#pragma unroll
        for (int c = 0; c < NF; ++c)
          fv[c] = *reinterpret_cast<const float4*>(sF + slot * NF * FSTR + c * FSTR + m0);
#pragma unroll
        for (int mm = 0; mm < 4; ++mm) {
          if (m0 + mm >= NFACE) break;
          const float4 bl = *reinterpret_cast<const float4*>(bL + (m0 + mm) * NpP);
#pragma unroll
          for (int c = 0; c < NF; ++c) {
            const float v = f4c(fv[c], mm);
            rh[c][0] = fmaf(bl.x, v, rh[c][0]);
            rh[c][1] = fmaf(bl.y, v, rh[c][1]);
            rh[c][2] = fmaf(bl.z, v, rh[c][2]);
            rh[c][3] = fmaf(bl.w, v, rh[c][3]);
          }
        }
      }
      // ---- epilogue
      float* ohi = static_cast<float*>(p.out);
      float* olo = ohi + nvec;
      const int nvalid = Np - 4 * grp;
#pragma unroll
      for (int c = 0; c < NF; ++c) {
        const size_t o = (size_t)(k0 + slot) * ESTR + c * NpP + 4 * grp;
        float r[4] = {rh[c][0], rh[c][1], rh[c][2], rh[c][3]};
        float h[4] = {0.0f, 0.0f, 0.0f, 0.0f}, l[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        if (p.mode == MODE_LSERK) {
          const float4 av = res4[c];
          const float4 hv = *reinterpret_cast<const float4*>(sH + slot * ESTR + c * NpP + 4 * grp);
          const float4 lv = *reinterpret_cast<const float4*>(sL + slot * ESTR + c * NpP + 4 * grp);
          const float a4[4] = {av.x, av.y, av.z, av.w};
          h[0] = hv.x; h[1] = hv.y; h[2] = hv.z; h[3] = hv.w;
          l[0] = lv.x; l[1] = lv.y; l[2] = lv.z; l[3] = lv.w;
#pragma unroll
          for (int n = 0; n < 4; ++n) {
            r[n] = cca * a4[n] + cdt * r[n];
            x2_add(h[n], l[n], ccb * r[n]);
          }
        } else {  // MODE_RHS: the operator value in hi, lo = 0
#pragma unroll
          for (int n = 0; n < 4; ++n) h[n] = r[n];
        }
#pragma unroll
        for (int n = 0; n < 4; ++n)
          if (n >= nvalid) { h[n] = 0.0f; l[n] = 0.0f; r[n] = 0.0f; }
        *reinterpret_cast<float4*>(ohi + o) = make_float4(h[0], h[1], h[2], h[3]);
        *reinterpret_cast<float4*>(olo + o) = make_float4(l[0], l[1], l[2], l[3]);
        if (p.mode == MODE_LSERK) *reinterpret_cast<float4*>(aux + o) = make_float4(r[0], r[1], r[2], r[3]);
      }
    }
    __syncthreads();
  }
}

}  // namespace dgk
