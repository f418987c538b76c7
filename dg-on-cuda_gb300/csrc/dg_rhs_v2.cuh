// dg_rhs_v2.cuh -- register-blocked variant of the fused RHS + stage kernel
// (dg_rhs.cuh) for FP32 at orders whose operator rows fit in registers.
//
// Same operator, fluxes and epilogues as dg_rhs_kernel; different mapping:
//   * thread (node i, group g) keeps row i of Dr, Ds and LIFT in registers for
//     the whole persistent CTA and applies them to EPT elements of each tile
//     (e = g, g + G, ...), reading operands as float4 from shared memory;
//   * tiles of TE = G * EPT elements are double-buffered: the bulk copy of the
//     next tile (state, geometry, neighbours) is in flight while the current
//     tile is computed;
//   * each thread issues the neighbour gathers of all its face nodes before
//     computing any flux, so the L2 latencies overlap.
#pragma once

#include "dg_rhs.cuh"

namespace dgk {

// Tile shapes compiled per order: G groups x Np threads per CTA, EPT elements
// per thread, TE = G * EPT elements per tile.  The autotuner (capi.cu,
// dgc_autotune) times them on the handle's mesh and keeps the fastest.
template <int N>
struct V2Shapes;
template <> struct V2Shapes<1> { static constexpr int G[3] = {32, 64, 32}, EPT[3] = {2, 2, 4}; };
template <> struct V2Shapes<2> { static constexpr int G[3] = {32, 16, 32}, EPT[3] = {2, 4, 4}; };
template <> struct V2Shapes<3> { static constexpr int G[3] = {24, 12, 16}, EPT[3] = {2, 4, 4}; };
template <> struct V2Shapes<4> { static constexpr int G[3] = {16, 8, 8}, EPT[3] = {4, 4, 8}; };
template <> struct V2Shapes<5> { static constexpr int G[3] = {12, 6, 6}, EPT[3] = {4, 4, 8}; };
template <> struct V2Shapes<6> { static constexpr int G[3] = {8, 4, 4}, EPT[3] = {4, 8, 4}; };
constexpr int kV2Variants = 3;

template <int N, int P, int G_, int EPT_>
struct V2Config {
  using O = Order<N>;
  static constexpr int G = G_, EPT = EPT_;
  static constexpr int kThreads = O::Np * G;
  static constexpr int TE = G * EPT;
  static constexpr int Nf = PhysTraits<P>::Nf;
  static constexpr int ESTR = Nf * O::NpP;
  static constexpr int FSTR = (O::Nface + 3) / 4 * 4;  // padded face-flux row
  static constexpr int kItems = (TE * O::Nface + kThreads - 1) / kThreads;
  static constexpr uint32_t kMat = MatLayout<float, N>::kBytes;
  static constexpr uint32_t kQ = TE * ESTR * 4, kG = TE * 16 * 4, kN = TE * 16;
  static constexpr uint32_t kBuf = kQ + kG + kN;  // one tile buffer (16-byte multiples)
  static constexpr uint32_t oBar = 0;
  static constexpr uint32_t oMats = 32;
  static constexpr uint32_t oBuf = oMats + kMat;
  static constexpr uint32_t oFlux = oBuf + 2 * kBuf;
  static constexpr uint32_t kSmem = oFlux + TE * Nf * FSTR * 4;
};

template <int N, int P, int G_, int EPT_>
__global__ void __launch_bounds__(V2Config<N, P, G_, EPT_>::kThreads) dg_rhs_v2_kernel(const RhsParams p) {
  using O = Order<N>;
  using C = V2Config<N, P, G_, EPT_>;
  constexpr int Np = O::Np, Nfp = O::Nfp, NpP = O::NpP, NFACE = O::Nface;
  constexpr int G = C::G, EPT = C::EPT, TE = C::TE, NF = C::Nf, ESTR = C::ESTR, FSTR = C::FSTR;
  constexpr int NT = C::kThreads;
  constexpr int kD = MatLayout<float, N>::kD;

  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + C::oBar);  // [0], [1]: tile buffers, [2]: matrices
  const float* sMat = reinterpret_cast<const float*>(smem + C::oMats);
  float* sF = reinterpret_cast<float*>(smem + C::oFlux);
  auto bufQ = [&](int b) { return reinterpret_cast<float*>(smem + C::oBuf + b * C::kBuf); };
  auto bufG = [&](int b) { return reinterpret_cast<float*>(smem + C::oBuf + b * C::kBuf + C::kQ); };
  auto bufN = [&](int b) { return reinterpret_cast<int4*>(smem + C::oBuf + b * C::kBuf + C::kQ + C::kG); };

  const int tid = threadIdx.x;
  const int gi = tid / Np, ni = tid - gi * Np;
  const int ntiles = (p.K + TE - 1) / TE;
  const float* qin = static_cast<const float*>(p.q_in);
  const double tnow = p.t_dev ? *p.t_dev + p.t : p.t;
  // FP32 copies of the scalar parameters (rhs_dispatch<float>)
  const float cax = p.fax, cay = p.fay, cca = p.fca, ccb = p.fcb, cdt = p.fdt;

  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_init(&bar[2], 1);
    fence_barrier_init();
  }
  // zero the padding of the flux rows (never written by the face phase)
  for (int x = tid; x < TE * NF * FSTR; x += NT) sF[x] = 0.0f;
  __syncthreads();

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
    mbar_arrive_expect_tx(&bar[2], C::kMat);
    bulk_g2s(const_cast<float*>(sMat), p.mats, C::kMat, &bar[2]);
    if ((int)blockIdx.x < ntiles) issue(blockIdx.x, 0);
  }
  if (!__syncthreads_and(mbar_wait(&bar[2], 0, p.status))) return;  // uniform exit on a timeout

  // operator rows of node ni in registers
  float dr[Np], ds[Np], lt[NFACE];
#pragma unroll
  for (int j = 0; j < Np; ++j) {
    dr[j] = sMat[j * Np + ni];
    ds[j] = sMat[kD + j * Np + ni];
  }
#pragma unroll
  for (int m = 0; m < NFACE; ++m) lt[m] = sMat[2 * kD + m * Np + ni];

  uint32_t ph[2] = {0, 0};
  int it = 0;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
    const int b = it & 1;
    const int k0 = tile * TE, ne = min(TE, p.K - k0);
    const int nxt = tile + gridDim.x;
    if (tid == 0 && nxt < ntiles) issue(nxt, b ^ 1);
    if (!__syncthreads_and(mbar_wait(&bar[b], ph[b], p.status))) return;
    ph[b] ^= 1;
    const float* sQ = bufQ(b);
    const float* sG = bufG(b);
    const int4* sN = bufN(b);

    // ---- face nodes: gather first, then fluxes
    {
      float av[C::kItems][NF], bv[C::kItems][NF];
      int item[C::kItems];
#pragma unroll
      for (int s = 0; s < C::kItems; ++s) {
        const int x = tid + s * NT;
        item[s] = x < ne * NFACE ? x : -1;
        if (item[s] < 0) continue;
        const int e = x / NFACE, fm = x - e * NFACE, f = fm / Nfp, d = fm - f * Nfp;
        const int nb = f == 0 ? sN[e].x : (f == 1 ? sN[e].y : sN[e].z);
        const int nd = fmask<N>(f, d);
#pragma unroll
        for (int c = 0; c < NF; ++c) av[s][c] = sQ[e * ESTR + c * NpP + nd];
        if (nb >= 0) {
          const int kn = nb >> 2, nd2 = fmask<N>(nb & 3, Nfp - 1 - d);
          if (kn >= k0 && kn < k0 + ne) {
#pragma unroll
            for (int c = 0; c < NF; ++c) bv[s][c] = sQ[(kn - k0) * ESTR + c * NpP + nd2];
          } else {
            const float* qb = qin + (size_t)kn * ESTR + nd2;
#pragma unroll
            for (int c = 0; c < NF; ++c) bv[s][c] = __ldg(qb + c * NpP);
          }
        } else if (P == PHYS_ADV) {
          const int bf = -1 - nb;
          const double xx = p.bxy[((size_t)bf * Nfp + d) * 2], yy = p.bxy[((size_t)bf * Nfp + d) * 2 + 1];
          bv[s][0] = (float)adv_exact(p, tnow, xx, yy);
        } else if (P == PHYS_TM) {
          bv[s][0] = av[s][0]; bv[s][1] = av[s][1]; bv[s][2] = -av[s][2];
        } else {
          bv[s][0] = -av[s][0]; bv[s][1] = -av[s][1]; bv[s][2] = av[s][2];
        }
      }
#pragma unroll
      for (int s = 0; s < C::kItems; ++s) {
        if (item[s] < 0) continue;
        const int x = item[s];
        const int e = x / NFACE, fm = x - e * NFACE, f = fm / Nfp;
        const float* g = sG + e * 16;
        const float nx = g[8 + f], ny = g[11 + f], fJ = g[5 + f];
        const float* a = av[s];
        const float* bb = bv[s];
        float* fo = sF + e * NF * FSTR + fm;
        if (P == PHYS_ADV) {
          const float an = cax * nx + cay * ny;
          fo[0] = ((an >= 0.0f) ? a[0] : bb[0]) * an * fJ;
        } else if (P == PHYS_TM) {
          const float w = (a[2] + bb[2]) + ny * (a[0] - bb[0]) - nx * (a[1] - bb[1]);
          fo[0] = 0.5f * ny * w * fJ;
          fo[FSTR] = -0.5f * nx * w * fJ;
          fo[2 * FSTR] = 0.5f * (ny * (a[0] + bb[0]) - nx * (a[1] + bb[1]) + a[2] - bb[2]) * fJ;
        } else {
          const float w = (a[2] + bb[2]) - ny * (a[0] - bb[0]) + nx * (a[1] - bb[1]);
          fo[0] = -0.5f * ny * w * fJ;
          fo[FSTR] = 0.5f * nx * w * fJ;
          fo[2 * FSTR] = 0.5f * (nx * (a[1] + bb[1]) - ny * (a[0] + bb[0]) + a[2] - bb[2]) * fJ;
        }
      }
    }
    __syncthreads();

    // ---- volume + lift + epilogue: node ni of elements gi, gi + G, ...
    if (ni < Np) {
#pragma unroll
      for (int l = 0; l < EPT; ++l) {
        const int e = gi + G * l;
        if (e >= ne) break;
        const float* qe = sQ + e * ESTR;
        float ur[NF], us[NF], lf[NF];
#pragma unroll
        for (int c = 0; c < NF; ++c) ur[c] = us[c] = lf[c] = 0.0f;
#pragma unroll
        for (int j = 0; j < (Np & ~3); j += 4) {
#pragma unroll
          for (int c = 0; c < NF; ++c) {
            const float4 v = *reinterpret_cast<const float4*>(qe + c * NpP + j);
            ur[c] = fmaf(dr[j], v.x, ur[c]); us[c] = fmaf(ds[j], v.x, us[c]);
            ur[c] = fmaf(dr[j + 1], v.y, ur[c]); us[c] = fmaf(ds[j + 1], v.y, us[c]);
            ur[c] = fmaf(dr[j + 2], v.z, ur[c]); us[c] = fmaf(ds[j + 2], v.z, us[c]);
            ur[c] = fmaf(dr[j + 3], v.w, ur[c]); us[c] = fmaf(ds[j + 3], v.w, us[c]);
          }
        }
#pragma unroll
        for (int j = (Np & ~3); j < Np; ++j) {
#pragma unroll
          for (int c = 0; c < NF; ++c) {
            const float v = qe[c * NpP + j];
            ur[c] = fmaf(dr[j], v, ur[c]);
            us[c] = fmaf(ds[j], v, us[c]);
          }
        }
        const float* fe = sF + e * NF * FSTR;
#pragma unroll
        for (int m = 0; m < (NFACE & ~3); m += 4) {
#pragma unroll
          for (int c = 0; c < NF; ++c) {
            const float4 v = *reinterpret_cast<const float4*>(fe + c * FSTR + m);
            lf[c] = fmaf(lt[m], v.x, lf[c]);
            lf[c] = fmaf(lt[m + 1], v.y, lf[c]);
            lf[c] = fmaf(lt[m + 2], v.z, lf[c]);
            lf[c] = fmaf(lt[m + 3], v.w, lf[c]);
          }
        }
#pragma unroll
        for (int m = (NFACE & ~3); m < NFACE; ++m) {
#pragma unroll
          for (int c = 0; c < NF; ++c) lf[c] = fmaf(lt[m], fe[c * FSTR + m], lf[c]);
        }
        const float* g = sG + e * 16;
        const float rx = g[0], ry = g[1], sx = g[2], sy = g[3];
        const float ilJ = g[4];  // -1/J
        float rhs[NF];
        if (P == PHYS_ADV) {
          const float dx = rx * ur[0] + sx * us[0], dy = ry * ur[0] + sy * us[0];
          rhs[0] = cax * dx + cay * dy + ilJ * lf[0];
        } else if (P == PHYS_TM) {
          rhs[0] = (ry * ur[2] + sy * us[2]) + ilJ * lf[0];
          rhs[1] = -(rx * ur[2] + sx * us[2]) + ilJ * lf[1];
          rhs[2] = -(rx * ur[1] + sx * us[1]) + (ry * ur[0] + sy * us[0]) + ilJ * lf[2];
        } else {
          rhs[0] = -(ry * ur[2] + sy * us[2]) + ilJ * lf[0];
          rhs[1] = (rx * ur[2] + sx * us[2]) + ilJ * lf[1];
          rhs[2] = (rx * ur[1] + sx * us[1]) - (ry * ur[0] + sy * us[0]) + ilJ * lf[2];
        }
        const size_t base = (size_t)(k0 + e) * ESTR + ni;
        float* out = static_cast<float*>(p.out);
        float* aux = static_cast<float*>(p.aux);
        if (p.mode == MODE_RHS) {
#pragma unroll
          for (int c = 0; c < NF; ++c) out[base + c * NpP] = rhs[c];
        } else if (p.mode == MODE_LSERK) {
          const float ca = cca, cb = ccb, dt = cdt;
#pragma unroll
          for (int c = 0; c < NF; ++c) {
            const size_t o = base + c * NpP;
            const float r = ca * aux[o] + dt * rhs[c];
            aux[o] = r;
            out[o] = qe[c * NpP + ni] + cb * r;
          }
        } else {
          float* q0 = static_cast<float*>(p.q0);
          const float co = cca, wa = ccb;
#pragma unroll
          for (int c = 0; c < NF; ++c) {
            const size_t o = base + c * NpP;
            if (p.stage == 0) {
              aux[o] = rhs[c];
              out[o] = qe[c * NpP + ni] + co * rhs[c];
            } else if (p.stage < 3) {
              aux[o] = aux[o] + wa * rhs[c];
              out[o] = q0[o] + co * rhs[c];
            } else {
              q0[o] = q0[o] + co * (aux[o] + rhs[c]);
            }
          }
        }
      }
    }
    __syncthreads();
  }
}

}  // namespace dgk
