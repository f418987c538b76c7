// ipdg_blk.cuh -- register-blocked FP32 kernels of the block-Jacobi CG
// iteration (the same three launches and device scalars as ipdg.cuh's
// GRAD_PCG / DIV_SPD_DOT / update kernels, which remain the FP64 path).
//
// Thread (slot, group) owns nodes 4 group .. 4 group + 3 of element `slot` of
// the tile; the operators are rows of Dr^T | Ds^T | LIFT^T (strong form) and of
// the mass matrix, padded to NpP columns, so one float4 row load feeds 4 (8 in
// the div pass) FMAs per column value.  Face fluxes are stored pre-scaled by
// -1/J so the lift accumulates straight into the result.  In the two operator
// passes the tiles (state fields, geometry, neighbours, penalties) are
// double-buffered bulk copies: the next tile is in flight while the current
// one is computed.  The block-Jacobi inverses are stored packed (upper
// triangle, row by row: 120 instead of 225 floats per element at N = 4) and
// staged per tile with the update's vectors.
#pragma once

#include "ipdg.cuh"

namespace dgk {

template <int N>
struct IpdgBlk {
  using O = Order<N>;
  static constexpr int Np = O::Np, NpP = O::NpP, Nfp = O::Nfp, NFACE = O::Nface;
  static constexpr int NG = NpP / 4;         // 4-node groups per element
  static constexpr int NT = 256;
  static constexpr int TE = NT / NG;         // elements per tile
  static constexpr int FSTR = (NFACE + 3) / 4 * 4;
  static constexpr int KB = 2 * Np + NFACE;  // operator rows: Dr^T | Ds^T | LIFT^T
  static constexpr uint32_t kOps = KB * NpP * 4;
  static constexpr uint32_t kMass = Np * NpP * 4;
  // packed symmetric block padded to a multiple of 4 floats with PK / 4 odd, so
  // the blocks of the 8 elements a warp covers start in different bank groups
  static constexpr int PK0 = (Np * (Np + 1) / 2 + 3) / 4 * 4;
  static constexpr int PK = (PK0 / 4) % 2 == 0 ? PK0 + 4 : PK0;
  // the 4-node groups of an element sit in one warp: column values are taken
  // from the owning lane by shuffle instead of (bank-conflicting) shared loads
  static constexpr bool kShfl = (32 % NG) == 0;
  static constexpr int FSG = 2 * FSTR + 1, FSD = FSTR + 1;  // odd flux-row strides (grad: x | y rows)
  static constexpr uint32_t kF = TE * NpP * 4;                // one field tile
  static constexpr uint32_t kG = TE * 16 * 4, kN = TE * 16, kT = TE * 4 * 4;
  // grad: buffers hold z | p_old | geometry | neighbours
  static constexpr uint32_t kBufG = 2 * kF + kG + kN;
  static constexpr uint32_t oBar = 0, oOps = 32;
  static constexpr uint32_t oBufG = oOps + kOps;
  static constexpr uint32_t oFluxG = oBufG + 2 * kBufG;
  static constexpr uint32_t kSmemGrad = oFluxG + TE * FSG * 4;
  // div: buffers hold qx | qy | p | geometry | neighbours | tau
  static constexpr uint32_t kBufD = 3 * kF + kG + kN + kT;
  static constexpr uint32_t oMassD = oOps + kOps;
  static constexpr uint32_t oBufD = oMassD + kMass;
  static constexpr uint32_t oFluxD = oBufD + 2 * kBufD;
  static constexpr uint32_t oWD = (oFluxD + TE * FSD * 4 + 15) / 16 * 16;  // float4 stores
  static constexpr uint32_t kSmemDiv = oWD + kF + 16 * 8;
  // update: buffers hold x | r | p | Ap | packed Binv (all bulk-copied)
  static constexpr uint32_t kBufU = 4 * kF + TE * PK * 4;
  static constexpr uint32_t oTabU = 32;                        // packed indices, [j][NpP] uint16
  static constexpr uint32_t kTabU = (Np * NpP * 2 + 15) / 16 * 16;
  static constexpr uint32_t oBufU = oTabU + kTabU;
  static constexpr uint32_t kSmemUpd = oBufU + 2 * kBufU + 16 * 8;
  static_assert(NpP % 4 == 0 && kOps % 16 == 0 && kMass % 16 == 0, "16-byte rows");
  // every region read or written with 16-byte accesses or bulk copies starts on 16 bytes
  static_assert(oBufG % 16 == 0 && kBufG % 16 == 0 && oFluxG % 16 == 0, "grad layout alignment");
  static_assert(oMassD % 16 == 0 && oBufD % 16 == 0 && kBufD % 16 == 0 && oWD % 16 == 0 && (oWD + kF) % 16 == 0,
                "div layout alignment");
  static_assert(oBufU % 16 == 0 && kBufU % 16 == 0 && (oBufU + 2 * kBufU) % 16 == 0 && PK % 4 == 0,
                "update layout alignment");
};

// packed index of (i, j) in the upper triangle stored row by row
template <int Np>
__device__ __forceinline__ constexpr int pk_row(int i) {
  return i * Np - i * (i - 1) / 2;
}

__device__ __forceinline__ float4 f4_fma(const float4 a, const float s, const float4 c) {
  return make_float4(fmaf(a.x, s, c.x), fmaf(a.y, s, c.y), fmaf(a.z, s, c.z), fmaf(a.w, s, c.w));
}
__device__ __forceinline__ float f4_at(const float4& v, int i) {
  return i == 0 ? v.x : (i == 1 ? v.y : (i == 2 ? v.z : v.w));
}

// node j of an element whose NG lanes (NG | 32) each hold 4 consecutive nodes
// as v: read from the owning lane.  All 32 lanes must take part.
template <int NG>
__device__ __forceinline__ float col_shfl(const float4& v, int j) {
  const int src = ((int)(threadIdx.x & 31) & ~(NG - 1)) + (j >> 2);
  return __shfl_sync(0xffffffffu, f4_at(v, j & 3), src);
}

// ---------------------------------------------------------------- grad pass
// p = z + beta p_old (written), qx, qy = grad p (strong form, jumps lifted)
template <int N>
__global__ void __launch_bounds__(256, 4) ipdg_grad_blk_kernel(const IpdgParams p) {
  using B = IpdgBlk<N>;
  constexpr int Np = B::Np, NpP = B::NpP, Nfp = B::Nfp, NFACE = B::NFACE, NG = B::NG, TE = B::TE;
  constexpr int FSTR = B::FSTR, FS = B::FSG;
  extern __shared__ __align__(128) unsigned char smem[];
  grid_dep_launch();  // the next launch may be scheduled; it waits for this grid before its reads
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + B::oBar);
  const float4* ops4 = reinterpret_cast<const float4*>(smem + B::oOps);
  float* sF = reinterpret_cast<float*>(smem + B::oFluxG);
  auto bufZ = [&](int b) { return reinterpret_cast<float*>(smem + B::oBufG + b * B::kBufG); };
  auto bufP = [&](int b) { return reinterpret_cast<float*>(smem + B::oBufG + b * B::kBufG + B::kF); };
  auto bufG = [&](int b) { return reinterpret_cast<float*>(smem + B::oBufG + b * B::kBufG + 2 * B::kF); };
  auto bufN = [&](int b) {
    return reinterpret_cast<int4*>(smem + B::oBufG + b * B::kBufG + 2 * B::kF + B::kG);
  };
  __shared__ float s_beta;
  const int tid = threadIdx.x;
  const int slot = tid / NG, grp = tid - slot * NG;
  const int ntiles = (p.K + TE - 1) / TE;
  const float* zin = static_cast<const float*>(p.u);
  const float* pold = static_cast<const float*>(p.p_old);
  float* pv = static_cast<float*>(p.p);
  float* qxo = static_cast<float*>(p.qx);
  float* qyo = static_cast<float*>(p.qy);

  auto issue = [&](int tile, int b) {
    const int k0 = tile * TE, ne = min(TE, p.K - k0);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    const uint32_t bf = ne * NpP * 4, bg = ne * 64, bn = ne * 16;
    mbar_arrive_expect_tx(&bar[b], 2 * bf + bg + bn);
    bulk_g2s(bufZ(b), zin + (size_t)k0 * NpP, bf, &bar[b]);
    bulk_g2s(bufP(b), pold + (size_t)k0 * NpP, bf, &bar[b]);
    bulk_g2s(bufG(b), static_cast<const float*>(p.geom) + (size_t)k0 * 16, bg, &bar[b]);
    bulk_g2s(bufN(b), p.nbr + k0, bn, &bar[b]);
  };
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_init(&bar[2], 1);
    fence_barrier_init();
  }
  // padding columns of the flux rows stay zero
  for (int x = tid; x < TE * FS; x += 256) sF[x] = 0.0f;
  __syncthreads();
  if (tid == 0) {
    mbar_arrive_expect_tx(&bar[2], B::kOps);
    bulk_g2s(const_cast<float4*>(ops4), p.mats_blk, B::kOps, &bar[2]);
  }
  // the CG scalars and vectors are earlier launches' output; the operators
  // are set-up data (their copy is in flight already)
  grid_dep_wait();
  const bool done = p.cg->done != 0;
  if (tid == 0 && !done) {
    s_beta = 0.0f;
    if (!p.first) {
      const int s = p.slot, sp = (s + 2) % 3;
      s_beta = (float)(p.cg->rz[s] / p.cg->rz[sp]);
    }
    if (blockIdx.x == 0) p.cg->pAp = 0.0;
    if ((int)blockIdx.x < ntiles) issue(blockIdx.x, 0);
  }
  if (!__syncthreads_and(mbar_wait(&bar[2], 0, p.status))) return;
  if (done) return;  // converged: nothing in flight once the operators have landed
  const float beta = s_beta;
  uint32_t ph[2] = {0, 0};
  int it = 0;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
    const int b = it & 1;
    const int k0 = tile * TE, ne = min(TE, p.K - k0);
    const int nxt = tile + gridDim.x;
    if (tid == 0 && nxt < ntiles) issue(nxt, b ^ 1);
    if (!__syncthreads_and(mbar_wait(&bar[b], ph[b], p.status))) return;
    ph[b] ^= 1;
    float* sU = bufZ(b);
    const float* sP = bufP(b);
    const float* sG = bufG(b);
    const int4* sN = bufN(b);
    // p = z + beta p_old on the tile (in place over z), written out
    if (slot < ne) {
      float4* u4 = reinterpret_cast<float4*>(sU) + slot * NG + grp;
      const float4 z4 = *u4, o4 = reinterpret_cast<const float4*>(sP)[slot * NG + grp];
      const float4 v = make_float4(fmaf(beta, o4.x, z4.x), fmaf(beta, o4.y, z4.y), fmaf(beta, o4.z, z4.z),
                                   fmaf(beta, o4.w, z4.w));
      *u4 = v;
      reinterpret_cast<float4*>(pv + (size_t)(k0 + slot) * NpP)[grp] = v;
    }
    __syncthreads();
    // jumps on face nodes, lifted later: flux rows pre-scaled by -1/J.  All
    // exterior values of the thread's items are gathered first (independent
    // loads in flight together), then the fluxes are formed:
    // u+ = vz + beta vp (vp = 0 except for p = z + beta p_old outside the tile)
    constexpr int kItems = (TE * NFACE + 255) / 256;
    float vz[kItems], vp[kItems];
#pragma unroll
    for (int q = 0; q < kItems; ++q) {
      const int x = tid + q * 256;
      vz[q] = 0.0f;
      vp[q] = 0.0f;
      if (x < ne * NFACE) {
        const int e = x / NFACE, fm = x - e * NFACE, f = fm / Nfp, d = fm - f * Nfp;
        const int4 n4 = sN[e];
        const int nb = f == 0 ? n4.x : (f == 1 ? n4.y : n4.z);
        if (nb >= 0) {
          const int kn = nb >> 2, nd2 = fmask<N>(nb & 3, Nfp - 1 - d);
          if (kn >= k0 && kn < k0 + ne) {
            vz[q] = sU[(kn - k0) * NpP + nd2];
          } else {
            vz[q] = __ldg(zin + (size_t)kn * NpP + nd2);
            vp[q] = __ldg(pold + (size_t)kn * NpP + nd2);
          }
        } else {  // Dirichlet: u+ = -u- (du = 2 u-); Neumann: u+ = u- (du = 0)
          const float um = sU[e * NpP + fmask<N>(f, d)];
          vz[q] = p.dirichlet ? -um : um;
        }
      }
    }
#pragma unroll
    for (int q = 0; q < kItems; ++q) {
      const int x = tid + q * 256;
      if (x < ne * NFACE) {
        const int e = x / NFACE, fm = x - e * NFACE, f = fm / Nfp, d = fm - f * Nfp;
        const float* g = sG + e * 16;
        const float du = sU[e * NpP + fmask<N>(f, d)] - fmaf(beta, vp[q], vz[q]);
        const float tl = du * g[5 + f] * 0.5f * g[4];  // g[4] = -1/J
        sF[e * FS + fm] = g[8 + f] * tl;
        sF[e * FS + FSTR + fm] = g[11 + f] * tl;
      }
    }
    __syncthreads();
    // with kShfl every thread has a slot (TE NG = 256) and takes part in the
    // shuffles; lanes past the tile compute on stale values and store nothing
    if (B::kShfl || slot < ne) {
      const float* ue = sU + slot * NpP;
      const float4 pown = reinterpret_cast<const float4*>(sU)[slot * NG + grp];  // this thread's 4 nodes of p
      float4 ur = make_float4(0.f, 0.f, 0.f, 0.f), us = ur, lx = ur, ly = ur;
      if constexpr (B::kShfl) {
        // nodes 4 jg .. 4 jg + 3 come from lane jg of the element's group; the
        // outer loop stays rolled to bound register pressure
        const int base = (int)(threadIdx.x & 31) & ~(NG - 1);
#pragma unroll 1
        for (int jg = 0; jg < NG; ++jg) {
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            const float v = __shfl_sync(0xffffffffu, f4_at(pown, c), base + jg);
            const int j = 4 * jg + c;
            if (j < Np) {
              ur = f4_fma(ops4[j * NG + grp], v, ur);
              us = f4_fma(ops4[(Np + j) * NG + grp], v, us);
            }
          }
        }
      } else {
#pragma unroll
        for (int j = 0; j < Np; ++j) {
          const float v = ue[j];
          ur = f4_fma(ops4[j * NG + grp], v, ur);
          us = f4_fma(ops4[(Np + j) * NG + grp], v, us);
        }
      }
      const float* fx = sF + slot * FS;
      const float* fy = fx + FSTR;
#pragma unroll
      for (int m = 0; m < NFACE; ++m) {
        const float4 l = ops4[(2 * Np + m) * NG + grp];
        lx = f4_fma(l, fx[m], lx);
        ly = f4_fma(l, fy[m], ly);
      }
      const float* g = sG + slot * 16;
      const float rx = g[0], ry = g[1], sx = g[2], sy = g[3];
      float4 qx, qy;
      qx.x = rx * ur.x + sx * us.x + lx.x;
      qx.y = rx * ur.y + sx * us.y + lx.y;
      qx.z = rx * ur.z + sx * us.z + lx.z;
      qx.w = rx * ur.w + sx * us.w + lx.w;
      qy.x = ry * ur.x + sy * us.x + ly.x;
      qy.y = ry * ur.y + sy * us.y + ly.y;
      qy.z = ry * ur.z + sy * us.z + ly.z;
      qy.w = ry * ur.w + sy * us.w + ly.w;
      if (slot < ne) {
        const size_t o = (size_t)(k0 + slot) * NpP;
        reinterpret_cast<float4*>(qxo + o)[grp] = qx;  // padding columns of the operators are zero
        reinterpret_cast<float4*>(qyo + o)[grp] = qy;
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------- div pass
// Ap = S p = -J M (div q + lifted penalty / flux jumps); pAp accumulated
template <int N>
__global__ void __launch_bounds__(256, 4) ipdg_div_blk_kernel(const IpdgParams p) {
  using B = IpdgBlk<N>;
  constexpr int Np = B::Np, NpP = B::NpP, Nfp = B::Nfp, NFACE = B::NFACE, NG = B::NG, TE = B::TE;
  constexpr int FS = B::FSD;
  extern __shared__ __align__(128) unsigned char smem[];
  grid_dep_launch();  // the next launch may be scheduled; it waits for this grid before its reads
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + B::oBar);
  const float4* ops4 = reinterpret_cast<const float4*>(smem + B::oOps);
  const float4* mass4 = reinterpret_cast<const float4*>(smem + B::oMassD);
  float* sF = reinterpret_cast<float*>(smem + B::oFluxD);
  float* sW = reinterpret_cast<float*>(smem + B::oWD);
  double* red = reinterpret_cast<double*>(smem + B::oWD + B::kF);
  auto bufX = [&](int b) { return reinterpret_cast<float*>(smem + B::oBufD + b * B::kBufD); };
  auto bufY = [&](int b) { return reinterpret_cast<float*>(smem + B::oBufD + b * B::kBufD + B::kF); };
  auto bufU = [&](int b) { return reinterpret_cast<float*>(smem + B::oBufD + b * B::kBufD + 2 * B::kF); };
  auto bufG = [&](int b) { return reinterpret_cast<float*>(smem + B::oBufD + b * B::kBufD + 3 * B::kF); };
  auto bufN = [&](int b) {
    return reinterpret_cast<int4*>(smem + B::oBufD + b * B::kBufD + 3 * B::kF + B::kG);
  };
  auto bufT = [&](int b) {
    return reinterpret_cast<float*>(smem + B::oBufD + b * B::kBufD + 3 * B::kF + B::kG + B::kN);
  };
  const int tid = threadIdx.x;
  const int slot = tid / NG, grp = tid - slot * NG;
  const int ntiles = (p.K + TE - 1) / TE;
  const float* qx = static_cast<const float*>(p.qx);
  const float* qy = static_cast<const float*>(p.qy);
  const float* uj = static_cast<const float*>(p.du_src);
  float* out = static_cast<float*>(p.out);

  auto issue = [&](int tile, int b) {
    const int k0 = tile * TE, ne = min(TE, p.K - k0);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    const uint32_t bf = ne * NpP * 4, bg = ne * 64, bn = ne * 16, bt = ne * 16;
    mbar_arrive_expect_tx(&bar[b], 3 * bf + bg + bn + bt);
    bulk_g2s(bufX(b), qx + (size_t)k0 * NpP, bf, &bar[b]);
    bulk_g2s(bufY(b), qy + (size_t)k0 * NpP, bf, &bar[b]);
    bulk_g2s(bufU(b), uj + (size_t)k0 * NpP, bf, &bar[b]);
    bulk_g2s(bufG(b), static_cast<const float*>(p.geom) + (size_t)k0 * 16, bg, &bar[b]);
    bulk_g2s(bufN(b), p.nbr + k0, bn, &bar[b]);
    bulk_g2s(bufT(b), static_cast<const float*>(p.tau) + (size_t)k0 * 4, bt, &bar[b]);
  };
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_init(&bar[2], 1);
    fence_barrier_init();
  }
  for (int x = tid; x < TE * FS; x += 256) sF[x] = 0.0f;
  __syncthreads();
  if (tid == 0) {
    mbar_arrive_expect_tx(&bar[2], B::kOps + B::kMass);
    bulk_g2s(const_cast<float4*>(ops4), p.mats_blk, B::kOps, &bar[2]);
    bulk_g2s(const_cast<float4*>(mass4), p.mass_blk, B::kMass, &bar[2]);
  }
  // the CG scalars and vectors are earlier launches' output; the operators
  // are set-up data (their copy is in flight already)
  grid_dep_wait();
  const bool done = p.cg->done != 0;
  if (tid == 0 && !done) {
    if (blockIdx.x == 0) {
      const int s1 = (p.slot + 1) % 3;
      p.cg->rz[s1] = 0.0;
      p.cg->rr[s1] = 0.0;
    }
    if ((int)blockIdx.x < ntiles) issue(blockIdx.x, 0);
  }
  if (!__syncthreads_and(mbar_wait(&bar[2], 0, p.status))) return;
  if (done) return;  // converged: nothing in flight once the operators have landed
  double dot = 0.0;
  uint32_t ph[2] = {0, 0};
  int it = 0;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
    const int b = it & 1;
    const int k0 = tile * TE, ne = min(TE, p.K - k0);
    const int nxt = tile + gridDim.x;
    if (tid == 0 && nxt < ntiles) issue(nxt, b ^ 1);
    if (!__syncthreads_and(mbar_wait(&bar[b], ph[b], p.status))) return;
    ph[b] ^= 1;
    // S p = -J M (A p): rows of the symmetric mass matrix cover the thread's 4
    // nodes; A p of node j from its owning lane (kShfl) or from shared memory
    auto mass_epilogue = [&](const float4& au, const float* we = nullptr) {
      float4 sm = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
      for (int j = 0; j < Np; ++j) sm = f4_fma(mass4[j * NG + grp], we ? we[j] : col_shfl<NG>(au, j), sm);
      if (slot < ne) {
        const float mJ = bufG(b)[slot * 16 + 14];  // -J
        sm.x *= mJ;
        sm.y *= mJ;
        sm.z *= mJ;
        sm.w *= mJ;
        reinterpret_cast<float4*>(out + (size_t)(k0 + slot) * NpP)[grp] = sm;
        const float4 pu = reinterpret_cast<const float4*>(bufU(b) + slot * NpP)[grp];
        dot += (double)pu.x * sm.x + (double)pu.y * sm.y + (double)pu.z * sm.z + (double)pu.w * sm.w;
      }
    };
    const float* sX = bufX(b);
    const float* sY = bufY(b);
    const float* sU = bufU(b);
    const float* sG = bufG(b);
    const int4* sN = bufN(b);
    const float* sT = bufT(b);
    // exterior traces of the thread's face-node items gathered first
    // (independent loads in flight together), then the fluxes
    constexpr int kItems = (TE * NFACE + 255) / 256;
    float vx[kItems], vy[kItems], vu[kItems];
#pragma unroll
    for (int q = 0; q < kItems; ++q) {
      const int x = tid + q * 256;
      vx[q] = 0.0f;
      vy[q] = 0.0f;
      vu[q] = 0.0f;
      if (x < ne * NFACE) {
        const int e = x / NFACE, fm = x - e * NFACE, f = fm / Nfp, d = fm - f * Nfp;
        const int4 n4 = sN[e];
        const int nb = f == 0 ? n4.x : (f == 1 ? n4.y : n4.z);
        if (nb >= 0) {
          const int kn = nb >> 2, nd2 = fmask<N>(nb & 3, Nfp - 1 - d);
          if (kn >= k0 && kn < k0 + ne) {
            const int o = (kn - k0) * NpP + nd2;
            vx[q] = sX[o];
            vy[q] = sY[o];
            vu[q] = sU[o];
          } else {
            const size_t o = (size_t)kn * NpP + nd2;
            vx[q] = __ldg(qx + o);
            vy[q] = __ldg(qy + o);
            vu[q] = __ldg(uj + o);
          }
        }
      }
    }
#pragma unroll
    for (int q = 0; q < kItems; ++q) {
      const int x = tid + q * 256;
      if (x < ne * NFACE) {
        const int e = x / NFACE, fm = x - e * NFACE, f = fm / Nfp, d = fm - f * Nfp;
        const float* g = sG + e * 16;
        const int4 n4 = sN[e];
        const int nb = f == 0 ? n4.x : (f == 1 ? n4.y : n4.z);
        const int nd = e * NpP + fmask<N>(f, d);
        const float nx = g[8 + f], ny = g[11 + f];
        const float qxm = sX[nd], qym = sY[nd], um = sU[nd];
        float dqn, du;
        if (nb >= 0) {
          dqn = (qxm - vx[q]) * nx + (qym - vy[q]) * ny;
          du = um - vu[q];
        } else if (p.dirichlet) {
          dqn = 0.0f;
          du = 2.0f * um;
        } else {
          dqn = 2.0f * (qxm * nx + qym * ny);
          du = 0.0f;
        }
        sF[e * FS + fm] = (dqn + 2.0f * sT[e * 4 + f] * du) * g[5 + f] * 0.5f * g[4];  // g[4] = -1/J
      }
    }
    __syncthreads();
    if (B::kShfl || slot < ne) {  // see the grad pass for the kShfl lanes
      const float* xe = sX + slot * NpP;
      const float* ye = sY + slot * NpP;
      const int l = slot * NG + grp;
      const float4 x4 = reinterpret_cast<const float4*>(sX)[l], y4 = reinterpret_cast<const float4*>(sY)[l];
      float4 xr = make_float4(0.f, 0.f, 0.f, 0.f), xs = xr, yr = xr, ys = xr, lf = xr;
#pragma unroll
      for (int j = 0; j < Np; ++j) {
        const float4 dr = ops4[j * NG + grp], ds = ops4[(Np + j) * NG + grp];
        const float vx = B::kShfl ? col_shfl<NG>(x4, j) : xe[j];
        const float vy = B::kShfl ? col_shfl<NG>(y4, j) : ye[j];
        xr = f4_fma(dr, vx, xr);
        xs = f4_fma(ds, vx, xs);
        yr = f4_fma(dr, vy, yr);
        ys = f4_fma(ds, vy, ys);
      }
      const float* fe = sF + slot * FS;
#pragma unroll
      for (int m = 0; m < NFACE; ++m) lf = f4_fma(ops4[(2 * Np + m) * NG + grp], fe[m], lf);
      const float* g = sG + slot * 16;
      const float rx = g[0], ry = g[1], sx = g[2], sy = g[3];
      float4 au;
      au.x = (rx * xr.x + sx * xs.x) + (ry * yr.x + sy * ys.x) + lf.x;
      au.y = (rx * xr.y + sx * xs.y) + (ry * yr.y + sy * ys.y) + lf.y;
      au.z = (rx * xr.z + sx * xs.z) + (ry * yr.z + sy * ys.z) + lf.z;
      au.w = (rx * xr.w + sx * xs.w) + (ry * yr.w + sy * ys.w) + lf.w;
      {  // (A - shift I) p
        const float sh = (float)p.shift;
        const float4 u4 = reinterpret_cast<const float4*>(bufU(b))[l];
        au.x -= sh * u4.x;
        au.y -= sh * u4.y;
        au.z -= sh * u4.z;
        au.w -= sh * u4.w;
      }
      if constexpr (B::kShfl) {
        mass_epilogue(au);
      } else {
        reinterpret_cast<float4*>(sW + slot * NpP)[grp] = au;
      }
    }
    if constexpr (!B::kShfl) {
      __syncthreads();
      if (slot < ne) {
        const float* we = sW + slot * NpP;
        float4 au;
        au.x = au.y = au.z = au.w = 0.0f;  // unused: the mass product reads we[]
        mass_epilogue(au, we);
      }
    }
    __syncthreads();
  }
  const double sdot = block_sum(dot, red);
  if (tid == 0) atomicAdd(&p.cg->pAp, sdot);
}

// ---------------------------------------------------------------- update
// alpha = rz / pAp; x += alpha p; r -= alpha Ap; z = Binv r (packed blocks);
// rz, rr of the next slot
template <int N>
__global__ void __launch_bounds__(256, 2) pcg_update_blk_kernel(const IpdgParams p) {
  using B = IpdgBlk<N>;
  constexpr int Np = B::Np, NpP = B::NpP, NG = B::NG, TE = B::TE, PK = B::PK;
  extern __shared__ __align__(128) unsigned char smem[];
  CgScalars* cg = p.cg;
  grid_dep_launch();  // the next launch may be scheduled; it waits for this grid before its reads
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem);
  double* red = reinterpret_cast<double*>(smem + B::oBufU + 2 * B::kBufU);
  auto buf = [&](int b, int f) { return reinterpret_cast<float*>(smem + B::oBufU + b * B::kBufU + f * B::kF); };
  auto bufB = [&](int b) { return reinterpret_cast<float*>(smem + B::oBufU + b * B::kBufU + 4 * B::kF); };
  __shared__ float s_alpha;
  const int tid = threadIdx.x;
  const int slot = tid / NG, grp = tid - slot * NG;
  const int s = p.slot, s1 = (s + 1) % 3;
  const int ntiles = (p.K + TE - 1) / TE;
  float* x = static_cast<float*>(p.x);
  float* r = static_cast<float*>(p.r);
  float* z = static_cast<float*>(p.z);
  const float* pv = static_cast<const float*>(p.p);
  const float* Ap = static_cast<const float*>(p.Ap);
  const float* bpk = static_cast<const float*>(p.binv_pk);
  auto issue = [&](int tile, int b) {
    const int k0 = tile * TE, ne = min(TE, p.K - k0);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    const uint32_t bf = ne * NpP * 4;
    mbar_arrive_expect_tx(&bar[b], 4 * bf + ne * PK * 4);
    bulk_g2s(buf(b, 0), x + (size_t)k0 * NpP, bf, &bar[b]);
    bulk_g2s(buf(b, 1), r + (size_t)k0 * NpP, bf, &bar[b]);
    bulk_g2s(buf(b, 2), pv + (size_t)k0 * NpP, bf, &bar[b]);
    bulk_g2s(buf(b, 3), Ap + (size_t)k0 * NpP, bf, &bar[b]);
    bulk_g2s(bufB(b), bpk + (size_t)k0 * PK, ne * PK * 4, &bar[b]);
  };
  // packed index of B(i, j) for column j and output node i (0 for padding nodes):
  // the four indices of a thread's nodes are one 8-byte load
  uint16_t* tab = reinterpret_cast<uint16_t*>(smem + B::oTabU);
  for (int q = tid; q < Np * NpP; q += 256) {
    const int j = q / NpP, i = q - j * NpP;
    tab[q] = (uint16_t)(i >= Np ? 0 : (i <= j ? pk_row<Np>(i) + (j - i) : pk_row<Np>(j) + (i - j)));
  }
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_barrier_init();
  }
  // the CG scalars and vectors are earlier launches' output
  grid_dep_wait();
  if (cg->done) return;  // nothing issued yet
  if (tid == 0) s_alpha = (float)(cg->rz[s] / cg->pAp);  // one FP64 division per CTA
  __syncthreads();
  if (tid == 0 && (int)blockIdx.x < ntiles) issue(blockIdx.x, 0);
  const float alpha = s_alpha;
  const uint2* tab2 = reinterpret_cast<const uint2*>(tab);
  double rz = 0.0, rr = 0.0;
  uint32_t ph[2] = {0, 0};
  int it = 0;
  const int i0 = grp * 4;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
    const int b = it & 1;
    const int k0 = tile * TE, ne = min(TE, p.K - k0);
    const int nxt = tile + gridDim.x;
    // buffer b ^ 1 was last read before the barrier that ended the previous tile
    if (tid == 0 && nxt < ntiles) issue(nxt, b ^ 1);
    if (!__syncthreads_and(mbar_wait(&bar[b], ph[b], p.status))) return;
    ph[b] ^= 1;
    float* sR = buf(b, 1);
    float4 r4 = make_float4(0.f, 0.f, 0.f, 0.f);
    if (slot < ne) {
      const int l = slot * NG + grp;
      float4 xv = reinterpret_cast<const float4*>(buf(b, 0))[l];
      r4 = reinterpret_cast<const float4*>(sR)[l];
      const float4 p4 = reinterpret_cast<const float4*>(buf(b, 2))[l];
      const float4 a4 = reinterpret_cast<const float4*>(buf(b, 3))[l];
      xv.x = fmaf(alpha, p4.x, xv.x);
      xv.y = fmaf(alpha, p4.y, xv.y);
      xv.z = fmaf(alpha, p4.z, xv.z);
      xv.w = fmaf(alpha, p4.w, xv.w);
      r4.x = fmaf(-alpha, a4.x, r4.x);
      r4.y = fmaf(-alpha, a4.y, r4.y);
      r4.z = fmaf(-alpha, a4.z, r4.z);
      r4.w = fmaf(-alpha, a4.w, r4.w);
      const size_t o = (size_t)(k0 + slot) * NpP;
      reinterpret_cast<float4*>(x + o)[grp] = xv;
      reinterpret_cast<float4*>(r + o)[grp] = r4;
      reinterpret_cast<float4*>(sR)[l] = r4;  // only this thread reads and writes slot l
      rr += (double)r4.x * r4.x + (double)r4.y * r4.y + (double)r4.z * r4.z + (double)r4.w * r4.w;
    }
    __syncthreads();  // the whole element's updated r before the block products
    if (slot < ne) {
      const float* re = sR + slot * NpP;
      const float* be = bufB(b) + slot * PK;
      float zc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
      for (int j = 0; j < Np; ++j) {
        const uint2 t = tab2[j * NG + grp];
        const float rj = re[j];
        zc[0] = fmaf(be[t.x & 0xffffu], rj, zc[0]);
        zc[1] = fmaf(be[t.x >> 16], rj, zc[1]);
        zc[2] = fmaf(be[t.y & 0xffffu], rj, zc[2]);
        zc[3] = fmaf(be[t.y >> 16], rj, zc[3]);
      }
#pragma unroll
      for (int c = 0; c < 4; ++c)
        if (i0 + c >= Np) zc[c] = 0.0f;
      reinterpret_cast<float4*>(z + (size_t)(k0 + slot) * NpP)[grp] = make_float4(zc[0], zc[1], zc[2], zc[3]);
      rz += (double)r4.x * zc[0] + (double)r4.y * zc[1] + (double)r4.z * zc[2] + (double)r4.w * zc[3];
    }
    __syncthreads();
  }
  const double a = block_sum(rz, red);
  const double bsum = block_sum(rr, red + 8);
  if (tid == 0) {
    atomicAdd(&cg->rz[s1], a);
    atomicAdd(&cg->rr[s1], bsum);
  }
}

// packed FP32 copy of the symmetric FP64 block inverses (row-major, stride bstr)
template <int N>
__global__ void pack_binv_kernel(int K, const double* __restrict__ binv, int bstr, float* __restrict__ out) {
  using B = IpdgBlk<N>;
  constexpr int Np = B::Np, PK = B::PK;
  const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (g >= (int64_t)K * PK) return;
  const int k = (int)(g / PK), q = (int)(g % PK);
  float v = 0.0f;
  if (q < Np * (Np + 1) / 2) {
    int i = 0;
    while (q >= pk_row<Np>(i + 1) && i < Np - 1) ++i;  // row of packed entry q
    const int j = i + (q - pk_row<Np>(i));
    v = (float)binv[(size_t)k * bstr + (size_t)i * Np + j];
  }
  out[(size_t)k * PK + q] = v;
}

}  // namespace dgk
