// mpnn_tc.cuh -- the message-passing layer of the learned preconditioner on the
// tensor cores (tcgen05, BF16 operands, FP32 accumulation in tensor memory).
//
// Per graph node e the layer computes
//   a_e = Ws h_e + Wn m_e + b,   m_e = sum of h over the face neighbours of e,
//   h'_e = h_e + relu(a_e)   (or h_e + a_e for the linear network),
// i.e. for a tile of 128 nodes the product D[128 x 64] = X[128 x 128] W^T with
// X = [h | m] (FP32) and W = [Ws | Wn] (64 x 128, BF16 copies of the FP32
// master weights).  W is exact in BF16; X is not, so X is split into three
// BF16 parts X = X0 + X1 + X2 (each the BF16 rounding of what the previous
// parts leave; 3 x 8 significand bits cover FP32's 24) and the tile is three
// accumulating products per K step.  The result matches the FP32 SIMT form of
// the same layer to FP32 accumulation round-off.
//
// CTA: 256 threads, one 128-node tile at a time (persistent over tiles).
//   * W is staged once per CTA in shared memory (K-major, no swizzle, core
//     matrices of 8 rows x 16 bytes: element (row, k) at byte
//     (row / 8) * 2048 + (k / 8) * 128 + (row % 8) * 16 + (k % 8) * 2);
//   * two threads per tile row gather h_e and the neighbour rows (float4
//     loads, two 8-channel chunks in flight at a time), sum, split and store
//     the three X parts in the same layout;
//   * one thread issues 8 K steps x 3 MMAs (M = 128, N = 64, K = 16) into 64
//     TMEM columns and commits to an mbarrier (bounded wait);
//   * the epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31 (its rows),
//     columns 32 (w / 4) .. + 31, adds the bias, writes a (optional) and h'.
// Shared memory 112 KB + barriers: 2 CTAs per SM; TMEM 64 columns per CTA.
// (Forming the neighbour sums in a separate gather kernel first, so that this
// kernel reads two contiguous rows per node, was measured: 22.5 us for this
// kernel plus the gather, 6 % slower per network application than the fused
// gather here.)
#pragma once

#include <cuda_bf16.h>

#include "dg_rhs_tct.cuh"

namespace dgk {

struct MpnnTc {
  static constexpr int kRows = 128;                 // nodes per tile (MMA M)
  static constexpr int kK = 128;                    // [h | m]
  static constexpr int kN = 64;                     // channels (MMA N)
  static constexpr int kThreads = 256;
  static constexpr uint32_t kSbo = (kK / 8) * 128;  // bytes between 8-row groups
  static constexpr uint32_t kBBytes = (kN / 8) * kSbo;     // 16 KB
  static constexpr uint32_t kABytes = (kRows / 8) * kSbo;  // 32 KB per split
  static constexpr uint32_t oBar = 0;               // mbarrier (8 B) + TMEM address (4 B)
  static constexpr uint32_t oBias = 16;             // 64 FP32 biases
  static constexpr uint32_t oB = 384;
  static constexpr uint32_t oA = oB + kBBytes;
  static constexpr uint32_t kSmem = oA + 3 * kABytes;
  static constexpr uint32_t kTmemCols = 64;
  // instruction descriptor: D f32 (bits 4-5 = 1), A and B bf16 (bits 7-9, 10-12 = 1),
  // both K-major, N >> 3 at bit 17, M >> 4 at bit 24
  static constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kN >> 3) << 17) |
                                     ((uint32_t)(kRows >> 4) << 24);
  static_assert(kSmem % 16 == 0 && oA % 128 == 0, "operand alignment");
};

// face neighbours of graph node e (sample s = e / K): up to 3 node indices, -1 on the boundary
__device__ __forceinline__ void neighbours(const int4* __restrict__ nbr, int K, int64_t e, int64_t (&j)[3]) {
  const int64_t s = e / K;
  const int4 n4 = __ldg(nbr + (e - s * K));
  const int c[3] = {n4.x, n4.y, n4.z};
#pragma unroll
  for (int f = 0; f < 3; ++f) j[f] = c[f] >= 0 ? s * K + (c[f] >> 2) : -1;
}

__device__ __forceinline__ uint32_t tc_off(int row, int k) {  // byte offset of (row, k) in an operand
  return (uint32_t)((row >> 3) * MpnnTc::kSbo + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ void tc_mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                            uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// eight FP32 values -> three 16-byte rows of BF16 parts (x = p0 + p1 + p2)
__device__ __forceinline__ void split3_store(const float (&v)[8], unsigned char* a0, unsigned char* a1,
                                             unsigned char* a2) {
  __align__(16) __nv_bfloat16 p[3][8];
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const __nv_bfloat16 b0 = __float2bfloat16_rn(v[i]);
    const float r1 = v[i] - __bfloat162float(b0);
    const __nv_bfloat16 b1 = __float2bfloat16_rn(r1);
    const float r2 = r1 - __bfloat162float(b1);
    p[0][i] = b0;
    p[1][i] = b1;
    p[2][i] = __float2bfloat16_rn(r2);
  }
  *reinterpret_cast<uint4*>(a0) = *reinterpret_cast<const uint4*>(p[0]);
  *reinterpret_cast<uint4*>(a1) = *reinterpret_cast<const uint4*>(p[1]);
  *reinterpret_cast<uint4*>(a2) = *reinterpret_cast<const uint4*>(p[2]);
}

__global__ void __launch_bounds__(MpnnTc::kThreads, 2)
    k_fwd_layer_tc(int64_t n, int K, const int4* __restrict__ nbr, const __nv_bfloat16* __restrict__ Ws,
                   const __nv_bfloat16* __restrict__ Wn, const __nv_bfloat16* __restrict__ bl,
                   const float* __restrict__ h, float* __restrict__ a_out, float* __restrict__ hn,
                   int linear, int* __restrict__ status) {
  using C = MpnnTc;
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + C::oBar);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + C::oBar + 8);
  unsigned char* sB = smem + C::oB;
  unsigned char* sA = smem + C::oA;
  float* sBias = reinterpret_cast<float*>(smem + C::oBias);
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;

  if (t == 0) {
    mbar_init(bar, 1);
    fence_barrier_init();
  }
  if (warp == 0) tmem_alloc_n(tmem_slot, C::kTmemCols);
  // W: row c = output channel, k < 64 from Ws[c][k], k >= 64 from Wn[c][k - 64];
  // 16-byte chunks of 8 consecutive k
  for (int q = t; q < C::kN * (C::kK / 8); q += C::kThreads) {
    const int c = q / (C::kK / 8), k0 = (q % (C::kK / 8)) * 8;
    const __nv_bfloat16* src = (k0 < C::kN ? Ws + c * C::kN + k0 : Wn + c * C::kN + (k0 - C::kN));
    *reinterpret_cast<uint4*>(sB + tc_off(c, k0)) = *reinterpret_cast<const uint4*>(src);
  }
  if (t < C::kN) sBias[t] = __bfloat162float(bl[t]);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  const uint32_t sA_u = smem_u32(sA), sB_u = smem_u32(sB);
  // thread t fills row t % 128, channel chunks (t / 128) * 4 .. + 3 of h and of m
  const int row = t & 127, half = t >> 7;
  // epilogue: rows of the warp's lane quadrant, its half of the channels
  const int erow = (warp & 3) * 32 + lane, ecol = (warp >> 2) * 32;
  uint32_t phase = 0;
  bool ok = true;
  for (int64_t n0 = (int64_t)blockIdx.x * C::kRows; n0 < n && ok; n0 += (int64_t)gridDim.x * C::kRows) {
    // ---- X = [h | m] of the tile, split into three BF16 parts
    {
      const int64_t e = n0 + row;
      int64_t j[3] = {-1, -1, -1};
      if (e < n) neighbours(nbr, K, e, j);
      // two chunks of 8 channels at a time, every load of both issued before use
#pragma unroll 1
      for (int cp = 0; cp < 2; ++cp) {
        float4 hl[2][2], ml[2][3][2];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          const int c0 = (half * 4 + cp * 2 + u) * 8;  // channels c0 .. c0 + 7
          const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
          hl[u][0] = hl[u][1] = z4;
          if (e < n) {
            const float4* hp = reinterpret_cast<const float4*>(h + e * C::kN + c0);
            hl[u][0] = hp[0];
            hl[u][1] = hp[1];
          }
#pragma unroll
          for (int f = 0; f < 3; ++f) {
            ml[u][f][0] = ml[u][f][1] = z4;
            if (j[f] >= 0) {
              const float4* mp = reinterpret_cast<const float4*>(h + j[f] * C::kN + c0);
              ml[u][f][0] = mp[0];
              ml[u][f][1] = mp[1];
            }
          }
        }
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          const int c0 = (half * 4 + cp * 2 + u) * 8;
          const float hv[8] = {hl[u][0].x, hl[u][0].y, hl[u][0].z, hl[u][0].w,
                               hl[u][1].x, hl[u][1].y, hl[u][1].z, hl[u][1].w};
          float mv[8];
#pragma unroll
          for (int q = 0; q < 2; ++q) {
            mv[4 * q] = (ml[u][0][q].x + ml[u][1][q].x) + ml[u][2][q].x;
            mv[4 * q + 1] = (ml[u][0][q].y + ml[u][1][q].y) + ml[u][2][q].y;
            mv[4 * q + 2] = (ml[u][0][q].z + ml[u][1][q].z) + ml[u][2][q].z;
            mv[4 * q + 3] = (ml[u][0][q].w + ml[u][1][q].w) + ml[u][2][q].w;
          }
          split3_store(hv, sA + tc_off(row, c0), sA + C::kABytes + tc_off(row, c0),
                       sA + 2 * C::kABytes + tc_off(row, c0));
          split3_store(mv, sA + tc_off(row, C::kN + c0), sA + C::kABytes + tc_off(row, C::kN + c0),
                       sA + 2 * C::kABytes + tc_off(row, C::kN + c0));
        }
      }
    }
    // generic-proxy stores of X -> visible to the tensor core's async proxy
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (t == 0) {
#pragma unroll
      for (int s = 0; s < C::kK / 16; ++s) {
        const uint64_t db = smem_desc(sB_u + s * 256, 128, C::kSbo);
#pragma unroll
        for (int p = 0; p < 3; ++p) {
          const uint64_t da = smem_desc(sA_u + p * C::kABytes + s * 256, 128, C::kSbo);
          tc_mma_bf16(tmem, da, db, C::kIdesc, (s > 0 || p > 0) ? 1u : 0u);
        }
      }
      tc_commit(bar);
    }
    ok = __syncthreads_and(mbar_wait(bar, phase, status));
    if (!ok) {
      // error path (recorded in the status word): give the MMAs in flight one
      // more bounded wait before the tensor memory is released
      mbar_wait(bar, phase, nullptr);
      break;
    }
    phase ^= 1;
    tc_fence_after();
    // ---- epilogue
    {
      float v[32];
      tmem_ld32(tmem + ((uint32_t)((warp & 3) * 32) << 16) + ecol, v);
      const int64_t e = n0 + erow;
      if (e < n) {
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const float4 bq = *reinterpret_cast<const float4*>(sBias + ecol + 4 * q);
          const float4 a = make_float4(v[4 * q] + bq.x, v[4 * q + 1] + bq.y, v[4 * q + 2] + bq.z,
                                       v[4 * q + 3] + bq.w);
          if (a_out) *reinterpret_cast<float4*>(a_out + e * C::kN + ecol + 4 * q) = a;
          const float4 hh = *reinterpret_cast<const float4*>(h + e * C::kN + ecol + 4 * q);
          *reinterpret_cast<float4*>(hn + e * C::kN + ecol + 4 * q) =
              linear ? make_float4(hh.x + a.x, hh.y + a.y, hh.z + a.z, hh.w + a.w)
                     : make_float4(hh.x + fmaxf(a.x, 0.f), hh.y + fmaxf(a.y, 0.f), hh.z + fmaxf(a.z, 0.f),
                                   hh.w + fmaxf(a.w, 0.f));
        }
      }
    }
    // TMEM read and the tile's shared rows consumed before the next tile overwrites them
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc_n(tmem, C::kTmemCols);
}

}  // namespace dgk
