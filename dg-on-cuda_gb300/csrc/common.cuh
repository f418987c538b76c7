// common.cuh -- shared device helpers: compile-time element sizes, bulk copies
// (cp.async.bulk) into shared memory with mbarrier completion, and bounded waits.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace dgk {

template <int N>
struct Order {
  static constexpr int Np = (N + 1) * (N + 2) / 2;
  static constexpr int Nfp = N + 1;
  static constexpr int NpP = (Np + 3) / 4 * 4;  // padded to 16-byte vectors of FP32
  static constexpr int Nface = 3 * Nfp;
};

// face-node index, counter-clockwise (see setup.hpp: face_node)
template <int N>
__host__ __device__ constexpr int fmask(int f, int d) {
  return f == 0 ? d
                : (f == 1 ? d * (N + 1) - d * (d - 1) / 2 + N - d
                          : (N - d) * (N + 1) - (N - d) * (N - d - 1) / 2);
}

// error codes written to the per-handle device status word
enum : int {
  kErrNone = 0,
  kErrBarrierTimeout = 1,  // an mbarrier wait gave up
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_barrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// plain arrival (release semantics for the arriving thread's prior writes)
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

// 1D bulk copy global -> shared, completion signalled on the mbarrier.
// dst, src 16-byte aligned; bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Wait for phase `parity` of the barrier to complete.  Gives up after about
// one second, records kErrBarrierTimeout in status[0] and returns false.  The
// first wait to give up also records, in the 8-byte words at status + 2,
// status + 4 and status + 6: the elapsed global-timer ns, the elapsed SM
// cycles and the number of polls.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* status) {
  const uint32_t a = smem_u32(bar);
  uint64_t t0 = 0, c0 = 0;
  for (uint32_t it = 0;; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
    if (it == 64) {
      t0 = globaltimer_ns();
      c0 = clock64();
    }
    if (it > 64 && (it & 255) == 0) {
      const uint64_t dt = globaltimer_ns() - t0;
      if (dt > 1000000000ull) {
        if (status && atomicCAS(status, kErrNone, kErrBarrierTimeout) == kErrNone) {
          unsigned long long* rec = reinterpret_cast<unsigned long long*>(status + 2);
          rec[0] = dt;
          rec[1] = (unsigned long long)(clock64() - c0);
          rec[2] = it;
        }
        return false;
      }
    }
  }
}

// mbar_wait for waits that are expected to be long (a warp-specialized
// pipeline stage waiting for another stage): after a few polls the thread
// sleeps between polls (32 ns doubling to 512 ns), so that waiting warps leave
// their scheduler's issue slots to the warps doing the work.  Same one-second
// limit and error record as mbar_wait.
__device__ __forceinline__ bool mbar_wait_backoff(uint64_t* bar, uint32_t parity, int* status) {
  const uint32_t a = smem_u32(bar);
  uint64_t t0 = 0;
  uint32_t ns = 32;
  for (uint32_t it = 0;; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
    if (it == 4) t0 = globaltimer_ns();
    if (it > 4) {
      __nanosleep(ns);
      if (ns < 512) ns <<= 1;
      if ((it & 63) == 0 && globaltimer_ns() - t0 > 1000000000ull) {
        if (status && atomicCAS(status, kErrNone, kErrBarrierTimeout) == kErrNone) {
          unsigned long long* rec = reinterpret_cast<unsigned long long*>(status + 2);
          rec[0] = globaltimer_ns() - t0;
          rec[1] = 0;
          rec[2] = it;
        }
        return false;
      }
    }
  }
}

// Programmatic dependent launch.  A stage kernel launched with programmatic
// stream serialization may start while the previous kernel of its stream is
// still running; grid_dep_wait blocks the calling thread until that kernel has
// completed and its memory operations are visible (a no-op for a kernel
// launched without the attribute), so it precedes every access to data the
// previous launch reads or writes.  grid_dep_launch lets the next kernel of the
// stream be scheduled once every CTA of this grid has executed it or exited;
// that kernel still waits for this one's completion before touching its data.
__device__ __forceinline__ void grid_dep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void grid_dep_launch() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <typename R>
struct Vec16;
template <>
struct Vec16<float> { using T = float4; static constexpr int n = 4; };
template <>
struct Vec16<double> { using T = double2; static constexpr int n = 2; };

}  // namespace dgk
