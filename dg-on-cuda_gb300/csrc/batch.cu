// batch.cu -- many independent FP32 advection / Maxwell problems in one
// persistent launch per LSERK4 stage (the batched configuration; C ABI in
// include/dgc_gb300.h, dgc_batch_*).
//
// Work queue.  Each instance is cut into work items of up to kChunk tiles of
// its own tile size (RhsConfig<float, N, P>::TE); the items of all instances
// are ordered by decreasing cost (element-node-field count of the item,
// weighted by Np for the O(Np^2) contractions) so that the longest items start
// first.  A launch zeroes the queue head; every CTA takes items with one
// atomicAdd per item, loads that instance's operator matrices into shared
// memory and runs the tiles, dispatching on (order, physics, tile code):
//   code 0: the tile code of dg_rhs_kernel (rhs_v1_load_mats / rhs_v1_tile,
//           the handle's variant 0);
//   code 1: the register-blocked tiles of dg_rhs_blk_kernel with one element
//           per thread slot (blk_tiles, variant 5 at orders 1..6 and 1 at
//           orders 7, 8), double-buffered within each work item.
// An instance runs code 1 when its handle is set to that variant (e.g. by
// dgc_autotune) and code 0 otherwise, so a batched step is bitwise equal to
// the handle's own dgc_lserk4_step with either of those two variants.  The
// launch's dynamic shared memory is the largest layout among the batch's
// instances, which sets the resident CTAs per SM.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "dgc_gb300.h"
#include "dgc_internal.hpp"

namespace dgk {

struct BatchLaunch {
  const RhsParams* params;  // [instances] parameters of this stage
  const int* kinds;         // [instances] ((N - 1) * 3 + physics) * 2 + tile code
  const int4* items;        // [items] {instance, first tile, tiles, 0}
  int nitems;
  unsigned int* head;       // work-queue head, zero at launch
};

template <int N, int P>
__device__ __forceinline__ bool batch_item(const RhsParams& p, unsigned char* smem, uint32_t& phase, int tile0,
                                           int ntile) {
  using C = RhsConfig<float, N, P>;
  const V1Smem<float, N, P> s(smem);
  if (!rhs_v1_load_mats<float, N, P>(p, s, phase)) return false;
  for (int t = tile0; t < tile0 + ntile; ++t) {
    const int k0 = t * C::TE;
    if (!rhs_v1_tile<float, N, P>(p, s, phase, k0, min(C::TE, p.K - k0))) return false;
  }
  return true;
}

// One work item with either tile code.  Not inlined: each (order, physics,
// code) body gets its own register allocation instead of the union of all of
// them in one kernel body.
template <int N, int P>
__device__ __noinline__ bool batch_item_v0(const RhsParams& p, unsigned char* smem, uint32_t* ph, int tile0,
                                           int ntile) {
  return batch_item<N, P>(p, smem, ph[0], tile0, ntile);
}
template <int N, int P>
__device__ __noinline__ bool batch_item_blk(const RhsParams& p, unsigned char* smem, uint32_t* ph, int tile0,
                                            int ntile) {
  uint32_t loc[3] = {ph[0], ph[1], ph[2]};
  const bool ok = blk_tiles<N, P, 1, 0>(p, smem, loc, tile0, 1, tile0 + ntile);
  ph[0] = loc[0];
  ph[1] = loc[1];
  ph[2] = loc[2];
  return ok;
}

// largest dynamic shared memory of the FP32 tile layouts (both codes), orders 1..8
constexpr uint32_t umax(uint32_t a, uint32_t b) { return a > b ? a : b; }
template <int N>
constexpr uint32_t batch_smem_upto() {
  constexpr uint32_t a = umax(RhsConfig<float, N, PHYS_ADV>::kSmem, BlkConfig<N, PHYS_ADV, 1, 0>::kSmem),
                     b = umax(RhsConfig<float, N, PHYS_TM>::kSmem, BlkConfig<N, PHYS_TM, 1, 0>::kSmem),
                     c = umax(RhsConfig<float, N, PHYS_TE>::kSmem, BlkConfig<N, PHYS_TE, 1, 0>::kSmem);
  constexpr uint32_t m = umax(a, umax(b, c));
  if constexpr (N == 1) {
    return m;
  } else {
    constexpr uint32_t r = batch_smem_upto<N - 1>();
    return m > r ? m : r;
  }
}
constexpr uint32_t kBatchSmem = batch_smem_upto<8>();

__global__ void __launch_bounds__(256, 3) dg_batch_kernel(const BatchLaunch b) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ int s_item;
  // offset 0 of both tile layouts: barrier 0 (tiles of code 0, buffer 0 of
  // code 1), 1 (buffer 1 of code 1), 2 (operators of code 1)
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem);
  grid_dep_launch();  // the next stage may be scheduled; it waits for this grid before its reads
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_init(&bar[2], 1);
    fence_barrier_init();
  }
  __syncthreads();
  grid_dep_wait();  // every instance's state and residual are the previous stage's output
  uint32_t ph[3] = {0, 0, 0};
  for (;;) {
    if (threadIdx.x == 0) s_item = (int)atomicAdd(b.head, 1u);
    __syncthreads();
    const int it = s_item;
    __syncthreads();  // every thread has read s_item before thread 0 takes the next item
    if (it >= b.nitems) break;
    const int4 w = b.items[it];
    const RhsParams& p = b.params[w.x];
    bool ok = false;
    switch (b.kinds[w.x]) {
#define DGK_BATCH_PHYS(n, P)                                                                   \
  case ((n - 1) * 3 + P) * 2: ok = batch_item_v0<n, P>(p, smem, ph, w.y, w.z); break;         \
  case ((n - 1) * 3 + P) * 2 + 1: ok = batch_item_blk<n, P>(p, smem, ph, w.y, w.z); break;
#define DGK_BATCH_CASE(n) DGK_BATCH_PHYS(n, PHYS_ADV) DGK_BATCH_PHYS(n, PHYS_TM) DGK_BATCH_PHYS(n, PHYS_TE)
      DGK_BATCH_CASE(1) DGK_BATCH_CASE(2) DGK_BATCH_CASE(3) DGK_BATCH_CASE(4)
      DGK_BATCH_CASE(5) DGK_BATCH_CASE(6) DGK_BATCH_CASE(7) DGK_BATCH_CASE(8)
#undef DGK_BATCH_CASE
#undef DGK_BATCH_PHYS
      default: ok = false;
    }
    if (!ok) break;  // uniform: every wait ends in a CTA-wide AND
  }
}

// advance each instance's device time by its step
// a plain launch: it ends the overlap chain of one step's stage launches
__global__ void k_batch_clock(int n, double* const* t, const double* dt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) t[i][0] += dt[i];
}

}  // namespace dgk

struct dgc_batch_s {
  std::vector<dgc_handle> inst;
  int device = 0, sm_count = 0, blocks_per_sm = 1;
  int smem = 0;                     // dynamic shared memory of a launch (largest instance layout)
  std::vector<int> tile_size;       // per instance
  int nitems = 0;
  int* d_kinds = nullptr;
  int4* d_items = nullptr;
  unsigned int* d_head = nullptr;   // [5] queue heads, one per stage of a step
  dgk::RhsParams* d_params = nullptr;   // [5][instances]
  dgk::RhsParams* h_params = nullptr;   // pinned staging of the same
  double** d_time_ptrs = nullptr;   // [instances] each handle's device time
  double* d_dt = nullptr;           // [instances]
  int64_t launches = 0;
};

namespace {

int berr(int code, const char* msg) {
  dgc::set_error(code, msg);
  return code;
}
int bcuda(cudaError_t e, const char* what) {
  std::string m = std::string(what) + ": " + cudaGetErrorString(e);
  return berr(DGC_ERR_CUDA, m.c_str());
}
#define CKB(call)                                      \
  do {                                                 \
    cudaError_t e_ = (call);                           \
    if (e_ != cudaSuccess) return bcuda(e_, #call);    \
  } while (0)

constexpr int kChunk = 8;  // tiles per work item (DGC_BATCH_CHUNK overrides, 1..64)

int chunk_tiles() {
  static const int c = [] {
    const char* v = std::getenv("DGC_BATCH_CHUNK");
    const int x = v ? std::atoi(v) : 0;
    return x >= 1 && x <= 64 ? x : kChunk;
  }();
  return c;
}

int physics_kind(int phys) {
  return phys == DGC_ADVECTION ? dgk::PHYS_ADV : (phys == DGC_MAXWELL_TM ? dgk::PHYS_TM : dgk::PHYS_TE);
}

// the FP32 variant that runs the register-blocked tiles with one element per
// thread slot (batch tile code 1)
int blk_variant(int N) { return N <= 6 ? 5 : 1; }

// tile size and shared memory of an (order, physics, variant) stage kernel
bool tile_info(int N, int phys, int variant, dgk::LaunchInfo* li) {
  dgk::RhsParams dummy{};
  return dgk::rhs_dispatch<float>(N, phys, variant, dummy, 1, 0, li) == cudaSuccess;
}

// parameters of one LSERK stage for every instance, into b->h_params[stage]
void fill_stage(dgc_batch b, int stage, void* const* q_in, void* const* q_out, void* const* res, const double* t,
                const double* dt, bool device_time) {
  const double* A = dgc::lserk_coeffs(0);
  const double* B = dgc::lserk_coeffs(1);
  const double* Cc = dgc::lserk_coeffs(2);
  const int n = (int)b->inst.size();
  for (int i = 0; i < n; ++i) {
    dgk::RhsParams p = dgc::rhs_base_params(b->inst[i]);
    p.mode = dgk::MODE_LSERK;
    p.q_in = q_in[i];
    p.out = q_out[i];
    p.aux = res[i];
    p.dt = dt[i];
    p.ca = A[stage];
    p.cb = B[stage];
    if (device_time) {
      p.t_dev = b->inst[i]->d_time;
      p.t = Cc[stage] * dt[i];
    } else {
      p.t = t[i] + Cc[stage] * dt[i];
    }
    b->h_params[(size_t)stage * n + i] = dgk::with_f32_scalars(p);
  }
}

// the five stage launches of one step (parameters already on the device)
int launch_step(dgc_batch b, cudaStream_t s) {
  const int n = (int)b->inst.size();
  const int grid = std::max(1, std::min(b->nitems, b->sm_count * b->blocks_per_sm));
  CKB(cudaMemsetAsync(b->d_head, 0, 5 * sizeof(unsigned int), s));
  for (int st = 0; st < 5; ++st) {
    dgk::BatchLaunch L{b->d_params + (size_t)st * n, b->d_kinds, b->d_items, b->nitems, b->d_head + st};
    CKB(dgk::launch_stage(dgk::dg_batch_kernel, grid, 256, b->smem, s, L));
    ++b->launches;
  }
  return DGC_OK;
}

int check_buffers(dgc_batch b, void* const* a, void* const* c, void* const* r) {
  if (!b || !a || !c || !r) return berr(DGC_ERR_ARG, "null argument");
  for (size_t i = 0; i < b->inst.size(); ++i) {
    if (!a[i] || !c[i] || !r[i]) return berr(DGC_ERR_ARG, "null state buffer");
    if (a[i] == c[i] || a[i] == r[i] || c[i] == r[i])
      return berr(DGC_ERR_ARG, "state, scratch and residual buffers must be distinct");
    if (((uintptr_t)a[i] | (uintptr_t)c[i] | (uintptr_t)r[i]) & 15u)
      return berr(DGC_ERR_ARG, "state buffers must be 16-byte aligned");
  }
  return DGC_OK;
}

}  // namespace

extern "C" int dgc_batch_create(const dgc_handle* handles, int n, dgc_batch* out) {
  if (!handles || !out || n <= 0) return berr(DGC_ERR_ARG, "null argument or empty batch");
  *out = nullptr;
  auto* b = new dgc_batch_s();
  auto fail = [&](int rc) {
    dgc_batch_destroy(b);
    return rc;
  };
  b->inst.assign(handles, handles + n);
  std::vector<int> kinds(n);
  struct Item { int inst, tile0, ntile; double cost; };
  std::vector<Item> items;
  for (int i = 0; i < n; ++i) {
    dgc_handle h = handles[i];
    if (!h) return fail(berr(DGC_ERR_ARG, "null handle in batch"));
    if (h->prec != DGC_F32) return fail(berr(DGC_ERR_UNSUPPORTED, "batches run FP32 handles"));
    if (h->desc.physics == DGC_LAPLACE) return fail(berr(DGC_ERR_UNSUPPORTED, "batches run time-dependent handles"));
    const int P = physics_kind(h->desc.physics);
    const int code = h->rhs_variant == blk_variant(h->N) ? 1 : 0;
    kinds[i] = ((h->N - 1) * 3 + P) * 2 + code;
    dgk::LaunchInfo li;
    if (!tile_info(h->N, h->desc.physics, code ? blk_variant(h->N) : 0, &li) || li.tile <= 0)
      return fail(berr(DGC_ERR_CUDA, "configure batch tile"));
    const int te = li.tile;
    b->smem = std::max(b->smem, li.smem);
    b->tile_size.push_back(te);
    const int ntiles = (h->K + te - 1) / te;
    const int chunk = chunk_tiles();
    for (int t0 = 0; t0 < ntiles; t0 += chunk) {
      const int nt = std::min(chunk, ntiles - t0);
      const int ne = std::min(nt * te, h->K - t0 * te);
      items.push_back({i, t0, nt, (double)ne * h->Nf * h->Np * (double)h->Np});
    }
  }
  std::stable_sort(items.begin(), items.end(), [](const Item& a, const Item& c) { return a.cost > c.cost; });
  std::vector<int4> hitems(items.size());
  for (size_t k = 0; k < items.size(); ++k) hitems[k] = make_int4(items[k].inst, items[k].tile0, items[k].ntile, 0);
  b->nitems = (int)items.size();
  cudaError_t e = cudaGetDevice(&b->device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, b->device);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(dgk::dg_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, dgk::kBatchSmem);
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b->blocks_per_sm, dgk::dg_batch_kernel, 256, b->smem);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_kinds, n * sizeof(int));
  if (e == cudaSuccess) e = cudaMemcpy(b->d_kinds, kinds.data(), n * sizeof(int), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_items, hitems.size() * sizeof(int4));
  if (e == cudaSuccess)
    e = cudaMemcpy(b->d_items, hitems.data(), hitems.size() * sizeof(int4), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_head, 5 * sizeof(unsigned int));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_params, (size_t)5 * n * sizeof(dgk::RhsParams));
  if (e == cudaSuccess) e = cudaMallocHost(&b->h_params, (size_t)5 * n * sizeof(dgk::RhsParams));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_time_ptrs, n * sizeof(double*));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_dt, n * sizeof(double));
  if (e == cudaSuccess) {
    std::vector<double*> tp(n);
    for (int i = 0; i < n; ++i) tp[i] = handles[i]->d_time;
    e = cudaMemcpy(b->d_time_ptrs, tp.data(), n * sizeof(double*), cudaMemcpyHostToDevice);
  }
  if (e != cudaSuccess) return fail(bcuda(e, "batch set-up"));
  if (b->blocks_per_sm < 1) b->blocks_per_sm = 1;
  *out = b;
  return DGC_OK;
}

extern "C" int dgc_batch_destroy(dgc_batch b) {
  if (!b) return DGC_OK;
  cudaFree(b->d_kinds);
  cudaFree(b->d_items);
  cudaFree(b->d_head);
  cudaFree(b->d_params);
  cudaFreeHost(b->h_params);
  cudaFree(b->d_time_ptrs);
  cudaFree(b->d_dt);
  delete b;
  return DGC_OK;
}

extern "C" int dgc_batch_lserk4_step(dgc_batch b, void* const* q_in, void* const* q_out, void* const* res,
                                     const double* t, const double* dt, void* stream) {
  if (int rc = check_buffers(b, q_in, q_out, res)) return rc;
  if (!t || !dt) return berr(DGC_ERR_ARG, "null time arrays");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int n = (int)b->inst.size();
  // the stage parameters ping-pong q_in -> q_out -> q_in ...; the staging
  // buffer is reused only after the copy that reads it has completed
  CKB(cudaStreamSynchronize(s));
  for (int st = 0; st < 5; ++st) {
    const bool even = (st % 2) == 0;
    fill_stage(b, st, even ? q_in : q_out, even ? q_out : q_in, res, t, dt, false);
  }
  CKB(cudaMemcpyAsync(b->d_params, b->h_params, (size_t)5 * n * sizeof(dgk::RhsParams), cudaMemcpyHostToDevice, s));
  return launch_step(b, s);
}

extern "C" int dgc_batch_lserk4_run(dgc_batch b, void* const* qa, void* const* qb, void* const* res,
                                    const double* t0, const double* dt, int nsteps, int use_graph, int* final_in_qb,
                                    void* stream) {
  if (int rc = check_buffers(b, qa, qb, res)) return rc;
  if (!t0 || !dt || nsteps < 0) return berr(DGC_ERR_ARG, "null time arrays or negative step count");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int n = (int)b->inst.size();
  CKB(cudaStreamSynchronize(s));
  // each instance's time lives in its handle's device word, advanced by dt
  for (int i = 0; i < n; ++i) CKB(cudaMemcpyAsync(b->inst[i]->d_time, &t0[i], sizeof(double), cudaMemcpyHostToDevice, s));
  CKB(cudaMemcpyAsync(b->d_dt, dt, n * sizeof(double), cudaMemcpyHostToDevice, s));
  // two parameter sets: even steps qa -> qb, odd steps qb -> qa (5 stages each)
  std::vector<dgk::RhsParams> sets((size_t)10 * n);
  for (int par = 0; par < 2; ++par) {
    void* const* x = par == 0 ? qa : qb;
    void* const* y = par == 0 ? qb : qa;
    for (int st = 0; st < 5; ++st) {
      const bool even = (st % 2) == 0;
      fill_stage(b, st, even ? x : y, even ? y : x, res, t0, dt, true);
    }
    std::memcpy(sets.data() + (size_t)par * 5 * n, b->h_params, (size_t)5 * n * sizeof(dgk::RhsParams));
  }
  // the device parameter array holds one step; alternate steps need the other set
  dgk::RhsParams* d_sets = nullptr;
  CKB(cudaMalloc(&d_sets, sets.size() * sizeof(dgk::RhsParams)));
  CKB(cudaMemcpyAsync(d_sets, sets.data(), sets.size() * sizeof(dgk::RhsParams), cudaMemcpyHostToDevice, s));
  dgk::RhsParams* saved = b->d_params;
  auto one_step = [&](int par, cudaStream_t cs) -> int {
    b->d_params = d_sets + (size_t)par * 5 * n;
    const int rc = launch_step(b, cs);
    b->d_params = saved;
    if (rc) return rc;
    dgk::k_batch_clock<<<(n + 127) / 128, 128, 0, cs>>>(n, b->d_time_ptrs, b->d_dt);
    CKB(cudaGetLastError());
    ++b->launches;
    return DGC_OK;
  };
  int done = 0, rc = DGC_OK;
  if (use_graph && nsteps >= 2) {
    // a graph of two steps (qa -> qb -> qa); replayed while at least two remain
    cudaStream_t cs;
    CKB(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    const int64_t l0 = b->launches;
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      rc = one_step(0, cs);
      if (rc == DGC_OK) rc = one_step(1, cs);
      e = cudaStreamEndCapture(cs, &g);
    }
    const int64_t per_graph = b->launches - l0;
    b->launches = l0;
    cudaStreamDestroy(cs);
    if (rc == DGC_OK && e == cudaSuccess) e = cudaGraphInstantiate(&ge, g, 0);
    if (g) cudaGraphDestroy(g);
    if (rc == DGC_OK && e != cudaSuccess) rc = bcuda(e, "batch graph");
    for (; rc == DGC_OK && done + 2 <= nsteps; done += 2) {
      e = cudaGraphLaunch(ge, s);
      if (e != cudaSuccess) rc = bcuda(e, "batch graph launch");
      b->launches += per_graph;
    }
    if (ge) cudaGraphExecDestroy(ge);
  }
  for (; rc == DGC_OK && done < nsteps; ++done) rc = one_step(done & 1, s);
  cudaError_t e2 = cudaStreamSynchronize(s);
  cudaFree(d_sets);
  if (rc) return rc;
  if (e2 != cudaSuccess) return bcuda(e2, "batch run");
  if (final_in_qb) *final_in_qb = nsteps & 1;
  return DGC_OK;
}

extern "C" int64_t dgc_batch_launch_count(dgc_batch b) { return b ? b->launches : -1; }
