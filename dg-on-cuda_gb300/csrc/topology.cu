// topology.cu -- half-edge matching on the GPU for large meshes: the twin map
// that simple_triangular_mesh_2d::build_topology builds with a std::map
// (src/mesh/simple_triangular_mesh_2d.h:151-217), and the host path in
// setup.cpp with a sort.
//
// Half-edge h = 3 k + f of cell k runs from cells[3k+f] to cells[3k+(f+1)%3];
// its key is the unordered vertex pair (min << 32 | max).  One thread per
// half-edge inserts the key into an open-addressing table (linear probing,
// capacity a power of two >= 2 x the half-edge count) and claims one of the
// two id slots of its entry with atomicCAS; a second pass reads the entry
// back: the other id is the twin, none means a boundary face.  Every probe
// loop is bounded by the capacity; edges shared by more than two cells,
// inconsistently oriented twins and a full table are reported through an
// error word, never by a trap.  The results equal the host sort's exactly
// (twins are unique), so build_mesh picks either path by size.
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "setup.hpp"

namespace dgk {

constexpr unsigned long long kEmptyKey = ~0ull;
enum TopoError : int { kTopoOk = 0, kTopoNonManifold = 1, kTopoOrientation = 2, kTopoFull = 3 };

__device__ __forceinline__ unsigned long long he_key(const int32_t* __restrict__ cells, int64_t h) {
  const int64_t k = h / 3;
  const int f = (int)(h - 3 * k);
  const uint32_t a = (uint32_t)cells[3 * k + f], b = (uint32_t)cells[3 * k + (f == 2 ? 0 : f + 1)];
  return (unsigned long long)(a < b ? a : b) << 32 | (a < b ? b : a);
}

__device__ __forceinline__ uint64_t he_hash(unsigned long long key) {
  // splitmix64 finaliser
  uint64_t z = key + 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

__device__ __forceinline__ void topo_fail(int* err, int64_t* where, int code, int64_t h) {
  if (atomicCAS(err, kTopoOk, code) == kTopoOk) *where = h;
}

__global__ void k_he_insert(int64_t nhe, const int32_t* __restrict__ cells, uint64_t mask,
                            unsigned long long* __restrict__ keys, int32_t* __restrict__ ids, int* err,
                            int64_t* where) {
  for (int64_t h = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; h < nhe; h += (int64_t)gridDim.x * blockDim.x) {
    const unsigned long long key = he_key(cells, h);
    uint64_t s = he_hash(key) & mask;
    bool placed = false;
    for (uint64_t probe = 0; probe <= mask; ++probe, s = (s + 1) & mask) {
      const unsigned long long prev = atomicCAS(&keys[s], kEmptyKey, key);
      if (prev != kEmptyKey && prev != key) continue;
      if (atomicCAS(&ids[2 * s], -1, (int32_t)h) != -1 && atomicCAS(&ids[2 * s + 1], -1, (int32_t)h) != -1)
        topo_fail(err, where, kTopoNonManifold, h);
      placed = true;
      break;
    }
    if (!placed) topo_fail(err, where, kTopoFull, h);
  }
}

// twin[h] = twin half-edge (k << 2 | f) or -1 on the boundary
__global__ void k_he_resolve(int64_t nhe, const int32_t* __restrict__ cells, uint64_t mask,
                             const unsigned long long* __restrict__ keys, const int32_t* __restrict__ ids,
                             int32_t* __restrict__ twin, int* err, int64_t* where) {
  for (int64_t h = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; h < nhe; h += (int64_t)gridDim.x * blockDim.x) {
    const unsigned long long key = he_key(cells, h);
    uint64_t s = he_hash(key) & mask;
    int32_t out = -1;
    for (uint64_t probe = 0; probe <= mask; ++probe, s = (s + 1) & mask) {
      const unsigned long long k = keys[s];
      if (k == kEmptyKey) break;  // not found: the insert pass reported it
      if (k != key) continue;
      const int32_t a = ids[2 * s], b = ids[2 * s + 1];
      const int32_t o = a == (int32_t)h ? b : a;
      if (o >= 0) {
        // a conforming, consistently oriented mesh traverses a shared edge in
        // opposite directions from its two sides
        if (cells[o] == cells[h]) topo_fail(err, where, kTopoOrientation, h);
        const int32_t ko = o / 3;
        out = ko << 2 | (o - 3 * ko);
      }
      break;
    }
    twin[h] = out;
  }
}

}  // namespace dgk

namespace dgc {

namespace {

struct DevBuf {
  void* p = nullptr;
  ~DevBuf() { cudaFree(p); }
};

}  // namespace

bool gpu_match_half_edges(const int32_t* cells, int K, std::vector<int32_t>& twin, std::string& err) {
  const int64_t nhe = 3 * (int64_t)K;
  uint64_t cap = 1;
  while (cap < 2 * (uint64_t)nhe) cap <<= 1;
  DevBuf dcells, dkeys, dids, dtwin, dstat;
  auto ck = [&](cudaError_t e, const char* what) {
    if (e == cudaSuccess) return true;
    err = std::string("GPU topology: ") + what + ": " + cudaGetErrorString(e);
    return false;
  };
  if (!ck(cudaMalloc(&dcells.p, nhe * 4), "allocation") || !ck(cudaMalloc(&dkeys.p, cap * 8), "allocation") ||
      !ck(cudaMalloc(&dids.p, cap * 8), "allocation") || !ck(cudaMalloc(&dtwin.p, nhe * 4), "allocation") ||
      !ck(cudaMalloc(&dstat.p, 16), "allocation"))
    return false;
  if (!ck(cudaMemcpy(dcells.p, cells, nhe * 4, cudaMemcpyHostToDevice), "upload") ||
      !ck(cudaMemset(dkeys.p, 0xff, cap * 8), "clear") || !ck(cudaMemset(dids.p, 0xff, cap * 8), "clear") ||
      !ck(cudaMemset(dstat.p, 0, 16), "clear"))
    return false;
  int* derr = static_cast<int*>(dstat.p);
  int64_t* dwhere = reinterpret_cast<int64_t*>(static_cast<char*>(dstat.p) + 8);
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int grid = (int)std::min<int64_t>((nhe + 255) / 256, (int64_t)sms * 8);
  const auto* c = static_cast<const int32_t*>(dcells.p);
  auto* keys = static_cast<unsigned long long*>(dkeys.p);
  auto* ids = static_cast<int32_t*>(dids.p);
  dgk::k_he_insert<<<grid, 256>>>(nhe, c, cap - 1, keys, ids, derr, dwhere);
  dgk::k_he_resolve<<<grid, 256>>>(nhe, c, cap - 1, keys, ids, static_cast<int32_t*>(dtwin.p), derr, dwhere);
  if (!ck(cudaGetLastError(), "launch")) return false;
  int code = 0;
  int64_t where = 0;
  twin.resize(nhe);
  if (!ck(cudaMemcpy(twin.data(), dtwin.p, nhe * 4, cudaMemcpyDeviceToHost), "download") ||
      !ck(cudaMemcpy(&code, derr, 4, cudaMemcpyDeviceToHost), "download") ||
      !ck(cudaMemcpy(&where, dwhere, 8, cudaMemcpyDeviceToHost), "download"))
    return false;
  if (code != dgk::kTopoOk) {
    const int k = (int)(where / 3);
    err = code == dgk::kTopoNonManifold  ? "non-manifold edge (more than two cells) at cell " + std::to_string(k)
          : code == dgk::kTopoOrientation ? "inconsistently oriented neighbours at cell " + std::to_string(k)
                                          : std::string("GPU topology: hash table full");
    return false;
  }
  return true;
}

}  // namespace dgc
