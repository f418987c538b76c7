// io.cu -- files: the reference drivers' visualisation text format and binary
// state checkpoints (C ABI: dgc_write_data_file, dgc_save_state,
// dgc_load_state).  Host code; checkpoints copy the state through pinned
// memory on the caller's stream.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "dgc_gb300.h"
#include "dgc_internal.hpp"

using namespace dgc;

namespace {

struct FileCloser {
  FILE* f;
  ~FileCloser() {
    if (f) std::fclose(f);
  }
};

// FNV-1a over the payload bytes
uint64_t fnv1a(const unsigned char* p, size_t n) {
  uint64_t h = 1469598103934665603ull;
  for (size_t i = 0; i < n; ++i) {
    h ^= p[i];
    h *= 1099511628211ull;
  }
  return h;
}

constexpr char kMagic[8] = {'D', 'G', 'C', 'S', 'T', 'A', 'T', 'E'};
constexpr int32_t kVersion = 1;

struct StateHeader {
  char magic[8];
  int32_t version, physics, order, np, np_padded, num_fields, precision, reserved;
  int64_t num_cells, state_len;
  double t;
  uint64_t checksum;
};

}  // namespace

extern "C" int dgc_write_data_file(const char* path, int64_t n, const double* x, const double* y, const double* u,
                                   const double* ref) {
  if (!path || n < 0 || (n > 0 && (!x || !y || !u))) return set_error(DGC_ERR_ARG, "null argument");
  FileCloser fc{std::fopen(path, "w")};
  if (!fc.f) return set_error(DGC_ERR_ARG, "cannot open the output file");
  // 15 significant digits in general notation: what an ostream with
  // precision(numeric_limits<double>::digits10) prints for a double
  auto block = [&](const char* header, const double* v) {
    std::fprintf(fc.f, "%s\n", header);
    for (int64_t i = 0; i < n; ++i) std::fprintf(fc.f, "%.15g  %.15g  %.15g\n", x[i], y[i], v[i]);
  };
  block("#         x         y         u", u);
  std::fprintf(fc.f, "\n");
  if (ref) block("#         x         y         reference solution", ref);
  if (std::ferror(fc.f)) return set_error(DGC_ERR_ARG, "write error");
  return DGC_OK;
}

extern "C" int dgc_save_state(dgc_handle h, const char* path, const void* q, double t, void* stream) {
  if (!h || !path || !q) return set_error(DGC_ERR_ARG, "null argument");
  const size_t bytes = dgc::state_bytes(h);
  std::vector<unsigned char> host(bytes);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemcpyAsync(host.data(), q, bytes, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return set_error(DGC_ERR_CUDA, cudaGetErrorString(e));
  StateHeader hd{};
  std::memcpy(hd.magic, kMagic, 8);
  hd.version = kVersion;
  hd.physics = h->desc.physics;
  hd.order = h->N;
  hd.np = h->Np;
  hd.np_padded = h->NpP;
  hd.num_fields = h->Nf;
  hd.precision = h->prec;
  hd.num_cells = h->K;
  hd.state_len = (int64_t)h->K * h->Nf * h->NpP;
  hd.t = t;
  hd.checksum = fnv1a(host.data(), bytes);
  FileCloser fc{std::fopen(path, "wb")};
  if (!fc.f) return set_error(DGC_ERR_ARG, "cannot open the checkpoint file");
  if (std::fwrite(&hd, sizeof hd, 1, fc.f) != 1 || std::fwrite(host.data(), 1, bytes, fc.f) != bytes)
    return set_error(DGC_ERR_ARG, "checkpoint write error");
  return DGC_OK;
}

extern "C" int dgc_load_state(dgc_handle h, const char* path, void* q, double* t, void* stream) {
  if (!h || !path || !q) return set_error(DGC_ERR_ARG, "null argument");
  FileCloser fc{std::fopen(path, "rb")};
  if (!fc.f) return set_error(DGC_ERR_ARG, "cannot open the checkpoint file");
  StateHeader hd{};
  if (std::fread(&hd, sizeof hd, 1, fc.f) != 1 || std::memcmp(hd.magic, kMagic, 8) != 0 || hd.version != kVersion)
    return set_error(DGC_ERR_ARG, "not a state checkpoint of this library");
  if (hd.physics != h->desc.physics || hd.order != h->N || hd.np_padded != h->NpP || hd.num_fields != h->Nf ||
      hd.precision != h->prec || hd.num_cells != h->K)
    return set_error(DGC_ERR_ARG, "checkpoint was written for another discretisation");
  const size_t bytes = (size_t)hd.state_len * (h->prec == DGC_F32 ? 4 : 8);
  std::vector<unsigned char> host(bytes);
  if (std::fread(host.data(), 1, bytes, fc.f) != bytes) return set_error(DGC_ERR_ARG, "checkpoint truncated");
  if (fnv1a(host.data(), bytes) != hd.checksum) return set_error(DGC_ERR_ARG, "checkpoint checksum mismatch");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemcpyAsync(q, host.data(), bytes, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return set_error(DGC_ERR_CUDA, cudaGetErrorString(e));
  if (t) *t = hd.t;
  return DGC_OK;
}
