// ref_adv1d.cpp -- drives the reference's own 1D advection example
// (examples/advection_1d/advection_1d.h, USE_CPU_ONLY) on K cells of order N
// and writes its operators and states as named arrays, plus the driver's error
// norm after `steps` RK4 steps.  Built only by oracle/Makefile against the
// reference sources; its outputs become golden vectors under tests/golden/.
//
// usage: ref_adv1d K N out.bin steps
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "advection_1d.h"
#include "axpy.h"
#include "explicit_runge_kutta.h"

static FILE* g_out = nullptr;

static void put(const char* name, const double* d, size_t n) {
  int32_t len = (int32_t)std::strlen(name), kind = 0;
  int64_t cnt = (int64_t)n;
  std::fwrite(&len, 4, 1, g_out); std::fwrite(name, 1, len, g_out);
  std::fwrite(&kind, 4, 1, g_out); std::fwrite(&cnt, 8, 1, g_out);
  std::fwrite(d, 8, n, g_out);
}
template <typename V> static void putv(const char* name, const V& v) { put(name, v.data(), v.size()); }

int main(int argc, char** argv) {
  if (argc < 5) { std::fprintf(stderr, "usage: ref_adv1d K N out.bin steps\n"); return 2; }
  const int K = std::atoi(argv[1]), N = std::atoi(argv[2]), steps = std::atoi(argv[4]);
  g_out = std::fopen(argv[3], "wb");
  if (!g_out) return 4;
  advection_1d<double> op(K, N);
  put("D", op.m_D.data(), op.m_D.size_row() * op.m_D.size_col());
  put("L", op.m_L.data(), op.m_L.size_row() * op.m_L.size_col());
  const int n = op.num_dofs();
  std::vector<double> x(n), u(n), out(n), w[5];
  for (auto& a : w) a.assign(n, 0.0);
  op.initialize_dofs(x.begin(), u.begin());
  putv("x", x);
  putv("u0", u);
  op(u.cbegin(), (std::size_t)n, 0.1, out.begin());
  putv("rhs", out);
  // the driver's time step (examples/advection_1d/main.cpp:94)
  const double dt = 0.25 / N / N * op.min_elem_size() / op.wave_speed();
  put("dt", &dt, 1);
  double t = 0.0;
  for (int i = 0; i < steps; ++i) {
    dgc::rk4(u.data(), (std::size_t)n, t, dt, op, &dgc::axpy_n<double, const double*, double*>,
             w[0].data(), w[1].data(), w[2].data(), w[3].data(), w[4].data());
    t += dt;
    if (i == 0) putv("rk4_1", u);
    if (i == 9) putv("rk4_10", u);
  }
  putv("rk4_final", u);
  // the driver's error norm (examples/advection_1d/main.cpp:41-47, 113-119)
  std::vector<double> ref(n);
  op.exact_solution(t, ref.begin());
  double err = 0.0;
  for (int i = 0; i < n; ++i) err += (ref[i] - u[i]) * (ref[i] - u[i]);
  err /= n;
  put("error_norm", &err, 1);
  put("t_final", &t, 1);
  std::fclose(g_out);
  return 0;
}
