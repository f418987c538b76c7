// ref_time.cpp -- times the reference's own USE_CPU_ONLY operators (serial) on a
// binary mesh: classical-RK4 steps of advection_2d and maxwell_2d through
// dgc::rk4, as the reference drivers do (examples/*/main.cpp).  Prints one JSON
// line.  Built only by oracle/Makefile against the reference sources.
//
// usage: ref_time mesh.bin order problem(adv|mx) steps [T]
//   with T > 0 the loop instead runs to time T, shortening the last step
//   (examples/maxwell_2d/main.cpp:199-209); the printed "mse" is the
//   reference's error measure (examples/advection_2d/main.cpp:45-51).
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include <thrust/host_vector.h>
#include <thrust/iterator/zip_iterator.h>

#include "simple_triangular_mesh_2d.h"
#include "advection_2d.h"
#include "maxwell_2d.h"
#include "axpy.h"
#include "explicit_runge_kutta.h"

using Mesh = dgc::simple_triangular_mesh_2d<double, int>;

int main(int argc, char** argv) {
  if (argc < 5) return 2;
  FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 3;
  int32_t nv, K;
  if (std::fread(&nv, 4, 1, f) != 1) return 3;
  std::vector<double> xy(2 * (size_t)nv);
  if (std::fread(xy.data(), 8, xy.size(), f) != xy.size()) return 3;
  if (std::fread(&K, 4, 1, f) != 1) return 3;
  std::vector<int> cells(3 * (size_t)K);
  if (std::fread(cells.data(), 4, cells.size(), f) != cells.size()) return 3;
  std::fclose(f);
  Mesh mesh;
  mesh.fill_vertices(xy.begin(), xy.end());
  mesh.fill_connectivity(cells.begin(), cells.end());
  mesh.build_topology();
  const int N = std::atoi(argv[2]);
  const std::string prob = argv[3];
  int steps = std::atoi(argv[4]);
  const double T = argc > 5 ? std::atof(argv[5]) : 0.0;
  const double l = 2.0 / std::sqrt((double)K);
  const double dt = (2.0 / 3.0) * (l / (double)N) * (l / (2.0 + std::sqrt(2.0)));
  double secs = 0.0, t = 0.0, mse = 0.0;
  long n = 0;
  int nf = 1;
  if (prob == "adv") {
    advection_2d<double, Mesh> op(mesh, N);
    n = op.total_num_nodes();
    std::vector<dgc::point_2d<double>> x(n);
    std::vector<double> u(n), w[5];
    for (auto& a : w) a.assign(n, 0.0);
    op.initialize_dofs(x.begin(), u.begin());
    auto t0 = std::chrono::steady_clock::now();
    for (int i = 0; i < steps; ++i) {
      dgc::rk4(u.data(), (std::size_t)n, t, dt, op, &dgc::axpy_n<double, const double*, double*>,
               w[0].data(), w[1].data(), w[2].data(), w[3].data(), w[4].data());
      t += dt;
    }
    secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::vector<double> ref(n);
    op.exact_solution(t, ref.begin());
    for (long i = 0; i < n; ++i) mse += (ref[i] - u[i]) * (ref[i] - u[i]);
    mse /= n;
  } else {
    nf = 3;
    maxwell_2d<double, Mesh> op(mesh, N);
    n = op.total_num_nodes();
    using HV = thrust::host_vector<double>;
    using HZ = thrust::zip_iterator<thrust::tuple<HV::iterator, HV::iterator, HV::iterator>>;
    HV fld[6][3];
    for (auto& a : fld) for (auto& b : a) b.assign(n, 0.0);
    auto zip = [&](int i) { return thrust::make_zip_iterator(thrust::make_tuple(fld[i][0].begin(), fld[i][1].begin(), fld[i][2].begin())); };
    std::vector<dgc::point_2d<double>> x(n);
    op.initialize_dofs(x.begin(), zip(0));
    double h = dt;
    auto t0 = std::chrono::steady_clock::now();
    if (T > 0.0) {
      steps = 0;
      while (t < T) {
        if (t + h > T) h = T - t;
        dgc::rk4(zip(0), (std::size_t)n, t, h, op, &dgc::axpy_n<double, HZ, HZ>, zip(1), zip(2), zip(3), zip(4), zip(5));
        t += h;
        ++steps;
      }
    } else {
      for (int i = 0; i < steps; ++i) {
        dgc::rk4(zip(0), (std::size_t)n, t, dt, op, &dgc::axpy_n<double, HZ, HZ>, zip(1), zip(2), zip(3), zip(4), zip(5));
        t += dt;
      }
    }
    secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    HV ex[3];
    for (auto& a : ex) a.assign(n, 0.0);
    op.exact_solution(t, thrust::make_zip_iterator(thrust::make_tuple(ex[0].begin(), ex[1].begin(), ex[2].begin())));
    for (int c = 0; c < 3; ++c)
      for (long i = 0; i < n; ++i) mse += (ex[c][i] - fld[0][c][i]) * (ex[c][i] - fld[0][c][i]);
    mse /= n;
  }
  const double rhs_evals = 4.0 * steps;
  std::printf("{\"problem\": \"%s\", \"K\": %d, \"order\": %d, \"steps\": %d, \"seconds\": %.6f, "
              "\"gdof_per_s\": %.6e, \"t_final\": %.17g, \"mse\": %.17g}\n",
              prob.c_str(), K, N, steps, secs, (double)nf * n * rhs_evals / secs / 1e9, t, mse);
  return 0;
}
