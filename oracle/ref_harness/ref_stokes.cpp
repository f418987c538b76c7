// ref_stokes.cpp -- probes the reference's Stokes example (examples/stokes_2d/
// stokes_2d.h, USE_CPU_ONLY layout [cell][node]) up to its linear solves.
// Built only by oracle/Makefile against the reference sources; its outputs
// become golden vectors under tests/golden/.
//
// Given u^(n-1), u^n, t_prev, t and dt it writes what pressure_step forms
// before solve_sys: pressure_bc's Neumann values (exterior_grad_n(x, y, 0) =
// 2 hp, in the order the reference consumes them), the right-hand side
// (div_2d of u~ with u_tilde_bc, times 1.5/dt, plus
// apply_inhomogeneous_as_rhs) and the matrix of build_poisson_sys_matrix.
// Given also p it writes what projection_step and viscous_step form: grad p
// (pressure_bc_proj), u~ after the projection, the matrix of
// build_helmholtz_sys_matrix and the two right-hand sides.  solve_sys (a
// cuSOLVER host LU; cusolverSpCreate needs a GPU) is never instantiated: the
// caller solves.  The mass matrix (V V^T)^-1 and the cell Jacobians come from
// the reference's own classes as well.
//
// The members are private: the probe derives from stokes_2d, with `private`
// defined as `public` around the one #include of stokes_2d.h (its other
// headers are included first, unaffected).
//
// usage: ref_stokes mesh.bin order state.bin out.bin
//   mesh.bin : int32 nv, f64 xy[2 nv], int32 K, int32 cells[3 K]
//   state.bin: f64 t_prev, t, dt, int32 has_p, f64 u0x[n], u0y[n], u1x[n], u1y[n] [, p[n]]
//              (n = K Np; u0 = u^(n-1), u1 = u^n)
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include <thrust/host_vector.h>
#include <thrust/iterator/zip_iterator.h>
#include <thrust/tuple.h>

#include <cusolverSp.h>
#include <cusparse.h>

#include "simple_triangular_mesh_2d.h"
#include "reference_triangle.h"
#include "simple_discretization_2d.h"
#include "div_2d.h"
#include "grad_2d.h"
#include "laplace_2d.h"

#define private public
#include "stokes_2d.h"
#undef private

using Mesh = dgc::simple_triangular_mesh_2d<double, int>;

static FILE* g_out = nullptr;

static void put(const char* name, const double* d, size_t n) {
  int32_t len = (int32_t)std::strlen(name), kind = 0;
  int64_t cnt = (int64_t)n;
  std::fwrite(&len, 4, 1, g_out); std::fwrite(name, 1, len, g_out);
  std::fwrite(&kind, 4, 1, g_out); std::fwrite(&cnt, 8, 1, g_out);
  std::fwrite(d, 8, n, g_out);
}
template <typename V> static void putv(const char* name, const V& v) { put(name, v.data(), v.size()); }

// dense row-major copy of (row, col, value) entries
static std::vector<double> dense(const std::vector<std::tuple<int, int, double>>& e, size_t n) {
  std::vector<double> a(n * n, 0.0);
  for (const auto& t : e) a[(size_t)std::get<0>(t) * n + std::get<1>(t)] += std::get<2>(t);
  return a;
}

struct probe : stokes_2d<Mesh> {
  using stokes_2d<Mesh>::stokes_2d;

  void run(double t_prev, double t, double dt, const std::vector<double>* u, const std::vector<double>* p) {
    const size_t n = m_u_tilde_x.size();
    const int Np = reference_element().num_nodes(this->m_order);
    // node positions [cell][node] and boundary nodes, as the reference maps them
    {
      std::vector<std::pair<double, double>> pos;
      reference_element().node_positions(this->m_order, std::back_inserter(pos));
      std::vector<double> x, y, bx, by;
      for (int c = 0; c < this->m_mesh->num_cells(); ++c) {
        const auto cell = this->m_mesh->get_cell(c);
        for (int j = 0; j < Np; ++j) {
          const auto q = mapping::rs_to_xy(cell, dgc::point_2d<double>(pos[j].first, pos[j].second));
          x.push_back(q.x());
          y.push_back(q.y());
        }
      }
      this->fill_boundary_nodes(std::back_inserter(bx), std::back_inserter(by));
      putv("x", x);
      putv("y", y);
      putv("bx", bx);
      putv("by", by);
    }
    // stage 1 (advance_timestep)
    for (size_t i = 0; i < n; ++i) {
      m_u_tilde_x[i] = (u[2][i] * 4. - u[0][i]) / 3.;
      m_u_tilde_y[i] = (u[3][i] * 4. - u[1][i]) / 3.;
    }
    putv("ut_x", m_u_tilde_x);
    putv("ut_y", m_u_tilde_y);
    // pressure_step, up to solve_sys
    pressure_bc bc(t + dt, this->m_order, this->Inv_Jacobians.data(), this->m_mesh, this->F0_Nodes.data(),
                   this->F1_Nodes.data(), this->F2_Nodes.data(), u[2].data(), u[3].data(), u[0].data(),
                   u[1].data());
    putv("hp", bc.m_hps);
    std::vector<double> temp(n);
    auto aN = build_poisson_sys_matrix(temp, bc);
    putv("A_N", dense(aN, n));
    std::copy(m_u_tilde_x.begin(), m_u_tilde_x.end(), m_workspace.begin());
    m_div_2d(m_workspace.begin(), m_u_tilde_y.begin(), u_tilde_bc(t, t_prev));
    for (std::size_t i = 0; i < m_workspace.size(); ++i) m_workspace[i] *= 1.5 / dt;
    putv("div_ut", m_workspace);
    std::vector<double> hp2;
    for (std::size_t i = 0; i < bc.m_hps.size(); ++i) hp2.push_back(bc.exterior_grad_n(0.0, 0.0, 0.0));
    putv("hp2", hp2);  // exterior_grad_n(x, y, 0) = 2 hp, in the order apply_inhomogeneous_as_rhs asks
    m_laplace_2d.apply_inhomogeneous_as_rhs(m_workspace.begin(), bc);
    putv("p_rhs", m_workspace);
    // mass matrix and Jacobians
    auto v = reference_element().vandermonde_matrix(this->m_order);
    auto M = (v * v.transpose()).inverse();
    std::vector<double> mm((size_t)Np * Np);
    for (int i = 0; i < Np; ++i)
      for (int j = 0; j < Np; ++j) mm[(size_t)i * Np + j] = M(i, j);
    putv("M", mm);
    std::vector<double> invj, J, fj;
    this->fill_cell_mappings(std::back_inserter(invj), std::back_inserter(J), std::back_inserter(fj));
    putv("J", J);
    if (!p) return;
    // projection_step
    std::copy(p->begin(), p->end(), m_p.begin());
    m_grad_2d(m_p.begin(), m_workspace.begin(), pressure_bc_proj());
    putv("grad_p_x", m_p);
    putv("grad_p_y", m_workspace);
    for (std::size_t i = 0; i < m_u_tilde_x.size(); ++i) {
      m_u_tilde_x[i] -= 2. * dt * m_p[i] / 3.;
      m_u_tilde_y[i] -= 2. * dt * m_workspace[i] / 3.;
    }
    putv("utp_x", m_u_tilde_x);
    putv("utp_y", m_u_tilde_y);
    // viscous_step, up to solve_sys
    auto aH = build_helmholtz_sys_matrix(dt, m_workspace, u_x_bc(t + dt));
    putv("H", dense(aH, n));
    for (std::size_t i = 0; i < m_u_tilde_x.size(); ++i) m_workspace[i] = -1.5 * m_u_tilde_x[i] / dt;
    m_laplace_2d.apply_inhomogeneous_as_rhs(m_workspace.begin(), u_x_bc(t + dt));
    putv("v_rhs_x", m_workspace);
    for (std::size_t i = 0; i < m_u_tilde_y.size(); ++i) m_workspace[i] = -1.5 * m_u_tilde_y[i] / dt;
    m_laplace_2d.apply_inhomogeneous_as_rhs(m_workspace.begin(), u_y_bc(t + dt));
    putv("v_rhs_y", m_workspace);
  }
};

int main(int argc, char** argv) {
  if (argc < 5) { std::fprintf(stderr, "usage: ref_stokes mesh.bin order state.bin out.bin\n"); return 2; }
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
  auto mesh = std::make_unique<Mesh>();
  mesh->fill_vertices(xy.begin(), xy.end());
  mesh->fill_connectivity(cells.begin(), cells.end());
  mesh->build_topology();
  const int N = std::atoi(argv[2]);
  const size_t n = (size_t)K * ((N + 1) * (N + 2) / 2);

  f = std::fopen(argv[3], "rb");
  if (!f) return 3;
  double tp[3];
  int32_t has_p = 0;
  if (std::fread(tp, 8, 3, f) != 3 || std::fread(&has_p, 4, 1, f) != 1) return 3;
  std::vector<double> u[4], p;
  for (auto& a : u) {
    a.resize(n);
    if (std::fread(a.data(), 8, n, f) != n) return 3;
  }
  if (has_p) {
    p.resize(n);
    if (std::fread(p.data(), 8, n, f) != n) return 3;
  }
  std::fclose(f);

  g_out = std::fopen(argv[4], "wb");
  if (!g_out) return 4;
  probe op(*mesh, N);
  op.run(tp[0], tp[1], tp[2], u, has_p ? &p : nullptr);
  std::fclose(g_out);
  return 0;
}
