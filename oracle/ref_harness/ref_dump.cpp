// ref_dump.cpp -- drives the reference's own USE_CPU_ONLY classes on one mesh and
// one order and writes their outputs as named arrays.  Built only by
// oracle/Makefile against the reference sources; its outputs become the golden
// vectors under tests/golden/ that pin the oracle restatement.
//
// usage: ref_dump (--msh file.msh | --bin mesh.bin) order out.bin [export.msh]
//   mesh.bin: int32 nv, f64 xy[2 nv], int32 K, int32 cells[3 K]
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <sstream>
#include <string>
#include <vector>

#include <thrust/host_vector.h>
#include <thrust/iterator/zip_iterator.h>

#include "simple_triangular_mesh_2d.h"
#include "gmsh_importer_exporter.h"
#include "reference_triangle.h"
#include "advection_2d.h"
#include "maxwell_2d.h"
#include "poisson_2d.h"
#include "axpy.h"
#include "explicit_runge_kutta.h"
#include "grad_2d.h"
#include "div_2d.h"

using Mesh = dgc::simple_triangular_mesh_2d<double, int>;

static FILE* g_out = nullptr;

static void put(const char* name, const double* d, size_t n) {
  int32_t len = (int32_t)std::strlen(name), kind = 0;
  int64_t cnt = (int64_t)n;
  std::fwrite(&len, 4, 1, g_out); std::fwrite(name, 1, len, g_out);
  std::fwrite(&kind, 4, 1, g_out); std::fwrite(&cnt, 8, 1, g_out);
  std::fwrite(d, 8, n, g_out);
}
static void puti(const char* name, const int* d, size_t n) {
  int32_t len = (int32_t)std::strlen(name), kind = 1;
  int64_t cnt = (int64_t)n;
  std::fwrite(&len, 4, 1, g_out); std::fwrite(name, 1, len, g_out);
  std::fwrite(&kind, 4, 1, g_out); std::fwrite(&cnt, 8, 1, g_out);
  std::fwrite(d, 4, n, g_out);
}
template <typename V> static void putv(const char* name, const V& v) { put(name, v.data(), v.size()); }

struct dirichlet_all {
  bool is_dirichlet(double, double) const { return true; }
  double exterior_val(double, double, double v) const { return -v; }
  double exterior_grad_n(double, double, double g) const { return g; }
};

// laplace_2d boundary object with both condition types and nonzero data
struct mixed_bc {
  bool is_dirichlet(double x, double y) const { return x + 0.3 * y < 0.2; }
  double exterior_val(double x, double y, double v) const { return 2.0 * std::sin(x + y) - v; }
  double exterior_grad_n(double x, double y, double gn) const { return 2.0 * std::cos(x * y) - gn; }
};

// boundary objects of the form u+ = g(x, y) + sign u- for grad_2d / div_2d
struct scalar_bc {
  double sign;
  double exterior_val(double x, double y, double v) const {
    return (sign < 0.0 ? 2.0 * std::sin(x) * std::cos(y) : 0.0) + sign * v;
  }
};
struct vector_bc {
  double exterior_val_x(double x, double y) const { return 2.0 * std::sin(x) * std::cos(y); }
  double exterior_val_y(double x, double y) const { return 2.0 * x * y; }
  std::pair<double, double> exterior_val(double x, double y, std::pair<double, double> v) const {
    return std::make_pair(exterior_val_x(x, y) - v.first, exterior_val_y(x, y) - v.second);
  }
};

int main(int argc, char** argv) {
  if (argc < 5) { std::fprintf(stderr, "usage: ref_dump --msh|--bin file order out\n"); return 2; }
  std::unique_ptr<Mesh> mesh;
  if (std::string(argv[1]) == "--msh") {
    mesh = dgc::gmsh_importer_exporter<double, int>::import_triangle_mesh_2d(argv[2]);
  } else {
    FILE* f = std::fopen(argv[2], "rb");
    if (!f) return 3;
    int32_t nv, K;
    if (std::fread(&nv, 4, 1, f) != 1) return 3;
    std::vector<double> xy(2 * (size_t)nv);
    if (std::fread(xy.data(), 8, xy.size(), f) != xy.size()) return 3;
    if (std::fread(&K, 4, 1, f) != 1) return 3;
    std::vector<int> cells(3 * (size_t)K);
    if (std::fread(cells.data(), 4, cells.size(), f) != cells.size()) return 3;
    std::fclose(f);
    mesh = std::make_unique<Mesh>();
    mesh->fill_vertices(xy.begin(), xy.end());
    mesh->fill_connectivity(cells.begin(), cells.end());
  }
  mesh->build_topology();
  const int N = std::atoi(argv[3]);
  g_out = std::fopen(argv[4], "wb");
  if (!g_out) return 4;

  const int K = mesh->num_cells();
  {
    std::vector<double> xy;
    for (int v = 0; v < mesh->num_vertices(); ++v) {
      auto p = mesh->get_vertex(v);
      xy.push_back(p.x()); xy.push_back(p.y());
    }
    putv("mesh_xy", xy);
    std::vector<int> cells, twin(3 * (size_t)K);
    for (int c = 0; c < K; ++c) {
      auto t = mesh->get_cell_connectivity(c);
      cells.push_back(std::get<0>(t)); cells.push_back(std::get<1>(t)); cells.push_back(std::get<2>(t));
    }
    puti("mesh_cells", cells.data(), cells.size());
    mesh->get_face_mapping(twin.begin());
    puti("twin_hf", twin.data(), twin.size());
  }

  // reference element
  dgc::reference_triangle<double> rt;
  std::vector<std::pair<double, double>> pos;
  rt.node_positions(N, std::back_inserter(pos));
  std::vector<double> r, s;
  for (auto& p : pos) { r.push_back(p.first); s.push_back(p.second); }
  putv("r", r); putv("s", s);
  auto V = rt.vandermonde_matrix(N);
  put("V", V.data(), V.size_row() * V.size_col());
  auto G = rt.grad_vandermonde_matrix(N);
  put("Vr", G.first.data(), G.first.size_row() * G.first.size_col());
  put("Vs", G.second.data(), G.second.size_row() * G.second.size_col());

  // advection (weak-form operators + discretisation arrays)
  advection_2d<double, Mesh> adv(*mesh, N);
  puti("F0", adv.F0_Nodes.data(), adv.F0_Nodes.size());
  puti("F1", adv.F1_Nodes.data(), adv.F1_Nodes.size());
  puti("F2", adv.F2_Nodes.data(), adv.F2_Nodes.size());
  put("Drw", adv.m_Dr.data(), adv.m_Dr.size_row() * adv.m_Dr.size_col());
  put("Dsw", adv.m_Ds.data(), adv.m_Ds.size_row() * adv.m_Ds.size_col());
  put("Lw", adv.m_L.data(), adv.m_L.size_row() * adv.m_L.size_col());
  {
    std::vector<double> invJ, J, fJ, bx, by, nx, ny;
    std::vector<int> ic, ifc;
    adv.fill_cell_mappings(std::back_inserter(invJ), std::back_inserter(J), std::back_inserter(fJ));
    adv.fill_cell_interfaces(std::back_inserter(ic), std::back_inserter(ifc));
    adv.fill_boundary_nodes(std::back_inserter(bx), std::back_inserter(by));
    adv.fill_outward_normals(std::back_inserter(nx), std::back_inserter(ny));
    putv("invJ", invJ); putv("J", J); putv("faceJ", fJ);
    puti("nbCell", ic.data(), ic.size()); puti("nbFace", ifc.data(), ifc.size());
    putv("bx", bx); putv("by", by); putv("nx", nx); putv("ny", ny);
  }
  const int n = adv.total_num_nodes();
  // time step of the reference drivers (examples/advection_2d/main.cpp:137-138)
  const double l = 2.0 / std::sqrt((double)K);
  const double dt = (2.0 / 3.0) * (l / (double)N) * (l / (2.0 + std::sqrt(2.0)));
  put("dt", &dt, 1);
  {
    std::vector<dgc::point_2d<double>> x(n);
    std::vector<double> u(n), out(n, 0.0), w[5];
    for (auto& a : w) a.assign(n, 0.0);
    adv.initialize_dofs(x.begin(), u.begin());
    putv("adv_u0", u);
    adv(u.cbegin(), (std::size_t)n, 0.05, out.begin());
    putv("adv_rhs", out);
    double t = 0.0;
    for (int i = 0; i < 10; ++i) {
      dgc::rk4(u.data(), (std::size_t)n, t, dt, adv, &dgc::axpy_n<double, const double*, double*>,
               w[0].data(), w[1].data(), w[2].data(), w[3].data(), w[4].data());
      t += dt;
      if (i == 0) putv("adv_rk4_1", u);
    }
    putv("adv_rk4_10", u);
    // the visualisation file of the advection driver, written by the same
    // stream statements (examples/advection_2d/main.cpp:164-174) into memory
    std::vector<double> ref_v(n), px(n), py(n);
    adv.exact_solution(t, ref_v.begin());
    for (int i = 0; i < n; ++i) { px[i] = x[i].x(); py[i] = x[i].y(); }
    putv("adv_x", px); putv("adv_y", py); putv("adv_exact_10", ref_v);
    std::ostringstream file;
    file.precision(std::numeric_limits<double>::digits10);
    file << "#         x         y         u" << std::endl;
    for (int i = 0; i < n; ++i)
      file << x[i].x() << "  " << x[i].y() << "  " << u[i] << std::endl;
    file << std::endl;
    file << "#         x         y         reference solution" << std::endl;
    for (int i = 0; i < n; ++i)
      file << x[i].x() << "  " << x[i].y() << "  " << ref_v[i] << std::endl;
    const std::string text = file.str();
    std::vector<int> bytes(text.begin(), text.end());
    puti("adv_datafile", bytes.data(), bytes.size());
  }

  // Maxwell TM cavity
  {
    maxwell_2d<double, Mesh> mx(*mesh, N);
    using HV = thrust::host_vector<double>;
    using HZ = thrust::zip_iterator<thrust::tuple<HV::iterator, HV::iterator, HV::iterator>>;
    HV f[6][3];
    for (auto& a : f) for (auto& b : a) b.assign(n, 0.0);
    auto zip = [&](int i) { return thrust::make_zip_iterator(thrust::make_tuple(f[i][0].begin(), f[i][1].begin(), f[i][2].begin())); };
    std::vector<dgc::point_2d<double>> x(n);
    mx.initialize_dofs(x.begin(), zip(0));
    auto dump3 = [&](const char* name, int i) {
      std::vector<double> v;
      for (int c = 0; c < 3; ++c) v.insert(v.end(), f[i][c].begin(), f[i][c].end());
      putv(name, v);
    };
    dump3("mx_q0", 0);
    mx(zip(0), (std::size_t)n, 0.0, zip(1));
    dump3("mx_rhs", 1);
    double t = 0.0;
    for (int i = 0; i < 10; ++i) {
      dgc::rk4(zip(0), (std::size_t)n, t, dt, mx, &dgc::axpy_n<double, HZ, HZ>, zip(1), zip(2), zip(3), zip(4), zip(5));
      t += dt;
      if (i == 0) dump3("mx_rk4_1", 0);
    }
    dump3("mx_rk4_10", 0);
  }

  // laplace_2d through poisson_2d (strong-form operators, homogeneous Dirichlet)
  {
    poisson_2d<double, Mesh> po(*mesh, N);
    put("Drs", po.m_Dr.data(), po.m_Dr.size_row() * po.m_Dr.size_col());
    put("Dss", po.m_Ds.data(), po.m_Ds.size_row() * po.m_Ds.size_col());
    put("Ls", po.m_L.data(), po.m_L.size_row() * po.m_L.size_col());
    std::vector<double> u(n), ex(n), f(n);
    for (int i = 0; i < n; ++i) u[i] = std::sin(1.3 * i + 0.2) + 0.1 * std::cos(0.7 * i);
    putv("lap_u", u);
    po(u.begin());
    putv("lap_out", u);
    po.exact_solution(ex.begin());
    po.rhs(f.begin());
    putv("poi_exact", ex);
    putv("poi_rhs", f);
    // laplace_2d directly, with an explicit all-Dirichlet BC object
    dgc::laplace_2d<double, Mesh> lap(*mesh, N);
    for (int i = 0; i < n; ++i) u[i] = std::sin(1.3 * i + 0.2) + 0.1 * std::cos(0.7 * i);
    lap(u.begin(), dirichlet_all());
    putv("lap2_out", u);
    // mixed condition types with boundary data: the homogeneous part, the data
    // contribution alone, and operator() (both)
    std::vector<double> lu(n);
    for (int i = 0; i < n; ++i) lu[i] = std::cos(0.8 * i + 0.5) - 0.2 * std::sin(1.9 * i);
    putv("lapm_u", lu);
    std::vector<double> a(lu);
    lap.apply_homogeneous(a.begin(), mixed_bc());
    putv("lapm_hom", a);
    std::vector<double> z(n, 0.0);
    lap.apply_inhomogeneous_as_rhs(z.begin(), mixed_bc());
    putv("lapm_rhs", z);
    std::vector<double> b(lu);
    lap(b.begin(), mixed_bc());
    putv("lapm_full", b);
  }

  // grad_2d and div_2d (weak form, central fluxes) with boundary data
  // u+ = 2 g - u- (g = sin x cos y; for div, (sin x cos y, x y)) and u+ = u-
  {
    dgc::grad_2d<double, Mesh> gr(*mesh, N);
    dgc::div_2d<double, Mesh> dv(*mesh, N);
    std::vector<double> u(n), v(n);
    for (int i = 0; i < n; ++i) {
      u[i] = std::sin(0.9 * i + 0.4) + 0.2 * std::cos(1.7 * i);
      v[i] = std::cos(0.6 * i + 0.1) - 0.3 * std::sin(2.3 * i);
    }
    putv("gd_u", u);
    putv("gd_v", v);
    for (double sign : {-1.0, 1.0}) {
      std::vector<double> gx(u), gy(n);
      gr(gx.begin(), gy.begin(), scalar_bc{sign});
      putv(sign < 0.0 ? "grad_dir_x" : "grad_mir_x", gx);
      putv(sign < 0.0 ? "grad_dir_y" : "grad_mir_y", gy);
    }
    std::vector<double> d(u), w(v);
    dv(d.begin(), w.begin(), vector_bc());
    putv("div_dir", d);
  }
  std::fclose(g_out);
  // optional: the mesh written back by the reference's MSH exporter
  if (argc > 5) dgc::gmsh_importer_exporter<double, int>::export_triangle_mesh_2d(*mesh, argv[5]);
  return 0;
}
