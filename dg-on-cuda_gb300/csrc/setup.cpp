// setup.cpp -- host-side set-up of the nodal DG discretisation (see setup.hpp).
#include "setup.hpp"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <numeric>

namespace dgc {

// ---------------------------------------------------------------- polynomials
// Orthonormal Jacobi polynomials by the three-term recurrence (Hesthaven &
// Warburton, "Nodal Discontinuous Galerkin Methods", 2008, App. A, JacobiP).
// Same function as src/jacobi_polynomial.h:45-73.
double jacobi(double a, double b, int n, double x) {
  const double g0 = std::pow(2.0, a + b + 1.0) / (a + b + 1.0) * std::tgamma(a + 1.0) *
                    std::tgamma(b + 1.0) / std::tgamma(a + b + 1.0);
  double pm1 = 1.0 / std::sqrt(g0);
  if (n == 0) return pm1;
  const double g1 = (a + 1.0) * (b + 1.0) / (a + b + 3.0) * g0;
  double p = ((a + b + 2.0) * x / 2.0 + (a - b) / 2.0) / std::sqrt(g1);
  if (n == 1) return p;
  double aold = 2.0 / (2.0 + a + b) * std::sqrt((a + 1.0) * (b + 1.0) / (a + b + 3.0));
  for (int i = 1; i < n; ++i) {
    const double h1 = 2.0 * i + a + b;
    const double anew = 2.0 / (h1 + 2.0) *
                        std::sqrt((i + 1.0) * (i + 1.0 + a + b) * (i + 1.0 + a) * (i + 1.0 + b) /
                                  (h1 + 1.0) / (h1 + 3.0));
    const double bnew = -(a * a - b * b) / h1 / (h1 + 2.0);
    const double pn = (-aold * pm1 + (x - bnew) * p) / anew;
    pm1 = p;
    p = pn;
    aold = anew;
  }
  return p;
}

double jacobi_grad(double a, double b, int n, double x) {
  if (n == 0) return 0.0;
  return std::sqrt(n * (n + a + b + 1.0)) * jacobi(a + 1.0, b + 1.0, n - 1, x);
}

// Legendre-Gauss-Lobatto points: Newton iteration on (1-x^2) P_N'(x) through
// x P_N - P_{N-1}, started from Chebyshev-Gauss-Lobatto points.
std::vector<double> gauss_lobatto(int npts) {
  const int N = npts - 1;
  std::vector<double> x(npts);
  if (N == 1) return {-1.0, 1.0};
  for (int i = 0; i <= N; ++i) x[i] = -std::cos(M_PI * i / N);
  for (int i = 1; i < N; ++i) {
    double xi = x[i];
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = xi;
      for (int k = 2; k <= N; ++k) {
        const double p2 = ((2.0 * k - 1.0) * xi * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      const double dx = (xi * p1 - p0) / ((N + 1.0) * p1);
      xi -= dx;
      if (std::fabs(dx) < 1e-17) break;
    }
    x[i] = xi;
  }
  // exact symmetry
  for (int i = 0; i < npts / 2; ++i) {
    const double m = 0.5 * (x[N - i] - x[i]);
    x[i] = -m;
    x[N - i] = m;
  }
  if (npts % 2) x[N / 2] = 0.0;
  x[0] = -1.0;
  x[N] = 1.0;
  return x;
}

// ---------------------------------------------------------------- dense helpers
std::vector<double> matmul(const std::vector<double>& A, const std::vector<double>& B, int m, int k, int n) {
  std::vector<double> C((size_t)m * n, 0.0);
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < n; ++j) {
      double acc = 0.0;
      for (int l = 0; l < k; ++l) acc += A[(size_t)i * k + l] * B[(size_t)l * n + j];
      C[(size_t)i * n + j] = acc;
    }
  return C;
}

std::vector<double> transpose(const std::vector<double>& A, int m, int n) {
  std::vector<double> T((size_t)m * n);
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < n; ++j) T[(size_t)j * m + i] = A[(size_t)i * n + j];
  return T;
}

// LU factorisation with partial pivoting, then n triangular solves.
bool invert(const std::vector<double>& A, int n, std::vector<double>& inv) {
  std::vector<double> lu(A);
  std::vector<int> piv(n);
  for (int c = 0; c < n; ++c) {
    int p = c;
    for (int r = c + 1; r < n; ++r)
      if (std::fabs(lu[(size_t)r * n + c]) > std::fabs(lu[(size_t)p * n + c])) p = r;
    piv[c] = p;
    if (lu[(size_t)p * n + c] == 0.0) return false;
    if (p != c)
      for (int j = 0; j < n; ++j) std::swap(lu[(size_t)p * n + j], lu[(size_t)c * n + j]);
    for (int r = c + 1; r < n; ++r) {
      const double f = lu[(size_t)r * n + c] / lu[(size_t)c * n + c];
      lu[(size_t)r * n + c] = f;
      for (int j = c + 1; j < n; ++j) lu[(size_t)r * n + j] -= f * lu[(size_t)c * n + j];
    }
  }
  inv.assign((size_t)n * n, 0.0);
  std::vector<double> col(n);
  for (int j = 0; j < n; ++j) {
    std::fill(col.begin(), col.end(), 0.0);
    col[j] = 1.0;
    for (int c = 0; c < n; ++c) std::swap(col[c], col[piv[c]]);
    for (int r = 0; r < n; ++r)
      for (int c = 0; c < r; ++c) col[r] -= lu[(size_t)r * n + c] * col[c];
    for (int r = n - 1; r >= 0; --r) {
      for (int c = r + 1; c < n; ++c) col[r] -= lu[(size_t)r * n + c] * col[c];
      col[r] /= lu[(size_t)r * n + r];
    }
    for (int r = 0; r < n; ++r) inv[(size_t)r * n + j] = col[r];
  }
  return true;
}

// ---------------------------------------------------------------- nodes
// Warburton's warp & blend construction with the alpha-optimised blending
// parameters (Hesthaven & Warburton 2008, Sec. 6.1, Nodes2D / Warpfactor);
// the reference implements the same construction in
// src/alpha_optimized_nodes_triangle.h:104-189.
namespace {
const double kAlphaOpt[15] = {0.0, 0.0, 1.4152, 0.1001, 0.2751, 0.9808, 1.0999, 1.2832,
                              1.3648, 1.4773, 1.4959, 1.5743, 1.5770, 1.6223, 1.6258};

struct Warp {
  int N;
  std::vector<double> interp;  // inverse transpose Vandermonde on equidistant nodes
  std::vector<double> shift;   // LGL - equidistant
  explicit Warp(int n) : N(n) {
    std::vector<double> eq(N + 1), vt((size_t)(N + 1) * (N + 1));
    for (int i = 0; i <= N; ++i) eq[i] = (i == 0) ? -1.0 : (i == N ? 1.0 : 2.0 * i / N - 1.0);
    for (int row = 0; row <= N; ++row)
      for (int col = 0; col <= N; ++col) vt[(size_t)row * (N + 1) + col] = jacobi(0.0, 0.0, row, eq[col]);
    invert(vt, N + 1, interp);
    const std::vector<double> gl = gauss_lobatto(N + 1);
    shift.resize(N + 1);
    for (int i = 0; i <= N; ++i) shift[i] = gl[i] - eq[i];
  }
  double operator()(double r) const {
    double w = 0.0;
    for (int i = 0; i <= N; ++i) {
      double li = 0.0;
      for (int j = 0; j <= N; ++j) li += interp[(size_t)i * (N + 1) + j] * jacobi(0.0, 0.0, j, r);
      w += li * shift[i];
    }
    return std::fabs(r) < 1.0 - 10.0 * DBL_EPSILON ? w / (1.0 - r * r) : 0.0;
  }
};
}  // namespace

void warp_blend_nodes(int N, std::vector<double>& r, std::vector<double>& s) {
  const Warp warp(N);
  const double alpha = N < 16 ? kAlphaOpt[N - 1] : 5.0 / 3.0;
  const double sq3 = std::sqrt(3.0);
  r.clear();
  s.clear();
  for (int i = 0; i <= N; ++i)
    for (int j = 0; j <= N - i; ++j) {
      const double L1 = (double)i / N, L3 = (double)j / N, L2 = 1.0 - L1 - L3;
      double X = L3 - L2, Y = (2.0 * L1 - L2 - L3) / sq3;
      const double w1 = 4.0 * L2 * L3 * (1.0 + (alpha * L1) * (alpha * L1)) * warp(L3 - L2);
      const double w2 = 4.0 * L3 * L1 * (1.0 + (alpha * L2) * (alpha * L2)) * warp(L1 - L3);
      const double w3 = 4.0 * L1 * L2 * (1.0 + (alpha * L3) * (alpha * L3)) * warp(L2 - L1);
      X += w1 - 0.5 * w2 - 0.5 * w3;
      Y += 0.5 * sq3 * (w2 - w3);
      // equilateral -> reference triangle through barycentric coordinates
      const double b1 = (1.0 + sq3 * Y) / 3.0;
      const double b2 = (2.0 - 3.0 * X - sq3 * Y) / 6.0;
      const double b3 = (2.0 + 3.0 * X - sq3 * Y) / 6.0;
      r.push_back(b3 - b2 - b1);
      s.push_back(b1 - b2 - b3);
    }
}

// ---------------------------------------------------------------- reference element
namespace {
// orthonormal Koornwinder-Dubiner mode (i, j) at (r, s) and its gradient
void mode(int i, int j, double r, double s, double& v, double& dr, double& ds) {
  const double a = (s != 1.0) ? 2.0 * (1.0 + r) / (1.0 - s) - 1.0 : -1.0, b = s;
  const double fa = jacobi(0.0, 0.0, i, a), dfa = jacobi_grad(0.0, 0.0, i, a);
  const double gb = jacobi(2.0 * i + 1.0, 0.0, j, b), dgb = jacobi_grad(2.0 * i + 1.0, 0.0, j, b);
  v = std::sqrt(2.0) * fa * gb * std::pow(1.0 - b, i);
  // H&W GradSimplex2DP, expressed with (1-b) powers
  const double hb = 0.5 * (1.0 - b);
  double dmr = dfa * gb, dms = dfa * gb * 0.5 * (1.0 + a);
  if (i > 0) {
    dmr *= std::pow(hb, i - 1);
    dms *= std::pow(hb, i - 1);
  }
  double tmp = dgb * std::pow(hb, i);
  if (i > 0) tmp -= 0.5 * i * gb * std::pow(hb, i - 1);
  dms += fa * tmp;
  const double scale = std::pow(2.0, i + 0.5);
  dr = scale * dmr;
  ds = scale * dms;
}
}  // namespace

bool build_ref_element(int N, RefElement& re, std::string& err) {
  if (N < 1 || N > kMaxOrder) {
    err = "order must be in [1, 8]";
    return false;
  }
  re.N = N;
  re.Np = num_nodes(N);
  re.Nfp = N + 1;
  const int Np = re.Np, Nfp = re.Nfp;
  warp_blend_nodes(N, re.r, re.s);
  re.V.assign((size_t)Np * Np, 0.0);
  re.Vr.assign((size_t)Np * Np, 0.0);
  re.Vs.assign((size_t)Np * Np, 0.0);
  int col = 0;
  for (int i = 0; i <= N; ++i)
    for (int j = 0; j <= N - i; ++j, ++col)
      for (int row = 0; row < Np; ++row) {
        double v, dr, ds;
        mode(i, j, re.r[row], re.s[row], v, dr, ds);
        re.V[(size_t)row * Np + col] = v;
        re.Vr[(size_t)row * Np + col] = dr;
        re.Vs[(size_t)row * Np + col] = ds;
      }
  const std::vector<double> VT = transpose(re.V, Np, Np);
  const std::vector<double> Minv = matmul(re.V, VT, Np, Np, Np);
  std::vector<double> Vinv;
  if (!invert(Minv, Np, re.M) || !invert(re.V, Np, Vinv)) {
    err = "singular Vandermonde matrix";
    return false;
  }
  // weak form: M^-1 Dr^T M = V Vr^T M  ;  strong form: Vr V^-1
  re.Drw = matmul(matmul(re.V, transpose(re.Vr, Np, Np), Np, Np, Np), re.M, Np, Np, Np);
  re.Dsw = matmul(matmul(re.V, transpose(re.Vs, Np, Np), Np, Np, Np), re.M, Np, Np, Np);
  re.Drs = matmul(re.Vr, Vinv, Np, Np, Np);
  re.Dss = matmul(re.Vs, Vinv, Np, Np, Np);
  // LIFT = M^-1 E, E = face mass matrices (1D Vandermonde on the face nodes)
  std::vector<double> E((size_t)Np * 3 * Nfp, 0.0);
  for (int f = 0; f < 3; ++f) {
    std::vector<double> fV((size_t)Nfp * Nfp), fMinv;
    for (int d = 0; d < Nfp; ++d) {
      const int nd = face_node(N, f, d);
      const double x = (f == 0) ? re.r[nd] : re.s[nd];
      for (int m = 0; m < Nfp; ++m) fV[(size_t)d * Nfp + m] = jacobi(0.0, 0.0, m, x);
    }
    std::vector<double> fM = matmul(fV, transpose(fV, Nfp, Nfp), Nfp, Nfp, Nfp);
    if (!invert(fM, Nfp, fMinv)) {
      err = "singular face mass matrix";
      return false;
    }
    for (int d = 0; d < Nfp; ++d)
      for (int m = 0; m < Nfp; ++m)
        E[(size_t)face_node(N, f, d) * 3 * Nfp + f * Nfp + m] = fMinv[(size_t)d * Nfp + m];
  }
  re.Lw = matmul(Minv, E, Np, Np, 3 * Nfp);
  re.Ls = re.Lw;
  return true;
}

// ---------------------------------------------------------------- mesh
bool build_mesh(const double* vxy, int nv, const int32_t* cells, int K, const RefElement& re,
                MeshData& m, std::string& err, bool gpu_topology) {
  char buf[256];
  if (K <= 0 || nv < 3 || !vxy || !cells) {
    err = "empty mesh";
    return false;
  }
  if ((int64_t)K >= (int64_t(1) << 29)) {
    err = "too many elements (limit 2^29)";
    return false;
  }
  m = MeshData();
  m.K = K;
  m.nv = nv;
  m.N = re.N;
  m.Np = re.Np;
  m.Nfp = re.Nfp;
  m.vx.resize(nv);
  m.vy.resize(nv);
  for (int i = 0; i < nv; ++i) {
    m.vx[i] = vxy[2 * i];
    m.vy[i] = vxy[2 * i + 1];
    if (!std::isfinite(m.vx[i]) || !std::isfinite(m.vy[i])) {
      std::snprintf(buf, sizeof buf, "vertex %d is not finite", i);
      err = buf;
      return false;
    }
  }
  m.cells.assign(cells, cells + 3 * (size_t)K);
  for (int k = 0; k < K; ++k)
    for (int v = 0; v < 3; ++v)
      if (cells[3 * k + v] < 0 || cells[3 * k + v] >= nv) {
        std::snprintf(buf, sizeof buf, "cell %d references vertex %d out of range", k, cells[3 * k + v]);
        err = buf;
        return false;
      }

  // geometry
  m.geom.assign((size_t)K * kGeomStride, 0.0);
  m.min_edge = 1e300;
  m.min_altitude = 1e300;
  for (int k = 0; k < K; ++k) {
    const int32_t* c = &cells[3 * k];
    const double x0 = m.vx[c[0]], y0 = m.vy[c[0]], x1 = m.vx[c[1]], y1 = m.vy[c[1]];
    const double x2 = m.vx[c[2]], y2 = m.vy[c[2]];
    const double xr = 0.5 * (x1 - x0), xs = 0.5 * (x2 - x0), yr = 0.5 * (y1 - y0), ys = 0.5 * (y2 - y0);
    const double J = 0.25 * ((x1 - x0) * (y2 - y0) - (x2 - x0) * (y1 - y0));
    if (!(J > 0.0)) {
      std::snprintf(buf, sizeof buf, "cell %d is degenerate or clockwise (J = %g)", k, J);
      err = buf;
      return false;
    }
    double* g = &m.geom[(size_t)k * kGeomStride];
    g[G_RX] = ys / J;
    g[G_RY] = -xs / J;
    g[G_SX] = -yr / J;
    g[G_SY] = xr / J;
    g[G_J] = J;
    for (int f = 0; f < 3; ++f) {
      const int a = c[f], b = c[(f + 1) % 3];
      const double dx = m.vx[b] - m.vx[a], dy = m.vy[b] - m.vy[a];
      const double len = std::sqrt(dy * dy + dx * dx);
      g[G_FJ0 + f] = 0.5 * len;
      g[G_NX0 + f] = dy / len;   // counter-clockwise cell: outward normal is (dy, -dx)/|e|
      g[G_NY0 + f] = -dx / len;
      m.min_edge = std::min(m.min_edge, len);
      m.min_altitude = std::min(m.min_altitude, 4.0 * J / len);
    }
  }

  for (int k = 0; k < K; ++k)
    for (int f = 0; f < 3; ++f)
      if (cells[3 * k + f] == cells[3 * k + (f + 1) % 3]) {
        std::snprintf(buf, sizeof buf, "cell %d has a repeated vertex", k);
        err = buf;
        return false;
      }
  m.nbr.assign((size_t)4 * K, 0);
  std::vector<int8_t> is_bnd((size_t)3 * K, 1);
  if (gpu_topology) {
    std::vector<int32_t> twin;
    if (!gpu_match_half_edges(cells, K, twin, err)) return false;
    for (size_t h = 0; h < twin.size(); ++h)
      if (twin[h] >= 0) {
        m.nbr[4 * (h / 3) + h % 3] = twin[h];
        is_bnd[h] = 0;
      }
  }
  // topology: sort half-edges by their unordered vertex pair; equal keys are twins
  struct HE { uint64_t key; int32_t k, f; };
  std::vector<HE> he(gpu_topology ? 0 : (size_t)3 * K);
  for (size_t i = 0; i < he.size(); ++i) {
    const int k = (int)(i / 3), f = (int)(i % 3);
    const uint32_t a = (uint32_t)cells[3 * k + f], b = (uint32_t)cells[3 * k + (f + 1) % 3];
    he[i] = HE{(uint64_t)std::min(a, b) << 32 | std::max(a, b), k, f};
  }
  std::sort(he.begin(), he.end(), [](const HE& x, const HE& y) {
    return x.key != y.key ? x.key < y.key : (x.k != y.k ? x.k < y.k : x.f < y.f);
  });
  for (size_t i = 0; i < he.size();) {
    size_t j = i + 1;
    while (j < he.size() && he[j].key == he[i].key) ++j;
    if (j - i > 2) {
      std::snprintf(buf, sizeof buf, "non-manifold edge shared by %d cells (cell %d)", (int)(j - i), he[i].k);
      err = buf;
      return false;
    }
    if (j - i == 2) {
      const HE &p = he[i], &q = he[i + 1];
      // a conforming, consistently oriented mesh traverses a shared edge in
      // opposite directions from its two sides
      if (cells[3 * p.k + p.f] == cells[3 * q.k + q.f]) {
        std::snprintf(buf, sizeof buf, "cells %d and %d are inconsistently oriented", p.k, q.k);
        err = buf;
        return false;
      }
      m.nbr[(size_t)4 * p.k + p.f] = (q.k << 2) | q.f;
      m.nbr[(size_t)4 * q.k + q.f] = (p.k << 2) | p.f;
      is_bnd[(size_t)3 * p.k + p.f] = 0;
      is_bnd[(size_t)3 * q.k + q.f] = 0;
    }
    i = j;
  }
  // boundary faces in element-then-face order, with the coordinates of their nodes
  const int Nfp = re.Nfp;
  for (int k = 0; k < K; ++k)
    for (int f = 0; f < 3; ++f)
      if (is_bnd[(size_t)3 * k + f]) {
        const int b = m.num_bfaces++;
        m.nbr[(size_t)4 * k + f] = -(1 + b);
        const int32_t* c = &cells[3 * k];
        for (int d = 0; d < Nfp; ++d) {
          const int nd = face_node(re.N, f, d);
          const double r = re.r[nd], s = re.s[nd];
          const double l1 = 0.5 * (s + 1.0), l2 = -0.5 * (r + s), l3 = 0.5 * (r + 1.0);
          m.bxy.push_back(l2 * m.vx[c[0]] + l3 * m.vx[c[1]] + l1 * m.vx[c[2]]);
          m.bxy.push_back(l2 * m.vy[c[0]] + l3 * m.vy[c[1]] + l1 * m.vy[c[2]]);
        }
      }
  fill_penalty(m, re);
  return true;
}

void fill_penalty(MeshData& m, const RefElement& re) {
  // laplace penalty tau_f = (N+1)^2 / h_f, h_f = smaller altitude onto the face
  const int K = m.K;
  m.tau.assign((size_t)4 * K, 0.0);
  const double n1 = (re.N + 1.0) * (re.N + 1.0);
  for (int k = 0; k < K; ++k)
    for (int f = 0; f < 3; ++f) {
      const double* g = &m.geom[(size_t)k * kGeomStride];
      double h = 2.0 * g[G_J] / g[G_FJ0 + f];
      const int32_t nb = m.nbr[(size_t)4 * k + f];
      if (nb >= 0) {
        const double* gn = &m.geom[(size_t)(nb >> 2) * kGeomStride];
        h = std::min(h, 2.0 * gn[G_J] / gn[G_FJ0 + (nb & 3)]);
      }
      m.tau[(size_t)4 * k + f] = n1 / h;
    }
}

bool build_mesh_from_arrays(int K, const RefElement& re, const double* invJ, const double* J, const double* faceJ,
                            const int32_t* nb_cell, const int32_t* nb_face, int num_boundary_nodes, const double* bx,
                            const double* by, const double* nx, const double* ny, MeshData& m, std::string& err) {
  char buf[200];
  auto bad = [&](const char* fmt, long a, long b) {
    std::snprintf(buf, sizeof buf, fmt, a, b);
    err = buf;
    return false;
  };
  if (K <= 0 || K >= (1 << 29)) return bad("cell count %ld outside [1, 2^29) (%ld)", K, 0);
  const int Nfp = re.Nfp;
  m = MeshData();
  m.K = K;
  m.N = re.N;
  m.Np = re.Np;
  m.Nfp = Nfp;
  m.geom.assign((size_t)K * kGeomStride, 0.0);
  m.nbr.assign((size_t)4 * K, 0);
  m.min_edge = 1e300;
  m.min_altitude = 1e300;
  int offset = 0;
  for (int k = 0; k < K; ++k) {
    double* g = &m.geom[(size_t)k * kGeomStride];
    for (int i = 0; i < 4; ++i) g[G_RX + i] = invJ[4 * (size_t)k + i];
    g[G_J] = J[k];
    if (!(J[k] > 0.0)) return bad("cell %ld: J is not positive (%ld)", k, 0);
    for (int f = 0; f < 3; ++f) {
      const size_t i = 3 * (size_t)k + f;
      g[G_FJ0 + f] = faceJ[i];
      g[G_NX0 + f] = nx[i];
      g[G_NY0 + f] = ny[i];
      if (!(faceJ[i] > 0.0)) return bad("cell %ld face %ld: faceJ is not positive", k, f);
      const double len = 2.0 * faceJ[i];
      m.min_edge = std::min(m.min_edge, len);
      m.min_altitude = std::min(m.min_altitude, 4.0 * J[k] / len);
      const int32_t c = nb_cell[i], e = nb_face[i];
      if (c < 0 || c >= K) return bad("cell %ld: neighbour cell %ld out of range", k, c);
      if (c == k) {
        // boundary face: nb_face is the running offset into the boundary nodes
        if (e != offset) return bad("cell %ld: boundary node offset %ld out of sequence", k, e);
        m.nbr[4 * (size_t)k + f] = -(1 + m.num_bfaces);
        ++m.num_bfaces;
        offset += Nfp;
      } else {
        if (e < 0 || e > 2) return bad("cell %ld: neighbour face %ld out of range", k, e);
        const size_t j = 3 * (size_t)c + e;
        if (nb_cell[j] != k || nb_face[j] != f) return bad("cells %ld and %ld: interface map not symmetric", k, c);
        m.nbr[4 * (size_t)k + f] = (c << 2) | e;
      }
    }
  }
  if (offset != num_boundary_nodes)
    return bad("boundary node count %ld does not match the interfaces (%ld)", num_boundary_nodes, offset);
  m.bxy.resize((size_t)2 * offset);
  for (int b = 0; b < offset; ++b) {
    m.bxy[2 * (size_t)b] = bx[b];
    m.bxy[2 * (size_t)b + 1] = by[b];
  }
  fill_penalty(m, re);
  return true;
}

}  // namespace dgc
