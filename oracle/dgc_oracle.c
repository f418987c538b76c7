/*
 * dgc_oracle.c -- CPU restatement of hsongxa/dg-on-cuda's nodal-DG hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker, never the product): see dgc_oracle.h.
 * Each routine cites the reference file:line it restates.  Operation order
 * follows the reference so that results agree with its USE_CPU_ONLY build to
 * rounding; tests/golden/ pins this against the reference's own outputs.
 */
#include "dgc_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ------------------------------------------------------------------------- */
/* dense row-major helpers: src/dense_matrix.h                                */
/* ------------------------------------------------------------------------- */

/* C = A(m x k) * B(k x n); each entry is std::inner_product of a row of A and a
 * row of B^T accumulated from 0 in ascending order (dense_matrix.h:394-416). */
static void mat_mul(int m, int k, int n, const double* A, const double* B, double* C) {
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < n; ++j) {
      double acc = 0.0;
      for (int l = 0; l < k; ++l) acc = acc + A[i * k + l] * B[l * n + j];
      C[i * n + j] = acc;
    }
}

static void mat_transpose(int m, int n, const double* A, double* T) {
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < n; ++j) T[j * m + i] = A[i * n + j];
}

/* Gauss-Jordan inverse with partial pivoting (dense_matrix.h:505-566). */
int orc_mat_inverse(int n, const double* A, double* inv) {
  if (n == 1) {
    if (A[0] == 0.0) return -1;
    inv[0] = 1.0 / A[0];
    return 0;
  }
  double* tmp = (double*)malloc(sizeof(double) * n * n);
  memcpy(tmp, A, sizeof(double) * n * n);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) inv[i * n + j] = (i == j) ? 1.0 : 0.0;
  for (int i = 0; i < n; ++i) {
    int pivot = i;
    for (int ii = i + 1; ii < n; ++ii)
      if (fabs(tmp[pivot * n + i]) < fabs(tmp[ii * n + i])) pivot = ii;
    if (pivot != i)
      for (int j = 0; j < n; ++j) {
        double t = tmp[i * n + j]; tmp[i * n + j] = tmp[pivot * n + j]; tmp[pivot * n + j] = t;
        t = inv[i * n + j]; inv[i * n + j] = inv[pivot * n + j]; inv[pivot * n + j] = t;
      }
    double d = tmp[i * n + i];
    if (d == 0.0) { free(tmp); return -1; }
    for (int j = 0; j < n; ++j) { tmp[i * n + j] /= d; inv[i * n + j] /= d; }
    for (int ii = 0; ii < n; ++ii)
      if (ii != i) {
        d = tmp[ii * n + i];
        for (int j = 0; j < n; ++j) {
          tmp[ii * n + j] -= d * tmp[i * n + j];
          inv[ii * n + j] -= d * inv[i * n + j];
        }
      }
  }
  free(tmp);
  return 0;
}

/* y = beta*y + sum_j (alpha*A_ij)*x_j, row-major (dense_matrix.h:466-491). */
static void gemv(int rows, int cols, const double* A, double alpha, const double* x,
                 double beta, double* y) {
  for (int i = 0; i < rows; ++i) {
    double acc = beta * y[i];
    const double* a = A + (size_t)i * cols;
    for (int j = 0; j < cols; ++j) acc += alpha * a[j] * x[j];
    y[i] = acc;
  }
}

/* ------------------------------------------------------------------------- */
/* Jacobi polynomials: src/jacobi_polynomial.h:45-112                         */
/* ------------------------------------------------------------------------- */
double orc_jacobi_p(double alpha, double beta, int n, double x) {
  double a1 = alpha + 1.0, b1 = beta + 1.0, ab2 = alpha + beta + 2.0;
  double pp = sqrt(tgamma(ab2) / tgamma(a1) / tgamma(b1) / pow(2.0, a1 + beta));
  if (n == 0) return pp;
  double p = 0.5 * pp * sqrt((ab2 + 1.0) / a1 / b1) * (ab2 * x + alpha - beta);
  if (n == 1) return p;
  double val = 0.0;
  double a_i = 2.0 / ab2 * sqrt((a1 + beta) * a1 * b1 / (ab2 - 1.0) / (ab2 + 1.0));
  for (int ii = 1; ii < n; ++ii) {
    double i = (double)ii;
    double iab = 2.0 * i + alpha + beta;
    double b_i = (alpha + beta) * (beta - alpha) / iab / (iab + 2.0);
    double a_n = 2.0 / (iab + 2.0) *
                 sqrt((i + 1.0) * (i + a1 + beta) * (i + a1) * (i + b1) / (iab + 1.0) / (iab + 3.0));
    val = ((x - b_i) * p - a_i * pp) / a_n;
    a_i = a_n;
    pp = p;
    p = val;
  }
  return val;
}

double orc_jacobi_dp(double alpha, double beta, int n, double x) {
  if (n == 0) return 0.0;
  double val = orc_jacobi_p(alpha + 1.0, beta + 1.0, n - 1, x);
  return sqrt((double)n * ((double)n + alpha + beta + 1.0)) * val;
}

/* ------------------------------------------------------------------------- */
/* Gauss-Lobatto points: src/quadrature_rules.h:70-149 for 2..7 points.       */
/* The reference throws beyond 7 points; for 8 and 9 points (orders 7, 8) the */
/* Legendre-Gauss-Lobatto nodes are computed by the published Newton          */
/* iteration on x P_N(x) - P_{N-1}(x) from Chebyshev-Gauss-Lobatto starting   */
/* points (G. von Winckel, "lglnodes").  No reference pin exists for these.   */
/* ------------------------------------------------------------------------- */
int orc_gl_points(int npts, double* x) {
  switch (npts) {
    case 2: x[0] = -1.0; x[1] = 1.0; return 0;
    case 3: x[0] = -1.0; x[1] = 0.0; x[2] = 1.0; return 0;
    case 4:
      x[0] = -1.0; x[1] = -sqrt(1.0 / 5.0); x[2] = sqrt(1.0 / 5.0); x[3] = 1.0; return 0;
    case 5:
      x[0] = -1.0; x[1] = -sqrt(3.0 / 7.0); x[2] = 0.0; x[3] = sqrt(3.0 / 7.0); x[4] = 1.0;
      return 0;
    case 6:
      x[0] = -1.0;
      x[1] = -sqrt(1.0 / 3.0 + 2.0 * sqrt(7.0) / 21.0);
      x[2] = -sqrt(1.0 / 3.0 - 2.0 * sqrt(7.0) / 21.0);
      x[3] = sqrt(1.0 / 3.0 - 2.0 * sqrt(7.0) / 21.0);
      x[4] = sqrt(1.0 / 3.0 + 2.0 * sqrt(7.0) / 21.0);
      x[5] = 1.0;
      return 0;
    case 7:
      x[0] = -1.0;
      x[1] = -sqrt(5.0 / 11.0 + 2.0 * sqrt(5.0 / 3.0) / 11.0);
      x[2] = -sqrt(5.0 / 11.0 - 2.0 * sqrt(5.0 / 3.0) / 11.0);
      x[3] = 0.0;
      x[4] = sqrt(5.0 / 11.0 - 2.0 * sqrt(5.0 / 3.0) / 11.0);
      x[5] = sqrt(5.0 / 11.0 + 2.0 * sqrt(5.0 / 3.0) / 11.0);
      x[6] = 1.0;
      return 0;
    default: break;
  }
  if (npts < 2 || npts > ORC_MAX_ORDER + 1) return -1;
  int N = npts - 1;
  double xs[ORC_MAX_ORDER + 1], P[ORC_MAX_ORDER + 2];
  for (int i = 0; i <= N; ++i) xs[i] = cos(M_PI * (double)i / (double)N);
  for (int iter = 0; iter < 100; ++iter) {
    double maxd = 0.0;
    for (int i = 0; i <= N; ++i) {
      double xi = xs[i];
      P[0] = 1.0; P[1] = xi;
      for (int k = 2; k <= N; ++k) P[k] = ((2.0 * k - 1.0) * xi * P[k - 1] - (k - 1.0) * P[k - 2]) / k;
      double xn = xi - (xi * P[N] - P[N - 1]) / ((double)(N + 1) * P[N]);
      maxd = fmax(maxd, fabs(xn - xi));
      xs[i] = xn;
    }
    if (maxd < 1e-16) break;
  }
  for (int i = 0; i <= N; ++i) x[i] = xs[N - i]; /* ascending, -1 .. 1 */
  x[0] = -1.0; x[N] = 1.0;
  return 0;
}

/* ------------------------------------------------------------------------- */
/* Warp & blend nodes: src/alpha_optimized_nodes_triangle.h:61-189            */
/* ------------------------------------------------------------------------- */
static const double s_alpha[] = {0.0, 0.0, 1.4152, 0.1001, 0.2751, 0.9808, 1.0999, 1.2832,
                                 1.3648, 1.4773, 1.4959, 1.5743, 1.5770, 1.6223, 1.6258};

typedef struct {
  int order;
  double winv[(ORC_MAX_ORDER + 1) * (ORC_MAX_ORDER + 1)];
  double dist[ORC_MAX_ORDER + 1];
} warp_ctx;

static void warp_init(warp_ctx* w, int order) {
  int n = order + 1;
  double eq[ORC_MAX_ORDER + 1], v[(ORC_MAX_ORDER + 1) * (ORC_MAX_ORDER + 1)];
  eq[0] = -1.0; eq[order] = 1.0;
  for (int i = 1; i < order; ++i) eq[i] = 2.0 * (double)i / (double)order - 1.0;
  /* transpose of the Vandermonde matrix on equidistant nodes (:157-165) */
  for (int col = 0; col < n; ++col)
    for (int row = 0; row < n; ++row) v[row * n + col] = orc_jacobi_p(0.0, 0.0, row, eq[col]);
  orc_mat_inverse(n, v, w->winv);
  double pos[ORC_MAX_ORDER + 1];
  orc_gl_points(n, pos);
  for (int i = 0; i <= order; ++i) w->dist[i] = pos[i] - eq[i];
  w->order = order;
}

static double warp_factor(const warp_ctx* w, double r) {
  int n = w->order + 1;
  double p[ORC_MAX_ORDER + 1], l[ORC_MAX_ORDER + 1];
  for (int i = 0; i < n; ++i) { p[i] = orc_jacobi_p(0.0, 0.0, i, r); l[i] = 0.0; }
  gemv(n, n, w->winv, 1.0, p, 0.0, l);
  double s = 0.0;
  for (int i = 0; i < n; ++i) s += l[i] * w->dist[i];
  return fabs(r) < (1.0 - DBL_EPSILON * 10) ? s / (1.0 - r * r) : 0.0;
}

int orc_nodes(int N, double* rr, double* ss) {
  if (N < 1 || N > ORC_MAX_ORDER) return -1;
  warp_ctx w;
  warp_init(&w, N);
  double alpha = N < 16 ? s_alpha[N - 1] : 5.0 / 3.0;
  double sqrt3 = sqrt(1.0 + 2.0);
  int k = 0;
  for (int i = 0; i <= N; ++i)
    for (int j = 0; j <= N - i; ++j) {
      double l1 = (double)i / (double)N;
      double l3 = (double)j / (double)N;
      double l2 = 1.0 - l1 - l3;
      double x = l3 - l2;
      double y = (2.0 * l1 - l2 - l3) / sqrt3;
      double w1 = 2.0 * 2.0 * l2 * l3 * (1.0 + alpha * l1 * alpha * l1) * warp_factor(&w, l3 - l2);
      double w2 = 2.0 * 2.0 * l3 * l1 * (1.0 + alpha * l2 * alpha * l2) * warp_factor(&w, l1 - l3);
      double w3 = 2.0 * 2.0 * l1 * l2 * (1.0 + alpha * l3 * alpha * l3) * warp_factor(&w, l2 - l1);
      x += (w1 - 0.5 * w2 - 0.5 * w3);
      y += 0.5 * sqrt3 * (w2 - w3);
      l1 = (1.0 + sqrt3 * y) / 3.0;
      l2 = (2.0 - 3.0 * x - sqrt3 * y) / 6.0;
      l3 = (2.0 + 3.0 * x - sqrt3 * y) / 6.0;
      rr[k] = l3 - l2 - l1;
      ss[k] = l1 - l2 - l3;
      ++k;
    }
  return 0;
}

/* face node lists, counter-clockwise (alpha_optimized_nodes_triangle.h:69-102) */
int orc_face_nodes(int N, int face, int* idx) {
  int Np = (N + 1) * (N + 2) / 2;
  int delta = face == 0 ? 1 : (face == 1 ? N : 2);
  int prev = face == 0 ? 0 : (face == 1 ? N : Np - 1);
  idx[0] = prev;
  for (int i = 1; i <= N; ++i) {
    int node;
    if (face == 0) node = prev + delta;
    else if (face == 1) node = prev + delta--;
    else node = prev - delta++;
    idx[i] = node;
    prev = node;
  }
  return 0;
}

/* ------------------------------------------------------------------------- */
/* Orthonormal basis on the triangle: src/orthonormal_basis_triangle.h:45-76 */
/* ------------------------------------------------------------------------- */
static void rs_to_ab(double r, double s, double* a, double* b) {
  *a = s == 1.0 ? -1.0 : 2.0 * (1.0 + r) / (1.0 - s) - 1.0;
  *b = s;
}

static double basis_value(int i, double r, int j, double s) {
  double a, b;
  rs_to_ab(r, s, &a, &b);
  return sqrt(2.0) * orc_jacobi_p(0.0, 0.0, i, a) * orc_jacobi_p(2.0 * i + 1.0, 0.0, j, b) *
         pow(1.0 - b, (double)i);
}

static void basis_grad(int i, double r, int j, double s, double* dr, double* ds) {
  double a, b;
  rs_to_ab(r, s, &a, &b);
  double va = orc_jacobi_p(0.0, 0.0, i, a);
  double vb = orc_jacobi_p(2.0 * i + 1.0, 0.0, j, b);
  double da = orc_jacobi_dp(0.0, 0.0, i, a);
  double db = orc_jacobi_dp(2.0 * i + 1.0, 0.0, j, b);
  double d_r = sqrt(2.0) * da * vb;
  if (i > 0) d_r *= (2.0 * pow(1.0 - b, (double)(i - 1)));
  double d_s = i == 0 ? sqrt(2.0) * (da * vb * 0.5 * (1.0 + a) + va * db)
                      : sqrt(2.0) * pow(1.0 - b, (double)(i - 1)) *
                            (da * vb * (1.0 + a) + va * db * (1.0 - b) - (double)i * va * vb);
  *dr = d_r;
  *ds = d_s;
}

/* reference_triangle.h:45-66 */
int orc_vandermonde(int N, double* V) {
  int Np = (N + 1) * (N + 2) / 2;
  double r[ORC_MAX_NP], s[ORC_MAX_NP];
  if (orc_nodes(N, r, s)) return -1;
  int col = 0;
  for (int i = 0; i <= N; ++i)
    for (int j = 0; j <= N - i; ++j) {
      for (int row = 0; row < Np; ++row) V[row * Np + col] = basis_value(i, r[row], j, s[row]);
      col++;
    }
  return 0;
}

/* reference_triangle.h:68-94 */
int orc_grad_vandermonde(int N, double* Vr, double* Vs) {
  int Np = (N + 1) * (N + 2) / 2;
  double r[ORC_MAX_NP], s[ORC_MAX_NP];
  if (orc_nodes(N, r, s)) return -1;
  int col = 0;
  for (int i = 0; i <= N; ++i)
    for (int j = 0; j <= N - i; ++j) {
      for (int row = 0; row < Np; ++row)
        basis_grad(i, r[row], j, s[row], &Vr[row * Np + col], &Vs[row * Np + col]);
      col++;
    }
  return 0;
}

/* reference_triangle.h:96-114; segment basis = normalised Legendre
 * (orthonormal_basis_segment.h:36-37) */
int orc_face_vandermonde(int N, int face, double* fV) {
  double r[ORC_MAX_NP], s[ORC_MAX_NP];
  int fn[ORC_MAX_NFP];
  if (orc_nodes(N, r, s)) return -1;
  orc_face_nodes(N, face, fn);
  int n = N + 1;
  for (int row = 0; row < n; ++row)
    for (int col = 0; col < n; ++col)
      fV[row * n + col] = orc_jacobi_p(0.0, 0.0, col, face == 0 ? r[fn[row]] : s[fn[row]]);
  return 0;
}

/* Operator matrices.
 *  weak form  (examples/advection_2d/advection_2d.h:78-101, maxwell_2d.h:83-106):
 *     Minv = V V^T, M = Minv^-1, Dr = V Vr^T M, Ds = V Vs^T M
 *  strong form (src/laplace_2d.h:88-112):  Dr = Vr V^-1, Ds = Vs V^-1
 *  LIFT = Minv E with E the face mass matrices (Vf Vf^T)^-1 placed on face rows. */
int orc_operators(int N, int form, double* Dr, double* Ds, double* L, double* Mout) {
  if (N < 1 || N > ORC_MAX_ORDER) return -1;
  int Np = (N + 1) * (N + 2) / 2, Nfp = N + 1;
  size_t nn = (size_t)Np * Np;
  double* V = calloc(nn, sizeof(double));
  double* Vr = calloc(nn, sizeof(double));
  double* Vs = calloc(nn, sizeof(double));
  double* VT = calloc(nn, sizeof(double));
  double* Minv = calloc(nn, sizeof(double));
  double* M = calloc(nn, sizeof(double));
  double* T1 = calloc(nn, sizeof(double));
  double* T2 = calloc(nn, sizeof(double));
  double* E = calloc((size_t)Np * 3 * Nfp, sizeof(double));
  orc_vandermonde(N, V);
  orc_grad_vandermonde(N, Vr, Vs);
  mat_transpose(Np, Np, V, VT);
  mat_mul(Np, Np, Np, V, VT, Minv);
  orc_mat_inverse(Np, Minv, M);
  if (form == ORC_WEAK) {
    mat_transpose(Np, Np, Vr, T1);
    mat_mul(Np, Np, Np, V, T1, T2);
    mat_mul(Np, Np, Np, T2, M, Dr);
    mat_transpose(Np, Np, Vs, T1);
    mat_mul(Np, Np, Np, V, T1, T2);
    mat_mul(Np, Np, Np, T2, M, Ds);
  } else {
    orc_mat_inverse(Np, V, T1);
    mat_mul(Np, Np, Np, Vr, T1, Dr);
    mat_mul(Np, Np, Np, Vs, T1, Ds);
  }
  for (int e = 0; e < 3; ++e) {
    int fn[ORC_MAX_NFP];
    double fV[ORC_MAX_NFP * ORC_MAX_NFP], fVT[ORC_MAX_NFP * ORC_MAX_NFP];
    double eM[ORC_MAX_NFP * ORC_MAX_NFP], eMi[ORC_MAX_NFP * ORC_MAX_NFP];
    orc_face_nodes(N, e, fn);
    orc_face_vandermonde(N, e, fV);
    mat_transpose(Nfp, Nfp, fV, fVT);
    mat_mul(Nfp, Nfp, Nfp, fV, fVT, eM);
    orc_mat_inverse(Nfp, eM, eMi);
    for (int row = 0; row < Nfp; ++row)
      for (int col = 0; col < Nfp; ++col) E[fn[row] * 3 * Nfp + e * Nfp + col] = eMi[row * Nfp + col];
  }
  mat_mul(Np, Np, 3 * Nfp, Minv, E, L);
  if (Mout) memcpy(Mout, M, sizeof(double) * nn);
  free(V); free(Vr); free(Vs); free(VT); free(Minv); free(M); free(T1); free(T2); free(E);
  return 0;
}

/* ------------------------------------------------------------------------- */
/* Mesh, geometry and discretisation                                          */
/* ------------------------------------------------------------------------- */
struct orc {
  int N, Np, Nfp, K, nv;
  double *vx, *vy;
  int32_t* EToV;
  double r[ORC_MAX_NP], s[ORC_MAX_NP];
  int Fmask[3][ORC_MAX_NFP];
  double *Drw, *Dsw, *Lw, *Drs, *Dss, *Ls, *M;
  /* per cell */
  double *invJ, *J, *faceJ, *nx, *ny;
  int32_t *nbC, *nbF; /* neighbour cell / face; boundary: self / offset into boundary nodes */
  int32_t* isB;
  int nbnd;
  double *bx, *by;
  /* work */
  double *flux, *qx, *qy, *du, *tmp;
  double *w[5];
  size_t wlen;
};

/* mapping_2d.h:82-99 */
static void rs_to_xy(const orc* o, int c, double r, double s, double* x, double* y) {
  const double half = 0.5;
  double l1 = half * (s + 1.0), l2 = -half * (r + s), l3 = half * (r + 1.0);
  const int32_t* v = o->EToV + 3 * c;
  *x = l2 * o->vx[v[0]] + l3 * o->vx[v[1]] + l1 * o->vx[v[2]];
  *y = l2 * o->vy[v[0]] + l3 * o->vy[v[1]] + l1 * o->vy[v[2]];
}

/* basic_geom_2d.h:110-153 */
static void outward_normal(const orc* o, int c, int edge, double* nxo, double* nyo) {
  const int32_t* v = o->EToV + 3 * c;
  double p0x = o->vx[v[0]], p0y = o->vy[v[0]], p1x = o->vx[v[1]], p1y = o->vy[v[1]];
  double p2x = o->vx[v[2]], p2y = o->vy[v[2]];
  double x, y, x1, y1;
  switch (edge) {
    case 0: x = p1x - p0x; y = p1y - p0y; x1 = p2x - p0x; y1 = p2y - p0y; break;
    case 1: x = p2x - p1x; y = p2y - p1y; x1 = p0x - p1x; y1 = p0y - p1y; break;
    default: x = p0x - p2x; y = p0y - p2y; x1 = p1x - p2x; y1 = p1y - p2y; break;
  }
  if ((y * x1 - x * y1) > 0.0) { y = -y; x = -x; }
  double l = sqrt(y * y + x * x);
  *nxo = y / l;
  *nyo = -x / l;
}

typedef struct { int32_t a, b, c, e; } half_edge;
static int he_cmp(const void* p, const void* q) {
  const half_edge* x = p; const half_edge* y = q;
  if (x->a != y->a) return x->a < y->a ? -1 : 1;
  if (x->b != y->b) return x->b < y->b ? -1 : 1;
  if (x->c != y->c) return x->c < y->c ? -1 : 1;
  return x->e < y->e ? -1 : (x->e > y->e);
}

orc* orc_create(int N, int nv, const double* vxy, int K, const int32_t* cells) {
  if (N < 1 || N > ORC_MAX_ORDER || K < 1 || nv < 3) return NULL;
  orc* o = calloc(1, sizeof(orc));
  o->N = N; o->Np = (N + 1) * (N + 2) / 2; o->Nfp = N + 1; o->K = K; o->nv = nv;
  int Np = o->Np, Nfp = o->Nfp;
  o->vx = malloc(sizeof(double) * nv); o->vy = malloc(sizeof(double) * nv);
  /* vertices are sequenced x then y; the reference's fill_vertices
   * (src/mesh/simple_triangular_mesh_2d.h:65) leaves that order unspecified */
  for (int i = 0; i < nv; ++i) { o->vx[i] = vxy[2 * i]; o->vy[i] = vxy[2 * i + 1]; }
  o->EToV = malloc(sizeof(int32_t) * 3 * K);
  memcpy(o->EToV, cells, sizeof(int32_t) * 3 * K);
  orc_nodes(N, o->r, o->s);
  for (int f = 0; f < 3; ++f) orc_face_nodes(N, f, o->Fmask[f]);
  size_t nn = (size_t)Np * Np, nl = (size_t)Np * 3 * Nfp;
  o->Drw = malloc(8 * nn); o->Dsw = malloc(8 * nn); o->Lw = malloc(8 * nl);
  o->Drs = malloc(8 * nn); o->Dss = malloc(8 * nn); o->Ls = malloc(8 * nl); o->M = malloc(8 * nn);
  orc_operators(N, ORC_WEAK, o->Drw, o->Dsw, o->Lw, o->M);
  orc_operators(N, ORC_STRONG, o->Drs, o->Dss, o->Ls, NULL);

  o->invJ = malloc(8 * 4 * (size_t)K); o->J = malloc(8 * (size_t)K);
  o->faceJ = malloc(8 * 3 * (size_t)K); o->nx = malloc(8 * 3 * (size_t)K); o->ny = malloc(8 * 3 * (size_t)K);
  for (int c = 0; c < K; ++c) {
    const int32_t* v = o->EToV + 3 * c;
    double v1x = o->vx[v[0]], v1y = o->vy[v[0]], v2x = o->vx[v[1]], v2y = o->vy[v[1]];
    double v3x = o->vx[v[2]], v3y = o->vy[v[2]];
    /* mapping_2d.h:101-118, inverted by Gauss-Jordan as in simple_discretization_2d.h:95-100 */
    double jac[4] = {0.5 * (v2x - v1x), 0.5 * (v3x - v1x), 0.5 * (v2y - v1y), 0.5 * (v3y - v1y)};
    double ji[4];
    orc_mat_inverse(2, jac, ji);
    for (int i = 0; i < 4; ++i) o->invJ[4 * c + i] = ji[i];
    /* mapping_2d.h:120-129 */
    o->J[c] = (1.0 / 4.0) * ((v2x - v1x) * (v3y - v1y) - (v3x - v1x) * (v2y - v1y));
    /* mapping_2d.h:131-158 */
    for (int f = 0; f < 3; ++f) {
      int a = v[f], b = v[(f + 1) % 3];
      double dx = o->vx[a] - o->vx[b], dy = o->vy[a] - o->vy[b];
      o->faceJ[3 * c + f] = 0.5 * sqrt(dx * dx + dy * dy);
      outward_normal(o, c, f, &o->nx[3 * c + f], &o->ny[3 * c + f]);
    }
  }
  /* twin half-edges (simple_triangular_mesh_2d.h:151-183): faces sharing the same
   * unordered vertex pair are twins; an unmatched face is a boundary face. */
  half_edge* he = malloc(sizeof(half_edge) * 3 * (size_t)K);
  for (int c = 0; c < K; ++c)
    for (int e = 0; e < 3; ++e) {
      int32_t v0 = o->EToV[3 * c + e], v1 = o->EToV[3 * c + (e + 1) % 3];
      half_edge h = {v0 < v1 ? v0 : v1, v0 < v1 ? v1 : v0, c, e};
      he[3 * c + e] = h;
    }
  qsort(he, 3 * (size_t)K, sizeof(half_edge), he_cmp);
  o->nbC = malloc(4 * 3 * (size_t)K); o->nbF = malloc(4 * 3 * (size_t)K); o->isB = malloc(4 * 3 * (size_t)K);
  for (int i = 0; i < 3 * K; ++i) { o->nbC[i] = -1; }
  for (int i = 0; i < 3 * K;) {
    if (i + 1 < 3 * K && he[i].a == he[i + 1].a && he[i].b == he[i + 1].b) {
      o->nbC[3 * he[i].c + he[i].e] = he[i + 1].c; o->nbF[3 * he[i].c + he[i].e] = he[i + 1].e;
      o->nbC[3 * he[i + 1].c + he[i + 1].e] = he[i].c; o->nbF[3 * he[i + 1].c + he[i + 1].e] = he[i].e;
      i += 2;
    } else {
      o->nbC[3 * he[i].c + he[i].e] = he[i].c; o->nbF[3 * he[i].c + he[i].e] = he[i].e;
      i += 1;
    }
  }
  free(he);
  /* boundary faces carry an offset into the boundary-node list
   * (simple_discretization_2d.h:136-162) */
  int offset = 0;
  for (int c = 0; c < K; ++c)
    for (int e = 0; e < 3; ++e) {
      int b = o->nbC[3 * c + e] == c;
      o->isB[3 * c + e] = b;
      if (b) { o->nbF[3 * c + e] = offset; offset += Nfp; }
    }
  o->nbnd = offset;
  o->bx = malloc(8 * (size_t)(offset + 1)); o->by = malloc(8 * (size_t)(offset + 1));
  int k = 0;
  for (int c = 0; c < K; ++c)
    for (int e = 0; e < 3; ++e)
      if (o->isB[3 * c + e])
        for (int i = 0; i < Nfp; ++i, ++k) {
          int nd = o->Fmask[e][i];
          rs_to_xy(o, c, o->r[nd], o->s[nd], &o->bx[k], &o->by[k]);
        }
  size_t KNp = (size_t)K * Np;
  o->flux = calloc(3 * 3 * (size_t)K * Nfp, 8);
  o->qx = calloc(KNp, 8); o->qy = calloc(KNp, 8); o->du = calloc(3 * (size_t)K * Nfp, 8);
  o->tmp = calloc(KNp, 8);
  o->wlen = 3 * KNp;
  for (int i = 0; i < 5; ++i) o->w[i] = calloc(o->wlen, 8);
  return o;
}

void orc_destroy(orc* o) {
  if (!o) return;
  free(o->vx); free(o->vy); free(o->EToV);
  free(o->Drw); free(o->Dsw); free(o->Lw); free(o->Drs); free(o->Dss); free(o->Ls); free(o->M);
  free(o->invJ); free(o->J); free(o->faceJ); free(o->nx); free(o->ny);
  free(o->nbC); free(o->nbF); free(o->isB); free(o->bx); free(o->by);
  free(o->flux); free(o->qx); free(o->qy); free(o->du); free(o->tmp);
  for (int i = 0; i < 5; ++i) free(o->w[i]);
  free(o);
}

int orc_num_boundary_nodes(const orc* o) { return o->nbnd; }

void orc_fill_cell_mappings(const orc* o, double* invJ, double* J, double* faceJ) {
  memcpy(invJ, o->invJ, 8 * 4 * (size_t)o->K);
  memcpy(J, o->J, 8 * (size_t)o->K);
  memcpy(faceJ, o->faceJ, 8 * 3 * (size_t)o->K);
}
void orc_fill_cell_interfaces(const orc* o, int32_t* cells, int32_t* faces) {
  memcpy(cells, o->nbC, 4 * 3 * (size_t)o->K);
  memcpy(faces, o->nbF, 4 * 3 * (size_t)o->K);
}
void orc_fill_boundary_nodes(const orc* o, double* bx, double* by) {
  memcpy(bx, o->bx, 8 * (size_t)o->nbnd);
  memcpy(by, o->by, 8 * (size_t)o->nbnd);
}
void orc_fill_outward_normals(const orc* o, double* nx, double* ny) {
  memcpy(nx, o->nx, 8 * 3 * (size_t)o->K);
  memcpy(ny, o->ny, 8 * 3 * (size_t)o->K);
}
void orc_node_xy(const orc* o, double* x, double* y) {
  for (int c = 0; c < o->K; ++c)
    for (int j = 0; j < o->Np; ++j)
      rs_to_xy(o, c, o->r[j], o->s[j], &x[(size_t)c * o->Np + j], &y[(size_t)c * o->Np + j]);
}

/* Dx = Dr*rx + Ds*sx (advection_2d.h:237-238), elementwise */
static void phys_matrix(const orc* o, const double* Dr, const double* Ds, int c, int dir, double* D) {
  double a = o->invJ[4 * c + dir], b = o->invJ[4 * c + 2 + dir];
  int nn = o->Np * o->Np;
  for (int i = 0; i < nn; ++i) D[i] = Dr[i] * a + Ds[i] * b;
}

/* Exterior trace at a face node: the neighbour's node (its face nodes in
 * reverse order) or, on the boundary, g[b] + sign * interior for boundary
 * node b -- the form of every exterior_val callback of the reference's
 * boundary-condition objects (examples/stokes_2d/stokes_2d.h:113-187). */
static double exterior(const orc* o, const double* u, const double* g, double sign, int c, int e, int d,
                       double a) {
  if (o->isB[3 * c + e]) return (g ? g[o->nbF[3 * c + e] + d] : 0.0) + sign * a;
  int nbc = o->nbC[3 * c + e], nbf = o->nbF[3 * c + e];
  return u[(size_t)nbc * o->Np + o->Fmask[nbf][o->Nfp - d - 1]];
}

/* grad_2d::numerical_fluxes + operator() (src/grad_2d.h:94-187): weak-form
 * gradient with the central flux (u- + u+)/2 projected on the outward normal. */
void orc_grad(orc* o, const double* u, const double* g, double sign, double* gx, double* gy) {
  int Np = o->Np, Nfp = o->Nfp, K = o->K;
  double D[ORC_MAX_NP * ORC_MAX_NP], mFx[3 * ORC_MAX_NFP], mFy[3 * ORC_MAX_NFP];
  for (int c = 0; c < K; ++c)
    for (int e = 0; e < 3; ++e)
      for (int d = 0; d < Nfp; ++d) {
        double a = u[(size_t)c * Np + o->Fmask[e][d]];
        o->flux[(size_t)c * 3 * Nfp + e * Nfp + d] = (a + exterior(o, u, g, sign, c, e, d, a)) / 2.0;
      }
  for (int c = 0; c < K; ++c) {
    size_t off = (size_t)c * Np;
    phys_matrix(o, o->Drw, o->Dsw, c, 0, D);
    gemv(Np, Np, D, -1.0, u + off, 0.0, gx + off);
    phys_matrix(o, o->Drw, o->Dsw, c, 1, D);
    gemv(Np, Np, D, -1.0, u + off, 0.0, gy + off);
    for (int e = 0; e < 3; ++e) {
      double fJ = o->faceJ[3 * c + e], nx = o->nx[3 * c + e], ny = o->ny[3 * c + e];
      for (int i = 0; i < Nfp; ++i) {
        double F = o->flux[(size_t)c * 3 * Nfp + e * Nfp + i];
        mFx[e * Nfp + i] = F * nx * fJ;
        mFy[e * Nfp + i] = F * ny * fJ;
      }
    }
    gemv(Np, 3 * Nfp, o->Lw, 1.0 / o->J[c], mFx, 1.0, gx + off);
    gemv(Np, 3 * Nfp, o->Lw, 1.0 / o->J[c], mFy, 1.0, gy + off);
  }
}

/* div_2d::numerical_fluxes + operator() (src/div_2d.h:94-190): weak-form
 * divergence with the central flux n.(u- + u+)/2. */
void orc_div(orc* o, const double* ux, const double* uy, const double* gx, const double* gy, double sign,
             double* out) {
  int Np = o->Np, Nfp = o->Nfp, K = o->K;
  double D[ORC_MAX_NP * ORC_MAX_NP], mF[3 * ORC_MAX_NFP];
  for (int c = 0; c < K; ++c)
    for (int e = 0; e < 3; ++e) {
      double nx = o->nx[3 * c + e], ny = o->ny[3 * c + e];
      for (int d = 0; d < Nfp; ++d) {
        size_t ia = (size_t)c * Np + o->Fmask[e][d];
        double a0 = ux[ia], a1 = uy[ia];
        double b0 = exterior(o, ux, gx, sign, c, e, d, a0), b1 = exterior(o, uy, gy, sign, c, e, d, a1);
        o->flux[(size_t)c * 3 * Nfp + e * Nfp + d] = ((a0 + b0) * nx + (a1 + b1) * ny) / 2.0;
      }
    }
  for (int c = 0; c < K; ++c) {
    size_t off = (size_t)c * Np;
    phys_matrix(o, o->Drw, o->Dsw, c, 0, D);
    gemv(Np, Np, D, -1.0, ux + off, 0.0, out + off);
    phys_matrix(o, o->Drw, o->Dsw, c, 1, D);
    gemv(Np, Np, D, -1.0, uy + off, 1.0, out + off);
    for (int e = 0; e < 3; ++e) {
      double fJ = o->faceJ[3 * c + e];
      for (int i = 0; i < Nfp; ++i) mF[e * Nfp + i] = o->flux[(size_t)c * 3 * Nfp + e * Nfp + i] * fJ;
    }
    gemv(Np, 3 * Nfp, o->Lw, 1.0 / o->J[c], mF, 1.0, out + off);
  }
}

/* ------------------------------------------------------------------------- */
/* Right-hand sides                                                           */
/* ------------------------------------------------------------------------- */
int orc_num_fields(const orc_problem* p) { return p->kind == ORC_ADVECTION ? 1 : 3; }

static double adv_exact(const orc_problem* p, double x, double y, double t) {
  switch (p->bc) {
    case ORC_BC_SINSIN: /* advection_2d.h:152,191 (there a = (1,1)) */
      return sin((x + 1.0 - p->ax * t) * M_PI) * sin((y + 1.0 - p->ay * t) * M_PI);
    case ORC_BC_GAUSS: {
      double dx = x - p->ax * t - p->gx0, dy = y - p->ay * t - p->gy0;
      return exp(-(dx * dx + dy * dy) / p->gw);
    }
    default: return 0.0;
  }
}

/* Advection: examples/advection_2d/advection_2d.h:156-258, generalised from the
 * hard-coded a = (1,1) to a = (ax, ay): the upwind test (n.x()+n.y()) becomes a.n
 * and the volume term Dx u + Dy u becomes ax Dx u + ay Dy u. */
static void adv_rhs(orc* o, const orc_problem* p, double t, const double* u, double* out) {
  int Np = o->Np, Nfp = o->Nfp, K = o->K;
  for (int c = 0; c < K; ++c)
    for (int e = 0; e < 3; ++e) {
      int isb = o->isB[3 * c + e], nbc = o->nbC[3 * c + e], nbf = o->nbF[3 * c + e];
      double nx = o->nx[3 * c + e], ny = o->ny[3 * c + e];
      double an = p->ax * nx + p->ay * ny;
      for (int d = 0; d < Nfp; ++d) {
        double aU = u[(size_t)c * Np + o->Fmask[e][d]], bU;
        if (isb) {
          double x, y;
          rs_to_xy(o, c, o->r[o->Fmask[e][d]], o->s[o->Fmask[e][d]], &x, &y);
          bU = adv_exact(p, x, y, t);
        } else {
          bU = u[(size_t)nbc * Np + o->Fmask[nbf][Nfp - d - 1]];
        }
        double U = an >= 0.0 ? aU : bU;
        o->flux[(size_t)c * 3 * Nfp + e * Nfp + d] = U * an;
      }
    }
  double D[ORC_MAX_NP * ORC_MAX_NP], mFl[3 * ORC_MAX_NFP];
  for (int c = 0; c < K; ++c) {
    size_t off = (size_t)c * Np;
    phys_matrix(o, o->Drw, o->Dsw, c, 0, D);
    gemv(Np, Np, D, p->ax, u + off, 0.0, out + off);
    phys_matrix(o, o->Drw, o->Dsw, c, 1, D);
    gemv(Np, Np, D, p->ay, u + off, 1.0, out + off);
    for (int e = 0; e < 3; ++e) {
      double fJ = o->faceJ[3 * c + e];
      for (int i = 0; i < Nfp; ++i) mFl[e * Nfp + i] = o->flux[(size_t)c * 3 * Nfp + e * Nfp + i] * fJ;
    }
    gemv(Np, 3 * Nfp, o->Lw, -1.0 / o->J[c], mFl, 1.0, out + off);
  }
}

/* Maxwell TM (Hx, Hy, Ez), PEC: examples/maxwell_2d/maxwell_2d.h:178-311.
 * Maxwell TE (Ex, Ey, Hz), PEC: the same upwind scheme under Hx -> -Ex,
 * Hy -> -Ey, Ez -> Hz, with the PEC ghost state E+ = -E-, Hz+ = Hz-. */
static void maxwell_rhs(orc* o, const orc_problem* p, const double* q, double* out) {
  int Np = o->Np, Nfp = o->Nfp, K = o->K;
  size_t KNp = (size_t)K * Np, KF = (size_t)K * 3 * Nfp;
  const double *q0 = q, *q1 = q + KNp, *q2 = q + 2 * KNp;
  double *o0 = out, *o1 = out + KNp, *o2 = out + 2 * KNp;
  double *f0 = o->flux, *f1 = o->flux + KF, *f2 = o->flux + 2 * KF;
  int te = p->kind == ORC_MAXWELL_TE;
  for (int c = 0; c < K; ++c)
    for (int e = 0; e < 3; ++e) {
      int isb = o->isB[3 * c + e], nbc = o->nbC[3 * c + e], nbf = o->nbF[3 * c + e];
      double nx = o->nx[3 * c + e], ny = o->ny[3 * c + e];
      for (int d = 0; d < Nfp; ++d) {
        size_t ia = (size_t)c * Np + o->Fmask[e][d];
        double a0 = q0[ia], a1 = q1[ia], a2 = q2[ia], b0, b1, b2;
        if (isb) {
          if (te) { b0 = -a0; b1 = -a1; b2 = a2; }
          else { b0 = a0; b1 = a1; b2 = -a2; }
        } else {
          size_t ib = (size_t)nbc * Np + o->Fmask[nbf][Nfp - d - 1];
          b0 = q0[ib]; b1 = q1[ib]; b2 = q2[ib];
        }
        size_t oi = (size_t)c * 3 * Nfp + e * Nfp + d;
        double dlt0 = a0 - b0, dlt1 = a1 - b1, sum2 = a2 + b2;
        if (!te) {
          f0[oi] = 0.5 * ny * (sum2 + ny * dlt0 - nx * dlt1);
          f1[oi] = -0.5 * nx * (sum2 + ny * dlt0 - nx * dlt1);
          f2[oi] = 0.5 * (ny * (a0 + b0) - nx * (a1 + b1) + a2 - b2);
        } else {
          f0[oi] = -0.5 * ny * (sum2 - ny * dlt0 + nx * dlt1);
          f1[oi] = 0.5 * nx * (sum2 - ny * dlt0 + nx * dlt1);
          f2[oi] = 0.5 * (nx * (a1 + b1) - ny * (a0 + b0) + a2 - b2);
        }
      }
    }
  double Dx[ORC_MAX_NP * ORC_MAX_NP], Dy[ORC_MAX_NP * ORC_MAX_NP];
  double g0[3 * ORC_MAX_NFP], g1[3 * ORC_MAX_NFP], g2[3 * ORC_MAX_NFP];
  for (int c = 0; c < K; ++c) {
    size_t off = (size_t)c * Np;
    phys_matrix(o, o->Drw, o->Dsw, c, 0, Dx);
    phys_matrix(o, o->Drw, o->Dsw, c, 1, Dy);
    if (!te) { /* maxwell_2d.h:286-289 */
      gemv(Np, Np, Dy, 1.0, q2 + off, 0.0, o0 + off);
      gemv(Np, Np, Dx, -1.0, q2 + off, 0.0, o1 + off);
      gemv(Np, Np, Dx, -1.0, q1 + off, 0.0, o2 + off);
      gemv(Np, Np, Dy, 1.0, q0 + off, 1.0, o2 + off);
    } else {
      gemv(Np, Np, Dy, -1.0, q2 + off, 0.0, o0 + off);
      gemv(Np, Np, Dx, 1.0, q2 + off, 0.0, o1 + off);
      gemv(Np, Np, Dx, 1.0, q1 + off, 0.0, o2 + off);
      gemv(Np, Np, Dy, -1.0, q0 + off, 1.0, o2 + off);
    }
    size_t offF = (size_t)c * 3 * Nfp;
    for (int e = 0; e < 3; ++e) {
      double fJ = o->faceJ[3 * c + e];
      for (int i = 0; i < Nfp; ++i) {
        int ei = e * Nfp + i;
        g0[ei] = f0[offF + ei] * fJ; g1[ei] = f1[offF + ei] * fJ; g2[ei] = f2[offF + ei] * fJ;
      }
    }
    double cJ = o->J[c];
    gemv(Np, 3 * Nfp, o->Lw, -1.0 / cJ, g0, 1.0, o0 + off);
    gemv(Np, 3 * Nfp, o->Lw, -1.0 / cJ, g1, 1.0, o1 + off);
    gemv(Np, 3 * Nfp, o->Lw, -1.0 / cJ, g2, 1.0, o2 + off);
  }
}

void orc_rhs(orc* o, const orc_problem* p, double t, const double* q, double* out) {
  if (p->kind == ORC_ADVECTION) adv_rhs(o, p, t, q, out);
  else maxwell_rhs(o, p, q, out);
}

void orc_exact(orc* o, const orc_problem* p, double t, double* q) {
  size_t KNp = (size_t)o->K * o->Np;
  for (int c = 0; c < o->K; ++c)
    for (int j = 0; j < o->Np; ++j) {
      double x, y;
      size_t i = (size_t)c * o->Np + j;
      rs_to_xy(o, c, o->r[j], o->s[j], &x, &y);
      double s2 = sqrt(2.0);
      if (p->kind == ORC_ADVECTION) {
        q[i] = adv_exact(p, x, y, t);
      } else if (p->kind == ORC_MAXWELL_TM) { /* maxwell_2d.h:172-174 */
        q[i] = -sin(x * M_PI) * cos(y * M_PI) * sin(s2 * M_PI * t) / s2;
        q[i + KNp] = cos(x * M_PI) * sin(y * M_PI) * sin(s2 * M_PI * t) / s2;
        q[i + 2 * KNp] = sin(x * M_PI) * sin(y * M_PI) * cos(s2 * M_PI * t);
      } else { /* TE cavity mode Hz = cos(pi x) cos(pi y) cos(sqrt2 pi t) */
        q[i] = -cos(x * M_PI) * sin(y * M_PI) * sin(s2 * M_PI * t) / s2;
        q[i + KNp] = sin(x * M_PI) * cos(y * M_PI) * sin(s2 * M_PI * t) / s2;
        q[i + 2 * KNp] = cos(x * M_PI) * cos(y * M_PI) * cos(s2 * M_PI * t);
      }
    }
}

/* ------------------------------------------------------------------------- */
/* Time integrators                                                           */
/* ------------------------------------------------------------------------- */
static void axpy_n(double a, const double* x, size_t n, const double* y, double* out) {
  for (size_t i = 0; i < n; ++i) out[i] = a * x[i] + y[i]; /* src/axpy.h:121 */
}

/* classical RK4: src/explicit_runge_kutta.h:33-51 */
void orc_rk4_step(orc* o, const orc_problem* p, double t, double dt, double* q) {
  size_t n = (size_t)orc_num_fields(p) * o->K * o->Np;
  double **w = o->w;
  orc_rhs(o, p, t, q, w[1]);
  axpy_n(0.5 * dt, w[1], n, q, w[0]);
  orc_rhs(o, p, t + 0.5 * dt, w[0], w[2]);
  axpy_n(0.5 * dt, w[2], n, q, w[0]);
  orc_rhs(o, p, t + 0.5 * dt, w[0], w[3]);
  axpy_n(dt, w[3], n, q, w[0]);
  orc_rhs(o, p, t + dt, w[0], w[4]);
  axpy_n(2.0, w[2], n, w[1], w[0]);
  axpy_n(2.0, w[3], n, w[4], w[1]);
  axpy_n(dt / 6.0, w[0], n, q, w[2]);
  axpy_n(dt / 6.0, w[1], n, w[2], q);
}

/* Low-storage 5-stage 4th-order Runge-Kutta of Carpenter & Kennedy (1994),
 * "Fourth-order 2N-storage Runge-Kutta schemes", NASA TM-109112, solution 3;
 * the reference has no LSERK4 (it uses classical RK4). */
void orc_lserk4_coeffs(double* a, double* b, double* c) {
  static const double A[5] = {0.0, -567301805773.0 / 1357537059087.0,
                              -2404267990393.0 / 2016746695238.0,
                              -3550918686646.0 / 2091501179385.0,
                              -1275806237668.0 / 842570457699.0};
  static const double B[5] = {1432997174477.0 / 9575080441755.0, 5161836677717.0 / 13612068292357.0,
                              1720146321549.0 / 2090206949498.0, 3134564353537.0 / 4481467310338.0,
                              2277821191437.0 / 14882151754819.0};
  static const double C[5] = {0.0, 1432997174477.0 / 9575080441755.0,
                              2526269341429.0 / 6820363962896.0, 2006345519317.0 / 3224310063776.0,
                              2802321613138.0 / 2924317926251.0};
  for (int i = 0; i < 5; ++i) { a[i] = A[i]; b[i] = B[i]; c[i] = C[i]; }
}

void orc_lserk4_step(orc* o, const orc_problem* p, double t, double dt, double* q, double* res) {
  size_t n = (size_t)orc_num_fields(p) * o->K * o->Np;
  double a[5], b[5], c[5];
  orc_lserk4_coeffs(a, b, c);
  double* rhs = o->w[0];
  for (int s = 0; s < 5; ++s) {
    orc_rhs(o, p, t + c[s] * dt, q, rhs);
    for (size_t i = 0; i < n; ++i) {
      res[i] = a[s] * res[i] + dt * rhs[i];
      q[i] = q[i] + b[s] * res[i];
    }
  }
}

/* scheme 0 = classical RK4, 1 = LSERK4; returns the final time */
double orc_run(orc* o, const orc_problem* p, int scheme, double t0, double dt, int nsteps, double* q) {
  size_t n = (size_t)orc_num_fields(p) * o->K * o->Np;
  double* res = calloc(n, 8);
  double t = t0;
  for (int i = 0; i < nsteps; ++i) {
    if (scheme == 0) orc_rk4_step(o, p, t, dt, q);
    else orc_lserk4_step(o, p, t, dt, q, res);
    t += dt;
  }
  free(res);
  return t;
}

/* ------------------------------------------------------------------------- */
/* laplace_2d: src/laplace_2d.h:130-251 (apply_homogeneous).                  */
/* The reference penalty is tau = 1 (:209-210, :244, "2 * du"); tau_mode 1    */
/* scales the jump term per face by tau_f = (N+1)^2 / h_f, h_f the smaller of  */
/* the two altitudes onto the face (2 J / faceJ in reference units).          */
/* With homogeneous Dirichlet data apply_inhomogeneous_as_rhs adds only zeros, */
/* so laplace_2d::operator() (:121-128) equals apply_homogeneous.             */
/* ------------------------------------------------------------------------- */
static double face_tau(const orc* o, int c, int e, int tau_mode) {
  if (tau_mode == 0) return 1.0;
  double N1 = (double)(o->N + 1);
  double hm = 2.0 * o->J[c] / o->faceJ[3 * c + e];
  if (!o->isB[3 * c + e]) {
    int nb = o->nbC[3 * c + e], nf = o->nbF[3 * c + e];
    double hp = 2.0 * o->J[nb] / o->faceJ[3 * nb + nf];
    if (hp < hm) hm = hp;
  }
  return N1 * N1 / hm;
}

/* boundary condition type of boundary node i of face (c, e): the per-node
 * flags when given (is_dirichlet(x, y) of the reference's BC objects), else
 * the uniform type */
static int bc_dir(const orc* o, int dirichlet, const uint8_t* bdir, int c, int e, int i) {
  return bdir ? bdir[o->nbF[3 * c + e] + i] != 0 : dirichlet;
}

/* pass 1 for one cell: q = D u - LIFT(n du faceJ / 2) / J; stores du */
static void lap_pass1_cell(orc* o, int dirichlet, const uint8_t* bdir, const double* u, int c, double* qx,
                           double* qy, double* du) {
  int Np = o->Np, Nfp = o->Nfp;
  double D[ORC_MAX_NP * ORC_MAX_NP], tlx[3 * ORC_MAX_NFP], tly[3 * ORC_MAX_NFP];
  size_t off = (size_t)c * Np;
  phys_matrix(o, o->Drs, o->Dss, c, 0, D);
  gemv(Np, Np, D, 1.0, u + off, 0.0, qx + off);
  phys_matrix(o, o->Drs, o->Dss, c, 1, D);
  gemv(Np, Np, D, 1.0, u + off, 0.0, qy + off);
  for (int e = 0; e < 3; ++e) {
    int isb = o->isB[3 * c + e], nbc = o->nbC[3 * c + e], nbf = o->nbF[3 * c + e];
    double nx = o->nx[3 * c + e], ny = o->ny[3 * c + e], fJ = o->faceJ[3 * c + e];
    for (int i = 0; i < Nfp; ++i) {
      double d;
      if (isb) d = bc_dir(o, dirichlet, bdir, c, e, i) ? 2.0 * u[off + o->Fmask[e][i]] : 0.0;
      else d = u[off + o->Fmask[e][i]] - u[(size_t)nbc * Np + o->Fmask[nbf][Nfp - i - 1]];
      du[(size_t)c * 3 * Nfp + e * Nfp + i] = d;
      tlx[e * Nfp + i] = nx * d * fJ / 2.0;
      tly[e * Nfp + i] = ny * d * fJ / 2.0;
    }
  }
  double cJ = o->J[c];
  gemv(Np, 3 * Nfp, o->Ls, -1.0 / cJ, tlx, 1.0, qx + off);
  gemv(Np, 3 * Nfp, o->Ls, -1.0 / cJ, tly, 1.0, qy + off);
}

static void lap_pass2_cell(orc* o, int dirichlet, const uint8_t* bdir, int tau_mode, const double* qx,
                           const double* qy, const double* du, int c, double* out) {
  int Np = o->Np, Nfp = o->Nfp;
  double D[ORC_MAX_NP * ORC_MAX_NP], tl[3 * ORC_MAX_NFP];
  size_t off = (size_t)c * Np;
  phys_matrix(o, o->Drs, o->Dss, c, 0, D);
  gemv(Np, Np, D, 1.0, qx + off, 0.0, out + off);
  phys_matrix(o, o->Drs, o->Dss, c, 1, D);
  gemv(Np, Np, D, 1.0, qy + off, 1.0, out + off);
  for (int e = 0; e < 3; ++e) {
    int isb = o->isB[3 * c + e], nbc = o->nbC[3 * c + e], nbf = o->nbF[3 * c + e];
    double nx = o->nx[3 * c + e], ny = o->ny[3 * c + e], fJ = o->faceJ[3 * c + e];
    double tau = face_tau(o, c, e, tau_mode);
    for (int i = 0; i < Nfp; ++i) {
      size_t ia = off + o->Fmask[e][i];
      double dqN;
      if (isb) {
        double gn = qx[ia] * nx + qy[ia] * ny;
        dqN = bc_dir(o, dirichlet, bdir, c, e, i) ? 0.0 : 2.0 * gn;
      } else {
        size_t ib = (size_t)nbc * Np + o->Fmask[nbf][Nfp - i - 1];
        dqN = (qx[ia] - qx[ib]) * nx + (qy[ia] - qy[ib]) * ny;
      }
      tl[e * Nfp + i] = (dqN + 2.0 * tau * du[(size_t)c * 3 * Nfp + e * Nfp + i]) * fJ / 2.0;
    }
  }
  gemv(Np, 3 * Nfp, o->Ls, -1.0 / o->J[c], tl, 1.0, out + off);
}

void orc_laplace_apply(orc* o, int dirichlet, int tau_mode, const double* u, double* out) {
  for (int c = 0; c < o->K; ++c) lap_pass1_cell(o, dirichlet, NULL, u, c, o->qx, o->qy, o->du);
  for (int c = 0; c < o->K; ++c) lap_pass2_cell(o, dirichlet, NULL, tau_mode, o->qx, o->qy, o->du, c, out);
}

/* apply_homogeneous with a condition type per boundary node (laplace_2d.h:130-251) */
void orc_laplace_apply_bc(orc* o, const uint8_t* bdir, int tau_mode, const double* u, double* out) {
  for (int c = 0; c < o->K; ++c) lap_pass1_cell(o, 1, bdir, u, c, o->qx, o->qy, o->du);
  for (int c = 0; c < o->K; ++c) lap_pass2_cell(o, 1, bdir, tau_mode, o->qx, o->qy, o->du, c, out);
}

/* apply_inhomogeneous_as_rhs (laplace_2d.h:253-348): adds to out, for every
 * cell with a boundary face, the contribution of the boundary data
 *   q  = -LIFT(n gu faceJ / 2) / J,  gu = g[b] at Dirichlet nodes, else 0
 *   out += Dx qx + Dy qy - LIFT((hq + 2 tau gu) faceJ / 2) / J,
 *          hq = h[b] at Neumann nodes, else 0
 * with g[b] = exterior_val(x, y, 0) and h[b] = exterior_grad_n(x, y, 0) of
 * boundary node b; tau as in the homogeneous passes (1 in the reference). */
void orc_laplace_bc_rhs(orc* o, const uint8_t* bdir, int tau_mode, const double* g, const double* h,
                        double* out) {
  int Np = o->Np, Nfp = o->Nfp;
  double D[ORC_MAX_NP * ORC_MAX_NP], tlx[3 * ORC_MAX_NFP], tly[3 * ORC_MAX_NFP];
  double qx[ORC_MAX_NP], qy[ORC_MAX_NP], gu[3 * ORC_MAX_NFP];
  for (int c = 0; c < o->K; ++c) {
    if (!o->isB[3 * c] && !o->isB[3 * c + 1] && !o->isB[3 * c + 2]) continue;
    for (int m = 0; m < 3 * Nfp; ++m) { tlx[m] = 0.0; tly[m] = 0.0; gu[m] = 0.0; }
    for (int i = 0; i < Np; ++i) { qx[i] = 0.0; qy[i] = 0.0; }  /* gemv reads y even with beta = 0 */
    for (int e = 0; e < 3; ++e) {
      if (!o->isB[3 * c + e]) continue;
      double nx = o->nx[3 * c + e], ny = o->ny[3 * c + e], fJ = o->faceJ[3 * c + e];
      for (int i = 0; i < Nfp; ++i) {
        int b = o->nbF[3 * c + e] + i;
        double v = bc_dir(o, 1, bdir, c, e, i) && g ? g[b] : 0.0;
        gu[e * Nfp + i] = v;
        tlx[e * Nfp + i] = nx * v * fJ / 2.0;
        tly[e * Nfp + i] = ny * v * fJ / 2.0;
      }
    }
    double cJ = o->J[c];
    gemv(Np, 3 * Nfp, o->Ls, -1.0 / cJ, tlx, 0.0, qx);
    gemv(Np, 3 * Nfp, o->Ls, -1.0 / cJ, tly, 0.0, qy);
    size_t off = (size_t)c * Np;
    phys_matrix(o, o->Drs, o->Dss, c, 0, D);
    gemv(Np, Np, D, 1.0, qx, 1.0, out + off);
    phys_matrix(o, o->Drs, o->Dss, c, 1, D);
    gemv(Np, Np, D, 1.0, qy, 1.0, out + off);
    for (int m = 0; m < 3 * Nfp; ++m) tlx[m] = 0.0;
    for (int e = 0; e < 3; ++e) {
      if (!o->isB[3 * c + e]) continue;
      double fJ = o->faceJ[3 * c + e], tau = face_tau(o, c, e, tau_mode);
      for (int i = 0; i < Nfp; ++i) {
        int b = o->nbF[3 * c + e] + i;
        double hq = !bc_dir(o, 1, bdir, c, e, i) && h ? h[b] : 0.0;
        tlx[e * Nfp + i] = (hq + 2.0 * tau * gu[e * Nfp + i]) * fJ / 2.0;
      }
    }
    gemv(Np, 3 * Nfp, o->Ls, -1.0 / cJ, tlx, 1.0, out + off);
  }
}

/* The part of the boundary-data contribution that apply_inhomogeneous_as_rhs
 * (laplace_2d.h:253-348) leaves out.  Its first pass lifts the Dirichlet data
 * into q_d on the boundary cells, but its second pass adds only their
 * boundary-face terms; the affine operator of the scheme also has the jumps of
 * q_d (apply_homogeneous's dqN, laplace_2d.h:222-242):
 *   out += -LIFT(dqN faceJ / 2) / J on every cell,
 *   dqN = (q_d(c) - q_d(nb)).n on interior faces, 2 q_d(c).n on Neumann
 *   boundary faces, 0 on Dirichlet faces (q_d = 0 off the boundary cells).
 * With it, laplace_apply(u) - bc_rhs - bc_jump is exact on polynomials of
 * degree <= N with their own boundary data; without it (the reference) it is
 * not, for non-zero Dirichlet data. */
void orc_laplace_bc_jump(orc* o, const uint8_t* bdir, const double* g, double* out) {
  int Np = o->Np, Nfp = o->Nfp;
  double tlx[3 * ORC_MAX_NFP], tly[3 * ORC_MAX_NFP], tl[3 * ORC_MAX_NFP];
  size_t n = (size_t)o->K * Np;
  for (size_t i = 0; i < n; ++i) { o->qx[i] = 0.0; o->qy[i] = 0.0; }
  if (!g) return;
  for (int c = 0; c < o->K; ++c) {
    if (!o->isB[3 * c] && !o->isB[3 * c + 1] && !o->isB[3 * c + 2]) continue;
    for (int m = 0; m < 3 * Nfp; ++m) { tlx[m] = 0.0; tly[m] = 0.0; }
    for (int e = 0; e < 3; ++e) {
      if (!o->isB[3 * c + e]) continue;
      double nx = o->nx[3 * c + e], ny = o->ny[3 * c + e], fJ = o->faceJ[3 * c + e];
      for (int i = 0; i < Nfp; ++i) {
        double v = bc_dir(o, 1, bdir, c, e, i) ? g[o->nbF[3 * c + e] + i] : 0.0;
        tlx[e * Nfp + i] = nx * v * fJ / 2.0;
        tly[e * Nfp + i] = ny * v * fJ / 2.0;
      }
    }
    size_t off = (size_t)c * Np;
    gemv(Np, 3 * Nfp, o->Ls, -1.0 / o->J[c], tlx, 0.0, o->qx + off);
    gemv(Np, 3 * Nfp, o->Ls, -1.0 / o->J[c], tly, 0.0, o->qy + off);
  }
  for (int c = 0; c < o->K; ++c) {
    size_t off = (size_t)c * Np;
    int any = 0;
    for (int e = 0; e < 3; ++e) {
      int isb = o->isB[3 * c + e], nbc = o->nbC[3 * c + e], nbf = o->nbF[3 * c + e];
      double nx = o->nx[3 * c + e], ny = o->ny[3 * c + e], fJ = o->faceJ[3 * c + e];
      for (int i = 0; i < Nfp; ++i) {
        size_t ia = off + o->Fmask[e][i];
        double dqN;
        if (isb) {
          dqN = bc_dir(o, 1, bdir, c, e, i) ? 0.0 : 2.0 * (o->qx[ia] * nx + o->qy[ia] * ny);
        } else {
          size_t ib = (size_t)nbc * Np + o->Fmask[nbf][Nfp - i - 1];
          dqN = (o->qx[ia] - o->qx[ib]) * nx + (o->qy[ia] - o->qy[ib]) * ny;
        }
        tl[e * Nfp + i] = dqN * fJ / 2.0;
        any |= dqN != 0.0;
      }
    }
    if (any) gemv(Np, 3 * Nfp, o->Ls, -1.0 / o->J[c], tl, 1.0, out + off);
  }
}

/* out = -J_k M (A u)_k : the mass-weighted, symmetric positive definite form */
void orc_spd_apply(orc* o, int tau_mode, const double* u, double* out) {
  int Np = o->Np;
  orc_laplace_apply(o, 1, tau_mode, u, o->tmp);
  for (int c = 0; c < o->K; ++c) {
    size_t off = (size_t)c * Np;
    gemv(Np, Np, o->M, -o->J[c], o->tmp + off, 0.0, out + off);
  }
}

void orc_mass_apply(orc* o, const double* f, double* out) {
  int Np = o->Np;
  for (int c = 0; c < o->K; ++c) {
    size_t off = (size_t)c * Np;
    gemv(Np, Np, o->M, o->J[c], f + off, 0.0, out + off);
  }
}

/* Diagonal blocks S_kk of the SPD form, computed locally: a unit vector on cell
 * k reaches the output of cell k through k's own pass 1 and through the pass-1
 * lift of its interior neighbours (their jumps on the shared faces). */
void orc_spd_diag_blocks(orc* o, int tau_mode, double* blocks) {
  int Np = o->Np, Nfp = o->Nfp, K = o->K;
  size_t KNp = (size_t)K * Np;
  double* u = calloc(KNp, 8);
  double* qx = calloc(KNp, 8); double* qy = calloc(KNp, 8);
  double* du = calloc(3 * (size_t)K * Nfp, 8);
  double* out = calloc(KNp, 8);
  for (int c = 0; c < K; ++c) {
    size_t off = (size_t)c * Np;
    for (int j = 0; j < Np; ++j) {
      u[off + j] = 1.0;
      lap_pass1_cell(o, 1, NULL, u, c, qx, qy, du);
      for (int e = 0; e < 3; ++e)
        if (!o->isB[3 * c + e]) lap_pass1_cell(o, 1, NULL, u, o->nbC[3 * c + e], qx, qy, du);
      lap_pass2_cell(o, 1, NULL, tau_mode, qx, qy, du, c, out);
      double col[ORC_MAX_NP];
      gemv(Np, Np, o->M, -o->J[c], out + off, 0.0, col);
      for (int i = 0; i < Np; ++i) blocks[(size_t)c * Np * Np + (size_t)i * Np + j] = col[i];
      u[off + j] = 0.0;
    }
  }
  free(u); free(qx); free(qy); free(du); free(out);
}

static double dot(const double* a, const double* b, size_t n) {
  double s = 0.0;
  for (size_t i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}

/* Block-Jacobi preconditioned CG on S x = b (the reference solves with a direct
 * sparse QR of the assembled matrix, examples/poisson_2d/main.cpp:130-223; CG is
 * the matrix-free replacement).  Returns iterations, or -1 if maxit reached. */
int orc_pcg(orc* o, int tau_mode, const double* b, double* x, double rtol, int maxit,
            double* final_relres) {
  int Np = o->Np, K = o->K;
  size_t n = (size_t)K * Np;
  double* blk = malloc(8 * (size_t)K * Np * Np);
  double* binv = malloc(8 * (size_t)K * Np * Np);
  orc_spd_diag_blocks(o, tau_mode, blk);
  for (int c = 0; c < K; ++c) orc_mat_inverse(Np, blk + (size_t)c * Np * Np, binv + (size_t)c * Np * Np);
  /* zeroed: gemv reads y even with beta = 0 */
  double *r = calloc(n, 8), *z = calloc(n, 8), *p = calloc(n, 8), *Ap = calloc(n, 8);
  orc_spd_apply(o, tau_mode, x, Ap);
  for (size_t i = 0; i < n; ++i) r[i] = b[i] - Ap[i];
  double bn = sqrt(dot(b, b, n));
  if (bn == 0.0) bn = 1.0;
  for (int c = 0; c < K; ++c) gemv(Np, Np, binv + (size_t)c * Np * Np, 1.0, r + (size_t)c * Np, 0.0, z + (size_t)c * Np);
  memcpy(p, z, 8 * n);
  double rz = dot(r, z, n);
  int it = 0, conv = 0;
  double rel = sqrt(dot(r, r, n)) / bn;
  while (it < maxit) {
    if (rel <= rtol) { conv = 1; break; }
    orc_spd_apply(o, tau_mode, p, Ap);
    double alpha = rz / dot(p, Ap, n);
    for (size_t i = 0; i < n; ++i) { x[i] += alpha * p[i]; r[i] -= alpha * Ap[i]; }
    ++it;
    rel = sqrt(dot(r, r, n)) / bn;
    for (int c = 0; c < K; ++c)
      gemv(Np, Np, binv + (size_t)c * Np * Np, 1.0, r + (size_t)c * Np, 0.0, z + (size_t)c * Np);
    double rz2 = dot(r, z, n);
    double beta = rz2 / rz;
    rz = rz2;
    for (size_t i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
  }
  if (rel <= rtol) conv = 1;
  if (final_relres) *final_relres = rel;
  free(blk); free(binv); free(r); free(z); free(p); free(Ap);
  return conv ? it : -1;
}

/* ------------------------------------------------------------------------- */
/* 1D advection: examples/advection_1d/advection_1d.h (u_t + c u_x = 0 on     */
/* [0, 2 pi], c = 2 pi, K cells of N+1 Gauss-Lobatto nodes, strong form,      */
/* upwind flux, inflow u(0, t) = -sin(2 pi t), outflow extrapolation).        */
/* ------------------------------------------------------------------------- */
struct orc1d {
  int K, N, np;
  double h, c;
  double D[(ORC_MAX_ORDER + 1) * (ORC_MAX_ORDER + 1)], L[(ORC_MAX_ORDER + 1) * (ORC_MAX_ORDER + 1)];
  double xr[ORC_MAX_ORDER + 1];
  double* flux;
  double* w[5];
};

/* advection_1d.h:91-104: V(i,j) = P_j(x_i), Dr = Vr V^-1, D = Dr 2/h, L = V V^T 2/h */
orc1d* orc1d_create(int K, int N) {
  if (K < 1 || N < 1 || N > ORC_MAX_ORDER) return NULL;
  orc1d* o = calloc(1, sizeof(orc1d));
  o->K = K; o->N = N; o->np = N + 1;
  o->c = 2.0 * M_PI;
  o->h = 2.0 * M_PI / K;
  int np = o->np;
  orc_gl_points(np, o->xr);
  double V[(ORC_MAX_ORDER + 1) * (ORC_MAX_ORDER + 1)], Vr[(ORC_MAX_ORDER + 1) * (ORC_MAX_ORDER + 1)];
  double Vi[(ORC_MAX_ORDER + 1) * (ORC_MAX_ORDER + 1)], Dr[(ORC_MAX_ORDER + 1) * (ORC_MAX_ORDER + 1)];
  double VT[(ORC_MAX_ORDER + 1) * (ORC_MAX_ORDER + 1)], Mi[(ORC_MAX_ORDER + 1) * (ORC_MAX_ORDER + 1)];
  for (int i = 0; i < np; ++i)
    for (int j = 0; j < np; ++j) {
      V[i * np + j] = orc_jacobi_p(0.0, 0.0, j, o->xr[i]);
      Vr[i * np + j] = orc_jacobi_dp(0.0, 0.0, j, o->xr[i]);
    }
  orc_mat_inverse(np, V, Vi);
  mat_mul(np, np, np, Vr, Vi, Dr);
  mat_transpose(np, np, V, VT);
  mat_mul(np, np, np, V, VT, Mi);
  for (int i = 0; i < np * np; ++i) {
    o->D[i] = Dr[i] * (2.0 / o->h);
    o->L[i] = Mi[i] * (2.0 / o->h);
  }
  o->flux = calloc((size_t)K + 1, 8);
  for (int i = 0; i < 5; ++i) o->w[i] = calloc((size_t)K * np, 8);
  return o;
}

void orc1d_destroy(orc1d* o) {
  if (!o) return;
  free(o->flux);
  for (int i = 0; i < 5; ++i) free(o->w[i]);
  free(o);
}

void orc1d_operators(const orc1d* o, double* D, double* L) {
  memcpy(D, o->D, sizeof(double) * o->np * o->np);
  memcpy(L, o->L, sizeof(double) * o->np * o->np);
}

/* advection_1d.h:107-146: x = i h + (1 + r_j) h / 2, [cell][node] */
void orc1d_node_x(const orc1d* o, double* x) {
  for (int i = 0; i < o->K; ++i)
    for (int j = 0; j < o->np; ++j) x[(size_t)i * o->np + j] = i * o->h + (1.0 + o->xr[j]) * 0.5 * o->h;
}

void orc1d_exact(const orc1d* o, double t, double* u) {
  for (int i = 0; i < o->K; ++i)
    for (int j = 0; j < o->np; ++j) {
      double x = i * o->h + (1.0 + o->xr[j]) * 0.5 * o->h;
      u[(size_t)i * o->np + j] = sin(x - o->c * t);
    }
}

/* advection_1d.h:148-196 (alpha = 0: upwind) */
void orc1d_rhs(orc1d* o, double t, const double* u, double* out) {
  int np = o->np, K = o->K;
  double c = o->c;
  for (int i = 0; i <= K; ++i) {
    double a = i > 0 ? u[(size_t)i * np - 1] : -sin(2.0 * M_PI * t);
    double b = i < K ? u[(size_t)i * np] : u[(size_t)i * np - 1];
    o->flux[i] = c * 0.5 * (a + b) + c * 0.5 * (1.0 - 0.0) * (a - b);
  }
  double in[ORC_MAX_ORDER + 1], ov[ORC_MAX_ORDER + 1];
  for (int k = 0; k < K; ++k) {
    size_t off = (size_t)k * np;
    gemv(np, np, o->D, -c, u + off, 0.0, out + off);
    for (int j = 0; j < np; ++j) { in[j] = 0.0; ov[j] = 0.0; }
    in[0] = o->flux[k] - c * u[off];
    in[np - 1] = c * u[off + np - 1] - o->flux[k + 1];
    gemv(np, np, o->L, 1.0, in, 1.0, ov);
    for (int j = 0; j < np; ++j) out[off + j] += ov[j];
  }
}

/* explicit_runge_kutta.h:33-51 with axpy_n (axpy.h:112-122) */
void orc1d_rk4_step(orc1d* o, double t, double dt, double* u) {
  size_t n = (size_t)o->K * o->np;
  double **w = o->w;
  orc1d_rhs(o, t, u, w[1]);
  axpy_n(0.5 * dt, w[1], n, u, w[0]);
  orc1d_rhs(o, t + 0.5 * dt, w[0], w[2]);
  axpy_n(0.5 * dt, w[2], n, u, w[0]);
  orc1d_rhs(o, t + 0.5 * dt, w[0], w[3]);
  axpy_n(dt, w[3], n, u, w[0]);
  orc1d_rhs(o, t + dt, w[0], w[4]);
  axpy_n(2.0, w[2], n, w[1], w[0]);
  axpy_n(2.0, w[3], n, w[4], w[1]);
  axpy_n(dt / 6.0, w[0], n, u, w[2]);
  axpy_n(dt / 6.0, w[1], n, w[2], u);
}
