/*
 * dgc_oracle.h -- CPU restatement of hsongxa/dg-on-cuda's nodal-DG hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA product:
 * only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / reference
 * legs may load it.  The product library never links or calls it.
 *
 * Every routine restates the reference algorithm it cites (file:line in the
 * reference project) in plain serial C, in the reference's operation order, so
 * that results agree with the reference's USE_CPU_ONLY build to rounding.
 * Where the reference hard-codes something a workload needs generalised
 * (advection velocity, TE Maxwell, LSERK4, penalty tau, orders 7 and 8) the
 * generalisation is stated next to the routine.
 *
 * Parity pin: tests/golden/ holds outputs of the reference's own CPU code
 * (compiled from its sources by oracle/Makefile into oracle/_ref/) on small
 * meshes; tests check this restatement against them.  Orders 7 and 8 have no
 * reference counterpart (its Gauss-Lobatto table stops at 7 points), so they
 * are validated by convergence only ("parity unpinned" for N = 7, 8).
 *
 * Layouts: all state vectors here use the reference CPU layout
 * q[field][cell][node]  (field-major, then cell-major, node fastest).
 */
#ifndef DGC_ORACLE_H
#define DGC_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_MAX_ORDER 8
#define ORC_MAX_NP 45
#define ORC_MAX_NFP 9

/* problems (right-hand sides) */
enum { ORC_ADVECTION = 0, ORC_MAXWELL_TM = 1, ORC_MAXWELL_TE = 2 };
/* advection inflow boundary values = the exact translated solution */
enum { ORC_BC_SINSIN = 0, ORC_BC_GAUSS = 1, ORC_BC_ZERO = 2 };
/* operator matrices: weak form (advection/Maxwell) or strong form (laplace) */
enum { ORC_WEAK = 0, ORC_STRONG = 1 };

typedef struct orc_problem {
  int kind;         /* ORC_ADVECTION / ORC_MAXWELL_TM / ORC_MAXWELL_TE */
  double ax, ay;    /* advection velocity */
  int bc;           /* advection boundary kind */
  double gx0, gy0, gw; /* gaussian pulse centre and width: exp(-((x-x0)^2+(y-y0)^2)/w) */
} orc_problem;

typedef struct orc orc;

/* 1D / reference-element building blocks */
double orc_jacobi_p(double alpha, double beta, int n, double x);
double orc_jacobi_dp(double alpha, double beta, int n, double x);
int orc_gl_points(int npts, double* x);
int orc_nodes(int N, double* r, double* s);
int orc_face_nodes(int N, int face, int* idx);
int orc_vandermonde(int N, double* V);
int orc_grad_vandermonde(int N, double* Vr, double* Vs);
int orc_face_vandermonde(int N, int face, double* fV);
int orc_operators(int N, int form, double* Dr, double* Ds, double* L, double* M);
int orc_mat_inverse(int n, const double* A, double* Ainv);

/* mesh + discretisation */
orc* orc_create(int N, int nv, const double* vxy, int K, const int32_t* cells);
void orc_destroy(orc* o);
int orc_num_boundary_nodes(const orc* o);
/* arrays in the reference's flattened form (simple_discretization_2d.h:112-218) */
void orc_fill_cell_mappings(const orc* o, double* invJ, double* J, double* faceJ);
void orc_fill_cell_interfaces(const orc* o, int32_t* cells, int32_t* faces);
void orc_fill_boundary_nodes(const orc* o, double* bx, double* by);
void orc_fill_outward_normals(const orc* o, double* nx, double* ny);
void orc_node_xy(const orc* o, double* x, double* y);  /* [cell][node] */

/* semi-discrete operators and time integrators (state layout [f][k][j]) */
int orc_num_fields(const orc_problem* p);
void orc_rhs(orc* o, const orc_problem* p, double t, const double* q, double* out);
void orc_rk4_step(orc* o, const orc_problem* p, double t, double dt, double* q);
void orc_lserk4_step(orc* o, const orc_problem* p, double t, double dt, double* q, double* res);
double orc_run(orc* o, const orc_problem* p, int scheme, double t0, double dt, int nsteps, double* q);
void orc_lserk4_coeffs(double* a, double* b, double* c);
void orc_exact(orc* o, const orc_problem* p, double t, double* q);

/* laplace_2d: strong-form LDG/IPDG apply, all boundary faces Dirichlet (dirichlet=1)
 * or all Neumann (dirichlet=0); tau_mode 0 = reference tau = 1, tau_mode 1 = per-face
 * tau = (N+1)^2 / h_f with h_f the smaller altitude onto the face. */
void orc_laplace_apply(orc* o, int dirichlet, int tau_mode, const double* u, double* out);
/* laplace_2d with a condition type per boundary node (bdir[b] != 0: Dirichlet)
 * and the boundary-data contribution apply_inhomogeneous_as_rhs adds */
void orc_laplace_apply_bc(orc* o, const uint8_t* bdir, int tau_mode, const double* u, double* out);
void orc_laplace_bc_rhs(orc* o, const uint8_t* bdir, int tau_mode, const double* g, const double* h,
                        double* out);
/* out += the jumps of the lifted Dirichlet data that apply_inhomogeneous_as_rhs
 * leaves out (the consistent boundary-data term is bc_rhs + bc_jump) */
void orc_laplace_bc_jump(orc* o, const uint8_t* bdir, const double* g, double* out);
/* SPD form S u = -blockdiag(J_k M) A u, and its diagonal blocks (K x Np x Np) */
void orc_spd_apply(orc* o, int tau_mode, const double* u, double* out);
void orc_spd_diag_blocks(orc* o, int tau_mode, double* blocks);
void orc_mass_apply(orc* o, const double* f, double* out);
/* weak-form gradient / divergence with central fluxes (grad_2d, div_2d);
 * boundary exterior value g[b] + sign * interior at boundary node b (g may be NULL) */
void orc_grad(orc* o, const double* u, const double* g, double sign, double* gx, double* gy);
void orc_div(orc* o, const double* ux, const double* uy, const double* gx, const double* gy, double sign,
             double* out);
int orc_pcg(orc* o, int tau_mode, const double* b, double* x, double rtol, int maxit,
            double* final_relres);

/* 1D advection (examples/advection_1d/advection_1d.h) */
typedef struct orc1d orc1d;
orc1d* orc1d_create(int K, int N);
void orc1d_destroy(orc1d* o);
void orc1d_operators(const orc1d* o, double* D, double* L);
void orc1d_node_x(const orc1d* o, double* x);
void orc1d_exact(const orc1d* o, double t, double* u);
void orc1d_rhs(orc1d* o, double t, const double* u, double* out);
void orc1d_rk4_step(orc1d* o, double t, double dt, double* u);

#ifdef __cplusplus
}
#endif
#endif
