/*
 * dgc_gb300.h -- C ABI of the GB300 (sm_103a) nodal-DG hot path.
 *
 * A drop-in for the GPU path of hsongxa/dg-on-cuda on 2D triangle meshes:
 * the device discretisation and operators (src/d_simple_discretization_2d.cuh,
 * examples/<example>/d_<example>.cuh), their launchers (src/device_SemiDiscOp_wrapper.cuh,
 * src/kernel_adapter.cuh), the time integrator (src/explicit_runge_kutta.h,
 * src/k_axpy.cuh) and the laplace_2d IPDG operator (src/laplace_2d.h).
 *
 * Conventions
 *  - Every function returns DGC_OK (0) or a negative dgc_status; no C++
 *    exception crosses this boundary.  dgc_last_error() gives a message for the
 *    calling thread's last failure.
 *  - State vectors are caller-owned device buffers in the native layout
 *    q[cell][field][NpP] (NpP = Np rounded up to a multiple of 4), 16-byte
 *    aligned, in the handle's precision (double for DGC_F64, float for DGC_F32).
 *    dgc_info.state_len gives the element count.  Padding entries are carried
 *    along and never used.  dgc_to_native / dgc_from_native convert from / to
 *    the reference's layouts.
 *  - `stream` is a cudaStream_t (NULL = legacy default stream).  All calls are
 *    asynchronous on that stream unless stated otherwise.
 *  - Geometry, connectivity and operator matrices are owned by the handle.
 */
#ifndef DGC_GB300_H
#define DGC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct dgc_handle_s* dgc_handle;

typedef enum dgc_status {
  DGC_OK = 0,
  DGC_ERR_ARG = -1,          /* invalid argument (null / misaligned pointer, bad enum, aliasing) */
  DGC_ERR_MESH = -2,         /* mesh rejected (out-of-range index, clockwise or degenerate cell, non-conforming) */
  DGC_ERR_CUDA = -3,         /* a CUDA runtime call failed */
  DGC_ERR_UNSUPPORTED = -4,  /* operation not defined for this handle (physics / precision) */
  DGC_ERR_DEVICE = -5,       /* a kernel reported a device-side error (bounded wait expired) */
  DGC_ERR_NOT_CONVERGED = -6 /* iterative solver stopped before reaching its tolerance */
} dgc_status;

typedef enum dgc_physics {
  DGC_ADVECTION = 0,   /* u_t + a.grad u = 0, upwind flux (examples/advection_2d/advection_2d.h:156-258) */
  DGC_MAXWELL_TM = 1,  /* (Hx, Hy, Ez), PEC walls (examples/maxwell_2d/maxwell_2d.h:178-311) */
  DGC_MAXWELL_TE = 2,  /* (Ex, Ey, Hz), PEC walls: E+ = -E-, Hz+ = Hz- */
  DGC_LAPLACE = 3      /* strong-form LDG/IPDG laplace_2d (src/laplace_2d.h:130-251) */
} dgc_physics;

/* DGC_F32C (advection / Maxwell handles): FP32 arithmetic with the state
 * carried as a compensated pair hi + lo of FP32 values.  A state buffer holds
 * 2 x state_len floats (the hi vector, then the lo vector; 8 bytes per entry
 * in all); residual registers are plain FP32 vectors of state_len floats
 * (a buffer of the state's size also serves).  The stage kernel evaluates the
 * strong form with jump-based surface terms, so the round-off floor of long
 * runs sits well below that of DGC_F32 (no reference counterpart: the
 * reference runs FP64 only).  dgc_to_native / dgc_from_native take and give
 * FP64 arrays in the reference layouts for these handles.  Classical RK4,
 * axpy, batches and grad / div are not offered for them. */
typedef enum dgc_precision { DGC_F64 = 0, DGC_F32 = 1, DGC_F32C = 2 } dgc_precision;

/* advection inflow values: the exact translated solution */
typedef enum dgc_bc {
  DGC_BC_SINSIN = 0, /* sin(pi(x+1-ax t)) sin(pi(y+1-ay t)) (advection_2d.h:152,191) */
  DGC_BC_GAUSS = 1,  /* exp(-((x-ax t-x0)^2 + (y-ay t-y0)^2)/w) */
  DGC_BC_ZERO = 2
} dgc_bc;

/* laplace penalty: 1 (reference, laplace_2d.h:244) or (N+1)^2/h_f per face */
typedef enum dgc_tau { DGC_TAU_ONE = 0, DGC_TAU_SCALED = 1 } dgc_tau;

typedef enum dgc_layout {
  DGC_LAYOUT_NATIVE = 0,
  DGC_LAYOUT_REF_CPU = 1, /* q[field][cell][node] (USE_CPU_ONLY, advection_2d.h:117-119) */
  DGC_LAYOUT_REF_GPU = 2  /* q[field][node][cell] (GPU build, advection_2d.h:120-123) */
} dgc_layout;

typedef enum dgc_operator {
  DGC_OP_DR_WEAK = 0, DGC_OP_DS_WEAK = 1, DGC_OP_LIFT = 2,
  DGC_OP_DR_STRONG = 3, DGC_OP_DS_STRONG = 4, DGC_OP_MASS = 5, DGC_OP_V = 6
} dgc_operator;

typedef struct dgc_problem_desc {
  int physics;        /* dgc_physics */
  int order;          /* N in [1, 8] */
  int precision;      /* dgc_precision */
  double ax, ay;      /* advection velocity */
  int bc;             /* dgc_bc (advection) */
  double gx0, gy0, gw;/* gaussian inflow data */
  int tau;            /* dgc_tau (laplace) */
  int dirichlet;      /* laplace: 1 = all boundary faces Dirichlet, 0 = all Neumann */
} dgc_problem_desc;

typedef struct dgc_info {
  int64_t num_cells;       /* K */
  int order, np, np_padded, nfp, num_fields;
  int precision;
  int64_t state_len;       /* K * num_fields * np_padded */
  int64_t scalar_bytes;    /* 8 or 4 */
  int num_boundary_faces;
  double min_edge, min_altitude;
  int rhs_tile, rhs_threads, rhs_smem, rhs_blocks_per_sm, sm_count;
} dgc_info;

/* Replaces create_simple_discretization_2d_on_device + the examples'
 * create_device_object (src/d_simple_discretization_2d.cuh:89-131,
 * examples/advection_2d/k_advection_2d.cu:45-100): builds the mesh topology,
 * geometry and operator matrices from vertex coordinates (x, y interleaved, as
 * simple_triangular_mesh_2d::fill_vertices takes them) and counter-clockwise
 * triangles (fill_connectivity), and uploads them to the current device.
 * The twin map (simple_triangular_mesh_2d::build_topology) is matched on the
 * GPU from 16384 cells (a hash of the edges' vertex pairs; the environment
 * variable DGC_GPU_TOPOLOGY_MIN sets the threshold) and by a host sort below;
 * both give the same result. */
int dgc_create(int num_vertices, const double* vertex_xy, int num_cells, const int32_t* cells,
               const dgc_problem_desc* desc, dgc_handle* out);

/* The same handle from the reference's flattened discretisation arrays, as
 * simple_discretization_2d's fill_cell_mappings (invJ [K][4] = rx, ry, sx, sy;
 * J [K]; faceJ [K][3]), fill_cell_interfaces (nb_cell, nb_face [K][3]: the
 * twin (cell, face), or for a boundary face the cell itself and the running
 * offset into the boundary nodes), fill_boundary_nodes (bx, by, the
 * num_boundary_nodes = boundary faces x (N+1) coordinates) and
 * fill_outward_normals (nx, ny [K][3]) produce them
 * (src/simple_discretization_2d.h:112-218), i.e. what the examples' host
 * code hands to create_device_object (examples/advection_2d/
 * k_advection_2d.cuh:32-50).  The geometry is used as given (bit for bit);
 * the interface map must be symmetric.  Such a handle has no vertex
 * coordinates: dgc_node_coordinates returns DGC_ERR_UNSUPPORTED. */
int dgc_create_from_arrays(int num_cells, const double* invJ, const double* J, const double* faceJ,
                           const int32_t* nb_cell, const int32_t* nb_face, int num_boundary_nodes, const double* bx,
                           const double* by, const double* nx, const double* ny, const dgc_problem_desc* desc,
                           dgc_handle* out);

/* Replaces destroy_simple_discretization_2d_on_device / destroy_device_object
 * (src/d_simple_discretization_2d.cuh:133-152). */
int dgc_destroy(dgc_handle h);

const char* dgc_last_error(void);
int dgc_get_info(dgc_handle h, dgc_info* out);

/* Physical coordinates of the nodes, host arrays [cell][node] (replaces the
 * position output of initialize_dofs, advection_2d.h:107-130). */
int dgc_node_coordinates(dgc_handle h, double* x, double* y);

/* Host copy of an operator matrix (row-major, FP64): Dr / Ds (Np x Np),
 * LIFT (Np x 3 Nfp), mass, Vandermonde (replaces reading m_Dr/m_Ds/m_L). */
int dgc_get_operator(dgc_handle h, int which, double* out);

/* Replace the operator matrices by caller-supplied FP64 ones (e.g. the
 * reference's own m_Dr, m_Ds, m_L, which k_advection_2d.cu:60-62 copies to
 * __constant__ memory).  form 0 = weak (advection/Maxwell), 1 = strong. */
int dgc_set_operators(dgc_handle h, int form, const double* Dr, const double* Ds, const double* L);

/* Layout conversion between the native layout and the reference's CPU or
 * GPU layout; both buffers on the device, in the handle's precision. */
int dgc_to_native(dgc_handle h, int src_layout, const void* src, void* dst, void* stream);
int dgc_from_native(dgc_handle h, int dst_layout, const void* src, void* dst, void* stream);

/* One evaluation of the semi-discrete operator: out = L_h(q, t).  Replaces
 * device_SemiDiscOp_wrapper<Op>::operator()(in, size, t, out)
 * (src/device_SemiDiscOp_wrapper.cuh:52-57).  q and out must not alias. */
int dgc_rhs(dgc_handle h, const void* q, double t, void* out, void* stream);

/* out = a x + y over the state vector.  Replaces k_axpy_auto / axpy_n
 * (src/k_axpy.cuh:47-55, src/axpy.h:112-122). */
int dgc_axpy(dgc_handle h, double a, const void* x, const void* y, void* out, void* stream);

/* One classical RK4 step in place on q, fused into 4 launches (replaces
 * dgc::rk4 with its 4 operator calls and 8 axpy launches,
 * src/explicit_runge_kutta.h:33-51).  work: 3 state vectors of scratch. */
int dgc_rk4_step(dgc_handle h, void* q, double t, double dt, void* const* work, void* stream);

/* dgc_rk4_step without caller work buffers, for callers that cannot allocate
 * device memory (code running under global-mode stream capture, real-time
 * loops that must not touch the allocator, plugins whose device memory is
 * owned by the host application).  No counterpart in the reference.  The
 * three work vectors live in a 6 MiB file-scope device array that every GPU
 * loading the library holds until exit; the state vector may be at most
 * 2 MiB (larger handles get DGC_ERR_ARG).  The first call on each device
 * looks up the array's device address (cudaGetSymbolAddress) with that device
 * current, so make it before any stream capture.  All calls share the array:
 * calls whose GPU work overlaps race on it. */
int dgc_rk4_step_static(dgc_handle h, void* q, double t, double dt, void* stream);

/* One low-storage RK4 step (Carpenter-Kennedy, 5 stages, each one fused
 * launch).  Reads q_in, writes the new state to q_out; q_in is used as
 * scratch and its contents are destroyed; res is the LSERK residual register
 * (zero it before the first step).  No reference counterpart (the reference
 * integrates with classical RK4 only). */
int dgc_lserk4_step(dgc_handle h, void* q_in, void* q_out, void* res, double t, double dt, void* stream);

/* One LSERK4 stage (stage in 0..4) as a single fused launch:
 * res = a_s res + dt L_h(q_in, t + c_s dt);  q_out = q_in + b_s res.
 * dgc_lserk4_step is these five stages with q_in / q_out alternating.
 * The stage launches use programmatic stream serialization: a stage's set-up
 * overlaps the end of the previous launch on the stream, and it waits for that
 * launch's completion before it touches its data, so the caller's stream
 * ordering is unchanged.  An event recorded between two stage launches cuts
 * the overlap.  DGC_STAGE_OVERLAP=0 in the environment turns it off. */
int dgc_lserk4_stage(dgc_handle h, int stage, const void* q_in, void* q_out, void* res, double t, double dt,
                     void* stream);

/* nsteps LSERK4 steps starting from qa at time t0; buffers ping-pong between
 * qa and qb; *final_state receives the buffer holding the result.  With
 * use_graph != 0 the launches are replayed from a captured CUDA graph. */
int dgc_lserk4_run(dgc_handle h, void* qa, void* qb, void* res, double t0, double dt, int nsteps,
                   int use_graph, void** final_state, void* stream);

/* ---- batches: many independent problems in one persistent launch --------- */

/* A batch over existing FP32 advection / Maxwell handles (any mix of orders
 * and mesh sizes).  Every LSERK4 stage of every instance runs in ONE launch:
 * persistent CTAs take work items (instance, run of tiles) from a device
 * queue ordered by decreasing cost, and evaluate them with the same tile code
 * as the handles' variant-0 stage kernel, so a batched step is bitwise equal
 * to per-instance dgc_lserk4_step calls with that variant.  The handles must
 * outlive the batch.  No reference counterpart (the reference integrates one
 * problem per process). */
typedef struct dgc_batch_s* dgc_batch;
int dgc_batch_create(const dgc_handle* handles, int num_instances, dgc_batch* out);
int dgc_batch_destroy(dgc_batch b);

/* One LSERK4 step of every instance i: q_in[i] -> q_out[i] (q_in[i] is scratch
 * afterwards), res[i] its residual register, at time t[i] with step dt[i]. */
int dgc_batch_lserk4_step(dgc_batch b, void* const* q_in, void* const* q_out, void* const* res, const double* t,
                          double const* dt, void* stream);

/* nsteps steps from qa[i] at time t0[i]; buffers ping-pong between qa and qb.
 * *final_in_qb is set to 1 when the results are in qb (odd step counts).  With
 * use_graph != 0 the step (5 stage launches and the per-instance clocks) is
 * replayed from a captured CUDA graph. */
int dgc_batch_lserk4_run(dgc_batch b, void* const* qa, void* const* qb, void* const* res, const double* t0,
                         const double* dt, int nsteps, int use_graph, int* final_in_qb, void* stream);

/* Kernels launched through the batch so far. */
int64_t dgc_batch_launch_count(dgc_batch b);

/* ---- grad_2d / div_2d (scalar-field handles: advection or laplace) ---------
 * Boundary data: at boundary face node b the exterior trace is
 *   u+ = g[b] + sign * u-,
 * the form of the reference's exterior_val callbacks (e.g. Dirichlet value
 * g_D: g = 2 g_D, sign = -1; zero jump: g = NULL, sign = +1).  Boundary nodes
 * are numbered by boundary face (element, then face order) and the face's
 * node order; g is an FP64 device array of num_boundary_faces * Nfp values. */

/* Coordinates of the boundary face nodes, host array [num_boundary_faces][Nfp][2]. */
int dgc_boundary_nodes(dgc_handle h, double* xy);

/* Weak-form gradient with the central flux: gx, gy = grad u (replaces
 * grad_2d::operator(), src/grad_2d.h:141-187, which writes gx over its input).
 * u, gx, gy: scalar fields in the handle's precision and native layout. */
int dgc_grad_apply(dgc_handle h, const void* u, void* gx, void* gy, const double* g, double sign,
                   void* stream);

/* Weak-form divergence with the central flux: out = div (ux, uy) (replaces
 * div_2d::operator(), src/div_2d.h:148-190); gx, gy the boundary data of the
 * two components (either may be NULL), one sign for both. */
int dgc_div_apply(dgc_handle h, const void* ux, const void* uy, void* out, const double* gx, const double* gy,
                  double sign, void* stream);

/* ---- laplace_2d (DGC_LAPLACE handles; scalar field, native layout) -------- */

/* out = A u, the discrete Laplacian with homogeneous boundary data (all faces
 * Dirichlet or all Neumann per desc->dirichlet).  Replaces
 * laplace_2d::operator() / apply_homogeneous (src/laplace_2d.h:121-251) and the
 * two-phase device operator launched through kernel_adapter::execute_phase
 * (src/kernel_adapter.cuh:77-82, examples/poisson_2d/d_poisson_2d.cuh:55-172).
 * u and out in the handle's precision. */
int dgc_laplace_apply(dgc_handle h, const void* u, void* out, void* stream);

/* Shift of the SPD form: S = -blockdiag(J_k M) (A - shift I) = S_0 + shift J M
 * for the Helmholtz-type systems (A - shift I) u = f of implicit diffusion
 * steps (examples/stokes_2d/stokes_2d.h:442-460 assembles A - 1.5/dt I).
 * Used by dgc_laplace_spd_apply, dgc_pcg_solve and the block-Jacobi blocks
 * (rebuilt when the shift changes); shift >= 0, default 0. */
int dgc_laplace_set_shift(dgc_handle h, double shift);

/* Boundary condition type per boundary face node (replaces the
 * is_dirichlet(x, y) callback of the reference's boundary objects,
 * src/laplace_2d.h:179, 233): flags[b] != 0 Dirichlet, 0 Neumann, boundary
 * nodes in dgc_boundary_nodes order (host array).  NULL returns to the
 * handle's uniform type (desc.dirichlet).  dgc_pcg_solve needs uniform
 * Dirichlet boundaries and refuses handles with per-node types. */
int dgc_laplace_set_bc_types(dgc_handle h, const uint8_t* flags);

/* out += the boundary-data contribution of apply_inhomogeneous_as_rhs
 * (src/laplace_2d.h:253-348): g[b] = exterior_val(x, y, 0) at Dirichlet nodes,
 * hn[b] = exterior_grad_n(x, y, 0) at Neumann nodes (FP64 device arrays, one
 * value per boundary node; NULL = 0); out in the handle's precision.
 * laplace_2d::operator() with boundary data (same file:121-128) is
 * dgc_laplace_apply minus this contribution. */
int dgc_laplace_bc_rhs(dgc_handle h, const double* g, const double* hn, void* out, void* stream);

/* What dgc_laplace_bc_rhs adds for Dirichlet data.  REFERENCE (default):
 * exactly apply_inhomogeneous_as_rhs, whose second pass adds the lifted data
 * q_d = -LIFT(n g faceJ / 2) / J only through boundary-face terms
 * (src/laplace_2d.h:310-348).  CONSISTENT: also the jumps of q_d across
 * interior faces and 2 q_d.n on Neumann faces, which apply_homogeneous has for
 * the same lift (same file:222-242); dgc_laplace_apply(u) minus this term is
 * then the affine operator of the scheme, exact on polynomials of degree <= N
 * with their own boundary data.  The two differ only for non-zero Dirichlet
 * data (the examples' Poisson problem has none; the Stokes example's
 * velocity solves do), and one extra launch over the boundary cells and their
 * neighbours. */
typedef enum dgc_bc_data_mode { DGC_BC_DATA_REFERENCE = 0, DGC_BC_DATA_CONSISTENT = 1 } dgc_bc_data_mode;
int dgc_laplace_set_bc_data_mode(dgc_handle h, int mode);

/* out = S u = -blockdiag(J_k M) A u: the mass-weighted form, symmetric
 * positive definite for Dirichlet problems. */
int dgc_laplace_spd_apply(dgc_handle h, const void* u, void* out, void* stream);

/* out = blockdiag(J_k M) f (FP64): turns nodal values of f into the right-hand
 * side of S u = M_J f for -laplace(u) = f. */
int dgc_mass_apply(dgc_handle h, const double* f, double* out, void* stream);

typedef enum dgc_solve_mode {
  DGC_SOLVE_FP64_PCG = 0, /* block-Jacobi PCG in FP64 */
  DGC_SOLVE_MIXED_IR = 1, /* FP32 block-Jacobi PCG inside FP64 iterative refinement */
  DGC_SOLVE_TWO_LEVEL = 2, /* FP64 PCG with M = Binv + P A_c^-1 P^T, the coarse space of
                              dgc_coarse_build (which must precede the solve), M applied
                              with FP32 blocks and smoothing; restarts from the true
                              residual; no counterpart in the reference */
  DGC_SOLVE_TWO_LEVEL_MIXED = 3 /* the same with S applied in FP32 inside each pass, each
                                   pass to inner_rtol, refined on the FP64 residual */
} dgc_solve_mode;

typedef struct dgc_solve_opts {
  int mode;           /* dgc_solve_mode */
  double rtol;        /* stop at ||b - S x||_2 <= rtol ||b||_2 (true FP64 residual) */
  int maxit;          /* total CG iteration budget */
  double inner_rtol;  /* mixed: relative tolerance of each FP32 inner solve (default 1e-4) */
  int max_outer;      /* mixed: refinement steps */
  int use_graph;      /* replay 3-iteration chunks from a CUDA graph */
} dgc_solve_opts;

typedef struct dgc_solve_stats {
  int iterations;       /* CG iterations (FP64 or FP32 inner, summed) */
  int outer_iterations; /* refinement steps (mixed) */
  int inner_iterations;
  int converged;
  double final_relres;  /* ||b - S x|| / ||b||, computed in FP64 */
  double seconds;       /* host wall time of the call (synchronises the stream) */
} dgc_solve_stats;

/* Solve S x = b with block-Jacobi preconditioned CG (b, x FP64 device
 * vectors, native layout; x holds the initial guess).  All-Neumann handles
 * without shift have the constants as null space: b is projected onto the
 * range (zero sum over the valid nodes) and x returned with zero mean.  No reference
 * counterpart: the reference assembles the matrix column by column and calls
 * cuSOLVER-Sp QR (examples/poisson_2d/main.cpp:130-223).  Returns
 * DGC_ERR_NOT_CONVERGED (with stats filled) if the tolerance is not met. */
int dgc_pcg_solve(dgc_handle h, const double* b, double* x, const dgc_solve_opts* opts, dgc_solve_stats* stats,
                  void* stream);

/* The block-Jacobi inverse blocks S_kk^-1 (FP64, K x Np x Np, device). */
int dgc_block_jacobi(dgc_handle h, double* blocks, void* stream);

/* ---- learned preconditioner (no reference counterpart) ---------------------
 * A message-passing network over element adjacency: per-element DOFs (NpP
 * values) -> width-W features; L layers h <- h + relu(Ws h + Wn sum_nbr h + b);
 * -> NpP outputs.  Weights are kept as FP32 masters and BF16 copies; every
 * contraction reads the BF16 weights and accumulates in FP32.  As a
 * preconditioner of the SPD form S (dirichlet laplace handles):
 *   M(r) = Binv r + (|r| / c) net(c r / |r|),   c = sqrt(K Np),
 * Binv the block-Jacobi inverse (c gives the input unit RMS per node); the
 * network is trained to predict (e - Binv r) c / |r| from pairs of residuals
 * r and errors e = x* - x. */
typedef struct dgc_mpnn_s* dgc_mpnn;
/* Initialisation from seed (width W = 64, layers L >= 1): Glorot-uniform
 * hidden weights, zero biases, zero output layer (M starts as block-Jacobi). */
int dgc_mpnn_create(dgc_handle h, int layers, uint64_t seed, dgc_mpnn* out);
int dgc_mpnn_destroy(dgc_mpnn m);
/* Number of parameters; get / set the FP32 master weights (BF16 copies follow). */
int64_t dgc_mpnn_num_params(dgc_mpnn m);
int dgc_mpnn_get_weights(dgc_mpnn m, float* host_out);
int dgc_mpnn_set_weights(dgc_mpnn m, const float* host_in);
/* Training loss over samples s with d_s = net(x_s) - t_s (padding nodes
 * excluded):
 *   DGC_MPNN_LOSS_ENERGY (default): mean_s d_s.S d_s / t_s.S t_s, S the SPD
 *     laplace form applied in FP32.  For t = (e - Binv r)/|r| this is the
 *     energy norm of the error left by one step x += M(r) from error e, which
 *     weights the components a local network can correct;
 *   DGC_MPNN_LOSS_L2: mean_s |d_s|^2 / |t_s|^2. */
enum { DGC_MPNN_LOSS_L2 = 0, DGC_MPNN_LOSS_ENERGY = 1 };
int dgc_mpnn_set_loss(dgc_mpnn m, int kind);
/* Activation of the hidden layers: DGC_MPNN_ACT_RELU (default) or
 * DGC_MPNN_ACT_LINEAR (no ReLU, and every bias set to and held at zero during
 * training).  The linear network is a fixed linear map of its input, and with
 * it the preconditioner's correction (|r|/c) net(c r/|r|) = net(r) is linear in
 * r, so flexible CG sees a fixed preconditioner. */
enum { DGC_MPNN_ACT_RELU = 0, DGC_MPNN_ACT_LINEAR = 1 };
int dgc_mpnn_set_activation(dgc_mpnn m, int kind);
/* Where the network's correction enters the preconditioner.
 * DGC_MPNN_CORR_ADDITIVE (default): M(r) = z0 + (|r|/c) net(c r/|r|).
 * DGC_MPNN_CORR_RESIDUAL: the network acts on what the rest leaves,
 *   M(r) = z0 + (|r'|/c) net(c r'/|r'|),  r' = r - S z0 (S in FP32),
 * with z0 = Binv r (+ the coarse term when dgc_mpnn_set_coarse is on); train it
 * on inputs r' c/|r'| and targets (e - z0) c/|r'|, the error left after z0,
 * which is S^-1 r'.  Costs one FP32 apply of S and one host round trip more
 * per application. */
enum { DGC_MPNN_CORR_ADDITIVE = 0, DGC_MPNN_CORR_RESIDUAL = 1 };
int dgc_mpnn_set_correction(dgc_mpnn m, int kind);
/* Loss and gradients on `samples` field pairs (device, FP32, native layout,
 * samples x K x NpP each): x the network inputs, t the targets.  grad_out
 * (device, num_params floats) receives d loss / d weights (may be NULL);
 * with lr > 0 one Adam step is applied afterwards (beta1 0.9, beta2 0.999,
 * eps 1e-8). */
int dgc_mpnn_train_step(dgc_mpnn m, const float* x, const float* t, int samples, float lr, float* loss,
                        float* grad_out, void* stream);
/* y = net(x) for one field (device FP32, K x NpP). */
int dgc_mpnn_forward(dgc_mpnn m, const float* x, float* y, void* stream);
/* z = M(r) (device FP64, native layout). */
int dgc_mpnn_precondition(dgc_mpnn m, const double* r, double* z, void* stream);

/* Two-level form of the learned preconditioner: with cells_per_aggregate > 0,
 * M(r) = Binv r + P A_c^-1 P^T r + (|r|/c) net(c r/|r|), the coarse space of
 * dgc_coarse_build on the network's handle (built here when missing; shared
 * by every network of the handle; its smoothing applies of S in FP32).  The network then learns the correction
 * that is left after both.  0 turns the coarse term off (the default). */
int dgc_mpnn_set_coarse(dgc_mpnn m, int cells_per_aggregate, void* stream);

/* ---- coarse space (two-level preconditioning of the SPD laplace form) ------
 * No counterpart in the reference.  Cells are grouped into aggregates of
 * about cells_per_aggregate face-connected cells (breadth-first, in cell
 * order; at most 8192 aggregates); P0 is constant on each aggregate, the
 * prolongation P = (I - omega Binv S) P0 is smoothed once with block Jacobi
 * (omega = 4 / (3 lambda_max(Binv S)), lambda_max from 20 power iterations
 * times 1.1), and A_c = P^T S P is the Galerkin coarse matrix of the SPD form
 * S (FP64 laplace handles with uniform boundary types; the shift at build
 * time), inverted once on the GPU.  All-Neumann handles without shift: A_c is
 * singular (P 1 = 1) and is used through a rank-one regularisation that acts
 * as its pseudo-inverse on zero-sum residuals.  Rebuilding with the same size
 * and shift is a no-op; a failed rebuild leaves the handle without one. */
int dgc_coarse_build(dgc_handle h, int cells_per_aggregate, void* stream);
/* z = P A_c^-1 P^T r (device FP64, native layout; z distinct from r).
 * precision DGC_F32 runs the two smoothing steps inside P and P^T (S and
 * Binv) in FP32 (what the two-level and learned preconditioners use);
 * DGC_F64 is exact. */
int dgc_coarse_apply(dgc_handle h, const double* r, double* z, int precision, void* stream);
/* The aggregate of each cell (host array of K), their count, the number of
 * colours used to assemble A_c and omega (any output may be NULL). */
int dgc_coarse_info(dgc_handle h, int32_t* agg, int* num_aggregates, int* num_colors, double* omega);
/* Truncated flexible CG (Notay's FCG(m)) on S x = b with M as the
 * preconditioner, to rtol on the true FP64 residual: each direction is
 * S-orthogonalised against the previous m, alpha = p.r / p.S p, and an
 * iteration whose M(r).r <= 0 takes the block-Jacobi direction instead.
 * The same options and statistics as dgc_pcg_solve; opts->max_outer is the
 * window m (1..8, 0 = 4); mode, inner_rtol and use_graph are ignored. */
int dgc_fpcg_solve(dgc_handle h, dgc_mpnn m, const double* b, double* x, const dgc_solve_opts* opts,
                   dgc_solve_stats* stats, void* stream);

/* Learned solve with block-Jacobi PCG as fallback and final check: dgc_fpcg_solve
 * for at most fcg_maxit iterations; if that has not reached opts->rtol,
 * dgc_pcg_solve (opts->mode: FP64 PCG or mixed refinement) continues from the
 * current iterate with the remaining budget.  Either way the result meets
 * rtol on the true FP64 residual or DGC_ERR_NOT_CONVERGED is returned.
 * *fell_back = 1 when the fallback ran; stats->iterations counts both parts,
 * stats->inner_iterations the flexible-CG part. */
int dgc_learned_solve(dgc_handle h, dgc_mpnn m, const double* b, double* x, const dgc_solve_opts* opts,
                      int fcg_maxit, dgc_solve_stats* stats, int* fell_back, void* stream);

/* ---- the 1D advection example (examples/advection_1d) ---------------------
 * u_t + c u_x = 0 on [0, 2 pi], c = 2 pi, K equal cells of N+1 Gauss-Lobatto
 * nodes, upwind flux, inflow u(0, t) = -sin(2 pi t), outflow extrapolation
 * (advection_1d.h:37-196).  State: device vector [cell][node] (the
 * reference's CPU layout), K (N+1) values in the handle's precision. */
typedef struct dgc_adv1d_s* dgc_adv1d;
/* Replaces advection_1d(numCells, order) and create_device_object
 * (examples/advection_1d/k_advection_1d.cu).  order in [1, 8]. */
int dgc_adv1d_create(int num_cells, int order, int precision, dgc_adv1d* out);
int dgc_adv1d_destroy(dgc_adv1d a);
/* min_elem_size() and wave_speed() of the reference class. */
int dgc_adv1d_info(dgc_adv1d a, double* min_elem_size, double* wave_speed);
/* Node positions, host array [cell][node] (initialize_dofs). */
int dgc_adv1d_node_x(dgc_adv1d a, double* x);
/* Host copy of m_D (which = 0) or m_L (which = 1), (N+1) x (N+1) row-major. */
int dgc_adv1d_get_operator(dgc_adv1d a, int which, double* out);
/* out = L_h(q, t) (advection_1d::operator()). */
int dgc_adv1d_rhs(dgc_adv1d a, const void* q, double t, void* out, void* stream);
/* One classical RK4 step in place on q in 4 fused launches (dgc::rk4 with
 * the operator and 8 axpy calls).  work: 3 state vectors of scratch. */
int dgc_adv1d_rk4_step(dgc_adv1d a, void* q, double t, double dt, void* const* work, void* stream);
int64_t dgc_adv1d_launch_count(dgc_adv1d a);

/* ---- the Stokes example's dual-splitting step (examples/stokes_2d) ---------
 * u_t = lap u - grad p, div u = 0 advanced by BDF2 dual splitting (Fehn et al.
 * 2017): u~ = (4 u^n - u^(n-1)) / 3; A_N p = 1.5/dt div u~ + Neumann data;
 * u~ -= 2 dt / 3 grad p; (A_D - 1.5/dt I) u^(n+1) = -1.5/dt u~ + Dirichlet
 * data, with the laplace_2d operator (tau = 1) on the pressure (all Neumann)
 * and the velocity (all Dirichlet).  Velocity and pressure are FP64 device
 * vectors in the native layout of a laplace handle (K x NpP).  The velocity
 * handle takes its Dirichlet data as the reference does (dgc_laplace_set_
 * bc_data_mode REFERENCE); with that term the example's scheme does not
 * converge to its analytic solution, with CONSISTENT on the velocity handle
 * (dgc_stokes_handles) it does. */
typedef struct dgc_stokes_s* dgc_stokes;
/* Boundary data, FP64 device arrays over the boundary face nodes in
 * dgc_boundary_nodes order (the reference's boundary objects evaluated there). */
typedef struct dgc_stokes_bc {
  const double* ut_x;   /* u_tilde_bc::exterior_val(x, y, 0): 2 (4 g(t^n) - g(t^(n-1))) / 3 */
  const double* ut_y;
  const double* dgdt_x; /* the dgdt term of pressure_bc's hp at t^(n+1) (stokes_2d.h:260-262; the
                           example's lamda g e^(-lamda t), i.e. -dg/dt) */
  const double* dgdt_y;
  const double* g_x;    /* u_x_bc / u_y_bc::exterior_val(x, y, 0): 2 g(t^(n+1)) */
  const double* g_y;
} dgc_stokes_bc;
/* Replaces stokes_2d(mesh, order) (examples/stokes_2d/stokes_2d.h:271-282):
 * two laplace handles on the mesh plus workspace.  order in [1, 8]. */
int dgc_stokes_create(int num_vertices, const double* vertex_xy, int num_cells, const int32_t* cells, int order,
                      dgc_stokes* out);
int dgc_stokes_destroy(dgc_stokes s);
/* The velocity (Dirichlet) and pressure (Neumann) laplace handles, owned by s:
 * node coordinates, layout conversion and boundary nodes come from them. */
int dgc_stokes_handles(dgc_stokes s, dgc_handle* velocity, dgc_handle* pressure);
/* Solver of the pressure and viscous systems (default: mixed refinement,
 * rtol 1e-10, maxit 200000).  The two-level modes build the coarse space on
 * the pressure handle (aggregates of 8 cells) and solve the pressure system
 * with it; the viscous systems then use mixed refinement.  The FP64 residual of the singular pressure
 * system stalls near 1e-16 cond(S), so tighter targets fail on fine meshes. */
int dgc_stokes_set_solver(dgc_stokes s, const dgc_solve_opts* opts);
/* One step t^n -> t^(n+1) = t^n + dt (advance_timestep, stokes_2d.h:393-423):
 * u_prev = u^(n-1), u = u^n; writes u^(n+1) to ux_out / uy_out (which may
 * alias u_prev, not u) and, when p_out is non-NULL, the zero-mean pressure.
 * stats sums the three solves (final_relres: the largest).  The reference
 * solves with a host sparse LU; here both systems run block-Jacobi PCG to
 * the solver's rtol. */
int dgc_stokes_step(dgc_stokes s, const double* ux_prev, const double* uy_prev, const double* ux, const double* uy,
                    double dt, const dgc_stokes_bc* bc, double* ux_out, double* uy_out, double* p_out,
                    dgc_solve_stats* stats, void* stream);

/* ---- files ------------------------------------------------------------------ */

/* The reference drivers' visualisation file (Advection2DDataFile.txt,
 * examples/advection_2d/main.cpp:164-174): "#         x         y         u",
 * one "x  y  u" line per node (15 significant digits), a blank line, then the
 * same block of `ref` under "#         x         y         reference solution"
 * (omitted when ref is NULL).  Host FP64 arrays of n nodes, e.g. one field in
 * the reference CPU layout with dgc_node_coordinates.  Needs no GPU. */
int dgc_write_data_file(const char* path, int64_t n, const double* x, const double* y, const double* u,
                        const double* ref);

/* Gmsh MSH 4 ASCII import (replaces gmsh_importer_exporter::
 * import_triangle_mesh_2d, src/mesh/gmsh_importer_exporter.h:49-167): the
 * triangles (element type 2) and node coordinates, node tags shifted by the
 * smallest tag, as dgc_create takes them.  Call with vertex_xy = cells = NULL
 * to get the counts; then with arrays whose capacities (vertices, cells) are
 * passed in *num_vertices / *num_cells.  Node tags must run contiguously in
 * file order (the reference assumes it; this reader checks). */
int dgc_msh_read(const char* path, int* num_vertices, double* vertex_xy, int* num_cells, int32_t* cells);
/* MSH 4.1 export (replaces export_triangle_mesh_2d, same file:191-213);
 * digits = significant digits of the coordinates, 0 = 6 as the reference
 * writes them (17 round-trips exactly). */
int dgc_msh_write(const char* path, int num_vertices, const double* vertex_xy, int num_cells, const int32_t* cells,
                  int digits);

/* State checkpoint: a header (discretisation, time t, FNV-1a checksum) and the
 * device state vector q in the native layout; synchronises the stream.  No
 * counterpart in the reference.  dgc_load_state rejects files written for
 * another discretisation or failing the checksum (DGC_ERR_ARG). */
int dgc_save_state(dgc_handle h, const char* path, const void* q, double t, void* stream);
int dgc_load_state(dgc_handle h, const char* path, void* q, double* t, void* stream);

/* Synchronise the handle's device status word: DGC_OK, or DGC_ERR_DEVICE if a
 * kernel recorded an error since the last call (the word is then cleared). */
int dgc_check_device_status(dgc_handle h, int* code);

/* Number of kernels this handle has launched (captured graph replays count
 * each kernel they contain). */
int64_t dgc_launch_count(dgc_handle h);

/* ---- tile-shape autotuning of the fused RHS kernel (no reference
 * counterpart: the reference takes grid and block sizes from argv,
 * examples/advection_2d/main.cpp:71-79) --------------------------------- */

/* Number of compiled tile-shape variants for this handle (>= 1). */
int dgc_num_variants(dgc_handle h);

/* Select variant v (0 <= v < dgc_num_variants). */
int dgc_set_variant(dgc_handle h, int v);

/* Time every variant with `reps` LSERK4-stage launches on this handle's mesh
 * (scratch buffers are allocated and freed inside) and select the fastest.
 * times_ms (optional, dgc_num_variants entries) receives the median time per
 * launch.  When times_ms is NULL and the file named by the environment
 * variable DGC_TUNE_CACHE holds a choice for this (GPU, physics, precision,
 * order, log2 K) key, that choice is applied without timing; new choices are
 * appended to that file.  Synchronises the stream. */
int dgc_autotune(dgc_handle h, int reps, double* times_ms, int* chosen, void* stream);

/* ---- host-only set-up queries (no GPU needed) ---------------------------- */

/* Reference-element nodes of order N (alpha_optimized_nodes_triangle::
 * node_positions, src/alpha_optimized_nodes_triangle.h:104-141). */
int dgc_ref_nodes(int order, double* r, double* s);

/* An operator matrix of order N, row-major FP64 (the m_Dr / m_Ds / m_L built
 * in examples/advection_2d/advection_2d.h:78-101 and src/laplace_2d.h:88-112). */
int dgc_ref_operator(int order, int which, double* out);

/* Mesh validation, topology and geometry on the host: geom [K][16] doubles
 * (rx, ry, sx, sy, J, faceJ[3], nx[3], ny[3], pad), nbr [K][4] int32
 * ((cell << 2 | face) of the twin face, or -(1 + b) for boundary face b, in
 * the order of simple_discretization_2d::fill_cell_interfaces,
 * src/simple_discretization_2d.h:136-162).  Any output may be NULL. */
int dgc_host_mesh(int num_vertices, const double* vertex_xy, int num_cells, const int32_t* cells, int order,
                  double* geom, int32_t* nbr, int* num_boundary_faces);

/* The handle's twin map, host array [K][4] in the dgc_host_mesh encoding. */
int dgc_mesh_neighbors(dgc_handle h, int32_t* nbr, int* num_boundary_faces);

#ifdef __cplusplus
}
#endif
#endif
