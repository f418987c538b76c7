// stokes.cu -- one time step of the Stokes example's dual-splitting scheme on
// the GPU (C ABI: dgc_stokes_*), examples/stokes_2d/stokes_2d.h:342-423:
//
//   u~ = (4 u^n - u^(n-1)) / 3                                (BDF2 extrapolation)
//   pressure:   A_N p = 1.5/dt div(u~) + (Neumann data 2 hp)  (all-Neumann laplace_2d)
//   projection: u~ -= 2 dt / 3 grad p
//   viscous:    (A_D - 1.5/dt I) u^(n+1) = -1.5/dt u~ + (Dirichlet data), per component
//
// The reference's boundary objects become per-node arrays over the boundary
// face nodes (the caller evaluates the example's analytic functions at
// dgc_boundary_nodes).  The pressure Neumann data hp (eq. 18 of Fehn et al.
// 2017, formed as in stokes_2d.h:191-269) is computed here on the boundary
// cells: the curl-curl term of u^n and u^(n-1) with the strong Dr, Ds, plus
// the caller's dg/dt dotted with the face normal.  Where the reference
// assembles A column by column and factors it with cuSOLVER's host LU
// (stokes_2d.h:424-526), both solves run the block-Jacobi PCG of the laplace
// handles (mixed FP32 / FP64 refinement by default, to a tight FP64
// residual): the pressure system as the all-Neumann SPD form with its
// constant null space projected out (p returned with zero mean; the
// reference's LU leaves that constant to its pivoting, and only grad p enters
// the velocity), the viscous systems as the Dirichlet SPD form shifted by
// 1.5/dt J M.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>

#include "common.cuh"
#include "dgc_gb300.h"
#include "dgc_internal.hpp"

struct dgc_stokes_s {
  dgc_handle vel = nullptr;   // all-Dirichlet laplace, tau = 1 (laplace_2d's penalty)
  dgc_handle pres = nullptr;  // all-Neumann laplace, tau = 1
  size_t n = 0;               // K * NpP
  double* ut[2] = {};         // u~ components
  double* work = nullptr;     // right-hand side being formed
  double* b = nullptr;        // -J M rhs
  double* grad[2] = {};       // grad p
  double* p = nullptr;        // pressure (kept: warm start of the next step)
  double* h2 = nullptr;       // 2 hp per boundary node
  // the FP64 residual floor of the singular pressure system is ~ eps cond(S_N), which grows as h^-2
  dgc_solve_opts opts{DGC_SOLVE_MIXED_IR, 1e-10, 200000, 1e-4, 0, 1};
};

namespace dgk {

// ut = (4 u - u_prev) / 3 for both components (stokes_2d.h:394-405)
__global__ void k_stokes_bdf2(size_t n, const double* __restrict__ ux0, const double* __restrict__ uy0,
                              const double* __restrict__ ux1, const double* __restrict__ uy1,
                              double* __restrict__ utx, double* __restrict__ uty) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    utx[i] = (ux1[i] * 4.0 - ux0[i]) / 3.0;
    uty[i] = (uy1[i] * 4.0 - uy0[i]) / 3.0;
  }
}

// y = a x, or y += a x when acc (y may be x: scaled in place)
__global__ void k_stokes_scal(size_t n, double a, const double* x, double* y, int acc) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    y[i] = acc ? y[i] + a * x[i] : a * x[i];
}

// Pressure Neumann data on the boundary cells, one CTA of 64 threads each
// (stokes_2d.h:191-269):
//   c = curl u^(n-1) - 2 curl u^n,  curl u = Dx uy - Dy ux,
//   h2[b] = 2 hp[b],  hp = (dg/dt).n + (Dy c) nx - (Dx c) ny   at boundary node b,
// the reference's exterior_grad_n(x, y, 0) = 2 hp.  Strong-form Dr, Ds
// (transposed: DrT[j Np + i] = Dr_ij), geometry records as in the RHS kernels.
template <int N>
__global__ void __launch_bounds__(64) k_stokes_hp(const int* __restrict__ cells, const int4* __restrict__ nbr,
                                                  const double* __restrict__ geom, const double* __restrict__ mats,
                                                  const double* __restrict__ ux0, const double* __restrict__ uy0,
                                                  const double* __restrict__ ux1, const double* __restrict__ uy1,
                                                  const double* __restrict__ dgdt_x,
                                                  const double* __restrict__ dgdt_y, double* __restrict__ h2) {
  using O = Order<N>;
  constexpr int Np = O::Np, NpP = O::NpP, Nfp = O::Nfp;
  constexpr int kD = (Np * Np + 3) / 4 * 4;
  __shared__ double c[Np];
  const int k = cells[blockIdx.x];
  const int t = threadIdx.x;
  const double* G = geom + (size_t)k * 16;
  const double rx = G[0], ry = G[1], sx = G[2], sy = G[3];
  const double* DrT = mats;
  const double* DsT = mats + kD;
  const size_t o = (size_t)k * NpP;
  for (int i = t; i < Np; i += blockDim.x) {
    double y0r = 0, y0s = 0, x0r = 0, x0s = 0, y1r = 0, y1s = 0, x1r = 0, x1s = 0;
    for (int j = 0; j < Np; ++j) {
      const double dr = DrT[j * Np + i], ds = DsT[j * Np + i];
      y0r += dr * uy0[o + j];
      y0s += ds * uy0[o + j];
      x0r += dr * ux0[o + j];
      x0s += ds * ux0[o + j];
      y1r += dr * uy1[o + j];
      y1s += ds * uy1[o + j];
      x1r += dr * ux1[o + j];
      x1s += ds * ux1[o + j];
    }
    const double curl0 = (rx * y0r + sx * y0s) - (ry * x0r + sy * x0s);
    const double curl1 = (rx * y1r + sx * y1s) - (ry * x1r + sy * x1s);
    c[i] = curl0 - 2.0 * curl1;
  }
  __syncthreads();
  const int4 n4 = nbr[k];
  for (int m = t; m < 3 * Nfp; m += blockDim.x) {
    const int f = m / Nfp, d = m - f * Nfp;
    const int nb = f == 0 ? n4.x : (f == 1 ? n4.y : n4.z);
    if (nb >= 0) continue;
    const int i = fmask<N>(f, d);
    double cr = 0, cs = 0;
    for (int j = 0; j < Np; ++j) {
      cr += DrT[j * Np + i] * c[j];
      cs += DsT[j * Np + i] * c[j];
    }
    const double dxc = rx * cr + sx * cs, dyc = ry * cr + sy * cs;
    const double nx = G[8 + f], ny = G[11 + f];
    const size_t b = (size_t)(-1 - nb) * Nfp + d;
    h2[b] = 2.0 * ((dgdt_x[b] * nx + dgdt_y[b] * ny) + (dyc * nx - dxc * ny));
  }
}

cudaError_t stokes_hp_launch(int N, int ncells, const int* cells, const int4* nbr, const double* geom,
                             const double* mats, const double* ux0, const double* uy0, const double* ux1,
                             const double* uy1, const double* gx, const double* gy, double* h2, cudaStream_t s) {
  if (ncells == 0) return cudaSuccess;
  switch (N) {
#define DGK_HP(n)                                                                                      \
  case n:                                                                                              \
    k_stokes_hp<n><<<ncells, 64, 0, s>>>(cells, nbr, geom, mats, ux0, uy0, ux1, uy1, gx, gy, h2); \
    break;
    DGK_HP(1) DGK_HP(2) DGK_HP(3) DGK_HP(4) DGK_HP(5) DGK_HP(6) DGK_HP(7) DGK_HP(8)
#undef DGK_HP
    default:
      return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace dgk

using namespace dgc;

namespace {

int grid(size_t n) { return (int)std::min<size_t>((n + 255) / 256, 4096); }

// prefix the solver's message with the system that failed
int solve_fail(int rc, const char* which) {
  const std::string m = std::string(which) + " solve: " + dgc_last_error();
  return set_error(rc, m.c_str());
}

int cuda_fail(cudaError_t e, const char* what) {
  const std::string m = std::string(what) + ": " + cudaGetErrorString(e);
  return set_error(DGC_ERR_CUDA, m.c_str());
}

}  // namespace

extern "C" int dgc_stokes_create(int num_vertices, const double* vertex_xy, int num_cells, const int32_t* cells,
                                 int order, dgc_stokes* out) {
  if (!out) return set_error(DGC_ERR_ARG, "null argument");
  *out = nullptr;
  auto* st = new dgc_stokes_s();
  dgc_problem_desc d{};
  d.physics = DGC_LAPLACE;
  d.order = order;
  d.precision = DGC_F64;
  d.tau = DGC_TAU_ONE;
  d.dirichlet = 1;
  int rc = dgc_create(num_vertices, vertex_xy, num_cells, cells, &d, &st->vel);
  if (rc == DGC_OK) {
    d.dirichlet = 0;
    rc = dgc_create(num_vertices, vertex_xy, num_cells, cells, &d, &st->pres);
  }
  if (rc != DGC_OK) {
    dgc_stokes_destroy(st);
    return rc;
  }
  st->n = (size_t)st->vel->K * st->vel->NpP;
  const size_t nb = std::max<size_t>(1, (size_t)st->vel->mesh.num_bfaces * st->vel->Nfp);
  double** bufs[7] = {&st->ut[0], &st->ut[1], &st->work, &st->b, &st->grad[0], &st->grad[1], &st->p};
  for (double** q : bufs) {
    if (cudaMalloc(q, st->n * 8) != cudaSuccess || cudaMemset(*q, 0, st->n * 8) != cudaSuccess) {
      dgc_stokes_destroy(st);
      return set_error(DGC_ERR_CUDA, "stokes workspace allocation");
    }
  }
  if (cudaMalloc(&st->h2, nb * 8) != cudaSuccess || cudaMemset(st->h2, 0, nb * 8) != cudaSuccess) {
    dgc_stokes_destroy(st);
    return set_error(DGC_ERR_CUDA, "stokes workspace allocation");
  }
  *out = st;
  return DGC_OK;
}

extern "C" int dgc_stokes_destroy(dgc_stokes s) {
  if (!s) return DGC_OK;
  for (double* q : {s->ut[0], s->ut[1], s->work, s->b, s->grad[0], s->grad[1], s->p, s->h2}) cudaFree(q);
  dgc_destroy(s->vel);
  dgc_destroy(s->pres);
  delete s;
  return DGC_OK;
}

extern "C" int dgc_stokes_handles(dgc_stokes s, dgc_handle* velocity, dgc_handle* pressure) {
  if (!s) return set_error(DGC_ERR_ARG, "null handle");
  if (velocity) *velocity = s->vel;
  if (pressure) *pressure = s->pres;
  return DGC_OK;
}

extern "C" int dgc_stokes_set_solver(dgc_stokes s, const dgc_solve_opts* opts) {
  if (!s || !opts) return set_error(DGC_ERR_ARG, "null argument");
  if (!(opts->rtol > 0.0) || opts->maxit <= 0 ||
      opts->mode < DGC_SOLVE_FP64_PCG || opts->mode > DGC_SOLVE_TWO_LEVEL_MIXED)
    return set_error(DGC_ERR_ARG, "bad solver settings");
  // two-level: the pressure system gets the coarse space (aggregates of 8 cells,
  // built once: the pressure handle's shift never changes)
  if (opts->mode == DGC_SOLVE_TWO_LEVEL || opts->mode == DGC_SOLVE_TWO_LEVEL_MIXED)
    if (int rc = dgc_coarse_build(s->pres, 8, nullptr)) return rc;
  s->opts = *opts;
  return DGC_OK;
}

extern "C" int dgc_stokes_step(dgc_stokes s, const double* ux_prev, const double* uy_prev, const double* ux,
                               const double* uy, double dt, const dgc_stokes_bc* bc, double* ux_out,
                               double* uy_out, double* p_out, dgc_solve_stats* stats, void* stream) {
  if (!s || !ux_prev || !uy_prev || !ux || !uy || !bc || !ux_out || !uy_out)
    return set_error(DGC_ERR_ARG, "null argument");
  if (!bc->ut_x || !bc->ut_y || !bc->dgdt_x || !bc->dgdt_y || !bc->g_x || !bc->g_y)
    return set_error(DGC_ERR_ARG, "missing boundary data");
  if (!(dt > 0.0)) return set_error(DGC_ERR_ARG, "dt must be > 0");
  if (ux_out == uy_out || ux_out == ux || ux_out == uy || uy_out == ux || uy_out == uy)
    return set_error(DGC_ERR_ARG, "outputs must not alias u^n or each other");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const size_t n = s->n;
  dgc_handle vel = s->vel, pres = s->pres;
  dgc_solve_stats S{}, acc{};
  acc.converged = 1;
  auto accum = [&]() {
    acc.iterations += S.iterations;
    acc.inner_iterations += S.inner_iterations;
    acc.outer_iterations += S.outer_iterations;
    acc.seconds += S.seconds;
    acc.final_relres = std::max(acc.final_relres, S.final_relres);
    acc.converged &= S.converged;
  };
  auto last = [](const char* what) {
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? DGC_OK : cuda_fail(e, what);
  };
  // stage 1: u~
  dgk::k_stokes_bdf2<<<grid(n), 256, 0, st>>>(n, ux_prev, uy_prev, ux, uy, s->ut[0], s->ut[1]);
  if (int rc = last("BDF2 extrapolation")) return rc;
  // stage 2a, pressure (stokes_2d.h:342-360): work = 1.5/dt div(u~) with the u~ boundary data
  // (u+ = ut - u-), then the Neumann data 2 hp as apply_inhomogeneous_as_rhs adds it
  if (int rc = dgc_div_apply(pres, s->ut[0], s->ut[1], s->work, bc->ut_x, bc->ut_y, -1.0, st)) return rc;
  dgk::k_stokes_scal<<<grid(n), 256, 0, st>>>(n, 1.5 / dt, s->work, s->work, 0);
  const int* bcells = nullptr;
  int nbc = 0;
  if (int rc = ipdg_boundary_cells(pres, &bcells, &nbc)) return rc;
  cudaError_t e = dgk::stokes_hp_launch(pres->N, nbc, bcells, reinterpret_cast<const int4*>(pres->d_nbr),
                                        pres->d_kgeom64, static_cast<const double*>(pres->d_mats64[1]), ux_prev,
                                        uy_prev, ux, uy, bc->dgdt_x, bc->dgdt_y, s->h2, st);
  if (e != cudaSuccess) return cuda_fail(e, "pressure boundary data");
  if (int rc = dgc_laplace_bc_rhs(pres, nullptr, s->h2, s->work, st)) return rc;
  // A_N p = work  <=>  S_N p = -J M work
  if (int rc = dgc_mass_apply(pres, s->work, s->b, st)) return rc;
  dgk::k_stokes_scal<<<grid(n), 256, 0, st>>>(n, -1.0, s->b, s->b, 0);
  if (int rc = last("pressure right-hand side")) return rc;
  if (int rc = dgc_pcg_solve(pres, s->b, s->p, &s->opts, &S, st)) return solve_fail(rc, "pressure");
  accum();
  // stage 2b, projection (stokes_2d.h:362-371): u~ -= 2 dt / 3 grad p, exterior p+ = p-
  if (int rc = dgc_grad_apply(pres, s->p, s->grad[0], s->grad[1], nullptr, 1.0, st)) return rc;
  dgk::k_stokes_scal<<<grid(n), 256, 0, st>>>(n, -2.0 * dt / 3.0, s->grad[0], s->ut[0], 1);
  dgk::k_stokes_scal<<<grid(n), 256, 0, st>>>(n, -2.0 * dt / 3.0, s->grad[1], s->ut[1], 1);
  if (int rc = last("projection")) return rc;
  // stage 3, viscous (stokes_2d.h:373-390): (A_D - 1.5/dt I) u = -1.5/dt u~ + data
  //   <=>  (S_D + 1.5/dt J M) u = -J M (-1.5/dt u~ + data)
  if (int rc = dgc_laplace_set_shift(vel, 1.5 / dt)) return rc;
  // the viscous systems are well conditioned (shifted by 1.5/dt J M): block-Jacobi
  // refinement, also when the pressure solve is two-level
  dgc_solve_opts vo = s->opts;
  if (vo.mode == DGC_SOLVE_TWO_LEVEL || vo.mode == DGC_SOLVE_TWO_LEVEL_MIXED) vo.mode = DGC_SOLVE_MIXED_IR;
  const double* gdir[2] = {bc->g_x, bc->g_y};
  double* uo[2] = {ux_out, uy_out};
  for (int c = 0; c < 2; ++c) {
    dgk::k_stokes_scal<<<grid(n), 256, 0, st>>>(n, -1.5 / dt, s->ut[c], s->work, 0);
    if (int rc = last("viscous right-hand side")) return rc;
    if (int rc = dgc_laplace_bc_rhs(vel, gdir[c], nullptr, s->work, st)) return rc;
    if (int rc = dgc_mass_apply(vel, s->work, s->b, st)) return rc;
    dgk::k_stokes_scal<<<grid(n), 256, 0, st>>>(n, -1.0, s->b, s->b, 0);
    // initial guess: u~ after the projection
    e = cudaMemcpyAsync(uo[c], s->ut[c], n * 8, cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return cuda_fail(e, "viscous initial guess");
    if (int rc = dgc_pcg_solve(vel, s->b, uo[c], &vo, &S, st)) return solve_fail(rc, c ? "viscous y" : "viscous x");
    accum();
  }
  if (p_out) {
    e = cudaMemcpyAsync(p_out, s->p, n * 8, cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return cuda_fail(e, "pressure output");
  }
  if (stats) *stats = acc;
  return DGC_OK;
}
