// setup.hpp -- host-side set-up of the nodal DG discretisation (FP64).
//
// Reference element (nodes, Vandermonde matrices, differentiation and lift
// operators), mesh topology and per-element geometric factors, computed once on
// the host and uploaded to the GPU by the C ABI (capi.cu).  This replaces the
// reference's host set-up path:
//   alpha_optimized_nodes_triangle (src/alpha_optimized_nodes_triangle.h:69-189),
//   reference_triangle (src/reference_triangle.h:45-114),
//   operator construction in advection_2d.h:78-101 / laplace_2d.h:88-112,
//   simple_triangular_mesh_2d::build_topology (src/mesh/simple_triangular_mesh_2d.h:151-217),
//   mapping_2d (src/mapping_2d.h:82-158) and simple_discretization_2d
//   (src/simple_discretization_2d.h:83-218).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace dgc {

constexpr int kMaxOrder = 8;

inline int num_nodes(int N) { return (N + 1) * (N + 2) / 2; }
inline int padded_nodes(int N) { return (num_nodes(N) + 3) / 4 * 4; }

// Node (i, j) of the triangle ordering (i: s-direction rows, j along r) has
// index i(N+1) - i(i-1)/2 + j.  Faces are walked counter-clockwise:
// face 0 = row i = 0, face 1 = the hypotenuse j = N - i, face 2 = column j = 0
// from i = N down to 0.
inline int face_node(int N, int f, int d) {
  if (f == 0) return d;
  if (f == 1) return d * (N + 1) - d * (d - 1) / 2 + N - d;
  const int i = N - d;
  return i * (N + 1) - i * (i - 1) / 2;
}

struct RefElement {
  int N = 0, Np = 0, Nfp = 0;
  std::vector<double> r, s;                 // node coordinates
  std::vector<double> V, Vr, Vs;            // Np x Np, row-major
  std::vector<double> M;                    // mass matrix (V V^T)^-1
  std::vector<double> Drw, Dsw, Lw;         // weak-form derivative / lift (advection, Maxwell)
  std::vector<double> Drs, Dss, Ls;         // strong-form derivative / lift (laplace)
};

// Normalised Jacobi polynomial P_n^(a,b)(x) and its derivative.
double jacobi(double a, double b, int n, double x);
double jacobi_grad(double a, double b, int n, double x);
// Legendre-Gauss-Lobatto points on [-1, 1], ascending.
std::vector<double> gauss_lobatto(int npts);
// Warp & blend nodes of Warburton's construction with the alpha-optimised table.
void warp_blend_nodes(int N, std::vector<double>& r, std::vector<double>& s);
bool build_ref_element(int N, RefElement& out, std::string& err);

// Small dense helpers (row-major).
std::vector<double> matmul(const std::vector<double>& A, const std::vector<double>& B, int m, int k, int n);
std::vector<double> transpose(const std::vector<double>& A, int m, int n);
bool invert(const std::vector<double>& A, int n, std::vector<double>& inv);

// Per-element geometry record (FP64), kGeomStride doubles per element.
enum GeomSlot : int {
  G_RX = 0, G_RY = 1, G_SX = 2, G_SY = 3, G_J = 4,
  G_FJ0 = 5,   // faceJ of faces 0..2 at 5, 6, 7
  G_NX0 = 8,   // outward normal x of faces 0..2 at 8, 9, 10
  G_NY0 = 11,  // outward normal y of faces 0..2 at 11, 12, 13
  G_TAU0 = 14, // laplace penalty of face 0 ... stored in a separate array (see MeshData::tau)
};
constexpr int kGeomStride = 16;

// Geometry record read by the stage kernels, stored in the kernel's own
// arithmetic type (FP64 or FP32).  Slots 0-3 and 5-13 are those of the FP64
// record; slot 4 holds -1/J (the lift scale) and slot 14 holds -J (the mass
// scale of the SPD form), so that an FP32 kernel performs no FP64 arithmetic.
enum KernelGeomSlot : int { KG_NEG_INV_J = 4, KG_NEG_J = 14 };

template <typename R>
std::vector<R> kernel_geometry(const std::vector<double>& geom, int K) {
  std::vector<R> g((size_t)K * kGeomStride, R(0));
  for (int k = 0; k < K; ++k) {
    const double* s = &geom[(size_t)k * kGeomStride];
    R* d = &g[(size_t)k * kGeomStride];
    for (int i = 0; i < 14; ++i) d[i] = (R)s[i];
    d[KG_NEG_INV_J] = (R)(-1.0 / s[G_J]);
    d[KG_NEG_J] = (R)(-s[G_J]);
  }
  return g;
}

struct MeshData {
  int K = 0, nv = 0, N = 0, Np = 0, Nfp = 0;
  std::vector<double> vx, vy;
  std::vector<int32_t> cells;      // K x 3
  std::vector<double> geom;        // K x kGeomStride
  // neighbour of face f of element k: (kn << 2 | fn) for an interior face,
  // -(1 + b) for the b-th boundary face (boundary faces numbered in element,
  // then face order, as the reference's fill_boundary_nodes does).
  std::vector<int32_t> nbr;        // K x 4 (4th unused)
  int num_bfaces = 0;
  std::vector<double> bxy;         // boundary face nodes: num_bfaces x Nfp x 2
  std::vector<double> tau;         // K x 4 laplace penalty per face ((N+1)^2 / h_f)
  double min_edge = 0.0;           // shortest edge length
  double min_altitude = 0.0;       // smallest triangle altitude
};

// gpu_topology: match the half-edges on the current GPU (gpu_match_half_edges)
// instead of sorting them on the host; the results are identical.
bool build_mesh(const double* vxy, int nv, const int32_t* cells, int K, const RefElement& re,
                MeshData& out, std::string& err, bool gpu_topology = false);

// The same MeshData from the reference's flattened arrays
// (simple_discretization_2d::fill_cell_mappings / fill_cell_interfaces /
// fill_boundary_nodes / fill_outward_normals, src/simple_discretization_2d.h:
// 112-218): the geometry is taken as given; boundary faces are the faces that
// map to their own cell, with the running boundary-node offset in nb_face.
// No vertex coordinates or connectivity (vx, vy, cells stay empty).
bool build_mesh_from_arrays(int K, const RefElement& re, const double* invJ, const double* J, const double* faceJ,
                            const int32_t* nb_cell, const int32_t* nb_face, int num_boundary_nodes, const double* bx,
                            const double* by, const double* nx, const double* ny, MeshData& m, std::string& err);
// the laplace penalty per face from the geometry and neighbours of m
void fill_penalty(MeshData& m, const RefElement& re);

// twin[3 k + f] = (k' << 2 | f') of the twin half-edge, or -1 on the boundary
// (csrc/topology.cu)
bool gpu_match_half_edges(const int32_t* cells, int K, std::vector<int32_t>& twin, std::string& err);

}  // namespace dgc
