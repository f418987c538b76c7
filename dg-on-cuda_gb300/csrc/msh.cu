// msh.cu -- Gmsh MSH version 4 (ASCII) triangle meshes: import into the
// vertex / cell arrays dgc_create takes, and export (C ABI: dgc_msh_read,
// dgc_msh_write).  Host code.
//
// Reading follows gmsh_importer_exporter::import_triangle_mesh_2d
// (src/mesh/gmsh_importer_exporter.h:49-167): a $MeshFormat of version 4 or
// later, the $Nodes blocks (x, y of each node; z ignored), the triangles
// (element type 2) of the $Elements blocks with node tags shifted by the
// smallest node tag.  Where the reference assumes that the node tags run
// contiguously in file order, this reader checks it and rejects other files.
// Writing follows export_triangle_mesh_2d (same file:191-213): one node block
// and one triangle block, coordinates printed with `digits` significant digits
// (0: the 6 of a default C++ stream, as the reference writes them).
#include <cerrno>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "dgc_gb300.h"
#include "dgc_internal.hpp"

using namespace dgc;

namespace {

struct Tokens {
  const char* p;
  bool next_ll(long long* v) {
    char* end = nullptr;
    errno = 0;
    const long long x = std::strtoll(p, &end, 10);
    if (end == p || errno) return false;
    p = end;
    *v = x;
    return true;
  }
  // coordinates are parsed as long double and narrowed, as the reference's
  // std::stold does, so the same file gives the same doubles on the same host
  bool next_d(double* v) {
    char* end = nullptr;
    const long double x = std::strtold(p, &end);
    if (end == p) return false;
    p = end;
    *v = (double)x;
    return true;
  }
};

struct MshData {
  std::vector<double> xy;
  std::vector<int32_t> cells;
};

int mesh_err(const std::string& what) { return set_error(DGC_ERR_MESH, ("MSH: " + what).c_str()); }

bool find_section(std::ifstream& f, const char* name) {
  std::string line;
  while (std::getline(f, line))
    if (line.find(name) != std::string::npos) return true;
  return false;
}

int parse_msh(const char* path, MshData& out) {
  std::ifstream f(path);
  if (!f.is_open()) return set_error(DGC_ERR_ARG, "cannot open the MSH file");
  std::string line;
  if (!find_section(f, "$MeshFormat") || !std::getline(f, line)) return mesh_err("no $MeshFormat section");
  if (std::strtod(line.c_str(), nullptr) < 4.0) return mesh_err("version 4 or later required");
  if (!find_section(f, "$Nodes") || !std::getline(f, line)) return mesh_err("no $Nodes section");
  long long nblocks, nnodes, tmin, tmax;
  Tokens t{line.c_str()};
  if (!t.next_ll(&nblocks) || !t.next_ll(&nnodes) || !t.next_ll(&tmin) || !t.next_ll(&tmax) || nblocks < 0)
    return mesh_err("bad $Nodes header");
  if (nnodes != tmax - tmin + 1 || nnodes < 0 || nnodes > INT32_MAX)
    return mesh_err("node tags are not contiguous");
  out.xy.reserve(2 * (size_t)nnodes);
  long long expect = tmin;
  for (long long b = 0; b < nblocks; ++b) {
    long long dim, tag, param, n;
    if (!std::getline(f, line)) return mesh_err("truncated $Nodes");
    Tokens h{line.c_str()};
    if (!h.next_ll(&dim) || !h.next_ll(&tag) || !h.next_ll(&param) || !h.next_ll(&n) || n < 0)
      return mesh_err("bad node block header");
    for (long long i = 0; i < n; ++i) {
      long long nt;
      if (!std::getline(f, line)) return mesh_err("truncated node tags");
      Tokens tt{line.c_str()};
      if (!tt.next_ll(&nt) || nt != expect++) return mesh_err("node tags are not contiguous in file order");
    }
    for (long long i = 0; i < n; ++i) {
      double x, y;
      if (!std::getline(f, line)) return mesh_err("truncated node coordinates");
      Tokens c{line.c_str()};
      if (!c.next_d(&x) || !c.next_d(&y)) return mesh_err("bad node coordinates");
      out.xy.push_back(x);
      out.xy.push_back(y);
    }
  }
  if ((long long)out.xy.size() != 2 * nnodes) return mesh_err("node count differs from the $Nodes header");
  if (!find_section(f, "$Elements") || !std::getline(f, line)) return mesh_err("no $Elements section");
  Tokens e{line.c_str()};
  long long neb;
  if (!e.next_ll(&neb) || neb < 0) return mesh_err("bad $Elements header");
  for (long long b = 0; b < neb; ++b) {
    long long dim, tag, type, n;
    if (!std::getline(f, line)) return mesh_err("truncated $Elements");
    Tokens h{line.c_str()};
    if (!h.next_ll(&dim) || !h.next_ll(&tag) || !h.next_ll(&type) || !h.next_ll(&n) || n < 0)
      return mesh_err("bad element block header");
    for (long long i = 0; i < n; ++i) {
      if (!std::getline(f, line)) return mesh_err("truncated element block");
      if (type != 2) continue;  // triangles only
      Tokens c{line.c_str()};
      long long et, v[3];
      if (!c.next_ll(&et) || !c.next_ll(&v[0]) || !c.next_ll(&v[1]) || !c.next_ll(&v[2]))
        return mesh_err("bad triangle line");
      for (long long vi : v) {
        if (vi < tmin || vi > tmax) return mesh_err("triangle references an unknown node");
        out.cells.push_back((int32_t)(vi - tmin));
      }
    }
  }
  if (out.cells.size() / 3 > (size_t)INT32_MAX) return mesh_err("too many triangles");
  return DGC_OK;
}

}  // namespace

extern "C" int dgc_msh_read(const char* path, int* num_vertices, double* vertex_xy, int* num_cells,
                            int32_t* cells) {
  if (!path || !num_vertices || !num_cells) return set_error(DGC_ERR_ARG, "null argument");
  MshData d;
  if (int rc = parse_msh(path, d)) return rc;
  const int nv = (int)(d.xy.size() / 2), K = (int)(d.cells.size() / 3);
  if (vertex_xy || cells) {
    if (!vertex_xy || !cells) return set_error(DGC_ERR_ARG, "give both output arrays or neither");
    if (*num_vertices < nv || *num_cells < K) return set_error(DGC_ERR_ARG, "output arrays too small");
    std::memcpy(vertex_xy, d.xy.data(), d.xy.size() * sizeof(double));
    std::memcpy(cells, d.cells.data(), d.cells.size() * sizeof(int32_t));
  }
  *num_vertices = nv;
  *num_cells = K;
  return DGC_OK;
}

extern "C" int dgc_msh_write(const char* path, int num_vertices, const double* vertex_xy, int num_cells,
                             const int32_t* cells, int digits) {
  if (!path || num_vertices < 0 || num_cells < 0 || (num_vertices && !vertex_xy) || (num_cells && !cells))
    return set_error(DGC_ERR_ARG, "null argument");
  if (digits < 0 || digits > 17) return set_error(DGC_ERR_ARG, "digits outside [0, 17]");
  const int prec = digits ? digits : 6;
  FILE* f = std::fopen(path, "w");
  if (!f) return set_error(DGC_ERR_ARG, "cannot open the output file");
  std::fprintf(f, "$MeshFormat\n4.1 0 8\n$EndMeshFormat\n");
  std::fprintf(f, "$Nodes\n1 %d 1 %d\n2 1 0 %d\n", num_vertices, num_vertices, num_vertices);
  for (int i = 1; i <= num_vertices; ++i) std::fprintf(f, "%d\n", i);
  for (int i = 0; i < num_vertices; ++i)
    std::fprintf(f, "%.*g %.*g 0\n", prec, vertex_xy[2 * i], prec, vertex_xy[2 * i + 1]);
  std::fprintf(f, "$EndNodes\n$Elements\n1 %d 1 %d\n2 1 2 %d\n", num_cells, num_cells, num_cells);
  for (int i = 0; i < num_cells; ++i)
    std::fprintf(f, "%d %d %d %d\n", i + 1, cells[3 * i] + 1, cells[3 * i + 1] + 1, cells[3 * i + 2] + 1);
  std::fprintf(f, "$EndElements\n");
  const bool bad = std::ferror(f) != 0;
  std::fclose(f);
  return bad ? set_error(DGC_ERR_ARG, "write error") : DGC_OK;
}
