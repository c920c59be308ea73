// Host-side mesh construction for the G/B assembly (setup code, C++).
#pragma once
#include <algorithm>
#include <string>
#include <thread>
#include <vector>

namespace fk {

// f(0..n-1) on the host cores in contiguous blocks (setup of large meshes;
// f must only write state owned by its index).
template <class F>
void host_parallel_for(int n, F f) {
  unsigned nt = std::thread::hardware_concurrency();
  nt = std::max(1u, std::min(nt, 64u));
  if (n < 2048) nt = 1;
  if (nt == 1) {
    for (int i = 0; i < n; ++i) f(i);
    return;
  }
  std::vector<std::thread> pool;
  const int per = (n + static_cast<int>(nt) - 1) / static_cast<int>(nt);
  for (unsigned t = 0; t < nt; ++t) {
    const int lo = static_cast<int>(t) * per, hi = std::min(n, lo + per);
    if (lo >= hi) break;
    pool.emplace_back([lo, hi, &f] {
      for (int i = lo; i < hi; ++i) f(i);
    });
  }
  for (std::thread& th : pool) th.join();
}

struct MeshNode {
  double x, y, theta;
  int gid, ifx, ify;
  bool frontera;
};

// A stencil of the mesh: an arc of the reference (Interfaz) or a square patch
// boundary (Gaussian k-nearest stencil).
struct MeshStencil {
  // arc
  double cx = 0, cy = 0, radius = 0, c2 = 0;
  int interior = 0;
  bool perimeter = false;
  // patch
  double rect[4] = {0, 0, 0, 0};
  bool closed = false;
  int side_first[4] = {0, 0, 0, 0}, side_count[4] = {0, 0, 0, 0}, side_axis[4] = {0, 0, 0, 0};
  double side_fixed[4] = {0, 0, 0, 0}, side_start[4] = {0, 0, 0, 0}, side_step[4] = {0, 0, 0, 0};
  // nodes on the stencil (circle / patch boundary), in stencil order
  std::vector<MeshNode> nodes;
  // nodes of other stencils strictly inside this one (Interfaz::nudos_interior)
  std::vector<MeshNode> inner;
};

struct MeshItem {
  double x, y;
  int row, stencil;
  bool frontera;
};

struct HostMesh {
  int kind = 0;  // 1 circles (reference), 2 square patches
  double dom[4];
  double spacing = 0, eps = 0;
  int knn = 0;
  std::vector<MeshStencil> stencils;
  std::vector<MeshNode> nodes;   // by global id
  std::vector<MeshItem> items;
  int n_rows = 0, nnz = 0;
  std::vector<int> rowptr, col;
  std::vector<double> val0;
};

// Malla::Construye_Cuadrado (Mesh/Malla.cpp:12-83) with Interfaz::Inicia_Cuadrado
// (Mesh/Interfaz.cpp:2-204) and the CSR pattern of SistemaLineal
// (Mesh/SistemaLineal.cpp:8-66).  Items: interior nodes of perimeter circles.
bool build_circle_mesh(const double dom[4], int n_side, double superposicion, double theta0, int nodes_per_circle,
                       double c2_corner, double c2_side, HostMesh& m, std::string& err);

// Square patches: see fk_mesh_square_patches in include/spac_fk.h.
bool build_square_patch_mesh(const double dom[4], int n_sub, int nodes_per_side, double enlarge, double eps_spacing,
                             int knn, HostMesh& m, std::string& err);

}  // namespace fk
