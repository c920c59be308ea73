// Host-side mesh construction (setup, not on the hot path).
#include "fk_mesh.h"

#include <algorithm>
#include <cmath>
#include <set>
#include <vector>

namespace fk {
namespace {

// Branch-cut arctangents, Mesh/Nudo.hpp:7-32.
double atan0(double x, double y) { double a = std::atan2(y, x); return a >= 0 ? a : a + 2.0 * M_PI; }
double atan90(double x, double y) { double a = std::atan2(y, x); return a <= 0.5 * M_PI ? 2.0 * M_PI + a : a; }
double atan180(double x, double y) { return std::atan2(y, x); }
double atan270(double x, double y) { double a = std::atan2(y, x); return a <= -0.5 * M_PI ? 2 * M_PI + a : a; }

// Interfaz::Inicia_Cuadrado (Mesh/Interfaz.cpp:2-204): the arc of circle
// (ix, iy) inside the rectangle, its node angles and the arc code.
int init_circle(double r, const double* dom, double theta0, double c2_corner, double c2_side, double cx, double cy,
                int ix, int iy, int imax, int n_total, int first_gid, MeshStencil& S) {
  S = MeshStencil();
  S.radius = r;
  S.cx = cx;
  S.cy = cy;
  double first = 0, last = 0, vx, vy;
  const double r2 = r * r;
  if (ix == 0) {
    if (iy == 0) {
      vy = dom[1] - cy; vx = std::sqrt(r2 - vy * vy); first = atan180(vx, vy);
      vx = dom[0] - cx; vy = std::sqrt(r2 - vx * vx); last = atan180(vx, vy);
      S.interior = -11;
    } else if (iy == imax) {
      vx = dom[0] - cx; vy = -std::sqrt(r2 - vx * vx); first = atan180(vx, vy);
      vy = dom[3] - cy; vx = std::sqrt(r2 - vy * vy); last = atan180(vx, vy);
      S.interior = -22;
    } else {
      vx = dom[0] - cx; vy = -std::sqrt(r2 - vx * vx); first = atan180(vx, vy);
      vy = std::sqrt(r2 - vx * vx); last = atan180(vx, vy);
      S.interior = -4;
    }
  } else if (ix == imax) {
    if (iy == 0) {
      vx = dom[2] - cx; vy = std::sqrt(r2 - vx * vx); first = atan0(vx, vy);
      vy = dom[1] - cy; vx = -std::sqrt(r2 - vy * vy); last = atan0(vx, vy);
      S.interior = -44;
    } else if (iy == imax) {
      vy = dom[3] - cy; vx = -std::sqrt(r2 - vy * vy); first = atan0(vx, vy);
      vx = dom[2] - cx; vy = -std::sqrt(r2 - vx * vx); last = atan0(vx, vy);
      S.interior = -33;
    } else {
      // the reference reads the y upper bound here (Interfaz.cpp:121); equal on square domains
      vx = dom[3] - cx; vy = std::sqrt(r2 - vx * vx); first = atan0(vx, vy);
      vy = -std::sqrt(r2 - vx * vx); last = atan0(vx, vy);
      S.interior = -2;
    }
  } else {
    if (iy == 0) {
      vy = dom[1] - cy; vx = +std::sqrt(r2 - vy * vy); first = atan270(vx, vy);
      vx = -std::sqrt(r2 - vy * vy); last = atan270(vx, vy);
      S.interior = -1;
    } else if (iy == imax) {
      vy = dom[3] - cy; vx = -std::sqrt(r2 - vy * vy); first = atan90(vx, vy);
      vx = +std::sqrt(r2 - vy * vy); last = atan90(vx, vy);
      S.interior = -3;
    } else {
      S.interior = 1;
    }
  }
  const double incr = 2 * (M_PI) / n_total;
  int gid = first_gid;
  auto add = [&](double th, bool frontera) {
    MeshNode nd;
    nd.theta = th;
    nd.x = cx + r * std::cos(th);
    nd.y = cy + r * std::sin(th);
    nd.gid = gid++;
    nd.ifx = ix;
    nd.ify = iy;
    nd.frontera = frontera;
    S.nodes.push_back(nd);
  };
  if (S.interior > 0) {
    first = theta0;
    for (int i = 0; i < n_total; ++i) add(first + incr * i, false);
    S.perimeter = false;
  } else {
    const int n_arc = static_cast<int>(n_total * std::fabs(last - first) / (2 * M_PI));
    add(first, true);
    for (int i = 0; i < n_arc; ++i) add(first + theta0 + incr * i, false);
    add(last, true);
    S.perimeter = true;
    S.c2 = (S.interior < -10) ? c2_corner : c2_side;
  }
  return gid;
}

// SistemaLineal adjacency -> sorted CSR with the diagonal count and the
// 1e-23 placeholder (Mesh/SistemaLineal.cpp:8-66).
void build_csr(HostMesh& m, const std::vector<std::vector<int>>& adj_in, const std::vector<double>& diag) {
  m.n_rows = static_cast<int>(adj_in.size());
  m.rowptr.assign(m.n_rows + 1, 0);
  m.col.clear();
  m.val0.clear();
  for (int r = 0; r < m.n_rows; ++r) {
    std::set<int> s(adj_in[r].begin(), adj_in[r].end());
    s.insert(r);
    m.rowptr[r] = static_cast<int>(m.col.size());
    for (int c : s) {
      m.col.push_back(c);
      m.val0.push_back(c == r ? diag[r] : 1.0E-23);
    }
  }
  m.rowptr[m.n_rows] = static_cast<int>(m.col.size());
  m.nnz = static_cast<int>(m.col.size());
}

void add_adjacency(const MeshStencil& S, std::vector<std::vector<int>>& adj, std::vector<double>& diag) {
  // SistemaLineal::Anadir_Lista_Adyacencia (Mesh/SistemaLineal.cpp:8-18)
  for (const MeshNode& in : S.inner) {
    for (const MeshNode& c : S.nodes) {
      adj[in.gid].push_back(c.gid);
      adj[c.gid].push_back(in.gid);
    }
    diag[in.gid] += 1.0;
  }
}

}  // namespace

bool build_circle_mesh(const double dom[4], int n_side, double superposicion, double theta0, int nodes_per_circle,
                       double c2_corner, double c2_side, HostMesh& m, std::string& err) {
  if (n_side < 2 || nodes_per_circle < 4 || superposicion < 1.0 || superposicion > 2.0) {
    err = "fk_mesh_circles: need n_side >= 2, nodes_per_circle >= 4, 1 <= superposicion <= 2";
    return false;
  }
  m = HostMesh();
  m.kind = 1;
  for (int i = 0; i < 4; ++i) m.dom[i] = dom[i];
  const double d = (dom[2] - dom[0]) / (n_side - 1);
  const double r = superposicion * d / std::sqrt(2.0);
  int gid = 0;
  for (int ix = 0; ix <= n_side - 1; ++ix)
    for (int iy = 0; iy <= n_side - 1; ++iy) {
      MeshStencil S;
      gid = init_circle(r, dom, theta0, c2_corner, c2_side, dom[0] + ix * d, dom[1] + iy * d, ix, iy, n_side - 1,
                        nodes_per_circle, gid, S);
      S.perimeter = (ix * iy == 0 || ix == n_side - 1 || iy == n_side - 1);
      m.stencils.push_back(S);
    }
  const int n_nodes = gid;
  m.nodes.resize(n_nodes);
  for (const MeshStencil& S : m.stencils)
    for (const MeshNode& nd : S.nodes) m.nodes[nd.gid] = nd;
  // neighbours in the order of the reference's std::map<std::string,int>
  // (E, N, NE, NW, S, SE, SW, W), Malla.cpp:52-80
  struct Dir { const char* name; int off; };
  const Dir dirs[8] = {{"E", n_side}, {"N", 1}, {"NE", n_side + 1}, {"NW", -n_side + 1},
                       {"S", -1}, {"SE", n_side - 1}, {"SW", -n_side - 1}, {"W", -n_side}};
  std::vector<std::vector<int>> adj(n_nodes);
  std::vector<double> diag(n_nodes, 0.0);
  for (int s = 0; s < static_cast<int>(m.stencils.size()); ++s) {
    MeshStencil& S = m.stencils[s];
    const int ix = s / n_side, iy = s % n_side;
    for (const Dir& dr : dirs) {
      const std::string nm = dr.name;
      if (nm.find('N') != std::string::npos && iy == n_side - 1) continue;
      if (nm.find('S') != std::string::npos && iy == 0) continue;
      if (nm.find('E') != std::string::npos && ix == n_side - 1) continue;
      if (nm.find('W') != std::string::npos && ix == 0) continue;
      const MeshStencil& Nb = m.stencils[s + dr.off];
      for (const MeshNode& nd : Nb.nodes) {
        const double dx = nd.x - S.cx, dy = nd.y - S.cy;
        if (std::sqrt(dx * dx + dy * dy) < S.radius) S.inner.push_back(nd);
      }
    }
    add_adjacency(S, adj, diag);
  }
  build_csr(m, adj, diag);
  // FK items: interior nodes of perimeter circles (main_test_serial.cpp:54-62)
  for (int s = 0; s < static_cast<int>(m.stencils.size()); ++s) {
    const MeshStencil& S = m.stencils[s];
    if (!S.perimeter) continue;
    for (const MeshNode& nd : S.inner) m.items.push_back(MeshItem{nd.x, nd.y, nd.gid, s, nd.frontera});
  }
  return true;
}

bool build_square_patch_mesh(const double dom[4], int n_sub, int nodes_per_side, double enlarge, double eps_spacing,
                             int knn, HostMesh& m, std::string& err) {
  if (n_sub < 2 || nodes_per_side < 2 || enlarge <= 0.0 || enlarge >= 0.5 || knn < 2 || eps_spacing <= 0.0) {
    err = "fk_mesh_square_patches: need n_sub >= 2, nodes_per_side >= 2, 0 < enlarge < 0.5, knn >= 2, eps > 0";
    return false;
  }
  m = HostMesh();
  m.kind = 2;
  for (int i = 0; i < 4; ++i) m.dom[i] = dom[i];
  const double Hx = (dom[2] - dom[0]) / n_sub, Hy = (dom[3] - dom[1]) / n_sub;
  const double Lx = (1.0 + 2.0 * enlarge) * Hx, Ly = (1.0 + 2.0 * enlarge) * Hy;
  const double sx = Lx / (nodes_per_side + 1), sy = Ly / (nodes_per_side + 1);
  m.spacing = sx;
  m.eps = eps_spacing / sx;
  m.knn = knn;
  const double tol = 1e-12 * std::max(dom[2] - dom[0], dom[3] - dom[1]);
  auto inside_dom = [&](double x, double y) {
    return x > dom[0] + tol && x < dom[2] - tol && y > dom[1] + tol && y < dom[3] - tol;
  };
  int gid = 0;
  for (int a = 0; a < n_sub; ++a)
    for (int b = 0; b < n_sub; ++b) {
      MeshStencil S;
      S.rect[0] = dom[0] + (a - enlarge) * Hx;
      S.rect[1] = dom[1] + (b - enlarge) * Hy;
      S.rect[2] = dom[0] + (a + 1 + enlarge) * Hx;
      S.rect[3] = dom[1] + (b + 1 + enlarge) * Hy;
      // counter-clockwise ring: bottom (x up), right (y up), top (x down), left (y down)
      struct Cand { double x, y; int side; };
      std::vector<Cand> ring;
      for (int side = 0; side < 4; ++side)
        for (int q = 1; q <= nodes_per_side; ++q) {
          double x, y;
          switch (side) {
            case 0: x = S.rect[0] + q * sx; y = S.rect[1]; break;
            case 1: x = S.rect[2]; y = S.rect[1] + q * sy; break;
            case 2: x = S.rect[2] - q * sx; y = S.rect[3]; break;
            default: x = S.rect[0]; y = S.rect[3] - q * sy; break;
          }
          ring.push_back(Cand{x, y, side});
        }
      const int R = static_cast<int>(ring.size());
      std::vector<bool> keep(R);
      int n_keep = 0;
      for (int i = 0; i < R; ++i) { keep[i] = inside_dom(ring[i].x, ring[i].y); n_keep += keep[i]; }
      if (n_keep < knn) {
        err = "fk_mesh_square_patches: a patch keeps fewer nodes than the stencil size";
        return false;
      }
      int start = 0;
      S.closed = (n_keep == R);
      if (!S.closed) {
        // the kept nodes form one cyclic run: start right after a dropped node
        for (int i = 0; i < R; ++i)
          if (!keep[i] && keep[(i + 1) % R]) { start = (i + 1) % R; break; }
      }
      for (int side = 0; side < 4; ++side) { S.side_count[side] = 0; S.side_first[side] = -1; }
      for (int t = 0; t < R; ++t) {
        const int i = (start + t) % R;
        if (!keep[i]) continue;
        const Cand& c = ring[i];
        MeshNode nd;
        nd.x = c.x; nd.y = c.y; nd.theta = 0.0; nd.gid = gid++; nd.ifx = a; nd.ify = b; nd.frontera = false;
        const int chain = static_cast<int>(S.nodes.size());
        if (S.side_count[c.side] == 0) {
          S.side_first[c.side] = chain;
          S.side_axis[c.side] = (c.side == 0 || c.side == 2) ? 0 : 1;
          S.side_fixed[c.side] = (c.side == 0 || c.side == 2) ? c.y : c.x;
          S.side_start[c.side] = (c.side == 0 || c.side == 2) ? c.x : c.y;
          S.side_step[c.side] = (c.side == 0) ? sx : (c.side == 1) ? sy : (c.side == 2) ? -sx : -sy;
        }
        S.side_count[c.side]++;
        S.nodes.push_back(nd);
      }
      m.stencils.push_back(S);
    }
  const int n_nodes = gid;
  m.nodes.resize(n_nodes);
  for (const MeshStencil& S : m.stencils)
    for (const MeshNode& nd : S.nodes) m.nodes[nd.gid] = nd;
  // nodes strictly inside each patch (other than its own boundary nodes), in
  // node order: the nodes are bucketed by subdomain cell, and a patch (its
  // cell enlarged by less than half a cell) only overlaps the 3 x 3 cells
  // around its own
  const int n_st = static_cast<int>(m.stencils.size());
  auto cell_of = [&](double v, double lo, double H) {
    return std::max(0, std::min(n_sub - 1, static_cast<int>(std::floor((v - lo) / H))));
  };
  std::vector<std::vector<int>> bucket(static_cast<size_t>(n_sub) * n_sub);
  for (const MeshNode& nd : m.nodes)
    bucket[static_cast<size_t>(cell_of(nd.x, dom[0], Hx)) * n_sub + cell_of(nd.y, dom[1], Hy)].push_back(nd.gid);
  host_parallel_for(n_st, [&](int s) {
    MeshStencil& S = m.stencils[s];
    const int a = s / n_sub, b = s % n_sub;
    std::vector<int> in;
    for (int ca = std::max(0, a - 1); ca <= std::min(n_sub - 1, a + 1); ++ca)
      for (int cb = std::max(0, b - 1); cb <= std::min(n_sub - 1, b + 1); ++cb)
        for (int g : bucket[static_cast<size_t>(ca) * n_sub + cb]) {
          const MeshNode& nd = m.nodes[g];
          if (nd.ifx * n_sub + nd.ify == s) continue;
          if (nd.x > S.rect[0] + tol && nd.x < S.rect[2] - tol && nd.y > S.rect[1] + tol && nd.y < S.rect[3] - tol)
            in.push_back(g);
        }
    std::sort(in.begin(), in.end());
    for (int g : in) S.inner.push_back(m.nodes[g]);
  });
  // patches holding each node inside (patch order); the node's own ring is its
  // patch (ifx, ify)
  std::vector<std::vector<int>> by_node(n_nodes);
  for (int s = 0; s < n_st; ++s)
    for (const MeshNode& nd : m.stencils[s].inner) by_node[nd.gid].push_back(s);
  // CSR pattern, as SistemaLineal::Anadir_Lista_Adyacencia + Inicializa_CSR
  // (Mesh/SistemaLineal.cpp:8-66) build it: row r couples to itself, to the
  // ring nodes of every patch holding r inside, and to the inner nodes of the
  // patch whose ring holds r; the diagonal counts the patches holding r inside
  std::vector<std::vector<int>> rows(n_nodes);
  host_parallel_for(n_nodes, [&](int r) {
    std::vector<int>& c = rows[r];
    c.push_back(r);
    for (int s : by_node[r])
      for (const MeshNode& nd : m.stencils[s].nodes) c.push_back(nd.gid);
    const MeshNode& me = m.nodes[r];
    for (const MeshNode& nd : m.stencils[me.ifx * n_sub + me.ify].inner) c.push_back(nd.gid);
    std::sort(c.begin(), c.end());
    c.erase(std::unique(c.begin(), c.end()), c.end());
  });
  m.n_rows = n_nodes;
  m.rowptr.assign(n_nodes + 1, 0);
  for (int r = 0; r < n_nodes; ++r) m.rowptr[r + 1] = m.rowptr[r] + static_cast<int>(rows[r].size());
  m.nnz = m.rowptr[n_nodes];
  m.col.resize(m.nnz);
  m.val0.resize(m.nnz);
  host_parallel_for(n_nodes, [&](int r) {
    int k = m.rowptr[r];
    for (int c : rows[r]) {
      m.col[k] = c;
      m.val0[k] = c == r ? static_cast<double>(by_node[r].size()) : 1.0E-23;
      ++k;
    }
    std::vector<int>().swap(rows[r]);
  });
  for (int g = 0; g < n_nodes; ++g)
    for (int s : by_node[g]) m.items.push_back(MeshItem{m.nodes[g].x, m.nodes[g].y, g, s, false});
  return true;
}

}  // namespace fk
