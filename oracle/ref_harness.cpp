// Test-only harness around the reference implementation (SpAc), compiled
// from the reference's own unmodified sources against oracle/shim (see
// oracle/Makefile).  It drives the reference's public classes exactly the
// way its serial driver does (main_test_serial.cpp:11-89) and exposes the
// results through a small extern "C" API for the pin tests and for the
// fixture generator tests/golden/make_golden.py.  Nothing in the product
// links this file.
//
// Problems (BVP coefficient sets):
//   0 = Franke Poisson        BVPs/Franke_Poisson.hpp:4-73
//   1 = Monegros, c = -1      BVPs/Monegros_Revamped.hpp (built in ref_harness_monegros.cpp)
//   2 = anisotropic advection-reaction problem on [0,1]^2 (coefficients
//       defined below with the reference's typedefs; u = Franke * (1+xy))
//   5 = Monegros, c = 0       BVPs/Monegros_Poisson.hpp (built in ref_harness_monegros_poisson.cpp)
#include <cstdio>
#include <cstring>
#include <unistd.h>
#include <vector>
#include <map>
#include <string>
#include <omp.h>
#include "BVPs/Franke_Poisson.hpp"
#include "Dominios/Circulo.hpp"
#include "Dominios/Rectangulo.hpp"
#include "Solvers/FeynmanKacSolver.hpp"
#include "Solvers/PseudoespectralCirculoSolver.hpp"
#include "Mesh/Malla.hpp"

// Defined in ref_harness_monegros.cpp (separate TU: the Monegros headers
// reuse inline names of Franke_Poisson.hpp).
void ref_fill_monegros(BVP& bvp);
void ref_fill_monegros_poisson(BVP& bvp);

namespace {

// ---- problem 2: anisotropic diffusion + rotation drift + reaction ------------
// sigma sigma^T = 2 (1 + 0.5 sin(2 pi x) sin(2 pi y)) I, b = (y - 1/2, 1/2 - x),
// c = -(1 + x^2 + y^2), u = Franke(x,y) (1 + x y), f = -(L u).
struct FrankeParts {
  double F, Fx, Fy, Fxx, Fyy;
};
FrankeParts franke_parts(Eigen::Vector2d X) {
  FrankeParts p;
  p.F = Franke_u(X);
  p.Fx = Franke_dudx(X);
  p.Fy = Franke_dudy(X);
  p.Fxx = Franke_d2udx2(X);
  p.Fyy = Franke_d2udy2(X);
  return p;
}
double Aniso_u(Eigen::Vector2d X) { return Franke_u(X) * (1.0 + X(0) * X(1)); }
double Aniso_g(Eigen::Vector2d X) { return Aniso_u(X); }
double Aniso_c(Eigen::Vector2d X) { return -(1.0 + X(0) * X(0) + X(1) * X(1)); }
Eigen::Vector2d Aniso_b(Eigen::Vector2d X) {
  Eigen::Vector2d b;
  b(0) = X(1) - 0.5;
  b(1) = 0.5 - X(0);
  return b;
}
double aniso_a(Eigen::Vector2d X) {
  return 1.0 + 0.5 * sin(2.0 * M_PI * X(0)) * sin(2.0 * M_PI * X(1));
}
Eigen::Matrix2d Aniso_sigma(Eigen::Vector2d X) {
  return Eigen::Matrix2d::Identity() * sqrt(2.0 * aniso_a(X));
}
double Aniso_f(Eigen::Vector2d X) {
  FrankeParts p = franke_parts(X);
  double q = 1.0 + X(0) * X(1);
  double ux = p.Fx * q + p.F * X(1);
  double uy = p.Fy * q + p.F * X(0);
  double lap = (p.Fxx + p.Fyy) * q + 2.0 * (p.Fx * X(1) + p.Fy * X(0));
  Eigen::Vector2d b = Aniso_b(X);
  return -(aniso_a(X) * lap + b(0) * ux + b(1) * uy + Aniso_c(X) * Aniso_u(X));
}
Eigen::Vector2d Aniso_F(Eigen::Vector2d X) {
  FrankeParts p = franke_parts(X);
  double q = 1.0 + X(0) * X(1);
  Eigen::Vector2d grad;
  grad(0) = p.Fx * q + p.F * X(1);
  grad(1) = p.Fy * q + p.F * X(0);
  return -Aniso_sigma(X).transpose() * grad;
}

void fill_bvp(BVP& bvp, int problem, int use_F) {
  bvp.Reset();
  if (problem == 0) {
    bvp.u.Inicializa(Franke_u);
    bvp.g.Inicializa(Franke_g);
    bvp.c.Inicializa(Franke_c);
    bvp.f.Inicializa(Franke_f);
    bvp.sigma.Inicializa(Franke_sigma);
    bvp.b.Inicializa(Franke_b);
    if (use_F) bvp.F.Inicializa(Franke_F);
  } else if (problem == 1 || problem == 5) {
    if (problem == 1)
      ref_fill_monegros(bvp);
    else
      ref_fill_monegros_poisson(bvp);
    if (!use_F) {
      Coeficiente_Vectorial zero;
      bvp.F = zero;
    }
  } else {
    bvp.u.Inicializa(Aniso_u);
    bvp.g.Inicializa(Aniso_g);
    bvp.c.Inicializa(Aniso_c);
    bvp.f.Inicializa(Aniso_f);
    bvp.sigma.Inicializa(Aniso_sigma);
    bvp.b.Inicializa(Aniso_b);
    if (use_F) bvp.F.Inicializa(Aniso_F);
  }
}

std::vector<double> vec(const double* p, int n) { return std::vector<double>(p, p + n); }

// ---- results of the last assembly -------------------------------------------
struct ItemResult {
  int row, iface, frontera;
  std::vector<int> cols;
  std::vector<double> G;
  double B;
  double stats[9];
};
struct MeshNode {
  int gid, iface_x, iface_y, frontera;
  double x, y, theta;
};
struct MeshIface {
  double cx, cy, radius, c2;
  int interior, perimeter, n;
  std::vector<int> gids;
  std::vector<double> theta;
  std::vector<double> iPsi;  // column-major n x n
  std::vector<int> interior_gids;
};
struct Last {
  int n_rows = 0, nnz = 0;
  std::vector<int> rowptr, col;
  std::vector<double> val, B, val0;
  std::vector<ItemResult> items;
  std::vector<MeshNode> nodes;
  std::vector<MeshIface> ifaces;
} g_last;

std::string g_out_dir;
int g_ps_radial = 0;  // N_radio of the pseudospectral disk solves; 0 = interior circles skipped

void stats_of(const FeynmanKacSolver& s, double out[9]) {
  out[0] = s.phi;
  out[1] = s.phiphi;
  out[2] = s.phi_VR;
  out[3] = s.phiphi_VR;
  out[4] = s.xi;
  out[5] = s.xixi;
  out[6] = s.xiphi;
  out[7] = s.APL;
  out[8] = s.RNGC;
}

}  // namespace

extern "C" {

// A solver session keeps the reference's RNG streams alive across calls, as
// one FeynmanKacSolver object does in the reference drivers.
void* ref_solver_new(int nthreads) {
  omp_set_num_threads(nthreads);
  return new FeynmanKacSolver();
}
void ref_solver_free(void* s) { delete static_cast<FeynmanKacSolver*>(s); }

int ref_circulo(const double p[3], double x, double y, double out[5]) {
  Eigen::Vector2d X(x, y), e, n;
  out[0] = Circulo(vec(p, 3), X, e, n);
  out[1] = e(0); out[2] = e(1); out[3] = n(0); out[4] = n(1);
  return 0;
}
int ref_rectangulo(const double p[4], double x, double y, double out[5]) {
  Eigen::Vector2d X(x, y), e, n;
  out[0] = Rectangulo(vec(p, 4), X, e, n);
  out[1] = e(0); out[2] = e(1); out[3] = n(0); out[4] = n(1);
  return 0;
}
// Coefficients of a problem at (x,y): u, g, c, f, b0, b1, s00, s01, s10, s11, F0, F1
int ref_coefficients(int problem, double x, double y, double out[12]) {
  BVP bvp;
  fill_bvp(bvp, problem, 1);
  Eigen::Vector2d X(x, y);
  out[0] = bvp.u.Evalua(X);
  out[1] = bvp.g.Evalua(X);
  out[2] = bvp.c.Evalua(X);
  out[3] = bvp.f.Evalua(X);
  Eigen::Vector2d b = bvp.b.Evalua(X);
  out[4] = b(0); out[5] = b(1);
  Eigen::Matrix2d s = bvp.sigma.Evalua(X);
  out[6] = s(0, 0); out[7] = s(0, 1); out[8] = s(1, 0); out[9] = s(1, 1);
  Eigen::Vector2d F = bvp.F.Evalua(X);
  out[10] = F(0); out[11] = F(1);
  return 0;
}

// FeynmanKacSolver::Solve_OMP_Analytic(X0, N, h, rho, bvp) (FeynmanKacSolver.cpp:335-342).
// dom = [x0,y0,x1,y1] rectangle; sub_kind 0: subdomain = same rectangle,
// 1: circle [r,cx,cy], 2: rectangle [x0,y0,x1,y1].
// out: phi, phiphi, phi_VR, phiphi_VR, xi, xixi, xiphi, APL, RNGC
int ref_point_solve(void* session, int problem, int use_F, const double dom[4], int sub_kind,
                    const double* sub, double x, double y, unsigned N, double h, double out[9]) {
  FeynmanKacSolver& s = *static_cast<FeynmanKacSolver*>(session);
  BVP bvp;
  fill_bvp(bvp, problem, use_F);
  bvp.frontera_dominio.Inicializa(vec(dom, 4), Rectangulo, Stopping, Stopping);
  if (sub_kind == 0) bvp.frontera_subdominio.Inicializa(vec(dom, 4), Rectangulo, Stopping, Stopping);
  else if (sub_kind == 1) bvp.frontera_subdominio.Inicializa(vec(sub, 3), Circulo, Stopping, Stopping);
  else bvp.frontera_subdominio.Inicializa(vec(sub, 4), Rectangulo, Stopping, Stopping);
  Eigen::Vector2d X0(x, y);
  s.Solve_OMP_Analytic(X0, N, h, 1.0, bvp);
  stats_of(s, out);
  return 0;
}

// Interfaz::Calcula_Psi on given node angles (Interfaz.cpp:206-217): writes
// iPsi (column-major) and returns ||iPsi||_F ||Psi||_F.
double ref_calcula_psi(int n, const double* theta, double c2, double* iPsi) {
  BVP bvp;
  Interfaz it;
  it.nudos_circunferencia.resize(n);
  for (int i = 0; i < n; ++i) it.nudos_circunferencia[i].posicion_angular = theta[i];
  double k = it.Calcula_Psi(bvp, c2);
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) iPsi[i + j * n] = it.iPsi(i, j);
  return k;
}

// PseudoespectralCirculoSolver::Inicializa + Resuelve(BVP, nudos_interior,
// nudos_periferia) (Solvers/PseudoespectralCirculoSolver.cpp:2-260) on one
// disk: periphery nodes at angles periph_theta (global ids 0..n_periph-1),
// interior nodes at inner_xy.  G (n_inner x n_periph, row-major) receives
// nudos_interior[i].G[j], B[i] nudos_interior[i].B.
int ref_ps_disk(int problem, double cx, double cy, double radius, int n_circle, int n_radial, double theta0,
                int n_periph, const double* periph_theta, int n_inner, const double* inner_xy, double* G,
                double* B) {
  BVP bvp;
  fill_bvp(bvp, problem, 0);
  std::vector<Nudo> inner(n_inner), periph(n_periph);
  for (int j = 0; j < n_periph; ++j) {
    periph[j].Resetea();
    periph[j].indice_global = j;
    periph[j].posicion_angular = periph_theta[j];
  }
  for (int i = 0; i < n_inner; ++i) {
    inner[i].Resetea();
    inner[i].indice_global = n_periph + i;
    inner[i].posicion_cartesiana = Eigen::Vector2d(inner_xy[2 * i], inner_xy[2 * i + 1]);
  }
  PseudoespectralCirculoSolver ps;
  ps.Inicializa(Eigen::Vector2d(cx, cy), radius, n_circle, n_radial, theta0, bvp);
  ps.Resuelve(bvp, inner, periph);
  for (int i = 0; i < n_inner; ++i) {
    B[i] = inner[i].B;
    for (int j = 0; j < n_periph; ++j) {
      auto it = inner[i].G.find(j);
      G[static_cast<size_t>(i) * n_periph + j] = it == inner[i].G.end() ? 0.0 : it->second;
    }
  }
  return 0;
}

// N_radio for the interior circles of the next ref_assemble_circles (0 =
// interior circles skipped).
void ref_set_ps_radial(int n_radial) { g_ps_radial = n_radial; }

// Builds the reference mesh (Malla::Construye_Cuadrado, Malla.cpp:12-83) and
// assembles G/B the way main_test_serial.cpp:54-80 does: FK node solves
// (Solve_OMP_Analytic(nudo,...), FeynmanKacSolver.cpp:344-355) for the
// interior nodes of perimeter circles and SistemaLineal::Actualiza_GB; interior
// circles are solved by PseudoespectralCirculoSolver when ref_set_ps_radial
// set N_radio (Actualiza_GB(Interfaz&)), else skipped.  do_solve: 0 = mesh
// only, 1 = both kinds of rows, 2 = pseudospectral rows only.  Nodes of full
// circles get frontera = false explicitly (left uninitialised by Nudo()).
int ref_assemble_circles(void* session, int problem, int use_F, const double dom[4], int Nl,
                         double superposicion, double theta0, int nodes_per_circle, double c2_corner,
                         double c2_side, unsigned N, double h, int do_solve) {
  FeynmanKacSolver& s = *static_cast<FeynmanKacSolver*>(session);
  BVP bvp;
  fill_bvp(bvp, problem, use_F);
  std::vector<double> pr = vec(dom, 4);
  std::vector<double> pc(3, 0.0);
  bvp.frontera_dominio.Inicializa(pr, Rectangulo, Stopping, Stopping);
  bvp.frontera_subdominio.Inicializa(pc, Circulo, Stopping, Stopping);
  Malla mesh;
  std::map<std::string, double> c2;
  c2["esquina"] = c2_corner;
  c2["lado"] = c2_side;
  mesh.Construye_Cuadrado(pr, Nl, superposicion, theta0, nodes_per_circle, bvp, c2);
  // mesh description
  g_last = Last();
  for (auto& itf : mesh.Interfaces) {
    for (auto& nd : itf.nudos_circunferencia)
      if (itf.interior == 1) nd.frontera = false;
  }
  for (auto& itf : mesh.Interfaces) {
    for (auto& nd : itf.nudos_interior) {
      const Interfaz& owner = mesh.Interfaces[nd.indice_interfaz[0] * Nl + nd.indice_interfaz[1]];
      if (owner.interior == 1) nd.frontera = false;
    }
  }
  for (auto& itf : mesh.Interfaces) {
    MeshIface mi;
    mi.cx = itf.centro(0); mi.cy = itf.centro(1); mi.radius = itf.radio; mi.c2 = itf.c2;
    mi.interior = itf.interior; mi.perimeter = itf.es_perimeter ? 1 : 0;
    mi.n = static_cast<int>(itf.nudos_circunferencia.size());
    for (auto& nd : itf.nudos_circunferencia) {
      mi.gids.push_back(nd.indice_global);
      mi.theta.push_back(nd.posicion_angular);
      MeshNode mn;
      mn.gid = nd.indice_global; mn.iface_x = nd.indice_interfaz[0]; mn.iface_y = nd.indice_interfaz[1];
      mn.frontera = nd.frontera ? 1 : 0;
      mn.x = nd.posicion_cartesiana(0); mn.y = nd.posicion_cartesiana(1); mn.theta = nd.posicion_angular;
      g_last.nodes.push_back(mn);
    }
    if (itf.es_perimeter && itf.iPsi.rows() == mi.n) {
      mi.iPsi.resize(static_cast<size_t>(mi.n) * mi.n);
      for (int j = 0; j < mi.n; ++j)
        for (int i = 0; i < mi.n; ++i) mi.iPsi[i + j * mi.n] = itf.iPsi(i, j);
    }
    for (auto& nd : itf.nudos_interior) mi.interior_gids.push_back(nd.indice_global);
    g_last.ifaces.push_back(mi);
  }
  SistemaLineal& S = mesh.sistema;
  g_last.n_rows = S.n_filas;
  g_last.nnz = S.nnz;
  g_last.rowptr.assign(S.G_i, S.G_i + S.n_filas + 1);
  g_last.col.assign(S.G_j, S.G_j + S.nnz);
  g_last.val0.assign(S.G_ij, S.G_ij + S.nnz);
  if (do_solve) {
    int idx = 0;
    for (auto& itf : mesh.Interfaces) {
      if (itf.es_perimeter && do_solve == 1) {
        pc[0] = itf.radio; pc[1] = itf.centro(0); pc[2] = itf.centro(1);
        bvp.frontera_subdominio.Inicializa(pc, Circulo, Stopping, Stopping);
        for (auto& nd : itf.nudos_interior) {
          nd.G.clear();
          nd.B = 0.0;
          s.Solve_OMP_Analytic(nd, N, h, 1.0, bvp, itf);
          ItemResult r;
          r.row = nd.indice_global; r.iface = idx; r.frontera = nd.frontera ? 1 : 0;
          for (auto& kv : nd.G) { r.cols.push_back(kv.first); r.G.push_back(kv.second); }
          r.B = nd.B;
          if (nd.frontera) for (double& v : r.stats) v = 0.0; else stats_of(s, r.stats);
          g_last.items.push_back(r);
          S.Actualiza_GB(nd);
        }
      } else if (!itf.es_perimeter && g_ps_radial > 0) {
        PseudoespectralCirculoSolver ps;
        ps.Inicializa(itf.centro, itf.radio, itf.nudos_circunferencia.size(), g_ps_radial,
                      itf.nudos_circunferencia[0].posicion_angular, bvp);
        ps.Resuelve(bvp, itf.nudos_interior, itf.nudos_circunferencia);
        S.Actualiza_GB(itf);
      }
      ++idx;
    }
  }
  g_last.val.assign(S.G_ij, S.G_ij + S.nnz);
  g_last.B.assign(S.B, S.B + S.n_filas);
  if (!g_out_dir.empty()) {
    // the reference writes into ./Output/ (SistemaLineal.cpp:96-138, Malla.cpp:99-112)
    char cwd[4096];
    if (getcwd(cwd, sizeof(cwd)) && chdir(g_out_dir.c_str()) == 0) {
      S.Escribe_GB_COO();
      S.Escribe_GB_CSR();
      mesh.Escribe_Posiciones(bvp);
      if (chdir(cwd) != 0) return -1;
    }
  }
  return 0;
}

// Directory (containing Output/) where the next assembly writes the
// reference's text outputs; empty = none.
void ref_set_output_dir(const char* dir) { g_out_dir = dir ? dir : ""; }

int ref_last_sizes(int* n_rows, int* nnz, int* n_items, int* n_nodes, int* n_ifaces) {
  *n_rows = g_last.n_rows; *nnz = g_last.nnz;
  *n_items = static_cast<int>(g_last.items.size());
  *n_nodes = static_cast<int>(g_last.nodes.size());
  *n_ifaces = static_cast<int>(g_last.ifaces.size());
  return 0;
}
int ref_last_csr(int* rowptr, int* col, double* val0, double* val, double* B) {
  std::memcpy(rowptr, g_last.rowptr.data(), sizeof(int) * g_last.rowptr.size());
  std::memcpy(col, g_last.col.data(), sizeof(int) * g_last.col.size());
  std::memcpy(val0, g_last.val0.data(), sizeof(double) * g_last.val0.size());
  std::memcpy(val, g_last.val.data(), sizeof(double) * g_last.val.size());
  std::memcpy(B, g_last.B.data(), sizeof(double) * g_last.B.size());
  return 0;
}
// node record: gid, iface_x, iface_y, frontera (ints) and x, y, theta (doubles)
int ref_last_node(int i, int* ints4, double* dbl3) {
  const MeshNode& m = g_last.nodes[i];
  ints4[0] = m.gid; ints4[1] = m.iface_x; ints4[2] = m.iface_y; ints4[3] = m.frontera;
  dbl3[0] = m.x; dbl3[1] = m.y; dbl3[2] = m.theta;
  return 0;
}
// interface record: ints = interior, perimeter, n, n_interior; dbl = cx, cy, radius, c2
int ref_last_iface(int i, int* ints4, double* dbl4) {
  const MeshIface& m = g_last.ifaces[i];
  ints4[0] = m.interior; ints4[1] = m.perimeter; ints4[2] = m.n;
  ints4[3] = static_cast<int>(m.interior_gids.size());
  dbl4[0] = m.cx; dbl4[1] = m.cy; dbl4[2] = m.radius; dbl4[3] = m.c2;
  return 0;
}
int ref_last_iface_arrays(int i, int* gids, double* theta, double* iPsi, int* interior_gids) {
  const MeshIface& m = g_last.ifaces[i];
  std::memcpy(gids, m.gids.data(), sizeof(int) * m.gids.size());
  std::memcpy(theta, m.theta.data(), sizeof(double) * m.theta.size());
  if (!m.iPsi.empty()) std::memcpy(iPsi, m.iPsi.data(), sizeof(double) * m.iPsi.size());
  std::memcpy(interior_gids, m.interior_gids.data(), sizeof(int) * m.interior_gids.size());
  return static_cast<int>(m.iPsi.empty() ? 0 : 1);
}
// item record: ints = row, iface, frontera, nG; dbl = B + 9 stats
int ref_last_item(int i, int* ints4, double* dbl10) {
  const ItemResult& r = g_last.items[i];
  ints4[0] = r.row; ints4[1] = r.iface; ints4[2] = r.frontera; ints4[3] = static_cast<int>(r.G.size());
  dbl10[0] = r.B;
  for (int k = 0; k < 9; ++k) dbl10[1 + k] = r.stats[k];
  return 0;
}
int ref_last_item_G(int i, int* cols, double* G) {
  const ItemResult& r = g_last.items[i];
  std::memcpy(cols, r.cols.data(), sizeof(int) * r.cols.size());
  std::memcpy(G, r.G.data(), sizeof(double) * r.G.size());
  return 0;
}

}  // extern "C"
