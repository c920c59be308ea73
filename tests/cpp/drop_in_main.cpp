// Drives FeynmanKacSolverGPU the way the reference's serial driver drives
// FeynmanKacSolver (main_test_serial.cpp:54-62, :96): one point solve, then
// one Solve_OMP_Analytic(Nudo&, ...) per node of an arc read from a file.
// Usage: drop_in_main <arc file> <seed>
// Arc file: cx cy radius c2 interior n / n lines "theta gid" / n*n iPsi
// (column-major) / item count / per item "x y frontera gid".
// drop_in_main --robin <seed>: one point solve with a reflecting domain side.
// drop_in_main --disk <disk file> drives PseudoespectralCirculoSolverGPU the
// way main_test_serial.cpp:67-75 drives PseudoespectralCirculoSolver.
// Disk file: cx cy radius N_circunferencia N_radio theta_0 / n_periph lines
// "theta gid" / n_inner / n_inner lines "x y gid".
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <exception>
#include <fstream>
#include <string>

#include "ref_types.hpp"
#include "spac_fk_gpu.hpp"

using namespace ref_like;

static double franke_u(Vector2d) { return 0.0; }          // identity only: the device functor computes
static Vector2d franke_F(Vector2d p) { return p; }
static double rectangulo(std::vector<double>, Vector2d, Vector2d&, Vector2d&) { return 0.0; }
static double circulo(std::vector<double>, Vector2d, Vector2d&, Vector2d&) { return 0.0; }

static int disk_main(const char* path) {
  FeynmanKacSolverGPU::Register_Problem(&franke_u, FK_PROBLEM_FRANKE, &franke_F);
  BVP bvp;
  bvp.u.funcion = &franke_u;
  std::ifstream in(path);
  Vector2d c;
  double R = 0.0, th0 = 0.0;
  unsigned nc = 0, nr = 0;
  int np = 0, ni = 0;
  in >> c[0] >> c[1] >> R >> nc >> nr >> th0 >> np;
  std::vector<Nudo> periph(np), inner;
  for (auto& nd : periph) in >> nd.posicion_angular >> nd.indice_global;
  in >> ni;
  inner.resize(ni);
  for (auto& nd : inner) in >> nd.posicion_cartesiana[0] >> nd.posicion_cartesiana[1] >> nd.indice_global;
  PseudoespectralCirculoSolverGPU ps(0);
  ps.Inicializa(c, R, nc, nr, th0, bvp);
  ps.Resuelve(bvp, inner, periph);
  for (auto& nd : inner) {
    std::printf("inner %d %.17g", nd.indice_global, nd.B);
    for (auto& kv : nd.G) std::printf(" %d:%.17g", kv.first, kv.second);
    std::printf("\n");
  }
  return 0;
}

// Solve_OMP_Analytic(X0, ...) on a BVP whose domain side x = 0 reflects
// (Frontera::Absorbente false there), registered as FK_PROBLEM_ROBIN with
// varphi = -0.5, rho = 0.1.
static double aniso_u(Vector2d) { return 0.0; }
static bool absorbing_except_left(Vector2d p) { return !(std::fabs(p[0]) < 1e-8); }
static int robin_main(unsigned long long seed) {
  const double prob[4] = {0.0, -0.5, 0.0, 0.0};
  FeynmanKacSolverGPU::Register_Problem(&aniso_u, FK_PROBLEM_ROBIN, nullptr, prob);
  FeynmanKacSolverGPU::Register_Distance(&rectangulo, FK_SHAPE_RECT);
  FeynmanKacSolverGPU solver(0, seed);
  BVP bvp;
  bvp.u.funcion = &aniso_u;
  bvp.frontera_dominio.Distancia = &rectangulo;
  bvp.frontera_dominio.parametros = {0.0, 0.0, 1.0, 1.0};
  bvp.frontera_dominio.Absorbente = &absorbing_except_left;
  Vector2d X0;
  X0[0] = 0.02;
  X0[1] = 0.4;
  solver.Solve_OMP_Analytic(X0, 2000, 1e-3, 0.1, bvp);
  std::printf("robin %.17g %.17g %.17g %.17g\n", solver.phi, solver.phiphi, solver.APL, solver.RNGC);
  return 0;
}

int main(int argc, char** argv) {
  if (argc == 3 && std::string(argv[1]) == "--robin") {
    try {
      return robin_main(std::strtoull(argv[2], nullptr, 10));
    } catch (const std::exception& e) {
      std::fprintf(stderr, "%s\n", e.what());
      return 3;
    }
  }
  if (argc == 3 && std::string(argv[1]) == "--disk") {
    try {
      return disk_main(argv[2]);
    } catch (const std::exception& e) {
      std::fprintf(stderr, "%s\n", e.what());
      return 3;
    }
  }
  if (argc < 3) return 2;
  FeynmanKacSolverGPU::Register_Problem(&franke_u, FK_PROBLEM_FRANKE, &franke_F);
  FeynmanKacSolverGPU::Register_Distance(&rectangulo, FK_SHAPE_RECT);
  FeynmanKacSolverGPU::Register_Distance(&circulo, FK_SHAPE_CIRCLE);
  FeynmanKacSolverGPU solver(0, std::strtoull(argv[2], nullptr, 10));
  BVP bvp;
  bvp.u.funcion = &franke_u;
  bvp.g.funcion = &franke_u;
  bvp.frontera_dominio.Distancia = &rectangulo;
  bvp.frontera_dominio.parametros = {0.0, 0.0, 1.0, 1.0};
  // point solve: no subdomain (unregistered distance)
  Vector2d X0;
  X0[0] = 0.31;
  X0[1] = 0.4;
  solver.Solve_OMP_Analytic(X0, 2000, 1e-3, 0.1, bvp);
  std::printf("point %.17g %.17g %.17g %.17g %.17g %.17g\n", solver.phi, solver.phiphi, solver.phi_VR, solver.APL,
              solver.RNGC, solver.xi);
  // exact-gradient control variate through BVP::F
  bvp.F.funcion = &franke_F;
  solver.Solve_OMP_Analytic(X0, 2000, 1e-3, 0.1, bvp);
  std::printf("pointcv %.17g %.17g %.17g\n", solver.phi, solver.phi_VR, solver.phiphi_VR);
  bvp.F.funcion = nullptr;
  // node solves on one arc
  std::ifstream in(argv[1]);
  Interfaz I;
  int n = 0;
  in >> I.centro[0] >> I.centro[1] >> I.radio >> I.c2 >> I.interior >> n;
  I.nudos_circunferencia.resize(n);
  for (int i = 0; i < n; ++i) in >> I.nudos_circunferencia[i].posicion_angular >> I.nudos_circunferencia[i].indice_global;
  I.iPsi.n = n;
  I.iPsi.a.resize(static_cast<size_t>(n) * n);
  for (auto& v : I.iPsi.a) in >> v;
  bvp.frontera_subdominio.Distancia = &circulo;
  bvp.frontera_subdominio.parametros = {I.radio, I.centro[0], I.centro[1]};
  int items = 0;
  in >> items;
  for (int k = 0; k < items; ++k) {
    Nudo nd;
    int fr = 0;
    in >> nd.posicion_cartesiana[0] >> nd.posicion_cartesiana[1] >> fr >> nd.indice_global;
    nd.frontera = fr != 0;
    solver.Solve_OMP_Analytic(nd, 500, 1e-3, 0.1, bvp, I);
    std::printf("node %d %.17g %.17g", nd.indice_global, nd.B, nd.frontera ? 0.0 : solver.phi);
    for (auto& kv : nd.G) std::printf(" %d:%.17g", kv.first, kv.second);
    std::printf("\n");
  }
  return 0;
}
