// spac_fk_gpu.hpp -- C++ drop-in for SpAc's FeynmanKacSolver on the GPU.
//
// FeynmanKacSolverGPU has the two Solve_OMP_Analytic entry points of
// FeynmanKacSolver (Solvers/FeynmanKacSolver.hpp:95-98) and fills the same
// public statistics (phi, phiphi, phi_VR, phiphi_VR, xi, xixi, xiphi, APL,
// RNGC, :80-83) and, for node solves, Nudo::G and Nudo::B in place, so a
// driver loop such as main_test_serial.cpp:54-62 runs unchanged with the
// solver object swapped.  It is header-only over the C ABI of libspac_fk
// (spac_fk.h) and is written against the reference's public members only:
// BVP (BVP/BVP.hpp:17-28), Frontera (BVP/Frontera.hpp:15-38), Nudo
// (Mesh/Nudo.hpp:33-55) and Interfaz (Mesh/Interfaz.hpp:14-37).  The member
// functions are templates over those classes, so the header compiles against
// the reference's own headers or any types with the same public members.
//
// Coefficient functions are host function pointers in the reference; a GPU
// cannot call them, so each BVP is matched to a compiled device functor set
// through a registry keyed by the pointers themselves:
//   Register_Problem(u, problem, F_exact)  u's function -> FK_PROBLEM_*;
//       F_exact (optional) is the function whose presence in BVP::F selects
//       the exact-gradient control variate (F = -sigma^T grad u);
//   Register_Distance(distance, shape)     Frontera::Distancia -> FK_SHAPE_*.
// An unregistered pointer is an error (std::runtime_error), never a silent
// CPU path.  Frontera::parametros are passed as they are: (x0, y0, x1, y1)
// for rectangles, (r, cx, cy) for circles.  A subdomain Frontera whose
// distance function is not registered is treated as "no subdomain" (point
// solves stop at the domain boundary).
// Reflecting sides: on a rectangular domain, Frontera::Absorbente is
// evaluated at the midpoint of each side (the device functors take one
// boundary type per side); sides where it is false reflect, which needs a u
// registered as FK_PROBLEM_ROBIN (prob[1] = varphi).  The side mask and the
// call's rho (the width of the zone where the reflecting step runs) are then
// passed in prob[0] and prob[2]; absorbing problems ignore rho.
#ifndef SPAC_FK_GPU_HPP
#define SPAC_FK_GPU_HPP
#include <cmath>
#include <cstdint>
#include <map>
#include <stdexcept>
#include <string>
#include <tuple>
#include <type_traits>
#include <vector>

#include "spac_fk.h"

namespace spac_fk_gpu {

struct ProblemBinding {
  int problem;
  std::uintptr_t F_exact;
  double prob[4];
};

inline std::map<std::uintptr_t, ProblemBinding>& problem_registry() {
  static std::map<std::uintptr_t, ProblemBinding> m;
  return m;
}
inline std::map<std::uintptr_t, int>& distance_registry() {
  static std::map<std::uintptr_t, int> m;
  return m;
}
template <class Fn>
std::uintptr_t key_of(Fn f) {
  return reinterpret_cast<std::uintptr_t>(f);
}

// argument type of a boundary-type predicate (Frontera::pftipo)
template <class T>
struct predicate_arg;
template <class R, class A>
struct predicate_arg<R (*)(A)> {
  using type = typename std::decay<A>::type;
};

// Reflecting sides of a rectangular domain (x0, y0, x1, y1): bit s set where
// Frontera::Absorbente is false at the midpoint of side s (0: x = x0,
// 1: y = y0, 2: x = x1, 3: y = y1; Frontera.hpp:23-36).
template <class FronteraT>
int reflecting_sides(const FronteraT& fr, const double d[4]) {
  if (!fr.Absorbente) return 0;
  using V = typename predicate_arg<decltype(fr.Absorbente)>::type;
  const double mid[4][2] = {{d[0], 0.5 * (d[1] + d[3])}, {0.5 * (d[0] + d[2]), d[1]},
                            {d[2], 0.5 * (d[1] + d[3])}, {0.5 * (d[0] + d[2]), d[3]}};
  int mask = 0;
  for (int s = 0; s < 4; ++s) {
    V p;
    p[0] = mid[s][0];
    p[1] = mid[s][1];
    if (!fr.Absorbente(p)) mask |= 1 << s;
  }
  return mask;
}

// Frontera -> (shape, parameters) through the distance registry.
template <class FronteraT>
bool shape_of(const FronteraT& fr, int* shape, double p[4], bool required) {
  auto& reg = distance_registry();
  const auto f = reg.find(key_of(fr.Distancia));
  if (f == reg.end()) {
    if (required) throw std::runtime_error("spac_fk_gpu: unregistered Frontera distance function");
    return false;
  }
  *shape = f->second;
  const size_t np = fr.parametros.size();
  if ((*shape == FK_SHAPE_RECT && np < 4) || (*shape == FK_SHAPE_CIRCLE && np < 3))
    throw std::runtime_error("spac_fk_gpu: Frontera parameters too short for its shape");
  for (size_t i = 0; i < 4; ++i) p[i] = i < np ? fr.parametros[i] : 0.0;
  return true;
}

// BVP -> fk_bvp_desc through the problem registry (u's function) and BVP::F
// (the exact-gradient control variate when it is the registered F_exact).
// need_domain: the domain's distance function must be registered.
template <class BVPT>
fk_bvp_desc describe_bvp(const BVPT& P, bool need_domain, double rho = 0.0) {
  auto& reg = problem_registry();
  const auto f = reg.find(key_of(P.u.funcion));
  if (f == reg.end()) throw std::runtime_error("spac_fk_gpu: unregistered BVP (its u function)");
  const ProblemBinding& b = f->second;
  fk_bvp_desc d;
  d.problem = b.problem;
  d.cv = (b.F_exact != 0 && key_of(P.F.funcion) == b.F_exact) ? FK_CV_EXACT : FK_CV_NONE;
  d.mlp_id = -1;
  if (!shape_of(P.frontera_dominio, &d.dom_shape, d.dom, need_domain)) {
    // no registered domain and none needed (the disk solve never reads it):
    // a unit domain of the shape the problem functor expects
    d.dom_shape = (b.problem == FK_PROBLEM_DISK) ? FK_SHAPE_CIRCLE : FK_SHAPE_RECT;
    const double unit_rect[4] = {0.0, 0.0, 1.0, 1.0}, unit_circle[4] = {1.0, 0.0, 0.0, 0.0};
    for (int i = 0; i < 4; ++i) d.dom[i] = (d.dom_shape == FK_SHAPE_CIRCLE) ? unit_circle[i] : unit_rect[i];
  }
  for (int i = 0; i < 4; ++i) d.prob[i] = b.prob[i];
  const int mask = d.dom_shape == FK_SHAPE_RECT ? reflecting_sides(P.frontera_dominio, d.dom) : 0;
  if (mask != 0 && b.problem != FK_PROBLEM_ROBIN)
    throw std::runtime_error("spac_fk_gpu: reflecting domain sides need a problem registered as FK_PROBLEM_ROBIN");
  if (b.problem == FK_PROBLEM_ROBIN) {
    d.prob[0] = mask;
    d.prob[2] = rho;
  }
  return d;
}

}  // namespace spac_fk_gpu

class FeynmanKacSolverGPU {
 public:
  // public statistics of FeynmanKacSolver after Update() (FeynmanKacSolver.hpp:72-83)
  double h = 0.0, sqrth = 0.0;
  unsigned int N = 0;
  double eps = 0.0;
  double phi = 0.0, phiphi = 0.0, phi_VR = 0.0, phiphi_VR = 0.0, xi = 0.0, xixi = 0.0, xiphi = 0.0, APL = 0.0,
         RNGC = 0.0;
  // stepping precision of the paths: FK_FP64 (the reference's arithmetic) or FK_FP32
  int precision = FK_FP64;

  // device: CUDA device ordinal; seed: Philox key.  MPIrank offsets the random
  // stream as the reference offsets its generators per rank
  // (FeynmanKacSolver.cpp:119,134).
  explicit FeynmanKacSolverGPU(int device = 0, unsigned long long seed = 0, unsigned int MPIrank = 0) {
    const int rc = fk_create(&ctx_, device, seed + (static_cast<unsigned long long>(MPIrank) << 32));
    if (rc != FK_OK) throw std::runtime_error("FeynmanKacSolverGPU: fk_create failed (no usable CUDA device?)");
  }
  ~FeynmanKacSolverGPU() {
    if (ctx_) fk_destroy(ctx_);
  }
  FeynmanKacSolverGPU(const FeynmanKacSolverGPU&) = delete;
  FeynmanKacSolverGPU& operator=(const FeynmanKacSolverGPU&) = delete;

  template <class ScalarFn, class VectorFn = std::nullptr_t>
  static void Register_Problem(ScalarFn u, int problem, VectorFn F_exact = nullptr, const double* prob = nullptr) {
    spac_fk_gpu::ProblemBinding b{problem, F_exact ? spac_fk_gpu::key_of(F_exact) : 0u, {0, 0, 0, 0}};
    if (prob)
      for (int i = 0; i < 4; ++i) b.prob[i] = prob[i];
    spac_fk_gpu::problem_registry()[spac_fk_gpu::key_of(u)] = b;
  }
  template <class DistanceFn>
  static void Register_Distance(DistanceFn distance, int shape) {
    spac_fk_gpu::distance_registry()[spac_fk_gpu::key_of(distance)] = shape;
  }

  fk_ctx* context() const { return ctx_; }

  // Solve_OMP_Analytic(Eigen::Vector2d X0, N, h, rho, BVP)  (FeynmanKacSolver.cpp:335-342)
  template <class Vec2, class BVPT>
  void Solve_OMP_Analytic(const Vec2& X0, unsigned int numero_trayectorias, double discretizacion_temporal,
                          double rho, const BVPT& Problema) {
    const int bvp = bvp_id(Problema, rho);
    int sub_shape = -1;
    double sub[4] = {0, 0, 0, 0};
    const bool has_sub = shape_of(Problema.frontera_subdominio, &sub_shape, sub, false);
    const double xy[2] = {X0[0], X0[1]};
    const unsigned paths = numero_trayectorias;
    const double hh = discretizacion_temporal;
    fk_stats st;
    check(fk_solve_points(ctx_, bvp, 1, xy, &paths, &hh, has_sub ? &sub_shape : nullptr, has_sub ? sub : nullptr,
                          precision, &st));
    set_stats(st, numero_trayectorias, discretizacion_temporal);
  }

  // Solve_OMP_Analytic(Nudo&, N, h, rho, BVP, Interfaz)  (FeynmanKacSolver.cpp:344-355)
  template <class NudoT, class BVPT, class InterfazT>
  void Solve_OMP_Analytic(NudoT& nudo, unsigned int numero_trayectorias, double discretizacion_temporal, double rho,
                          const BVPT& Problema, const InterfazT& interfaz) {
    const int bvp = bvp_id(Problema, rho);
    const int n = static_cast<int>(interfaz.nudos_circunferencia.size());
    std::vector<double> theta(n);
    std::vector<int> gids(n);
    for (int i = 0; i < n; ++i) {
      theta[i] = interfaz.nudos_circunferencia[i].posicion_angular;
      gids[i] = interfaz.nudos_circunferencia[i].indice_global;
    }
    const int arc = arc_id(interfaz, theta, gids);
    fk_node_item it;
    it.x = nudo.posicion_cartesiana[0];
    it.y = nudo.posicion_cartesiana[1];
    it.h = discretizacion_temporal;
    it.paths = numero_trayectorias;
    it.frontera = nudo.frontera ? 1 : 0;
    it.row = nudo.indice_global;
    it.stencil = arc;
    std::vector<double> G(n);
    double B = 0.0;
    fk_stats st;
    check(fk_solve_nodes_arc(ctx_, bvp, 1, &it, precision, G.data(), &B, &st));
    nudo.B = B;
    if (!nudo.frontera) {
      for (int i = 0; i < n; ++i) nudo.G[gids[i]] = G[i];
      set_stats(st, numero_trayectorias, discretizacion_temporal);
    }
  }

 private:
  fk_ctx* ctx_ = nullptr;
  std::map<std::tuple<int, int, int, double, double, double, double, double, double, double, double>, int> bvps_;
  std::map<std::tuple<double, double, double, double, int, int, int>, int> arcs_;

  void check(int rc) {
    if (rc != FK_OK && rc != FK_ERR_STEP_CAP)
      throw std::runtime_error(std::string("FeynmanKacSolverGPU: ") + fk_last_error(ctx_));
  }

  template <class FronteraT>
  static bool shape_of(const FronteraT& fr, int* shape, double p[4], bool required) {
    return spac_fk_gpu::shape_of(fr, shape, p, required);
  }

  template <class BVPT>
  int bvp_id(const BVPT& P, double rho) {
    const fk_bvp_desc d = spac_fk_gpu::describe_bvp(P, true, rho);
    const auto key = std::make_tuple(d.problem, d.cv, d.dom_shape, d.dom[0], d.dom[1], d.dom[2], d.dom[3], d.prob[0],
                                     d.prob[1], d.prob[2], d.prob[3]);
    const auto it = bvps_.find(key);
    if (it != bvps_.end()) return it->second;
    int id = -1;
    check(fk_register_bvp(ctx_, &d, &id));
    bvps_[key] = id;
    return id;
  }

  template <class InterfazT>
  int arc_id(const InterfazT& I, const std::vector<double>& theta, const std::vector<int>& gids) {
    const int n = static_cast<int>(theta.size());
    const auto key = std::make_tuple(static_cast<double>(I.centro[0]), static_cast<double>(I.centro[1]),
                                     static_cast<double>(I.radio), static_cast<double>(I.c2), I.interior, n,
                                     n > 0 ? gids[0] : -1);
    const auto it = arcs_.find(key);
    if (it != arcs_.end()) return it->second;
    fk_arc_desc a;
    a.cx = I.centro[0];
    a.cy = I.centro[1];
    a.radius = I.radio;
    a.c2 = I.c2;
    a.interior = I.interior;
    a.n = n;
    a.theta = theta.data();
    a.gids = gids.data();
    // the interface's own iPsi (Interfaz::Calcula_Psi) when it has one
    a.iPsi = (static_cast<int>(I.iPsi.rows()) == n && n > 0) ? I.iPsi.data() : nullptr;
    int id = -1;
    check(fk_register_arc(ctx_, &a, &id));
    arcs_[key] = id;
    return id;
  }

  void set_stats(const fk_stats& s, unsigned int n, double hh) {
    N = n;
    h = hh;
    sqrth = std::sqrt(hh);
    phi = s.phi;
    phiphi = s.phiphi;
    phi_VR = s.phi_VR;
    phiphi_VR = s.phiphi_VR;
    xi = s.xi;
    xixi = s.xixi;
    xiphi = s.xiphi;
    APL = s.APL;
    RNGC = s.RNGC;
  }
};

// PseudoespectralCirculoSolver on the GPU (Solvers/PseudoespectralCirculoSolver.hpp:8-18):
// Inicializa records the disk, Resuelve(BVP, nudos_interior, nudos_periferia)
// fills nudos_interior[p].B and nudos_interior[p].G[periphery indice_global]
// as the reference does (PseudoespectralCirculoSolver.cpp:215-260), through
// fk_solve_disks_ps.  The BVP goes through the same registry as
// FeynmanKacSolverGPU (Register_Problem); its domain distance need not be
// registered.  The reference's Resuelve(BVP) (grid values of the Dirichlet
// problem with boundary data g, kept in interpolador.valores.z) has no
// counterpart: its solution table is not exposed.
class PseudoespectralCirculoSolverGPU {
 public:
  explicit PseudoespectralCirculoSolverGPU(int device = 0) {
    if (fk_create(&ctx_, device, 0) != FK_OK)
      throw std::runtime_error("PseudoespectralCirculoSolverGPU: fk_create failed (no usable CUDA device?)");
  }
  ~PseudoespectralCirculoSolverGPU() {
    if (ctx_) fk_destroy(ctx_);
  }
  PseudoespectralCirculoSolverGPU(const PseudoespectralCirculoSolverGPU&) = delete;
  PseudoespectralCirculoSolverGPU& operator=(const PseudoespectralCirculoSolverGPU&) = delete;

  // Inicializa(centro, radio, N_circunferencia, N_radio, theta_0, BVP)  (:2-189)
  template <class Vec2, class BVPT>
  void Inicializa(const Vec2& centro, double radio, unsigned int N_circunferencia, unsigned int N_radio,
                  double theta_0, const BVPT& Problema) {
    (void)Problema;
    cx_ = centro[0];
    cy_ = centro[1];
    radius_ = radio;
    n_circle_ = static_cast<int>(N_circunferencia);
    n_radial_ = static_cast<int>(N_radio);
    theta0_ = theta_0;
  }

  // Resuelve(BVP, nudos_interior, nudos_periferia)  (:215-260)
  template <class BVPT, class NudoT>
  void Resuelve(const BVPT& Problema, std::vector<NudoT>& nudos_interior, std::vector<NudoT> nudos_periferia) {
    const fk_bvp_desc desc = spac_fk_gpu::describe_bvp(Problema, false);
    const auto key = std::make_tuple(desc.problem, desc.prob[0], desc.prob[1], desc.prob[2], desc.prob[3]);
    auto found = bvps_.find(key);
    if (found == bvps_.end()) {
      int id = -1;
      check(fk_register_bvp(ctx_, &desc, &id));
      found = bvps_.emplace(key, id).first;
    }
    const int bvp = found->second;
    const int np = static_cast<int>(nudos_periferia.size()), ni = static_cast<int>(nudos_interior.size());
    std::vector<double> theta(np), xy(2 * static_cast<size_t>(ni)), G(static_cast<size_t>(ni) * np), B(ni);
    for (int i = 0; i < np; ++i) theta[i] = nudos_periferia[i].posicion_angular;
    for (int p = 0; p < ni; ++p) {
      xy[2 * p] = nudos_interior[p].posicion_cartesiana[0];
      xy[2 * p + 1] = nudos_interior[p].posicion_cartesiana[1];
    }
    fk_disk_desc d;
    d.cx = cx_;
    d.cy = cy_;
    d.radius = radius_;
    d.theta0 = theta0_;
    d.n_circle = n_circle_;
    d.n_radial = n_radial_;
    d.n_periph = np;
    d.periph_theta = theta.data();
    d.n_inner = ni;
    d.inner_xy = xy.data();
    check(fk_solve_disks_ps(ctx_, bvp, 1, &d, G.data(), B.data()));
    for (int p = 0; p < ni; ++p) {
      nudos_interior[p].B = B[p];
      for (int i = 0; i < np; ++i) nudos_interior[p].G[nudos_periferia[i].indice_global] = G[static_cast<size_t>(p) * np + i];
    }
  }

  fk_ctx* context() const { return ctx_; }

 private:
  fk_ctx* ctx_ = nullptr;
  std::map<std::tuple<int, double, double, double, double>, int> bvps_;  // registered problems
  double cx_ = 0.0, cy_ = 0.0, radius_ = 0.0, theta0_ = 0.0;
  int n_circle_ = 0, n_radial_ = 0;

  void check(int rc) {
    if (rc != FK_OK) throw std::runtime_error(std::string("PseudoespectralCirculoSolverGPU: ") + fk_last_error(ctx_));
  }
};

#endif
