// CPU oracle for SpAc's Feynman-Kac hot path -- TEST INFRASTRUCTURE ONLY.
//
// Scalar FP64 restatement of the reference algorithm, written for this
// project.  Each function names the reference lines it follows.  In
// sequential-stream mode it reproduces the reference compiled against
// oracle/shim bit for bit (same operation order, -ffp-contract=off); in
// Philox mode it follows the GPU kernels' random stream.  The product library
// never links or calls this file.
#include "fk_oracle.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <random>
#include <vector>

namespace {

const double kTwoPi = 6.283185307179586;
const double kInv32 = 2.3283064365386962890625e-10;  // 2^-32
const double kGobet = -0.5826;                       // FeynmanKacSolver.cpp:169,184

// ---------------------------------------------------------------- Philox -----
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
// as 1, 2, 3", SC'11): 10 rounds of two 32x32->64 multiplies with Weyl key bumps.
void philox(const uint32_t in[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c0 = in[0], c1 = in[1], c2 = in[2], c3 = in[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = static_cast<uint64_t>(0xD2511F53u) * c0;
    uint64_t p1 = static_cast<uint64_t>(0xCD9E8D57u) * c2;
    uint32_t hi0 = static_cast<uint32_t>(p0 >> 32), lo0 = static_cast<uint32_t>(p0);
    uint32_t hi1 = static_cast<uint32_t>(p1 >> 32), lo1 = static_cast<uint32_t>(p1);
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n1 = lo1;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    uint32_t n3 = lo0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

struct Session {
  int mode;
  uint64_t seed;
  uint32_t stream = 0;
  std::mt19937 mt;  // sequential mode: the shim's boost::mt19937 stream
  Session(int m, uint64_t s) : mode(m), seed(s), mt(5489u) {}

  // Shim normal_distribution<double> (oracle/shim/boost/random.hpp):
  // Box-Muller from two 32-bit words, cosine branch, mean + sigma * z.
  double seq_normal() {
    uint32_t a = static_cast<uint32_t>(mt());
    uint32_t b = static_cast<uint32_t>(mt());
    double u1 = (static_cast<double>(a) + 0.5) * kInv32;
    double u2 = (static_cast<double>(b) + 0.5) * kInv32;
    double z = std::sqrt(-2.0 * std::log(u1)) * std::cos(kTwoPi * u2);
    return 0.0 + 1.0 * z;
  }
};

// Brownian increment for step k of a path (Actualiza_Incremento,
// FeynmanKacSolver.cpp:2-6).  Philox mode: counter (k, path, item, stream),
// key (seed lo, seed hi); words (r0, r1) feed the step's Box-Muller pair.
void increment(Session& S, uint32_t item, uint32_t path, int k, double sqrth, double dW[2]) {
  if (S.mode == ORC_RNG_SEQUENTIAL) {
    dW[0] = sqrth * S.seq_normal();
    dW[1] = sqrth * S.seq_normal();
    return;
  }
  uint32_t ctr[4] = {static_cast<uint32_t>(k), path, item, S.stream};
  uint32_t key[2] = {static_cast<uint32_t>(S.seed), static_cast<uint32_t>(S.seed >> 32)};
  uint32_t r[4];
  philox(ctr, key, r);
  uint32_t a = r[0];
  uint32_t b = r[1];
  double u1 = (static_cast<double>(a) + 0.5) * kInv32;
  double u2 = (static_cast<double>(b) + 0.5) * kInv32;
  double rad = std::sqrt(-2.0 * std::log(u1));
  double ang = kTwoPi * u2;
  dW[0] = sqrth * (rad * std::cos(ang));
  dW[1] = sqrth * (rad * std::sin(ang));
}

// ------------------------------------------------- small 2-D linear algebra --
// Same coefficient order as the shim's Eigen products.
struct V2 { double x, y; };
struct M2 { double a00, a01, a10, a11; };
inline double dot(V2 a, V2 b) { double s = 0.0; s += a.x * b.x; s += a.y * b.y; return s; }
inline double norm(V2 a) { double s = 0.0; s += a.x * a.x; s += a.y * a.y; return std::sqrt(s); }
inline V2 mul(M2 m, V2 v) { return V2{m.a00 * v.x + m.a01 * v.y, m.a10 * v.x + m.a11 * v.y}; }
// row vector N^T times matrix
inline V2 tmul(V2 n, M2 m) { return V2{n.x * m.a00 + n.y * m.a10, n.x * m.a01 + n.y * m.a11}; }

// ------------------------------------------------------------ boundaries ----
// Circulo (Dominios/Circulo.hpp:7-22): params [r, cx, cy]; distance negative inside.
double circulo(const double* p, V2 X, V2& exitp, V2& nrm) {
  nrm.x = X.x - p[1];
  nrm.y = X.y - p[2];
  double r = norm(nrm);
  r = std::max(5E-4, r);
  nrm.x = nrm.x / r;
  nrm.y = nrm.y / r;
  exitp.x = nrm.x * p[0] + p[1];
  exitp.y = nrm.y * p[0] + p[2];
  return r - p[0];
}

// Rectangulo (Dominios/Rectangulo.hpp:7-229): params [x0, y0, x1, y1].  The
// four quadrant branches of the reference collapse to one with signs sx, sy
// (a point on a centre line belongs to the lower/left quadrant, as there).
// Inside: the side with the larger (dx - hx) vs (dy - hy) wins, ties go to
// the horizontal side.  Outside: corner if both offsets exceed the half
// sides (diagonal normal 0.70710678118f as a float literal), else the side.
double rectangulo(const double* p, V2 X, V2& exitp, V2& nrm) {
  const double kDiag = static_cast<double>(0.70710678118f);
  double cx = 0.5 * (p[0] + p[2]), cy = 0.5 * (p[1] + p[3]);
  double hx = p[2] - cx, hy = p[3] - cy;
  double dx = std::fabs(X.x - cx), dy = std::fabs(X.y - cy);
  double sx = (X.x > cx) ? 1.0 : -1.0;
  double sy = (X.y > cy) ? 1.0 : -1.0;
  exitp = X;
  if ((dx <= hx) && (dy <= hy)) {
    if (dx - hx > dy - hy) {
      exitp.x = (sx > 0) ? hx + cx : -hx + cx;
      nrm.x = sx; nrm.y = 0.0;
      return dx - hx;
    }
    exitp.y = (sy > 0) ? hy + cy : -hy + cy;
    nrm.x = 0.0; nrm.y = sy;
    return dy - hy;
  }
  if (dx > hx) {
    if (dy > hy) {
      double r = std::sqrt((dx - hx) * (dx - hx) + (dy - hy) * (dy - hy));
      exitp.x = (sx > 0) ? hx + cx : -hx + cx;
      exitp.y = (sy > 0) ? hy + cy : -hy + cy;
      nrm.x = sx * kDiag; nrm.y = sy * kDiag;
      return r;
    }
    exitp.x = (sx > 0) ? hx + cx : -hx + cx;
    nrm.x = sx; nrm.y = 0.0;
    return dx - hx;
  }
  exitp.y = (sy > 0) ? hy + cy : -hy + cy;
  nrm.x = 0.0; nrm.y = sy;
  return dy - hy;
}

double shape_dist(int shape, const double* p, V2 X, V2& e, V2& n) {
  return shape == ORC_SHAPE_CIRCLE ? circulo(p, X, e, n) : rectangulo(p, X, e, n);
}

// ------------------------------------------------------------- problems -----
struct Coef {
  double u, g, c, f;
  V2 b, F;
  M2 s;
};

// Franke test function and its derivatives as written in BVPs/Franke_Poisson.hpp:4-60
// (each exponential evaluated once; the reference re-evaluates identical
// expressions, which gives identical values).
struct Franke {
  double e1, e2, e3, e4, x, y;
  explicit Franke(double X, double Y) : x(X), y(Y) {
    e1 = std::exp(-0.25 * (std::pow(9.0 * x - 2.0, 2) + std::pow(9.0 * y - 2.0, 2)));
    e2 = std::exp((-1.0 / 49.0) * std::pow(9.0 * x + 1.0, 2) - 0.1 * (9.0 * y + 1.0));
    e3 = std::exp(-0.25 * (std::pow(9.0 * x - 7.0, 2) + std::pow(9.0 * y - 3.0, 2)));
    e4 = std::exp(-1.0 * (std::pow(9.0 * x - 4.0, 2) + std::pow(9.0 * y - 7.0, 2)));
  }
  double u() const { return 0.75 * e1 + 0.75 * e2 + 0.5 * e3 - 0.2 * e4; }
  double dudx() const {
    return -3.375 * (9.0 * x - 2.0) * e1 - (27.0 / 98.0) * (9.0 * x + 1.0) * e2 -
           2.25 * (9.0 * x - 7.0) * e3 + 3.6 * (9.0 * x - 4) * e4;
  }
  double dudy() const {
    return -3.375 * (9.0 * y - 2.0) * e1 - 0.675 * e2 - 2.25 * (9.0 * y - 3.0) * e3 +
           3.6 * (9.0 * y - 7.0) * e4;
  }
  double d2udx2() const {
    return -3.375 * (9.0 - 4.5 * std::pow(9.0 * x - 2.0, 2)) * e1 -
           (27.0 / 98.0) * (9.0 - (18.0 / 49.0) * std::pow(9.0 * x + 1.0, 2)) * e2 -
           2.25 * (9.0 - 4.5 * std::pow(9.0 * x - 7.0, 2)) * e3 +
           3.6 * (9.0 - 18.0 * std::pow(9.0 * x - 4.0, 2)) * e4;
  }
  double d2udy2() const {
    return -3.375 * (9.0 - 4.5 * std::pow((9.0 * y - 2.0), 2)) * e1 + (243.0 / 400.0) * e2 -
           2.25 * (9.0 - 4.5 * std::pow(9.0 * y - 3.0, 2)) * e3 +
           3.6 * (9.0 - 18.0 * std::pow(9.0 * y - 7.0, 2)) * e4;
  }
};

// The Monegros solution u and its derivatives, the same in
// BVPs/Monegros_Revamped.hpp:4-40 and BVPs/Monegros_Poisson.hpp:4-40.
const double mk1 = 1.0, mk2 = 0.01, mk3 = 0.02, mk4 = 0.12, mk5 = 0.05, mk6 = 0.05, mk7 = -0.12, msf = 0.333;
double mon_u(double x, double y) {
  return 3.0 + msf * (std::sin(std::sqrt(mk1 + mk2 * x * x + mk3 * y * y)) +
                      std::tanh(std::sin(mk4 * x + mk5 * y) + std::sin(mk6 * x + mk7 * y)));
}
double mon_dudx(double x, double y) {
  return msf * ((std::cos(std::sqrt(mk1 + mk2 * x * x + mk3 * y * y)) * mk2 * x /
                 std::sqrt(mk1 + mk2 * x * x + mk3 * y * y)) -
                (mk4 * std::cos(mk4 * x + mk5 * y) + mk6 * std::cos(mk6 * x + mk7 * y)) *
                    (std::pow(std::tanh(std::sin(mk4 * x + mk5 * y) + std::sin(mk6 * x + mk7 * y)), 2) - 1));
}
double mon_dudy(double x, double y) {
  return msf * (std::cos(std::sqrt(mk1 + mk2 * x * x + mk3 * y * y)) * mk1 * mk3 * y /
                    std::sqrt(mk1 + mk2 * x * x + mk3 * y * y) -
                (mk5 * std::cos(mk4 * x + mk5 * y) + mk7 * std::cos(mk6 * x + mk7 * y)) *
                    (std::pow(std::tanh(std::sin(mk4 * x + mk5 * y) + std::sin(mk6 * x + mk7 * y)), 2) - 1));
}
double mon_d2udx2(double x, double y) {
  double aux1 = std::sqrt(mk1 + mk2 * x * x + mk3 * y * y),
         aux2 = std::tanh(std::sin(mk4 * x + mk5 * y) + std::sin(mk6 * x + mk7 * y));
  return msf * (((mk2 / aux1) - (mk2 * mk2 * x * x / std::pow(aux1, 3))) * std::cos(aux1) -
                (x * x * mk2 * mk2 / (aux1 * aux1)) * std::sin(aux1) +
                2.0 * std::pow(mk4 * std::cos(mk4 * x + mk5 * y) + mk6 * std::cos(mk6 * x + mk7 * y), 2) *
                    (std::pow(aux2, 2) - 1) * aux2 +
                (mk4 * mk4 * std::sin(mk4 * x + mk5 * y) + mk6 * mk6 * std::sin(mk6 * x + mk7 * y)) *
                    (std::pow(aux2, 2) - 1));
}
double mon_d2udy2(double x, double y) {
  double aux1 = std::sqrt(mk1 + mk2 * x * x + mk3 * y * y),
         aux2 = std::tanh(std::sin(mk4 * x + mk5 * y) + std::sin(mk6 * x + mk7 * y));
  return msf * (((mk3 / aux1) - (mk3 * mk3 * y * y / std::pow(aux1, 3))) * std::cos(aux1) -
                (y * y * mk3 * mk3 / (aux1 * aux1)) * std::sin(aux1) +
                2.0 * std::pow(mk5 * std::cos(mk4 * x + mk5 * y) + mk7 * std::cos(mk6 * x + mk7 * y), 2) *
                    (std::pow(aux2, 2) - 1) * aux2 +
                (mk5 * mk5 * std::sin(mk4 * x + mk5 * y) + mk7 * mk7 * std::sin(mk6 * x + mk7 * y)) *
                    (std::pow(aux2, 2) - 1));
}

// Anisotropic problem on [0,1]^2 (defined with the reference's BVP API in
// oracle/ref_harness.cpp): a = 1 + 0.5 sin(2 pi x) sin(2 pi y),
// sigma = sqrt(2a) I, b = (y - 1/2, 1/2 - x), c = -(1 + x^2 + y^2),
// u = Franke (1 + x y), f = -(a Lap u + b.grad u + c u).
double aniso_a(double x, double y) {
  return 1.0 + 0.5 * std::sin(2.0 * M_PI * x) * std::sin(2.0 * M_PI * y);
}

double mlp_grad(const orc_mlp* m, double x, double y, double g[2], double* val);

// Tabulated grad u_hat (cv == 3).  The learned control variate has no
// counterpart in the reference; this is the library's own deployment of it
// (the FK_CV_MLP step interpolates its gradient table), restated in FP64 so
// that the GPU's FP64 stepping can be checked path for path: the point mapped
// to lattice units and clamped to [0, grid - 1 - 1e-3], then bilinear between
// the four surrounding lattice points.
void cv_table_grad(const orc_cv_table* T, double x, double y, double g[2]) {
  const int G = T->grid;
  const double sx = (G - 1) / (T->rect[2] - T->rect[0]), sy = (G - 1) / (T->rect[3] - T->rect[1]);
  double u = (x - T->rect[0]) * sx, v = (y - T->rect[1]) * sy;
  u = std::fmin(std::fmax(u, 0.0), static_cast<double>(G - 1) - 1e-3);
  v = std::fmin(std::fmax(v, 0.0), static_cast<double>(G - 1) - 1e-3);
  const int i = static_cast<int>(u), j = static_cast<int>(v);
  const double fu = u - i, fv = v - j;
  const float* t00 = T->tab + 2 * (static_cast<long>(j) * G + i);
  const float* t10 = t00 + 2;
  const float* t01 = t00 + 2 * G;
  const float* t11 = t01 + 2;
  for (int c = 0; c < 2; ++c)
    g[c] = (1.0 - fv) * ((1.0 - fu) * t00[c] + fu * t10[c]) + fv * ((1.0 - fu) * t01[c] + fu * t11[c]);
}

Coef coefficients(const orc_bvp* B, double x, double y) {
  Coef c;
  c.b = V2{0.0 * x, 0.0 * y};  // Vector_Defecto: position * 0.0
  c.F = V2{0.0 * x, 0.0 * y};
  if (B->problem == ORC_PROBLEM_FRANKE) {
    Franke fr(x, y);
    c.u = fr.u();
    c.g = c.u;
    c.c = -0.0;
    c.f = -fr.d2udx2() - fr.d2udy2();
    c.b = V2{0.0, 0.0};
    c.s = M2{1.41421356237, 0.0, 0.0, 1.41421356237};
    if (B->cv == 1) {
      V2 gr{fr.dudx(), fr.dudy()};
      M2 nt{-c.s.a00, -c.s.a10, -c.s.a01, -c.s.a11};  // -(sigma^T)
      c.F = mul(nt, gr);
    }
  } else if (B->problem == ORC_PROBLEM_MONEGROS || B->problem == ORC_PROBLEM_MONEGROS_POISSON) {
    c.u = mon_u(x, y);
    c.g = c.u;
    if (B->problem == ORC_PROBLEM_MONEGROS) {  // Monegros_Revamped.hpp:41-43,57-59
      c.c = -1.0;
      c.f = -mon_d2udx2(x, y) - mon_d2udy2(x, y) - c.c * c.u;
    } else {  // Monegros_Poisson.hpp:41-43,57-59
      c.c = -0.0;
      c.f = -mon_d2udx2(x, y) - mon_d2udy2(x, y);
    }
    c.b = V2{0.0, 0.0};
    c.s = M2{1.41421356237, 0.0, 0.0, 1.41421356237};
    if (B->cv == 1) {
      V2 gr{mon_dudx(x, y), mon_dudy(x, y)};
      M2 nt{-c.s.a00, -c.s.a10, -c.s.a01, -c.s.a11};
      c.F = mul(nt, gr);
    }
  } else if (B->problem == ORC_PROBLEM_ANISO || B->problem == ORC_PROBLEM_ROBIN) {
    Franke fr(x, y);
    double q = 1.0 + x * y;
    double F = fr.u(), Fx = fr.dudx(), Fy = fr.dudy(), Fxx = fr.d2udx2(), Fyy = fr.d2udy2();
    c.u = F * q;
    c.g = c.u;
    c.c = -(1.0 + x * x + y * y);
    c.b = V2{y - 0.5, 0.5 - x};
    double a = aniso_a(x, y);
    double s = std::sqrt(2.0 * a);
    c.s = M2{1.0 * s, 0.0 * s, 0.0 * s, 1.0 * s};  // Identity() * s
    double ux = Fx * q + F * y;
    double uy = Fy * q + F * x;
    double lap = (Fxx + Fyy) * q + 2.0 * (Fx * y + Fy * x);
    c.f = -(a * lap + c.b.x * ux + c.b.y * uy + c.c * c.u);
    if (B->cv == 1) {
      V2 gr{ux, uy};
      M2 nt{-c.s.a00, -c.s.a10, -c.s.a01, -c.s.a11};
      c.F = mul(nt, gr);
    }
  } else {  // ORC_PROBLEM_DISK: Franke rescaled to the disk (cx, cy, R)
    double cx = B->prob[0], cy = B->prob[1], R = B->prob[2];
    double inv = 1.0 / (2.0 * R);
    double xi = (x - cx) * inv + 0.5, eta = (y - cy) * inv + 0.5;
    Franke fr(xi, eta);
    c.u = fr.u();
    c.g = c.u;
    c.c = -0.0;
    c.f = -(fr.d2udx2() + fr.d2udy2()) * (inv * inv);
    c.b = V2{0.0, 0.0};
    c.s = M2{1.41421356237, 0.0, 0.0, 1.41421356237};
    if (B->cv == 1) {
      V2 gr{fr.dudx() * inv, fr.dudy() * inv};
      M2 nt{-c.s.a00, -c.s.a10, -c.s.a01, -c.s.a11};
      c.F = mul(nt, gr);
    }
  }
  if (B->cv == 2 && B->mlp) {
    double g[2], v;
    mlp_grad(static_cast<const orc_mlp*>(B->mlp), x, y, g, &v);
    // F = -sigma^T grad u_hat (the reference's control-variate hook)
    c.F = V2{-(c.s.a00 * g[0] + c.s.a10 * g[1]), -(c.s.a01 * g[0] + c.s.a11 * g[1])};
  }
  if (B->cv == 3 && B->mlp) {
    double g[2];
    cv_table_grad(static_cast<const orc_cv_table*>(B->mlp), x, y, g);
    c.F = V2{-(c.s.a00 * g[0] + c.s.a10 * g[1]), -(c.s.a01 * g[0] + c.s.a11 * g[1])};
  }
  return c;
}

// sigma alone (the same expressions as in coefficients())
M2 sigma_of(const orc_bvp* B, double x, double y) {
  if (B->problem == ORC_PROBLEM_ANISO || B->problem == ORC_PROBLEM_ROBIN) {
    double s = std::sqrt(2.0 * aniso_a(x, y));
    return M2{1.0 * s, 0.0 * s, 0.0 * s, 1.0 * s};
  }
  return M2{1.41421356237, 0.0, 0.0, 1.41421356237};
}

// ------------------------------------------------------------ exit rule -----
// Dentro (FeynmanKacSolver.cpp:68-106) for absorbing boundaries: the boundary
// with the larger signed distance wins (tie -> domain); the path stops once
// within the Gobet-Menozzi shifted band 0.5826 |N^T sigma| sqrt(h).
int dentro(const orc_bvp* B, int sub_shape, const double* sub, V2 X, double sqrth, V2& proj, V2& N) {
  V2 pa, na;
  double da = shape_dist(B->dom_shape, B->dom, X, pa, na);
  double d = shape_dist(sub_shape, sub, X, proj, N);
  if (da >= d) {
    d = da;
    proj = pa;
    N = na;
    M2 s = (d < 0.0) ? sigma_of(B, X.x, X.y) : sigma_of(B, proj.x, proj.y);
    return (d < kGobet * norm(tmul(N, s)) * sqrth) ? ORC_OUT_INSIDE : ORC_OUT_DOMAIN;
  }
  M2 s = (d < 0.0) ? sigma_of(B, X.x, X.y) : sigma_of(B, proj.x, proj.y);
  return (d < kGobet * norm(tmul(N, s)) * sqrth) ? ORC_OUT_INSIDE : ORC_OUT_SUBDOMAIN;
}

// ---------------------------------------------------- reflecting sides -----
// ORC_PROBLEM_ROBIN: psi = d_n u - varphi u at a boundary point with outward
// normal n (u = Franke (1 + x y)), so u solves the Robin problem.
double robin_psi(const orc_bvp* B, double x, double y, double nx, double ny) {
  Franke fr(x, y);
  double q = 1.0 + x * y;
  double F = fr.u();
  double ux = fr.dudx() * q + F * y, uy = fr.dudy() * q + F * x;
  return nx * ux + ny * uy - B->prob[1] * (F * q);
}

// Whether the domain can ever win Dentro's comparison: not when the
// subdomain lies strictly inside the rectangular domain (its distance is
// then always the larger).  Reflection only happens where it can.
bool dom_can_win(const orc_bvp* B, int sub_shape, const double* s) {
  const double* d = B->dom;
  if (B->dom_shape != ORC_SHAPE_RECT) return true;
  if (sub_shape == ORC_SHAPE_CIRCLE)
    return !(s[1] - s[0] > d[0] && s[1] + s[0] < d[2] && s[2] - s[0] > d[1] && s[2] + s[0] < d[3]);
  return !(s[0] > d[0] && s[1] > d[1] && s[2] < d[2] && s[3] < d[3]);
}

// Dentro's nearest boundary at X, if it is a reflecting side of the domain
// (0: x = x0, 1: y = y0, 2: x = x1, 3: y = y1; -1 otherwise), and the domain
// distance.
int robin_side(const orc_bvp* B, int sub_shape, const double* sub, int mask, V2 X, double* dist) {
  V2 pa, na, ps, ns;
  double da = shape_dist(B->dom_shape, B->dom, X, pa, na);
  double d = shape_dist(sub_shape, sub, X, ps, ns);
  *dist = da;
  if (!(da >= d)) return -1;
  int side = (na.x == -1.0) ? 0 : (na.y == -1.0) ? 1 : (na.x == 1.0) ? 2 : (na.y == 1.0) ? 3 : -1;
  return (side >= 0 && ((mask >> side) & 1)) ? side : -1;
}

// One path: Simulacion_OMP loop body (FeynmanKacSolver.cpp:161-194) with
// Paso_Absorbente (:7-18), and for ORC_PROBLEM_ROBIN the reflecting step
// Paso_Reflejante (:19-67) near reflecting sides.  The reference's reflecting
// step reads two uninitialised values (the proposal's projection Nprop in
// its loop test, :46, and dist_k on a path's first step, :158), draws
// omega ~ Exp(1) where its comment states mean 2h (:33) and clamps an inside
// distance to zero (:39); it is restated as the scheme it implements,
// Lepingle's reflected Euler step: on every reflecting side within rho of
// the current point, the push-back is the exact maximum of the Brownian
// bridge of the normal displacement, 1/2 (uc + sqrt(uc^2 + 2 s^2 h E)),
// E ~ Exp(1), started from the point's distance to the side (the normals
// are coordinate axes and sigma = s I, so corner pushes are independent).
// A reflecting side crossed all the same puts the path back on it with the
// overshoot as local time (:49-58); psi is taken at the side's point nearest
// the new position.  The Exp(1) variate of side q is word q of Philox counter
// (2^31 | k, path, item, stream).
int simulate_robin(Session& S, const orc_bvp* B, int sub_shape, const double* sub, double x0, double y0,
                   double h, uint32_t item, uint32_t path, int max_steps, orc_exit* out) {
  if (S.mode != ORC_RNG_PHILOX) return -2;
  double sqrth = std::sqrt(h);
  V2 X{x0, y0}, proj{0, 0}, N{0, 0};
  double Y = 1, Z = 0, xi = 0, t = 0;
  const double* d = B->dom;
  const int mask = dom_can_win(B, sub_shape, sub) ? (static_cast<int>(B->prob[0]) & 15) : 0;
  const double rphi = B->prob[1], rho = B->prob[2];
  dentro(B, sub_shape, sub, X, sqrth, proj, N);
  int status = ORC_OUT_INSIDE, k = 0;
  const uint32_t key[2] = {static_cast<uint32_t>(S.seed), static_cast<uint32_t>(S.seed >> 32)};
  do {
    Coef c = coefficients(B, X.x, X.y);
    double dW[2];
    increment(S, item, path, k, sqrth, dW);
    V2 inc{dW[0], dW[1]};
    const double s = c.s.a00;  // sigma = s I
    double xn = X.x + (c.b.x * h + s * dW[0]), yn = X.y + (c.b.y * h + s * dW[1]);
    double lt[4] = {0.0, 0.0, 0.0, 0.0}, ploc = 0.0, vloc = 0.0;
    if (mask) {
      uint32_t r[4] = {0, 0, 0, 0};
      bool drawn = false;
      for (int q = 0; q < 4; ++q) {
        if (!((mask >> q) & 1)) continue;
        double dq = q == 0 ? d[0] - X.x : (q == 1 ? d[1] - X.y : (q == 2 ? X.x - d[2] : X.y - d[3]));
        if (!(dq > -rho)) continue;
        if (!drawn) {
          uint32_t ctr[4] = {0x80000000u | static_cast<uint32_t>(k), path, item, S.stream};
          philox(ctr, key, r);
          drawn = true;
        }
        double E = -std::log((static_cast<double>(r[q]) + 0.5) * kInv32);
        double nx = q == 0 ? -1.0 : (q == 2 ? 1.0 : 0.0);
        double ny = q == 1 ? -1.0 : (q == 3 ? 1.0 : 0.0);
        double uc = s * (nx * dW[0] + ny * dW[1]) + (nx * c.b.x + ny * c.b.y) * h;
        double nu = 0.5 * (uc + std::sqrt(uc * uc + 2.0 * s * s * h * E));
        double L = std::max(0.0, nu + std::min(dq, 0.0));
        xn -= L * nx;
        yn -= L * ny;
        lt[q] = L;
      }
      for (int q = 0; q < 4; ++q) {
        if (!((mask >> q) & 1)) continue;
        double o = q == 0 ? d[0] - xn : (q == 1 ? d[1] - yn : (q == 2 ? xn - d[2] : yn - d[3]));
        if (o > 0.0) {
          if (q == 0) xn = d[0]; else if (q == 1) yn = d[1]; else if (q == 2) xn = d[2]; else yn = d[3];
          lt[q] += o;
        }
      }
      for (int q = 0; q < 4; ++q) {
        if (lt[q] > 0.0) {
          double px = q == 0 ? d[0] : (q == 2 ? d[2] : std::min(std::max(xn, d[0]), d[2]));
          double py = q == 1 ? d[1] : (q == 3 ? d[3] : std::min(std::max(yn, d[1]), d[3]));
          double nx = q == 0 ? -1.0 : (q == 2 ? 1.0 : 0.0);
          double ny = q == 1 ? -1.0 : (q == 3 ? 1.0 : 0.0);
          ploc += robin_psi(B, px, py, nx, ny) * lt[q];
          vloc += rphi * lt[q];
        }
      }
    }
    Z += c.f * Y * h + ploc * Y;
    xi += Y * dot(c.F, inc);
    Y += c.c * Y * h + vloc * Y;
    X.x = xn;
    X.y = yn;
    t += h;
    ++k;
    status = dentro(B, sub_shape, sub, X, sqrth, proj, N);
    double dd;
    if (mask && robin_side(B, sub_shape, sub, mask, X, &dd) >= 0) {
      // the nearest boundary reflects: no stop there (dentro / reflejada,
      // :82-84), but a stop within the Gobet band of the nearer of the
      // subdomain and the absorbing sides
      double da = -FLT_MAX;
      int qa = -1;
      for (int q = 0; q < 4; ++q) {
        if ((mask >> q) & 1) continue;
        double dq = q == 0 ? d[0] - X.x : (q == 1 ? d[1] - X.y : (q == 2 ? X.x - d[2] : X.y - d[3]));
        if (dq > da) { da = dq; qa = q; }
      }
      int cand = ORC_OUT_DOMAIN;
      V2 pc{0, 0};
      if (qa >= 0) {
        pc.x = qa == 0 ? d[0] : (qa == 2 ? d[2] : std::min(std::max(X.x, d[0]), d[2]));
        pc.y = qa == 1 ? d[1] : (qa == 3 ? d[3] : std::min(std::max(X.y, d[1]), d[3]));
      } else {
        da = -FLT_MAX;
      }
      if (sub != B->dom) {
        // a subdomain boundary on the reflecting side (a tie the domain wins) is no candidate
        V2 ps, ns;
        double ds = shape_dist(sub_shape, sub, X, ps, ns);
        if (ds < dd && !(da >= ds)) { da = ds; pc = ps; cand = ORC_OUT_SUBDOMAIN; }
      }
      // the threshold of the reflecting side's test (sigma where Dentro takes it)
      M2 sg = (dd < 0.0) ? sigma_of(B, X.x, X.y) : sigma_of(B, proj.x, proj.y);
      const double thr = kGobet * norm(tmul(N, sg)) * sqrth;
      status = ORC_OUT_INSIDE;
      if (!(da < thr)) { status = cand; proj = pc; }
    }
  } while (status == ORC_OUT_INSIDE && k < max_steps);
  out->x = proj.x;
  out->y = proj.y;
  out->Y = Y;
  out->Z = Z;
  out->xi = xi;
  out->t = t;
  out->outcome = status;
  out->steps = k;
  return status == ORC_OUT_INSIDE ? -1 : 0;
}

// One path: Simulacion_OMP loop body (FeynmanKacSolver.cpp:161-194) with
// Paso_Absorbente (:7-18).  psi, varphi and mu are the reference's zero
// defaults; their terms are kept so the floating-point order is the same.
int simulate(Session& S, const orc_bvp* B, int sub_shape, const double* sub, double x0, double y0,
             double h, uint32_t item, uint32_t path, int max_steps, orc_exit* out) {
  if (B->problem == ORC_PROBLEM_ROBIN) return simulate_robin(S, B, sub_shape, sub, x0, y0, h, item, path, max_steps, out);
  double sqrth = std::sqrt(h);
  V2 X{x0, y0}, proj{0, 0}, N{0, 0};
  double Y = 1, Z = 0, xi = 0, t = 0, ji_t = 0;
  dentro(B, sub_shape, sub, X, sqrth, proj, N);  // status ignored, as in :169
  int status = ORC_OUT_INSIDE, k = 0;
  do {
    Coef c = coefficients(B, X.x, X.y);
    M2 sig = c.s;
    double dW[2];
    increment(S, item, path, k, sqrth, dW);
    V2 inc{dW[0], dW[1]};
    V2 mu{0.0 * X.x, 0.0 * X.y};
    double psi = 0.0, varphi = 0.0;
    Z += c.f * Y * h + psi * Y * ji_t;
    xi += Y * dot(c.F, inc);
    Y += c.c * Y * h + Y * dot(mu, inc) + varphi * Y * ji_t;
    V2 smu = mul(sig, mu), sdw = mul(sig, inc);
    V2 drift{(c.b.x - smu.x) * h, (c.b.y - smu.y) * h};
    X.x += drift.x + sdw.x;
    X.y += drift.y + sdw.y;
    t += h;
    ++k;
    status = dentro(B, sub_shape, sub, X, sqrth, proj, N);
  } while (status == ORC_OUT_INSIDE && k < max_steps);
  out->x = proj.x;
  out->y = proj.y;
  out->Y = Y;
  out->Z = Z;
  out->xi = xi;
  out->t = t;
  out->outcome = status;
  out->steps = k;
  return status == ORC_OUT_INSIDE ? -1 : 0;
}

// Branch-cut arctangents (Mesh/Nudo.hpp:7-32) and the arc-code dispatch of
// Interfaz::Update_G (Mesh/Interfaz.cpp:222-251).
double arc_theta(int interior, double dx, double dy) {
  double a = std::atan2(dy, dx);
  switch (interior) {
    case -11: case -22: case -4: return a;                               // Atan180
    case -33: case -44: case -2: return (a >= 0) ? a : a + 2.0 * M_PI;   // Atan0
    case -1: return (a <= -0.5 * M_PI) ? 2 * M_PI + a : a;               // Atan270
    case -3: return (a <= 0.5 * M_PI) ? 2.0 * M_PI + a : a;              // Atan90
    default: return std::nan("");
  }
}

inline double imq(double t, double tj, double c2) { return 1.0 / std::sqrt(std::pow(t - tj, 2) + c2); }

void gj_inverse(int n, std::vector<double>& a, std::vector<double>& inv) {
  inv.assign(static_cast<size_t>(n) * n, 0.0);
  for (int i = 0; i < n; ++i) inv[i + i * n] = 1.0;
  std::vector<int> piv(n);
  for (int k = 0; k < n; ++k) {
    int pr = k, pc = k;
    double best = -1.0;
    for (int i = k; i < n; ++i)
      for (int j = k; j < n; ++j) {
        double v = std::fabs(a[i + j * n]);
        if (v > best) { best = v; pr = i; pc = j; }
      }
    if (pr != k)
      for (int j = 0; j < n; ++j) { std::swap(a[k + j * n], a[pr + j * n]); std::swap(inv[k + j * n], inv[pr + j * n]); }
    if (pc != k)
      for (int i = 0; i < n; ++i) std::swap(a[i + k * n], a[i + pc * n]);
    piv[k] = pc;
    double p = a[k + k * n];
    for (int j = 0; j < n; ++j) { a[k + j * n] = a[k + j * n] / p; inv[k + j * n] = inv[k + j * n] / p; }
    for (int i = 0; i < n; ++i) {
      if (i == k) continue;
      double f = a[i + k * n];
      if (f == 0.0) continue;
      for (int j = 0; j < n; ++j) {
        a[i + j * n] = a[i + j * n] - f * a[k + j * n];
        inv[i + j * n] = inv[i + j * n] - f * inv[k + j * n];
      }
    }
  }
  for (int k = n - 1; k >= 0; --k)
    if (piv[k] != k)
      for (int j = 0; j < n; ++j) std::swap(inv[k + j * n], inv[piv[k] + j * n]);
}

// Statistics of Reduce_Analytic (FeynmanKacSolver.cpp:198-231, 266-274) and
// Update (:294-323), including the enum aliasing XiLinear2 == XiLinear that
// makes xi and xixi both hold sum(xi + xi^2)/N (FeynmanKacSolver.hpp:16-23).
struct Sums {
  double s[30];
  Sums() { for (double& v : s) v = 0.0; }
  void add(double score, double xi, unsigned rngcalls, double tau) {
    s[0] += score;
    s[4] += score * score;
    s[8] += xi;
    s[8] += xi * xi;
    s[12] += score + xi;
    s[16] += std::pow(score + xi, 2);
    s[20] += xi * (score);
    s[26] += rngcalls;
    s[24] += tau;
  }
  void finish(unsigned N, double out[9]) const {
    double n = static_cast<double>(N);
    // The merge into the solver's sums (:219-227, :281-289) adds the thread
    // sum of slot 8 twice, once as XiLinear and once as XiLinear2.
    double xi8 = s[8] + s[8];
    out[0] = s[0] / n; out[1] = s[4] / n; out[2] = s[12] / n; out[3] = s[16] / n;
    out[4] = xi8 / n; out[5] = xi8 / n; out[6] = s[20] / n; out[7] = s[24] / n;
    out[8] = s[26];
  }
};

int sub_of(const orc_bvp* B, const orc_shape* sub, int* shape, const double** p) {
  if (sub) { *shape = sub->shape; *p = sub->p; } else { *shape = B->dom_shape; *p = B->dom; }
  return 0;
}

const int kMaxSteps = 100000000;

// ---------------------------------------------------------------- MLP -------
inline double silu(double z) { return z / (1.0 + std::exp(-z)); }
inline double dsilu(double z) {
  double s = 1.0 / (1.0 + std::exp(-z));
  return s * (1.0 + z * (1.0 - s));
}

double mlp_forward(const orc_mlp* m, double x, double y, std::vector<double>* acts) {
  int W = m->width;
  double z0 = (x - m->in_lo[0]) * m->in_scale[0], z1 = (y - m->in_lo[1]) * m->in_scale[1];
  std::vector<double> p1(W), h1(W), p2(W), h2(W), p3(W), h3(W);
  for (int i = 0; i < W; ++i) { p1[i] = m->W1[i * 2] * z0 + m->W1[i * 2 + 1] * z1 + m->b1[i]; h1[i] = silu(p1[i]); }
  for (int i = 0; i < W; ++i) {
    double a = m->b2[i];
    for (int j = 0; j < W; ++j) a += m->W2[i * W + j] * h1[j];
    p2[i] = a; h2[i] = silu(a);
  }
  for (int i = 0; i < W; ++i) {
    double a = m->b3[i];
    for (int j = 0; j < W; ++j) a += m->W3[i * W + j] * h2[j];
    p3[i] = a; h3[i] = silu(a);
  }
  double o = m->b4[0];
  for (int j = 0; j < W; ++j) o += m->W4[j] * h3[j];
  if (acts) {
    acts->clear();
    acts->push_back(z0); acts->push_back(z1);
    for (auto* v : {&p1, &h1, &p2, &h2, &p3, &h3}) acts->insert(acts->end(), v->begin(), v->end());
  }
  return o;
}

// value and input gradient by forward-mode differentiation (tangents along x and y)
double mlp_grad(const orc_mlp* m, double x, double y, double g[2], double* val) {
  int W = m->width;
  double z0 = (x - m->in_lo[0]) * m->in_scale[0], z1 = (y - m->in_lo[1]) * m->in_scale[1];
  std::vector<double> h(W), tx(W), ty(W), nh(W), ntx(W), nty(W);
  for (int i = 0; i < W; ++i) {
    double p = m->W1[i * 2] * z0 + m->W1[i * 2 + 1] * z1 + m->b1[i];
    double d = dsilu(p);
    h[i] = silu(p);
    tx[i] = d * m->W1[i * 2] * m->in_scale[0];
    ty[i] = d * m->W1[i * 2 + 1] * m->in_scale[1];
  }
  const double* Ws[2] = {m->W2, m->W3};
  const double* bs[2] = {m->b2, m->b3};
  for (int l = 0; l < 2; ++l) {
    for (int i = 0; i < W; ++i) {
      double p = bs[l][i], px = 0, py = 0;
      for (int j = 0; j < W; ++j) { p += Ws[l][i * W + j] * h[j]; px += Ws[l][i * W + j] * tx[j]; py += Ws[l][i * W + j] * ty[j]; }
      double d = dsilu(p);
      nh[i] = silu(p); ntx[i] = d * px; nty[i] = d * py;
    }
    h.swap(nh); tx.swap(ntx); ty.swap(nty);
  }
  double o = m->b4[0], ox = 0, oy = 0;
  for (int j = 0; j < W; ++j) { o += m->W4[j] * h[j]; ox += m->W4[j] * tx[j]; oy += m->W4[j] * ty[j]; }
  g[0] = ox; g[1] = oy;
  if (val) *val = o;
  return o;
}

// ------------------------------------------------- pseudospectral disk -----
// Dense collocation operator of PseudoespectralCirculoSolver::Inicializa
// (Solvers/PseudoespectralCirculoSolver.cpp:2-189): Laplacian in polar
// coordinates on Nc equispaced angles x (N2+1) Chebyshev radii (half of the
// N_radio+1 points of a diameter, Trefethen's cheb.m), plus c(x) on the
// diagonal, the Nc rows of the outer ring replaced by identity rows.  Row and
// column index j*Nc + l: radius j, angle l.
struct PsDisk {
  int nc, nr, n2, n;
  double radius, theta0;
  std::vector<double> r, theta, L;  // L: n x n row-major
};

void ps_build(const orc_bvp* B, double cx, double cy, double radius, int nc, int nr, double theta0, PsDisk& P) {
  const int np = nr + 1;
  P.nc = nc; P.nr = nr; P.n2 = (nr - 1) / 2; P.radius = radius; P.theta0 = theta0;
  P.r.resize(np);
  std::vector<int> cw(np);
  for (int i = 0; i < np; ++i) {
    P.r[i] = radius * std::cos(M_PI * i / nr);
    cw[i] = static_cast<int>(((i == 0 || i == nr) ? 2 : 1) * std::pow(-1, i));
  }
  // cheb.m: D_ij = (c_i / c_j) / (r_i - r_j), diagonal = 1 - row sum (incl. its own 1)
  std::vector<double> D(static_cast<size_t>(np) * np);
  for (int i = 0; i < np; ++i) {
    for (int j = 0; j < np; ++j) {
      const double cij = cw[i] * (1.0 / cw[j]);
      D[i * np + j] = cij / ((P.r[i] - P.r[j]) + (i == j ? 1.0 : 0.0));
    }
    double s = 0.0;
    for (int j = 0; j < np; ++j) s += D[i * np + j];
    D[i * np + i] = D[i * np + i] - s;
  }
  std::vector<double> DD(static_cast<size_t>(np) * np);
  for (int i = 0; i < np; ++i)
    for (int j = 0; j < np; ++j) {
      double s = D[i * np] * D[j];
      for (int k = 1; k < np; ++k) s += D[i * np + k] * D[k * np + j];
      DD[i * np + j] = s;
    }
  const int m = P.n2 + 1, M2 = nc / 2;
  // radial blocks: A1 = D1 + R E1 (same radius), A2 = D2 + R E2 (mirrored radius), 1/r^2
  std::vector<double> A1(m * m), A2(m * m), rinv(m), r2inv(m);
  for (int i = 0; i < m; ++i) {
    rinv[i] = 1.0 / P.r[i];
    r2inv[i] = rinv[i] * rinv[i];
  }
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < m; ++j) {
      A1[i * m + j] = DD[i * np + j] + rinv[i] * D[i * np + j];
      A2[i * m + j] = DD[i * np + (nr - j)] + rinv[i] * D[i * np + (nr - j)];
    }
  // periodic second-derivative matrix (Toeplitz): D2t(l, l') = a((l' - l) mod Nc)
  const double dt = 2 * M_PI / nc;
  std::vector<double> a(nc);
  P.theta.resize(nc);
  for (int l = 0; l < nc; ++l) {
    P.theta[l] = l * dt + theta0;
    a[l] = (l == 0) ? -(M_PI * M_PI / (3 * dt * dt)) - (1.0 / 6)
                    : 0.5 * std::pow(-1, l + 1) / std::pow(std::sin(dt * l * 0.5), 2);
  }
  P.n = m * nc;
  const int n = P.n;
  P.L.assign(static_cast<size_t>(n) * n, 0.0);
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < m; ++j)
      for (int l = 0; l < nc; ++l)
        for (int lp = 0; lp < nc; ++lp) {
          const double e1 = (l == lp) ? A1[i * m + j] : 0.0;
          const double e2 = (lp == (l + M2) % nc) ? A2[i * m + j] : 0.0;
          const double e3 = (i == j ? r2inv[i] : 0.0) * a[((lp - l) % nc + nc) % nc];
          P.L[static_cast<size_t>(i * nc + l) * n + (j * nc + lp)] = (e1 + e2) + e3;
        }
  for (int j = 0; j < m; ++j)
    for (int l = 0; l < nc; ++l) {
      const double x = P.r[j] * std::cos(P.theta[l]) + cx, y = P.r[j] * std::sin(P.theta[l]) + cy;
      const size_t d = static_cast<size_t>(j * nc + l);
      P.L[d * n + d] += coefficients(B, x, y).c;
    }
  for (int l = 0; l < nc; ++l) {
    for (int k = 0; k < n; ++k) P.L[static_cast<size_t>(l) * n + k] = 0.0;
    P.L[static_cast<size_t>(l) * n + l] = 1.0;
  }
}

// Gaussian elimination with partial pivoting on A (n x n row-major, copied)
// for the columns of X (n x nrhs row-major), solved in place.
void ps_solve(int n, std::vector<double> A, int nrhs, std::vector<double>& X) {
  for (int k = 0; k < n; ++k) {
    int p = k;
    for (int i = k + 1; i < n; ++i)
      if (std::fabs(A[static_cast<size_t>(i) * n + k]) > std::fabs(A[static_cast<size_t>(p) * n + k])) p = i;
    if (p != k) {
      for (int j = 0; j < n; ++j) std::swap(A[static_cast<size_t>(k) * n + j], A[static_cast<size_t>(p) * n + j]);
      for (int j = 0; j < nrhs; ++j) std::swap(X[static_cast<size_t>(k) * nrhs + j], X[static_cast<size_t>(p) * nrhs + j]);
    }
    const double piv = A[static_cast<size_t>(k) * n + k];
    for (int i = k + 1; i < n; ++i) {
      const double f = A[static_cast<size_t>(i) * n + k] / piv;
      if (f == 0.0) continue;
      for (int j = k; j < n; ++j) A[static_cast<size_t>(i) * n + j] -= f * A[static_cast<size_t>(k) * n + j];
      for (int j = 0; j < nrhs; ++j) X[static_cast<size_t>(i) * nrhs + j] -= f * X[static_cast<size_t>(k) * nrhs + j];
    }
  }
  for (int k = n - 1; k >= 0; --k)
    for (int j = 0; j < nrhs; ++j) {
      double s = X[static_cast<size_t>(k) * nrhs + j];
      for (int q = k + 1; q < n; ++q) s -= A[static_cast<size_t>(k) * n + q] * X[static_cast<size_t>(q) * nrhs + j];
      X[static_cast<size_t>(k) * nrhs + j] = s / A[static_cast<size_t>(k) * n + k];
    }
}

// Interpolador_PS::Interpola (BVP/Interpolador_PS.cpp:34-61) of the grid
// values z (index j*Nc + l): Fourier interpolation in the angle along the
// diameter through the point (the opposite half through cos(k pi)), then
// barycentric interpolation in the radius with the weights of
// Interpolador_PS::Inicializa (:18-33) on the Chebyshev diameter.
double ps_interpola(const PsDisk& P, const double* z, int zstride, double cx, double cy, double px, double py) {
  const int N = P.nc, n = N / 2, half = P.n2 + 1, m = 2 * half;
  const double dx = px - cx, dy = py - cy;
  const double rp = std::sqrt(dx * dx + dy * dy) / P.radius;
  double tp = std::atan2(dy, dx);
  tp = (tp >= 0) ? tp : tp + 2.0 * M_PI;
  std::vector<double> head(half, 0.0), tail(half, 0.0);
  for (int l = 0; l < N; ++l)
    for (int k = -n; k < n; ++k) {
      const double ck = std::cos(k * (tp - P.theta[l]));
      const double sk = std::cos(k * M_PI);
      for (int j = 0; j < half; ++j) {
        const double v = ck * z[static_cast<size_t>(j * N + l) * zstride];
        head[j] = head[j] + v;
        tail[j] = tail[j] + sk * v;
      }
    }
  // u = normN * reverse(head, reverse(tail)): u_i = tail_i (i < half), head_{m-1-i}
  const double normN = 1.0 / N;
  std::vector<double> u(m), diam(m), c(m);
  for (int i = 0; i < half; ++i) {
    u[i] = normN * tail[i];
    u[m - 1 - i] = normN * head[i];
    diam[i] = -P.r[i] / P.radius;
    diam[m - 1 - i] = P.r[i] / P.radius;
  }
  const double its = -1.0 + 1.0 / m;
  for (int i = 0; i < m; ++i) c[i] = std::pow(-1, i) * std::sin(M_PI * (its + (2.0 / m) * i + 1) / 2);
  double num = 0, den = 0;
  for (int i = 0; i < m; ++i) {
    const double t = c[i] / (rp - diam[i]);
    num = num + t * u[i];
    den = den + t;
  }
  return num / den;
}

}  // namespace

extern "C" {

void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) { philox(ctr, key, out); }

void* orc_session_new(int rng_mode, uint64_t seed) { return new Session(rng_mode, seed); }
void orc_session_free(void* s) { delete static_cast<Session*>(s); }
void orc_session_set_stream(void* s, uint32_t stream) { static_cast<Session*>(s)->stream = stream; }

int orc_circulo(const double p[3], double x, double y, double out[5]) {
  V2 e, n;
  out[0] = circulo(p, V2{x, y}, e, n);
  out[1] = e.x; out[2] = e.y; out[3] = n.x; out[4] = n.y;
  return 0;
}
int orc_rectangulo(const double p[4], double x, double y, double out[5]) {
  V2 e, n;
  out[0] = rectangulo(p, V2{x, y}, e, n);
  out[1] = e.x; out[2] = e.y; out[3] = n.x; out[4] = n.y;
  return 0;
}
int orc_coefficients(const orc_bvp* b, double x, double y, double out[12]) {
  Coef c = coefficients(b, x, y);
  out[0] = c.u; out[1] = c.g; out[2] = c.c; out[3] = c.f; out[4] = c.b.x; out[5] = c.b.y;
  out[6] = c.s.a00; out[7] = c.s.a01; out[8] = c.s.a10; out[9] = c.s.a11; out[10] = c.F.x; out[11] = c.F.y;
  return 0;
}

int orc_path(void* s, const orc_bvp* b, const orc_shape* sub, double x0, double y0, double h,
             uint32_t item, uint32_t path, int max_steps, orc_exit* out) {
  int shape;
  const double* p;
  sub_of(b, sub, &shape, &p);
  return simulate(*static_cast<Session*>(s), b, shape, p, x0, y0, h, item, path,
                  max_steps > 0 ? max_steps : kMaxSteps, out);
}

int orc_point_solve(void* s, const orc_bvp* b, const orc_shape* sub, double x, double y, unsigned N,
                    double h, uint32_t item, double out[9]) {
  Session& S = *static_cast<Session*>(s);
  int shape;
  const double* p;
  sub_of(b, sub, &shape, &p);
  std::vector<orc_exit> ex(N);
  for (unsigned n = 0; n < N; ++n)
    if (simulate(S, b, shape, p, x, y, h, item, n, kMaxSteps, &ex[n]) != 0) return -1;
  Sums sums;
  for (unsigned n = 0; n < N; ++n) {
    double score = ex[n].Z + ex[n].Y * coefficients(b, ex[n].x, ex[n].y).g;
    sums.add(score, ex[n].xi, 4u * static_cast<unsigned>(ex[n].steps), ex[n].t);
  }
  sums.finish(N, out);
  return 0;
}

int orc_node_solve_arc(void* s, const orc_bvp* b, double x, double y, int frontera, const orc_arc* arc,
                       unsigned N, double h, uint32_t item, double* G, double* B, double stats[9]) {
  Session& S = *static_cast<Session*>(s);
  if (frontera) {  // FeynmanKacSolver.cpp:346-347
    *B = coefficients(b, x, y).g;
    for (int k = 0; k < 9; ++k) stats[k] = 0.0;
    return 0;
  }
  double sub[4] = {arc->radius, arc->cx, arc->cy, 0.0};
  std::vector<orc_exit> ex(N);
  for (unsigned n = 0; n < N; ++n)
    if (simulate(S, b, ORC_SHAPE_CIRCLE, sub, x, y, h, item, n, kMaxSteps, &ex[n]) != 0) return -1;
  // Reduce_Analytic(BVP, N, Nudo&, Interfaz) (FeynmanKacSolver.cpp:233-292)
  int n_ = arc->n;
  std::vector<double> Gl(n_, 0.0);
  double Bl = 0.0;
  Sums sums;
  for (unsigned n = 0; n < N; ++n) {
    double score;
    if (ex[n].outcome == ORC_OUT_DOMAIN) {
      score = ex[n].Z + ex[n].Y * coefficients(b, ex[n].x, ex[n].y).g;
      Bl += score + ex[n].xi;
    } else {
      score = ex[n].Z + ex[n].Y * coefficients(b, ex[n].x, ex[n].y).u;
      // Interfaz::Update_G (Mesh/Interfaz.cpp:219-264)
      double theta = arc_theta(arc->interior, ex[n].x - arc->cx, ex[n].y - arc->cy);
      double Yv = ex[n].Y;
      for (int j = 0; j < n_; ++j)
        for (int i = 0; i < n_; ++i) Gl[j] += -Yv * arc->iPsi[i + j * n_] * imq(theta, arc->theta[i], arc->c2);
      Bl += ex[n].Z + ex[n].xi;
    }
    sums.add(score, ex[n].xi, 4u * static_cast<unsigned>(ex[n].steps), ex[n].t);
  }
  double Nd = static_cast<double>(N);
  for (int j = 0; j < n_; ++j) G[j] = (0.0 + Gl[j]) / Nd;  // Update(Nudo&) :324-334
  *B = (0.0 + Bl) / Nd;
  sums.finish(N, stats);
  return 0;
}

}  // extern "C"

namespace {
// k nearest patch-boundary nodes of (x, y), ascending local index
void knn_select(const orc_knn* st, double x, double y, int* idx) {
  int m = st->m, k = st->k;
  std::vector<std::pair<double, int>> d(m);
  for (int a = 0; a < m; ++a) {
    double dx = x - st->xy[2 * a], dy = y - st->xy[2 * a + 1];
    d[a] = std::make_pair(dx * dx + dy * dy, a);
  }
  std::partial_sort(d.begin(), d.begin() + k, d.end());
  for (int a = 0; a < k; ++a) idx[a] = d[a].second;
  std::sort(idx, idx + k);
}
// inverse of A_W(a,b) = exp(-eps^2 |x_a - x_b|^2) for the window idx
std::vector<double> knn_inverse(const orc_knn* st, const int* idx) {
  int k = st->k;
  double e2 = st->eps * st->eps;
  std::vector<double> A(static_cast<size_t>(k) * k), inv;
  for (int j = 0; j < k; ++j)
    for (int i = 0; i < k; ++i) {
      double dx = st->xy[2 * idx[i]] - st->xy[2 * idx[j]], dy = st->xy[2 * idx[i] + 1] - st->xy[2 * idx[j] + 1];
      A[i + j * k] = std::exp(-e2 * (dx * dx + dy * dy));
    }
  gj_inverse(k, A, inv);
  return inv;
}
// w = A_W^{-1} phi_W(x)
void knn_apply(const orc_knn* st, const int* idx, const std::vector<double>& inv, double x, double y, double* w) {
  int k = st->k;
  double e2 = st->eps * st->eps;
  std::vector<double> phi(k);
  for (int a = 0; a < k; ++a) {
    double dx = x - st->xy[2 * idx[a]], dy = y - st->xy[2 * idx[a] + 1];
    phi[a] = std::exp(-e2 * (dx * dx + dy * dy));
  }
  for (int a = 0; a < k; ++a) {
    double s = 0.0;
    for (int c = 0; c < k; ++c) s += inv[a + c * k] * phi[c];
    w[a] = s;
  }
}
}  // namespace

extern "C" {

int orc_knn_weights(const orc_knn* st, double x, double y, int* idx, double* w) {
  knn_select(st, x, y, idx);
  knn_apply(st, idx, knn_inverse(st, idx), x, y, w);
  return 0;
}

int orc_node_solve_knn(void* s, const orc_bvp* b, double x, double y, const orc_shape* patch,
                       const orc_knn* st, unsigned N, double h, uint32_t item, double* G, double* B,
                       double stats[9], double extra[4]) {
  Session& S = *static_cast<Session*>(s);
  std::vector<orc_exit> ex(N);
  for (unsigned n = 0; n < N; ++n)
    if (simulate(S, b, patch->shape, patch->p, x, y, h, item, n, kMaxSteps, &ex[n]) != 0) return -1;
  int m = st->m, k = st->k;
  std::vector<double> Gl(m, 0.0), w(k);
  std::vector<int> idx(k);
  std::map<std::vector<int>, std::vector<double>> cache;
  double Bl = 0.0, e0 = 0.0, e1 = 0.0, ndom = 0.0, nsteps = 0.0;
  Sums sums;
  for (unsigned n = 0; n < N; ++n) {
    double score;
    Coef c = coefficients(b, ex[n].x, ex[n].y);
    if (ex[n].outcome == ORC_OUT_DOMAIN) {
      score = ex[n].Z + ex[n].Y * c.g;
      Bl += score + ex[n].xi;
      ndom += 1.0;
    } else {
      score = ex[n].Z + ex[n].Y * c.u;
      // one inverse per distinct window (a CPU solver would tabulate them)
      knn_select(st, ex[n].x, ex[n].y, idx.data());
      auto itc = cache.find(idx);
      if (itc == cache.end()) itc = cache.emplace(idx, knn_inverse(st, idx.data())).first;
      knn_apply(st, idx.data(), itc->second, ex[n].x, ex[n].y, w.data());
      for (int a = 0; a < k; ++a) Gl[idx[a]] += -ex[n].Y * w[a];
      Bl += ex[n].Z + ex[n].xi;
    }
    e0 += score + ex[n].xi;
    e1 += (score + ex[n].xi) * (score + ex[n].xi);
    nsteps += ex[n].steps;
    sums.add(score, ex[n].xi, 4u * static_cast<unsigned>(ex[n].steps), ex[n].t);
  }
  double Nd = static_cast<double>(N);
  for (int a = 0; a < m; ++a) G[a] = Gl[a] / Nd;
  *B = Bl / Nd;
  sums.finish(N, stats);
  if (extra) { extra[0] = e0; extra[1] = e1; extra[2] = ndom; extra[3] = nsteps; }
  return 0;
}

int orc_full_pivot_inverse(int n, const double* a, double* inv) {
  std::vector<double> A(a, a + static_cast<size_t>(n) * n), I;
  gj_inverse(n, A, I);
  std::memcpy(inv, I.data(), sizeof(double) * I.size());
  return 0;
}

double orc_calcula_psi(int n, const double* theta, double c2, double* iPsi) {
  // Interfaz::Calcula_Psi (Mesh/Interfaz.cpp:206-217) with BVP::RBF = Inverse_Multiquadric (BVP/BVP.cpp:22-24)
  std::vector<double> P(static_cast<size_t>(n) * n), I;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) P[i + j * n] = imq(theta[i], theta[j], c2);
  std::vector<double> Pc = P;
  gj_inverse(n, Pc, I);
  std::memcpy(iPsi, I.data(), sizeof(double) * I.size());
  double a = 0.0, bsum = 0.0;
  for (double v : I) a += v * v;
  for (double v : P) bsum += v * v;
  return std::sqrt(a) * std::sqrt(bsum);
}

int orc_actualiza_gb(int row, int nG, const int* cols, const double* G, double b, const int* rowptr,
                     const int* colidx, double* val, double* Bv) {
  // SistemaLineal::Actualiza_GB(Nudo&) (Mesh/SistemaLineal.cpp:68-88)
  Bv[row] += b;
  if (nG <= 0) return 0;
  int j;
  for (j = rowptr[row]; j < rowptr[row + 1]; ++j)
    if (colidx[j] == cols[0]) break;
  if (j == rowptr[row + 1]) return -1;
  for (int a = 0; a < nG; ++a) val[j + a] += G[a];
  return 0;
}

int orc_ps_disk(const orc_bvp* b, double cx, double cy, double radius, int n_circle, int n_radial, double theta0,
                int n_periph, const double* periph_theta, int n_inner, const double* inner_xy, double* G,
                double* Bv) {
  // PseudoespectralCirculoSolver::Inicializa + Resuelve(BVP, nudos_interior,
  // nudos_periferia) (Solvers/PseudoespectralCirculoSolver.cpp:2-189, :215-260)
  if (n_circle < 2 || n_circle % 2 || n_radial < 3 || n_radial % 2 == 0) return -1;
  PsDisk P;
  ps_build(b, cx, cy, radius, n_circle, n_radial, theta0, P);
  const int n = P.n, nrhs = n_periph + 1;
  std::vector<double> X(static_cast<size_t>(n) * nrhs, 0.0);
  for (int q = n_circle; q < n; ++q) {
    const int j = q / n_circle, l = q % n_circle;
    const double x = P.r[j] * std::cos(P.theta[l]) + cx, y = P.r[j] * std::sin(P.theta[l]) + cy;
    X[static_cast<size_t>(q) * nrhs] = (-1.0) * coefficients(b, x, y).f;
  }
  // Cardinal_Fourier (BVP/BVP.cpp:25-29) of each periphery node on the outer ring
  const int nh = n_periph / 2;
  for (int i = 0; i < n_periph; ++i)
    for (int l = 0; l < n_circle; ++l) {
      double acc = 0.0;
      for (int k = -nh; k < nh; ++k) acc += std::cos(k * (P.theta[l] - periph_theta[i]));
      X[static_cast<size_t>(l) * nrhs + 1 + i] = acc / (2 * nh);
    }
  ps_solve(n, P.L, nrhs, X);
  for (int p = 0; p < n_inner; ++p) {
    const double px = inner_xy[2 * p], py = inner_xy[2 * p + 1];
    Bv[p] = ps_interpola(P, X.data(), nrhs, cx, cy, px, py);
    for (int i = 0; i < n_periph; ++i)
      G[static_cast<size_t>(p) * n_periph + i] = (-1.0) * ps_interpola(P, X.data() + 1 + i, nrhs, cx, cy, px, py);
  }
  return 0;
}

int orc_mlp_eval(const orc_mlp* m, double x, double y, double out[3]) {
  double g[2], v;
  mlp_grad(m, x, y, g, &v);
  out[0] = v; out[1] = g[0]; out[2] = g[1];
  return 0;
}

double orc_mlp_loss_grad(const orc_mlp* m, int n, const double* xy, const double* target, double* grad) {
  int W = m->width;
  size_t off_b1 = 2 * W, off_W2 = off_b1 + W, off_b2 = off_W2 + W * W, off_W3 = off_b2 + W,
         off_b3 = off_W3 + W * W, off_W4 = off_b3 + W, off_b4 = off_W4 + W, total = off_b4 + 1;
  std::fill(grad, grad + total, 0.0);
  double loss = 0.0;
  std::vector<double> acts, d3(W), d2(W), d1(W);
  for (int s = 0; s < n; ++s) {
    double o = mlp_forward(m, xy[2 * s], xy[2 * s + 1], &acts);
    const double* z = acts.data();
    const double *p1 = z + 2, *h1 = p1 + W, *p2 = h1 + W, *h2 = p2 + W, *p3 = h2 + W, *h3 = p3 + W;
    double e = o - target[s];
    loss += e * e;
    double go = 2.0 * e / n;  // d loss / d o for loss = mean(e^2)
    grad[off_b4] += go;
    for (int j = 0; j < W; ++j) { grad[off_W4 + j] += go * h3[j]; d3[j] = go * m->W4[j] * dsilu(p3[j]); }
    for (int i = 0; i < W; ++i) {
      grad[off_b3 + i] += d3[i];
      for (int j = 0; j < W; ++j) grad[off_W3 + i * W + j] += d3[i] * h2[j];
    }
    for (int j = 0; j < W; ++j) {
      double a = 0;
      for (int i = 0; i < W; ++i) a += m->W3[i * W + j] * d3[i];
      d2[j] = a * dsilu(p2[j]);
    }
    for (int i = 0; i < W; ++i) {
      grad[off_b2 + i] += d2[i];
      for (int j = 0; j < W; ++j) grad[off_W2 + i * W + j] += d2[i] * h1[j];
    }
    for (int j = 0; j < W; ++j) {
      double a = 0;
      for (int i = 0; i < W; ++i) a += m->W2[i * W + j] * d2[i];
      d1[j] = a * dsilu(p1[j]);
    }
    for (int i = 0; i < W; ++i) {
      grad[off_b1 + i] += d1[i];
      grad[i * 2] += d1[i] * z[0];
      grad[i * 2 + 1] += d1[i] * z[1];
    }
  }
  return loss / n;
}

}  // extern "C"
