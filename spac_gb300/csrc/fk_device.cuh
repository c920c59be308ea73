// Device building blocks of the GB300 Feynman-Kac path kernels: Philox4x32-10
// normals, the Frontera distance functors, the fused BVP coefficient functors
// and the exit rule.  Everything is templated on the stepping type R (float
// or double); accumulations above the path level are FP64.
#pragma once
#include <cstdint>
#include <type_traits>
#include <utility>

#include <cuda_runtime.h>

namespace fk {

constexpr double kGobet = -0.5826;  // Gobet-Menozzi shift, FeynmanKacSolver.cpp:169,184

// ------------------------------------------------------------------ Philox ----
// Philox4x32-10 (Salmon et al., SC'11).  Counter (step, path, item, stream),
// key (seed lo, seed hi); the step's Box-Muller pair takes words x and y.
constexpr uint32_t kPhiloxM0 = 0xD2511F53u, kPhiloxM1 = 0xCD9E8D57u;  // round multipliers
constexpr uint32_t kPhiloxW0 = 0x9E3779B9u, kPhiloxW1 = 0xBB67AE85u;  // key increments
// Both words of the 64-bit product m c from one wide multiply.
__device__ __forceinline__ void mul_hilo(uint32_t m, uint32_t c, uint32_t& hi, uint32_t& lo) {
  const unsigned long long p = static_cast<unsigned long long>(m) * c;
  hi = static_cast<uint32_t>(p >> 32);
  lo = static_cast<uint32_t>(p);
}
__device__ __forceinline__ uint4 philox10(uint4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0, lo0, hi1, lo1;
    mul_hilo(kPhiloxM0, c.x, hi0, lo0);
    mul_hilo(kPhiloxM1, c.z, hi1, lo1);
    c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
    k0 += kPhiloxW0;
    k1 += kPhiloxW1;
  }
  return c;
}
// The same with the ten rounds' keys given (rk[2r], rk[2r + 1]): from a
// kernel's parameters each key is an operand of the round's xor.
__device__ __forceinline__ uint4 philox10_rk(uint4 c, const uint32_t* rk) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0, lo0, hi1, lo1;
    mul_hilo(kPhiloxM0, c.x, hi0, lo0);
    mul_hilo(kPhiloxM1, c.z, hi1, lo1);
    c = make_uint4(hi1 ^ c.y ^ rk[2 * r], lo1, hi0 ^ c.w ^ rk[2 * r + 1], lo0);
  }
  return c;
}

// Box-Muller pair from two 32-bit words: u = (word + 1/2) 2^-32 in (0,1).
__device__ __forceinline__ void box_muller(uint32_t a, uint32_t b, double& z0, double& z1) {
  const double inv32 = 2.3283064365386962890625e-10;
  const double u1 = (static_cast<double>(a) + 0.5) * inv32;
  const double u2 = (static_cast<double>(b) + 0.5) * inv32;
  const double rad = sqrt(-2.0 * log(u1));
  double s, c;
  sincos(6.283185307179586 * u2, &s, &c);
  z0 = rad * c;
  z1 = rad * s;
}
// FP32 stepping uses the SFU forms (ex2/lg2.approx, sqrt.approx and an
// approximate division): relative errors ~1e-6 at most, far below the Monte
// Carlo error of any node estimate.  FP64 stepping keeps the correctly
// rounded forms (it follows the oracle's paths).
__device__ __forceinline__ float fexp(float v) { return __expf(v); }
// 2^v (ex2.approx: the SFU's base-2 exponential)
__device__ __forceinline__ float fexp2(float v) {
  float r;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(v));
  return r;
}
__device__ __forceinline__ double fexp(double v) { return exp(v); }
__device__ __forceinline__ float fsqrt(float v) {
  float r;
  asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(v));
  return r;
}
__device__ __forceinline__ double fsqrt(double v) { return sqrt(v); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdividef(a, b); }
__device__ __forceinline__ double fdiv(double a, double b) { return a / b; }

__device__ __forceinline__ void box_muller(uint32_t a, uint32_t b, float& z0, float& z1) {
  const float inv32 = 2.3283064365386962890625e-10f;
  const float u1 = (static_cast<float>(a) + 0.5f) * inv32;  // rounds into (0, 1]
  const float u2 = (static_cast<float>(b) + 0.5f) * inv32;
  const float rad = fsqrt(-2.0f * __logf(u1));
  float s, c;
  __sincosf(6.28318530717958647692f * u2, &s, &c);
  z0 = rad * c;
  z1 = rad * s;
}

// Exp(1) variate from one 32-bit word: -log(u), u = (word + 1/2) 2^-32.
__device__ __forceinline__ double exp1_draw(uint32_t w, double) {
  return -log((static_cast<double>(w) + 0.5) * 2.3283064365386962890625e-10);
}
__device__ __forceinline__ float exp1_draw(uint32_t w, float) {
  return -__logf((static_cast<float>(w) + 0.5f) * 2.3283064365386962890625e-10f);
}

// FP32 -> FP64 by bit manipulation on the integer pipes (the F2F conversion
// runs on the FP64 pipe, a 64th of the FP32 rate on this part).  Exact for
// normal numbers and infinities; subnormal inputs (below 1.2e-38, far under
// any stencil weight that is added) become zero.
__device__ __forceinline__ double f32_to_f64(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xffu;
  if (e == 0u) return (u & 0x80000000u) ? -0.0 : 0.0;
  const unsigned e64 = (e == 0xffu) ? 0x7ffu : e + 896u;
  const unsigned hi = (u & 0x80000000u) | (e64 << 20) | ((u & 0x7fffffu) >> 3);
  const unsigned lo = (u & 0x7u) << 29;
  return __hiloint2double(static_cast<int>(hi), static_cast<int>(lo));
}

// FP64 -> FP32 on the integer pipes, rounded toward zero (|error| < 1 ulp of
// the result): for operands of small corrections only.  Magnitudes below the
// FP32 normal range become zero, above it infinity; NaN stays NaN.
__device__ __forceinline__ float f64_to_f32_rz(double d) {
  const unsigned long long u = static_cast<unsigned long long>(__double_as_longlong(d));
  const unsigned hi = static_cast<unsigned>(u >> 32), lo = static_cast<unsigned>(u);
  const unsigned sign = hi & 0x80000000u;
  const int e = static_cast<int>((hi >> 20) & 0x7ffu);
  const unsigned mant = ((hi & 0xfffffu) << 3) | (lo >> 29);
  unsigned r;
  if (e == 0x7ff) r = sign | 0x7f800000u | (mant ? 0x400000u : 0u);
  else if (e - 896 <= 0) r = sign;
  else if (e - 896 >= 255) r = sign | 0x7f800000u;
  else r = sign | (static_cast<unsigned>(e - 896) << 23) | mant;
  return __uint_as_float(r);
}

// ------------------------------------------------------------ geometry -------
template <typename R>
struct Bnd {
  R d;        // signed distance (negative inside)
  R ex, ey;   // closest boundary point (exit point)
  R nx, ny;   // outward normal
};

// Circulo (Dominios/Circulo.hpp:7-22): p = [r, cx, cy]; |x - c| clamped at 5e-4.
template <typename R>
__device__ __forceinline__ Bnd<R> circle_dist(R x, R y, R r0, R cx, R cy) {
  Bnd<R> b;
  R nx = x - cx, ny = y - cy;
  R r = fsqrt(nx * nx + ny * ny);
  r = r > R(5e-4) ? r : R(5e-4);
  nx = fdiv(nx, r);
  ny = fdiv(ny, r);
  b.nx = nx;
  b.ny = ny;
  b.ex = nx * r0 + cx;
  b.ey = ny * r0 + cy;
  b.d = r - r0;
  return b;
}

// Rectangulo (Dominios/Rectangulo.hpp:7-229): p = [x0, y0, x1, y1].  Signs
// sx, sy pick the quadrant (a point on a centre line is in the lower/left
// one); inside, the side with the larger offset wins (tie -> horizontal side);
// outside, the corner if both offsets exceed the half sides.
template <typename R>
__device__ __forceinline__ Bnd<R> rect_dist(R x, R y, R x0, R y0, R x1, R y1) {
  const R kDiag = R(0.70710678118f);
  Bnd<R> b;
  const R cx = R(0.5) * (x0 + x1), cy = R(0.5) * (y0 + y1);
  const R hx = x1 - cx, hy = y1 - cy;
  const R dx = fabs(x - cx), dy = fabs(y - cy);
  const bool px = x > cx, py = y > cy;
  const R sx = px ? R(1) : R(-1), sy = py ? R(1) : R(-1);
  const R bx = px ? hx + cx : -hx + cx;
  const R by = py ? hy + cy : -hy + cy;
  const R ox = dx - hx, oy = dy - hy;
  b.ex = x;
  b.ey = y;
  bool side_x;
  if ((dx <= hx) && (dy <= hy)) {
    side_x = ox > oy;
  } else if (dx > hx && dy > hy) {
    b.ex = bx;
    b.ey = by;
    b.nx = sx * kDiag;
    b.ny = sy * kDiag;
    b.d = fsqrt(ox * ox + oy * oy);
    return b;
  } else {
    side_x = dx > hx;
  }
  if (side_x) {
    b.ex = bx;
    b.nx = sx;
    b.ny = R(0);
    b.d = ox;
  } else {
    b.ey = by;
    b.nx = R(0);
    b.ny = sy;
    b.d = oy;
  }
  return b;
}

// Branch-cut angle of an exit point for the arc stencil (Mesh/Nudo.hpp:7-32
// dispatched as in Interfaz::Update_G, Mesh/Interfaz.cpp:222-251).
__device__ __forceinline__ double arc_theta(int interior, double dx, double dy) {
  const double a = atan2(dy, dx);
  const double pi = 3.141592653589793;
  switch (interior) {
    case -33: case -44: case -2: return (a >= 0) ? a : a + 2.0 * pi;
    case -1: return (a <= -0.5 * pi) ? 2.0 * pi + a : a;
    case -3: return (a <= 0.5 * pi) ? 2.0 * pi + a : a;
    default: return a;  // -11, -22, -4
  }
}

// ----------------------------------------------------------- problems -------
struct BvpDev {
  int problem, cv, dom_shape, mlp;
  double dom[4];
  double prob[4];
};

template <typename R>
struct StepCoef {
  R f, c, bx, by, s, Fx, Fy;  // source, potential, drift, sigma = s I, control field F
};

// Franke test function with its gradient and Laplacian, each exponential
// evaluated once (BVPs/Franke_Poisson.hpp:4-60).
template <typename R>
struct FrankeEval {
  R e1, e2, e3, e4, a, b, c, d, p, q, r, t;
  R s1, s3, s4;  // a^2 + b^2, p^2 + q^2, r^2 + t^2 (the exponents' sums, reused by lap)
  __device__ __forceinline__ FrankeEval(R x, R y) {
    a = R(9) * x - R(2);
    b = R(9) * y - R(2);
    c = R(9) * x + R(1);
    d = R(9) * y + R(1);
    p = R(9) * x - R(7);
    q = R(9) * y - R(3);
    r = R(9) * x - R(4);
    t = R(9) * y - R(7);
    s1 = a * a + b * b;
    s3 = p * p + q * q;
    s4 = r * r + t * t;
    if constexpr (std::is_same<R, float>::value) {
      // 2^(log2(e) v): the log2(e) scale folded into each exponent's constants
      constexpr float L2E = 1.44269504088896340736f;
      e1 = fexp2(-0.25f * L2E * s1);
      e2 = fexp2((-1.0f / 49.0f * L2E) * (c * c) - 0.1f * L2E * d);
      e3 = fexp2(-0.25f * L2E * s3);
      e4 = fexp2(-L2E * s4);
    } else {
      e1 = fexp(R(-0.25) * s1);
      e2 = fexp(R(-1.0 / 49.0) * (c * c) - R(0.1) * d);
      e3 = fexp(R(-0.25) * s3);
      e4 = fexp(R(-1) * s4);
    }
  }
  // uxx + uyy with each exponential's two second derivatives combined:
  // -3.375 (18 - 4.5 s1) e1 + (-(27/98)(9 - (18/49) c^2) + 243/400) e2
  // - 2.25 (18 - 4.5 s3) e3 + 3.6 (18 - 18 s4) e4
  __device__ __forceinline__ R lap() const {
    return (R(15.1875) * s1 - R(60.75)) * e1 + (R(27.0 * 18.0 / (98.0 * 49.0)) * (c * c) - R(243.0 / 98.0 - 243.0 / 400.0)) * e2 +
           (R(10.125) * s3 - R(40.5)) * e3 + (R(64.8) - R(64.8) * s4) * e4;
  }
  __device__ __forceinline__ R u() const { return R(0.75) * e1 + R(0.75) * e2 + R(0.5) * e3 - R(0.2) * e4; }
  __device__ __forceinline__ R ux() const {
    return R(-3.375) * a * e1 - R(27.0 / 98.0) * c * e2 - R(2.25) * p * e3 + R(3.6) * r * e4;
  }
  __device__ __forceinline__ R uy() const {
    return R(-3.375) * b * e1 - R(0.675) * e2 - R(2.25) * q * e3 + R(3.6) * t * e4;
  }
  __device__ __forceinline__ R uxx() const {
    return R(-3.375) * (R(9) - R(4.5) * (a * a)) * e1 -
           R(27.0 / 98.0) * (R(9) - R(18.0 / 49.0) * (c * c)) * e2 -
           R(2.25) * (R(9) - R(4.5) * (p * p)) * e3 + R(3.6) * (R(9) - R(18) * (r * r)) * e4;
  }
  __device__ __forceinline__ R uyy() const {
    return R(-3.375) * (R(9) - R(4.5) * (b * b)) * e1 + R(243.0 / 400.0) * e2 -
           R(2.25) * (R(9) - R(4.5) * (q * q)) * e3 + R(3.6) * (R(9) - R(18) * (t * t)) * e4;
  }
};

// sin(pi v): SFU form for FP32 stepping (|v| <= 2 here), accurate for FP64
__device__ __forceinline__ float sinpi_(float v) { return __sinf(3.14159265358979323846f * v); }
__device__ __forceinline__ double sinpi_(double v) { return sinpi(v); }

// Monegros with c = -1 (BVPs/Monegros_Revamped.hpp:4-75).
template <typename R>
struct MonegrosEval {
  R u, ux, uy, lap;
  __device__ __forceinline__ MonegrosEval(R x, R y) {
    const R k1 = R(1.0), k2 = R(0.01), k3 = R(0.02), k4 = R(0.12), k5 = R(0.05), k6 = R(0.05), k7 = R(-0.12),
            sf = R(0.333);
    const R rho = fsqrt(k1 + k2 * x * x + k3 * y * y);
    R sr, cr;
    sr = sin(rho);
    cr = cos(rho);
    const R a1 = k4 * x + k5 * y, a2 = k6 * x + k7 * y;
    const R s1 = sin(a1), c1 = cos(a1), s2 = sin(a2), c2 = cos(a2);
    const R th = tanh(s1 + s2);
    const R th2m1 = th * th - R(1);
    u = R(3) + sf * (sr + th);
    ux = sf * (cr * k2 * x / rho - (k4 * c1 + k6 * c2) * th2m1);
    uy = sf * (cr * k1 * k3 * y / rho - (k5 * c1 + k7 * c2) * th2m1);
    const R r3 = rho * rho * rho;
    const R uxx = sf * (((k2 / rho) - (k2 * k2 * x * x / r3)) * cr - (x * x * k2 * k2 / (rho * rho)) * sr +
                        R(2) * (k4 * c1 + k6 * c2) * (k4 * c1 + k6 * c2) * th2m1 * th +
                        (k4 * k4 * s1 + k6 * k6 * s2) * th2m1);
    const R uyy = sf * (((k3 / rho) - (k3 * k3 * y * y / r3)) * cr - (y * y * k3 * k3 / (rho * rho)) * sr +
                        R(2) * (k5 * c1 + k7 * c2) * (k5 * c1 + k7 * c2) * th2m1 * th +
                        (k5 * k5 * s1 + k7 * k7 * s2) * th2m1);
    lap = uxx + uyy;
  }
};

// Problem functors.  state(x, y) is what sigma needs at a point (the
// anisotropy factor a(x, y) of FK_PROBLEM_ANISO; nothing for constant sigma);
// the exit rule computes it and sigma_of(state) at the new point, and the
// next step reuses both: step(bvp, x, y, a, s, cv, o) gets the state a and
// s = sigma_of(a).
template <int PROB>
struct Problem;

// FK_PROBLEM_FRANKE: sigma = 1.41421356237 I, b = 0, c = 0, f = -Lap u.
template <>
struct Problem<0> {
  template <typename R>
  __device__ static R state(const BvpDev&, R, R) { return R(0); }
  template <typename R>
  __device__ static R sigma_of(R) { return R(1.41421356237); }
  template <typename R>
  __device__ static void step(const BvpDev&, R x, R y, R, R, bool cv, StepCoef<R>& o) {
    FrankeEval<R> F(x, y);
    o.s = R(1.41421356237);
    o.f = -F.lap();
    o.c = R(0);
    o.bx = R(0);
    o.by = R(0);
    if (cv) {
      o.Fx = -o.s * F.ux();
      o.Fy = -o.s * F.uy();
    }
  }
  template <typename R>
  __device__ static R u(const BvpDev&, R x, R y) { return FrankeEval<R>(x, y).u(); }
};

// FK_PROBLEM_MONEGROS: sigma = 1.41421356237 I, b = 0, c = -1, f = -Lap u + u.
template <>
struct Problem<1> {
  template <typename R>
  __device__ static R state(const BvpDev&, R, R) { return R(0); }
  template <typename R>
  __device__ static R sigma_of(R) { return R(1.41421356237); }
  template <typename R>
  __device__ static void step(const BvpDev&, R x, R y, R, R, bool cv, StepCoef<R>& o) {
    MonegrosEval<R> M(x, y);
    o.s = R(1.41421356237);
    o.c = R(-1);
    o.f = -M.lap - o.c * M.u;
    o.bx = R(0);
    o.by = R(0);
    if (cv) {
      o.Fx = -o.s * M.ux;
      o.Fy = -o.s * M.uy;
    }
  }
  template <typename R>
  __device__ static R u(const BvpDev&, R x, R y) { return MonegrosEval<R>(x, y).u; }
};

// FK_PROBLEM_ANISO.
template <>
struct Problem<2> {
  template <typename R>
  __device__ static R coef_a(R x, R y) {
    return R(1) + R(0.5) * sinpi_(R(2) * x) * sinpi_(R(2) * y);
  }
  template <typename R>
  __device__ static R state(const BvpDev&, R x, R y) { return coef_a(x, y); }
  template <typename R>
  __device__ static R sigma_of(R a) { return fsqrt(R(2) * a); }
  template <typename R>
  __device__ static void step(const BvpDev&, R x, R y, R a, R s, bool cv, StepCoef<R>& o) {
    FrankeEval<R> F(x, y);
    const R q = R(1) + x * y;
    const R Fv = F.u(), Fx = F.ux(), Fy = F.uy();
    const R u = Fv * q;
    const R ux = Fx * q + Fv * y, uy = Fy * q + Fv * x;
    const R lap = F.lap() * q + R(2) * (Fx * y + Fy * x);
    o.s = s;  // sigma_of(a), formed where the state was
    o.c = -(R(1) + x * x + y * y);
    o.bx = y - R(0.5);
    o.by = R(0.5) - x;
    o.f = -(a * lap + o.bx * ux + o.by * uy + o.c * u);
    if (cv) {
      o.Fx = -o.s * ux;
      o.Fy = -o.s * uy;
    }
  }
  template <typename R>
  __device__ static R u(const BvpDev&, R x, R y) { return FrankeEval<R>(x, y).u() * (R(1) + x * y); }
};

// FK_PROBLEM_DISK: Franke mapped from the disk's bounding box to [0,1]^2.
template <>
struct Problem<3> {
  template <typename R>
  __device__ static R state(const BvpDev&, R, R) { return R(0); }
  template <typename R>
  __device__ static R sigma_of(R) { return R(1.41421356237); }
  template <typename R>
  __device__ static void step(const BvpDev& b, R x, R y, R, R, bool cv, StepCoef<R>& o) {
    const R inv = R(1) / (R(2) * R(b.prob[2]));
    const R xi = (x - R(b.prob[0])) * inv + R(0.5), eta = (y - R(b.prob[1])) * inv + R(0.5);
    FrankeEval<R> F(xi, eta);
    o.s = R(1.41421356237);
    o.f = -F.lap() * (inv * inv);
    o.c = R(0);
    o.bx = R(0);
    o.by = R(0);
    if (cv) {
      o.Fx = -o.s * F.ux() * inv;
      o.Fy = -o.s * F.uy() * inv;
    }
  }
  template <typename R>
  __device__ static R u(const BvpDev& b, R x, R y) {
    const R inv = R(1) / (R(2) * R(b.prob[2]));
    return FrankeEval<R>((x - R(b.prob[0])) * inv + R(0.5), (y - R(b.prob[1])) * inv + R(0.5)).u();
  }
};

// FK_PROBLEM_ROBIN: the anisotropic problem on a rectangle whose sides in the
// mask prob[0] (1: x = x0, 2: y = y0, 4: x = x1, 8: y = y1) reflect instead of
// absorbing (Frontera::Absorbente false there, Frontera.hpp:23-36), with the
// Robin coefficients of Paso_Reflejante (FeynmanKacSolver.cpp:19-67):
// varphi = prob[1] (Y += varphi Y dL) and psi = d_n u - varphi u (Z += psi Y dL),
// so that u stays the exact solution.  prob[2] = rho: the reflecting step is
// taken while the path is within rho of its reflecting side.
template <>
struct Problem<4> : Problem<2> {
  template <typename R>
  __device__ static R psi(const BvpDev& b, R x, R y, R nx, R ny) {
    FrankeEval<R> F(x, y);
    const R q = R(1) + x * y;
    const R Fv = F.u();
    const R ux = F.ux() * q + Fv * y, uy = F.uy() * q + Fv * x;
    return nx * ux + ny * uy - R(b.prob[1]) * (Fv * q);
  }
};

// FK_PROBLEM_MONEGROS_POISSON: BVPs/Monegros_Poisson.hpp, the Monegros u of
// FK_PROBLEM_MONEGROS with c = 0 and f = -Lap u (the problem of the MPI
// drivers, main_test_mpi.cpp:3,24-30).
template <>
struct Problem<5> {
  template <typename R>
  __device__ static R state(const BvpDev&, R, R) { return R(0); }
  template <typename R>
  __device__ static R sigma_of(R) { return R(1.41421356237); }
  template <typename R>
  __device__ static void step(const BvpDev&, R x, R y, R, R, bool cv, StepCoef<R>& o) {
    MonegrosEval<R> M(x, y);
    o.s = R(1.41421356237);
    o.c = R(0);
    o.f = -M.lap;
    o.bx = R(0);
    o.by = R(0);
    if (cv) {
      o.Fx = -o.s * M.ux;
      o.Fy = -o.s * M.uy;
    }
  }
  template <typename R>
  __device__ static R u(const BvpDev&, R x, R y) { return MonegrosEval<R>(x, y).u; }
};

// Problems with reflecting sides (the Paso_Reflejante branch of the step).
template <int PROB>
struct RobinOf {
  static constexpr bool value = false;
};
template <>
struct RobinOf<4> {
  static constexpr bool value = true;
};

// ---- the compiled problem functor sets --------------------------------------
// Every BVP functor set the library compiles, indexed by FK_PROBLEM_*
// (include/spac_fk.h).  To add one: write its Problem<N> (state, sigma_of,
// step and u as above, all for both stepping types; psi and a RobinOf<N>
// specialisation if it has reflecting sides; a DomainOf<N> specialisation if
// its domain is a circle), give it FK_PROBLEM_ value N = kNumProblems and
// raise kNumProblems.  with_problem then instantiates and dispatches every
// kernel (paths, finalize, disk rows) for it; the registry accepts it and
// checks its domain shape.
constexpr int kNumProblems = 6;
template <int PROB>
struct DomainOf {
  static constexpr int shape = 0;  // FK_SHAPE_RECT: Dominios/Rectangulo.hpp
};
template <>
struct DomainOf<3> {
  static constexpr int shape = 1;  // FK_SHAPE_CIRCLE: Dominios/Circulo.hpp
};
template <int P>
using ProblemTag = std::integral_constant<int, P>;
// f(ProblemTag<problem>{}) for a problem id in [0, kNumProblems) (host code:
// picks the kernel instantiation of a launch).
template <int P = 0, typename F>
inline auto with_problem(int problem, F&& f) -> decltype(f(ProblemTag<0>{})) {
  if constexpr (P + 1 < kNumProblems) {
    if (problem != P) return with_problem<P + 1>(problem, std::forward<F>(f));
  }
  return f(ProblemTag<P>{});
}
inline int problem_domain_shape(int problem) {
  return with_problem(problem, [](auto t) { return DomainOf<decltype(t)::value>::shape; });
}

// Side of a rectangle that Dentro's nearest boundary point lies on (0: x = x0,
// 1: y = y0, 2: x = x1, 3: y = y1), if it is in the reflecting mask; -1 for
// absorbing sides and for corners (diagonal normals).
template <typename R>
__device__ __forceinline__ int robin_side(const Bnd<R>& w, int mask) {
  const int s = (w.nx == R(-1)) ? 0 : (w.ny == R(-1)) ? 1 : (w.nx == R(1)) ? 2 : (w.ny == R(1)) ? 3 : -1;
  return (s >= 0 && ((mask >> s) & 1)) ? s : -1;
}

}  // namespace fk
