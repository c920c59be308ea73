// GB300 kernels of the pseudospectral disk rows (the solver is described in
// fk_disk.h):
//   disk_coef_kernel   per disk: c and -f at the N_c x (N2+1) polar grid
//                      points, whether c varies over the disk and its mean
//   disk_modes_kernel  per (disk, Fourier mode k), one warp: the (N2+1)^2 mode
//                      matrix M_k and its inverse (Gauss-Jordan, partial pivoting)
//   disk_solve_kernel  per (disk, right-hand side): the right-hand side of
//                      PseudoespectralCirculoSolver::Resuelve (-f for B, the
//                      Fourier cardinal function of one periphery node for
//                      G, BVP/BVP.cpp:25-29); constant c: kept as a spectrum
//                      (B: DFT -> modes; G: the outer ring's DFT alone);
//                      varying c: grid values by DFT -> modes -> inverse DFT
//                      with Richardson sweeps
//   disk_interp_kernel per interior node (one warp): the linear functional of
//                      Interpolador_PS::Interpola at the node, applied to
//                      every solution of its disk: B, and G = -interpolant;
//                      optionally added into the CSR values and B
//                      (SistemaLineal::Actualiza_GB(Interfaz&),
//                      Mesh/SistemaLineal.cpp:90-95)
// All arithmetic is FP64 (the rows are a deterministic FP64 alternative to
// the Feynman-Kac rows).
#include <cfloat>
#include <cmath>
#include <map>
#include <utility>

#include "fk_device.cuh"
#include "fk_disk.h"

namespace fk {

namespace {

constexpr int kCoefThreads = 256;
constexpr int kSolveThreads = 256;
constexpr int kInterpSmemBudget = 200 * 1024;

// radial class table layout (offsets from DiskDev::tab_off)
__host__ __device__ inline long long tab_r(int) { return 0; }
__host__ __device__ inline long long tab_a1(int half) { return half; }
__host__ __device__ inline long long tab_a2(int half) { return half + static_cast<long long>(half) * half; }
__host__ __device__ inline long long tab_r2inv(int half) { return half + 2LL * half * half; }
__host__ __device__ inline long long tab_bw(int half) { return 2LL * half + 2LL * half * half; }
__host__ __device__ inline long long tab_diam(int half) { return 4LL * half + 2LL * half * half; }
__host__ __device__ inline long long tab_size(int half) { return 6LL * half + 2LL * half * half; }

// Radial operators of PseudoespectralCirculoSolver::Inicializa
// (Solvers/PseudoespectralCirculoSolver.cpp:8-65, cheb.m on a diameter of
// N_radio + 1 Chebyshev points) and the barycentric data of
// Interpolador_PS::Inicializa (BVP/Interpolador_PS.cpp:18-33).
void radial_class(double radius, int nr, std::vector<double>& t) {
  const int np = nr + 1, half = (nr + 1) / 2, m = 2 * half;
  std::vector<double> r(np);
  std::vector<int> cw(np);
  for (int i = 0; i < np; ++i) {
    r[i] = radius * std::cos(M_PI * i / nr);
    cw[i] = ((i == 0 || i == nr) ? 2 : 1) * ((i & 1) ? -1 : 1);
  }
  std::vector<double> D(static_cast<size_t>(np) * np), DD(static_cast<size_t>(np) * np);
  for (int i = 0; i < np; ++i) {
    for (int j = 0; j < np; ++j)
      D[i * np + j] = (cw[i] * (1.0 / cw[j])) / ((r[i] - r[j]) + (i == j ? 1.0 : 0.0));
    double s = 0.0;
    for (int j = 0; j < np; ++j) s += D[i * np + j];
    D[i * np + i] -= s;
  }
  for (int i = 0; i < np; ++i)
    for (int j = 0; j < np; ++j) {
      double s = D[i * np] * D[j];
      for (int k = 1; k < np; ++k) s += D[i * np + k] * D[k * np + j];
      DD[i * np + j] = s;
    }
  const size_t base = t.size();
  t.resize(base + tab_size(half), 0.0);
  double* T = t.data() + base;
  for (int i = 0; i < half; ++i) {
    const double ri = 1.0 / r[i];
    T[tab_r(half) + i] = r[i];
    T[tab_r2inv(half) + i] = ri * ri;
    for (int j = 0; j < half; ++j) {
      T[tab_a1(half) + i * half + j] = DD[i * np + j] + ri * D[i * np + j];
      T[tab_a2(half) + i * half + j] = DD[i * np + (nr - j)] + ri * D[i * np + (nr - j)];
    }
    T[tab_diam(half) + i] = -r[i] / radius;
    T[tab_diam(half) + m - 1 - i] = r[i] / radius;
  }
  const double its = -1.0 + 1.0 / m;
  for (int i = 0; i < m; ++i)
    T[tab_bw(half) + i] = ((i & 1) ? -1.0 : 1.0) * std::sin(M_PI * (its + (2.0 / m) * i + 1) / 2);
}

// Eigenvalues of the periodic second-derivative (Toeplitz) matrix
// (PseudoespectralCirculoSolver.cpp:66-92): mu_k = sum_d a(d) cos(2 pi k d / N).
void mode_eigenvalues(int nc, std::vector<double>& t) {
  const double dt = 2 * M_PI / nc;
  std::vector<double> a(nc), c(nc);
  for (int l = 0; l < nc; ++l) {
    a[l] = (l == 0) ? -(M_PI * M_PI / (3 * dt * dt)) - (1.0 / 6)
                    : 0.5 * ((l & 1) ? 1.0 : -1.0) / std::pow(std::sin(dt * l * 0.5), 2);
    c[l] = std::cos(2 * M_PI * l / nc);
  }
  for (int k = 0; k <= nc / 2; ++k) {
    double s = 0.0;
    for (int d = 0; d < nc; ++d) s += a[d] * c[(static_cast<long long>(k) * d) % nc];
    t.push_back(s);
  }
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// ------------------------------------------------------------------ coef ----
template <int PROB>
__global__ void __launch_bounds__(kCoefThreads) disk_coef_kernel(const DiskArgs a) {
  __shared__ double s_sum[kCoefThreads / 32];
  __shared__ int s_var[kCoefThreads / 32];
  const int d = blockIdx.x;
  const DiskDev D = a.disks[d];
  const BvpDev bvp = *a.bvp;
  const int nc = D.nc, n = nc * D.half;
  const double* r = a.tab + D.tab_off + tab_r(D.half);
  double* cg = a.grid + D.grid_off;
  double* fg = cg + n;
  const double dt = 2 * M_PI / nc;
  for (int q = threadIdx.x; q < n; q += blockDim.x) {
    const int j = q / nc, l = q - j * nc;
    const double th = l * dt + D.theta0;
    const double x = r[j] * cos(th) + D.cx, y = r[j] * sin(th) + D.cy;
    StepCoef<double> o;
    const double a_xy = Problem<PROB>::template state<double>(bvp, x, y);
    Problem<PROB>::template step<double>(bvp, x, y, a_xy, Problem<PROB>::template sigma_of<double>(a_xy), false, o);
    cg[q] = o.c;
    fg[q] = (-1.0) * o.f;
  }
  __syncthreads();
  // rows of the outer ring (j = 0) are identity rows: c matters inside only
  const double c0 = cg[nc];
  double sum = 0.0;
  int var = 0;
  for (int q = nc + threadIdx.x; q < n; q += blockDim.x) {
    sum += cg[q];
    var |= (cg[q] != c0) ? 1 : 0;
  }
  sum = warp_sum(sum);
  var = __any_sync(0xffffffffu, var);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) { s_sum[w] = sum; s_var[w] = var; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    int v = 0;
    for (int i = 0; i < static_cast<int>(blockDim.x >> 5); ++i) { t += s_sum[i]; v |= s_var[i]; }
    a.cbar[d] = v ? t / (n - nc) : c0;
    a.varying[d] = v;
  }
}

// ----------------------------------------------------------------- modes ----
// One warp per (disk, mode): M_k and [M_k | I] reduced by Gauss-Jordan with
// partial pivoting (first maximum wins), rows of `half` doubles in shared memory.
constexpr int kModeWarps = 8;
__global__ void __launch_bounds__(32 * kModeWarps) disk_modes_kernel(const DiskArgs a, int max_half) {
  extern __shared__ double smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int d = blockIdx.x, k = blockIdx.y * kModeWarps + warp;
  const DiskDev D = a.disks[d];
  if (k > D.nc / 2) return;  // whole warp; no block-wide barrier below
  const int half = D.half, w = 2 * half, ld = 2 * max_half + 1;
  double* S = smem + static_cast<long long>(warp) * max_half * ld;
  const double* T = a.tab + D.tab_off;
  const double* A1 = T + tab_a1(half);
  const double* A2 = T + tab_a2(half);
  const double* r2inv = T + tab_r2inv(half);
  const double mu = a.tab[D.mu_off + k], sgn = (k & 1) ? -1.0 : 1.0, cb = a.cbar[d];
  for (int idx = lane; idx < half * w; idx += 32) {
    const int i = idx / w, c = idx - i * w;
    double v;
    if (c < half) {
      if (i == 0) v = (c == 0) ? 1.0 : 0.0;  // outer ring: identity row
      else v = A1[i * half + c] + sgn * A2[i * half + c] + ((i == c) ? mu * r2inv[i] + cb : 0.0);
    } else {
      v = (c - half == i) ? 1.0 : 0.0;
    }
    S[i * ld + c] = v;
  }
  __syncwarp();
  for (int col = 0; col < half; ++col) {
    // pivot: the first row of largest |S[i][col]|, i >= col
    double best = (lane >= col && lane < half) ? fabs(S[lane * ld + col]) : -1.0;
    int bi = lane;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double ob = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
    }
    const int p = bi;
    const double pv = S[p * ld + col];
    if (pv == 0.0) {  // uniform over the warp: singular mode matrix
      if (lane == 0) atomicOr(&a.flags[0], 1);
      return;
    }
    if (p != col)
      for (int c = lane; c < w; c += 32) {
        const double t = S[col * ld + c];
        S[col * ld + c] = S[p * ld + c];
        S[p * ld + c] = t;
      }
    __syncwarp();
    const double fac = (lane < half) ? S[lane * ld + col] : 0.0;  // column col, after the swap
    __syncwarp();
    // columns < col of the left block are already unit vectors: only the
    // columns from col + 1 on change (column col itself is not read again)
    const double inv = 1.0 / pv;
    for (int c = col + 1 + lane; c < w; c += 32) S[col * ld + c] = S[col * ld + c] * inv;
    __syncwarp();
    for (int i = 0; i < half; ++i) {
      const double f = __shfl_sync(0xffffffffu, fac, i);
      if (i == col) continue;
      for (int c = col + 1 + lane; c < w; c += 32) S[i * ld + c] = S[i * ld + c] - f * S[col * ld + c];
    }
    __syncwarp();
  }
  double* out = a.minv + D.minv_off + static_cast<long long>(k) * half * half;
  for (int idx = lane; idx < half * half; idx += 32) {
    const int i = idx / half, j = idx - i * half;
    out[idx] = S[i * ld + half + j];
  }
}

// ----------------------------------------------------------------- solve ----
struct SolveSmem {
  double *cosT, *sinT, *rhs, *z, *w, *C, *S, *C2, *S2, *red;
};

// Real DFT in the angle of the first `radii` radii of `in`: C[k][j] =
// sum_l in(l, j) cos(2 pi k l / N), S[k][j] the same with sin, k = 0 .. N/2.
__device__ void forward_dft(const DiskDev& D, const SolveSmem& m, const double* in, int radii) {
  const int nc = D.nc, half = D.half, nm = nc / 2 + 1, tid = threadIdx.x, nt = blockDim.x;
  for (int idx = tid; idx < nm * radii; idx += nt) {
    const int k = idx / radii, j = idx - k * radii;
    double c = 0.0, s = 0.0;
    int q = 0;
    for (int l = 0; l < nc; ++l) {
      const double v = in[j * nc + l];
      c += v * m.cosT[q];
      s += v * m.sinT[q];
      q += k;
      if (q >= nc) q -= nc;
    }
    m.C[k * half + j] = c;
    m.S[k * half + j] = s;
  }
  __syncthreads();
}

// The inverse mode matrix per frequency, using the first `radii` radii of
// the transform (the others are zero): C2 = M_k^-1 C, S2 = M_k^-1 S.
__device__ void mode_product(const DiskDev& D, const double* __restrict__ minv, const SolveSmem& m, int radii) {
  const int nc = D.nc, half = D.half, nm = nc / 2 + 1, tid = threadIdx.x, nt = blockDim.x;
  for (int idx = tid; idx < nm * half; idx += nt) {
    const int k = idx / half, i = idx - k * half;
    const double* Mi = minv + (static_cast<long long>(k) * half + i) * half;
    double c = 0.0, s = 0.0;
    for (int j = 0; j < radii; ++j) {
      c += Mi[j] * m.C[k * half + j];
      s += Mi[j] * m.S[k * half + j];
    }
    m.C2[idx] = c;
    m.S2[idx] = s;
  }
  __syncthreads();
}

// out(l, j) = inverse real DFT of (C2, S2).
__device__ void inverse_dft(const DiskDev& D, const SolveSmem& m, double* out) {
  const int nc = D.nc, half = D.half, tid = threadIdx.x, nt = blockDim.x;
  const double inv_n = 1.0 / nc;
  for (int idx = tid; idx < nc * half; idx += nt) {
    const int j = idx / nc, l = idx - j * nc;
    double acc = m.C2[j];
    int q = l;
    double mid = 0.0;
    for (int k = 1; k < nc / 2; ++k) {
      mid += m.C2[k * half + j] * m.cosT[q] + m.S2[k * half + j] * m.sinT[q];
      q += l;
      if (q >= nc) q -= nc;
    }
    acc += 2.0 * mid + m.C2[(nc / 2) * half + j] * ((l & 1) ? -1.0 : 1.0);
    out[idx] = acc * inv_n;
  }
  __syncthreads();
}

// out = L0^-1 in (in and out may alias).  ring_only: `in` is zero off the
// outer ring (radius 0), so only that radius is transformed and only column
// 0 of each mode inverse is used.
__device__ void apply_l0inv(const DiskDev& D, const double* __restrict__ minv, const SolveSmem& m, const double* in,
                            double* out, bool ring_only) {
  const int radii = ring_only ? 1 : D.half;
  forward_dft(D, m, in, radii);
  mode_product(D, minv, m, radii);
  inverse_dft(D, m, out);
}

__global__ void __launch_bounds__(kSolveThreads) disk_solve_kernel(const DiskArgs a, int max_nc, int max_half) {
  extern __shared__ double smem[];
  const int d = blockIdx.x, rho = blockIdx.y;
  const DiskDev D = a.disks[d];
  if (rho > D.n_periph) return;
  const int nc = D.nc, half = D.half, n = nc * half, tid = threadIdx.x, nt = blockDim.x;
  const int max_n = max_nc * max_half, max_nm = (max_nc / 2 + 1) * max_half;
  SolveSmem m;
  m.cosT = smem;
  m.sinT = m.cosT + max_nc;
  m.rhs = m.sinT + max_nc;
  m.z = m.rhs + max_n;
  m.w = m.z + max_n;
  m.C = m.w + max_n;
  m.S = m.C + max_nm;
  m.C2 = m.S + max_nm;
  m.S2 = m.C2 + max_nm;
  m.red = m.S2 + max_nm;
  for (int q = tid; q < nc; q += nt) sincospi(2.0 * q / nc, &m.sinT[q], &m.cosT[q]);
  const double* fg = a.grid + D.grid_off + n;
  if (rho == 0) {
    for (int q = tid; q < n; q += nt) m.rhs[q] = (q < nc) ? 0.0 : fg[q];
  } else {
    // Cardinal_Fourier(t_l, theta_i, n_periph / 2) on the outer ring
    const double ti = a.periph_theta[D.periph_off + rho - 1];
    const int nh = D.n_periph / 2;
    const double dt = 2 * M_PI / nc;
    for (int q = tid; q < n; q += nt) {
      double v = 0.0;
      if (q < nc) {
        // sum_{k=-nh}^{nh-1} cos(k del) = 1 + 2 sum_{k=1}^{nh-1} cos(k del) + cos(nh del),
        // the cosines by rotation from one sincos
        const double del = (q * dt + D.theta0) - ti;
        double s1, c1;
        sincos(del, &s1, &c1);
        double ck = 1.0, sk = 0.0, acc = 0.0;
        for (int k = 1; k <= nh; ++k) {
          const double cn = ck * c1 - sk * s1;
          sk = sk * c1 + ck * s1;
          ck = cn;
          acc += (k < nh) ? 2.0 * ck : ck;
        }
        v = (1.0 + acc) / (2 * nh);
      }
      m.rhs[q] = v;
    }
  }
  __syncthreads();
  const double* minv = a.minv + D.minv_off;
  if (!a.varying[d]) {
    // constant c: the solution is kept as its spectrum.  B: (C2, S2) over
    // all radii; a periphery right-hand side (zero off the outer ring): the
    // ring's transform (C, S) alone, its mode products are folded into the
    // interpolation (disk_interp_kernel)
    double* so = a.z + D.z_off + static_cast<long long>(rho) * D.zstride;
    const int nm = nc / 2 + 1;
    if (rho == 0) {
      forward_dft(D, m, m.rhs, half);
      mode_product(D, minv, m, half);
      for (int q = tid; q < nm * half; q += nt) {
        so[q] = m.C2[q];
        so[nm * half + q] = m.S2[q];
      }
    } else {
      forward_dft(D, m, m.rhs, 1);
      for (int k = tid; k < nm; k += nt) {
        so[k] = m.C[k * half];
        so[nm + k] = m.S[k * half];
      }
    }
    return;
  }
  apply_l0inv(D, minv, m, m.rhs, m.z, rho > 0);  // the cardinal right-hand sides live on the outer ring
  if (a.varying[d]) {
    const double cb = a.cbar[d];
    const double* cg = a.grid + D.grid_off;
    bool done = false;
    for (int it = 0; it < kDiskMaxIter && !done; ++it) {
      for (int q = tid; q < n; q += nt) m.w[q] = (q < nc) ? m.rhs[q] : m.rhs[q] - (cg[q] - cb) * m.z[q];
      __syncthreads();
      apply_l0inv(D, minv, m, m.w, m.w, false);
      double dmax = 0.0, zmax = 0.0;
      for (int q = tid; q < n; q += nt) {
        dmax = fmax(dmax, fabs(m.w[q] - m.z[q]));
        zmax = fmax(zmax, fabs(m.w[q]));
        m.z[q] = m.w[q];
      }
      dmax = warp_max(dmax);
      zmax = warp_max(zmax);
      if ((tid & 31) == 0) { m.red[tid >> 5] = dmax; m.red[32 + (tid >> 5)] = zmax; }
      __syncthreads();
      double dm = 0.0, zm = 0.0;
      for (int i = 0; i < (nt >> 5); ++i) { dm = fmax(dm, m.red[i]); zm = fmax(zm, m.red[32 + i]); }
      done = !(dm > 1e-15 * zm);
      __syncthreads();
    }
    if (!done && tid == 0) atomicOr(&a.flags[1], 1);
  }
  double* zo = a.z + D.z_off + static_cast<long long>(rho) * D.zstride;
  for (int q = tid; q < n; q += nt) zo[q] = m.z[q];
}

// ---------------------------------------------------------------- interp ----
// Interpolador_PS::Interpola at an interior node as a linear functional of the
// grid values z(l, j): the angular Fourier sums F_l = sum_{k=-n}^{n-1}
// cos(k (theta_p - t_l)) and F'_l = sum_k cos(k pi) cos(k (theta_p - t_l))
// (the opposite half of the diameter), the barycentric weights
// w_i = bw_i / (r_p - diam_i) and u_i = z(., i) F' (i < half),
// z(., m-1-i) F (i >= half):  value = sum_{l,j} z(l,j) (F_l w_{m-1-j} +
// F'_l w_j) / (N sum_i w_i).
__global__ void disk_interp_kernel(const DiskArgs a, long long n_inner, int max_nc, int max_half) {
  extern __shared__ double smem[];
  const int wpb = blockDim.x >> 5, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long node = static_cast<long long>(blockIdx.x) * wpb + warp;
  if (node >= n_inner) return;
  const int per = max_nc * max_half + 2 * max_nc + 2 * max_half;
  double* aco = smem + static_cast<long long>(warp) * per;
  double* Fv = aco + max_nc * max_half;
  double* Fp = Fv + max_nc;
  double* wv = Fp + max_nc;
  const int d = a.inner_disk[node];
  const DiskDev D = a.disks[d];
  const long long p = node - D.inner_off;
  const int nc = D.nc, half = D.half, m = 2 * half, n = nc * half, nh = nc / 2;
  const double px = a.inner_xy[2 * node], py = a.inner_xy[2 * node + 1];
  const double dx = px - D.cx, dy = py - D.cy;
  const double rp = sqrt(dx * dx + dy * dy) / D.radius;
  double tp = atan2(dy, dx);
  tp = (tp >= 0) ? tp : tp + 2.0 * M_PI;
  const double* T = a.tab + D.tab_off;
  double sw = 0.0;
  for (int i = lane; i < m; i += 32) {
    const double wi = T[tab_bw(half) + i] / (rp - T[tab_diam(half) + i]);
    wv[i] = wi;
    sw += wi;
  }
  sw = warp_sum(sw);
  const double scale = (1.0 / nc) / sw;
  const int np = D.n_periph;
  __syncwarp();
  if (!a.varying[d]) {
    // Spectral form (constant c).  With z's transform (C2_k(j), S2_k(j)),
    // sum_l z(l,j) F_l = sum_{k=0}^{N/2} e_k (C2_k(j) cos k phi + S2_k(j) sin k phi)
    // (e_k = 2 for 0 < k < N/2, else 1; phi = theta_p - theta_0) and F'_l adds
    // (-1)^k, so value = scale sum_{k,j} a_k(j) (C2 cos k phi + S2 sin k phi)
    // with a_k(j) = e_k (w_{m-1-j} + (-1)^k w_j).  A periphery right-hand side
    // has C2_k(j) = M_k^-1(j,0) C_k (its ring transform), so its value is
    // sum_k b_k (C_k cos k phi + S_k sin k phi), b_k = scale sum_j a_k(j) M_k^-1(j,0).
    const int nm = nh + 1;
    const double phi = tp - D.theta0;
    for (int k = lane; k < nm; k += 32) sincos(k * phi, &Fp[k], &Fv[k]);
    __syncwarp();
    const double* sb = a.z + D.z_off;
    double acc = 0.0;
    for (int q = lane; q < nm * half; q += 32) {
      const int k = q / half, j = q - k * half;
      const double e = (k == 0 || k == nh) ? 1.0 : 2.0;
      const double al = e * (wv[m - 1 - j] + ((k & 1) ? -wv[j] : wv[j]));
      acc += al * (sb[q] * Fv[k] + sb[nm * half + q] * Fp[k]);
    }
    acc = warp_sum(acc) * scale;
    if (lane == 0) {
      if (a.B) a.B[D.inner_off + p] = acc;
      if (a.Bcsr) atomicAdd(&a.Bcsr[a.inner_row[node]], acc);
    }
    const double* minv = a.minv + D.minv_off;
    for (int k = lane; k < nm; k += 32) {
      const double e = (k == 0 || k == nh) ? 1.0 : 2.0;
      double b = 0.0;
      for (int j = 0; j < half; ++j)
        b += (wv[m - 1 - j] + ((k & 1) ? -wv[j] : wv[j])) * minv[(static_cast<long long>(k) * half + j) * half];
      b *= e * scale;
      aco[k] = b * Fv[k];
      aco[nm + k] = b * Fp[k];
    }
    __syncwarp();
    for (int rho = 1 + lane; rho <= np; rho += 32) {
      const double* sr = a.z + D.z_off + static_cast<long long>(rho) * D.zstride;
      double v = 0.0;
      for (int k = 0; k < nm; ++k) v += aco[k] * sr[k] + aco[nm + k] * sr[nm + k];
      const long long g = D.g_off + p * np + (rho - 1);
      if (a.G) a.G[g] = -v;
      if (a.val) atomicAdd(&a.val[a.csr_pos[g]], -v);
    }
    return;
  }
  const double dt = 2 * M_PI / nc;
  for (int l = lane; l < nc; l += 32) {
    double s1, c1;
    sincos(tp - (l * dt + D.theta0), &s1, &c1);
    double F = 1.0, G = 1.0, ck = 1.0, sk = 0.0;
    for (int k = 1; k <= nh; ++k) {
      const double cn = ck * c1 - sk * s1;
      sk = sk * c1 + ck * s1;
      ck = cn;
      const double sg = (k & 1) ? -1.0 : 1.0;
      if (k < nh) { F += 2.0 * ck; G += 2.0 * sg * ck; }
      else { F += ck; G += sg * ck; }
    }
    Fv[l] = F;
    Fp[l] = G;
  }
  __syncwarp();
  for (int q = lane; q < n; q += 32) {
    const int j = q / nc, l = q - j * nc;
    aco[q] = Fv[l] * wv[m - 1 - j] + Fp[l] * wv[j];
  }
  __syncwarp();
  for (int rho = 0; rho <= np; ++rho) {
    const double* zr = a.z + D.z_off + static_cast<long long>(rho) * D.zstride;
    double acc = 0.0;
    for (int q = lane; q < n; q += 32) acc += aco[q] * zr[q];
    acc = warp_sum(acc);
    if (lane == 0) {
      const double v = acc * scale;
      if (rho == 0) {
        if (a.B) a.B[D.inner_off + p] = v;
        if (a.Bcsr) atomicAdd(&a.Bcsr[a.inner_row[node]], v);
      } else {
        const long long g = D.g_off + p * np + (rho - 1);
        if (a.G) a.G[g] = -v;
        if (a.val) atomicAdd(&a.val[a.csr_pos[g]], -v);
      }
    }
  }
}

}  // namespace

bool disk_prepare(const std::vector<DiskHost>& in, DiskBatch& out, std::string& err) {
  out = DiskBatch();
  std::map<std::pair<double, int>, long long> classes;
  std::map<int, long long> modes;
  long long inner = 0, g = 0, periph = 0;
  out.has_csr = !in.empty();
  for (size_t di = 0; di < in.size(); ++di) {
    const DiskHost& h = in[di];
    const int np = static_cast<int>(h.periph_theta.size());
    const int ni = static_cast<int>(h.inner_xy.size() / 2);
    if (h.n_circle < 2 || h.n_circle % 2 || h.n_circle > kDiskMaxCircle) {
      err = "disk: N_circunferencia must be even, 2.." + std::to_string(kDiskMaxCircle);
      return false;
    }
    if (h.n_radial < 3 || h.n_radial % 2 == 0 || h.n_radial > kDiskMaxRadial) {
      err = "disk: N_radio must be odd, 3.." + std::to_string(kDiskMaxRadial);
      return false;
    }
    if (np < 2 || np > kDiskMaxPeriph) {
      err = "disk: periphery nodes must number 2.." + std::to_string(kDiskMaxPeriph);
      return false;
    }
    if (!(h.radius > 0) || h.inner_xy.size() % 2) {
      err = "disk: radius must be > 0 and interior positions come in (x, y) pairs";
      return false;
    }
    const bool csr = !h.csr_pos.empty();
    if (csr && (h.csr_pos.size() != static_cast<size_t>(ni) * np || h.inner_row.size() != static_cast<size_t>(ni))) {
      err = "disk: CSR positions must cover every (interior, periphery) pair";
      return false;
    }
    out.has_csr = out.has_csr && csr;
    DiskDev D;
    D.cx = h.cx; D.cy = h.cy; D.radius = h.radius; D.theta0 = h.theta0;
    D.nc = h.n_circle;
    D.half = (h.n_radial + 1) / 2;
    D.n_periph = np;
    D.n_inner = ni;
    const auto ck = std::make_pair(h.radius, h.n_radial);
    auto it = classes.find(ck);
    if (it == classes.end()) {
      it = classes.emplace(ck, static_cast<long long>(out.tab.size())).first;
      radial_class(h.radius, h.n_radial, out.tab);
    }
    D.tab_off = it->second;
    auto mt = modes.find(h.n_circle);
    if (mt == modes.end()) {
      mt = modes.emplace(h.n_circle, static_cast<long long>(out.tab.size())).first;
      mode_eigenvalues(h.n_circle, out.tab);
    }
    D.mu_off = mt->second;
    const long long n = static_cast<long long>(D.nc) * D.half;
    D.grid_off = out.grid_total;
    out.grid_total += 2 * n;
    D.minv_off = out.minv_total;
    out.minv_total += static_cast<long long>(D.nc / 2 + 1) * D.half * D.half;
    // per right-hand side: grid values (varying c) or the spectrum (constant c)
    D.zstride = std::max(n, 2LL * (D.nc / 2 + 1) * D.half);
    D.z_off = out.z_total;
    out.z_total += (np + 1) * D.zstride;
    D.inner_off = inner;
    D.g_off = g;
    D.periph_off = periph;
    inner += ni;
    g += static_cast<long long>(ni) * np;
    periph += np;
    out.periph_theta.insert(out.periph_theta.end(), h.periph_theta.begin(), h.periph_theta.end());
    out.inner_xy.insert(out.inner_xy.end(), h.inner_xy.begin(), h.inner_xy.end());
    out.inner_disk.insert(out.inner_disk.end(), ni, static_cast<int>(di));
    out.inner_row.insert(out.inner_row.end(), h.inner_row.begin(), h.inner_row.end());
    out.csr_pos.insert(out.csr_pos.end(), h.csr_pos.begin(), h.csr_pos.end());
    out.max_nc = std::max(out.max_nc, D.nc);
    out.max_half = std::max(out.max_half, D.half);
    out.max_rhs = std::max(out.max_rhs, np + 1);
    out.max_modes = std::max(out.max_modes, D.nc / 2 + 1);
    out.disks.push_back(D);
  }
  out.n_inner = inner;
  out.g_total = g;
  if (!out.has_csr) {
    out.inner_row.clear();
    out.csr_pos.clear();
  }
  return true;
}

cudaError_t disk_launch(int problem, const DiskArgs& a, const DiskBatch& b, cudaStream_t s, cudaEvent_t* ev) {
  if (a.n_disks == 0) return cudaSuccess;
  if (ev) cudaEventRecord(ev[0], s);
  with_problem(problem, [&](auto t) { disk_coef_kernel<decltype(t)::value><<<a.n_disks, kCoefThreads, 0, s>>>(a); });
  const size_t mode_smem = static_cast<size_t>(kModeWarps) * b.max_half * (2 * b.max_half + 1) * sizeof(double);
  cudaError_t em = cudaFuncSetAttribute(disk_modes_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        static_cast<int>(mode_smem));
  if (em != cudaSuccess) return em;
  disk_modes_kernel<<<dim3(a.n_disks, (b.max_modes + kModeWarps - 1) / kModeWarps), 32 * kModeWarps, mode_smem, s>>>(
      a, b.max_half);
  const size_t max_n = static_cast<size_t>(b.max_nc) * b.max_half;
  const size_t max_nm = static_cast<size_t>(b.max_nc / 2 + 1) * b.max_half;
  const size_t solve_smem = (2 * b.max_nc + 3 * max_n + 4 * max_nm + 64) * sizeof(double);
  cudaError_t e = cudaFuncSetAttribute(disk_solve_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(solve_smem));
  if (e != cudaSuccess) return e;
  disk_solve_kernel<<<dim3(a.n_disks, b.max_rhs), kSolveThreads, solve_smem, s>>>(a, b.max_nc, b.max_half);
  if (ev) cudaEventRecord(ev[1], s);
  if (b.n_inner > 0) {
    const size_t per = (max_n + 2 * b.max_nc + 2 * b.max_half) * sizeof(double);
    const int wpb = static_cast<int>(std::max<size_t>(1, std::min<size_t>(8, kInterpSmemBudget / per)));
    const size_t smem = per * wpb;
    e = cudaFuncSetAttribute(disk_interp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    const long long grid = (b.n_inner + wpb - 1) / wpb;
    disk_interp_kernel<<<static_cast<unsigned>(grid), 32 * wpb, smem, s>>>(a, b.n_inner, b.max_nc, b.max_half);
  }
  if (ev) cudaEventRecord(ev[2], s);
  return cudaGetLastError();
}

}  // namespace fk
