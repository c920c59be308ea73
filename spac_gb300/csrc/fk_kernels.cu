// GB300 (sm_103a) kernels of the Feynman-Kac hot path.
//
//  paths_kernel   persistent grid; each CTA takes chunks of one item's paths
//                 from a global queue, every thread runs one path at a time and
//                 pulls the next path index of the chunk as soon as its path
//                 exits (per-lane regeneration: lanes never wait for the
//                 longest path of a warp).  The exit is processed in place:
//                 exit value, B and statistics into per-thread registers,
//                 stencil weights into shared-memory accumulators, flushed to
//                 FP64 per-item accumulators at the end of the chunk.
//                 Replaces Simulacion_OMP + Reduce_Analytic + Interfaz::Update_G
//                 (Solvers/FeynmanKacSolver.cpp:137-292, Mesh/Interfaz.cpp:219-264).
//  finalize_kernel  per item: applies the stencil inverse to the accumulated
//                 RBF moments (FP64), averages (Update(Nudo&), :324-334) and
//                 scatters G into the CSR row and B into the right-hand side
//                 (SistemaLineal::Actualiza_GB, Mesh/SistemaLineal.cpp:68-88).
//  inverse_kernel FP64 Gauss-Jordan with full pivoting, one CTA per matrix,
//                 non-contracted arithmetic: the same bits as the CPU
//                 restatement of Eigen::FullPivLU::inverse (Interfaz.cpp:214).
#include <cfloat>
#include <type_traits>

#include "fk_device.cuh"
#include "fk_internal.h"

namespace fk {

// ------------------------------------------------------------ accumulators --
struct AccD {
  double s = 0.0;
  __device__ __forceinline__ void add(double v) { s += v; }
  __device__ __forceinline__ double get() const { return s; }
};
// Compensated (Kahan) FP32 sum for FP32 stepping: FP64-grade sums of a
// thread's exits without FP64 arithmetic in the path loop.
struct AccK {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float v) {
    const float y = v - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ __forceinline__ double get() const { return static_cast<double>(s) - static_cast<double>(c); }
};

constexpr int kNumAcc = 11;  // accumulated per thread: see the exit block
constexpr int kMaxWarps = 32;

template <typename R, int ST>
struct SAccType {
  // arc stencils (kappa(Psi) ~ 1e10) always accumulate in FP64
  using type = typename std::conditional<std::is_same<R, double>::value || ST == 1, double, float>::type;
};

// Window (first chain index) of the k nearest patch-boundary nodes to an exit
// point on the patch boundary.  The k nearest nodes of a point on a convex
// boundary chain are a contiguous run of the chain; start from the run
// centred on the nearest node of the exit side and slide while an outside
// neighbour is closer than the opposite end of the run.
template <typename R>
__device__ __forceinline__ int knn_window(const PatchDev& P, const double* __restrict__ nodes, R ex, R ey) {
  int best_s = -1;
  R best = R(FLT_MAX);
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    if (P.side_count[s] > 0) {
      const R dist = fabs((P.side_axis[s] == 0 ? ey : ex) - R(P.side_fixed[s]));
      if (dist < best) { best = dist; best_s = s; }
    }
  }
  const int m = P.m, k = P.k;
  int nearest = 0;
  if (best_s >= 0) {
    const R coord = P.side_axis[best_s] == 0 ? ex : ey;
    int j = __double2int_rn((static_cast<double>(coord) - P.side_start[best_s]) / P.side_step[best_s]);
    j = max(0, min(P.side_count[best_s] - 1, j));
    nearest = P.side_first[best_s] + j;
  }
  auto d2 = [&](int idx) -> R {
    if (P.closed) { idx %= m; if (idx < 0) idx += m; }
    const R dx = ex - R(nodes[2 * idx]), dy = ey - R(nodes[2 * idx + 1]);
    return dx * dx + dy * dy;
  };
  int L = nearest - k / 2;
  if (P.closed) {
    for (int it = 0; it < m && d2(L - 1) < d2(L + k - 1); ++it) --L;
    for (int it = 0; it < m && d2(L + k) < d2(L); ++it) ++L;
    L %= m;
    if (L < 0) L += m;
  } else {
    L = max(0, min(m - k, L));
    while (L > 0 && d2(L - 1) < d2(L + k - 1)) --L;
    while (L < m - k && d2(L + k) < d2(L)) ++L;
  }
  return L;
}

template <typename R, int PROB, int ST>
__global__ void __launch_bounds__(256) paths_kernel(const LaunchArgs a) {
  using SAcc = typename SAccType<R, ST>::type;
  using Acc = typename std::conditional<std::is_same<R, double>::value, AccD, AccK>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SAcc* sacc = reinterpret_cast<SAcc*>(smem_raw);
  __shared__ int s_chunk;
  __shared__ unsigned s_next;
  __shared__ double s_red[kNumAcc][kMaxWarps];

  const BvpDev bvp = *a.bvp;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const bool cv = a.cv != 0;

  for (;;) {
    if (threadIdx.x == 0) s_chunk = atomicAdd(a.queue, 1);
    __syncthreads();
    const int c = s_chunk;
    if (c >= a.n_chunks) break;
    const ChunkDev ch = a.chunks[c];
    const ItemDev it = a.items[ch.item];
    for (int i = threadIdx.x; i < a.acc_words; i += blockDim.x) sacc[i] = SAcc(0);
    if (threadIdx.x == 0) s_next = ch.p0 + blockDim.x;
    __syncthreads();

    const R h = R(it.h), sqrth = R(it.sqrth), x0 = R(it.x), y0 = R(it.y);
    const R s0 = R(it.sub[0]), s1 = R(it.sub[1]), s2 = R(it.sub[2]), s3 = R(it.sub[3]);
    // stencil metadata
    ArcDev arc;
    PatchDev patch;
    const double* theta = nullptr;
    if (ST == 1) { arc = a.arcs[it.stencil]; theta = a.arc_theta + arc.theta_off; }
    if (ST == 2) { patch = a.patches[it.stencil]; }
    const double* pnodes = (ST == 2) ? a.patch_nodes + patch.node_off : nullptr;

    Acc acc[kNumAcc];
    R x = x0, y = y0, Y = R(1), Z = R(0), xi = R(0);
    int k = 0;
    uint32_t w2 = 0, w3 = 0;
    unsigned p = ch.p0 + threadIdx.x;

    while (p < ch.p1) {
      // ---- one Euler-Maruyama step (Paso_Absorbente, FeynmanKacSolver.cpp:7-18)
      StepCoef<R> co;
      Problem<PROB>::step(bvp, x, y, cv, co);
      uint32_t wa, wb;
      if ((k & 1) == 0) {
        const uint4 r = philox10(make_uint4(static_cast<uint32_t>(k >> 1), p, static_cast<uint32_t>(ch.item), a.stream),
                                 a.key0, a.key1);
        wa = r.x; wb = r.y; w2 = r.z; w3 = r.w;
      } else {
        wa = w2; wb = w3;
      }
      R z0, z1;
      box_muller(wa, wb, z0, z1);
      const R dWx = sqrth * z0, dWy = sqrth * z1;
      Z += co.f * Y * h;
      if (cv) xi += Y * (co.Fx * dWx + co.Fy * dWy);
      Y += co.c * Y * h;
      x += co.bx * h + co.s * dWx;
      y += co.by * h + co.s * dWy;
      ++k;
      // ---- exit rule (Dentro, FeynmanKacSolver.cpp:68-106)
      Bnd<R> w = (PROB == 3) ? circle_dist<R>(x, y, R(bvp.dom[0]), R(bvp.dom[1]), R(bvp.dom[2]))
                             : rect_dist<R>(x, y, R(bvp.dom[0]), R(bvp.dom[1]), R(bvp.dom[2]), R(bvp.dom[3]));
      bool dom_wins = true;
      if (ST != 0 || it.sub_shape >= 0) {
        const Bnd<R> sb = (ST == 1 || (ST == 0 && it.sub_shape == 1)) ? circle_dist<R>(x, y, s0, s1, s2)
                                                                       : rect_dist<R>(x, y, s0, s1, s2, s3);
        if (!(w.d >= sb.d)) { w = sb; dom_wins = false; }
      }
      const R sg = (w.d < R(0)) ? Problem<PROB>::sigma(bvp, x, y) : Problem<PROB>::sigma(bvp, w.ex, w.ey);
      const R nsx = w.nx * sg, nsy = w.ny * sg;
      const R thr = R(kGobet) * sqrt(nsx * nsx + nsy * nsy) * sqrth;
      const bool capped = k >= a.max_steps;
      if (!(w.d < thr) || capped) {
        // ---- exit: Reduce_Analytic (FeynmanKacSolver.cpp:198-292)
        const R g = Problem<PROB>::u(bvp, w.ex, w.ey);  // g = u for every registered problem
        const R score = Z + Y * g;
        const R vr = score + xi;
        R bpart = vr;
        if (ST != 0 && !dom_wins) {
          bpart = Z + xi;
          if (ST == 1) {
            // Interfaz::Update_G moments: s_i += Y phi_i(theta), FP64
            const double th = arc_theta(arc.interior, static_cast<double>(w.ex) - arc.cx,
                                        static_cast<double>(w.ey) - arc.cy);
            const double Yd = static_cast<double>(Y);
            for (int i = 0; i < arc.n; ++i) {
              const double d = th - theta[i];
              atomicAdd(reinterpret_cast<double*>(&sacc[i]), Yd / sqrt(d * d + arc.c2));
            }
          } else if (ST == 2) {
            const int L = knn_window<R>(patch, pnodes, w.ex, w.ey);
            const int m = patch.m, kk = patch.k;
            const R e2 = R(patch.eps2);
            for (int q = 0; q < kk; ++q) {
              int idx = L + q;
              if (idx >= m) idx -= m;
              const R dx = w.ex - R(pnodes[2 * idx]), dy = w.ey - R(pnodes[2 * idx + 1]);
              atomicAdd(&sacc[L * kk + q], static_cast<SAcc>(Y * exp(-e2 * (dx * dx + dy * dy))));
            }
          }
        }
        acc[0].add(score);
        acc[1].add(score * score);
        acc[2].add(xi + xi * xi);
        acc[3].add(vr);
        acc[4].add(vr * vr);
        acc[5].add(xi * score);
        acc[6].add(R(k));
        acc[7].add(bpart);
        acc[8].add(dom_wins ? R(1) : R(0));
        acc[9].add(capped ? R(1) : R(0));
        acc[10].add(xi * xi);
        // regenerate: next path of this chunk
        p = atomicAdd(&s_next, 1u);
        x = x0; y = y0; Y = R(1); Z = R(0); xi = R(0); k = 0;
      }
    }
    // xi (plain sum) is recovered at finalize from slots 2 and 10
    __syncthreads();
    // ---- chunk flush: block reduction of the thread sums, FP64 atomics per item
#pragma unroll
    for (int j = 0; j < kNumAcc; ++j) {
      double v = acc[j].get();
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) s_red[j][warp] = v;
    }
    __syncthreads();
    if (threadIdx.x < kNumAcc) {
      double v = 0.0;
      for (int w = 0; w < nwarps; ++w) v += s_red[threadIdx.x][w];
      if (v != 0.0) atomicAdd(&a.stats[static_cast<long long>(ch.item) * kNumStats + threadIdx.x], v);
    }
    if (ST != 0) {
      double* gacc = a.acc + it.acc_off;
      for (int i = threadIdx.x; i < a.acc_words; i += blockDim.x) {
        const double v = static_cast<double>(sacc[i]);
        if (v != 0.0) atomicAdd(&gacc[i], v);
      }
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------- finalize -----
// fk_stats layout (16 doubles): phi, phiphi, phi_VR, phiphi_VR, xi, xixi,
// xiphi, APL, RNGC, B, n_paths, n_domain_exits, n_capped, xi_mean,
// xi_sq_mean, mean_steps.
template <int PROB>
__global__ void finalize_kernel(const FinalizeArgs a) {
  const int item = blockIdx.x;
  if (item >= a.n_items) return;
  const ItemDev it = a.items[item];
  const BvpDev bvp = *a.bvp;
  const double N = static_cast<double>(it.paths);
  const double* S = a.stats + static_cast<long long>(item) * kNumStats;
  double Bv;
  if (it.frontera) {
    Bv = Problem<PROB>::u(bvp, it.x, it.y);  // Solve_OMP_Analytic :346-347
  } else {
    Bv = S[7] / N;
  }
  if (threadIdx.x == 0) {
    if (a.item_stats) {
      double* o = a.item_stats + static_cast<long long>(item) * 16;
      if (it.frontera) {
        for (int j = 0; j < 16; ++j) o[j] = 0.0;
        o[9] = Bv;
      } else {
        // slot 2 holds sum(xi + xi^2); the reference adds it twice (xi/xixi aliasing)
        o[0] = S[0] / N; o[1] = S[1] / N; o[2] = S[3] / N; o[3] = S[4] / N;
        o[4] = (S[2] + S[2]) / N; o[5] = (S[2] + S[2]) / N; o[6] = S[5] / N;
        o[7] = it.h * S[6] / N; o[8] = 4.0 * S[6]; o[9] = Bv; o[10] = N; o[11] = S[8]; o[12] = S[9];
        o[13] = (S[2] - S[10]) / N; o[14] = S[10] / N; o[15] = S[6] / N;
      }
    }
    if (a.item_B) a.item_B[item] = Bv;
    if (a.B) atomicAdd(&a.B[a.row[item]], Bv);
  }
  if (a.stencil_kind == 0 || it.stencil < 0) return;
  const double* acc = a.acc + it.acc_off;
  const long long goff = a.g_off ? a.g_off[item] : 0;
  if (a.stencil_kind == 1) {
    const ArcDev arc = a.arcs[it.stencil];
    const double* iPsi = a.arc_ipsi + arc.ipsi_off;
    for (int j = threadIdx.x; j < arc.n; j += blockDim.x) {
      double g = 0.0;
      if (!it.frontera) {
        for (int i = 0; i < arc.n; ++i) g += iPsi[i + j * arc.n] * acc[i];
        g = -g / N;
      }
      if (a.item_G) a.item_G[goff + j] = g;
      if (a.csr_val && !it.frontera) a.csr_val[a.csr_idx[goff + j]] += g;
    }
  } else {
    const PatchDev P = a.patches[it.stencil];
    const double* Ainv = a.patch_ainv + P.ainv_off;
    const int m = P.m, k = P.k;
    for (int gi = threadIdx.x; gi < m; gi += blockDim.x) {
      double g = 0.0;
      if (!it.frontera) {
        if (P.closed) {
          for (int t = 0; t < k; ++t) {
            int W = gi - t;
            if (W < 0) W += m;
            const double* Ai = Ainv + static_cast<long long>(W) * k * k;
            const double* tw = acc + static_cast<long long>(W) * k;
            for (int b = 0; b < k; ++b) g += Ai[t + b * k] * tw[b];
          }
        } else {
          const int wlo = max(0, gi - k + 1), whi = min(gi, m - k);
          for (int W = wlo; W <= whi; ++W) {
            const int t = gi - W;
            const double* Ai = Ainv + static_cast<long long>(W) * k * k;
            const double* tw = acc + static_cast<long long>(W) * k;
            for (int b = 0; b < k; ++b) g += Ai[t + b * k] * tw[b];
          }
        }
        g = -g / N;
      }
      if (a.item_G) a.item_G[goff + gi] = g;
      if (a.csr_val && !it.frontera) a.csr_val[a.csr_idx[goff + gi]] += g;
    }
  }
}

// ---------------------------------------------------- FP64 matrix builders --
// Psi_ij = 1/sqrt((theta_i - theta_j)^2 + c2)  (Interfaz::Calcula_Psi with
// BVP::RBF = Inverse_Multiquadric, BVP/BVP.cpp:22-24), correctly rounded
// operations only.
__global__ void build_psi_kernel(const ArcDev* arcs, const double* theta, int n_arcs, double* out) {
  const int a = blockIdx.y;
  if (a >= n_arcs) return;
  const ArcDev A = arcs[a];
  const double* th = theta + A.theta_off;
  double* o = out + A.ipsi_off;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < A.n * A.n; e += gridDim.x * blockDim.x) {
    const int i = e % A.n, j = e / A.n;
    const double d = __dsub_rn(th[i], th[j]);
    o[i + j * A.n] = __ddiv_rn(1.0, __dsqrt_rn(__dadd_rn(__dmul_rn(d, d), A.c2)));
  }
}

// A_W(a,b) = exp(-eps^2 |x_a - x_b|^2) for every window of every patch.
__global__ void build_windows_kernel(const PatchDev* patches, const double* nodes, int n_patches,
                                     const long long* win_base, long long total, int k, double* out) {
  const long long gw = blockIdx.x;
  if (gw >= total) return;
  int p = 0;
  while (p + 1 < n_patches && win_base[p + 1] <= gw) ++p;
  const PatchDev P = patches[p];
  const int W = static_cast<int>(gw - win_base[p]);
  const double* nd = nodes + P.node_off;
  double* o = out + P.ainv_off + static_cast<long long>(W) * k * k;
  for (int e = threadIdx.x; e < k * k; e += blockDim.x) {
    const int a = e % k, b = e / k;
    int ia = W + a, ib = W + b;
    if (ia >= P.m) ia -= P.m;
    if (ib >= P.m) ib -= P.m;
    const double dx = nd[2 * ia] - nd[2 * ib], dy = nd[2 * ia + 1] - nd[2 * ib + 1];
    o[a + b * k] = exp(-P.eps2 * (dx * dx + dy * dy));
  }
}

// Gauss-Jordan with full pivoting (same pivot order and the same
// non-contracted FP64 operations as the CPU restatement): pivot = first
// maximum of |a_ij| over the trailing block in row-major order.
__global__ void inverse_kernel(const double* A, double* inv, const int* ns, const long long* offs) {
  extern __shared__ double sm[];
  const int n = ns[blockIdx.x];
  double* a = sm;                 // n*n
  double* v = sm + n * n;         // n*n
  __shared__ int s_piv[128];
  __shared__ double s_bv[256];
  __shared__ int s_bi[256];
  __shared__ double s_col[128];
  const double* Ag = A + offs[blockIdx.x];
  double* Vg = inv + offs[blockIdx.x];
  const int nn = n * n;
  for (int e = threadIdx.x; e < nn; e += blockDim.x) {
    a[e] = Ag[e];
    v[e] = ((e % n) == (e / n)) ? 1.0 : 0.0;
  }
  __syncthreads();
  for (int k = 0; k < n; ++k) {
    // pivot search
    double bv = -1.0;
    int bi = 0x7fffffff;
    const int m = n - k;
    for (int e = threadIdx.x; e < m * m; e += blockDim.x) {
      const int i = k + e / m, j = k + e % m;  // row-major scan order
      const double val = fabs(a[i + j * n]);
      const int lin = i * n + j;
      if (val > bv || (val == bv && lin < bi)) { bv = val; bi = lin; }
    }
    s_bv[threadIdx.x] = bv;
    s_bi[threadIdx.x] = bi;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
      if (threadIdx.x < o) {
        const double v2 = s_bv[threadIdx.x + o];
        const int i2 = s_bi[threadIdx.x + o];
        if (v2 > s_bv[threadIdx.x] || (v2 == s_bv[threadIdx.x] && i2 < s_bi[threadIdx.x])) {
          s_bv[threadIdx.x] = v2;
          s_bi[threadIdx.x] = i2;
        }
      }
      __syncthreads();
    }
    const int pr = s_bi[0] / n, pc = s_bi[0] % n;
    __syncthreads();
    if (pr != k)
      for (int j = threadIdx.x; j < n; j += blockDim.x) {
        double t = a[k + j * n]; a[k + j * n] = a[pr + j * n]; a[pr + j * n] = t;
        t = v[k + j * n]; v[k + j * n] = v[pr + j * n]; v[pr + j * n] = t;
      }
    __syncthreads();
    if (pc != k)
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double t = a[i + k * n]; a[i + k * n] = a[i + pc * n]; a[i + pc * n] = t;
      }
    if (threadIdx.x == 0) s_piv[k] = pc;
    __syncthreads();
    const double piv = a[k + k * n];
    __syncthreads();
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
      a[k + j * n] = __ddiv_rn(a[k + j * n], piv);
      v[k + j * n] = __ddiv_rn(v[k + j * n], piv);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) s_col[i] = a[i + k * n];
    __syncthreads();
    for (int e = threadIdx.x; e < nn; e += blockDim.x) {
      const int i = e % n, j = e / n;
      const double f = s_col[i];
      if (i == k || f == 0.0) continue;
      a[i + j * n] = __dsub_rn(a[i + j * n], __dmul_rn(f, a[k + j * n]));
      v[i + j * n] = __dsub_rn(v[i + j * n], __dmul_rn(f, v[k + j * n]));
    }
    __syncthreads();
  }
  for (int k = n - 1; k >= 0; --k) {
    const int pc = s_piv[k];
    if (pc != k)
      for (int j = threadIdx.x; j < n; j += blockDim.x) {
        const double t = v[k + j * n]; v[k + j * n] = v[pc + j * n]; v[pc + j * n] = t;
      }
    __syncthreads();
  }
  for (int e = threadIdx.x; e < nn; e += blockDim.x) Vg[e] = v[e];
}

// --------------------------------------------------------------- dispatch ---
template <typename R, int PROB>
static const void* paths_fn(int st) {
  switch (st) {
    case 1: return reinterpret_cast<const void*>(&paths_kernel<R, PROB, 1>);
    case 2: return reinterpret_cast<const void*>(&paths_kernel<R, PROB, 2>);
    default: return reinterpret_cast<const void*>(&paths_kernel<R, PROB, 0>);
  }
}
template <typename R>
static const void* paths_fn_r(int problem, int st) {
  switch (problem) {
    case 1: return paths_fn<R, 1>(st);
    case 2: return paths_fn<R, 2>(st);
    case 3: return paths_fn<R, 3>(st);
    default: return paths_fn<R, 0>(st);
  }
}
static const void* select_paths(int problem, int precision, int st) {
  return precision == 1 ? paths_fn_r<float>(problem, st) : paths_fn_r<double>(problem, st);
}

cudaError_t launch_paths(const LaunchArgs& a, int problem, int precision, int grid, int block, size_t smem,
                         cudaStream_t s) {
  const void* fn = select_paths(problem, precision, a.stencil_kind);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess) return e;
  }
  void* args[] = {const_cast<LaunchArgs*>(&a)};
  return cudaLaunchKernel(fn, dim3(grid), dim3(block), args, smem, s);
}

int paths_kernel_occupancy(int problem, int precision, int stencil_kind, int, int block, size_t smem) {
  const void* fn = select_paths(problem, precision, stencil_kind);
  if (smem > 48 * 1024) cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, block, smem) != cudaSuccess) return 1;
  return n > 0 ? n : 1;
}

cudaError_t launch_finalize(const FinalizeArgs& a, int problem, cudaStream_t s) {
  if (a.n_items <= 0) return cudaSuccess;
  const dim3 grid(a.n_items), block(128);
  switch (problem) {
    case 1: finalize_kernel<1><<<grid, block, 0, s>>>(a); break;
    case 2: finalize_kernel<2><<<grid, block, 0, s>>>(a); break;
    case 3: finalize_kernel<3><<<grid, block, 0, s>>>(a); break;
    default: finalize_kernel<0><<<grid, block, 0, s>>>(a); break;
  }
  return cudaGetLastError();
}

cudaError_t launch_inverse(const double* A, double* inv, const int* ns, const long long* offs, int nmax, int count,
                           cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  if (nmax > 64) return cudaErrorInvalidValue;
  const size_t smem = 2ull * nmax * nmax * sizeof(double);
  cudaError_t e = cudaFuncSetAttribute(inverse_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(smem));
  if (e != cudaSuccess) return e;
  inverse_kernel<<<count, 256, smem, s>>>(A, inv, ns, offs);
  return cudaGetLastError();
}

cudaError_t launch_build_psi(const ArcDev* arcs, const double* theta, int n_arcs, double* out, cudaStream_t s) {
  if (n_arcs <= 0) return cudaSuccess;
  build_psi_kernel<<<dim3(4, n_arcs), 256, 0, s>>>(arcs, theta, n_arcs, out);
  return cudaGetLastError();
}

cudaError_t launch_build_windows(const PatchDev* patches, const double* nodes, int n_patches,
                                 const long long* win_base, long long total_windows, int k, double* out,
                                 cudaStream_t s) {
  if (total_windows <= 0) return cudaSuccess;
  build_windows_kernel<<<static_cast<unsigned>(total_windows), 128, 0, s>>>(patches, nodes, n_patches, win_base,
                                                                             total_windows, k, out);
  return cudaGetLastError();
}

}  // namespace fk
