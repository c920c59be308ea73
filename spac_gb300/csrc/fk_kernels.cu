// GB300 (sm_103a) kernels of the Feynman-Kac hot path.
//
//  (the path kernel itself is in fk_paths.cu)
//  finalize_kernel  per item: applies the stencil inverse to the accumulated
//                 RBF moments (FP64), averages (Update(Nudo&), :324-334) and
//                 scatters G into the CSR row and B into the right-hand side
//                 (SistemaLineal::Actualiza_GB, Mesh/SistemaLineal.cpp:68-88).
//  inverse_kernel FP64 Gauss-Jordan with full pivoting, one CTA per matrix,
//                 non-contracted arithmetic: the same bits as the CPU
//                 restatement of Eigen::FullPivLU::inverse (Interfaz.cpp:214).
#include "fk_device.cuh"
#include "fk_internal.h"

namespace fk {

// ------------------------------------------------------------- finalize -----
constexpr int kMaxFinalizeWindows = 1024;  // windows flagged in shared memory (more: no skipping)
constexpr int kMaxSplitWords = 6144;       // FP32 moments staged in shared memory (more: FP64 path)
constexpr int kFinalizeParts = 4;          // threads per G entry of a patch row
constexpr int kFinalizeThreads = 512;

// fk_stats layout (16 doubles): phi, phiphi, phi_VR, phiphi_VR, xi, xixi,
// xiphi, APL, RNGC, B, n_paths, n_domain_exits, n_capped, xi_mean,
// xi_sq_mean, mean_steps.
// Per-item statistics, B and the result flags (thread 0 of the item's CTA).
template <int PROB>
__device__ __forceinline__ void finalize_item_head(const FinalizeArgs& a, int item, const ItemDev& it, bool live,
                                                   double N) {
  const BvpDev bvp = a.bvp[it.bvp];
  const double* S = a.stats + static_cast<long long>(item) * kNumStats;
  double Bv;
  if (it.frontera) {
    Bv = Problem<PROB>::u(bvp, it.x, it.y);  // Solve_OMP_Analytic :346-347
  } else {
    Bv = live ? S[7] / N : 0.0;
  }
  if (a.item_stats) {
    double* o = a.item_stats + static_cast<long long>(item) * 16;
    if (!live) {
      for (int j = 0; j < 16; ++j) o[j] = 0.0;
      o[9] = Bv;
    } else {
      // slot 2 holds sum(xi + xi^2); the reference adds it twice (xi/xixi aliasing)
      o[0] = S[0] / N; o[1] = S[1] / N; o[2] = S[3] / N; o[3] = S[4] / N;
      o[4] = (S[2] + S[2]) / N; o[5] = (S[2] + S[2]) / N; o[6] = S[5] / N;
      o[7] = it.h * S[6] / N; o[8] = 4.0 * S[6]; o[9] = Bv; o[10] = S[kStatPaths]; o[11] = S[8]; o[12] = S[9];
      o[13] = (S[2] - S[10]) / N; o[14] = S[10] / N; o[15] = S[6] / N;
    }
  }
  if (a.item_B) a.item_B[item] = Bv;
  if (a.B) atomicAdd(&a.B[a.row[item]], Bv);
  if (a.flags && live) {
    if (S[kStatCap] > 0.0) atomicOr(&a.flags[0], 1);
    if (S[kStatPaths] != N) {  // every requested path must have completed, once
      atomicOr(&a.flags[1], 1);
      if (a.lost && atomicCAS(&a.lost[0], 0, item + 1) == 0) a.lost[1] = static_cast<int>(S[kStatPaths]);
    }
  }
}

template <int PROB>
__global__ void finalize_kernel(const FinalizeArgs a) {
  const int item = blockIdx.x;
  if (item >= a.n_items) return;
  const ItemDev it = a.items[item];
  const double N = static_cast<double>(it.paths);
  // an item given no paths contributes nothing (G = 0, B = 0)
  const bool live = !it.frontera && it.paths > 0;
  if (threadIdx.x == 0) finalize_item_head<PROB>(a, item, it, live, N);
  if (a.stencil_kind == 0 || it.stencil < 0) return;
  const double* acc = a.acc + it.acc_off;
  const long long goff = a.g_off ? a.g_off[item] : 0;
  if (a.stencil_kind == 1) {
    const ArcDev arc = a.arcs[it.stencil];
    const double* iPsi = a.arc_ipsi + arc.ipsi_off;
    for (int j = threadIdx.x; j < arc.n; j += blockDim.x) {
      double g = 0.0;
      if (live) {
        for (int i = 0; i < arc.n; ++i) g += iPsi[i + j * arc.n] * acc[i];
        g = -g / N;
      }
      if (a.item_G) a.item_G[goff + j] = g;
      if (a.csr_val && live) atomicAdd(&a.csr_val[a.csr_idx[goff + j]], g);  // rows of several items may share columns
    }
  } else {
    const PatchDev P = a.patches[it.stencil];
    const double* Ainv = a.patch_ainv + P.ainv_off;
    const int m = P.m, k = P.k;
    // windows that no exit of this item chose have zero moments: flag the
    // visited ones so that the FP64 products below skip the others
    __shared__ unsigned char visited[kMaxFinalizeWindows];
    const bool flags = m <= kMaxFinalizeWindows;
    if (flags && live) {
      for (int W = threadIdx.x; W < P.nwin; W += blockDim.x) {
        const double* tw = acc + static_cast<long long>(W) * k;
        bool any = false;
        for (int b = 0; b < k; ++b) any |= tw[b] != 0.0;
        visited[W] = any ? 1 : 0;
      }
    }
    // FP32-stepping assemblies with a well-conditioned stencil (A_W^-1 = I + E,
    // max |E| < kSplitMaxE): G = -(sum_W t_W[t] + sum_W E_W t_W) / N with the
    // first sum in FP64 and the correction in FP32 (relative error of G
    // ~1e-7 max|E|); the moments are staged as FP32 in shared memory
    __shared__ float t32[kMaxSplitWords];
    const long long words = static_cast<long long>(P.nwin) * k;
    const bool split = a.split_ok && a.patch_e32 && a.patch_emax[it.stencil] < kSplitMaxE && words <= kMaxSplitWords;
    if (split && live)
      for (int i = threadIdx.x; i < words; i += blockDim.x) t32[i] = static_cast<float>(acc[i]);
    __syncthreads();
    const float* E = split ? a.patch_e32 + P.ainv_off : nullptr;
    // kFinalizeParts consecutive threads per G entry, each over every
    // kFinalizeParts-th window covering it (short dependency chains); the
    // partial sums are combined by a fixed shuffle tree
    const int part = threadIdx.x % kFinalizeParts;
    for (int base = 0; base < m; base += blockDim.x / kFinalizeParts) {
      const int gi = base + threadIdx.x / kFinalizeParts;
      double g = 0.0;
      float corr = 0.f;
      if (gi < m && live) {
        auto add = [&](int W, int t) {
          if (flags && !visited[W]) return;
          const double* tw = acc + static_cast<long long>(W) * k;
          if (split) {
            g += tw[t];
            const float* Ew = E + static_cast<long long>(W) * k * k;
            const float* tw32 = t32 + W * k;
            for (int b = 0; b < k; ++b) corr = fmaf(Ew[t + b * k], tw32[b], corr);
          } else {
            const double* Ai = Ainv + static_cast<long long>(W) * k * k;
            for (int b = 0; b < k; ++b) g += Ai[t + b * k] * tw[b];
          }
        };
        if (P.closed) {
          for (int t = part; t < k; t += kFinalizeParts) {
            int W = gi - t;
            if (W < 0) W += m;
            add(W, t);
          }
        } else {
          const int wlo = max(0, gi - k + 1), whi = min(gi, m - k);
          for (int W = wlo + part; W <= whi; W += kFinalizeParts) add(W, gi - W);
        }
      }
#pragma unroll
      for (int o = 1; o < kFinalizeParts; o <<= 1) {
        g += __shfl_xor_sync(0xffffffffu, g, o);
        corr += __shfl_xor_sync(0xffffffffu, corr, o);
      }
      if (gi < m && part == 0) {
        if (live) g = -(g + static_cast<double>(corr)) / N;
        if (a.item_G) a.item_G[goff + gi] = g;
        if (a.csr_val && live) atomicAdd(&a.csr_val[a.csr_idx[goff + gi]], g);
      }
    }
  }
}

// ------------------------------------------------- patch-stencil finalize --
// Items of a square-patch mesh, one CTA per item, everything of the item in
// shared memory:
//  1. its nwin x k FP64 moments t_W (one coalesced sweep) and CSR positions;
//  2. the windows some exit chose (a nonzero moment);
//  3. v_W = E_W t_W (FP32 assemblies with A_W^-1 = I + E_W, max |E| small)
//     or A_W^-1 t_W (FP64): one warp per window and lane per row, so a
//     warp's loads of one column of the window's matrix are k consecutive
//     words; a warp keeps two windows' loads in flight;
//  4. G entry gi: -(sum over the windows covering it, in a fixed order) / N,
//     written to item_G and added to its CSR position.
// The matrices (12.7 MB for the 8x8 mesh) stay in L2; each item's moments
// are read from DRAM once.
constexpr int kPatchThreads = 256;

template <typename T, int K>
__device__ __forceinline__ void window_products(const T* __restrict__ Mw0, const T* __restrict__ Mw1,
                                                const T* t0, const T* t1, int k, int r, T& s0, T& s1) {
  // s = sum_b M(r, b) t(b), M column-major; K > 0: k == K at compile time
  const int kk = K > 0 ? K : k;
  s0 = T(0);
  s1 = T(0);
  if (K > 0) {
    T m0[K > 0 ? K : 1], m1[K > 0 ? K : 1];
#pragma unroll
    for (int b = 0; b < (K > 0 ? K : 1); ++b) {
      m0[b] = __ldg(Mw0 + r + b * kk);
      m1[b] = Mw1 ? __ldg(Mw1 + r + b * kk) : T(0);
    }
#pragma unroll
    for (int b = 0; b < (K > 0 ? K : 1); ++b) {
      s0 = fma(m0[b], t0[b], s0);
      if (Mw1) s1 = fma(m1[b], t1[b], s1);
    }
  } else {
    for (int b = 0; b < kk; ++b) {
      s0 = fma(__ldg(Mw0 + r + b * kk), t0[b], s0);
      if (Mw1) s1 = fma(__ldg(Mw1 + r + b * kk), t1[b], s1);
    }
  }
}

template <typename T, int K>
__device__ __forceinline__ void patch_window_pass(const T* __restrict__ M, const T* tw, const unsigned char* vis,
                                                  int nwin, int k, T* v) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int W0 = warp; W0 < nwin; W0 += 2 * nw) {
    const int W1 = W0 + nw;
    const bool a0 = vis[W0] != 0, a1 = W1 < nwin && vis[W1] != 0;
    if (!a0 && !a1) continue;
    const int w0 = a0 ? W0 : W1;  // the first live window of the pair
    const T* M0 = M + static_cast<long long>(w0) * k * k;
    const T* M1 = (a0 && a1) ? M + static_cast<long long>(W1) * k * k : nullptr;
    for (int r = lane; r < k; r += 32) {
      T s0, s1;
      window_products<T, K>(M0, M1, tw + w0 * k, tw + W1 * k, k, r, s0, s1);
      v[w0 * k + r] = s0;
      if (M1) v[W1 * k + r] = s1;
    }
  }
}

template <int PROB, int K>
__global__ void __launch_bounds__(kPatchThreads, 4) finalize_patch_kernel(const FinalizeArgs a) {
  extern __shared__ __align__(16) unsigned char fsm[];
  const int item = blockIdx.x;
  if (item >= a.n_items) return;
  const ItemDev it = a.items[item];
  const bool live = !it.frontera && it.paths > 0;
  // -1/N once per item (the FP64 pipe is the scarce one), broadcast through shared memory
  __shared__ double s_ninv;
  if (threadIdx.x == 0) {
    const double N = static_cast<double>(it.paths);
    finalize_item_head<PROB>(a, item, it, live, N);
    s_ninv = live ? -1.0 / N : 0.0;
  }
  if (it.stencil < 0) return;
  const PatchDev P = a.patches[it.stencil];
  const int m = P.m, k = P.k, nwin = P.nwin, words = nwin * k;
  const long long goff = a.g_off ? a.g_off[item] : 0;
  if (!live) {
    if (a.item_G)
      for (int gi = threadIdx.x; gi < m; gi += blockDim.x) a.item_G[goff + gi] = 0.0;
    return;
  }
  // moments (FP64), results (FP64, or FP32 in the first half), moments in
  // FP32 for the split products (converted once: F2F runs on the FP64 pipe)
  double* tw = reinterpret_cast<double*>(fsm);
  double* v64 = tw + a.fin_words;
  float* v32 = reinterpret_cast<float*>(v64);
  float* t32 = reinterpret_cast<float*>(v64 + a.fin_words);
  int* cidx = reinterpret_cast<int*>(t32 + a.fin_words);
  unsigned char* vis = reinterpret_cast<unsigned char*>(cidx + a.fin_m);
  const double* acc = a.acc + it.acc_off;
  const bool split = a.split_ok && a.patch_e32 && a.patch_emax[it.stencil] < kSplitMaxE;
  for (int i = threadIdx.x; i < words; i += blockDim.x) {
    const double t = acc[i];
    tw[i] = t;
    if (split) t32[i] = f64_to_f32_rz(t);  // (the F2F instruction runs on the FP64 pipe)
  }
  if (a.csr_val)
    for (int j = threadIdx.x; j < m; j += blockDim.x) cidx[j] = a.csr_idx[goff + j];
  __syncthreads();
  for (int W = threadIdx.x; W < nwin; W += blockDim.x) {
    // nonzero test on the bits (+-0 are zero), off the FP64 pipe
    unsigned long long any = 0ull;
    for (int b = 0; b < k; ++b) any |= static_cast<unsigned long long>(__double_as_longlong(tw[W * k + b])) << 1;
    vis[W] = any != 0ull ? 1 : 0;
  }
  __syncthreads();
  if (threadIdx.x == 0 && a.vis_count) {
    int nvis = 0;
    for (int W = 0; W < nwin; ++W) nvis += vis[W];
    if (nvis) atomicAdd(a.vis_count, nvis);
  }
  if (split)
    patch_window_pass<float, K>(a.patch_e32 + P.ainv_off, t32, vis, nwin, k, v32);
  else
    patch_window_pass<double, K>(a.patch_ainv + P.ainv_off, tw, vis, nwin, k, v64);
  __syncthreads();
  // the identity part in FP64, the correction E_W t_W summed in FP32 (at
  // most a few of k window terms of size max |E| |t|, so ~1e-7 relative)
  const double ninv = s_ninv;
  for (int gi = threadIdx.x; gi < m; gi += blockDim.x) {
    double g = 0.0;
    float corr = 0.f;
    auto add = [&](int W, int t) {
      if (!vis[W]) return;
      if (split) {
        g += tw[W * k + t];
        corr += v32[W * k + t];
      } else {
        g += v64[W * k + t];
      }
    };
    if (P.closed) {
      for (int t = 0; t < k; ++t) {
        int W = gi - t;
        if (W < 0) W += m;
        add(W, t);
      }
    } else {
      const int wlo = max(0, gi - k + 1), whi = min(gi, m - k);
      for (int W = wlo; W <= whi; ++W) add(W, gi - W);
    }
    g = (g + f32_to_f64(corr)) * ninv;
    if (a.item_G) a.item_G[goff + gi] = g;
    // a row with several items (a node inside several patches) may meet a
    // column twice: the additions are atomic
    if (a.csr_val) atomicAdd(&a.csr_val[cidx[gi]], g);
  }
}

// Shared memory of finalize_patch_kernel (0: the item-per-CTA generic path).
size_t finalize_patch_smem(const FinalizeArgs& a) {
  if (a.stencil_kind != 2 || a.fin_words <= 0) return 0;
  const size_t b = static_cast<size_t>(a.fin_words) * (2 * sizeof(double) + sizeof(float)) +
                   static_cast<size_t>(a.fin_m) * sizeof(int) + static_cast<size_t>(a.fin_m);
  return b <= 160 * 1024 ? (b + 15) / 16 * 16 : 0;
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

// Items whose G rows the path kernel already added (fused flush): statistics,
// B and result flags only, one thread per item; items that ran no paths
// (Dirichlet nodes, zero path counts) get zero G rows.
template <int PROB>
__global__ void finalize_head_kernel(const FinalizeArgs a) {
  const int item = blockIdx.x * blockDim.x + threadIdx.x;
  if (item >= a.n_items) return;
  const ItemDev it = a.items[item];
  const bool live = !it.frontera && it.paths > 0;
  finalize_item_head<PROB>(a, item, it, live, static_cast<double>(it.paths));
  if (!live && a.item_G && it.stencil >= 0) {
    const int m = a.patches[it.stencil].m;
    const long long goff = a.g_off[item];
    for (int gi = 0; gi < m; ++gi) a.item_G[goff + gi] = 0.0;
  }
}

// ------------------------------------------------ adaptive assembly rounds --
// After a round: its per-item statistics are added to the running sums, its
// per-path variance of phi_VR is reported per item, and the result flags are
// raised as the finalize kernels raise them.
__global__ void round_stats_kernel(const ItemDev* items, int n, const double* stats, double* run_stats,
                                   double* item_var, int* flags) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const ItemDev it = items[i];
  const double* S = stats + static_cast<long long>(i) * kNumStats;
  double* R = run_stats + static_cast<long long>(i) * kNumStats;
  for (int j = 0; j < kNumStats; ++j) R[j] += S[j];
  const bool live = !it.frontera && it.paths > 0;
  double var = 0.0;
  if (live) {
    const double N = static_cast<double>(it.paths), m = S[kStatVR] / N;
    var = fmax(S[kStatVR2] / N - m * m, 0.0);
    if (flags) {
      if (S[kStatCap] > 0.0) atomicOr(&flags[0], 1);
      if (S[kStatPaths] != N) atomicOr(&flags[1], 1);
    }
  }
  if (item_var) item_var[i] = var;
}

// End of an adaptive assembly: item i's G row is its running row sum over
// its total path count N_i (items[i].paths), added to its CSR positions and
// written to item_G if requested; one warp per item.
__global__ void rows_from_sums_kernel(const ItemDev* items, int n, const PatchDev* patches, const long long* g_off,
                                      const double* g_sum, const int* csr_idx, double* csr_val, double* item_G) {
  const int i = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32, lane = threadIdx.x & 31;
  if (i >= n) return;
  const ItemDev it = items[i];
  if (it.stencil < 0) return;
  const int m = patches[it.stencil].m;
  const long long goff = g_off[i];
  const bool live = !it.frontera && it.paths > 0;
  const double ninv = live ? 1.0 / static_cast<double>(it.paths) : 0.0;
  for (int gi = lane; gi < m; gi += 32) {
    const double g = live ? g_sum[goff + gi] * ninv : 0.0;
    if (item_G) item_G[goff + gi] = g;
    if (csr_val && live) atomicAdd(&csr_val[csr_idx[goff + gi]], g);
  }
}

cudaError_t launch_round_stats(const ItemDev* items, int n, const double* stats, double* run_stats, double* item_var,
                               int* flags, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  round_stats_kernel<<<(n + 255) / 256, 256, 0, s>>>(items, n, stats, run_stats, item_var, flags);
  return cudaGetLastError();
}

cudaError_t launch_rows_from_sums(const ItemDev* items, int n, const PatchDev* patches, const long long* g_off,
                                  const double* g_sum, const int* csr_idx, double* csr_val, double* item_G,
                                  cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  rows_from_sums_kernel<<<(n + 7) / 8, 256, 0, s>>>(items, n, patches, g_off, g_sum, csr_idx, csr_val, item_G);
  return cudaGetLastError();
}

// --------------------------------------------------------------- launchers --
template <int PROB, int K>
cudaError_t launch_patch_finalize(const FinalizeArgs& a, size_t smem, cudaStream_t s) {
  cudaError_t e = cudaFuncSetAttribute(finalize_patch_kernel<PROB, K>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(smem));
  if (e != cudaSuccess) return e;
  finalize_patch_kernel<PROB, K><<<a.n_items, kPatchThreads, smem, s>>>(a);
  return cudaGetLastError();
}

template <int PROB>
cudaError_t launch_patch_finalize_k(const FinalizeArgs& a, size_t smem, cudaStream_t s) {
  return a.fin_k == 20 ? launch_patch_finalize<PROB, 20>(a, smem, s) : launch_patch_finalize<PROB, 0>(a, smem, s);
}

cudaError_t launch_finalize(const FinalizeArgs& a, int problem, cudaStream_t s) {
  if (a.n_items <= 0) return cudaSuccess;
  if (a.g_fused) {
    const dim3 grid((a.n_items + 255) / 256), block(256);
    with_problem(problem, [&](auto t) { finalize_head_kernel<decltype(t)::value><<<grid, block, 0, s>>>(a); });
    return cudaGetLastError();
  }
  const size_t psmem = finalize_patch_smem(a);
  if (psmem > 0)
    return with_problem(problem, [&](auto t) { return launch_patch_finalize_k<decltype(t)::value>(a, psmem, s); });
  const dim3 grid(a.n_items), block(kFinalizeThreads);
  with_problem(problem, [&](auto t) { finalize_kernel<decltype(t)::value><<<grid, block, 0, s>>>(a); });
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

// One CTA per patch: E = A_W^-1 - I for every window of the patch in FP32,
// and max |E| over the patch (an exact FP64 max, rounded up to FP32).
__global__ void split_inverse_kernel(const PatchDev* patches, int n_patches, const double* ainv, float* e32,
                                     float* emax) {
  const int p = blockIdx.x;
  if (p >= n_patches) return;
  const PatchDev P = patches[p];
  const int kk = P.k * P.k;
  const long long n = static_cast<long long>(P.nwin) * kk;
  double mx = 0.0;
  for (long long i = threadIdx.x; i < n; i += blockDim.x) {
    const int q = static_cast<int>(i % kk);
    const double e = ainv[P.ainv_off + i] - ((q % P.k) == (q / P.k) ? 1.0 : 0.0);
    e32[P.ainv_off + i] = static_cast<float>(e);
    mx = fmax(mx, fabs(e));
  }
  __shared__ double red[128];
  red[threadIdx.x] = mx;
  __syncthreads();
  for (int o = 64; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + o]);
    __syncthreads();
  }
  if (threadIdx.x == 0) emax[p] = __double2float_ru(red[0]);
}

cudaError_t launch_split_inverse(const PatchDev* patches, int n_patches, const double* ainv, float* e32, float* emax,
                                 cudaStream_t s) {
  if (n_patches <= 0) return cudaSuccess;
  split_inverse_kernel<<<n_patches, 128, 0, s>>>(patches, n_patches, ainv, e32, emax);
  return cudaGetLastError();
}

}  // namespace fk
