// GB300 (sm_103a) path kernel of the Feynman-Kac hot path.
//
// Persistent grid.  Each CTA takes chunks of one item's paths from a global
// queue; every thread runs one path at a time and pulls the next path index
// of the chunk as soon as its path exits (per-lane regeneration: a lane never
// waits for the longest path of its warp).  An exiting lane only pushes its
// exit (X_tau, Y, Z, xi, steps, flags) onto its warp's shared-memory queue and
// starts the next path; once 32 exits are queued the whole warp processes
// them, one exit per lane, so the exit work runs at full SIMD width:
//  - exit value u(X_tau), B and the statistics into per-thread registers
//    (compensated FP32 sums for FP32 stepping, FP64 for FP64 stepping);
//  - the stencil moments Y phi of subdomain exits into the chunk's
//    shared-memory accumulators (FP64 for the arc stencil, whose inverse has
//    condition ~1e10, with lanes over the arc nodes; FP32 chunk partials for
//    the Gaussian k-nearest stencil, one exit and its window per lane).
// At the end of a chunk the thread sums are block-reduced and the moments
// flushed into FP64 per-item accumulators.  On the FP32 path no FP64
// instruction runs inside the step loop.
// Replaces Simulacion_OMP + Reduce_Analytic + Interfaz::Update_G
// (Solvers/FeynmanKacSolver.cpp:137-292, Mesh/Interfaz.cpp:219-264).
#include <cfloat>
#include <type_traits>

#include "fk_device.cuh"
#include "fk_internal.h"

namespace fk {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kMaxWarps = 32;
constexpr int kNumAcc = 8;   // floating-point sums per thread

struct AccD {
  double s = 0.0;
  __device__ __forceinline__ void add(double v) { s += v; }
  __device__ __forceinline__ double get() const { return s; }
};
// Compensated (Kahan) FP32 sum: FP64-grade thread sums without FP64 work.
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

template <typename R, int ST>
struct SAccType {
  using type = typename std::conditional<std::is_same<R, double>::value || ST == 1, double, float>::type;
};

// Per-warp queue of exits awaiting processing (exit point, Y, Z, xi, and
// steps | domain-exit << 30 | capped << 31); at most 31 + 32 entries.
constexpr int kMaxBlockWarps = 8;
template <typename R>
struct ExitQueue {
  R x[64], y[64], Y[64], Z[64], xi[64];
  unsigned kf[64];
};

// Per-chunk copy of the exit patch in shared memory (stepping precision).
template <typename R>
struct PatchSh {
  int m, k, closed;
  int side_first[4], side_count[4], side_axis[4];
  R side_fixed[4], side_start[4], side_inv_step[4];
  R e2;
};

// Window (first chain index) of the k nearest patch-boundary nodes to an exit
// point on the patch boundary.  The k nearest nodes of a point of a convex
// boundary chain form a contiguous run of the chain: start from the run
// centred on the nearest node of the exit side, slide while an outside
// neighbour is closer than the opposite end of the run.
template <typename R>
__device__ __forceinline__ int knn_window(const PatchSh<R>& P, const R* __restrict__ nx, const R* __restrict__ ny,
                                          R ex, R ey) {
  int best_s = -1;
  R best = R(FLT_MAX);
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    if (P.side_count[s] > 0) {
      const R dist = fabs((P.side_axis[s] == 0 ? ey : ex) - P.side_fixed[s]);
      if (dist < best) { best = dist; best_s = s; }
    }
  }
  const int m = P.m, k = P.k;
  int nearest = 0;
  if (best_s >= 0) {
    const R coord = P.side_axis[best_s] == 0 ? ex : ey;
    int j = static_cast<int>(rint((coord - P.side_start[best_s]) * P.side_inv_step[best_s]));
    j = max(0, min(P.side_count[best_s] - 1, j));
    nearest = P.side_first[best_s] + j;
  }
  auto d2 = [&](int idx) -> R {
    if (idx >= m) idx -= m;
    if (idx < 0) idx += m;
    const R dx = ex - nx[idx], dy = ey - ny[idx];
    return dx * dx + dy * dy;
  };
  int L = nearest - k / 2;
  if (P.closed) {
    if (L < 0) L += m;
    for (int it = 0; it < m && d2(L - 1) < d2(L + k - 1); ++it) { --L; if (L < 0) L += m; }
    for (int it = 0; it < m && d2(L + k) < d2(L); ++it) { ++L; if (L >= m) L -= m; }
  } else {
    L = max(0, min(m - k, L));
    while (L > 0 && d2(L - 1) < d2(L + k - 1)) --L;
    while (L < m - k && d2(L + k) < d2(L)) ++L;
  }
  return L;
}

template <typename R, int PROB, int ST>
__global__ void __launch_bounds__(256, 3) paths_kernel(const LaunchArgs a) {
  using SAcc = typename SAccType<R, ST>::type;
  using Acc = typename std::conditional<std::is_same<R, double>::value, AccD, AccK>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SAcc* sacc = reinterpret_cast<SAcc*>(smem_raw);
  // after the accumulators: patch nodes (x[], y[]) or arc angles
  R* snx = reinterpret_cast<R*>(smem_raw + static_cast<size_t>(a.acc_words) * sizeof(SAcc));
  R* sny = snx + a.smem_nodes;
  double* sth = reinterpret_cast<double*>(smem_raw + static_cast<size_t>(a.acc_words) * sizeof(SAcc));
  __shared__ int s_chunk;
  __shared__ unsigned s_next;
  __shared__ double s_red[kNumAcc + 3][kMaxWarps];
  __shared__ PatchSh<R> sp;
  __shared__ ArcDev sarc;
  __shared__ ExitQueue<R> sq[kMaxBlockWarps];

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const bool cv = a.cv != 0;         // any control term
  const bool cv_exact = a.cv == 1;   // F from the problem functor
  const bool cv_table = a.cv == 2;   // F from the learned gradient table

  for (;;) {
    if (threadIdx.x == 0) s_chunk = atomicAdd(a.queue, 1);
    __syncthreads();
    const int c = s_chunk;
    if (c >= a.n_chunks) break;
    const ChunkDev ch = a.chunks[c];
    const ItemDev& itg = a.items[ch.item];
    for (int i = threadIdx.x; i < a.acc_words; i += blockDim.x) sacc[i] = SAcc(0);
    if (ST == 2) {
      const PatchDev& P = a.patches[itg.stencil];
      const double* nd = a.patch_nodes + P.node_off;
      for (int i = threadIdx.x; i < P.m; i += blockDim.x) { snx[i] = R(nd[2 * i]); sny[i] = R(nd[2 * i + 1]); }
      if (threadIdx.x == 0) {
        sp.m = P.m; sp.k = P.k; sp.closed = P.closed; sp.e2 = R(P.eps2);
        for (int s = 0; s < 4; ++s) {
          sp.side_first[s] = P.side_first[s]; sp.side_count[s] = P.side_count[s]; sp.side_axis[s] = P.side_axis[s];
          sp.side_fixed[s] = R(P.side_fixed[s]); sp.side_start[s] = R(P.side_start[s]);
          sp.side_inv_step[s] = R(1.0 / P.side_step[s]);
        }
      }
    }
    if (ST == 1) {
      const ArcDev& A = a.arcs[itg.stencil];
      for (int i = threadIdx.x; i < A.n; i += blockDim.x) sth[i] = a.arc_theta[A.theta_off + i];
      if (threadIdx.x == 0) sarc = A;
    }
    if (threadIdx.x == 0) s_next = ch.p0 + blockDim.x;
    __syncthreads();

    // the item's BVP (independent problems of one functor share a launch)
    const BvpDev& bvp = a.bvp[itg.bvp];
    const R d0 = R(bvp.dom[0]), d1 = R(bvp.dom[1]), d2 = R(bvp.dom[2]), d3 = R(bvp.dom[3]);
    const R h = R(itg.h), sqrth = R(itg.sqrth), x0 = R(itg.x), y0 = R(itg.y);
    const R s0 = R(itg.sub[0]), s1 = R(itg.sub[1]), s2 = R(itg.sub[2]), s3 = R(itg.sub[3]);
    const bool has_sub = (ST != 0) || itg.sub_shape >= 0;
    const bool sub_circle = (ST == 1) || (ST == 0 && itg.sub_shape == 1);
    const R st0 = Problem<PROB>::template state<R>(bvp, x0, y0);  // sigma state at the start point
    const uint32_t item = static_cast<uint32_t>(ch.item);
    // learned control variate: grad u_hat table of this item's region
    const float2* ctab = nullptr;
    R cx0 = R(0), cy0 = R(0), csx = R(0), csy = R(0);
    const int G = a.cv_grid;
    if (cv_table) {
      const int r = itg.cv_region;
      const double* rc = a.cv_rect + 4 * r;
      ctab = a.cv_tab + static_cast<long long>(r) * G * G;
      cx0 = R(rc[0]);
      cy0 = R(rc[1]);
      csx = R((G - 1) / (rc[2] - rc[0]));
      csy = R((G - 1) / (rc[3] - rc[1]));
    }

    Acc acc[kNumAcc];
    unsigned n_steps = 0, n_dom = 0, n_cap = 0;
    R x = x0, y = y0, Y = R(1), Z = R(0), xi = R(0), st = st0;
    int k = 0;
    uint32_t w2 = 0, w3 = 0;
    unsigned p = ch.p0 + threadIdx.x;
    bool active = p < ch.p1;
    ExitQueue<R>& q = sq[warp];
    int qn = 0;  // queued exits of this warp (warp-uniform)

    // Processes the top `cnt` (<= 32) queued exits, one per lane: exit value
    // and statistics (Reduce_Analytic, FeynmanKacSolver.cpp:198-292) and the
    // stencil moments of subdomain exits.
    auto process = [&](int cnt) {
      const int base = qn - cnt;
      const bool mine = lane < cnt;
      R ex = R(0), ey = R(0), Yv = R(0);
      bool sub_exit = false;
      if (mine) {
        const int e = base + lane;
        ex = q.x[e]; ey = q.y[e]; Yv = q.Y[e];
        const R Zv = q.Z[e], xv = q.xi[e];
        const unsigned kf = q.kf[e];
        const bool dw = (kf >> 30) & 1u, cp = (kf >> 31) & 1u;
        sub_exit = (ST != 0) && !dw;
        const R g = Problem<PROB>::u(bvp, ex, ey);  // g = u for every registered problem
        const R score = Zv + Yv * g;
        const R vr = score + xv;
        acc[0].add(score);
        acc[1].add(score * score);
        acc[2].add(xv + xv * xv);
        acc[3].add(vr);
        acc[4].add(vr * vr);
        acc[5].add(xv * score);
        acc[6].add(sub_exit ? Zv + xv : vr);
        acc[7].add(xv * xv);
        n_steps += kf & 0x3fffffffu;
        n_dom += dw ? 1u : 0u;
        n_cap += cp ? 1u : 0u;
      }
      if (ST == 2) {
        if (sub_exit) {
          // Gaussian k-nearest moments t_W[j] += Y phi_j, one exit per lane
          const int L = knn_window<R>(sp, snx, sny, ex, ey);
          const int kk = sp.k, m = sp.m;
          const R e2 = sp.e2;
          for (int j = 0; j < kk; ++j) {
            int idx = L + j;
            if (idx >= m) idx -= m;
            const R dx = ex - snx[idx], dy = ey - sny[idx];
            atomicAdd(&sacc[L * kk + j], static_cast<SAcc>(Yv * fexp(-e2 * (dx * dx + dy * dy))));
          }
        }
      } else if (ST == 1) {
        // Interfaz::Update_G moments s_i += Y phi_i(theta), FP64, lanes over i
        double th = 0.0;
        if (sub_exit)
          th = arc_theta(sarc.interior, static_cast<double>(ex) - sarc.cx, static_cast<double>(ey) - sarc.cy);
        unsigned em = __ballot_sync(kFull, sub_exit);
        const int n = sarc.n;
        const double c2 = sarc.c2;
        while (em) {
          const int src = __ffs(em) - 1;
          em &= em - 1;
          const double tb = __shfl_sync(kFull, th, src);
          const double Yb = static_cast<double>(__shfl_sync(kFull, Yv, src));
          for (int i = lane; i < n; i += 32) {
            const double d = tb - sth[i];
            atomicAdd(reinterpret_cast<double*>(&sacc[i]), Yb / sqrt(d * d + c2));
          }
        }
      }
      qn = base;
    };

    while (__any_sync(kFull, active)) {
      bool exits = false, dom_wins = true, capped = false;
      R ex = R(0), ey = R(0);
      if (active) {
        // ---- one Euler-Maruyama step (Paso_Absorbente, FeynmanKacSolver.cpp:7-18)
        StepCoef<R> co;
        Problem<PROB>::step(bvp, x, y, st, cv_exact, co);
        if (cv_table) {
          // F = -sigma^T grad u_hat, bilinear in the region's table
          R u = (x - cx0) * csx, v = (y - cy0) * csy;
          u = fmin(fmax(u, R(0)), R(G - 1) - R(1e-3));
          v = fmin(fmax(v, R(0)), R(G - 1) - R(1e-3));
          const int i = static_cast<int>(u), j = static_cast<int>(v);
          const R fu = u - R(i), fv = v - R(j);
          const float2* T = ctab + j * G + i;
          const float2 t00 = __ldg(T), t10 = __ldg(T + 1), t01 = __ldg(T + G), t11 = __ldg(T + G + 1);
          const R gx = (R(1) - fv) * ((R(1) - fu) * R(t00.x) + fu * R(t10.x)) + fv * ((R(1) - fu) * R(t01.x) + fu * R(t11.x));
          const R gy = (R(1) - fv) * ((R(1) - fu) * R(t00.y) + fu * R(t10.y)) + fv * ((R(1) - fu) * R(t01.y) + fu * R(t11.y));
          co.Fx = -co.s * gx;
          co.Fy = -co.s * gy;
        }
        uint32_t wa, wb;
        if ((k & 1) == 0) {
          const uint4 r = philox10(make_uint4(static_cast<uint32_t>(k >> 1), p, item, a.stream), a.key0, a.key1);
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
        Bnd<R> w = (PROB == 3) ? circle_dist<R>(x, y, d0, d1, d2) : rect_dist<R>(x, y, d0, d1, d2, d3);
        if (has_sub) {
          const Bnd<R> sb = sub_circle ? circle_dist<R>(x, y, s0, s1, s2) : rect_dist<R>(x, y, s0, s1, s2, s3);
          if (!(w.d >= sb.d)) { w = sb; dom_wins = false; }
        }
        // sigma at the new point (kept for the next step) or at the projection
        R sg;
        if (w.d < R(0)) {
          st = Problem<PROB>::template state<R>(bvp, x, y);
          sg = Problem<PROB>::template sigma_of<R>(st);
        } else {
          sg = Problem<PROB>::template sigma_of<R>(Problem<PROB>::template state<R>(bvp, w.ex, w.ey));
        }
        const R nsx = w.nx * sg, nsy = w.ny * sg;
        const R thr = R(kGobet) * sqrt(nsx * nsx + nsy * nsy) * sqrth;
        capped = k >= a.max_steps;
        exits = !(w.d < thr) || capped;
        ex = w.ex;
        ey = w.ey;
      }
      // ---- queue the exits; the exiting lanes start their next path at once
      const unsigned em = __ballot_sync(kFull, exits);
      if (exits) {
        const int e = qn + __popc(em & ((1u << lane) - 1u));
        q.x[e] = ex; q.y[e] = ey; q.Y[e] = Y; q.Z[e] = Z; q.xi[e] = xi;
        q.kf[e] = static_cast<unsigned>(k) | (dom_wins ? 1u << 30 : 0u) | (capped ? 1u << 31 : 0u);
        p = atomicAdd(&s_next, 1u);
        active = p < ch.p1;
        x = x0; y = y0; Y = R(1); Z = R(0); xi = R(0); k = 0; st = st0;
      }
      qn += __popc(em);
      __syncwarp();
      if (qn >= 32) {
        process(32);
        __syncwarp();
      }
    }
    if (qn > 0) process(qn);
    __syncthreads();
    // ---- chunk flush: block reduction of the thread sums, FP64 atomics per item
    double v[kNumAcc + 3];
#pragma unroll
    for (int j = 0; j < kNumAcc; ++j) v[j] = acc[j].get();
    v[kNumAcc] = static_cast<double>(n_steps);
    v[kNumAcc + 1] = static_cast<double>(n_dom);
    v[kNumAcc + 2] = static_cast<double>(n_cap);
#pragma unroll
    for (int j = 0; j < kNumAcc + 3; ++j) {
      double t = v[j];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(kFull, t, o);
      if (lane == 0) s_red[j][warp] = t;
    }
    __syncthreads();
    if (threadIdx.x < kNumAcc + 3) {
      double t = 0.0;
      for (int w = 0; w < nwarps; ++w) t += s_red[threadIdx.x][w];
      // slot layout of kStat*: score, score^2, xi+xi^2, vr, vr^2, xi score, steps, B, dom, cap, xi^2
      const int slot_of[kNumAcc + 3] = {kStatScore, kStatScore2, kStatXiAlias, kStatVR, kStatVR2, kStatXiScore,
                                        kStatB, kStatXi2, kStatSteps, kStatDom, kStatCap};
      if (t != 0.0) atomicAdd(&a.stats[static_cast<long long>(ch.item) * kNumStats + slot_of[threadIdx.x]], t);
    }
    if (ST != 0) {
      double* gacc = a.acc + itg.acc_off;
      for (int i = threadIdx.x; i < a.acc_words; i += blockDim.x) {
        const double t = static_cast<double>(sacc[i]);
        if (t != 0.0) atomicAdd(&gacc[i], t);
      }
    }
    __syncthreads();
  }
}

template <typename R, int PROB>
const void* paths_fn(int st) {
  switch (st) {
    case 1: return reinterpret_cast<const void*>(&paths_kernel<R, PROB, 1>);
    case 2: return reinterpret_cast<const void*>(&paths_kernel<R, PROB, 2>);
    default: return reinterpret_cast<const void*>(&paths_kernel<R, PROB, 0>);
  }
}
template <typename R>
const void* paths_fn_r(int problem, int st) {
  switch (problem) {
    case 1: return paths_fn<R, 1>(st);
    case 2: return paths_fn<R, 2>(st);
    case 3: return paths_fn<R, 3>(st);
    default: return paths_fn<R, 0>(st);
  }
}
const void* select_paths(int problem, int precision, int st) {
  return precision == 1 ? paths_fn_r<float>(problem, st) : paths_fn_r<double>(problem, st);
}

}  // namespace

size_t paths_smem_bytes(int precision, int stencil_kind, int acc_words, int smem_nodes) {
  const size_t acc = static_cast<size_t>(acc_words) * ((precision == 0 || stencil_kind == 1) ? 8 : 4);
  if (stencil_kind == 2) return acc + 2ull * smem_nodes * (precision == 0 ? 8 : 4);
  if (stencil_kind == 1) return acc + static_cast<size_t>(smem_nodes) * 8;
  return acc;
}

cudaError_t launch_paths(const LaunchArgs& a, int problem, int precision, int grid, int block, size_t smem,
                         cudaStream_t s) {
  const void* fn = select_paths(problem, precision, a.stencil_kind);
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  if (e != cudaSuccess) return e;
  void* args[] = {const_cast<LaunchArgs*>(&a)};
  return cudaLaunchKernel(fn, dim3(grid), dim3(block), args, smem, s);
}

int paths_kernel_occupancy(int problem, int precision, int stencil_kind, int, int block, size_t smem) {
  const void* fn = select_paths(problem, precision, stencil_kind);
  cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, block, smem) != cudaSuccess) return 1;
  return n > 0 ? n : 1;
}

}  // namespace fk
