// GB300 (sm_103a) path kernel of the Feynman-Kac hot path (included by
// fk_paths.cu and fk_paths_plain.cu, which instantiate it).
//
// Persistent grid.  Each CTA keeps a ring of chunk slots in shared memory (a
// chunk is a range of one item's paths; its slot holds the chunk's stencil
// accumulators and stencil nodes).  The warps of a CTA walk the CTA's
// sequence of chunks in order.  Inside a chunk every lane runs one path at a
// time and takes the next path index of the chunk as soon as its path exits
// (per-lane regeneration).  Once a chunk's paths are all taken its warps go
// on to the next slot while the chunk's last paths finish: there is no
// CTA-wide barrier between chunks, so the tail of one chunk overlaps the
// next.  The last warp to leave a chunk flushes the chunk's stencil moments
// into the item's FP64 accumulators and refills the slot from the global
// chunk queue.  Items of few paths run in warp mode instead: each warp takes
// its own chunks and adds the moments to global memory (see paths_kernel).
//
// An exiting lane only pushes its exit (X_tau, Y, Z, xi, steps, flags) onto
// its warp's shared-memory queue and starts the next path; once 32 exits are
// queued the whole warp processes them, one exit per lane, so the exit work
// runs at full SIMD width:
//  - exit value u(X_tau), B and the statistics into per-thread registers
//    (compensated FP32 sums for FP32 stepping, FP64 for FP64 stepping);
//  - the stencil moments Y phi of subdomain exits into the chunk's
//    shared-memory accumulators (FP64 for the arc stencil, whose inverse has
//    condition ~1e10, with lanes over the arc nodes; FP32 chunk partials for
//    the Gaussian k-nearest stencil, one exit and its window per lane).
// A warp leaving a chunk reduces its thread sums (compensated FP32 shuffles
// on the FP32 path) and adds them to the item's FP64 sums.  On the FP32 path
// no FP64 arithmetic runs inside the step loop.
// Replaces Simulacion_OMP + Reduce_Analytic + Interfaz::Update_G
// (Solvers/FeynmanKacSolver.cpp:137-292, Mesh/Interfaz.cpp:219-264).
#pragma once
#include <cfloat>
#include <type_traits>

#include "fk_device.cuh"
#include "fk_internal.h"

namespace fk {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kNumAcc = 8;   // floating-point sums per thread

struct AccD {
  double s = 0.0;
  __device__ __forceinline__ void add(double v) { s += v; }
};
// Compensated (Kahan) FP32 sum: FP64-grade thread sums without FP64 work.
// The sum is s - c.
struct AccK {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float v) {
    const float y = v - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
  }
};

// Warp total of a thread sum; lane 0 holds the result.
__device__ __forceinline__ double warp_reduce(const AccD& a, int) {
  double t = a.s;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(kFull, t, o);
  return t;
}
// Compensated FP32 butterfly: the (sum, correction) pairs are combined with
// Knuth's TwoSum, so the warp total keeps the accuracy of the compensated
// thread sums; only lane 0 converts the pair to FP64.
__device__ __forceinline__ double warp_reduce(const AccK& a, int lane) {
  float s = a.s, c = -a.c;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float s2 = __shfl_xor_sync(kFull, s, o), c2 = __shfl_xor_sync(kFull, c, o);
    const float t = s + s2;
    const float bp = t - s;
    const float e = (s - (t - bp)) + (s2 - bp);
    s = t;
    c = c + c2 + e;
  }
  return lane == 0 ? static_cast<double>(s) + static_cast<double>(c) : 0.0;
}

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
  int m, k, closed, walk;
  int side_first[4], side_count[4], side_axis[4];
  R side_fixed[4], side_start[4], side_inv_step[4];
  R e2;
  const unsigned short* ktab;  // the patch's window table
  int knn_base[4], knn_n[4];
  R knn_u0[4];
};

// A chunk slot.  `ready` is written last, after the slot's contents.
template <typename R>
struct SlotSh {
  int ready;        // position in the CTA's chunk sequence that the slot holds
  int chunk;        // chunk index; -1: the chunk queue was exhausted
  int warps_left;   // warps that have not yet left the chunk
  unsigned next;    // next chunk-local path index
  PatchSh<R> sp;
  ArcDev sarc;
};

__device__ __forceinline__ int ld_volatile(const int* p) { return *reinterpret_cast<const volatile int*>(p); }
__device__ __forceinline__ void st_volatile(int* p, int v) { *reinterpret_cast<volatile int*>(p) = v; }
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Waits until a slot holds sequence position `seq` (lane 0 polls, with
// back-off).  The wait is for another warp of this CTA to finish the paths it
// is running, which the step cap bounds; `limit_ns` bounds it again.  Returns
// false if the wait gave up.
__device__ bool wait_slot(const int* ready, int seq, unsigned long long limit_ns, int lane) {
  int ok = 1;
  if (lane == 0 && ld_volatile(ready) != seq) {
    const unsigned long long t0 = global_ns();
    while (ld_volatile(ready) != seq) {
      if (global_ns() - t0 > limit_ns) {
        ok = 0;
        break;
      }
      __nanosleep(64);
    }
  }
  ok = __shfl_sync(kFull, ok, 0);
  __threadfence_block();
  return ok != 0;
}

// One warp copies an item's stencil into shared memory: patch node
// coordinates (stepping precision) and side descriptors, or arc angles.
template <typename R, int ST>
__device__ void stage_stencil(const LaunchArgs& a, SlotSh<R>& sl, unsigned char* nodes_mem, int stencil, int lane) {
  if (ST == 2) {
    R* snx = reinterpret_cast<R*>(nodes_mem);
    R* sny = snx + a.smem_nodes;
    const PatchDev& P = a.patches[stencil];
    const double* nd = a.patch_nodes + P.node_off;
    for (int i = lane; i < P.m; i += 32) {
      snx[i] = R(nd[2 * i]);
      sny[i] = R(nd[2 * i + 1]);
    }
    if (lane < 4) {
      const int s = lane;
      sl.sp.side_first[s] = P.side_first[s];
      sl.sp.side_count[s] = P.side_count[s];
      sl.sp.side_axis[s] = P.side_axis[s];
      sl.sp.side_fixed[s] = R(P.side_fixed[s]);
      sl.sp.side_start[s] = R(P.side_start[s]);
      sl.sp.side_inv_step[s] = R(1.0 / P.side_step[s]);
      sl.sp.knn_base[s] = P.knn_base[s];
      sl.sp.knn_n[s] = P.knn_n[s];
      sl.sp.knn_u0[s] = R(P.knn_u0[s]);
    }
    if (lane == 0) {
      sl.sp.m = P.m;
      sl.sp.k = P.k;
      sl.sp.closed = P.closed;
      sl.sp.walk = std::is_same<R, float>::value ? P.walk32 : P.walk;
      sl.sp.e2 = R(P.eps2);
      sl.sp.ktab = a.knn_tab + P.knn_off;
    }
  }
  if (ST == 1) {
    double* sth = reinterpret_cast<double*>(nodes_mem);
    const ArcDev& A = a.arcs[stencil];
    for (int i = lane; i < A.n; i += 32) sth[i] = a.arc_theta[A.theta_off + i];
    if (lane == 0) sl.sarc = A;
  }
}

// One warp claims the next chunk of the global queue for a slot, clears the
// slot's accumulators, stages the chunk's stencil and publishes the slot as
// sequence position `seq`.
template <typename R, int ST>
__device__ void fill_slot(const LaunchArgs& a, int n_chunks, SlotSh<R>& sl, unsigned char* mem, size_t acc_bytes,
                          int seq, int nwarps, int lane) {
  int c = 0;
  if (lane == 0) c = atomicAdd(a.queue, 1);
  c = __shfl_sync(kFull, c, 0);
  if (c < n_chunks) {
    const ChunkDev ch = a.chunks[c];
    const ItemDev& itg = a.items[ch.item];
    uint4* z = reinterpret_cast<uint4*>(mem);
    for (int i = lane; i < static_cast<int>(acc_bytes / 16); i += 32) z[i] = make_uint4(0u, 0u, 0u, 0u);
    stage_stencil<R, ST>(a, sl, mem + acc_bytes, itg.stencil, lane);
    if (lane == 0) {
      sl.chunk = c;
      sl.next = 0u;
      sl.warps_left = nwarps;
    }
  } else if (lane == 0) {
    sl.chunk = -1;
  }
  __syncwarp();
  __threadfence_block();
  if (lane == 0) st_volatile(&sl.ready, seq);
  __syncwarp();
}

// Window (first chain index) of the k nearest patch-boundary nodes to an exit
// point on the patch boundary.  The k nearest nodes of a point of a convex
// boundary chain form a contiguous run of the chain: start from the run
// centred on the nearest node of the exit side, slide while an outside
// neighbour is closer than the opposite end of the run.
template <typename R>
__device__ __forceinline__ int knn_window(const PatchSh<R>& P, const R* __restrict__ nx, const R* __restrict__ ny,
                                          R ex, R ey, int& nearest_out) {
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
  auto d2 = [&](int idx) -> R {
    if (idx >= m) idx -= m;
    if (idx < 0) idx += m;
    const R dx = ex - nx[idx], dy = ey - ny[idx];
    return dx * dx + dy * dy;
  };
  int nearest = 0;
  if (best_s >= 0) {
    const R coord = P.side_axis[best_s] == 0 ? ex : ey;
    const R u = (coord - P.side_start[best_s]) * P.side_inv_step[best_s];
    int j = static_cast<int>(rint(u));
    j = max(0, min(P.side_count[best_s] - 1, j));
    nearest = P.side_first[best_s] + j;
    // the window table: L0 or L0 + 1, by the sliding search's own comparison
    const int nb = P.knn_n[best_s];
    if (nb > 0) {
      int b = static_cast<int>(floor((u - P.knn_u0[best_s]) * R(kKnnBins)));
      b = max(0, min(nb - 1, b));
      const unsigned short e = __ldg(P.ktab + P.knn_base[best_s] + b);
      if (!(e & kKnnFull)) {
        int L = e;
        const int up = L + k;  // the node that enters the window when it moves up
        if (P.closed || up < m) {
          if (d2(up) < d2(L)) L = (L + 1 == m) ? 0 : L + 1;
        }
        nearest_out = nearest;
        return L;
      }
    }
  }
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
  nearest_out = nearest;
  return L;
}

// The last warp out of a chunk (slot mode, patch stencil) turns the chunk's
// window moments t_W, held in the slot's shared memory, into the chunk's
// part of the item's G row, as finalize_patch_kernel does for a whole item:
//   row[(W + r) mod m] = sum over the windows W covering the node of
//                        (A_W^-1 t_W)[r],
// with A_W^-1 t_W = t_W + E_W t_W in FP32 for FP32 moments (E_W = A_W^-1 - I,
// when patch_e32 is set) and the FP64 inverse otherwise, one visited window
// at a time (lane
// r < k takes row r: one column of the matrix is k consecutive words),
// summed in FP64 in `gbuf` (the slot's stencil node area, free once every
// warp has left the chunk).  Then either
//   fuse_g == 1 (the chunk is the whole item): G = -row / N is added to the
//     item's CSR positions (SistemaLineal::Actualiza_GB,
//     Mesh/SistemaLineal.cpp:68-88) and written to item_G if requested;
//   fuse_g == 2 (rounds of an adaptive assembly): -row is added to the
//     item's running row sum g_sum, normalised once by the total path count
//     at the end of the assembly.
__device__ __forceinline__ double widen(float v) { return f32_to_f64(v); }  // (integer pipes)
__device__ __forceinline__ double widen(double v) { return v; }

// Fast path of fused_patch_row for FP32 moments, k = 20 and E_W in FP32:
// each lane takes whole visited windows, W = lane, lane + 32, ...: the
// window's 20 moments into registers, E_W's 100 float4 words loaded with all
// loads in flight (one L2 round trip per window instead of one per row), and
// v_W = t_W + E_W t_W written back over the moments; then lane gi sums the
// (at most k) window terms of node gi in FP64 in a fixed order, with no
// atomics.  Returns false where it does not apply.
constexpr int kFastK = 20;
template <typename R>
__device__ bool fused_patch_row_fast(const LaunchArgs& a, const ItemDev& itg, int item, const PatchSh<R>& sp,
                                     float* sacc, int lane) {
  const int m = sp.m, k = sp.k, nwin = sp.closed ? m : m - k + 1;
  if (k != kFastK || !a.patch_e32) return false;
  const float* E = a.patch_e32 + a.patches[itg.stencil].ainv_off;
  unsigned nvis = 0;
  for (int W = lane; W < nwin; W += 32) {
    float* t = sacc + W * kFastK;
    float tv[kFastK];
    bool vis = false;
#pragma unroll
    for (int b = 0; b < kFastK; ++b) {
      tv[b] = t[b];
      vis |= tv[b] != 0.f;
    }
    if (!vis) continue;
    ++nvis;
    const float4* Ew = reinterpret_cast<const float4*>(E + static_cast<long long>(W) * kFastK * kFastK);
    float v[kFastK];
#pragma unroll
    for (int r = 0; r < kFastK; ++r) v[r] = 0.f;
#pragma unroll
    for (int b = 0; b < kFastK; ++b) {  // column b of E_W: rows 0..19 in 5 float4 words
#pragma unroll
      for (int q = 0; q < kFastK / 4; ++q) {
        const float4 e = __ldg(Ew + b * (kFastK / 4) + q);
        v[4 * q] = fmaf(e.x, tv[b], v[4 * q]);
        v[4 * q + 1] = fmaf(e.y, tv[b], v[4 * q + 1]);
        v[4 * q + 2] = fmaf(e.z, tv[b], v[4 * q + 2]);
        v[4 * q + 3] = fmaf(e.w, tv[b], v[4 * q + 3]);
      }
    }
#pragma unroll
    for (int r = 0; r < kFastK; ++r) t[r] = tv[r] + v[r];
  }
  nvis = __reduce_add_sync(kFull, nvis);
  if (lane == 0 && a.vis_count && nvis) atomicAdd(a.vis_count, static_cast<int>(nvis));
  __syncwarp();
  const long long goff = a.g_off[item];
  double ninv = 0.0;
  if (a.fuse_g == 1) {
    if (lane == 0) ninv = -1.0 / static_cast<double>(itg.paths);
    ninv = __shfl_sync(kFull, ninv, 0);
  }
  for (int gi = lane; gi < m; gi += 32) {
    double g = 0.0;
    if (sp.closed) {
      for (int tt = 0; tt < kFastK; ++tt) {
        int W = gi - tt;
        if (W < 0) W += m;
        g += f32_to_f64(sacc[W * kFastK + tt]);
      }
    } else {
      const int wlo = max(0, gi - kFastK + 1), whi = min(gi, m - kFastK);
      for (int W = wlo; W <= whi; ++W) g += f32_to_f64(sacc[W * kFastK + gi - W]);
    }
    if (a.fuse_g == 2) {
      if (g != 0.0) atomicAdd(&a.g_sum[goff + gi], -g);
    } else {
      g *= ninv;
      if (a.item_G) a.item_G[goff + gi] = g;
      // a row of several items (a node inside several patches) may meet a column twice
      atomicAdd(&a.csr_val[a.csr_idx[goff + gi]], g);
    }
  }
  __syncwarp();
  return true;
}

// Warp mode (FP32 stepping, k = 20, E_W in FP32, the chunk is the whole
// item): the warp that ran the item forms its G row from the item's FP64
// moments in global memory, which only this warp has added to.  `wvis`
// marks the windows its exits chose (a bit per window, in the warp's shared
// memory).  Lanes take visited windows: t_W is read (from L2: another item's
// flush may have left a stale L1 copy of a shared cache line), v_W = t_W +
// E_W t_W (the correction in FP32, as in the finalize kernel's split
// products) is written over it; then lane gi sums node gi's window terms in
// FP64 in a fixed order and adds -row/N to the item's CSR positions; last the
// visited windows are zeroed, so that the accumulators are all zero again
// when the launch ends (the next warp-mode launch needs no memset).
template <typename R>
__device__ void fused_patch_row_wm(const LaunchArgs& a, const ItemDev& itg, int item, const PatchSh<R>& sp,
                                   double* gacc, const unsigned* wvis, int lane) {
  const int m = sp.m, nwin = sp.closed ? m : m - kFastK + 1;
  const float* E = a.patch_e32 + a.patches[itg.stencil].ainv_off;
  auto visited = [&](int W) { return ((wvis[W >> 5] >> (W & 31)) & 1u) != 0u; };
  __threadfence_block();
  __syncwarp();
  if (lane == 0 && a.vis_count) {
    int nvis = 0;
    for (int i = 0; i < (nwin + 31) / 32; ++i) nvis += __popc(wvis[i]);
    if (nvis) atomicAdd(a.vis_count, nvis);
  }
  for (int W = lane; W < nwin; W += 32) {
    if (!visited(W)) continue;
    double* t = gacc + static_cast<long long>(W) * kFastK;
    float tf[kFastK], v[kFastK];
#pragma unroll
    for (int b = 0; b < kFastK; ++b) {
      tf[b] = f64_to_f32_rz(__ldcg(t + b));
      v[b] = 0.f;
    }
    const float4* Ew = reinterpret_cast<const float4*>(E + static_cast<long long>(W) * kFastK * kFastK);
#pragma unroll
    for (int b = 0; b < kFastK; ++b) {
#pragma unroll
      for (int q = 0; q < kFastK / 4; ++q) {
        const float4 e = __ldg(Ew + b * (kFastK / 4) + q);
        v[4 * q] = fmaf(e.x, tf[b], v[4 * q]);
        v[4 * q + 1] = fmaf(e.y, tf[b], v[4 * q + 1]);
        v[4 * q + 2] = fmaf(e.z, tf[b], v[4 * q + 2]);
        v[4 * q + 3] = fmaf(e.w, tf[b], v[4 * q + 3]);
      }
    }
#pragma unroll
    for (int r = 0; r < kFastK; ++r) t[r] = __ldcg(t + r) + f32_to_f64(v[r]);
  }
  __threadfence_block();
  __syncwarp();
  const long long goff = a.g_off[item];
  double ninv = 0.0;
  if (lane == 0) ninv = -1.0 / static_cast<double>(itg.paths);
  ninv = __shfl_sync(kFull, ninv, 0);
  for (int gi = lane; gi < m; gi += 32) {
    double g = 0.0;
    if (sp.closed) {
      for (int tt = 0; tt < kFastK; ++tt) {
        int W = gi - tt;
        if (W < 0) W += m;
        if (visited(W)) g += __ldcg(gacc + static_cast<long long>(W) * kFastK + tt);
      }
    } else {
      const int wlo = max(0, gi - kFastK + 1), whi = min(gi, m - kFastK);
      for (int W = wlo; W <= whi; ++W)
        if (visited(W)) g += __ldcg(gacc + static_cast<long long>(W) * kFastK + gi - W);
    }
    g *= ninv;
    if (a.item_G) a.item_G[goff + gi] = g;
    atomicAdd(&a.csr_val[a.csr_idx[goff + gi]], g);
  }
  __syncwarp();
  for (int W = lane; W < nwin; W += 32) {
    if (!visited(W)) continue;
    double* t = gacc + static_cast<long long>(W) * kFastK;
#pragma unroll
    for (int b = 0; b < kFastK; ++b) t[b] = 0.0;
  }
  __syncwarp();
}

template <typename R, typename SAcc>
__device__ void fused_patch_row(const LaunchArgs& a, const ItemDev& itg, int item, const PatchSh<R>& sp,
                                SAcc* sacc, double* gbuf, int lane) {
  constexpr bool k32 = std::is_same<SAcc, float>::value;
  if constexpr (k32) {
    if (fused_patch_row_fast<R>(a, itg, item, sp, sacc, lane)) return;
  }
  const int m = sp.m, k = sp.k, nwin = sp.closed ? m : m - k + 1;
  const long long moff = a.patches[itg.stencil].ainv_off;
  for (int i = lane; i < m; i += 32) gbuf[i] = 0.0;
  __syncwarp();
  for (int W0 = 0; W0 < nwin; W0 += 32) {
    const int Wl = W0 + lane;
    bool vis = false;
    if (Wl < nwin) {
      const SAcc* t = sacc + Wl * k;
      for (int b = 0; b < k; ++b) vis |= t[b] != SAcc(0);
    }
    unsigned vm = __ballot_sync(kFull, vis);
    if (lane == 0 && a.vis_count && vm) atomicAdd(a.vis_count, __popc(vm));
    while (vm) {
      const int W = W0 + __ffs(vm) - 1;
      vm &= vm - 1;
      if (lane < k) {
        const SAcc* t = sacc + W * k;
        int gi = W + lane;
        if (gi >= m) gi -= m;
        if (k32 && a.patch_e32) {
          const float* Ew = a.patch_e32 + moff + static_cast<long long>(W) * k * k + lane;
          float v = 0.f;
#pragma unroll 4
          for (int b = 0; b < k; ++b) v = fmaf(__ldg(Ew + b * k), static_cast<float>(t[b]), v);
          gbuf[gi] += widen(t[lane]) + f32_to_f64(v);
        } else {
          const double* Aw = a.patch_ainv + moff + static_cast<long long>(W) * k * k + lane;
          double v = 0.0;
#pragma unroll 4
          for (int b = 0; b < k; ++b) v = fma(__ldg(Aw + b * k), static_cast<double>(t[b]), v);
          gbuf[gi] += v;
        }
      }
      __syncwarp();
    }
  }
  const long long goff = a.g_off[item];
  if (a.fuse_g == 2) {
    for (int gi = lane; gi < m; gi += 32) {
      const double g = gbuf[gi];
      if (g != 0.0) atomicAdd(&a.g_sum[goff + gi], -g);
    }
  } else {
    double ninv = 0.0;
    if (lane == 0) ninv = -1.0 / static_cast<double>(itg.paths);
    ninv = __shfl_sync(kFull, ninv, 0);
    for (int gi = lane; gi < m; gi += 32) {
      const double g = gbuf[gi] * ninv;
      if (a.item_G) a.item_G[goff + gi] = g;
      // a row of several items (a node inside several patches) may meet a column twice
      atomicAdd(&a.csr_val[a.csr_idx[goff + gi]], g);
    }
  }
  __syncwarp();
}

// FP64 stepping is bound by the FP64 pipe, not by latency: it trades
// occupancy for registers (2 CTAs of 256 per SM instead of 3).
//
// WM (warp mode, for items of few paths): every warp claims its own chunk
// from the queue, stages the item's stencil in its own shared-memory
// corner and adds the stencil moments straight to the item's FP64
// accumulators with global atomics; no warp ever waits for another, so an
// item's longest path delays only its own warp.  Otherwise the CTA's warps
// share the chunk slots described above.
// MB: minimum CTAs of 256 per SM the registers are sized for.  FP64: 2.
// FP32: 3 (80 registers, no spills), and for patch-stencil slot mode also a
// 4-CTA build (64 registers, ~150 B of spills), used where shared memory
// admits 4 CTAs: it runs the 8x8 assembly 2.9 % faster, while point solves,
// warp mode and the larger patches of the 32x32 mesh measured slower at 64
// registers.
template <typename R, int PROB, int ST, bool WM, int MB, bool CV>
__global__ void __launch_bounds__(256, MB) paths_kernel(const LaunchArgs a) {
  using SAcc = typename std::conditional<WM, double, typename SAccType<R, ST>::type>::type;
  using Acc = typename std::conditional<std::is_same<R, double>::value, AccD, AccK>::type;
  constexpr int kPrec = std::is_same<R, double>::value ? 0 : 1;
  constexpr int S = WM ? kMaxBlockWarps : (kPrec == 0 ? 2 : kSlotsFP32);  // slots, or one per warp
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ SlotSh<R> slots[S];
  __shared__ ExitQueue<R> sq[kMaxBlockWarps];
  // warp mode with per-warp FP32 moment accumulators in shared memory (FP32
  // patch stencils): the warp forms its chunk's G row itself when it leaves
  constexpr bool kWmsCapable = WM && ST == 2 && std::is_same<R, float>::value;
  const bool wms = kWmsCapable && a.wm_shared;
  // warp mode whose warps form their items' G rows from the global moments
  const bool wfuse = kWmsCapable && !wms && a.fuse_g == 1;
  const size_t acc_bytes = (!WM || wms) ? paths_slot_acc_bytes(kPrec, ST, a.acc_words) : 0;
  const size_t slot_bytes = paths_slot_bytes(kPrec, ST, (!WM || wms) ? a.acc_words : 0, a.smem_nodes);

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const unsigned long long limit_ns =
      a.wait_limit_ns ? a.wait_limit_ns : 60000000000ull + 1000ull * static_cast<unsigned long long>(a.max_steps);
  const int n_chunks = a.n_chunks_dev ? *a.n_chunks_dev : a.n_chunks;

  if (!WM) {
    if (threadIdx.x < S) slots[threadIdx.x].ready = -1;
    __syncthreads();
    for (int s = warp; s < S; s += nwarps)
      fill_slot<R, ST>(a, n_chunks, slots[s], smem_raw + s * slot_bytes, acc_bytes, s, nwarps, lane);
  }

  ExitQueue<R>& q = sq[warp];
  // Slots known to hold no further chunk: a slot whose chunk queue came up
  // empty is never refilled, so the walk ends once every slot is dead.
  unsigned dead = 0u;
  for (int g = 0;; ++g) {
    int si, c;
    if (WM) {
      // this warp's next chunk
      si = warp;
      int cc = 0;
      if (lane == 0) cc = atomicAdd(a.queue, 1);
      c = __shfl_sync(kFull, cc, 0);
      if (c >= n_chunks) break;
      if (wms) {
        uint4* z = reinterpret_cast<uint4*>(smem_raw + si * slot_bytes);
        for (int i = lane; i < static_cast<int>(acc_bytes / 16); i += 32) z[i] = make_uint4(0u, 0u, 0u, 0u);
      }
      stage_stencil<R, ST>(a, slots[si], smem_raw + si * slot_bytes + acc_bytes, a.items[a.chunks[c].item].stencil,
                           lane);
      if (wfuse) {
        unsigned* vm = reinterpret_cast<unsigned*>(smem_raw + si * slot_bytes + acc_bytes +
                                                   paths_slot_nodes_bytes(kPrec, ST, a.smem_nodes));
        for (int i = lane; i < (a.smem_nodes + 31) / 32; i += 32) vm[i] = 0u;
      }
      __syncwarp();
    } else {
      if (dead == (1u << S) - 1u) break;
      si = g % S;
      if (dead & (1u << si)) continue;
      if (!wait_slot(&slots[si].ready, g, limit_ns, lane)) {
        if (lane == 0) atomicExch(a.queue + 1, 1);
        break;
      }
      c = ld_volatile(&slots[si].chunk);
      if (c < 0) {
        dead |= 1u << si;
        continue;
      }
    }
    SlotSh<R>& sl = slots[si];
    unsigned char* mem = smem_raw + si * slot_bytes;
    const ChunkDev ch = a.chunks[c];
    const ItemDev& itg = a.items[ch.item];
    // stencil moments: the slot's shared accumulators, or (warp mode) the
    // item's FP64 accumulators in global memory
    SAcc* sacc = WM ? reinterpret_cast<SAcc*>(a.acc + itg.acc_off) : reinterpret_cast<SAcc*>(mem);
    float* wacc = reinterpret_cast<float*>(mem);  // (wms: the warp's FP32 moments)
    unsigned* wvis = reinterpret_cast<unsigned*>(mem + acc_bytes + paths_slot_nodes_bytes(kPrec, ST, a.smem_nodes));
    const R* snx = reinterpret_cast<const R*>(mem + acc_bytes);
    const R* sny = snx + a.smem_nodes;
    const double* sth = reinterpret_cast<const double*>(mem + acc_bytes);
    const PatchSh<R>& sp = sl.sp;
    const ArcDev& sarc = sl.sarc;
    const unsigned n_ch = ch.p1 - ch.p0;

    // the item's BVP (independent problems of one functor share a launch; the
    // control variate is the item's own, so learned-CV items and their plain
    // fallback can share one launch)
    const BvpDev& bvp = a.bvp[itg.bvp];
    const bool cv_exact = CV && bvp.cv == 1;                // F from the problem functor
    const bool cv_table = CV && a.cv == 2 && bvp.cv == 2;   // F from the learned gradient table
    const bool cv = cv_exact || cv_table;             // any control term
    const R d0 = R(bvp.dom[0]), d1 = R(bvp.dom[1]), d2 = R(bvp.dom[2]), d3 = R(bvp.dom[3]);
    const R h = R(itg.h), sqrth = R(itg.sqrth), x0 = R(itg.x), y0 = R(itg.y);
    const R s0 = R(itg.sub[0]), s1 = R(itg.sub[1]), s2 = R(itg.sub[2]), s3 = R(itg.sub[3]);
    const bool has_sub = (ST != 0) || itg.sub_shape >= 0;
    const bool sub_circle = (ST == 1) || (ST == 0 && itg.sub_shape == 1);
    // A subdomain strictly inside the rectangular domain is always nearer (in
    // Dentro's signed distance) than the domain boundary, wherever the path
    // is, so the domain distance cannot decide an exit and is not evaluated.
    bool dom_can_win = true;
    if (has_sub && DomainOf<PROB>::shape == 0) {
      if (sub_circle)  // (r, cx, cy)
        dom_can_win = !(s1 - s0 > d0 && s1 + s0 < d2 && s2 - s0 > d1 && s2 + s0 < d3);
      else             // (x0, y0, x1, y1)
        dom_can_win = !(s0 > d0 && s1 > d1 && s2 < d2 && s3 < d3);
    }
    const R st0 = Problem<PROB>::template state<R>(bvp, x0, y0);  // sigma state at the start point
    const R sg0 = Problem<PROB>::template sigma_of<R>(st0);
    // Reflecting sides (FK_PROBLEM_ROBIN), only where the domain can win
    // Dentro's comparison.
    int rmask = 0;
    R rho = R(0), rphi = R(0);
    if constexpr (RobinOf<PROB>::value) {
      rmask = dom_can_win ? (static_cast<int>(bvp.prob[0]) & 15) : 0;
      rphi = R(bvp.prob[1]);
      rho = R(bvp.prob[2]);
    }
    const uint32_t item = static_cast<uint32_t>(ch.item);
    // learned control variate: grad u_hat table of this item's region
    const float2* ctab = nullptr;
    R cx0 = R(0), cy0 = R(0), csx = R(0), csy = R(0);
    float tex_y0 = 0.f;  // the region's first texel row of the filtered table
    const int G = a.cv_grid;
    if (cv_table) {
      const int r = itg.cv_region;
      tex_y0 = static_cast<float>(r * G) + 0.5f;
      const double* rc = a.cv_rect + 4 * r;
      ctab = a.cv_tab + static_cast<long long>(r) * G * G;
      cx0 = R(rc[0]);
      cy0 = R(rc[1]);
      csx = R((G - 1) / (rc[2] - rc[0]));
      csy = R((G - 1) / (rc[3] - rc[1]));
    }

    Acc acc[kNumAcc];
    unsigned long long n_steps = 0;
    unsigned n_dom = 0, n_cap = 0, n_done = 0;
    R x = x0, y = y0, Y = R(1), Z = R(0), xi = R(0), st = st0, sgc = sg0;  // sgc = sigma_of(st)
    int k = 0;
    // learned control variate: grad u_hat at (px, py), bilinear in the
    // region's table (clamped to it)
    auto cv_grad = [&](R px, R py, R& gx, R& gy) {
      R u = (px - cx0) * csx, v = (py - cy0) * csy;
      u = fmin(fmax(u, R(0)), R(G - 1) - R(1e-3));
      v = fmin(fmax(v, R(0)), R(G - 1) - R(1e-3));
      if (std::is_same<R, float>::value && a.cv_tex) {
        // the texture unit's bilinear filter (texel centres at i + 1/2)
        const float2 g = tex2D<float2>(a.cv_tex, static_cast<float>(u) + 0.5f, static_cast<float>(v) + tex_y0);
        gx = R(g.x);
        gy = R(g.y);
      } else {
        const int i = static_cast<int>(u), j = static_cast<int>(v);
        const R fu = u - R(i), fv = v - R(j);
        const float2* T = ctab + j * G + i;
        const float2 t00 = __ldg(T), t10 = __ldg(T + 1), t01 = __ldg(T + G), t11 = __ldg(T + G + 1);
        gx = (R(1) - fv) * ((R(1) - fu) * R(t00.x) + fu * R(t10.x)) + fv * ((R(1) - fu) * R(t01.x) + fu * R(t11.x));
        gy = (R(1) - fv) * ((R(1) - fu) * R(t00.y) + fu * R(t10.y)) + fv * ((R(1) - fu) * R(t01.y) + fu * R(t11.y));
      }
    };
    // grad u_hat at the lane's current point: fetched as soon as the lane
    // reaches the point, so that the lookup's latency overlaps the rest of
    // the iteration and the next step's coefficients and normals
    R cgx = R(0), cgy = R(0);
    // every lane's first path of the chunk (chunk-local index); in warp mode
    // the warp owns the chunk and counts its paths in a register
    unsigned base = 0, wnext = 32u;
    if (!WM && lane == 0) base = atomicAdd(&sl.next, 32u);
    unsigned pl = __shfl_sync(kFull, base, 0) + lane;
    bool active = pl < n_ch;
    if (cv_table && active) cv_grad(x, y, cgx, cgy);
    int qn = 0;  // queued exits of this warp (warp-uniform)

    // Processes the top `cnt` (<= 32) queued exits, one per lane: exit value
    // and statistics (Reduce_Analytic, FeynmanKacSolver.cpp:198-292) and the
    // stencil moments of subdomain exits.
    auto process = [&](int cnt) {
      const int qb = qn - cnt;
      const bool mine = lane < cnt;
      R ex = R(0), ey = R(0), Yv = R(0);
      bool sub_exit = false;
      if (mine) {
        const int e = qb + lane;
        ex = q.x[e]; ey = q.y[e]; Yv = q.Y[e];
        const R Zv = q.Z[e], xv = CV ? q.xi[e] : R(0);
        const unsigned kf = q.kf[e];
        const bool dw = (kf >> 30) & 1u, cp = (kf >> 31) & 1u;
        sub_exit = (ST != 0) && !dw;
        const R g = Problem<PROB>::u(bvp, ex, ey);  // g = u for every registered problem
        const R score = Zv + Yv * g;
        const R vr = score + xv;
        acc[0].add(score);
        acc[1].add(score * score);
        if constexpr (CV) {
          acc[2].add(xv + xv * xv);
          acc[3].add(vr);
          acc[4].add(vr * vr);
          acc[5].add(xv * score);
          acc[6].add(sub_exit ? Zv + xv : vr);
          acc[7].add(xv * xv);
        } else {  // xi = 0: the VR sums equal the plain ones
          acc[6].add(sub_exit ? Zv : score);
        }
        n_steps += kf & 0x3fffffffu;
        n_dom += dw ? 1u : 0u;
        n_cap += cp ? 1u : 0u;
        ++n_done;
      }
      if (ST == 2) {
        if (sub_exit) {
          // Gaussian k-nearest moments t_W[j] += Y phi_j, one exit per lane
          int nearest;
          const int L = knn_window<R>(sp, snx, sny, ex, ey, nearest);
          const int kk = sp.k, m = sp.m;
          const R e2 = sp.e2;
          // Weights below exp(-kPhiCut) ~ 1e-30 (FP64 stepping) or
          // exp(-kPhiCut32) ~ 3e-8 (FP32 stepping, below the FP32 resolution of
          // the moments) are not added.  The exit
          // point lies on the patch boundary next to the window's node
          // `nearest`; walking the window away from it (down from it, up from
          // the next node) the distances grow until the opposite side, which
          // lies beyond the cutoff on patches marked `walk`: each walk then
          // stops at its first cut node, once past the nodes around the exit.
          int jn = nearest - L;
          if (jn < 0) jn += m;
          if (wfuse) atomicOr(&wvis[L >> 5], 1u << (L & 31));  // the window this exit chose
          auto add = [&](int j) -> bool {
            int idx = L + j;
            if (idx >= m) idx -= m;
            const R dx = ex - snx[idx], dy = ey - sny[idx];
            const R arg = e2 * (dx * dx + dy * dy);
            if (!(arg < R(std::is_same<R, float>::value ? kPhiCut32 : kPhiCut))) return false;
            const R wv = Yv * fexp(-arg);
            if constexpr (WM && std::is_same<R, float>::value) {
              if (wms) atomicAdd(&wacc[L * kk + j], wv);     // the warp's FP32 moments in shared memory
              else atomicAdd(&sacc[L * kk + j], f32_to_f64(wv));  // the item's FP64 accumulator in global memory
            } else
              atomicAdd(&sacc[L * kk + j], static_cast<SAcc>(wv));
            return true;
          };
          if (sp.walk == kWalkSpan && jn < kk) {
            constexpr int kSpan = std::is_same<R, float>::value ? kSpanMax32 : kSpanMax;
#pragma unroll
            for (int t = -kSpan; t <= kSpan; ++t) {
              const int j = jn + t;
              if (j >= 0 && j < kk) add(j);
            }
          } else if (sp.walk == kWalkStop && jn < kk) {
            for (int j = jn; j >= 0; --j)
              if (!add(j) && j < jn - 1) break;
            for (int j = jn + 1; j < kk; ++j)
              if (!add(j) && j > jn + 1) break;
          } else {
            for (int j = 0; j < kk; ++j) add(j);
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
      qn = qb;
    };

    // One loop, one call site of process(): while any lane has a path it
    // steps; queued exits are processed 32 at a time and, once the chunk is
    // exhausted for this warp, the remainder.
    for (;;) {
      const bool any = __any_sync(kFull, active);
      if (!any && qn == 0) break;
      bool exits = false, dom_wins = true, capped = false;
      R ex = R(0), ey = R(0);
      if (active) {
        // ---- one Euler-Maruyama step (Paso_Absorbente, FeynmanKacSolver.cpp:7-18)
        StepCoef<R> co;
        Problem<PROB>::step(bvp, x, y, st, sgc, cv_exact, co);
        if (cv_table) {
          // F = -sigma^T grad u_hat at the step's start point, looked up
          // when the lane reached it (end of the previous iteration)
          co.Fx = -co.s * cgx;
          co.Fy = -co.s * cgy;
        }
        // one Philox block per step, counter (step, path, item, stream), words
        // x and y: every lane computes a block at every step, so the warp
        // stays converged (a block split over two steps put the lanes' step
        // parities, and with them the Philox branch, out of step)
        const uint4 r = philox10_rk(make_uint4(static_cast<uint32_t>(k), ch.p0 + pl, item, a.stream), a.rkey);
        const uint32_t wa = r.x, wb = r.y;
        R z0, z1;
        box_muller(wa, wb, z0, z1);
        const R dWx = sqrth * z0, dWy = sqrth * z1;
        if constexpr (RobinOf<PROB>::value) {
          // ---- Paso_Reflejante (FeynmanKacSolver.cpp:19-67) on reflecting sides
          R xn = x + (co.bx * h + co.s * dWx), yn = y + (co.by * h + co.s * dWy);
          R lt[4] = {R(0), R(0), R(0), R(0)};  // local time pushed back through each side
          R ploc = R(0), vloc = R(0);
          if (rmask) {
            // Lepingle's step on every reflecting side within rho of the
            // current point: the push-back through the side is the maximum
            // over the step of the Brownian bridge of the normal
            // displacement, drawn exactly from an Exp(1) variate (mean 2h of
            // the reference's omega, :33-36) and started from the distance
            // to the side.  The sides' normals are the coordinate axes and
            // sigma is s I, so in a corner the two pushes are independent.
            uint4 re = make_uint4(0u, 0u, 0u, 0u);
            bool drawn = false;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              if (!((rmask >> q) & 1)) continue;
              const R dq = q == 0 ? d0 - x : (q == 1 ? d1 - y : (q == 2 ? x - d2 : y - d3));
              if (!(dq > -rho)) continue;
              if (!drawn) {
                re = philox10_rk(make_uint4(0x80000000u | static_cast<uint32_t>(k), ch.p0 + pl, item, a.stream),
                                 a.rkey);
                drawn = true;
              }
              const R E = exp1_draw(q == 0 ? re.x : (q == 1 ? re.y : (q == 2 ? re.z : re.w)), R(0));
              const R nx = q == 0 ? R(-1) : (q == 2 ? R(1) : R(0));
              const R ny = q == 1 ? R(-1) : (q == 3 ? R(1) : R(0));
              const R uc = co.s * (nx * dWx + ny * dWy) + (nx * co.bx + ny * co.by) * h;
              const R nu = R(0.5) * (uc + fsqrt(uc * uc + R(2) * co.s * co.s * h * E));
              const R L = fmax(R(0), nu + fmin(dq, R(0)));
              xn -= L * nx;
              yn -= L * ny;
              lt[q] = L;
            }
            // a reflecting side crossed in the step: back onto it, the
            // overshoot added to its local time (:49-58)
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              if (!((rmask >> q) & 1)) continue;
              const R o = q == 0 ? d0 - xn : (q == 1 ? d1 - yn : (q == 2 ? xn - d2 : yn - d3));
              if (o > R(0)) {
                if (q == 0) xn = d0; else if (q == 1) yn = d1; else if (q == 2) xn = d2; else yn = d3;
                lt[q] += o;
              }
            }
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              const R l = lt[q];
              if (l > R(0)) {
                // psi at the side's point nearest the new position
                const R px = q == 0 ? d0 : (q == 2 ? d2 : fmin(fmax(xn, d0), d2));
                const R py = q == 1 ? d1 : (q == 3 ? d3 : fmin(fmax(yn, d1), d3));
                const R nx = q == 0 ? R(-1) : (q == 2 ? R(1) : R(0));
                const R ny = q == 1 ? R(-1) : (q == 3 ? R(1) : R(0));
                ploc += Problem<PROB>::psi(bvp, px, py, nx, ny) * l;
                vloc += rphi * l;
              }
            }
          }
          Z += co.f * Y * h + ploc * Y;
          if (cv) xi += Y * (co.Fx * dWx + co.Fy * dWy);
          Y += co.c * Y * h + vloc * Y;
          x = xn;
          y = yn;
        } else {
          Z += co.f * Y * h;
          if (cv) xi += Y * (co.Fx * dWx + co.Fy * dWy);
          Y += co.c * Y * h;
          x += co.bx * h + co.s * dWx;
          y += co.by * h + co.s * dWy;
        }
        ++k;
        // ---- exit rule (Dentro, FeynmanKacSolver.cpp:68-106)
        Bnd<R> w;
        if (dom_can_win) {
          w = (DomainOf<PROB>::shape == 1) ? circle_dist<R>(x, y, d0, d1, d2) : rect_dist<R>(x, y, d0, d1, d2, d3);
          if (has_sub) {
            const Bnd<R> sb = sub_circle ? circle_dist<R>(x, y, s0, s1, s2) : rect_dist<R>(x, y, s0, s1, s2, s3);
            if (!(w.d >= sb.d)) { w = sb; dom_wins = false; }
          }
        } else {
          w = sub_circle ? circle_dist<R>(x, y, s0, s1, s2) : rect_dist<R>(x, y, s0, s1, s2, s3);
          dom_wins = false;
        }
        // sigma at the new point (kept for the next step) or at the
        // projection: one evaluation at the selected point, no divergence
        const bool inside = w.d < R(0);
        const R stq = Problem<PROB>::template state<R>(bvp, inside ? x : w.ex, inside ? y : w.ey);
        const R sg = Problem<PROB>::template sigma_of<R>(stq);
        if (inside) {
          st = stq;
          sgc = sg;
        }
        // Gobet shift kGobet |sigma^T n| sqrt(h) (FeynmanKacSolver.cpp:85,92).
        // Every registered sigma is s I, and the normals are unit vectors (axes
        // or the normalised diagonal), so FP32 stepping takes |sigma^T n| = s;
        // FP64 stepping forms the norm as the reference does.
        R thr;
        if constexpr (std::is_same<R, float>::value) {
          thr = R(kGobet) * sg * sqrth;
        } else {
          const R nsx = w.nx * sg, nsy = w.ny * sg;
          thr = R(kGobet) * fsqrt(nsx * nsx + nsy * nsy) * sqrth;
        }
        capped = k >= a.max_steps;
        exits = !(w.d < thr) || capped;
        if constexpr (RobinOf<PROB>::value) {
          if (rmask && dom_wins && robin_side<R>(w, rmask) >= 0) {
            // The nearest boundary is a reflecting side: no stop there
            // (dentro / reflejada, :82-84).  The path still stops within the
            // Gobet band of the subdomain or of an absorbing side, the
            // nearer of them (the reference tests only the nearest boundary,
            // which lets paths near a mixed corner cross the absorbing side).
            const R dref = w.d;  // the reflecting side's distance
            R da = R(-FLT_MAX);
            int qa = -1;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              if ((rmask >> q) & 1) continue;
              const R dq = q == 0 ? d0 - x : (q == 1 ? d1 - y : (q == 2 ? x - d2 : y - d3));
              if (dq > da) { da = dq; qa = q; }
            }
            if (qa >= 0) {
              w.d = da;
              w.ex = qa == 0 ? d0 : (qa == 2 ? d2 : fmin(fmax(x, d0), d2));
              w.ey = qa == 1 ? d1 : (qa == 3 ? d3 : fmin(fmax(y, d1), d3));
            } else {
              w.d = R(-FLT_MAX);
            }
            if (has_sub) {
              // (a subdomain boundary that coincides with the reflecting side,
              // a tie that the domain wins, is not a candidate)
              const Bnd<R> sb = sub_circle ? circle_dist<R>(x, y, s0, s1, s2) : rect_dist<R>(x, y, s0, s1, s2, s3);
              if (sb.d < dref && !(w.d >= sb.d)) { w = sb; dom_wins = false; }
            }
            exits = !(w.d < thr) || capped;
          }
          // a path that goes on from a point on (or, by rounding, just past)
          // a reflecting side steps with sigma at that point
          if (!exits && !inside) {
            st = Problem<PROB>::template state<R>(bvp, x, y);
            sgc = Problem<PROB>::template sigma_of<R>(st);
          }
        }
        ex = w.ex;
        ey = w.ey;
      }
      // ---- queue the exits; the exiting lanes start their next path at once
      const unsigned em = __ballot_sync(kFull, exits);
      if (em) {
        const int rank = __popc(em & ((1u << lane) - 1u));
        const int leader = __ffs(em) - 1;
        unsigned nb = 0;
        if (WM) {
          nb = wnext;
          wnext += static_cast<unsigned>(__popc(em));
        } else {
          if (lane == leader) nb = atomicAdd(&sl.next, static_cast<unsigned>(__popc(em)));
          nb = __shfl_sync(kFull, nb, leader);
        }
        if (exits) {
          const int e = qn + rank;
          q.x[e] = ex; q.y[e] = ey; q.Y[e] = Y; q.Z[e] = Z; if constexpr (CV) q.xi[e] = xi;
          q.kf[e] = static_cast<unsigned>(k) | (dom_wins ? 1u << 30 : 0u) | (capped ? 1u << 31 : 0u);
          pl = nb + rank;
          active = pl < n_ch;
          x = x0; y = y0; Y = R(1); Z = R(0); xi = R(0); k = 0; st = st0; sgc = sg0;
        }
        qn += __popc(em);
        __syncwarp();
      }
      // the next step's grad u_hat: at the new point, or at the start point
      // of the lane's next path
      if (cv_table && active) cv_grad(x, y, cgx, cgy);
      if (qn >= 32 || !any) {
        process(qn >= 32 ? 32 : qn);
        __syncwarp();
      }
    }

    // ---- the warp leaves the chunk: its sums into the item's FP64 sums
    double* sums = a.stats + static_cast<long long>(ch.item) * kNumStats;
    const int slot_of[kNumAcc] = {kStatScore, kStatScore2, kStatXiAlias, kStatVR,
                                  kStatVR2, kStatXiScore, kStatB, kStatXi2};
#pragma unroll
    for (int j = 0; j < kNumAcc; ++j) {
      if (!CV && j != 0 && j != 1 && j != 6) continue;
      const double t = warp_reduce(acc[j], lane);
      if (lane == 0 && t != 0.0) {
        atomicAdd(&sums[slot_of[j]], t);
        if (!CV && j < 2) atomicAdd(&sums[slot_of[j + 3]], t);  // score -> VR, score^2 -> VR^2
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      n_steps += __shfl_xor_sync(kFull, n_steps, o);
      n_dom += __shfl_xor_sync(kFull, n_dom, o);
      n_cap += __shfl_xor_sync(kFull, n_cap, o);
      n_done += __shfl_xor_sync(kFull, n_done, o);
    }
    if (lane == 0) {
      if (n_steps) atomicAdd(&sums[kStatSteps], static_cast<double>(n_steps));
      if (n_dom) atomicAdd(&sums[kStatDom], static_cast<double>(n_dom));
      if (n_cap) atomicAdd(&sums[kStatCap], static_cast<double>(n_cap));
      if (n_done) atomicAdd(&sums[kStatPaths], static_cast<double>(n_done));
    }
    __syncwarp();
    if (WM) {
      if constexpr (kWmsCapable) {
        // the chunk's G row from the warp's own moments
        if (wms) fused_patch_row<R, float>(a, itg, ch.item, sp, wacc, reinterpret_cast<double*>(mem + acc_bytes), lane);
        if (wfuse) fused_patch_row_wm<R>(a, itg, ch.item, sp, a.acc + itg.acc_off, wvis, lane);
      }
      continue;  // (otherwise the warp's moments are already in global memory)
    }
    __threadfence_block();
    int left = 0;
    if (lane == 0) left = atomicSub(&sl.warps_left, 1);
    left = __shfl_sync(kFull, left, 0);
    if (left == 1) {
      // last warp out: flush the chunk's stencil moments, refill the slot
      __threadfence_block();
      bool fused = false;
      if constexpr (ST == 2) {
        if (a.fuse_g) {
          // the chunk's G row straight from shared memory
          fused_patch_row<R, SAcc>(a, itg, ch.item, sp, sacc, reinterpret_cast<double*>(mem + acc_bytes), lane);
          fused = true;
        }
      }
      if (ST != 0 && !fused) {
        double* gacc = a.acc + itg.acc_off;
        if (!a.acc_zeroed) {
          // the chunk is the whole item: its moments are stored, zeros included
          // (no memset of the accumulators and no atomics)
          const int words = (ST == 2) ? (sp.closed ? sp.m : sp.m - sp.k + 1) * sp.k : sarc.n;
          for (int i = lane; i < words; i += 32) {
            if constexpr (std::is_same<SAcc, float>::value) gacc[i] = f32_to_f64(sacc[i]);
            else gacc[i] = static_cast<double>(sacc[i]);
          }
        } else {
          for (int i = lane; i < a.acc_words; i += 32) {
            if constexpr (std::is_same<SAcc, float>::value) {
              // FP32 chunk partials: widened on the integer pipes (F2F runs on the FP64 pipe)
              const float t = sacc[i];
              if (t != 0.f) atomicAdd(&gacc[i], f32_to_f64(t));
            } else {
              const double t = static_cast<double>(sacc[i]);
              if (t != 0.0) atomicAdd(&gacc[i], t);
            }
          }
        }
      }
      __syncwarp();
      fill_slot<R, ST>(a, n_chunks, sl, mem, acc_bytes, g + S, nwarps, lane);
    }
  }
}

// The kernel instantiation of a launch: stencil kind st (0 points, 1 arcs,
// 2 patches), `four` the 4-CTA build of FP32 patch slot mode; CV: the build
// with the control-variate terms (without them xi = 0 and the VR sums are the
// plain ones).
template <typename R, int PROB, bool WM, bool CV>
const void* paths_fn(int st, bool four) {
  constexpr int MB = std::is_same<R, double>::value ? 2 : 3;
  switch (st) {
    case 1: return reinterpret_cast<const void*>(&paths_kernel<R, PROB, 1, WM, MB, CV>);
    case 2:
      if constexpr (std::is_same<R, float>::value && !WM)
        if (four) return reinterpret_cast<const void*>(&paths_kernel<R, PROB, 2, WM, 4, CV>);
      return reinterpret_cast<const void*>(&paths_kernel<R, PROB, 2, WM, MB, CV>);
    default: return reinterpret_cast<const void*>(&paths_kernel<R, PROB, 0, WM, MB, CV>);
  }
}
template <typename R, bool WM, bool CV>
const void* paths_fn_r(int problem, int st, bool four) {
  return with_problem(problem, [&](auto t) { return paths_fn<R, decltype(t)::value, WM, CV>(st, four); });
}

}  // namespace
}  // namespace fk
