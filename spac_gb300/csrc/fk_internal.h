// Internal host/device interface of libspac_fk: the device-side records the
// kernels read and the host launchers the C ABI calls.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace fk {

struct BvpDev;

// One solve item: a point (Solve_OMP_Analytic(X0,...)) or a node of a mesh
// solved against one stencil (Solve_OMP_Analytic(Nudo&, ..., Interfaz)).
struct ItemDev {
  double x, y, h, sqrth;
  double sub[4];          // subdomain boundary parameters
  unsigned paths;
  int stencil;            // arc / patch index, -1 for point solves
  int frontera;           // B = g(x), no paths
  int sub_shape;          // point solves: 0 rect, 1 circle, -1 = domain
  int cv_region;          // learned control variate: region of the grad table
  int bvp;                // index into the launch's BVP records
  long long acc_off;      // first double of this item's stencil accumulator
};

struct ChunkDev {
  int item;
  unsigned p0, p1;
};

// Reference arc stencil (Interfaz): iPsi applied per item after the paths.
struct ArcDev {
  double cx, cy, c2, radius;
  int interior, n;
  long long theta_off, ipsi_off;  // into the arc theta / iPsi pools
};

// Gaussian k-nearest stencil on a rectangular patch boundary.
struct PatchDev {
  double rect[4];
  double eps2;
  int m, k, closed, nwin;
  int walk, walk32;     // kWalkFull, kWalkStop or kWalkSpan (how an exit visits its window's nodes), FP64 / FP32 cutoff
  long long node_off;   // 2*m doubles (x, y) in chain order
  long long ainv_off;   // nwin * k * k doubles, column-major per window
  // sides: chain index of the first node, node count, axis (0: node x varies),
  // fixed coordinate, coordinate of the first node and signed step
  int side_first[4], side_count[4], side_axis[4];
  double side_fixed[4], side_start[4], side_step[4];
  // window table (kKnnBins bins per side step): side s has knn_n[s] entries
  // from knn_off + knn_base[s], bin b covering u in knn_u0[s] + [b, b+1) /
  // kKnnBins, u = (coordinate along the side - side_start) / side_step
  long long knn_off;
  int knn_base[4], knn_n[4];
  double knn_u0[4];
};

// Per-item FP64 sums written by the path kernel: score, score^2, xi + xi^2
// (the reference's aliased xi slot), score + xi, (score + xi)^2, xi score,
// steps, B, domain exits, capped paths, xi^2, paths completed.
enum { kStatScore = 0, kStatScore2, kStatXiAlias, kStatVR, kStatVR2, kStatXiScore, kStatSteps, kStatB, kStatDom,
       kStatCap, kStatXi2, kStatPaths, kNumStats = 12 };

// Path-kernel shared memory: each CTA keeps paths_slots() chunks in flight
// (kSlotsFP32 for FP32 stepping, 2 for FP64), so that its warps move on to
// the next chunk while the last paths of the previous one finish.  A slot
// holds the chunk's stencil accumulators followed by its stencil nodes (patch
// node coordinates in the stepping precision, or arc angles in FP64), each
// part padded to 16 bytes.
constexpr int kSlotsFP32 = 3;

// Gaussian stencil weights exp(-arg) with arg >= kPhiCut (< 1e-30) are not
// added; FP32 stepping drops them from arg >= kPhiCut32 (< 3.1e-8 = 2^-25,
// below FP32 resolution next to the exit's own nearest weight: at least
// exp(-(eps spacing / 2)^2) along a side, 0.78 at eps spacing = 1 and 0.105
// at 3, and exp(-(eps spacing)^2) in a patch corner).
constexpr float kPhiCut = 69.0f;
constexpr float kPhiCut32 = 17.3f;
// How an exit visits the nodes of its k-window (PatchDev::walk):
//   kWalkFull  every node of the window;
//   kWalkStop  outward from the exit's nearest node, each way until the first
//              node beyond the weight cutoff;
//   kWalkSpan  the nodes within kSpanMax (FP64 stepping) or kSpanMax32 (FP32)
//              chain places of the nearest node, a fixed unrolled range that
//              holds every node within the stepping precision's cutoff.
constexpr int kWalkFull = 0, kWalkStop = 1, kWalkSpan = 2;
constexpr int kSpanMax = 4, kSpanMax32 = 2;
// Window table of a patch side: the exit's k-window is L0 or L0 + 1 (the
// latter iff node L0 + k is nearer than node L0); an entry with kKnnFull set
// sends the exit to the sliding search.
constexpr int kKnnBins = 16;
constexpr unsigned short kKnnFull = 0x8000;
__host__ __device__ inline int paths_slots(int precision) { return precision == 0 ? 2 : kSlotsFP32; }
__host__ __device__ inline size_t paths_slot_acc_bytes(int precision, int stencil_kind, int acc_words) {
  const size_t w = (precision == 0 || stencil_kind == 1) ? 8 : 4;
  return (static_cast<size_t>(acc_words) * w + 15) & ~static_cast<size_t>(15);
}
// The slot's stencil nodes (patch: x and y in the stepping precision; arc: angles).
__host__ __device__ inline size_t paths_slot_nodes_bytes(int precision, int stencil_kind, int smem_nodes) {
  size_t nodes = 0;
  if (stencil_kind == 2) nodes = 2ull * smem_nodes * (precision == 0 ? 8 : 4);
  if (stencil_kind == 1) nodes = static_cast<size_t>(smem_nodes) * 8;
  return (nodes + 15) & ~static_cast<size_t>(15);
}
// Slot layout: moment accumulators, stencil nodes, and for patch stencils a
// bit per window (the windows a warp-mode chunk's exits chose).
__host__ __device__ inline size_t paths_slot_bytes(int precision, int stencil_kind, int acc_words, int smem_nodes) {
  const size_t vis = stencil_kind == 2 ? ((4ull * ((smem_nodes + 31) / 32) + 15) & ~static_cast<size_t>(15)) : 0;
  return paths_slot_acc_bytes(precision, stencil_kind, acc_words) + paths_slot_nodes_bytes(precision, stencil_kind, smem_nodes) +
         vis;
}

struct LaunchArgs {
  int acc_zeroed;  // 1: the moment accumulators were zeroed (chunks add atomically);
                   // 0: every chunk is a whole item (slot mode), its flush stores them
  const BvpDev* bvp;
  const ItemDev* items;
  const ChunkDev* chunks;
  int n_chunks;
  const int* n_chunks_dev; // if set, the chunk count is read from device memory (chunks built on the device)
  const ArcDev* arcs;
  const double* arc_theta;
  const PatchDev* patches;
  const double* patch_nodes;
  const unsigned short* knn_tab;  // window tables of the patches (PatchDev::knn_off)
  int* queue;              // [0] chunk counter, [1] error word (both zeroed before launch)
  int* vis_count;          // may be null: += windows whose moments the kernel formed into G rows
  double* stats;           // n_items * kNumStats
  double* acc;             // stencil accumulators
  uint32_t key0, key1, stream;
  uint32_t rkey[20];        // Philox round keys from (key0, key1): set_round_keys
  int max_steps;
  unsigned long long wait_limit_ns;  // slot waits give up after this (0: 60 s + 1 us x max_steps)
  int cv;                  // 0 none, 1 exact gradient functor, 2 learned (gradient table)
  int any_cv;              // 1: some item of the launch has a control variate (else the build without xi)
  const float2* cv_tab;    // [regions][grid][grid] grad u_hat
  const double* cv_rect;   // 4 per region
  int cv_grid;
  unsigned long long cv_tex;  // the table as a filtered texture (FP32 stepping), or 0
  int stencil_kind;        // 0 none, 1 arc, 2 patch
  int acc_words;           // shared accumulator length (elements) per CTA
  int smem_nodes;          // patch nodes / arc angles staged in shared memory (max over stencils)
  const void* mlp;         // device MLP parameters (FK_CV_MLP)
  // Fused G rows (patch stencils, slot mode): the last warp out of a chunk
  // applies A_W^-1 to the chunk's moments in shared memory, so that the
  // moments never reach global memory.  1: every chunk is a whole item, whose
  // G row goes into the CSR values (and item_G if set); 2: adaptive rounds,
  // the chunk's unnormalised row is added to g_sum.
  int fuse_g;
  int wm_shared;           // warp mode: moments in per-warp shared FP32 accumulators, rows fused
  const float* patch_e32;  // FP32 moments: E_W = A_W^-1 - I, the layout of the FP64 inverses
  const double* patch_ainv;  // FP64 moments: A_W^-1
  double* g_sum;           // fuse_g == 2: running row sums, g_off indexed
  const long long* g_off;  // item -> first entry of its G row in item_G / csr_idx
  const int* csr_idx;      // G entry -> CSR position
  double* csr_val;
  double* item_G;          // may be null
};
// The ten Philox4x32-10 round keys of a launch's seed key (key0, key1):
// round r uses (key0 + r 0x9E3779B9, key1 + r 0xBB67AE85) mod 2^32.
inline void set_round_keys(LaunchArgs& a) {
  uint32_t k0 = a.key0, k1 = a.key1;
  for (int r = 0; r < 10; ++r) {
    a.rkey[2 * r] = k0;
    a.rkey[2 * r + 1] = k1;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}


struct FinalizeArgs {
  const BvpDev* bvp;
  const ItemDev* items;
  int n_items;
  const ArcDev* arcs;
  const double* arc_ipsi;
  const PatchDev* patches;
  const double* patch_ainv;
  // FP32-stepping assemblies: A_W^-1 = I + E_W with E_W in FP32 (same layout
  // as patch_ainv) and max |E| per patch; the identity part is applied in
  // FP64, E_W t_W in FP32 when max |E| < kSplitMaxE (may be null: FP64 only)
  const float* patch_e32;
  const float* patch_emax;
  int split_ok;
  const double* stats;
  const double* acc;
  int stencil_kind;
  const long long* g_off;   // item -> first entry in item_G
  double* item_G;           // may be null
  double* item_B;           // may be null
  double* item_stats;       // n_items * 16 (fk_stats layout), may be null
  const int* csr_idx;       // item -> csr positions (g_off indexed), may be null
  double* csr_val;          // may be null
  const int* row;           // item -> row (for B scatter)
  double* B;                // may be null
  int* flags;               // may be null: [0] |= an item had capped paths, [1] |= an item lost paths
  int* lost;                // may be null: [0] = 1 + the first item whose completed paths differ, [1] = their count
  int* vis_count;           // may be null: += windows whose moments the kernel formed into G rows
  int g_fused;              // 1: the path kernel already added the live items' G rows (LaunchArgs::fuse_g)
  // patch stencils: the largest nwin * k, m and the common k over the
  // launch's patches (fin_words = 0: the generic per-item path)
  int fin_words, fin_m, fin_k;
};

// host launchers (fk_paths.cu)
// warp_mode: every warp works its own chunks and adds the stencil moments to
// the items' global accumulators (items of few paths); otherwise the CTA's
// warps share chunk slots with shared-memory accumulators
// wm_shared: warp mode with per-warp FP32 moment accumulators in shared memory
size_t paths_smem_bytes(int precision, int stencil_kind, int acc_words, int smem_nodes, bool warp_mode = false,
                        int block = 256, bool wm_shared = false);
cudaError_t launch_paths(const LaunchArgs& a, int problem, int precision, int grid, int block,
                         size_t smem, cudaStream_t s, bool warp_mode = false);
// path-kernel builds without the control-variate terms (fk_paths_plain.cu)
const void* select_paths_plain(int problem, int precision, int st, bool warp_mode, bool four);
int paths_kernel_occupancy(int problem, int precision, int stencil_kind, int cv, int block, size_t smem,
                           bool warp_mode = false);
// host launchers (fk_kernels.cu)
cudaError_t launch_finalize(const FinalizeArgs& a, int problem, cudaStream_t s);
// batched FP64 full-pivot Gauss-Jordan inverse: matrix b is ns[b] x ns[b],
// column-major at offset offs[b] of A (input) and inv (output); ns[b] <= 64
cudaError_t launch_inverse(const double* A, double* inv, const int* ns, const long long* offs, int nmax, int count,
                           cudaStream_t s);
// builds Psi for arcs (theta-IMQ) / A_W for patch windows into `out` (column-major)
cudaError_t launch_build_psi(const ArcDev* arcs, const double* theta, int n_arcs, double* out, cudaStream_t s);
cudaError_t launch_build_windows(const PatchDev* patches, const double* nodes, int n_patches,
                                 const long long* win_base, long long total_windows, int k, double* out,
                                 cudaStream_t s);
// adaptive assembly rounds (fk_assembly_*): a round's statistics into the
// running sums (and its per-path variance per item); the rows from the
// running row sums at the end
cudaError_t launch_round_stats(const ItemDev* items, int n, const double* stats, double* run_stats, double* item_var,
                               int* flags, cudaStream_t s);
cudaError_t launch_rows_from_sums(const ItemDev* items, int n, const PatchDev* patches, const long long* g_off,
                                  const double* g_sum, const int* csr_idx, double* csr_val, double* item_G,
                                  cudaStream_t s);
// E = A^-1 - I of every window in FP32, and max |E| per patch
cudaError_t launch_split_inverse(const PatchDev* patches, int n_patches, const double* ainv, float* e32, float* emax,
                                 cudaStream_t s);
// FP32-stepping assemblies apply E_W = A_W^-1 - I in FP32 (relative error of
// a G entry ~ 1e-7 max |E| sqrt(k), far below the Monte Carlo error of any
// row): in the finalize kernel and in the path kernel's fused G rows.  A
// patch with larger entries (Gaussian windows with eps * spacing well below
// 1: max |E| is 1.2e-4 at eps * spacing = 3, 0.6 at 1 and 1.8 at 0.8) keeps
// the finalize kernel's FP64 products.
constexpr float kSplitMaxE = 64.0f;

}  // namespace fk
