// C ABI of libspac_fk (include/spac_fk.h): context, registries, meshes and the
// launch sequence path kernel -> finalize/scatter on the context stream.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/spac_fk.h"
#include "fk_device.cuh"
#include "fk_internal.h"
#include "fk_disk.h"
#include "fk_mesh.h"
#include "fk_mlp.h"

namespace fk {

// device buffer that grows and never shrinks; owns its allocation (not copyable)
struct DBuf {
  void* p = nullptr;
  size_t bytes = 0;
  DBuf() = default;
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  cudaError_t ensure(size_t n) {
    if (n <= bytes) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    cudaError_t e = cudaMalloc(&p, n);
    if (e == cudaSuccess) bytes = n;
    return e;
  }
  template <typename T> T* as() const { return static_cast<T*>(p); }
  ~DBuf() { if (p) cudaFree(p); }
};

// Page-locked host staging (per-call uploads and result reads; every API call
// drains its stream before it returns, so a staging buffer is free again at
// the next call).
struct HBuf {
  void* p = nullptr;
  size_t bytes = 0;
  HBuf() = default;
  HBuf(const HBuf&) = delete;
  HBuf& operator=(const HBuf&) = delete;
  cudaError_t ensure(size_t n) {
    if (n <= bytes) return cudaSuccess;
    if (p) cudaFreeHost(p);
    p = nullptr;
    bytes = 0;
    cudaError_t e = cudaMallocHost(&p, n);
    if (e == cudaSuccess) bytes = n;
    return e;
  }
  ~HBuf() { if (p) cudaFreeHost(p); }
};

template <typename T>
static cudaError_t upload_pinned(DBuf& b, HBuf& h, const std::vector<T>& v, cudaStream_t s) {
  const size_t n = v.size() * sizeof(T);
  cudaError_t e = b.ensure(std::max<size_t>(n, 16));
  if (e != cudaSuccess || v.empty()) return e;
  if ((e = h.ensure(n)) != cudaSuccess) return e;
  std::memcpy(h.p, v.data(), n);
  return cudaMemcpyAsync(b.p, h.p, n, cudaMemcpyHostToDevice, s);
}

template <typename T>
static cudaError_t upload(DBuf& b, const std::vector<T>& v, cudaStream_t s) {
  cudaError_t e = b.ensure(std::max<size_t>(v.size() * sizeof(T), 16));
  if (e != cudaSuccess || v.empty()) return e;
  return cudaMemcpyAsync(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s);
}

struct StencilSet {
  int kind = 0;  // 0 none, 1 arcs, 2 patches
  std::vector<ArcDev> arcs;
  std::vector<double> arc_theta;
  std::vector<int> arc_gid_off;  // per arc: offset into arc_gids
  std::vector<int> arc_gids;
  std::vector<PatchDev> patches;
  std::vector<double> patch_nodes;
  std::vector<int> patch_gids;
  std::vector<unsigned short> knn_tab;  // window tables (PatchDev::knn_off)
  long long ipsi_total = 0, ainv_total = 0;
  int nmax = 0;
  DBuf d_arcs, d_theta, d_ipsi, d_patches, d_nodes, d_ainv, d_knn;
  DBuf d_e32, d_emax;  // patches: A^-1 - I in FP32 and its max |.| per patch
  std::vector<float> emax;  // host copy of d_emax
  bool uploaded = false;
  int size_of(int s) const { return kind == 1 ? arcs[s].n : patches[s].m; }
  long long acc_of(int s) const {
    return kind == 1 ? arcs[s].n : static_cast<long long>(patches[s].nwin) * patches[s].k;
  }
};

// device copies of a disk batch
struct DiskBufs {
  DBuf disks, tab, pth, ixy, idisk, irow, cpos;
  bool uploaded = false;
};

struct Mesh {
  HostMesh host;
  int disk_radial = 0;   // fk_mesh_set_disk_solver
  DiskBatch disk;
  DiskBufs dbufs;
  StencilSet st;
  std::vector<long long> g_off;  // per item
  long long g_total = 0;
  std::vector<int> csr_idx;      // per item entry
  std::vector<int> rows;         // per item
  DBuf d_val0, d_csr_idx, d_g_off, d_row;
  bool uploaded = false;
  // adaptive assembly (fk_assembly_*): running per-item row sums and
  // statistics on the device, paths and BVP per item on the host
  DBuf r_gsum, r_stats, r_var;
  std::vector<unsigned long long> r_paths;
  std::vector<fk::ItemDev> r_items;  // the rounds' solve records (only paths and BVP change between rounds)
  std::vector<fk::ItemDev> a_items;  // fk_assemble's solve records (only h and paths change between calls)
  double r_items_h = 0.0;
  std::vector<int> r_bvp;
  double r_h = 0.0;
  bool r_active = false;
};

}  // namespace fk

struct fk_ctx {
  int device = 0;
  unsigned long long seed = 0;
  unsigned stream_id = 0;
  int max_steps = 1 << 24;
  unsigned long long slot_wait_ns = 0, barrier_ns = 0;  // fk_set_wait_limits (0: defaults)
  int block = 256, chunk = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  double timing[3] = {0, 0, 0};
  size_t acc_clean = 0;
  long long last_windows = 0;  // windows formed into G rows by the last solve (fk_last_windows)  // bytes at the start of w_acc known to be zero (left so by warp-mode fused launches)
  std::string err;
  std::vector<fk::BvpDev> bvps;
  fk::DBuf d_bvps;
  fk::StencilSet arcs;   // arcs registered with fk_register_arc
  std::vector<std::unique_ptr<fk::Mesh>> meshes;
  std::vector<std::unique_ptr<fk::Mlp>> mlps;
  // workspace
  fk::DBuf w_items, w_chunks, w_stats, w_acc, w_queue, w_gout, w_bout, w_sout, w_val, w_B, w_goff, w_row, w_tmp;
  fk::DBuf w_dgrid, w_dcbar, w_dvar, w_dminv, w_dz, w_dG, w_dB, w_dflags;
  fk::DiskBufs w_disk;
  fk::HBuf h_items, h_chunks, h_goff, h_stats, h_queue;  // pinned staging of the per-call transfers
  std::vector<fk::ItemDev> tmp_items;            // host scratch kept across calls
  std::vector<fk::ChunkDev> tmp_chunks, tmp_chunks2;
  std::vector<unsigned> tmp_count;
};

namespace {

// shared memory per CTA of warp mode with per-warp moment accumulators (5
// such CTAs fit on an SM)
constexpr size_t kWmsCtaBytes = 45 * 1024;
// items of at most this many paths on average run the path kernel in warp
// mode (on the 8x8 assembly at h = 5e-5 warp mode is 26 % faster at 800 paths
// per item, 4 % at 2000, and 6 % slower at 4000)
constexpr long long kWarpModeMaxPaths = 3072;

int fail(fk_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}
int cuda_fail(fk_ctx* c, cudaError_t e, const char* where) {
  return fail(c, FK_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}
#define FK_CUDA(call)                                      \
  do {                                                     \
    cudaError_t e_ = (call);                               \
    if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
  } while (0)

bool is_device_ptr(const void* p) {
  if (!p) return false;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

// copy n bytes from device workspace to a user pointer (host or device)
cudaError_t copy_out(void* dst, const void* src, size_t n, cudaStream_t s) {
  if (!dst || n == 0) return cudaSuccess;
  return cudaMemcpyAsync(dst, src, n, is_device_ptr(dst) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s);
}

int need_device(fk_ctx* ctx) {
  if (ctx->device < 0) return fail(ctx, FK_ERR_NO_DEVICE, "host-only context (device -1) cannot solve");
  cudaSetDevice(ctx->device);
  return FK_OK;
}

int upload_stencils(fk_ctx* ctx, fk::StencilSet& S, const std::vector<char>* have_ipsi,
                    const std::vector<double>* host_ipsi);

int check_bvp(fk_ctx* ctx, int bvp_id) {
  if (bvp_id < 0 || bvp_id >= static_cast<int>(ctx->bvps.size())) return fail(ctx, FK_ERR_REGISTRY, "unknown bvp id");
  return FK_OK;
}

// Uploads a stencil set and computes its FP64 inverses on the GPU.
int upload_stencils(fk_ctx* ctx, fk::StencilSet& S, const std::vector<char>* have_ipsi,
                    const std::vector<double>* host_ipsi) {
  cudaStream_t s = ctx->stream;
  if (S.kind == 1) {
    FK_CUDA(fk::upload(S.d_arcs, S.arcs, s));
    FK_CUDA(fk::upload(S.d_theta, S.arc_theta, s));
    FK_CUDA(S.d_ipsi.ensure(std::max<long long>(S.ipsi_total, 1) * sizeof(double)));
    const int n_arcs = static_cast<int>(S.arcs.size());
    if (n_arcs > 0) {
      FK_CUDA(ctx->w_tmp.ensure(std::max<long long>(S.ipsi_total, 1) * sizeof(double)));
      FK_CUDA(fk::launch_build_psi(S.d_arcs.as<fk::ArcDev>(), S.d_theta.as<double>(), n_arcs,
                                   ctx->w_tmp.as<double>(), s));
      std::vector<int> ns;
      std::vector<long long> offs;
      for (int a = 0; a < n_arcs; ++a)
        if (!have_ipsi || !(*have_ipsi)[a]) { ns.push_back(S.arcs[a].n); offs.push_back(S.arcs[a].ipsi_off); }
      if (!ns.empty()) {
        fk::DBuf dn, doff;
        FK_CUDA(fk::upload(dn, ns, s));
        FK_CUDA(fk::upload(doff, offs, s));
        FK_CUDA(fk::launch_inverse(ctx->w_tmp.as<double>(), S.d_ipsi.as<double>(), dn.as<int>(), doff.as<long long>(),
                                   S.nmax, static_cast<int>(ns.size()), s));
        FK_CUDA(cudaStreamSynchronize(s));
      }
      if (have_ipsi && host_ipsi) {
        for (int a = 0; a < n_arcs; ++a)
          if ((*have_ipsi)[a])
            FK_CUDA(cudaMemcpyAsync(S.d_ipsi.as<double>() + S.arcs[a].ipsi_off, host_ipsi->data() + S.arcs[a].ipsi_off,
                                    sizeof(double) * S.arcs[a].n * S.arcs[a].n, cudaMemcpyHostToDevice, s));
      }
    }
  } else if (S.kind == 2) {
    FK_CUDA(fk::upload(S.d_patches, S.patches, s));
    FK_CUDA(fk::upload(S.d_nodes, S.patch_nodes, s));
    FK_CUDA(fk::upload(S.d_knn, S.knn_tab, s));
    FK_CUDA(S.d_ainv.ensure(std::max<long long>(S.ainv_total, 1) * sizeof(double)));
    const int n_p = static_cast<int>(S.patches.size());
    std::vector<long long> win_base(n_p + 1, 0);
    for (int p = 0; p < n_p; ++p) win_base[p + 1] = win_base[p] + S.patches[p].nwin;
    const long long total = win_base[n_p];
    if (total > 0) {
      const int k = S.patches[0].k;
      fk::DBuf dwb;
      FK_CUDA(fk::upload(dwb, win_base, s));
      FK_CUDA(ctx->w_tmp.ensure(std::max<long long>(S.ainv_total, 1) * sizeof(double)));
      FK_CUDA(fk::launch_build_windows(S.d_patches.as<fk::PatchDev>(), S.d_nodes.as<double>(), n_p,
                                       dwb.as<long long>(), total, k, ctx->w_tmp.as<double>(), s));
      std::vector<int> ns(total, k);
      std::vector<long long> offs(total);
      for (long long w = 0; w < total; ++w) offs[w] = w * k * k;  // windows are contiguous in pool order
      fk::DBuf dn, doff;
      FK_CUDA(fk::upload(dn, ns, s));
      FK_CUDA(fk::upload(doff, offs, s));
      FK_CUDA(fk::launch_inverse(ctx->w_tmp.as<double>(), S.d_ainv.as<double>(), dn.as<int>(), doff.as<long long>(), k,
                                 static_cast<int>(total), s));
      FK_CUDA(S.d_e32.ensure(std::max<long long>(S.ainv_total, 1) * sizeof(float)));
      FK_CUDA(S.d_emax.ensure(std::max(n_p, 1) * sizeof(float)));
      FK_CUDA(fk::launch_split_inverse(S.d_patches.as<fk::PatchDev>(), n_p, S.d_ainv.as<double>(), S.d_e32.as<float>(),
                                       S.d_emax.as<float>(), s));
      S.emax.assign(n_p, 0.f);
      FK_CUDA(cudaMemcpyAsync(S.emax.data(), S.d_emax.p, n_p * sizeof(float), cudaMemcpyDeviceToHost, s));
      FK_CUDA(cudaStreamSynchronize(s));
    }
  }
  S.uploaded = true;
  return FK_OK;
}

void add_arc(fk::StencilSet& S, const fk::MeshStencil& M, const int* gids_override) {
  fk::ArcDev a;
  a.cx = M.cx; a.cy = M.cy; a.c2 = M.c2; a.radius = M.radius; a.interior = M.interior;
  a.n = static_cast<int>(M.nodes.size());
  a.theta_off = static_cast<long long>(S.arc_theta.size());
  a.ipsi_off = S.ipsi_total;
  S.ipsi_total += static_cast<long long>(a.n) * a.n;
  S.nmax = std::max(S.nmax, a.n);
  S.arc_gid_off.push_back(static_cast<int>(S.arc_gids.size()));
  for (int i = 0; i < a.n; ++i) {
    S.arc_theta.push_back(M.nodes[i].theta);
    S.arc_gids.push_back(gids_override ? gids_override[i] : M.nodes[i].gid);
  }
  S.arcs.push_back(a);
}

// Largest chain offset |d| between an exit's nearest node and a node within
// the weight cutoff rcut of the exit (a bound).  The exit e lies on the patch
// boundary within d_en of its nearest node n (half a side step, or the gap
// between a side's end node and the corner); consecutive chain nodes are at
// least s_min apart, so the boundary path from e to the node d places away is
// at least |d| s_min - d_en long.  On one side or two adjacent sides of a
// rectangle the straight distance is at least that path / sqrt 2 (nodes of the
// opposite side are beyond the cutoff wherever a walk is used), so a node
// within rcut has |d| < (sqrt 2 rcut + d_en) / s_min.
int patch_span_bound(const fk::MeshStencil& M, double rcut) {
  const int m = static_cast<int>(M.nodes.size());
  if (m < 2) return 1 << 20;
  double s_min = 1e300, d_en = 0.0;
  for (int i = 0; i + 1 < m + (M.closed ? 1 : 0); ++i) {
    const fk::MeshNode& a = M.nodes[i];
    const fk::MeshNode& b = M.nodes[(i + 1) % m];
    s_min = std::min(s_min, std::hypot(b.x - a.x, b.y - a.y));
  }
  for (int s = 0; s < 4; ++s) {
    const int c = M.side_count[s];
    if (c <= 0) continue;
    const int ax = M.side_axis[s];  // the coordinate that varies along the side
    const double lo = ax == 0 ? M.rect[0] : M.rect[1], hi = ax == 0 ? M.rect[2] : M.rect[3];
    double cmin = 1e300, cmax = -1e300;
    for (int i = 0; i < c; ++i) {
      const fk::MeshNode& nd = M.nodes[M.side_first[s] + i];
      const double v = ax == 0 ? nd.x : nd.y;
      cmin = std::min(cmin, v);
      cmax = std::max(cmax, v);
    }
    d_en = std::max(d_en, std::max(0.5 * std::fabs(M.side_step[s]), std::max(cmin - lo, hi - cmax)));
  }
  if (!(s_min > 0.0)) return 1 << 20;
  return static_cast<int>(std::floor((std::sqrt(2.0) * rcut + d_en) / s_min));
}

// The k-window start of a point on the patch boundary by the path kernel's
// sliding search (knn_window in fk_paths_kernel.cuh), in FP64.
int knn_window_host(const fk::MeshStencil& M, int k, double ex, double ey) {
  const int m = static_cast<int>(M.nodes.size());
  int best_s = -1;
  double best = 1e300;
  for (int s = 0; s < 4; ++s) {
    if (M.side_count[s] > 0) {
      const double dist = std::fabs((M.side_axis[s] == 0 ? ey : ex) - M.side_fixed[s]);
      if (dist < best) { best = dist; best_s = s; }
    }
  }
  int nearest = 0;
  if (best_s >= 0) {
    const double coord = M.side_axis[best_s] == 0 ? ex : ey;
    int j = static_cast<int>(std::rint((coord - M.side_start[best_s]) * (1.0 / M.side_step[best_s])));
    j = std::max(0, std::min(M.side_count[best_s] - 1, j));
    nearest = M.side_first[best_s] + j;
  }
  auto d2 = [&](int idx) {
    if (idx >= m) idx -= m;
    if (idx < 0) idx += m;
    const double dx = ex - M.nodes[idx].x, dy = ey - M.nodes[idx].y;
    return dx * dx + dy * dy;
  };
  int L = nearest - k / 2;
  if (M.closed) {
    if (L < 0) L += m;
    for (int it = 0; it < m && d2(L - 1) < d2(L + k - 1); ++it) { --L; if (L < 0) L += m; }
    for (int it = 0; it < m && d2(L + k) < d2(L); ++it) { ++L; if (L >= m) L -= m; }
  } else {
    L = std::max(0, std::min(m - k, L));
    while (L > 0 && d2(L - 1) < d2(L + k - 1)) --L;
    while (L < m - k && d2(L + k) < d2(L)) ++L;
  }
  return L;
}

// Window table of a patch: for each side, the window start at kKnnBins bins
// per side step over the side's whole extent (corner to corner).  Along the
// boundary the k-window moves monotonically with the exit point, so a bin
// whose two ends (and middle) have windows L0 and L0 or L0 + 1 holds only
// those two: the path kernel picks L0 + 1 iff node L0 + k is nearer than node
// L0, the sliding search's own step.  Other bins are marked kKnnFull.
void add_knn_table(fk::StencilSet& S, fk::PatchDev& p, const fk::MeshStencil& M, int k) {
  const int m = static_cast<int>(M.nodes.size());
  p.knn_off = static_cast<long long>(S.knn_tab.size());
  int base = 0;
  for (int s = 0; s < 4; ++s) {
    p.knn_base[s] = base;
    p.knn_n[s] = 0;
    p.knn_u0[s] = 0.0;
    const int c = M.side_count[s];
    if (c <= 0 || !(M.side_step[s] != 0.0) || m < k) continue;
    const int ax = M.side_axis[s];
    const double lo = ax == 0 ? M.rect[0] : M.rect[1], hi = ax == 0 ? M.rect[2] : M.rect[3];
    const double ua = (lo - M.side_start[s]) / M.side_step[s], ub = (hi - M.side_start[s]) / M.side_step[s];
    const double u0 = std::min(ua, ub), u1 = std::max(ua, ub);
    const int nb = std::max(1, static_cast<int>(std::ceil((u1 - u0) * fk::kKnnBins)));
    auto point_at = [&](double u, double& x, double& y) {
      const double along = M.side_start[s] + u * M.side_step[s];
      x = ax == 0 ? along : M.side_fixed[s];
      y = ax == 0 ? M.side_fixed[s] : along;
    };
    auto win_at = [&](double u) {
      double x, y;
      point_at(u, x, y);
      return knn_window_host(M, k, x, y);
    };
    int left = win_at(u0);
    for (int b = 0; b < nb; ++b) {
      const int right = win_at(u0 + static_cast<double>(b + 1) / fk::kKnnBins);
      const int mid = win_at(u0 + (b + 0.5) / fk::kKnnBins);
      int step = right - left;
      if (M.closed && step < 0) step += m;
      int smid = mid - left;
      if (M.closed && smid < 0) smid += m;
      const bool ok = (step == 0 || step == 1) && (smid == 0 || smid == step) && left < 0x4000;
      S.knn_tab.push_back(ok ? static_cast<unsigned short>(left) : fk::kKnnFull);
      left = right;
    }
    p.knn_n[s] = nb;
    p.knn_u0[s] = u0;
    base += nb;
  }
}

void add_patch(fk::StencilSet& S, const fk::MeshStencil& M, int k, double eps) {
  fk::PatchDev p;
  std::memset(&p, 0, sizeof(p));
  for (int i = 0; i < 4; ++i) {
    p.rect[i] = M.rect[i];
    p.side_first[i] = M.side_first[i]; p.side_count[i] = M.side_count[i]; p.side_axis[i] = M.side_axis[i];
    p.side_fixed[i] = M.side_fixed[i]; p.side_start[i] = M.side_start[i]; p.side_step[i] = M.side_step[i];
  }
  p.eps2 = eps * eps;
  p.m = static_cast<int>(M.nodes.size());
  p.k = k;
  p.closed = M.closed ? 1 : 0;
  p.nwin = p.closed ? p.m : p.m - k + 1;
  // Along the chain, the distance from an exit point (projected onto a side)
  // grows monotonically over its own side and the two adjacent ones; nodes of
  // the opposite side lie at least the patch width W away.  When those are
  // always beyond the weight cutoff, a walk outward from the exit may stop
  // at its first cut node (0.9 W leaves a margin for rounding).
  const double W = 0.9 * std::min(M.rect[2] - M.rect[0], M.rect[3] - M.rect[1]);
  auto walk_mode = [&](double cut, int span_max) {
    if (p.eps2 * W * W < cut) return fk::kWalkFull;
    return patch_span_bound(M, std::sqrt(cut / p.eps2)) <= span_max ? fk::kWalkSpan : fk::kWalkStop;
  };
  p.walk = walk_mode(static_cast<double>(fk::kPhiCut), fk::kSpanMax);
  p.walk32 = walk_mode(static_cast<double>(fk::kPhiCut32), fk::kSpanMax32);
  p.node_off = static_cast<long long>(S.patch_nodes.size());
  p.ainv_off = S.ainv_total;
  S.ainv_total += static_cast<long long>(p.nwin) * k * k;
  for (const fk::MeshNode& nd : M.nodes) {
    S.patch_nodes.push_back(nd.x);
    S.patch_nodes.push_back(nd.y);
    S.patch_gids.push_back(nd.gid);
  }
  S.nmax = std::max(S.nmax, p.m);
  add_knn_table(S, p, M, k);
  S.patches.push_back(p);
}

// Options of run_items.
struct RunOpts {
  bool multi_bvp = false;    // items carry their own BVP index (one problem functor)
  bool need_item_G = true;   // the per-item G rows are wanted (else only the CSR values get them)
  // Adaptive assembly round (fk_assembly_round): the chunks' G rows are added
  // to g_sum (slot mode, fused rows), the call's statistics to run_stats,
  // each item's per-path variance goes to item_var (device, may be null), and
  // no finalize runs.
  double* g_sum = nullptr;
  double* run_stats = nullptr;
  double* item_var = nullptr;
  bool defer = false;  // queue the launch and leave the stream synchronisation and the checks to finish_run
};

// Runs items through the path kernel and the finalize kernel.
struct RunOut {
  double* item_G = nullptr;       // device workspace results
  double* item_B = nullptr;
  double* item_stats = nullptr;
  bool capped = false;
  // RunOpts::defer: the launch is queued with its check words copied to
  // pinned memory; finish_run, after the caller's own stream synchronisation,
  // reads them (one synchronisation for the whole call)
  bool deferred = false;
  int kernels = 0;
  size_t acc_clean_after = 0;
};

// The completed-paths check failed: the first item the finalize kernel
// found (q[5] - 1) and the paths it completed (q[6]).
int fail_lost(fk_ctx* ctx, const int* q) {
  char msg[160];
  std::snprintf(msg, sizeof(msg), "path kernel: an item completed a different number of paths than requested "
                "(item %d: %d completed)", q[5] - 1, q[6]);
  return fail(ctx, FK_ERR_CUDA, msg);
}

// The kernels' own checks of a queued launch (slot waits, completed paths,
// capped paths) and its timing, once its stream has drained.
int finish_run(fk_ctx* ctx, RunOut& out) {
  if (!out.deferred) return FK_OK;
  out.deferred = false;
  float t0 = 0, t1 = 0;
  cudaEventElapsedTime(&t0, ctx->ev[0], ctx->ev[1]);
  cudaEventElapsedTime(&t1, ctx->ev[1], ctx->ev[2]);
  ctx->timing[0] = t0;
  ctx->timing[1] = t1;
  ctx->timing[2] = out.kernels;
  const int* q = static_cast<const int*>(ctx->h_queue.p);
  ctx->last_windows = q[4];
  if (q[1] != 0) return fail(ctx, FK_ERR_CUDA, "path kernel: a wait for a chunk slot timed out");
  if (q[3] != 0) return fail_lost(ctx, q);
  out.capped = q[2] != 0;
  ctx->acc_clean = out.acc_clean_after;  // every warp zeroed the moments it used
  return FK_OK;
}

int run_items(fk_ctx* ctx, int bvp_id, int precision, std::vector<fk::ItemDev>& it, fk::StencilSet* S,
              const std::vector<long long>* g_off, long long g_total, const int* d_csr_idx, double* d_csr_val,
              const int* d_row, double* d_B, RunOut& out, const RunOpts& o = RunOpts()) {
  // o.multi_bvp: items carry their own BVP index (same functor as bvp_id,
  // whose control mode and network the launch takes); otherwise every item
  // uses bvp_id
  const bool multi_bvp = o.multi_bvp, need_item_G = o.need_item_G;
  const bool round = o.g_sum != nullptr;
  cudaStream_t s = ctx->stream;
  const int n = static_cast<int>(it.size());
  const int kind = S ? S->kind : 0;
  const fk::BvpDev& bvp = ctx->bvps[bvp_id];
  if (precision != FK_FP64 && precision != FK_FP32) return fail(ctx, FK_ERR_ARG, "precision must be FK_FP64 or FK_FP32");
  // per-item stencil accumulator offsets (set in the caller's item vector)
  long long acc_total = 0;
  int acc_words = 0;
  // learned control variate: one network region per stencil, or region 0
  int n_stencils = 0;
  if (S) n_stencils = static_cast<int>(S->kind == 1 ? S->arcs.size() : S->patches.size());
  const bool per_stencil = bvp.cv == FK_CV_MLP && n_stencils > 0 && ctx->mlps[bvp.mlp]->n_regions == n_stencils;
  // one pass over the items: accumulator offsets, control variates, path
  // totals, the largest stencil and the live items
  bool any_cv = false;  // some item has a control variate: the kernel build with the xi terms
  long long total_paths = 0, n_live = 0;
  int smem_nodes = 0;
  const int n_bvps = static_cast<int>(ctx->bvps.size());
  for (auto& x : it) {
    if (!multi_bvp) x.bvp = bvp_id;
    if (x.bvp >= 0 && x.bvp < n_bvps && ctx->bvps[x.bvp].cv != FK_CV_NONE) any_cv = true;
    x.cv_region = (per_stencil && x.stencil >= 0) ? x.stencil : 0;
    x.acc_off = acc_total;
    if (kind != 0 && x.stencil >= 0) {
      const long long w = S->acc_of(x.stencil);
      acc_total += w;
      acc_words = std::max<int>(acc_words, static_cast<int>(w));
      smem_nodes = std::max(smem_nodes, S->size_of(x.stencil));
    }
    if (!x.frontera) total_paths += x.paths;
    if (!x.frontera && x.paths > 0) ++n_live;
  }
  // chunks: balance the persistent grid
  const int block = ctx->block;
  // Items of few paths (on average at most kWarpModeMaxPaths) run in warp
  // mode: every warp takes its own chunks and adds the stencil moments to
  // global memory, so an item's slowest path holds up one warp only.  A
  // launch shape set by the caller (fk_set_launch, the autotuner) keeps the
  // shared chunk slots.
  bool warp_mode = ctx->chunk <= 0 && n_live > 0 && total_paths <= kWarpModeMaxPaths * n_live;
  // Adaptive rounds with items of few paths: warp mode with per-warp FP32
  // moment accumulators in shared memory, so that the kernel forms the G rows
  // (the rounds keep no moments in global memory).  CTAs of 4 warps (2 for
  // large patches).  The accumulators and exit queues bound such a launch to
  // about 12 warps per SM: on the 8 x 8 assembly at 870 paths per item the
  // plain warp mode with global FP64 moments and the finalize kernel measured
  // 5.9 ms against 7.9 ms, so CSR assemblies keep it.
  int lblock = block;
  bool wms = false;
  if (warp_mode && kind == 2 && precision == FK_FP32 && round) {
    const size_t P = fk::paths_slot_bytes(precision, kind, acc_words, smem_nodes);
    const int wpb = 4 * P <= kWmsCtaBytes ? 4 : (2 * P <= kWmsCtaBytes ? 2 : 0);
    if (wpb) {
      wms = true;
      lblock = 32 * wpb;
    }
  }
  if (round && warp_mode && !wms) warp_mode = false;  // (rounds need rows formed in the kernel)
  const size_t sacc_bytes = fk::paths_smem_bytes(precision, kind, acc_words, smem_nodes, warp_mode, lblock, wms);
  if (sacc_bytes > 200 * 1024) return fail(ctx, FK_ERR_CAPACITY, "stencil accumulators exceed shared memory");
  const int occ = fk::paths_kernel_occupancy(bvp.problem, precision, kind, any_cv ? 1 : 0, lblock, sacc_bytes, warp_mode);
  const int grid = std::max(1, ctx->num_sms * occ);
  const int block_used = lblock;
  // Chunk size.  Slots: at least 4 chunks per CTA of the persistent grid, at
  // most 32768 paths.  Warp mode: about 2 chunks per warp, 64..4096 paths
  // (measured on the 8x8 assembly and on point solves, finer chunks cost
  // more in per-chunk work than they save in the last round).  An item is
  // split into equal chunks (no small remainder).
  long long chunk = ctx->chunk;
  if (chunk <= 0 && warp_mode) {
    chunk = total_paths / (2LL * grid * (block_used / 32));
    chunk = std::max<long long>(64, std::min<long long>(chunk, 4096));
  } else if (chunk <= 0) {
    chunk = total_paths / (4LL * grid);
    chunk = std::max<long long>(block_used, std::min<long long>(chunk, 32768));
  }
  std::vector<fk::ChunkDev>& chunks = ctx->tmp_chunks;  // (reused: no page faults per call)
  chunks.clear();
  for (int i = 0; i < n; ++i) {
    if (it[i].frontera || it[i].paths == 0) continue;
    const long long np = it[i].paths;
    const long long pieces = (np + chunk - 1) / chunk;
    const long long per = (np + pieces - 1) / pieces;
    for (long long p0 = 0; p0 < np; p0 += per) {
      const long long p1 = std::min<long long>(np, p0 + per);
      chunks.push_back(fk::ChunkDev{i, static_cast<unsigned>(p0), static_cast<unsigned>(p1)});
    }
  }
  // longest chunks first (uneven path counts, as in batched solves)
  bool uneven = false;
  for (size_t c = 1; c < chunks.size() && !uneven; ++c)
    uneven = (chunks[c].p1 - chunks[c].p0) != (chunks[0].p1 - chunks[0].p0);
  if (uneven) {
    // stable, by descending length: a counting sort (lengths are at most the
    // chunk size), the order std::stable_sort gives, in linear time
    unsigned maxlen = 0;
    for (const fk::ChunkDev& c : chunks) maxlen = std::max(maxlen, c.p1 - c.p0);
    if (maxlen <= (1u << 16)) {
      std::vector<unsigned>& start = ctx->tmp_count;
      start.assign(maxlen + 2, 0u);
      for (const fk::ChunkDev& c : chunks) ++start[maxlen - (c.p1 - c.p0) + 1];
      for (unsigned l = 1; l <= maxlen + 1; ++l) start[l] += start[l - 1];
      std::vector<fk::ChunkDev>& sorted = ctx->tmp_chunks2;
      sorted.resize(chunks.size());
      for (const fk::ChunkDev& c : chunks) sorted[start[maxlen - (c.p1 - c.p0)]++] = c;
      chunks.swap(sorted);
    } else {
      std::stable_sort(chunks.begin(), chunks.end(),
                       [](const fk::ChunkDev& a, const fk::ChunkDev& b) { return (a.p1 - a.p0) > (b.p1 - b.p0); });
    }
  }
  FK_CUDA(fk::upload_pinned(ctx->w_items, ctx->h_items, it, s));
  FK_CUDA(fk::upload_pinned(ctx->w_chunks, ctx->h_chunks, chunks, s));
  FK_CUDA(ctx->w_stats.ensure(std::max<size_t>(static_cast<size_t>(n) * fk::kNumStats * sizeof(double), 16)));
  FK_CUDA(cudaMemsetAsync(ctx->w_stats.p, 0, static_cast<size_t>(n) * fk::kNumStats * sizeof(double), s));
  // slot mode with every item in one chunk: the chunks store their moments,
  // so the accumulators need no zeroing
  bool all_whole = true;
  for (const fk::ChunkDev& c : chunks)
    if (c.p0 != 0 || c.p1 != it[c.item].paths) { all_whole = false; break; }
  bool whole_items = !warp_mode && all_whole;
  // Warp mode with FP32 patch stencils (k = 20, window corrections in FP32)
  // and whole items into the CSR values: each warp forms its item's G row
  // from the item's global moments and zeroes them again (wfuse).
  bool wfuse = warp_mode && !wms && !round && precision == FK_FP32 && kind == 2 && all_whole && g_off && d_csr_idx &&
               d_csr_val && !chunks.empty();
  if (wfuse) {
    for (const fk::PatchDev& P : S->patches) wfuse = wfuse && P.k == 20;
    for (float e : S->emax) wfuse = wfuse && e < fk::kSplitMaxE;
  }
  const size_t acc_need = static_cast<size_t>(acc_total) * sizeof(double);
  if (round || wms) {
    whole_items = false;  // (the rows are formed in the kernel: no moment accumulators in global memory)
  } else {
    void* before = ctx->w_acc.p;
    FK_CUDA(ctx->w_acc.ensure(std::max<size_t>(acc_need, 16)));
    if (ctx->w_acc.p != before) ctx->acc_clean = 0;
    if (acc_total > 0 && !whole_items && !(wfuse && ctx->acc_clean >= acc_need)) {
      FK_CUDA(cudaMemsetAsync(ctx->w_acc.p, 0, acc_need, s));
      ctx->acc_clean = std::max(ctx->acc_clean, acc_need);
    }
  }
  // (until this launch has finished without error, nothing is known to be zero)
  const size_t acc_clean_after = wfuse ? ctx->acc_clean : 0;
  if (!(round || wms)) ctx->acc_clean = 0;
  FK_CUDA(ctx->w_queue.ensure(32));
  // queue, error word, result flags, windows formed into rows, the first item
  // whose completed path count differs and that count
  FK_CUDA(cudaMemsetAsync(ctx->w_queue.p, 0, 7 * sizeof(int), s));

  fk::LaunchArgs a;
  std::memset(&a, 0, sizeof(a));
  a.acc_zeroed = whole_items ? 0 : 1;
  a.bvp = ctx->d_bvps.as<fk::BvpDev>();
  a.items = ctx->w_items.as<fk::ItemDev>();
  a.chunks = ctx->w_chunks.as<fk::ChunkDev>();
  a.n_chunks = static_cast<int>(chunks.size());
  if (kind == 1) { a.arcs = S->d_arcs.as<fk::ArcDev>(); a.arc_theta = S->d_theta.as<double>(); }
  if (kind == 2) {
    a.patches = S->d_patches.as<fk::PatchDev>();
    a.patch_nodes = S->d_nodes.as<double>();
    a.knn_tab = S->d_knn.as<unsigned short>();
  }
  a.queue = ctx->w_queue.as<int>();
  a.vis_count = ctx->w_queue.as<int>() + 4;
  a.stats = ctx->w_stats.as<double>();
  a.acc = round ? nullptr : ctx->w_acc.as<double>();
  a.key0 = static_cast<uint32_t>(ctx->seed);
  a.key1 = static_cast<uint32_t>(ctx->seed >> 32);
  fk::set_round_keys(a);
  a.stream = ctx->stream_id;
  a.max_steps = ctx->max_steps;
  a.wait_limit_ns = ctx->slot_wait_ns;
  a.cv = (bvp.cv == FK_CV_EXACT) ? 1 : 0;
  a.any_cv = any_cv ? 1 : 0;
  if (bvp.cv == FK_CV_MLP) {
    const fk::Mlp& M = *ctx->mlps[bvp.mlp];
    if (M.table_grid < 2 || !M.d_table) return fail(ctx, FK_ERR_ARG, "learned control variate: build its table first");
    a.cv = 2;
    a.cv_tab = M.d_table;
    a.cv_rect = M.d_rect;
    a.cv_grid = M.table_grid;
    a.cv_tex = M.d_tex;
  }
  a.stencil_kind = kind;
  a.acc_words = acc_words;
  a.smem_nodes = smem_nodes;
  // per-item G buffers
  FK_CUDA(ctx->w_gout.ensure(std::max<size_t>(g_total * sizeof(double), 16)));
  if (g_off) FK_CUDA(fk::upload_pinned(ctx->w_goff, ctx->h_goff, *g_off, s));
  double* item_G = (kind && need_item_G) ? ctx->w_gout.as<double>() : nullptr;
  // G rows in the path kernel's flush: FP32 patch stencils whose chunks are
  // whole items and whose window corrections are small enough for FP32
  const bool fuse = (precision == FK_FP32 && kind == 2 && all_whole && (wms || !warp_mode) && g_off && d_csr_idx &&
                     d_csr_val && !chunks.empty()) || wfuse;
  if (round && !(kind == 2 && g_off)) return fail(ctx, FK_ERR_ARG, "adaptive rounds need a square-patch mesh");
  if (fuse || round) {
    a.fuse_g = round ? 2 : 1;
    a.wm_shared = wms ? 1 : 0;
    // FP32 moments with small window corrections: I + E_W in FP32; otherwise the FP64 inverses
    bool e32 = precision == FK_FP32;
    for (float e : S->emax) e32 = e32 && e < fk::kSplitMaxE;
    a.patch_e32 = e32 ? S->d_e32.as<float>() : nullptr;
    a.patch_ainv = S->d_ainv.as<double>();
    a.g_off = ctx->w_goff.as<long long>();
    a.csr_idx = d_csr_idx;
    a.csr_val = d_csr_val;
    a.item_G = item_G;
    a.g_sum = o.g_sum;
  }
  FK_CUDA(cudaEventRecord(ctx->ev[0], s));
  if (!chunks.empty())
    FK_CUDA(fk::launch_paths(a, bvp.problem, precision, grid, block_used, sacc_bytes, s, warp_mode));
  FK_CUDA(cudaEventRecord(ctx->ev[1], s));
  if (round) {
    FK_CUDA(fk::launch_round_stats(a.items, n, a.stats, o.run_stats, o.item_var, ctx->w_queue.as<int>() + 2, s));
    FK_CUDA(cudaEventRecord(ctx->ev[2], s));
    FK_CUDA(cudaStreamSynchronize(s));
    float t0 = 0, t1 = 0;
    cudaEventElapsedTime(&t0, ctx->ev[0], ctx->ev[1]);
    cudaEventElapsedTime(&t1, ctx->ev[1], ctx->ev[2]);
    ctx->timing[0] = t0;
    ctx->timing[1] = t1;
    ctx->timing[2] = chunks.empty() ? 1 : 2;
    ctx->stream_id++;
    int q[5] = {0, 0, 0, 0, 0};
    FK_CUDA(cudaMemcpy(q, ctx->w_queue.p, sizeof(q), cudaMemcpyDeviceToHost));
    ctx->last_windows = q[4];
    if (q[1] != 0) return fail(ctx, FK_ERR_CUDA, "path kernel: a wait for a chunk slot timed out");
    if (q[3] != 0) return fail(ctx, FK_ERR_CUDA, "path kernel: an item completed fewer paths than requested");
    out.capped = q[2] != 0;
    return FK_OK;
  }

  // finalize
  FK_CUDA(ctx->w_bout.ensure(std::max<size_t>(n * sizeof(double), 16)));
  FK_CUDA(ctx->w_sout.ensure(std::max<size_t>(static_cast<size_t>(n) * 16 * sizeof(double), 16)));
  fk::FinalizeArgs f;
  std::memset(&f, 0, sizeof(f));
  f.bvp = a.bvp;
  f.items = a.items;
  f.n_items = n;
  if (kind == 1) { f.arcs = a.arcs; f.arc_ipsi = S->d_ipsi.as<double>(); }
  if (kind == 2) {
    f.patches = a.patches;
    f.patch_ainv = S->d_ainv.as<double>();
    f.patch_e32 = S->d_e32.as<float>();
    f.patch_emax = S->d_emax.as<float>();
    f.split_ok = precision == FK_FP32 ? 1 : 0;
    int kcommon = -1;
    for (const fk::PatchDev& P : S->patches) {
      f.fin_words = std::max(f.fin_words, P.nwin * P.k);
      f.fin_m = std::max(f.fin_m, P.m);
      kcommon = (kcommon < 0 || kcommon == P.k) ? P.k : 0;
    }
    f.fin_k = std::max(kcommon, 0);
  }
  f.stats = a.stats;
  f.acc = a.acc;
  f.stencil_kind = kind;
  f.g_off = g_off ? ctx->w_goff.as<long long>() : nullptr;
  f.item_G = item_G;
  f.g_fused = a.fuse_g;
  f.item_B = ctx->w_bout.as<double>();
  f.item_stats = ctx->w_sout.as<double>();
  f.csr_idx = d_csr_idx;
  f.csr_val = d_csr_val;
  f.row = d_row;
  f.B = d_B;
  f.flags = ctx->w_queue.as<int>() + 2;
  f.vis_count = ctx->w_queue.as<int>() + 4;
  f.lost = ctx->w_queue.as<int>() + 5;
  FK_CUDA(fk::launch_finalize(f, bvp.problem, s));
  FK_CUDA(cudaEventRecord(ctx->ev[2], s));
  out.item_G = kind ? ctx->w_gout.as<double>() : nullptr;
  out.item_B = f.item_B;
  out.item_stats = f.item_stats;
  if (o.defer) {
    FK_CUDA(ctx->h_queue.ensure(32));
    FK_CUDA(cudaMemcpyAsync(ctx->h_queue.p, ctx->w_queue.p, 7 * sizeof(int), cudaMemcpyDeviceToHost, s));
    out.deferred = true;
    out.kernels = chunks.empty() ? 1 : 2;
    out.acc_clean_after = acc_clean_after;
    ctx->stream_id++;
    return FK_OK;
  }
  FK_CUDA(cudaStreamSynchronize(s));
  float t0 = 0, t1 = 0;
  cudaEventElapsedTime(&t0, ctx->ev[0], ctx->ev[1]);
  cudaEventElapsedTime(&t1, ctx->ev[1], ctx->ev[2]);
  ctx->timing[0] = t0;
  ctx->timing[1] = t1;
  ctx->timing[2] = chunks.empty() ? 1 : 2;
  ctx->stream_id++;
  // the kernels' own checks: slot waits, completed paths, capped paths
  int q[7] = {0, 0, 0, 0, 0, 0, 0};
  FK_CUDA(cudaMemcpy(q, ctx->w_queue.p, sizeof(q), cudaMemcpyDeviceToHost));
  ctx->last_windows = q[4];
  if (q[1] != 0) return fail(ctx, FK_ERR_CUDA, "path kernel: a wait for a chunk slot timed out");
  if (q[3] != 0) return fail_lost(ctx, q);
  out.capped = q[2] != 0;
  ctx->acc_clean = acc_clean_after;  // every warp zeroed the moments it used
  return FK_OK;
}

}  // namespace

extern "C" {

int fk_create(fk_ctx** out, int device, unsigned long long seed) {
  if (!out) return FK_ERR_ARG;
  *out = nullptr;
  if (device == -1) {  // host-only context: meshes and CSR patterns, no solves
    fk_ctx* ctx = new fk_ctx();
    ctx->device = -1;
    ctx->seed = seed;
    ctx->arcs.kind = 1;
    *out = ctx;
    return FK_OK;
  }
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n <= device || device < 0) {
    cudaGetLastError();
    return FK_ERR_NO_DEVICE;
  }
  fk_ctx* ctx = new fk_ctx();
  ctx->device = device;
  ctx->seed = seed;
  if (cudaSetDevice(device) != cudaSuccess ||
      cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete ctx;
    return FK_ERR_NO_DEVICE;
  }
  for (auto& e : ctx->ev) cudaEventCreate(&e);
  ctx->arcs.kind = 1;
  *out = ctx;
  return FK_OK;
}

int fk_destroy(fk_ctx* ctx) {
  if (!ctx) return FK_ERR_ARG;
  if (ctx->device < 0) {
    delete ctx;
    return FK_OK;
  }
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  for (auto& e : ctx->ev) if (e) cudaEventDestroy(e);
  ctx->meshes.clear();
  ctx->mlps.clear();
  cudaStream_t s = ctx->stream;
  delete ctx;
  if (s) cudaStreamDestroy(s);
  return FK_OK;
}

const char* fk_last_error(const fk_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int fk_set_stream(fk_ctx* ctx, unsigned id) { if (!ctx) return FK_ERR_ARG; ctx->stream_id = id; return FK_OK; }
int fk_get_stream(const fk_ctx* ctx, unsigned* id) { if (!ctx || !id) return FK_ERR_ARG; *id = ctx->stream_id; return FK_OK; }
int fk_set_max_steps(fk_ctx* ctx, int m) {
  if (!ctx || m < 1 || m > (1 << 30)) return fail(ctx, FK_ERR_ARG, "max_steps must be in [1, 2^30]");
  ctx->max_steps = m;
  return FK_OK;
}
int fk_set_wait_limits(fk_ctx* ctx, double slot_wait_s, double barrier_s) {
  if (!ctx) return FK_ERR_ARG;
  if (!(slot_wait_s >= 0 && slot_wait_s <= 1e6 && barrier_s >= 0 && barrier_s <= 1e6))
    return fail(ctx, FK_ERR_ARG, "wait limits must be in [0, 1e6] seconds");
  // (a positive limit below 1 ns becomes 1 ns, not the default)
  auto ns = [](double sec) -> unsigned long long {
    return sec > 0 ? std::max(1ull, static_cast<unsigned long long>(sec * 1e9)) : 0ull;
  };
  ctx->slot_wait_ns = ns(slot_wait_s);
  ctx->barrier_ns = ns(barrier_s);
  return FK_OK;
}

int fk_set_launch(fk_ctx* ctx, int block, int chunk) {
  if (!ctx) return FK_ERR_ARG;
  if (block != 0 && (block < 32 || block > 256 || block % 32)) return fail(ctx, FK_ERR_ARG, "block must be 32..256, multiple of 32");
  if (chunk < 0) return fail(ctx, FK_ERR_ARG, "chunk must be >= 0");
  ctx->block = block ? block : 256;
  ctx->chunk = chunk;
  return FK_OK;
}
int fk_cuda_stream(const fk_ctx* ctx, void** s) { if (!ctx || !s) return FK_ERR_ARG; *s = ctx->stream; return FK_OK; }
int fk_last_windows(const fk_ctx* ctx, long long* windows) {
  if (!ctx || !windows) return FK_ERR_ARG;
  *windows = ctx->last_windows;
  return FK_OK;
}

int fk_last_timing(const fk_ctx* ctx, double out[3]) {
  if (!ctx || !out) return FK_ERR_ARG;
  for (int i = 0; i < 3; ++i) out[i] = ctx->timing[i];
  return FK_OK;
}

int fk_register_bvp(fk_ctx* ctx, const fk_bvp_desc* d, int* id) {
  if (!ctx || !d || !id) return fail(ctx, FK_ERR_ARG, "null argument");
  if (d->problem < 0 || d->problem >= fk::kNumProblems) return fail(ctx, FK_ERR_REGISTRY, "unknown problem functor");
  if (d->cv < FK_CV_NONE || d->cv > FK_CV_MLP) return fail(ctx, FK_ERR_ARG, "unknown control-variate mode");
  const int need_shape = fk::problem_domain_shape(d->problem);
  if (d->dom_shape != need_shape) return fail(ctx, FK_ERR_ARG, "domain shape does not match the problem functor");
  if (d->cv == FK_CV_MLP && (d->mlp_id < 0 || d->mlp_id >= static_cast<int>(ctx->mlps.size())))
    return fail(ctx, FK_ERR_REGISTRY, "unknown mlp id");
  for (int i = 0; i < 4; ++i)
    if (!std::isfinite(d->dom[i]) || !std::isfinite(d->prob[i])) return fail(ctx, FK_ERR_ARG, "non-finite parameters");
  if (d->dom_shape == FK_SHAPE_RECT && !(d->dom[2] > d->dom[0] && d->dom[3] > d->dom[1]))
    return fail(ctx, FK_ERR_ARG, "empty rectangle domain");
  if (d->dom_shape == FK_SHAPE_CIRCLE && !(d->dom[0] > 0)) return fail(ctx, FK_ERR_ARG, "non-positive radius");
  if (d->problem == FK_PROBLEM_ROBIN) {
    const double m = d->prob[0];
    if (!(m >= 0 && m <= 15 && m == std::floor(m))) return fail(ctx, FK_ERR_ARG, "reflecting side mask must be 0..15");
    if (!(d->prob[2] >= 0)) return fail(ctx, FK_ERR_ARG, "rho must be >= 0");
  }
  fk::BvpDev b;
  std::memset(&b, 0, sizeof(b));
  b.problem = d->problem;
  b.cv = d->cv;
  b.dom_shape = d->dom_shape;
  b.mlp = d->mlp_id;
  for (int i = 0; i < 4; ++i) { b.dom[i] = d->dom[i]; b.prob[i] = d->prob[i]; }
  ctx->bvps.push_back(b);
  if (ctx->device >= 0) {
    cudaSetDevice(ctx->device);
    FK_CUDA(fk::upload(ctx->d_bvps, ctx->bvps, ctx->stream));
    FK_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  *id = static_cast<int>(ctx->bvps.size()) - 1;
  return FK_OK;
}

// The device's per-item statistics record is fk_stats itself (16 doubles in
// the struct's field order), so it is copied as it is.
static_assert(sizeof(fk_stats) == 16 * sizeof(double), "fk_stats is the device's per-item record");

// Per-item statistics (device, fk_stats layout) into out[n]: straight into a
// page-locked out, else through the pinned staging buffer; drains the
// context stream.
static int read_stats(fk_ctx* ctx, const double* d_stats, int n, fk_stats* out) {
  const size_t bytes = static_cast<size_t>(n) * sizeof(fk_stats);
  cudaPointerAttributes at;
  bool pinned = false;
  if (cudaPointerGetAttributes(&at, out) == cudaSuccess) pinned = at.type == cudaMemoryTypeHost;
  else cudaGetLastError();
  if (pinned) {
    FK_CUDA(cudaMemcpyAsync(out, d_stats, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    FK_CUDA(cudaStreamSynchronize(ctx->stream));
    return FK_OK;
  }
  FK_CUDA(ctx->h_stats.ensure(std::max<size_t>(bytes, 16)));
  FK_CUDA(cudaMemcpyAsync(ctx->h_stats.p, d_stats, bytes, cudaMemcpyDeviceToHost, ctx->stream));
  FK_CUDA(cudaStreamSynchronize(ctx->stream));
  std::memcpy(out, ctx->h_stats.p, bytes);
  return FK_OK;
}

int fk_solve_points(fk_ctx* ctx, int bvp_id, int n, const double* xy, const unsigned* paths, const double* h,
                    const int* sub_shape, const double* sub_params, int precision, fk_stats* out) {
  if (!ctx) return FK_ERR_ARG;
  if (n < 0 || (n > 0 && (!xy || !paths || !h || !out))) return fail(ctx, FK_ERR_ARG, "null argument");
  int rc = check_bvp(ctx, bvp_id);
  if (rc) return rc;
  if (n == 0) return FK_OK;
  if ((rc = need_device(ctx))) return rc;
  std::vector<fk::ItemDev>& items = ctx->tmp_items;
  items.resize(n);
  for (int i = 0; i < n; ++i) {
    fk::ItemDev& it = items[i];
    std::memset(&it, 0, sizeof(it));
    if (!(h[i] > 0) || !std::isfinite(xy[2 * i]) || !std::isfinite(xy[2 * i + 1]))
      return fail(ctx, FK_ERR_ARG, "point solve: h must be > 0 and coordinates finite");
    it.x = xy[2 * i]; it.y = xy[2 * i + 1]; it.h = h[i]; it.sqrth = std::sqrt(h[i]);
    it.paths = paths[i]; it.stencil = -1; it.frontera = 0;
    it.sub_shape = sub_shape ? sub_shape[i] : -1;
    if (sub_params) for (int q = 0; q < 4; ++q) it.sub[q] = sub_params[4 * i + q];
    if (it.sub_shape > 1) return fail(ctx, FK_ERR_ARG, "unknown subdomain shape");
  }
  RunOut ro;
  RunOpts o;
  o.defer = true;  // one stream synchronisation: read_stats's
  rc = run_items(ctx, bvp_id, precision, items, nullptr, nullptr, 0, nullptr, nullptr, nullptr, nullptr, ro, o);
  if (rc) return rc;
  if ((rc = read_stats(ctx, ro.item_stats, n, out))) return rc;
  if ((rc = finish_run(ctx, ro))) return rc;
  if (ro.capped) return fail(ctx, FK_ERR_STEP_CAP, "paths reached max_steps");
  return FK_OK;
}

// Points of several registered BVPs (one problem functor and control mode) in
// one persistent launch.
static int build_multi(fk_ctx* ctx, int n, const int* bvp_ids, const double* xy, const unsigned* paths,
                       const double* h, double paths_scale, std::vector<fk::ItemDev>& items) {
  items.assign(n, fk::ItemDev());
  const fk::BvpDev& b0 = ctx->bvps[bvp_ids[0]];
  for (int i = 0; i < n; ++i) {
    if (check_bvp(ctx, bvp_ids[i])) return FK_ERR_REGISTRY;
    const fk::BvpDev& b = ctx->bvps[bvp_ids[i]];
    if (b.problem != b0.problem || b.cv != b0.cv || b.mlp != b0.mlp)
      return fail(ctx, FK_ERR_ARG, "one launch needs BVPs of one problem functor and control mode");
    if (!(h[i] > 0) || !std::isfinite(xy[2 * i]) || !std::isfinite(xy[2 * i + 1]))
      return fail(ctx, FK_ERR_ARG, "point solve: h must be > 0 and coordinates finite");
    fk::ItemDev& it = items[i];
    std::memset(&it, 0, sizeof(it));
    it.x = xy[2 * i]; it.y = xy[2 * i + 1]; it.h = h[i]; it.sqrth = std::sqrt(h[i]);
    it.paths = std::max(1u, static_cast<unsigned>(std::ceil(paths[i] * paths_scale)));
    it.stencil = -1; it.sub_shape = -1; it.bvp = bvp_ids[i];
  }
  return FK_OK;
}

int fk_solve_points_multi(fk_ctx* ctx, int n, const int* bvp_ids, const double* xy, const unsigned* paths,
                          const double* h, int precision, fk_stats* out) {
  if (!ctx) return FK_ERR_ARG;
  if (n < 0 || (n > 0 && (!bvp_ids || !xy || !paths || !h || !out))) return fail(ctx, FK_ERR_ARG, "null argument");
  if (n == 0) return FK_OK;
  int rc = need_device(ctx);
  if (rc) return rc;
  std::vector<fk::ItemDev> items;
  if ((rc = build_multi(ctx, n, bvp_ids, xy, paths, h, 1.0, items))) return rc;
  RunOut ro;
  RunOpts opts;
  opts.multi_bvp = true;
  opts.defer = true;  // one stream synchronisation: read_stats's
  rc = run_items(ctx, bvp_ids[0], precision, items, nullptr, nullptr, 0, nullptr, nullptr, nullptr, nullptr, ro, opts);
  if (rc) return rc;
  if ((rc = read_stats(ctx, ro.item_stats, n, out))) return rc;
  if ((rc = finish_run(ctx, ro))) return rc;
  if (ro.capped) return fail(ctx, FK_ERR_STEP_CAP, "paths reached max_steps");
  return FK_OK;
}

int fk_autotune_points(fk_ctx* ctx, int n, const int* bvp_ids, const double* xy, const unsigned* paths,
                       const double* h, int precision, double sample_fraction, int* best_block, int* best_chunk,
                       double* best_ms) {
  if (!ctx || n < 1 || !bvp_ids || !xy || !paths || !h) return fail(ctx, FK_ERR_ARG, "null argument");
  if (!(sample_fraction > 0 && sample_fraction <= 1)) return fail(ctx, FK_ERR_ARG, "sample_fraction in (0, 1]");
  int rc = need_device(ctx);
  if (rc) return rc;
  std::vector<fk::ItemDev> items;
  if ((rc = build_multi(ctx, n, bvp_ids, xy, paths, h, sample_fraction, items))) return rc;
  const unsigned saved_stream = ctx->stream_id;
  const int blocks[] = {64, 128, 256};
  const int chunks[] = {512, 2048, 8192, 32768};
  int bb = 256, bc = 0;
  double best = 1e300;
  for (int b : blocks)
    for (int c : chunks) {
      if (c % b) continue;
      ctx->block = b;
      ctx->chunk = c;
      double t = 1e300;
      for (int rep = 0; rep < 2; ++rep) {
        RunOut ro;
        RunOpts opts;
        opts.multi_bvp = true;
        rc = run_items(ctx, bvp_ids[0], precision, items, nullptr, nullptr, 0, nullptr, nullptr, nullptr, nullptr, ro,
                       opts);
        if (rc && rc != FK_ERR_STEP_CAP) {
          ctx->stream_id = saved_stream;
          return rc;
        }
        t = std::min(t, ctx->timing[0]);
      }
      if (t < best) { best = t; bb = b; bc = c; }
    }
  ctx->block = bb;
  ctx->chunk = bc;
  ctx->stream_id = saved_stream;  // tuning runs do not advance the random stream
  if (best_block) *best_block = bb;
  if (best_chunk) *best_chunk = bc;
  if (best_ms) *best_ms = best;
  return FK_OK;
}

int fk_register_arc(fk_ctx* ctx, const fk_arc_desc* d, int* id) {
  if (!ctx || !d || !id) return fail(ctx, FK_ERR_ARG, "null argument");
  if (d->n < 1 || d->n > 64 || !d->theta || !d->gids) return fail(ctx, FK_ERR_ARG, "arc needs 1..64 nodes with angles and ids");
  if (int rc0 = need_device(ctx)) return rc0;
  fk::MeshStencil M;
  M.cx = d->cx; M.cy = d->cy; M.radius = d->radius; M.c2 = d->c2; M.interior = d->interior;
  for (int i = 0; i < d->n; ++i) {
    fk::MeshNode nd;
    std::memset(&nd, 0, sizeof(nd));
    nd.theta = d->theta[i];
    nd.gid = d->gids[i];
    M.nodes.push_back(nd);
  }
  // append and (re)upload the registered-arc pool
  fk::StencilSet& S = ctx->arcs;
  std::vector<char> have(S.arcs.size(), 1);
  std::vector<double> host_ipsi;
  {
    // keep already computed inverses
    host_ipsi.assign(S.ipsi_total + static_cast<long long>(d->n) * d->n, 0.0);
    if (S.ipsi_total > 0) FK_CUDA(cudaMemcpy(host_ipsi.data(), S.d_ipsi.p, S.ipsi_total * sizeof(double), cudaMemcpyDeviceToHost));
  }
  add_arc(S, M, nullptr);
  have.push_back(d->iPsi ? 1 : 0);
  if (d->iPsi) std::memcpy(host_ipsi.data() + S.arcs.back().ipsi_off, d->iPsi, sizeof(double) * d->n * d->n);
  int rc = upload_stencils(ctx, S, &have, &host_ipsi);
  if (rc) return rc;
  FK_CUDA(cudaStreamSynchronize(ctx->stream));
  *id = static_cast<int>(S.arcs.size()) - 1;
  return FK_OK;
}

int fk_arc_ipsi(fk_ctx* ctx, int arc_id, double* iPsi) {
  if (!ctx || !iPsi) return fail(ctx, FK_ERR_ARG, "null argument");
  if (arc_id < 0 || arc_id >= static_cast<int>(ctx->arcs.arcs.size())) return fail(ctx, FK_ERR_REGISTRY, "unknown arc id");
  const fk::ArcDev& a = ctx->arcs.arcs[arc_id];
  FK_CUDA(cudaMemcpy(iPsi, ctx->arcs.d_ipsi.as<double>() + a.ipsi_off, sizeof(double) * a.n * a.n, cudaMemcpyDeviceToHost));
  return FK_OK;
}

int fk_solve_nodes_arc(fk_ctx* ctx, int bvp_id, int n, const fk_node_item* items, int precision, double* G, double* B,
                       fk_stats* stats) {
  if (!ctx) return FK_ERR_ARG;
  if (n < 0 || (n > 0 && (!items || !G || !B))) return fail(ctx, FK_ERR_ARG, "null argument");
  int rc = check_bvp(ctx, bvp_id);
  if (rc) return rc;
  if (n == 0) return FK_OK;
  if ((rc = need_device(ctx))) return rc;
  fk::StencilSet& S = ctx->arcs;
  std::vector<fk::ItemDev>& it = ctx->tmp_items;
  it.resize(n);
  std::vector<long long> goff(n);
  long long gt = 0;
  for (int i = 0; i < n; ++i) {
    const fk_node_item& q = items[i];
    if (q.stencil < 0 || q.stencil >= static_cast<int>(S.arcs.size())) return fail(ctx, FK_ERR_REGISTRY, "unknown arc id");
    if (!(q.h > 0)) return fail(ctx, FK_ERR_ARG, "h must be > 0");
    fk::ItemDev& d = it[i];
    std::memset(&d, 0, sizeof(d));
    const fk::ArcDev& a = S.arcs[q.stencil];
    d.x = q.x; d.y = q.y; d.h = q.h; d.sqrth = std::sqrt(q.h); d.paths = q.paths; d.stencil = q.stencil;
    d.frontera = q.frontera ? 1 : 0; d.sub_shape = FK_SHAPE_CIRCLE;
    d.sub[0] = a.radius; d.sub[1] = a.cx; d.sub[2] = a.cy;
    goff[i] = gt;
    gt += a.n;
  }
  RunOut ro;
  rc = run_items(ctx, bvp_id, precision, it, &S, &goff, gt, nullptr, nullptr, nullptr, nullptr, ro);
  if (rc) return rc;
  FK_CUDA(copy_out(G, ro.item_G, gt * sizeof(double), ctx->stream));
  FK_CUDA(copy_out(B, ro.item_B, n * sizeof(double), ctx->stream));
  if (stats) {
    if ((rc = read_stats(ctx, ro.item_stats, n, stats))) return rc;
  }
  FK_CUDA(cudaStreamSynchronize(ctx->stream));
  if (ro.capped) return fail(ctx, FK_ERR_STEP_CAP, "paths reached max_steps");
  return FK_OK;
}

static int finish_mesh(fk_ctx* ctx, std::unique_ptr<fk::Mesh>& M, int* id) {
  fk::HostMesh& h = M->host;
  fk::StencilSet& S = M->st;
  S.kind = h.kind;
  for (const fk::MeshStencil& st : h.stencils) {
    if (h.kind == 1) add_arc(S, st, nullptr); else add_patch(S, st, h.knn, h.eps);
  }
  if (h.kind == 1 && S.nmax > 64) return fail(ctx, FK_ERR_CAPACITY, "arcs with more than 64 nodes");
  // item -> G offsets and CSR positions (binary search in the sorted row;
  // items in parallel on the host cores)
  const int n_items = static_cast<int>(h.items.size());
  M->g_off.resize(n_items);
  M->rows.resize(n_items);
  M->g_total = 0;
  for (int i = 0; i < n_items; ++i) {
    M->g_off[i] = M->g_total;
    M->g_total += S.size_of(h.items[i].stencil);
    M->rows[i] = h.items[i].row;
  }
  M->csr_idx.assign(static_cast<size_t>(M->g_total), -1);
  std::atomic<int> missing{0};
  fk::host_parallel_for(n_items, [&](int i) {
    const fk::MeshItem& q = h.items[i];
    const int sz = S.size_of(q.stencil);
    const int* row_begin = h.col.data() + h.rowptr[q.row];
    const int* row_end = h.col.data() + h.rowptr[q.row + 1];
    for (int j = 0; j < sz; ++j) {
      const int gid = (h.kind == 1) ? S.arc_gids[S.arc_gid_off[q.stencil] + j] : h.stencils[q.stencil].nodes[j].gid;
      const int* p = std::lower_bound(row_begin, row_end, gid);
      if (p == row_end || *p != gid) {
        missing.store(1);
        return;
      }
      M->csr_idx[M->g_off[i] + j] = static_cast<int>(p - h.col.data());
    }
  });
  if (missing.load()) return fail(ctx, FK_ERR_NOT_FOUND, "stencil node missing from the CSR row");
  ctx->meshes.push_back(std::move(M));
  *id = static_cast<int>(ctx->meshes.size()) - 1;
  return FK_OK;
}

int fk_mesh_circles(fk_ctx* ctx, const double dom[4], int n_side, double superposicion, double theta0,
                    int nodes_per_circle, double c2_corner, double c2_side, int* mesh_id) {
  if (!ctx || !dom || !mesh_id) return fail(ctx, FK_ERR_ARG, "null argument");
  std::unique_ptr<fk::Mesh> M(new fk::Mesh());
  if (!fk::build_circle_mesh(dom, n_side, superposicion, theta0, nodes_per_circle, c2_corner, c2_side, M->host, ctx->err))
    return FK_ERR_ARG;
  return finish_mesh(ctx, M, mesh_id);
}

int fk_mesh_square_patches(fk_ctx* ctx, const double dom[4], int n_sub, int nodes_per_side, double enlarge,
                           double eps_spacing, int knn, int* mesh_id) {
  if (!ctx || !dom || !mesh_id) return fail(ctx, FK_ERR_ARG, "null argument");
  if (knn > 32) return fail(ctx, FK_ERR_ARG, "knn must be <= 32");
  std::unique_ptr<fk::Mesh> M(new fk::Mesh());
  if (!fk::build_square_patch_mesh(dom, n_sub, nodes_per_side, enlarge, eps_spacing, knn, M->host, ctx->err))
    return FK_ERR_ARG;
  return finish_mesh(ctx, M, mesh_id);
}

static fk::Mesh* get_mesh(fk_ctx* ctx, int id) {
  if (!ctx || id < 0 || id >= static_cast<int>(ctx->meshes.size())) return nullptr;
  return ctx->meshes[id].get();
}

static int upload_mesh(fk_ctx* ctx, fk::Mesh* M) {
  if (M->uploaded) return FK_OK;
  int rc = upload_stencils(ctx, M->st, nullptr, nullptr);
  if (rc) return rc;
  cudaStream_t s = ctx->stream;
  FK_CUDA(fk::upload(M->d_val0, M->host.val0, s));
  FK_CUDA(fk::upload(M->d_csr_idx, M->csr_idx, s));
  FK_CUDA(fk::upload(M->d_row, M->rows, s));
  FK_CUDA(cudaStreamSynchronize(s));
  M->uploaded = true;
  return FK_OK;
}

// Disk rows: uploads the batch once, runs the four disk kernels on the
// context stream into G/B (device, may be null) and/or the CSR values and B
// (device, may be null), and checks the kernels' error flags.
static int run_disks(fk_ctx* ctx, int bvp_id, const fk::DiskBatch& b, fk::DiskBufs& u, double* G, double* B,
                     double* val, double* Bcsr, bool timed) {
  cudaStream_t s = ctx->stream;
  if (!u.uploaded) {
    FK_CUDA(fk::upload(u.disks, b.disks, s));
    FK_CUDA(fk::upload(u.tab, b.tab, s));
    FK_CUDA(fk::upload(u.pth, b.periph_theta, s));
    FK_CUDA(fk::upload(u.ixy, b.inner_xy, s));
    FK_CUDA(fk::upload(u.idisk, b.inner_disk, s));
    FK_CUDA(fk::upload(u.irow, b.inner_row, s));
    FK_CUDA(fk::upload(u.cpos, b.csr_pos, s));
    u.uploaded = true;
  }
  const int nd = static_cast<int>(b.disks.size());
  FK_CUDA(ctx->w_dgrid.ensure(std::max<long long>(b.grid_total, 1) * sizeof(double)));
  FK_CUDA(ctx->w_dcbar.ensure(std::max(nd, 1) * sizeof(double)));
  FK_CUDA(ctx->w_dvar.ensure(std::max(nd, 1) * sizeof(int)));
  FK_CUDA(ctx->w_dminv.ensure(std::max<long long>(b.minv_total, 1) * sizeof(double)));
  FK_CUDA(ctx->w_dz.ensure(std::max<long long>(b.z_total, 1) * sizeof(double)));
  FK_CUDA(ctx->w_dflags.ensure(2 * sizeof(int)));
  FK_CUDA(cudaMemsetAsync(ctx->w_dflags.p, 0, 2 * sizeof(int), s));
  fk::DiskArgs a;
  a.bvp = ctx->d_bvps.as<fk::BvpDev>() + bvp_id;
  a.disks = u.disks.as<fk::DiskDev>();
  a.n_disks = nd;
  a.tab = u.tab.as<double>();
  a.periph_theta = u.pth.as<double>();
  a.inner_xy = u.ixy.as<double>();
  a.inner_disk = u.idisk.as<int>();
  a.grid = ctx->w_dgrid.as<double>();
  a.cbar = ctx->w_dcbar.as<double>();
  a.varying = ctx->w_dvar.as<int>();
  a.minv = ctx->w_dminv.as<double>();
  a.z = ctx->w_dz.as<double>();
  a.G = G;
  a.B = B;
  const bool csr = val && b.has_csr;
  a.inner_row = csr ? u.irow.as<int>() : nullptr;
  a.csr_pos = csr ? u.cpos.as<int>() : nullptr;
  a.val = csr ? val : nullptr;
  a.Bcsr = csr ? Bcsr : nullptr;
  a.flags = ctx->w_dflags.as<int>();
  FK_CUDA(fk::disk_launch(ctx->bvps[bvp_id].problem, a, b, s, timed ? ctx->ev : nullptr));
  int flags[2];
  FK_CUDA(cudaMemcpyAsync(flags, ctx->w_dflags.p, sizeof(flags), cudaMemcpyDeviceToHost, s));
  FK_CUDA(cudaStreamSynchronize(s));
  if (timed) {
    float t0 = 0, t1 = 0;
    cudaEventElapsedTime(&t0, ctx->ev[0], ctx->ev[1]);
    cudaEventElapsedTime(&t1, ctx->ev[1], ctx->ev[2]);
    ctx->timing[0] = t0;
    ctx->timing[1] = t1;
    ctx->timing[2] = 4;
  }
  if (flags[0]) return fail(ctx, FK_ERR_NUMERIC, "disk solve: singular Fourier-mode matrix");
  if (flags[1]) return fail(ctx, FK_ERR_NUMERIC, "disk solve: iteration on the varying c did not converge");
  return FK_OK;
}

int fk_mesh_get_info(fk_ctx* ctx, int mesh_id, fk_mesh_info* info) {
  fk::Mesh* M = get_mesh(ctx, mesh_id);
  if (!M || !info) return fail(ctx, FK_ERR_REGISTRY, "unknown mesh id");
  info->n_rows = M->host.n_rows;
  info->nnz = M->host.nnz;
  info->n_items = static_cast<int>(M->host.items.size());
  info->n_nodes = static_cast<int>(M->host.nodes.size());
  info->n_stencils = static_cast<int>(M->host.stencils.size());
  int mx = 0;
  for (size_t s = 0; s < M->host.stencils.size(); ++s) mx = std::max<int>(mx, static_cast<int>(M->host.stencils[s].nodes.size()));
  info->max_stencil = mx;
  info->spacing = M->host.spacing;
  return FK_OK;
}

int fk_mesh_nodes(fk_ctx* ctx, int mesh_id, double* xy, int* flags) {
  fk::Mesh* M = get_mesh(ctx, mesh_id);
  if (!M) return fail(ctx, FK_ERR_REGISTRY, "unknown mesh id");
  for (size_t i = 0; i < M->host.nodes.size(); ++i) {
    if (xy) { xy[2 * i] = M->host.nodes[i].x; xy[2 * i + 1] = M->host.nodes[i].y; }
    if (flags) flags[i] = M->host.nodes[i].frontera ? 1 : 0;
  }
  return FK_OK;
}

int fk_mesh_items(fk_ctx* ctx, int mesh_id, int* row, double* xy, int* stencil, int* frontera) {
  fk::Mesh* M = get_mesh(ctx, mesh_id);
  if (!M) return fail(ctx, FK_ERR_REGISTRY, "unknown mesh id");
  for (size_t i = 0; i < M->host.items.size(); ++i) {
    const fk::MeshItem& q = M->host.items[i];
    if (row) row[i] = q.row;
    if (xy) { xy[2 * i] = q.x; xy[2 * i + 1] = q.y; }
    if (stencil) stencil[i] = q.stencil;
    if (frontera) frontera[i] = q.frontera ? 1 : 0;
  }
  return FK_OK;
}

int fk_mesh_stencil_nodes(fk_ctx* ctx, int mesh_id, int s, int* gids, int* n) {
  fk::Mesh* M = get_mesh(ctx, mesh_id);
  if (!M || !n) return fail(ctx, FK_ERR_REGISTRY, "unknown mesh id");
  if (s < 0 || s >= static_cast<int>(M->host.stencils.size())) return fail(ctx, FK_ERR_REGISTRY, "unknown stencil");
  const fk::MeshStencil& S = M->host.stencils[s];
  *n = static_cast<int>(S.nodes.size());
  if (gids) for (size_t i = 0; i < S.nodes.size(); ++i) gids[i] = S.nodes[i].gid;
  return FK_OK;
}

int fk_mesh_window(fk_ctx* ctx, int mesh_id, int s, double x, double y, int* window, int* nearest, int* walk) {
  fk::Mesh* M = get_mesh(ctx, mesh_id);
  if (!M) return fail(ctx, FK_ERR_REGISTRY, "unknown mesh id");
  if (M->host.kind != 2) return fail(ctx, FK_ERR_ARG, "not a square-patch mesh");
  if (s < 0 || s >= static_cast<int>(M->st.patches.size())) return fail(ctx, FK_ERR_REGISTRY, "unknown stencil");
  if (!window || !nearest || !walk) return fail(ctx, FK_ERR_ARG, "null argument");
  const fk::PatchDev& P = M->st.patches[s];
  const fk::MeshStencil& MS = M->host.stencils[s];
  const int m = P.m, k = P.k;
  *walk = (P.walk32 & 3) | ((P.walk & 3) << 2);
  // the kernel's knn_window, in FP64: the side nearest to the point ...
  int best_s = -1;
  double best = 1e300;
  for (int q = 0; q < 4; ++q) {
    if (P.side_count[q] > 0) {
      const double dist = std::fabs((P.side_axis[q] == 0 ? y : x) - P.side_fixed[q]);
      if (dist < best) { best = dist; best_s = q; }
    }
  }
  if (best_s < 0) return fail(ctx, FK_ERR_ARG, "patch without sides");
  const double u = ((P.side_axis[best_s] == 0 ? x : y) - P.side_start[best_s]) * (1.0 / P.side_step[best_s]);
  int j = static_cast<int>(std::rint(u));
  j = std::max(0, std::min(P.side_count[best_s] - 1, j));
  *nearest = P.side_first[best_s] + j;
  // ... then its window-table bin and the one comparison
  if (P.knn_n[best_s] > 0) {
    int b = static_cast<int>(std::floor((u - P.knn_u0[best_s]) * fk::kKnnBins));
    b = std::max(0, std::min(P.knn_n[best_s] - 1, b));
    const unsigned short t = M->st.knn_tab[P.knn_off + P.knn_base[best_s] + b];
    if (!(t & fk::kKnnFull)) {
      int L = t;
      const int up = L + k;
      if (P.closed || up < m) {
        auto d2 = [&](int idx) {
          if (idx >= m) idx -= m;
          const double dx = x - MS.nodes[idx].x, dy = y - MS.nodes[idx].y;
          return dx * dx + dy * dy;
        };
        if (d2(up) < d2(L)) L = (L + 1 == m) ? 0 : L + 1;
      }
      *window = L;
      return FK_OK;
    }
  }
  *window = knn_window_host(MS, k, x, y);  // a bin the table does not certify: the sliding search
  return FK_OK;
}

int fk_mesh_csr(fk_ctx* ctx, int mesh_id, int* rowptr, int* col, double* val0) {
  fk::Mesh* M = get_mesh(ctx, mesh_id);
  if (!M) return fail(ctx, FK_ERR_REGISTRY, "unknown mesh id");
  if (rowptr) std::memcpy(rowptr, M->host.rowptr.data(), sizeof(int) * M->host.rowptr.size());
  if (col) std::memcpy(col, M->host.col.data(), sizeof(int) * M->host.col.size());
  if (val0) std::memcpy(val0, M->host.val0.data(), sizeof(double) * M->host.val0.size());
  return FK_OK;
}

int fk_solve_disks_ps(fk_ctx* ctx, int bvp_id, int n_disks, const fk_disk_desc* disks, double* G, double* B) {
  if (!ctx || n_disks < 0 || (n_disks > 0 && !disks)) return fail(ctx, FK_ERR_ARG, "null argument");
  int rc = check_bvp(ctx, bvp_id);
  if (rc) return rc;
  if ((rc = need_device(ctx))) return rc;
  std::vector<fk::DiskHost> in(n_disks);
  for (int d = 0; d < n_disks; ++d) {
    const fk_disk_desc& q = disks[d];
    if (q.n_periph < 0 || q.n_inner < 0 || (q.n_periph > 0 && !q.periph_theta) || (q.n_inner > 0 && !q.inner_xy))
      return fail(ctx, FK_ERR_ARG, "disk: null node arrays");
    fk::DiskHost& h = in[d];
    h.cx = q.cx; h.cy = q.cy; h.radius = q.radius; h.theta0 = q.theta0;
    h.n_circle = q.n_circle; h.n_radial = q.n_radial;
    h.periph_theta.assign(q.periph_theta, q.periph_theta + q.n_periph);
    h.inner_xy.assign(q.inner_xy, q.inner_xy + 2 * static_cast<size_t>(q.n_inner));
  }
  fk::DiskBatch b;
  if (!fk::disk_prepare(in, b, ctx->err)) return FK_ERR_ARG;
  if (ctx->bvps.size() * sizeof(fk::BvpDev) > ctx->d_bvps.bytes) {
    FK_CUDA(fk::upload(ctx->d_bvps, ctx->bvps, ctx->stream));
  }
  cudaStream_t s = ctx->stream;
  FK_CUDA(ctx->w_dG.ensure(std::max<long long>(b.g_total, 1) * sizeof(double)));
  FK_CUDA(ctx->w_dB.ensure(std::max<long long>(b.n_inner, 1) * sizeof(double)));
  ctx->w_disk.uploaded = false;
  rc = run_disks(ctx, bvp_id, b, ctx->w_disk, ctx->w_dG.as<double>(), ctx->w_dB.as<double>(), nullptr, nullptr, true);
  if (rc) return rc;
  FK_CUDA(copy_out(G, ctx->w_dG.p, b.g_total * sizeof(double), s));
  FK_CUDA(copy_out(B, ctx->w_dB.p, b.n_inner * sizeof(double), s));
  FK_CUDA(cudaStreamSynchronize(s));
  return FK_OK;
}

int fk_mesh_set_disk_solver(fk_ctx* ctx, int mesh_id, int n_radial) {
  fk::Mesh* M = get_mesh(ctx, mesh_id);
  if (!M) return fail(ctx, FK_ERR_REGISTRY, "unknown mesh id");
  if (M->host.kind != 1) return fail(ctx, FK_ERR_ARG, "disk rows need a circle mesh");
  if (n_radial < 0) return fail(ctx, FK_ERR_ARG, "n_radial must be >= 0");
  M->disk_radial = 0;
  M->disk = fk::DiskBatch();
  M->dbufs.uploaded = false;
  if (n_radial == 0) return FK_OK;
  const fk::HostMesh& hm = M->host;
  std::vector<fk::DiskHost> in;
  for (const fk::MeshStencil& S : hm.stencils) {
    if (S.perimeter || S.inner.empty()) continue;
    fk::DiskHost h;
    h.cx = S.cx; h.cy = S.cy; h.radius = S.radius;
    h.theta0 = S.nodes.empty() ? 0.0 : S.nodes[0].theta;
    h.n_circle = static_cast<int>(S.nodes.size());
    h.n_radial = n_radial;
    for (const fk::MeshNode& nd : S.nodes) h.periph_theta.push_back(nd.theta);
    for (const fk::MeshNode& in_nd : S.inner) {
      h.inner_xy.push_back(in_nd.x);
      h.inner_xy.push_back(in_nd.y);
      h.inner_row.push_back(in_nd.gid);
      const int* row_begin = hm.col.data() + hm.rowptr[in_nd.gid];
      const int* row_end = hm.col.data() + hm.rowptr[in_nd.gid + 1];
      for (const fk::MeshNode& c : S.nodes) {
        const int* p = std::lower_bound(row_begin, row_end, c.gid);
        if (p == row_end || *p != c.gid) return fail(ctx, FK_ERR_NOT_FOUND, "circle node missing from the CSR row");
        h.csr_pos.push_back(static_cast<int>(p - hm.col.data()));
      }
    }
    in.push_back(std::move(h));
  }
  if (!fk::disk_prepare(in, M->disk, ctx->err)) return FK_ERR_ARG;
  M->disk_radial = n_radial;
  return FK_OK;
}

int fk_assemble(fk_ctx* ctx, int mesh_id, int bvp_id, unsigned paths, const unsigned* paths_per_item, double h,
                int precision, double* val, double* B, double* item_G, double* item_B, fk_stats* item_stats) {
  fk::Mesh* M = get_mesh(ctx, mesh_id);
  if (!M) return fail(ctx, FK_ERR_REGISTRY, "unknown mesh id");
  int rc = check_bvp(ctx, bvp_id);
  if (rc) return rc;
  if (!(h > 0)) return fail(ctx, FK_ERR_ARG, "h must be > 0");
  if ((rc = need_device(ctx))) return rc;
  if (ctx->bvps.size() * sizeof(fk::BvpDev) > ctx->d_bvps.bytes) {
    FK_CUDA(fk::upload(ctx->d_bvps, ctx->bvps, ctx->stream));
  }
  if ((rc = upload_mesh(ctx, M))) return rc;
  const fk::HostMesh& hm = M->host;
  const int n = static_cast<int>(hm.items.size());
  // the mesh's solve records (kept across calls: only h and the path counts change)
  std::vector<fk::ItemDev>& it = M->a_items;
  if (static_cast<int>(it.size()) != n) {
    it.resize(n);
    for (int i = 0; i < n; ++i) {
      const fk::MeshItem& q = hm.items[i];
      fk::ItemDev& d = it[i];
      std::memset(&d, 0, sizeof(d));
      d.x = q.x; d.y = q.y;
      d.stencil = q.stencil; d.frontera = q.frontera ? 1 : 0;
      const fk::MeshStencil& S = hm.stencils[q.stencil];
      if (hm.kind == 1) { d.sub_shape = FK_SHAPE_CIRCLE; d.sub[0] = S.radius; d.sub[1] = S.cx; d.sub[2] = S.cy; }
      else { d.sub_shape = FK_SHAPE_RECT; for (int k = 0; k < 4; ++k) d.sub[k] = S.rect[k]; }
    }
  }
  const double sqrth = std::sqrt(h);
  for (int i = 0; i < n; ++i) {
    fk::ItemDev& d = it[i];
    d.h = h;
    d.sqrth = sqrth;
    d.paths = paths_per_item ? paths_per_item[i] : paths;
  }
  cudaStream_t s = ctx->stream;
  FK_CUDA(ctx->w_val.ensure(std::max<size_t>(hm.nnz * sizeof(double), 16)));
  FK_CUDA(ctx->w_B.ensure(std::max<size_t>(hm.n_rows * sizeof(double), 16)));
  FK_CUDA(cudaMemcpyAsync(ctx->w_val.p, M->d_val0.p, hm.nnz * sizeof(double), cudaMemcpyDeviceToDevice, s));
  FK_CUDA(cudaMemsetAsync(ctx->w_B.p, 0, hm.n_rows * sizeof(double), s));
  RunOut ro;
  RunOpts asm_opts;
  asm_opts.need_item_G = item_G != nullptr;
  asm_opts.defer = !(M->disk_radial > 0 && !M->disk.disks.empty());  // (the disk rows run their own launches)
  rc = run_items(ctx, bvp_id, precision, it, &M->st, &M->g_off, M->g_total, M->d_csr_idx.as<int>(),
                 ctx->w_val.as<double>(), M->d_row.as<int>(), ctx->w_B.as<double>(), ro, asm_opts);
  if (rc) return rc;
  if (M->disk_radial > 0 && !M->disk.disks.empty()) {
    rc = run_disks(ctx, bvp_id, M->disk, M->dbufs, nullptr, nullptr, ctx->w_val.as<double>(), ctx->w_B.as<double>(),
                   false);
    if (rc) return rc;
  }
  FK_CUDA(copy_out(val, ctx->w_val.p, hm.nnz * sizeof(double), s));
  FK_CUDA(copy_out(B, ctx->w_B.p, hm.n_rows * sizeof(double), s));
  FK_CUDA(copy_out(item_G, ro.item_G, M->g_total * sizeof(double), s));
  FK_CUDA(copy_out(item_B, ro.item_B, n * sizeof(double), s));
  if (item_stats) {
    if ((rc = read_stats(ctx, ro.item_stats, n, item_stats))) return rc;
  }
  FK_CUDA(cudaStreamSynchronize(s));
  if ((rc = finish_run(ctx, ro))) return rc;
  if (ro.capped) return fail(ctx, FK_ERR_STEP_CAP, "paths reached max_steps");
  return FK_OK;
}

// ---- adaptive assembly in rounds ---------------------------------------------
// Items of a mesh as solve records (fk_assemble's layout), paths and BVP per item.
static void mesh_items_dev(const fk::HostMesh& hm, std::vector<fk::ItemDev>& it, double h,
                           const unsigned long long* paths, const int* bvp) {
  const int n = static_cast<int>(hm.items.size());
  it.resize(n);
  for (int i = 0; i < n; ++i) {
    const fk::MeshItem& q = hm.items[i];
    fk::ItemDev& d = it[i];
    std::memset(&d, 0, sizeof(d));
    d.x = q.x; d.y = q.y; d.h = h; d.sqrth = std::sqrt(h);
    d.paths = static_cast<unsigned>(paths[i]);
    d.stencil = q.stencil; d.frontera = q.frontera ? 1 : 0;
    d.bvp = bvp[i];
    const fk::MeshStencil& S = hm.stencils[q.stencil];
    if (hm.kind == 1) { d.sub_shape = FK_SHAPE_CIRCLE; d.sub[0] = S.radius; d.sub[1] = S.cx; d.sub[2] = S.cy; }
    else { d.sub_shape = FK_SHAPE_RECT; for (int k = 0; k < 4; ++k) d.sub[k] = S.rect[k]; }
  }
}

int fk_assembly_begin(fk_ctx* ctx, int mesh_id) {
  fk::Mesh* M = get_mesh(ctx, mesh_id);
  if (!M) return fail(ctx, FK_ERR_REGISTRY, "unknown mesh id");
  if (M->host.kind != 2) return fail(ctx, FK_ERR_ARG, "adaptive rounds need a square-patch mesh");
  int rc = need_device(ctx);
  if (rc) return rc;
  if ((rc = upload_mesh(ctx, M))) return rc;
  const int n = static_cast<int>(M->host.items.size());
  cudaStream_t s = ctx->stream;
  FK_CUDA(M->r_gsum.ensure(std::max<size_t>(M->g_total * sizeof(double), 16)));
  FK_CUDA(M->r_stats.ensure(std::max<size_t>(static_cast<size_t>(n) * fk::kNumStats * sizeof(double), 16)));
  FK_CUDA(M->r_var.ensure(std::max<size_t>(n * sizeof(double), 16)));
  FK_CUDA(cudaMemsetAsync(M->r_gsum.p, 0, M->g_total * sizeof(double), s));
  FK_CUDA(cudaMemsetAsync(M->r_stats.p, 0, static_cast<size_t>(n) * fk::kNumStats * sizeof(double), s));
  FK_CUDA(cudaStreamSynchronize(s));
  M->r_paths.assign(n, 0ull);
  M->r_bvp.assign(n, -1);
  M->r_h = 0.0;
  M->r_active = true;
  return FK_OK;
}

int fk_assembly_round(fk_ctx* ctx, int mesh_id, int bvp_id, const int* bvp_of_item, const unsigned* paths_per_item,
                      double h, int precision, double* item_var) {
  fk::Mesh* M = get_mesh(ctx, mesh_id);
  if (!M) return fail(ctx, FK_ERR_REGISTRY, "unknown mesh id");
  if (!M->r_active) return fail(ctx, FK_ERR_ARG, "fk_assembly_round before fk_assembly_begin");
  if (!paths_per_item) return fail(ctx, FK_ERR_ARG, "null argument");
  int rc = check_bvp(ctx, bvp_id);
  if (rc) return rc;
  if (!(h > 0)) return fail(ctx, FK_ERR_ARG, "h must be > 0");
  if (M->r_h > 0 && h != M->r_h) return fail(ctx, FK_ERR_ARG, "every round of an assembly takes the same h");
  if ((rc = need_device(ctx))) return rc;
  const fk::HostMesh& hm = M->host;
  const int n = static_cast<int>(hm.items.size());
  // one problem functor; the items' control variates may differ, and the
  // items with a learned one share one network (whose BVP the launch takes)
  std::vector<int> bv(n, bvp_id);
  int launch_bvp = bvp_id;
  const fk::BvpDev& b0 = ctx->bvps[bvp_id];
  int mlp = b0.cv == FK_CV_MLP ? b0.mlp : -1;
  for (int i = 0; i < n; ++i) {
    if (bvp_of_item) bv[i] = bvp_of_item[i];
    if ((rc = check_bvp(ctx, bv[i]))) return rc;
    const fk::BvpDev& b = ctx->bvps[bv[i]];
    if (b.problem != b0.problem) return fail(ctx, FK_ERR_ARG, "one round needs BVPs of one problem functor");
    if (b.cv == FK_CV_MLP) {
      if (mlp >= 0 && b.mlp != mlp) return fail(ctx, FK_ERR_ARG, "one round takes one learned network");
      mlp = b.mlp;
      if (paths_per_item[i] > 0) launch_bvp = bv[i];
    }
  }
  if (ctx->bvps.size() * sizeof(fk::BvpDev) > ctx->d_bvps.bytes) FK_CUDA(fk::upload(ctx->d_bvps, ctx->bvps, ctx->stream));
  std::vector<fk::ItemDev>& it = M->r_items;
  if (static_cast<int>(it.size()) != n || M->r_items_h != h) {
    std::vector<unsigned long long> p(paths_per_item, paths_per_item + n);
    mesh_items_dev(hm, it, h, p.data(), bv.data());
    M->r_items_h = h;
  } else {
    for (int i = 0; i < n; ++i) {
      it[i].paths = paths_per_item[i];
      it[i].bvp = bv[i];
    }
  }
  RunOut ro;
  RunOpts o;
  o.multi_bvp = true;
  o.g_sum = M->r_gsum.as<double>();
  o.run_stats = M->r_stats.as<double>();
  o.item_var = item_var ? M->r_var.as<double>() : nullptr;
  rc = run_items(ctx, launch_bvp, precision, it, &M->st, &M->g_off, M->g_total, M->d_csr_idx.as<int>(), nullptr,
                 nullptr, nullptr, ro, o);
  if (rc) return rc;
  for (int i = 0; i < n; ++i) {
    M->r_paths[i] += paths_per_item[i];
    if (paths_per_item[i] > 0 || M->r_bvp[i] < 0) M->r_bvp[i] = bv[i];
  }
  M->r_h = h;
  if (item_var) {
    FK_CUDA(copy_out(item_var, M->r_var.p, n * sizeof(double), ctx->stream));
    FK_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  if (ro.capped) return fail(ctx, FK_ERR_STEP_CAP, "paths reached max_steps");
  return FK_OK;
}

int fk_assembly_end(fk_ctx* ctx, int mesh_id, double* val, double* B, double* item_G, double* item_B,
                    fk_stats* item_stats) {
  fk::Mesh* M = get_mesh(ctx, mesh_id);
  if (!M) return fail(ctx, FK_ERR_REGISTRY, "unknown mesh id");
  if (!M->r_active) return fail(ctx, FK_ERR_ARG, "fk_assembly_end before fk_assembly_begin");
  int rc = need_device(ctx);
  if (rc) return rc;
  const fk::HostMesh& hm = M->host;
  const int n = static_cast<int>(hm.items.size());
  cudaStream_t s = ctx->stream;
  std::vector<int> bv(M->r_bvp);
  int problem = 0;
  for (int i = 0; i < n; ++i) {
    if (bv[i] < 0) bv[i] = 0;  // (an item no round gave paths: B = g(x) or 0, no G)
    problem = ctx->bvps.empty() ? 0 : ctx->bvps[bv[i]].problem;
  }
  if (ctx->bvps.empty()) return fail(ctx, FK_ERR_REGISTRY, "no BVP registered");
  for (int i = 0; i < n; ++i)
    if (M->r_paths[i] > 0xffffffffull) return fail(ctx, FK_ERR_CAPACITY, "an item ran more than 2^32 - 1 paths");
  // the rounds' solve records with the path totals (built afresh if no round ran)
  std::vector<fk::ItemDev>& it = M->r_items;
  if (static_cast<int>(it.size()) != n || !(M->r_h > 0) || M->r_items_h != M->r_h) {
    mesh_items_dev(hm, it, M->r_h > 0 ? M->r_h : 1.0, M->r_paths.data(), bv.data());
    M->r_items_h = M->r_h;
  } else {
    for (int i = 0; i < n; ++i) {
      it[i].paths = static_cast<unsigned>(M->r_paths[i]);
      it[i].bvp = bv[i];
    }
  }
  FK_CUDA(fk::upload_pinned(ctx->w_items, ctx->h_items, it, s));
  FK_CUDA(fk::upload_pinned(ctx->w_goff, ctx->h_goff, M->g_off, s));
  FK_CUDA(ctx->w_val.ensure(std::max<size_t>(hm.nnz * sizeof(double), 16)));
  FK_CUDA(ctx->w_B.ensure(std::max<size_t>(hm.n_rows * sizeof(double), 16)));
  FK_CUDA(ctx->w_gout.ensure(std::max<size_t>(M->g_total * sizeof(double), 16)));
  FK_CUDA(ctx->w_bout.ensure(std::max<size_t>(n * sizeof(double), 16)));
  FK_CUDA(ctx->w_sout.ensure(std::max<size_t>(static_cast<size_t>(n) * 16 * sizeof(double), 16)));
  FK_CUDA(ctx->w_queue.ensure(16));
  FK_CUDA(cudaMemsetAsync(ctx->w_queue.p, 0, 7 * sizeof(int), s));  // (run_items' seven check words)
  FK_CUDA(cudaMemcpyAsync(ctx->w_val.p, M->d_val0.p, hm.nnz * sizeof(double), cudaMemcpyDeviceToDevice, s));
  FK_CUDA(cudaMemsetAsync(ctx->w_B.p, 0, hm.n_rows * sizeof(double), s));
  fk::FinalizeArgs f;
  std::memset(&f, 0, sizeof(f));
  f.bvp = ctx->d_bvps.as<fk::BvpDev>();
  f.items = ctx->w_items.as<fk::ItemDev>();
  f.n_items = n;
  f.patches = M->st.d_patches.as<fk::PatchDev>();
  f.stats = M->r_stats.as<double>();
  f.stencil_kind = 2;
  f.g_off = ctx->w_goff.as<long long>();
  f.item_G = item_G ? ctx->w_gout.as<double>() : nullptr;
  f.item_B = ctx->w_bout.as<double>();
  f.item_stats = ctx->w_sout.as<double>();
  f.row = M->d_row.as<int>();
  f.B = ctx->w_B.as<double>();
  f.flags = ctx->w_queue.as<int>() + 2;
  f.g_fused = 1;  // statistics and B only; the rows come from the running sums
  FK_CUDA(cudaEventRecord(ctx->ev[0], s));
  FK_CUDA(fk::launch_finalize(f, problem, s));
  FK_CUDA(fk::launch_rows_from_sums(f.items, n, f.patches, f.g_off, M->r_gsum.as<double>(), M->d_csr_idx.as<int>(),
                                    ctx->w_val.as<double>(), f.item_G, s));
  FK_CUDA(cudaEventRecord(ctx->ev[1], s));
  FK_CUDA(copy_out(val, ctx->w_val.p, hm.nnz * sizeof(double), s));
  FK_CUDA(copy_out(B, ctx->w_B.p, hm.n_rows * sizeof(double), s));
  FK_CUDA(copy_out(item_G, ctx->w_gout.p, M->g_total * sizeof(double), s));
  FK_CUDA(copy_out(item_B, ctx->w_bout.p, n * sizeof(double), s));
  if (item_stats) {
    if ((rc = read_stats(ctx, ctx->w_sout.as<double>(), n, item_stats))) return rc;
  }
  FK_CUDA(cudaStreamSynchronize(s));
  float t1 = 0;
  cudaEventElapsedTime(&t1, ctx->ev[0], ctx->ev[1]);
  ctx->timing[0] = 0;
  ctx->timing[1] = t1;
  ctx->timing[2] = 2;
  int q[4] = {0, 0, 0, 0};
  FK_CUDA(cudaMemcpy(q, ctx->w_queue.p, sizeof(q), cudaMemcpyDeviceToHost));
  if (q[2] != 0) return fail(ctx, FK_ERR_STEP_CAP, "paths reached max_steps");
  return FK_OK;
}

// ---- learned control variate ------------------------------------------------
static fk::Mlp* get_mlp(fk_ctx* ctx, int id) {
  if (!ctx || id < 0 || id >= static_cast<int>(ctx->mlps.size())) return nullptr;
  return ctx->mlps[id].get();
}

int fk_mlp_create(fk_ctx* ctx, int n_regions, const double* rects, unsigned long long seed, int* mlp_id) {
  if (!ctx || !rects || !mlp_id || n_regions < 1) return fail(ctx, FK_ERR_ARG, "mlp: need >= 1 region rectangle");
  int rc = need_device(ctx);
  if (rc) return rc;
  std::unique_ptr<fk::Mlp> M(new fk::Mlp());
  rc = fk::mlp_init(*M, n_regions, rects, seed, ctx->stream, ctx->err);
  if (rc) return rc;
  ctx->mlps.push_back(std::move(M));
  *mlp_id = static_cast<int>(ctx->mlps.size()) - 1;
  return FK_OK;
}

int fk_mlp_num_params(fk_ctx* ctx, int mlp_id, int* n) {
  fk::Mlp* M = get_mlp(ctx, mlp_id);
  if (!M || !n) return fail(ctx, FK_ERR_REGISTRY, "unknown mlp id");
  *n = fk::mlp_nparam();
  return FK_OK;
}

int fk_mlp_get_params(fk_ctx* ctx, int mlp_id, float* params) {
  fk::Mlp* M = get_mlp(ctx, mlp_id);
  if (!M || !params) return fail(ctx, FK_ERR_REGISTRY, "unknown mlp id");
  cudaSetDevice(ctx->device);
  FK_CUDA(cudaMemcpyAsync(params, M->d_master, sizeof(float) * M->n_regions * fk::mlp_nparam(), cudaMemcpyDeviceToHost,
                          ctx->stream));
  FK_CUDA(cudaStreamSynchronize(ctx->stream));
  return FK_OK;
}

int fk_mlp_set_params(fk_ctx* ctx, int mlp_id, const float* params) {
  fk::Mlp* M = get_mlp(ctx, mlp_id);
  if (!M || !params) return fail(ctx, FK_ERR_REGISTRY, "unknown mlp id");
  cudaSetDevice(ctx->device);
  const int rc = fk::mlp_set_params(*M, params, ctx->stream);
  if (rc) return fail(ctx, rc, "mlp: set params failed");
  M->table_grid = 0;  // the gradient table is stale
  return FK_OK;
}

int fk_mlp_train(fk_ctx* ctx, int mlp_id, int n, const double* xy, const double* target, const int* region,
                 int steps, int batch, double lr, unsigned long long seed, float* loss_history) {
  fk::Mlp* M = get_mlp(ctx, mlp_id);
  if (!M) return fail(ctx, FK_ERR_REGISTRY, "unknown mlp id");
  if (n < 1 || !xy || !target || !(lr > 0)) return fail(ctx, FK_ERR_ARG, "mlp train: need samples and lr > 0");
  cudaSetDevice(ctx->device);
  M->barrier_ns = ctx->barrier_ns;
  const int rc = fk::mlp_train(*M, n, xy, target, region, steps, batch, lr, seed, loss_history, ctx->stream, ctx->err);
  if (rc == FK_OK) M->table_grid = 0;
  return rc;
}

int fk_mlp_fit_output(fk_ctx* ctx, int mlp_id, int n, const double* xy, const double* target, const int* region,
                      double ridge) {
  fk::Mlp* M = get_mlp(ctx, mlp_id);
  if (!M) return fail(ctx, FK_ERR_REGISTRY, "unknown mlp id");
  if (n < 1 || !xy || !target) return fail(ctx, FK_ERR_ARG, "mlp fit: need samples");
  cudaSetDevice(ctx->device);
  const int rc = fk::mlp_fit_output(*M, n, xy, target, region, ridge, ctx->stream, ctx->err);
  if (rc == FK_OK) M->table_grid = 0;
  return rc;
}

int fk_mlp_set_trainer(fk_ctx* ctx, int mlp_id, int trainer) {
  fk::Mlp* M = get_mlp(ctx, mlp_id);
  if (!M) return fail(ctx, FK_ERR_REGISTRY, "unknown mlp id");
  if (trainer < FK_TRAIN_AUTO || trainer > FK_TRAIN_STEPS) return fail(ctx, FK_ERR_ARG, "unknown trainer");
  M->trainer = trainer;
  return FK_OK;
}

int fk_mlp_eval(fk_ctx* ctx, int mlp_id, int n, const double* xy, const int* region, double* out) {
  fk::Mlp* M = get_mlp(ctx, mlp_id);
  if (!M) return fail(ctx, FK_ERR_REGISTRY, "unknown mlp id");
  if (n < 0 || (n > 0 && (!xy || !out))) return fail(ctx, FK_ERR_ARG, "null argument");
  cudaSetDevice(ctx->device);
  return fk::mlp_eval_host(*M, n, xy, region, out, ctx->stream, ctx->err);
}

int fk_mlp_loss_grad(fk_ctx* ctx, int mlp_id, int n, const double* xy, const double* target, double* loss,
                     float* grad) {
  fk::Mlp* M = get_mlp(ctx, mlp_id);
  if (!M) return fail(ctx, FK_ERR_REGISTRY, "unknown mlp id");
  if (n < 1 || !xy || !target || !loss || !grad) return fail(ctx, FK_ERR_ARG, "null argument");
  cudaSetDevice(ctx->device);
  return fk::mlp_loss_grad(*M, n, xy, target, loss, grad, ctx->stream, ctx->err);
}

int fk_mlp_build_table(fk_ctx* ctx, int mlp_id, int grid) {
  fk::Mlp* M = get_mlp(ctx, mlp_id);
  if (!M) return fail(ctx, FK_ERR_REGISTRY, "unknown mlp id");
  cudaSetDevice(ctx->device);
  return fk::mlp_build_table(*M, grid, ctx->stream, ctx->err);
}

int fk_mlp_get_table(fk_ctx* ctx, int mlp_id, int* grid, float* table) {
  fk::Mlp* M = get_mlp(ctx, mlp_id);
  if (!M) return fail(ctx, FK_ERR_REGISTRY, "unknown mlp id");
  if (!grid) return fail(ctx, FK_ERR_ARG, "null argument");
  const int G = (M->table_grid >= 2 && M->d_table) ? M->table_grid : 0;
  *grid = G;
  if (table && G) {
    cudaSetDevice(ctx->device);
    const size_t bytes = static_cast<size_t>(M->n_regions) * G * G * 2 * sizeof(float);
    FK_CUDA(cudaMemcpyAsync(table, M->d_table, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    FK_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  return FK_OK;
}

}  // extern "C"

