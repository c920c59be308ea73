// Learned control variate: MLP 2 -> 64 -> 64 -> 64 -> 1 (SiLU), one network
// per region (a patch or the whole domain), trained by the library's own
// kernels:
//  mlp_pass_kernel  32 rows per CTA (8 warps): forward and backward through
//                   the two 64x64 layers on the tensor cores (mma.sync
//                   m16n8k16 BF16, FP32 accumulate), activations staged in
//                   shared memory.  Modes: training-gradient partials on a
//                   Philox-sampled batch, full-data loss gradient, and the
//                   input gradient du_hat/dx (value + gradient at points).
//  mlp_adam_kernel  sums the per-CTA gradient partials in a fixed order,
//                   Adam update of the FP32 master weights, refresh of the
//                   BF16 copies used by the GEMMs (the backward products read
//                   weights and activations transposed with ldmatrix.trans).
//  mlp_train_kernel all training steps in one cooperative launch (pass,
//                   grid barrier, Adam on each CTA's slice, grid barrier).
//  mlp_table        grad u_hat on a grid per region (the inference pass),
//                   read by the path kernel with bilinear interpolation to
//                   form the control term F = -sigma^T grad u_hat of every step.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "../../include/spac_fk.h"
#include "fk_device.cuh"
#include "fk_mlp.h"
#include "fk_mma.cuh"

namespace fk {

Mlp::~Mlp() {
  if (d_tex) cudaDestroyTextureObject(static_cast<cudaTextureObject_t>(d_tex));
  for (void* p : {static_cast<void*>(d_master), d_bf16, static_cast<void*>(d_m), static_cast<void*>(d_v),
                  static_cast<void*>(d_norm), static_cast<void*>(d_partial), static_cast<void*>(d_loss),
                  static_cast<void*>(d_rect), static_cast<void*>(d_table), static_cast<void*>(d_samples),
                  static_cast<void*>(d_hist), static_cast<void*>(d_sync), static_cast<void*>(d_sched), d_fit,
                  d_tabwork})
    if (p) cudaFree(p);
}

namespace {

constexpr int W = 64;
// The training step is latency-bound (a chain of small dependent GEMMs), so
// the batch is spread thin: 32 rows per CTA (128 CTAs at batch 4096) and 8
// warps per CTA, warp w owning the 16 rows 16 (w % 2).. and the 16 columns
// 16 (w / 2).. of every 64-wide product; two warps share each SM
// sub-partition to hide latencies.
#ifndef FK_MLP_ROWS
#define FK_MLP_ROWS 32
#endif
constexpr int kRows = FK_MLP_ROWS;
constexpr int kThreads = 256;
constexpr int kRowGroups = kRows / 16;
constexpr int kWarpRows = kRows / kRowGroups;
constexpr int kMT = kWarpRows / 16;  // m16 tiles per warp
constexpr int kNT = kRows / 16;      // n8 tiles per warp (8 warps = row groups x column groups)
constexpr int kColsPerWarp = 8 * kNT;
constexpr int kColGroups = W / kColsPerWarp;
constexpr int kQuarters = kThreads / W;  // row groups of the per-column sums
// weight-gradient products dW = dp^T h are 64 x 64 whatever the rows per CTA:
// warp w owns output units 16 (w % 4).. and input units 32 (w / 4)..
constexpr int kDwNT = 4;
constexpr int kDwCols = 8 * kDwNT;
static_assert(kThreads / 32 == (W / 16) * (W / kDwCols), "weight-gradient tiling");
constexpr int LD = 72;          // bf16 leading dimension of [rows][64] tiles (144 B rows)
static_assert(kMT == 1 && kWarpRows % 16 == 0, "rows per warp");
static_assert(kThreads / 32 == kRowGroups * (W / kColsPerWarp), "warp tiling");
// largest first-layer weight of the initialisation (normalised input in [-1, 1]^2)
constexpr float kInitScale = 5.0f;
constexpr int OFF_W1 = 0, OFF_B1 = 128, OFF_W2 = 192, OFF_B2 = OFF_W2 + W * W, OFF_W3 = OFF_B2 + W,
              OFF_B3 = OFF_W3 + W * W, OFF_W4 = OFF_B3 + W, OFF_B4 = OFF_W4 + W, NPARAM = OFF_B4 + 1;
constexpr int BF_PER_REGION = 2 * W * W;  // W2, W3 (the backward reads them transposed with ldmatrix.trans)

enum { MODE_TRAIN = 0, MODE_LOSSGRAD = 1, MODE_GRADX = 2 };

// SiLU and its derivative with the logistic function from the SFU tanh:
// sigmoid(z) = 1/2 + tanh(z/2)/2 (tanh.approx.f32, max rel. error ~2^-11,
// below the BF16 rounding these values go through).
__device__ __forceinline__ float tanh_approx(float v) {
  float r;
  asm("tanh.approx.f32 %0, %1;" : "=f"(r) : "f"(v));
  return r;
}
__device__ __forceinline__ float silu_f(float z, float& dsilu) {
  const float s = fmaf(0.5f, tanh_approx(0.5f * z), 0.5f);
  dsilu = s * (1.0f + z * (1.0f - s));
  return z * s;
}

struct PassArgs {
  int mode, n_regions, ctas_per_region, rows_per_cta;
  const float* params;          // [R][NPARAM]
  const __nv_bfloat16* wbf;     // [R][2][W*W]: W2, W3
  const float4* norm;           // per region: (lo_x, lo_y, scale_x, scale_y)
  // samples (TRAIN / LOSSGRAD): region r owns [sample_off[r], sample_off[r+1])
  const float4* samples;        // (x, y, target, -)
  const int* sample_off;
  uint32_t seed0, seed1, step;
  float inv_batch;              // 1 / rows per region that contribute to the loss
  float* partial;               // [R][C][NPARAM]
  float* loss;                  // [R][C]
  float* loss_add;              // if set: the CTA's loss times loss_add_scale is added here instead
  float loss_add_scale;
  // GRADX
  int n_points;
  const float2* points;
  const int* point_region;      // may be null (region 0)
  float* out;                   // [n][3]
  float* feat;                  // GRADX: if set, the layer-3 activations [n][W] instead (forward only)
};

struct Smem {
  __nv_bfloat16 w2[W * LD], w3[W * LD];
  __nv_bfloat16 h1[kRows * LD], h2[kRows * LD], s1[kRows * LD], s2[kRows * LD];
  // h3 and s3 are adjacent: after the layer-3 backward they hold dp1 in FP32
  __nv_bfloat16 h3[kRows * LD], s3[kRows * LD];
  __nv_bfloat16 dp[kRows * LD];
  float w1[2 * W], b1[W], b2[W], b3[W], w4[W], b4;
  float z[kRows][2], tgt[kRows], dO[kRows], o[kRows];
  float o_part[kColGroups][kRows];   // output-unit partial sums of the column groups
  float csum[7][kQuarters][W];       // per-column gradient sums of the row quarters
  int valid[kRows];
};

// One pass over a CTA's rows (see the modes above).  Shared by the one-step
// kernel and the persistent training kernel; the weights are read through
// L2 (ld.global.cg), since the persistent kernel rewrites them between passes.
__device__ void mlp_pass_body(const PassArgs& a, int region, int cta, int grid_x, unsigned char* smem_raw) {
  Smem& S = *reinterpret_cast<Smem*>(smem_raw);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int g = lane >> 2, t4 = lane & 3;
  const float* P = a.params + static_cast<long long>(region) * NPARAM;
  const __nv_bfloat16* WB = a.wbf + static_cast<long long>(region) * BF_PER_REGION;
  int n_tiles, row0;
  if (a.mode == MODE_GRADX) {
    n_tiles = 1;
    row0 = (cta + region * grid_x) * kRows;
  } else {
    n_tiles = a.rows_per_cta / kRows;
    row0 = cta * a.rows_per_cta;
  }
  // row r of a tile's samples (GRADX: points; TRAIN: Philox-drawn samples;
  // LOSSGRAD: consecutive samples)
  auto fetch = [&](int tile, int r, float& x, float& y, float& tg, int& valid) {
    x = 0.f; y = 0.f; tg = 0.f; valid = 0;
    if (a.mode == MODE_GRADX) {
      const int pi = row0 + r;
      if (pi < a.n_points) {
        const float2 p = a.points[pi];
        x = p.x; y = p.y; valid = 1;
      }
    } else {
      const int lo = a.sample_off[region], cnt = a.sample_off[region + 1] - lo;
      const int gr = row0 + tile * kRows + r;  // row of the region's batch
      if (cnt > 0) {
        int si;
        if (a.mode == MODE_TRAIN) {
          const uint4 rr = philox10(make_uint4(a.step, static_cast<uint32_t>(gr), static_cast<uint32_t>(region), 0x6d6c70u),
                                    a.seed0, a.seed1);
          si = lo + static_cast<int>(rr.x % static_cast<uint32_t>(cnt));
          valid = 1;
        } else {
          si = lo + gr;
          valid = gr < cnt;
          if (!valid) si = lo;
        }
        const float4 s = a.samples[si];
        x = s.x; y = s.y; tg = s.z;
      }
    }
  };
  // the first tile's sample loads go out before the weight loads, so the
  // two L2 round trips overlap
  float px = 0.f, py = 0.f, ptg = 0.f;
  int pvalid = 0;
  if (tid < kRows) fetch(0, tid, px, py, ptg, pvalid);
  // weights into shared memory, 8 bf16 (16 bytes) per load
  for (int e8 = tid; e8 < W * W / 8; e8 += kThreads) {
    const int r = (e8 * 8) / W, c = (e8 * 8) % W;
    const uint4* src = reinterpret_cast<const uint4*>(WB) + e8;
    *reinterpret_cast<uint4*>(&S.w2[r * LD + c]) = __ldcg(src);
    *reinterpret_cast<uint4*>(&S.w3[r * LD + c]) = __ldcg(src + W * W / 8);
  }
  for (int e = tid; e < 2 * W; e += kThreads) S.w1[e] = __ldcg(P + OFF_W1 + e);
  for (int e = tid; e < W; e += kThreads) {
    S.b1[e] = __ldcg(P + OFF_B1 + e);
    S.b2[e] = __ldcg(P + OFF_B2 + e);
    S.b3[e] = __ldcg(P + OFF_B3 + e);
    S.w4[e] = __ldcg(P + OFF_W4 + e);
  }
  if (tid == 0) S.b4 = __ldcg(P + OFF_B4);
  const float4 nm = a.norm[region];
  const bool train = a.mode != MODE_GRADX;

  // warp tile: rows m0.., columns n0.. of every 64x64 product
  const int m0 = (warp % kRowGroups) * kWarpRows, n0 = (warp / kRowGroups) * kColsPerWarp;
  // per-column sums: thread <-> (column cj, row quarter cq)
  const int cj = tid % W, cq = tid / W;
  constexpr int kQRows = kRows / kQuarters;
  // persistent gradient accumulators: this warp's (16-row, 32-column) tile of
  // the 64x64 dW2 / dW3 (output unit x input unit, summed over the rows)
  const int mw = (warp % (W / 16)) * 16, nw = (warp / (W / 16)) * kDwCols;
  float cW2[1][kDwNT][4], cW3[1][kDwNT][4];
#pragma unroll
  for (int j = 0; j < kDwNT; ++j)
#pragma unroll
    for (int q = 0; q < 4; ++q) cW2[0][j][q] = cW3[0][j][q] = 0.f;
  float gW4 = 0.f, gB3 = 0.f, gB2 = 0.f, gB1 = 0.f, gW10 = 0.f, gW11 = 0.f, gB4 = 0.f, lsum = 0.f;

  __syncthreads();

  for (int tile = 0; tile < n_tiles; ++tile) {
    // ---- samples: row tid of this tile
    if (tid < kRows) {
      const int r = tid;
      float x = px, y = py, tg = ptg;
      int valid = pvalid;
      if (tile > 0) fetch(tile, r, x, y, tg, valid);
      const float z0 = (x - nm.x) * nm.z, z1 = (y - nm.y) * nm.w;
      S.z[r][0] = z0; S.z[r][1] = z1; S.tgt[r] = tg; S.valid[r] = valid;
    }
    __syncthreads();
    // layer 1 (K = 2) in FP32; thread <-> (row, unit), unit-contiguous stores
    for (int e = tid; e < kRows * W; e += kThreads) {
      const int r = e >> 6, j = e & (W - 1);
      const float p = fmaf(S.w1[2 * j], S.z[r][0], fmaf(S.w1[2 * j + 1], S.z[r][1], S.b1[j]));
      float ds;
      const float hv = silu_f(p, ds);
      S.h1[r * LD + j] = __float2bfloat16_rn(hv);
      S.s1[r * LD + j] = __float2bfloat16_rn(ds);
    }
    __syncthreads();
    // ---- layers 2 and 3 on the tensor cores, one (16-row, 32-column) tile per warp
    for (int layer = 0; layer < 2; ++layer) {
      const __nv_bfloat16* Ain = layer == 0 ? S.h1 : S.h2;
      const __nv_bfloat16* Bw = layer == 0 ? S.w2 : S.w3;
      const float* bias = layer == 0 ? S.b2 : S.b3;
      __nv_bfloat16* Hout = layer == 0 ? S.h2 : S.h3;
      __nv_bfloat16* Sout = layer == 0 ? S.s2 : S.s3;
      float c[kMT][kNT][4];
#pragma unroll
      for (int mt = 0; mt < kMT; ++mt)
#pragma unroll
        for (int nt = 0; nt < kNT; ++nt)
#pragma unroll
          for (int q = 0; q < 4; ++q) c[mt][nt][q] = 0.f;
      warp_gemm_tn<kMT, kNT, W>(c, Ain, LD, m0, Bw, LD, n0, lane);
      float orow[kMT][2] = {};
#pragma unroll
      for (int mt = 0; mt < kMT; ++mt)
#pragma unroll
        for (int nt = 0; nt < kNT; ++nt)
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const int r = m0 + mt * 16 + g + ((q >> 1) << 3);
            const int col = n0 + nt * 8 + 2 * t4 + (q & 1);
            float ds;
            const float hv = silu_f(c[mt][nt][q] + bias[col], ds);
            Hout[r * LD + col] = __float2bfloat16_rn(hv);
            Sout[r * LD + col] = __float2bfloat16_rn(ds);
            if (layer == 1) {
              orow[mt][q >> 1] += S.w4[col] * hv;
              if (a.feat && row0 + r < a.n_points) a.feat[static_cast<long long>(row0 + r) * W + col] = hv;
            }
          }
      if (layer == 1) {
        // output unit: this warp's column half of each row, reduced over the quad
#pragma unroll
        for (int mt = 0; mt < kMT; ++mt)
#pragma unroll
          for (int hh = 0; hh < 2; ++hh) {
            float v = orow[mt][hh];
            v += __shfl_xor_sync(0xffffffffu, v, 1);
            v += __shfl_xor_sync(0xffffffffu, v, 2);
            if (t4 == 0) S.o_part[n0 / kColsPerWarp][m0 + mt * 16 + g + hh * 8] = v;
          }
      }
      __syncthreads();
    }
    if (a.feat) return;  // features only (uniform over the CTA)
    // ---- output gradient and dp3 = dO * w4 * silu'(p3)
    if (tid < kRows) {
      const int r = tid;
      float o = S.b4;
#pragma unroll
      for (int cg = 0; cg < kColGroups; ++cg) o += S.o_part[cg][r];
      S.o[r] = o;
      float d;
      if (a.mode == MODE_GRADX) {
        d = 1.f;
      } else {
        const float e = S.valid[r] ? (o - S.tgt[r]) : 0.f;
        lsum += e * e;
        d = 2.f * e * a.inv_batch;
      }
      S.dO[r] = d;
    }
    __syncthreads();
    for (int e = tid; e < kRows * W; e += kThreads) {
      const int r = e >> 6, j = e & (W - 1);
      const __nv_bfloat16 vb = __float2bfloat16_rn(S.dO[r] * S.w4[j] * __bfloat162float(S.s3[r * LD + j]));
      S.dp[r * LD + j] = vb;
    }
    __syncthreads();
    // layer-3 backward: dW3 += dp3^T h2, db3, dW4, db4; dh2 = dp3 W3
    if (train) {
      // dW3[out][in] = sum_r dp[r][out] h2[r][in]: both operands read transposed
      warp_gemm<1, kDwNT, kRows, true, true>(cW3, S.dp, LD, mw, S.h2, LD, nw, lane);
      for (int r = cq * kQRows; r < (cq + 1) * kQRows; ++r) {
        gW4 += S.dO[r] * __bfloat162float(S.h3[r * LD + cj]);
        gB3 += __bfloat162float(S.dp[r * LD + cj]);
        if (cj == 0) gB4 += S.dO[r];
      }
    }
    {
      float c[kMT][kNT][4];
#pragma unroll
      for (int mt = 0; mt < kMT; ++mt)
#pragma unroll
        for (int nt = 0; nt < kNT; ++nt)
#pragma unroll
          for (int q = 0; q < 4; ++q) c[mt][nt][q] = 0.f;
      // dh2[r][in] = sum_out dp[r][out] W3[out][in]: W3 read transposed
      warp_gemm<kMT, kNT, W, false, true>(c, S.dp, LD, m0, S.w3, LD, n0, lane);
      __syncthreads();  // everyone is done reading dp of layer 3
#pragma unroll
      for (int mt = 0; mt < kMT; ++mt)
#pragma unroll
        for (int nt = 0; nt < kNT; ++nt)
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const int r = m0 + mt * 16 + g + ((q >> 1) << 3);
            const int col = n0 + nt * 8 + 2 * t4 + (q & 1);
            const __nv_bfloat16 vb = __float2bfloat16_rn(c[mt][nt][q] * __bfloat162float(S.s2[r * LD + col]));
            S.dp[r * LD + col] = vb;
          }
    }
    __syncthreads();
    // layer-2 backward: dW2 += dp2^T h1, db2; dh1 = dp2 W2
    if (train) {
      warp_gemm<1, kDwNT, kRows, true, true>(cW2, S.dp, LD, mw, S.h1, LD, nw, lane);
      for (int r = cq * kQRows; r < (cq + 1) * kQRows; ++r) gB2 += __bfloat162float(S.dp[r * LD + cj]);
    }
    {
      float c[kMT][kNT][4];
#pragma unroll
      for (int mt = 0; mt < kMT; ++mt)
#pragma unroll
        for (int nt = 0; nt < kNT; ++nt)
#pragma unroll
          for (int q = 0; q < 4; ++q) c[mt][nt][q] = 0.f;
      warp_gemm<kMT, kNT, W, false, true>(c, S.dp, LD, m0, S.w2, LD, n0, lane);
      __syncthreads();
      // dp1 = dh1 * silu'(p1), kept in FP32 in the (now free) h3 / s3 area as pairs
      static_assert(sizeof(float) * kRows * W <= 2 * sizeof(__nv_bfloat16) * kRows * LD, "dp1 overlay");
      float* dp1 = reinterpret_cast<float*>(S.h3);  // [kRows][W] FP32 over h3 + s3
#pragma unroll
      for (int mt = 0; mt < kMT; ++mt)
#pragma unroll
        for (int nt = 0; nt < kNT; ++nt)
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const int r = m0 + mt * 16 + g + ((q >> 1) << 3);
            const int col = n0 + nt * 8 + 2 * t4 + (q & 1);
            dp1[r * W + col] = c[mt][nt][q] * __bfloat162float(S.s1[r * LD + col]);
          }
    }
    __syncthreads();
    {
      const float* dp1 = reinterpret_cast<const float*>(S.h3);
      if (a.mode == MODE_GRADX && tid < kRows) {
        const int r = tid, pi = row0 + r;
        float gx = 0.f, gy = 0.f;
        for (int j = 0; j < W; ++j) {
          gx += dp1[r * W + j] * S.w1[2 * j];
          gy += dp1[r * W + j] * S.w1[2 * j + 1];
        }
        if (pi < a.n_points) {
          a.out[3 * pi] = S.o[r];
          a.out[3 * pi + 1] = gx * nm.z;
          a.out[3 * pi + 2] = gy * nm.w;
        }
      } else if (a.mode != MODE_GRADX) {
        for (int r = cq * kQRows; r < (cq + 1) * kQRows; ++r) {
          const float d = dp1[r * W + cj];
          gB1 += d;
          gW10 += d * S.z[r][0];
          gW11 += d * S.z[r][1];
        }
      }
    }
    __syncthreads();
  }
  if (a.mode == MODE_GRADX) return;
  // ---- write this CTA's gradient partial
  float* out = a.partial + (static_cast<long long>(region) * a.ctas_per_region + cta) * NPARAM;
#pragma unroll
  for (int nt = 0; nt < kDwNT; ++nt)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int r = mw + g + ((q >> 1) << 3);
      const int col = nw + nt * 8 + 2 * t4 + (q & 1);
      out[OFF_W2 + r * W + col] = cW2[0][nt][q];
      out[OFF_W3 + r * W + col] = cW3[0][nt][q];
    }
  // per-column sums: the row quarters combined in a fixed order
  S.csum[0][cq][cj] = gW4;
  S.csum[1][cq][cj] = gB3;
  S.csum[2][cq][cj] = gB2;
  S.csum[3][cq][cj] = gB1;
  S.csum[4][cq][cj] = gW10;
  S.csum[5][cq][cj] = gW11;
  S.csum[6][cq][cj] = gB4;
  __syncthreads();
  if (tid < W) {
    const int j = tid;
    float v[7];
#pragma unroll
    for (int k = 0; k < 7; ++k) {
      v[k] = S.csum[k][0][j];
#pragma unroll
      for (int qd = 1; qd < kQuarters; ++qd) v[k] += S.csum[k][qd][j];
    }
    out[OFF_W4 + j] = v[0];
    out[OFF_B3 + j] = v[1];
    out[OFF_B2 + j] = v[2];
    out[OFF_B1 + j] = v[3];
    out[OFF_W1 + 2 * j] = v[4];
    out[OFF_W1 + 2 * j + 1] = v[5];
    if (j == 0) {
      float b4 = S.csum[6][0][0];
      for (int qd = 1; qd < kQuarters; ++qd) b4 += S.csum[6][qd][0];
      out[OFF_B4] = b4;
    }
  }
  // loss partial (sum of squared errors of this CTA): warp sums, then the warps in order
  __shared__ float red[kThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
  if (lane == 0) red[warp] = lsum;
  __syncthreads();
  if (tid == 0) {
    float l = red[0];
    for (int w = 1; w < kThreads / 32; ++w) l += red[w];
    if (a.loss_add) atomicAdd(a.loss_add, l * a.loss_add_scale);  // off the training step's critical path
    else a.loss[region * a.ctas_per_region + cta] = l;
  }
}

__global__ void __launch_bounds__(kThreads, 1) mlp_pass_kernel(const PassArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  mlp_pass_body(a, blockIdx.y, blockIdx.x, gridDim.x, smem_raw);
}

// Adam update of parameter e (= region r, index p) with gradient gsum; keeps
// the BF16 copies (W and W^T of the two 64x64 layers) in step.
__device__ __forceinline__ void adam_apply_vals(long long e, int r, int p, float gsum, float m_old, float v_old,
                                                float th_old, float* params, __nv_bfloat16* wbf, float* m, float* v,
                                                float lr, float b1, float b2, float eps, float bc1, float bc2) {
  const float mm = b1 * m_old + (1.f - b1) * gsum;
  const float vv = b2 * v_old + (1.f - b2) * gsum * gsum;
  m[e] = mm;
  v[e] = vv;
  const float th = th_old - lr * (mm / bc1) / (sqrtf(vv / bc2) + eps);
  params[e] = th;
  __nv_bfloat16* B = wbf + static_cast<long long>(r) * BF_PER_REGION;
  const __nv_bfloat16 tb = __float2bfloat16_rn(th);
  if (p >= OFF_W2 && p < OFF_W2 + W * W)
    B[p - OFF_W2] = tb;
  else if (p >= OFF_W3 && p < OFF_W3 + W * W)
    B[W * W + (p - OFF_W3)] = tb;
}
__device__ __forceinline__ void adam_apply(long long e, int r, int p, float gsum, float* params, __nv_bfloat16* wbf,
                                           float* m, float* v, float lr, float b1, float b2, float eps, float bc1,
                                           float bc2) {
  adam_apply_vals(e, r, p, gsum, m[e], v[e], params[e], params, wbf, m, v, lr, b1, b2, eps, bc1, bc2);
}

// Sum of partials (fixed order) and Adam update; refreshes the BF16 copies.
__global__ void mlp_adam_kernel(float* params, __nv_bfloat16* wbf, float* m, float* v, const float* partial,
                                const float* loss, int n_regions, int ctas, float lr, float b1, float b2, float eps,
                                float bc1, float bc2, int apply, float* grad_out, float* hist, float loss_scale) {
  // 8 lanes per parameter: lane q sums the partials c = q, q+8, ... (fixed
  // order), then a fixed shuffle tree combines the 8 lane sums
  const long long total = static_cast<long long>(n_regions) * NPARAM;
  const int sub = threadIdx.x & 7;
  const long long lanes = static_cast<long long>(gridDim.x) * blockDim.x;
  const long long rounds = (total * 8 + lanes - 1) / lanes;
  for (long long it = 0; it < rounds; ++it) {
    const long long e = (it * lanes + blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x) >> 3;
    const bool live = e < total;
    float part = 0.f;
    int r = 0, p = 0;
    if (live) {
      r = static_cast<int>(e / NPARAM);
      p = static_cast<int>(e % NPARAM);
      const float* src = partial + static_cast<long long>(r) * ctas * NPARAM + p;
      float a0 = 0.f, a1 = 0.f;
      int c = sub;
      for (; c + 8 < ctas; c += 16) {
        a0 += __ldg(src + static_cast<long long>(c) * NPARAM);
        a1 += __ldg(src + static_cast<long long>(c + 8) * NPARAM);
      }
      if (c < ctas) a0 += __ldg(src + static_cast<long long>(c) * NPARAM);
      part = a0 + a1;
    }
    part += __shfl_xor_sync(0xffffffffu, part, 1);
    part += __shfl_xor_sync(0xffffffffu, part, 2);
    part += __shfl_xor_sync(0xffffffffu, part, 4);
    if (!live || sub != 0) continue;
    const float gsum = part;
    if (grad_out) grad_out[e] = gsum;
    if (!apply) continue;
    adam_apply(e, r, p, gsum, params, wbf, m, v, lr, b1, b2, eps, bc1, bc2);
  }
  if (hist && blockIdx.x == 0 && threadIdx.x == 0) {
    float s = 0.f;
    for (int i = 0; i < n_regions * ctas; ++i) s += loss[i];
    *hist = s * loss_scale;
  }
}

// ---------------------------------------------------- persistent training --
// All training steps in one cooperative launch: every CTA runs its pass,
// the grid meets at a barrier, each CTA applies Adam to its slice of the
// parameters (the partials summed in a fixed CTA order, as in
// mlp_adam_kernel), and the grid meets again before the next pass reads the
// new weights.  The barrier is a monotonic arrival counter; its waits give
// up after kBarrierNs, set the error word and end the kernel.
struct TrainArgs {
  PassArgs a;
  float* params;
  __nv_bfloat16* wbf;
  float* m;
  float* v;
  unsigned* bar;     // arrival counter, zeroed before the launch
  int* err;          // error word, zeroed before the launch
  float* hist;       // loss per step
  float loss_scale;
  int steps;
  long long t0;      // Adam steps taken before this launch
  const float* sched;  // per step: learning rate, 1 - beta1^t, 1 - beta2^t
  unsigned long long barrier_ns;  // a barrier wait gives up after this
};
constexpr unsigned long long kBarrierNs = 5000000000ull;  // default barrier_ns
// Adam on the CTA partials: kAdamGroups thread groups of kAdamRound, each
// loading up to kMaxPartialLoads partials per parameter; the persistent grid
// has at most 2 x 80 = 160 CTAs per region (one per SM of a 152-SM part)
constexpr int kAdamGroups = 2;
constexpr int kAdamRound = kThreads / kAdamGroups;
constexpr int kMaxPartialLoads = 80;
constexpr int kMaxPersistentCtas = kAdamGroups * kMaxPartialLoads;

__device__ __forceinline__ unsigned long long mlp_global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Arrival with release semantics (the CTA's writes, gathered by the block
// barrier, become visible before the count), wait with acquire loads.
__device__ __forceinline__ void bar_arrive_release(unsigned* bar) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(bar), "r"(1u) : "memory");
}
__device__ __forceinline__ unsigned bar_load_acquire(const unsigned* bar) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(bar) : "memory");
  return v;
}

__device__ bool grid_barrier(unsigned* bar, unsigned target, int* err, unsigned long long limit_ns) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    bar_arrive_release(bar);
    const unsigned long long t0 = mlp_global_ns();
    while (bar_load_acquire(bar) < target) {
      if (*reinterpret_cast<volatile int*>(err) != 0) { ok = 0; break; }
      if (mlp_global_ns() - t0 > limit_ns) {
        atomicExch(err, 1);
        ok = 0;
        break;
      }
      __nanosleep(32);
    }
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

__global__ void __launch_bounds__(kThreads, 1) mlp_train_kernel(const TrainArgs t) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int nb = gridDim.x * gridDim.y;
  const int bid = blockIdx.y * gridDim.x + blockIdx.x;
  const int ctas = t.a.ctas_per_region;
  const long long total = static_cast<long long>(t.a.n_regions) * NPARAM;
  const long long per = (total + nb - 1) / nb;
  const long long e0 = bid * per, e1 = min(total, e0 + per);
  PassArgs a = t.a;
  unsigned target = 0;
  a.loss_add_scale = t.loss_scale;
  for (int s = 0; s < t.steps; ++s) {
    a.step = static_cast<uint32_t>(t.t0 + s);
    a.loss_add = t.hist + s;  // (zeroed before the launch)
    mlp_pass_body(a, blockIdx.y, blockIdx.x, gridDim.x, smem_raw);
    target += nb;
    if (!grid_barrier(t.bar, target, t.err, t.barrier_ns)) return;
    // the step's learning rate and bias corrections, computed on the host
    const float lr_t = __ldg(t.sched + 3 * s), bc1 = __ldg(t.sched + 3 * s + 1), bc2 = __ldg(t.sched + 3 * s + 2);
    // Thread (g, j): parameter e0 + j of a kAdamRound-parameter round (one
    // round covers a CTA's slice) and the CTA partials g, g + kAdamGroups, ...
    // in order; a warp's loads of one CTA's partial are 32 consecutive
    // floats.  The step is bound by L2 latency, so every thread issues all its
    // loads (predicated), and the parameter's Adam state with them, before it
    // adds any; the group sums are combined in a fixed order.
    __shared__ float s_part[kAdamGroups][kAdamRound];
    const int j = threadIdx.x % kAdamRound, grp = threadIdx.x / kAdamRound;
    for (long long base = e0; base < e1; base += kAdamRound) {
      const long long e = base + j;
      const bool live = e < e1;
      int r = 0, p = 0;
      float part = 0.f, m_old = 0.f, v_old = 0.f, th_old = 0.f;
      if (live) {
        r = static_cast<int>(e / NPARAM);
        p = static_cast<int>(e % NPARAM);
        if (grp == 0) {
          m_old = t.m[e];
          v_old = t.v[e];
          th_old = t.params[e];
        }
        const float* src = a.partial + static_cast<long long>(r) * ctas * NPARAM + p;
        float vals[kMaxPartialLoads];
#pragma unroll
        for (int i = 0; i < kMaxPartialLoads; ++i) {
          const int c = grp + kAdamGroups * i;
          vals[i] = c < ctas ? __ldcg(src + static_cast<long long>(c) * NPARAM) : 0.f;
        }
#pragma unroll
        for (int i = 0; i < kMaxPartialLoads; ++i) part += vals[i];
      }
      s_part[grp][j] = part;
      __syncthreads();
      if (grp == 0 && live) {
        float gsum = s_part[0][j];
#pragma unroll
        for (int q = 1; q < kAdamGroups; ++q) gsum += s_part[q][j];
        adam_apply_vals(e, r, p, gsum, m_old, v_old, th_old, t.params, t.wbf, t.m, t.v, lr_t, 0.9f, 0.999f, 1e-8f,
                        bc1, bc2);
      }
      __syncthreads();
    }
    target += nb;
    if (!grid_barrier(t.bar, target, t.err, t.barrier_ns)) return;
  }
}

__global__ void mlp_refresh_bf16(const float* params, __nv_bfloat16* wbf, int n_regions) {
  const long long total = static_cast<long long>(n_regions) * W * W;
  for (long long e = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; e < total;
       e += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int r = static_cast<int>(e / (W * W)), q = static_cast<int>(e % (W * W));
    const float* P = params + static_cast<long long>(r) * NPARAM;
    __nv_bfloat16* B = wbf + static_cast<long long>(r) * BF_PER_REGION;
    B[q] = __float2bfloat16_rn(P[OFF_W2 + q]);
    B[W * W + q] = __float2bfloat16_rn(P[OFF_W3 + q]);
  }
}

// grid point (i, j) of region r: out table[r][j][i] = (du/dx, du/dy)
__global__ void mlp_grid_points(const double* rects, int n_regions, int G, float2* pts, int* reg) {
  const long long total = static_cast<long long>(n_regions) * G * G;
  for (long long e = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; e < total;
       e += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int r = static_cast<int>(e / (G * G)), q = static_cast<int>(e % (G * G)), j = q / G, i = q % G;
    const double* R = rects + 4 * r;
    pts[e] = make_float2(static_cast<float>(R[0] + (R[2] - R[0]) * i / (G - 1)),
                         static_cast<float>(R[1] + (R[3] - R[1]) * j / (G - 1)));
    reg[e] = r;
  }
}

// Output-layer least squares: Gram matrix of A = [features, 1] and A^T t.
// gram: (W + 1) x (W + 2) FP64, row i = (A^T A)[i][0..W], (A^T t)[i]; one
// CTA per 64 samples adds its FP32 partial with FP64 atomics.
constexpr int kGramRows = 64;
constexpr int kGramCols = W + 2;
__global__ void __launch_bounds__(256) mlp_gram_kernel(const float* feat, const float* tgt, int n, double* gram) {
  __shared__ float A[kGramRows][W + 2];  // features, 1, target
  const int r0 = blockIdx.x * kGramRows;
  for (int e = threadIdx.x; e < kGramRows * (W + 2); e += blockDim.x) {
    const int r = e / (W + 2), c = e % (W + 2), row = r0 + r;
    float v = 0.f;
    if (row < n) v = c < W ? feat[static_cast<long long>(row) * W + c] : (c == W ? 1.f : tgt[row]);
    A[r][c] = v;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < (W + 1) * kGramCols; e += blockDim.x) {
    const int i = e / kGramCols, j = e % kGramCols;
    if (j < W + 1 && j < i) continue;  // lower triangle mirrored by the solver
    float acc = 0.f;
    for (int r = 0; r < kGramRows; ++r) acc = fmaf(A[r][i], A[r][j], acc);
    atomicAdd(&gram[e], static_cast<double>(acc));
  }
}

// Ridge solve (A^T A + lambda I) w = A^T t by Cholesky in FP64, lambda =
// ridge x mean diagonal; writes W4 (w[0..W)) and b4 (w[W]) into the region's
// FP32 parameters.  flag is set if the matrix is not positive definite.
// One CTA: right-looking factorisation with the pivot's reciprocal (one FP64
// division per column) and the trailing update over the lower triangle only,
// then both triangular solves column by column across the CTA (a row's
// unknown, then every later row updated in parallel), instead of one thread
// walking the 65 x 65 triangles.
__global__ void __launch_bounds__(256) mlp_lsq_kernel(const double* gram, float* params, double ridge, int* flag) {
  constexpr int N = W + 1;
  __shared__ double M[N][N + 1];
  __shared__ double rhs[N];
  __shared__ double rinv[N];
  __shared__ double s_lam;
  __shared__ int s_bad;
  const int tid = threadIdx.x;
  if (tid == 0) {
    double tr = 0.0;
    for (int i = 0; i < N; ++i) tr += gram[i * kGramCols + i];
    s_lam = ridge * tr / N;
    s_bad = 0;
  }
  __syncthreads();
  for (int e = tid; e < N * N; e += blockDim.x) {
    const int i = e / N, j = e % N;
    const double v = (j >= i) ? gram[i * kGramCols + j] : gram[j * kGramCols + i];
    M[i][j] = v + (i == j ? s_lam : 0.0);
  }
  for (int i = tid; i < N; i += blockDim.x) rhs[i] = gram[i * kGramCols + W + 1];
  __syncthreads();
  // M = L L^T, L in the lower triangle
  for (int k = 0; k < N; ++k) {
    if (tid == 0) {
      const double d = M[k][k];
      if (!(d > 0.0)) s_bad = 1;
      const double piv = sqrt(d > 0.0 ? d : 1.0);
      M[k][k] = piv;
      rinv[k] = 1.0 / piv;
    }
    __syncthreads();
    const double r = rinv[k];
    for (int i = k + 1 + tid; i < N; i += blockDim.x) M[i][k] *= r;
    __syncthreads();
    // rows i > k, columns k < j <= i: T (T + 1) / 2 entries, T = N - k - 1
    const int T = N - k - 1;
    for (int e = tid; e < T * (T + 1) / 2; e += blockDim.x) {
      // e -> (a, b), 0 <= b <= a < T, row-major over the triangle
      int a = static_cast<int>((sqrtf(8.f * e + 1.f) - 1.f) * 0.5f);
      if ((a + 1) * (a + 2) / 2 <= e) ++a;
      if (a * (a + 1) / 2 > e) --a;
      const int b = e - a * (a + 1) / 2;
      const int i = k + 1 + a, j = k + 1 + b;
      M[i][j] -= M[i][k] * M[j][k];
    }
    __syncthreads();
  }
  // L y = rhs: y_i, then every later row updated
  for (int i = 0; i < N; ++i) {
    if (tid == 0) rhs[i] *= rinv[i];
    __syncthreads();
    const double yi = rhs[i];
    for (int j = i + 1 + tid; j < N; j += blockDim.x) rhs[j] -= M[j][i] * yi;
    __syncthreads();
  }
  // L^T w = y: w_i, then every earlier row updated
  for (int i = N - 1; i >= 0; --i) {
    if (tid == 0) rhs[i] *= rinv[i];
    __syncthreads();
    const double wi = rhs[i];
    for (int j = tid; j < i; j += blockDim.x) rhs[j] -= M[i][j] * wi;
    __syncthreads();
  }
  if (tid == 0) {
    if (s_bad) {
      atomicOr(flag, 1);
    } else {
      for (int i = 0; i < W; ++i) params[OFF_W4 + i] = static_cast<float>(rhs[i]);
      params[OFF_B4] = static_cast<float>(rhs[W]);
    }
  }
}

__global__ void mlp_pack_table(const float* eval, long long n, float2* table) {
  for (long long e = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; e < n;
       e += static_cast<long long>(gridDim.x) * blockDim.x)
    table[e] = make_float2(eval[3 * e + 1], eval[3 * e + 2]);
}

}  // namespace

size_t mlp_pass_smem() { return sizeof(Smem); }
int mlp_nparam() { return NPARAM; }

// Evaluates (u_hat, du/dx, du/dy) at n device points of one region.
cudaError_t mlp_eval_device(const float* params, const void* wbf, const float4* norm, int n, const float2* d_pts,
                            float* d_out, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  PassArgs a;
  std::memset(&a, 0, sizeof(a));
  a.mode = MODE_GRADX;
  a.n_regions = 1;
  a.params = params;
  a.wbf = static_cast<const __nv_bfloat16*>(wbf);
  a.norm = norm;
  a.n_points = n;
  a.points = d_pts;
  a.out = d_out;
  cudaError_t e = cudaFuncSetAttribute(mlp_pass_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(sizeof(Smem)));
  if (e != cudaSuccess) return e;
  const int tiles = (n + kRows - 1) / kRows;
  mlp_pass_kernel<<<dim3(tiles, 1), kThreads, sizeof(Smem), s>>>(a);
  return cudaGetLastError();
}

}  // namespace fk

// ============================================================== C ABI =======
// (the context-side parts live in fk_api.cu; these helpers are called there)
namespace fk {

int mlp_init(Mlp& M, int n_regions, const double* rects, unsigned long long seed, cudaStream_t s,
             std::string& err) {
  M.n_regions = n_regions;
  M.n_params = NPARAM;
  M.rects.assign(rects, rects + 4 * n_regions);
  std::vector<float4> norm(n_regions);
  for (int r = 0; r < n_regions; ++r) {
    const double* R = rects + 4 * r;
    if (!(R[2] > R[0] && R[3] > R[1])) { err = "mlp region rectangles must be non-empty"; return FK_ERR_ARG; }
    // (x - lo) * scale maps the rectangle to [-1, 1]^2
    norm[r] = make_float4(static_cast<float>(0.5 * (R[0] + R[2])), static_cast<float>(0.5 * (R[1] + R[3])),
                          static_cast<float>(2.0 / (R[2] - R[0])), static_cast<float>(2.0 / (R[3] - R[1])));
  }
  std::vector<float> p(static_cast<size_t>(n_regions) * NPARAM, 0.f);
  std::mt19937_64 rng(seed);
  auto uni = [&](float a) { return std::uniform_real_distribution<float>(-a, a)(rng); };
  for (int r = 0; r < n_regions; ++r) {
    float* P = p.data() + static_cast<size_t>(r) * NPARAM;
    // First layer: unit j is SiLU(w_j . (z - c_j)) on the normalised input z,
    // with a uniform direction, |w_j| = kInitScale sqrt(U) and its kink
    // through a uniform point c_j of the region, so that the units' kinks
    // cover the region at several widths from the start (with Glorot weights
    // and zero biases every kink passes through the centre, and the output
    // refit of the untrained features reduces the variance of the 8 x 8
    // assembly only 1.8-fold, against ~30-fold with these).  Hidden and
    // output layers: Glorot uniform, zero biases.
    for (int j = 0; j < W; ++j) {
      const float ang = 3.14159265358979f * uni(1.f);
      const float mag = kInitScale * std::sqrt(0.5f * (uni(1.f) + 1.f));
      const float cx = uni(1.f), cy = uni(1.f);
      const float wx = mag * std::cos(ang), wy = mag * std::sin(ang);
      P[OFF_W1 + 2 * j] = wx;
      P[OFF_W1 + 2 * j + 1] = wy;
      P[OFF_B1 + j] = -(wx * cx + wy * cy);
    }
    const float a2 = std::sqrt(6.f / (2 * W)), a4 = std::sqrt(6.f / (W + 1));
    for (int e = 0; e < W * W; ++e) { P[OFF_W2 + e] = uni(a2); P[OFF_W3 + e] = uni(a2); }
    for (int e = 0; e < W; ++e) P[OFF_W4 + e] = uni(a4);
  }
  const size_t np = p.size();
  if (cudaMalloc(&M.d_master, np * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&M.d_m, np * sizeof(float)) != cudaSuccess || cudaMalloc(&M.d_v, np * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&M.d_bf16, static_cast<size_t>(n_regions) * BF_PER_REGION * sizeof(__nv_bfloat16)) != cudaSuccess ||
      cudaMalloc(&M.d_norm, n_regions * sizeof(float4)) != cudaSuccess ||
      cudaMalloc(&M.d_rect, 4 * n_regions * sizeof(double)) != cudaSuccess) {
    err = "mlp: device allocation failed";
    return FK_ERR_CUDA;
  }
  cudaMemcpyAsync(M.d_master, p.data(), np * sizeof(float), cudaMemcpyHostToDevice, s);
  cudaMemsetAsync(M.d_m, 0, np * sizeof(float), s);
  cudaMemsetAsync(M.d_v, 0, np * sizeof(float), s);
  cudaMemcpyAsync(M.d_norm, norm.data(), n_regions * sizeof(float4), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(M.d_rect, rects, 4 * n_regions * sizeof(double), cudaMemcpyHostToDevice, s);
  mlp_refresh_bf16<<<64, 256, 0, s>>>(M.d_master, static_cast<__nv_bfloat16*>(M.d_bf16), n_regions);
  if (cudaStreamSynchronize(s) != cudaSuccess || cudaGetLastError() != cudaSuccess) {
    err = "mlp: init kernels failed";
    return FK_ERR_CUDA;
  }
  return FK_OK;
}

// (on the context's stream, which does not synchronise with the legacy
// default stream: queued training, refit and table work is ordered before it)
int mlp_set_params(Mlp& M, const float* host, cudaStream_t s) {
  const size_t np = static_cast<size_t>(M.n_regions) * NPARAM;
  cudaError_t e = cudaMemcpyAsync(M.d_master, host, np * sizeof(float), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(M.d_m, 0, np * sizeof(float), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(M.d_v, 0, np * sizeof(float), s);
  if (e != cudaSuccess) return FK_ERR_CUDA;
  M.adam_t = 0;
  mlp_refresh_bf16<<<64, 256, 0, s>>>(M.d_master, static_cast<__nv_bfloat16*>(M.d_bf16), M.n_regions);
  return cudaStreamSynchronize(s) == cudaSuccess ? FK_OK : FK_ERR_CUDA;
}

// Uploads (x, y, target) samples grouped by region.
// Grow-only device buffer: reallocated only when `need` exceeds its capacity.
template <typename T>
static cudaError_t grow(T*& p, size_t& cap, size_t need) {
  if (need <= cap && p) return cudaSuccess;
  if (p) cudaFree(p);
  p = nullptr;
  cap = 0;
  void* q = nullptr;
  const cudaError_t e = cudaMalloc(&q, need);
  if (e == cudaSuccess) { p = static_cast<T*>(q); cap = need; }
  return e;
}

static int upload_samples(Mlp& M, int n, const double* xy, const double* target, const int* region,
                          std::vector<int>& off, cudaStream_t s, std::string& err) {
  std::vector<std::vector<float4>> by(M.n_regions);
  for (int i = 0; i < n; ++i) {
    const int r = region ? region[i] : 0;
    if (r < 0 || r >= M.n_regions) { err = "sample region out of range"; return FK_ERR_ARG; }
    by[r].push_back(make_float4(static_cast<float>(xy[2 * i]), static_cast<float>(xy[2 * i + 1]),
                                static_cast<float>(target[i]), 0.f));
  }
  std::vector<float4> flat;
  off.assign(M.n_regions + 1, 0);
  for (int r = 0; r < M.n_regions; ++r) {
    off[r] = static_cast<int>(flat.size());
    flat.insert(flat.end(), by[r].begin(), by[r].end());
  }
  off[M.n_regions] = static_cast<int>(flat.size());
  if (grow(M.d_samples, M.cap_samples,
           std::max<size_t>(flat.size(), 1) * sizeof(float4) + (M.n_regions + 1) * sizeof(int)) != cudaSuccess) {
    err = "mlp: sample allocation failed";
    return FK_ERR_CUDA;
  }
  // (pageable sources: each copy has read its source when it returns)
  int* d_off = reinterpret_cast<int*>(M.d_samples + std::max<size_t>(flat.size(), 1));
  cudaError_t e = cudaSuccess;
  if (!flat.empty()) e = cudaMemcpyAsync(M.d_samples, flat.data(), flat.size() * sizeof(float4), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_off, off.data(), (M.n_regions + 1) * sizeof(int), cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) { err = cudaGetErrorString(e); return FK_ERR_CUDA; }
  M.d_sample_off = d_off;
  return FK_OK;
}

int mlp_train(Mlp& M, int n, const double* xy, const double* target, const int* region, int steps, int batch,
              double lr, unsigned long long seed, float* loss_hist, cudaStream_t s, std::string& err) {
  if (steps < 0 || batch < kRows || batch % kRows) { err = "batch must be a positive multiple of " + std::to_string(kRows); return FK_ERR_ARG; }
  std::vector<int> off;
  int rc = upload_samples(M, n, xy, target, region, off, s, err);
  if (rc) return rc;
  // Persistent training (all steps in one cooperative launch) when the grid
  // fits on the device at once, with as many CTAs (one 64-row tile each) as
  // fit; otherwise one graph-captured pass + Adam launch pair per step.
  int dev = 0, coop = 0, sms = 0, occ = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (cudaFuncSetAttribute(mlp_train_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           static_cast<int>(sizeof(Smem))) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, mlp_train_kernel, kThreads, sizeof(Smem)) != cudaSuccess)
    occ = 0;
  const long long capacity = static_cast<long long>(occ) * sms;
  int rows_per_cta = kRows;
  bool persistent = false;
  if (coop && steps > 0 && capacity > 0 && M.trainer != 2) {
    while (rows_per_cta < batch && batch % (2 * rows_per_cta) == 0 &&
           static_cast<long long>(batch / rows_per_cta) * M.n_regions > capacity)
      rows_per_cta *= 2;
    persistent = static_cast<long long>(batch / rows_per_cta) * M.n_regions <= capacity &&
                 batch / rows_per_cta <= kMaxPersistentCtas;
  }
  if (!persistent) {
    // one 64-row tile per CTA (the step is latency-bound: more CTAs, shorter
    // step); larger tiles per CTA only when the grid would exceed ~4 waves
    rows_per_cta = kRows;
    while (rows_per_cta < 1024 && batch % (2 * rows_per_cta) == 0 &&
           static_cast<long long>(batch / rows_per_cta) * M.n_regions > 4 * 152)
      rows_per_cta *= 2;
  }
  const int ctas = batch / rows_per_cta;
  const size_t np = static_cast<size_t>(M.n_regions) * NPARAM;
  if (grow(M.d_partial, M.cap_partial, np * ctas * sizeof(float)) != cudaSuccess ||
      grow(M.d_loss, M.cap_loss, static_cast<size_t>(M.n_regions) * ctas * sizeof(float)) != cudaSuccess ||
      grow(M.d_hist, M.cap_hist, std::max(steps, 1) * sizeof(float)) != cudaSuccess) {
    err = "mlp: training buffers";
    return FK_ERR_CUDA;
  }
  cudaError_t e = cudaFuncSetAttribute(mlp_pass_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(sizeof(Smem)));
  if (e != cudaSuccess) { err = cudaGetErrorString(e); return FK_ERR_CUDA; }
  PassArgs a;
  std::memset(&a, 0, sizeof(a));
  a.mode = MODE_TRAIN;
  a.n_regions = M.n_regions;
  a.ctas_per_region = ctas;
  a.rows_per_cta = rows_per_cta;
  a.params = M.d_master;
  a.wbf = static_cast<const __nv_bfloat16*>(M.d_bf16);
  a.norm = M.d_norm;
  a.samples = M.d_samples;
  a.sample_off = M.d_sample_off;
  a.seed0 = static_cast<uint32_t>(seed);
  a.seed1 = static_cast<uint32_t>(seed >> 32);
  a.inv_batch = 1.f / batch;
  a.partial = M.d_partial;
  a.loss = M.d_loss;
  if (M.trainer == 1 && steps > 0 && !persistent) {
    err = "mlp: the grid trainer needs a cooperative launch that fits the device";
    return FK_ERR_ARG;
  }
  if (persistent) {
    if (!M.d_sync && cudaMalloc(&M.d_sync, 2 * sizeof(unsigned)) != cudaSuccess) {
      err = "mlp: training buffers";
      return FK_ERR_CUDA;
    }
    TrainArgs t;
    std::memset(&t, 0, sizeof(t));
    t.a = a;
    t.params = M.d_master;
    t.wbf = static_cast<__nv_bfloat16*>(M.d_bf16);
    t.m = M.d_m;
    t.v = M.d_v;
    t.bar = M.d_sync;
    t.err = reinterpret_cast<int*>(M.d_sync + 1);
    t.hist = M.d_hist;
    t.loss_scale = 1.f / (static_cast<float>(batch) * M.n_regions);
    t.steps = steps;
    t.t0 = M.adam_t;
    t.barrier_ns = M.barrier_ns ? M.barrier_ns : kBarrierNs;
    // learning-rate schedule and Adam bias corrections of every step (the
    // same values as the per-step launches below compute)
    std::vector<float> sched(3 * static_cast<size_t>(steps));
    for (int st = 0; st < steps; ++st) {
      const double tt = static_cast<double>(M.adam_t + st + 1);
      sched[3 * st] = static_cast<float>(lr * (0.01 + 0.99 * 0.5 * (1.0 + std::cos(M_PI * st / std::max(1, steps)))));
      sched[3 * st + 1] = static_cast<float>(1.0 - std::pow(0.9, tt));
      sched[3 * st + 2] = static_cast<float>(1.0 - std::pow(0.999, tt));
    }
    if (grow(M.d_sched, M.cap_sched, sched.size() * sizeof(float)) != cudaSuccess) {
      err = "mlp: training buffers";
      return FK_ERR_CUDA;
    }
    t.sched = M.d_sched;
    e = cudaMemcpyAsync(M.d_sched, sched.data(), sched.size() * sizeof(float), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(M.d_sync, 0, 2 * sizeof(unsigned), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(M.d_hist, 0, std::max(steps, 1) * sizeof(float), s);
    void* args[] = {&t};
    if (e == cudaSuccess)
      e = cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(mlp_train_kernel), dim3(ctas, M.n_regions),
                                      dim3(kThreads), args, sizeof(Smem), s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) { err = cudaGetErrorString(e); return FK_ERR_CUDA; }
    unsigned sync[2] = {0u, 0u};
    if (cudaMemcpy(sync, M.d_sync, sizeof(sync), cudaMemcpyDeviceToHost) != cudaSuccess || sync[1] != 0u) {
      err = "mlp: a training barrier timed out";
      return FK_ERR_CUDA;
    }
    M.adam_t += steps;
    if (loss_hist) cudaMemcpy(loss_hist, M.d_hist, steps * sizeof(float), cudaMemcpyDeviceToHost);
    return FK_OK;
  }
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  // capture the whole loop in one CUDA graph: 2 kernels per step
  cudaGraph_t graph;
  e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) { err = cudaGetErrorString(e); return FK_ERR_CUDA; }
  const int adam_blocks = static_cast<int>(std::min<size_t>((8 * np + 255) / 256, 4096));
  for (int st = 0; st < steps; ++st) {
    a.step = static_cast<uint32_t>(M.adam_t + st);
    mlp_pass_kernel<<<dim3(ctas, M.n_regions), kThreads, sizeof(Smem), s>>>(a);
    const double t = static_cast<double>(M.adam_t + st + 1);
    const float bc1 = static_cast<float>(1.0 - std::pow(0.9, t)), bc2 = static_cast<float>(1.0 - std::pow(0.999, t));
    // cosine decay of the learning rate from lr to lr/100 over this training call
    const double lr_t = lr * (0.01 + 0.99 * 0.5 * (1.0 + std::cos(M_PI * st / std::max(1, steps))));
    mlp_adam_kernel<<<adam_blocks, 256, 0, s>>>(M.d_master, static_cast<__nv_bfloat16*>(M.d_bf16), M.d_m, M.d_v,
                                                M.d_partial, M.d_loss, M.n_regions, ctas, static_cast<float>(lr_t), b1,
                                                b2, eps, bc1, bc2, 1, nullptr, M.d_hist + st,
                                                1.f / (static_cast<float>(batch) * M.n_regions));
  }
  e = cudaStreamEndCapture(s, &graph);
  if (e != cudaSuccess) { err = cudaGetErrorString(e); return FK_ERR_CUDA; }
  cudaGraphExec_t exec;
  e = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) { err = cudaGetErrorString(e); return FK_ERR_CUDA; }
  e = cudaGraphLaunch(exec, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaGraphExecDestroy(exec);
  if (e != cudaSuccess) { err = cudaGetErrorString(e); return FK_ERR_CUDA; }
  M.adam_t += steps;
  if (loss_hist && steps > 0) cudaMemcpy(loss_hist, M.d_hist, steps * sizeof(float), cudaMemcpyDeviceToHost);
  return FK_OK;
}

int mlp_loss_grad(Mlp& M, int n, const double* xy, const double* target, double* loss, float* grad, cudaStream_t s,
                  std::string& err) {
  // region 0, all n samples, no sampling
  std::vector<int> off;
  std::vector<int> reg(n, 0);
  int rc = upload_samples(M, n, xy, target, reg.data(), off, s, err);
  if (rc) return rc;
  const int rows = (n + kRows - 1) / kRows * kRows;
  const int ctas = rows / kRows;
  float *d_partial = nullptr, *d_loss = nullptr, *d_grad = nullptr;
  const size_t np = static_cast<size_t>(M.n_regions) * NPARAM;
  if (cudaMalloc(&d_partial, np * ctas * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&d_loss, static_cast<size_t>(M.n_regions) * ctas * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&d_grad, np * sizeof(float)) != cudaSuccess) {
    err = "mlp: loss-grad buffers";
    return FK_ERR_CUDA;
  }
  // (on s: the legacy default stream does not order work on the context's non-blocking stream)
  cudaMemsetAsync(d_partial, 0, np * ctas * sizeof(float), s);
  cudaMemsetAsync(d_loss, 0, static_cast<size_t>(M.n_regions) * ctas * sizeof(float), s);
  cudaFuncSetAttribute(mlp_pass_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(sizeof(Smem)));
  PassArgs a;
  std::memset(&a, 0, sizeof(a));
  a.mode = MODE_LOSSGRAD;
  a.n_regions = 1;
  a.ctas_per_region = ctas;
  a.rows_per_cta = kRows;
  a.params = M.d_master;
  a.wbf = static_cast<const __nv_bfloat16*>(M.d_bf16);
  a.norm = M.d_norm;
  a.samples = M.d_samples;
  a.sample_off = M.d_sample_off;
  a.inv_batch = 1.f / n;
  a.partial = d_partial;
  a.loss = d_loss;
  mlp_pass_kernel<<<dim3(ctas, 1), kThreads, sizeof(Smem), s>>>(a);
  mlp_adam_kernel<<<64, 256, 0, s>>>(M.d_master, static_cast<__nv_bfloat16*>(M.d_bf16), M.d_m, M.d_v, d_partial,
                                     d_loss, 1, ctas, 0.f, 0.f, 0.f, 0.f, 1.f, 1.f, 0, d_grad, nullptr, 0.f);
  std::vector<float> l(ctas);
  cudaError_t e = cudaStreamSynchronize(s);
  if (e == cudaSuccess) e = cudaMemcpy(grad, d_grad, NPARAM * sizeof(float), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(l.data(), d_loss, ctas * sizeof(float), cudaMemcpyDeviceToHost);
  cudaFree(d_partial);
  cudaFree(d_loss);
  cudaFree(d_grad);
  if (e != cudaSuccess) { err = cudaGetErrorString(e); return FK_ERR_CUDA; }
  double sum = 0;
  for (float v : l) sum += v;
  *loss = sum / n;
  return FK_OK;
}

int mlp_eval_host(Mlp& M, int n, const double* xy, const int* region, double* out, cudaStream_t s,
                  std::string& err) {
  // group by region: evaluate each region's points in one launch
  std::vector<float> res(3 * static_cast<size_t>(n));
  for (int r = 0; r < M.n_regions; ++r) {
    std::vector<int> idx;
    for (int i = 0; i < n; ++i)
      if ((region ? region[i] : 0) == r) idx.push_back(i);
    if (idx.empty()) continue;
    std::vector<float2> pts(idx.size());
    for (size_t k = 0; k < idx.size(); ++k)
      pts[k] = make_float2(static_cast<float>(xy[2 * idx[k]]), static_cast<float>(xy[2 * idx[k] + 1]));
    float2* d_pts = nullptr;
    float* d_out = nullptr;
    if (cudaMalloc(&d_pts, pts.size() * sizeof(float2)) != cudaSuccess ||
        cudaMalloc(&d_out, 3 * pts.size() * sizeof(float)) != cudaSuccess) {
      err = "mlp eval buffers";
      return FK_ERR_CUDA;
    }
    cudaError_t e = cudaMemcpyAsync(d_pts, pts.data(), pts.size() * sizeof(float2), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
      e = mlp_eval_device(M.d_master + static_cast<size_t>(r) * NPARAM,
                          static_cast<__nv_bfloat16*>(M.d_bf16) + static_cast<size_t>(r) * BF_PER_REGION,
                          M.d_norm + r, static_cast<int>(pts.size()), d_pts, d_out, s);
    std::vector<float> o(3 * pts.size());
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e == cudaSuccess) e = cudaMemcpy(o.data(), d_out, o.size() * sizeof(float), cudaMemcpyDeviceToHost);
    cudaFree(d_pts);
    cudaFree(d_out);
    if (e != cudaSuccess) { err = cudaGetErrorString(e); return FK_ERR_CUDA; }
    for (size_t k = 0; k < idx.size(); ++k)
      for (int q = 0; q < 3; ++q) res[3 * idx[k] + q] = o[3 * k + q];
  }
  for (size_t i = 0; i < res.size(); ++i) out[i] = res[i];
  return FK_OK;
}

int mlp_fit_output(Mlp& M, int n, const double* xy, const double* target, const int* region, double ridge,
                   cudaStream_t s, std::string& err) {
  if (!(ridge >= 0.0)) { err = "mlp fit: ridge must be >= 0"; return FK_ERR_ARG; }
  for (int r = 0; r < M.n_regions; ++r) {
    std::vector<float2> pts;
    std::vector<float> tg;
    for (int i = 0; i < n; ++i)
      if ((region ? region[i] : 0) == r) {
        pts.push_back(make_float2(static_cast<float>(xy[2 * i]), static_cast<float>(xy[2 * i + 1])));
        tg.push_back(static_cast<float>(target[i]));
      }
    const int m = static_cast<int>(pts.size());
    if (m == 0) continue;
    // one scratch block, kept in the Mlp: Gram (FP64) | flag | points | features | targets
    auto up = [](size_t b) { return (b + 255) / 256 * 256; };
    const size_t b_gram = up((W + 1) * kGramCols * sizeof(double)), b_flag = up(sizeof(int));
    const size_t b_pts = up(m * sizeof(float2)), b_feat = up(static_cast<size_t>(m) * W * sizeof(float));
    const size_t need = b_gram + b_flag + b_pts + b_feat + up(m * sizeof(float));
    cudaError_t e = cudaSuccess;
    if (need > M.fit_bytes) {
      if (M.d_fit) cudaFree(M.d_fit);
      M.d_fit = nullptr;
      M.fit_bytes = 0;
      e = cudaMalloc(&M.d_fit, need);
      if (e == cudaSuccess) M.fit_bytes = need;
    }
    if (e != cudaSuccess) { err = cudaGetErrorString(e); return FK_ERR_CUDA; }
    unsigned char* base = static_cast<unsigned char*>(M.d_fit);
    double* d_gram = reinterpret_cast<double*>(base);
    int* d_flag = reinterpret_cast<int*>(base + b_gram);
    float2* d_pts = reinterpret_cast<float2*>(base + b_gram + b_flag);
    float* d_feat = reinterpret_cast<float*>(base + b_gram + b_flag + b_pts);
    float* d_tgt = reinterpret_cast<float*>(base + b_gram + b_flag + b_pts + b_feat);
    e = cudaMemcpyAsync(d_pts, pts.data(), m * sizeof(float2), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_tgt, tg.data(), m * sizeof(float), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_gram, 0, (W + 1) * kGramCols * sizeof(double), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_flag, 0, sizeof(int), s);
    if (e == cudaSuccess) {
      PassArgs a;
      std::memset(&a, 0, sizeof(a));
      a.mode = MODE_GRADX;
      a.n_regions = 1;
      a.params = M.d_master + static_cast<size_t>(r) * NPARAM;
      a.wbf = static_cast<const __nv_bfloat16*>(M.d_bf16) + static_cast<size_t>(r) * BF_PER_REGION;
      a.norm = M.d_norm + r;
      a.n_points = m;
      a.points = d_pts;
      a.feat = d_feat;
      e = cudaFuncSetAttribute(mlp_pass_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               static_cast<int>(sizeof(Smem)));
      if (e == cudaSuccess) {
        mlp_pass_kernel<<<(m + kRows - 1) / kRows, kThreads, sizeof(Smem), s>>>(a);
        mlp_gram_kernel<<<(m + kGramRows - 1) / kGramRows, 256, 0, s>>>(d_feat, d_tgt, m, d_gram);
        mlp_lsq_kernel<<<1, 256, 0, s>>>(d_gram, M.d_master + static_cast<size_t>(r) * NPARAM, ridge, d_flag);
        e = cudaGetLastError();
      }
    }
    int flag = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&flag, d_flag, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) { err = cudaGetErrorString(e); return FK_ERR_CUDA; }
    if (flag) { err = "mlp fit: the feature Gram matrix is not positive definite (raise the ridge)"; return FK_ERR_NUMERIC; }
  }
  return FK_OK;
}

int mlp_build_table(Mlp& M, int G, cudaStream_t s, std::string& err) {
  if (G < 2 || G > 2048) { err = "table grid must be 2..2048"; return FK_ERR_ARG; }
  const long long npts = static_cast<long long>(M.n_regions) * G * G;
  // the table and its scratch only grow: a rebuild of the same size allocates nothing
  const size_t tab_bytes = npts * sizeof(float2);
  const bool same = M.d_table && M.table_cap >= tab_bytes && M.d_tex && M.tex_grid == G;
  if (M.d_tex && !same) cudaDestroyTextureObject(static_cast<cudaTextureObject_t>(M.d_tex));
  if (!same) {
    M.d_tex = 0;
    M.tex_grid = 0;
  }
  if (M.table_cap < tab_bytes) {
    if (M.d_table) cudaFree(M.d_table);
    M.d_table = nullptr;
    M.table_cap = 0;
    if (cudaMalloc(&M.d_table, tab_bytes) != cudaSuccess) { err = "mlp table buffers"; return FK_ERR_CUDA; }
    M.table_cap = tab_bytes;
  }
  auto up = [](size_t b) { return (b + 255) / 256 * 256; };
  const size_t b_pts = up(npts * sizeof(float2)), b_reg = up(npts * sizeof(int)), b_eval = up(3 * npts * sizeof(float));
  if (M.tabwork_bytes < b_pts + b_reg + b_eval) {
    if (M.d_tabwork) cudaFree(M.d_tabwork);
    M.d_tabwork = nullptr;
    M.tabwork_bytes = 0;
    if (cudaMalloc(&M.d_tabwork, b_pts + b_reg + b_eval) != cudaSuccess) { err = "mlp table buffers"; return FK_ERR_CUDA; }
    M.tabwork_bytes = b_pts + b_reg + b_eval;
  }
  unsigned char* wk = static_cast<unsigned char*>(M.d_tabwork);
  float2* d_pts = reinterpret_cast<float2*>(wk);
  int* d_reg = reinterpret_cast<int*>(wk + b_pts);
  float* d_eval = reinterpret_cast<float*>(wk + b_pts + b_reg);
  mlp_grid_points<<<256, 256, 0, s>>>(M.d_rect, M.n_regions, G, d_pts, d_reg);
  cudaError_t e = cudaSuccess;
  for (int r = 0; r < M.n_regions && e == cudaSuccess; ++r)
    e = mlp_eval_device(M.d_master + static_cast<size_t>(r) * NPARAM,
                        static_cast<__nv_bfloat16*>(M.d_bf16) + static_cast<size_t>(r) * BF_PER_REGION, M.d_norm + r,
                        G * G, d_pts + static_cast<long long>(r) * G * G, d_eval + 3LL * r * G * G, s);
  if (e == cudaSuccess) {
    mlp_pack_table<<<256, 256, 0, s>>>(d_eval, npts, M.d_table);
    e = cudaStreamSynchronize(s);
  }
  if (e != cudaSuccess) { err = cudaGetErrorString(e); return FK_ERR_CUDA; }
  if (same) {
    M.table_grid = G;  // (the texture object still describes this table)
    return FK_OK;
  }
  M.table_grid = G;
  // The texture unit interpolates the FP32 lookups (bilinear with 8-bit
  // fractional weights: the control term stays a martingale whatever grad
  // u_hat it uses, and the weights' rounding is far below the network's fit
  // error).  Pitch-linear 2-D texture: G x (regions G) float2.
  int dev = 0, pitch_align = 0, tex_align = 0, max_w = 0, max_h = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&pitch_align, cudaDevAttrTexturePitchAlignment, dev);
  cudaDeviceGetAttribute(&tex_align, cudaDevAttrTextureAlignment, dev);
  cudaDeviceGetAttribute(&max_w, cudaDevAttrMaxTexture2DLinearWidth, dev);
  cudaDeviceGetAttribute(&max_h, cudaDevAttrMaxTexture2DLinearHeight, dev);
  const size_t pitch = static_cast<size_t>(G) * sizeof(float2);
  const long long height = static_cast<long long>(M.n_regions) * G;
  if (pitch_align > 0 && tex_align > 0 && pitch % pitch_align == 0 &&
      reinterpret_cast<uintptr_t>(M.d_table) % tex_align == 0 && G <= max_w && height <= max_h) {
    cudaResourceDesc rd;
    std::memset(&rd, 0, sizeof(rd));
    rd.resType = cudaResourceTypePitch2D;
    rd.res.pitch2D.devPtr = M.d_table;
    rd.res.pitch2D.desc = cudaCreateChannelDesc<float2>();
    rd.res.pitch2D.width = G;
    rd.res.pitch2D.height = static_cast<size_t>(height);
    rd.res.pitch2D.pitchInBytes = pitch;
    cudaTextureDesc td;
    std::memset(&td, 0, sizeof(td));
    td.addressMode[0] = cudaAddressModeClamp;
    td.addressMode[1] = cudaAddressModeClamp;
    td.filterMode = cudaFilterModeLinear;
    td.readMode = cudaReadModeElementType;
    td.normalizedCoords = 0;
    cudaTextureObject_t t = 0;
    if (cudaCreateTextureObject(&t, &rd, &td, nullptr) == cudaSuccess) {
      M.d_tex = t;
      M.tex_grid = G;
    } else {
      cudaGetLastError();
    }
  }
  return FK_OK;
}

}  // namespace fk
