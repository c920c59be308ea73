// Warp-level BF16 tensor-core helpers (mma.sync m16n8k16, FP32 accumulate)
// for the small MLP GEMMs of the learned control variate.  Operands are
// staged in shared memory K-contiguous ("TN": C[m][n] = sum_k A[m][k] B[n][k])
// and loaded with ldmatrix.
#pragma once
#include <cstdint>
#include <cuda_bf16.h>

namespace fk {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void ldsm_x4(uint32_t r[4], const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(smem_u32(p)));
}

// The same four 8x8 tiles, transposed on the way in: each lane supplies the
// address of a row of the stored (transposed) tile.
__device__ __forceinline__ void ldsm_x4_trans(uint32_t r[4], const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(smem_u32(p)));
}

__device__ __forceinline__ void mma_bf16_16816(float c[4], const uint32_t a[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// One warp: C (MT m16-tiles starting at row m0, all NT n8-tiles starting at
// n0) += A[m0.., 0..K) * B[n0.., 0..K)^T.  A and B are bf16 row-major in
// shared memory with leading dimensions lda / ldb (elements, rows 16-byte
// aligned).  c[mt][nt][4] is the m16n8 accumulator layout: thread (g =
// lane/4, t = lane%4) holds rows g and g+8, columns 2t and 2t+1.
//
// AT / BT select the stored layout of each operand: false = K-contiguous
// (A[m][k], B[n][k]), true = the transpose (A stored as [k][m], B as [k][n]),
// loaded with ldmatrix.trans so that no transposed copy is ever written.
template <int MT, int NT, int K, bool AT = false, bool BT = false>
__device__ __forceinline__ void warp_gemm(float (&c)[MT][NT][4], const __nv_bfloat16* A, int lda, int m0,
                                          const __nv_bfloat16* B, int ldb, int n0, int lane) {
  static_assert(NT % 2 == 0, "pairs of n8 tiles");
  const int i = lane >> 3, r8 = lane & 7;  // tile of the x4 load this lane addresses, row within it
#pragma unroll
  for (int k0 = 0; k0 < K; k0 += 16) {
    uint32_t a[MT][4];
#pragma unroll
    for (int mt = 0; mt < MT; ++mt) {
      if (AT) {
        // tiles (m 0-7, k 0-7), (m 8-15, k 0-7), (m 0-7, k 8-15), (m 8-15, k 8-15)
        const int krow = k0 + r8 + ((i >> 1) << 3);
        const int mcol = m0 + mt * 16 + ((i & 1) << 3);
        ldsm_x4_trans(a[mt], A + krow * lda + mcol);
      } else {
        const int r = m0 + mt * 16 + (lane & 15);
        const int col = k0 + ((lane >> 4) << 3);
        ldsm_x4(a[mt], A + r * lda + col);
      }
    }
#pragma unroll
    for (int np = 0; np < NT / 2; ++np) {
      uint32_t b[4];
      if (BT) {
        // tiles (n 0-7, k 0-7), (n 0-7, k 8-15), (n 8-15, k 0-7), (n 8-15, k 8-15)
        const int krow = k0 + r8 + ((i & 1) << 3);
        const int ncol = n0 + np * 16 + ((i >> 1) << 3);
        ldsm_x4_trans(b, B + krow * ldb + ncol);
      } else {
        const int n = n0 + np * 16 + (lane & 7) + ((lane >> 4) << 3);
        const int col = k0 + (((lane >> 3) & 1) << 3);
        ldsm_x4(b, B + n * ldb + col);
      }
#pragma unroll
      for (int mt = 0; mt < MT; ++mt) {
        mma_bf16_16816(c[mt][2 * np], a[mt], b[0], b[1]);
        mma_bf16_16816(c[mt][2 * np + 1], a[mt], b[2], b[3]);
      }
    }
  }
}
template <int MT, int NT, int K>
__device__ __forceinline__ void warp_gemm_tn(float (&c)[MT][NT][4], const __nv_bfloat16* A, int lda, int m0,
                                             const __nv_bfloat16* B, int ldb, int n0, int lane) {
  warp_gemm<MT, NT, K, false, false>(c, A, lda, m0, B, ldb, n0, lane);
}

}  // namespace fk
