// Path-kernel launches: the instantiations with the control-variate terms
// (FP32 and FP64 stepping), the choice of build for a launch and the launch
// itself.  The kernel is in fk_paths_kernel.cuh; the builds without the
// control-variate terms are instantiated in fk_paths_plain.cu.
#include "fk_paths_kernel.cuh"

namespace fk {

namespace {

const void* select_paths_v(int problem, int precision, int st, bool warp_mode, bool four, bool cv) {
  if (!cv) return select_paths_plain(problem, precision, st, warp_mode, four);
  if (warp_mode)
    return precision == 1 ? paths_fn_r<float, true, true>(problem, st, false)
                          : paths_fn_r<double, true, true>(problem, st, false);
  return precision == 1 ? paths_fn_r<float, false, true>(problem, st, four)
                        : paths_fn_r<double, false, true>(problem, st, false);
}
// The variant a launch uses: the 4-CTA build for FP32 patch-stencil slot
// mode when 4 of its CTAs fit on an SM with this shared memory and block.
const void* select_paths(int problem, int precision, int st, bool warp_mode, int block, size_t smem, bool cv) {
  if (precision == 1 && st == 2 && !warp_mode && block == 256) {
    const void* f4 = select_paths_v(problem, precision, st, warp_mode, true, cv);
    int n = 0;
    if (cudaFuncSetAttribute(f4, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)) == cudaSuccess &&
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, f4, block, smem) == cudaSuccess && n >= 4)
      return f4;
    cudaGetLastError();
  }
  return select_paths_v(problem, precision, st, warp_mode, false, cv);
}

}  // namespace

size_t paths_smem_bytes(int precision, int stencil_kind, int acc_words, int smem_nodes, bool warp_mode, int block,
                        bool wm_shared) {
  if (warp_mode)
    return static_cast<size_t>(block / 32) *
           paths_slot_bytes(precision, stencil_kind, wm_shared ? acc_words : 0, smem_nodes);
  return static_cast<size_t>(paths_slots(precision)) * paths_slot_bytes(precision, stencil_kind, acc_words, smem_nodes);
}

cudaError_t launch_paths(const LaunchArgs& a, int problem, int precision, int grid, int block, size_t smem,
                         cudaStream_t s, bool warp_mode) {
  if (block < 32 || block > 256 || block % 32 != 0) return cudaErrorInvalidValue;
  const void* fn = select_paths(problem, precision, a.stencil_kind, warp_mode, block, smem, a.any_cv != 0);
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  if (e != cudaSuccess) return e;
  void* args[] = {const_cast<LaunchArgs*>(&a)};
  return cudaLaunchKernel(fn, dim3(grid), dim3(block), args, smem, s);
}

int paths_kernel_occupancy(int problem, int precision, int stencil_kind, int cv, int block, size_t smem, bool warp_mode) {
  const void* fn = select_paths(problem, precision, stencil_kind, warp_mode, block, smem, cv != 0);
  cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, block, smem) != cudaSuccess) return 1;
  return n > 0 ? n : 1;
}

}  // namespace fk
