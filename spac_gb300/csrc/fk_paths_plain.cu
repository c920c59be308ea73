// FP32 path-kernel builds without the control-variate terms (xi = 0), for
// launches whose items all use FK_CV_NONE: five of the eight per-thread
// compensated sums and the xi state drop out of the step loop, which frees
// the registers the 4-CTA build otherwise spills.
#include "fk_paths_kernel.cuh"

namespace fk {

const void* select_paths_plain(int problem, int st, bool warp_mode, bool four) {
  return warp_mode ? paths_fn_r<float, true, false>(problem, st, false) : paths_fn_r<float, false, false>(problem, st, four);
}

}  // namespace fk
