// Path-kernel builds without the control-variate terms (xi = 0), for launches
// whose items all use FK_CV_NONE: five of the eight per-thread compensated
// sums and the xi state drop out of the step loop.  In FP32 this frees the
// registers the 4-CTA build otherwise spills; in FP64 it halves the spills of
// the 2-CTA build (about 3 % of an FP64 assembly).
#include "fk_paths_kernel.cuh"

namespace fk {

const void* select_paths_plain(int problem, int precision, int st, bool warp_mode, bool four) {
  if (precision == 1)
    return warp_mode ? paths_fn_r<float, true, false>(problem, st, false)
                     : paths_fn_r<float, false, false>(problem, st, four);
  return warp_mode ? paths_fn_r<double, true, false>(problem, st, false)
                   : paths_fn_r<double, false, false>(problem, st, false);
}

}  // namespace fk
