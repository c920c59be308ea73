// Learned control variate: MLP 2 -> W -> W -> W -> 1 (SiLU) with BF16 weights
// for the tensor-core kernels and an FP32 master copy for Adam.
#pragma once
#include <cuda_runtime.h>
#include <vector>

namespace fk {

struct Mlp {
  int width = 64;
  double in_lo[2] = {0, 0}, in_scale[2] = {1, 1};
  int n_params = 0;
  float* d_master = nullptr;    // FP32 master parameters (packed)
  void* d_bf16 = nullptr;       // BF16 copy used by the kernels
  float* d_m = nullptr;         // Adam moments
  float* d_v = nullptr;
  long long adam_t = 0;
  ~Mlp();
};

}  // namespace fk
