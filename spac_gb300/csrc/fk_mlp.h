// Learned control variate: MLP 2 -> 64 -> 64 -> 64 -> 1 (SiLU) per region,
// BF16 weights for the tensor-core kernels, FP32 master copy for Adam.
#pragma once
#include <cuda_runtime.h>
#include <string>
#include <vector>

namespace fk {

struct Mlp {
  int n_regions = 0;
  int n_params = 0;                 // per region
  std::vector<double> rects;        // 4 per region
  float* d_master = nullptr;        // FP32 master parameters [R][P]
  void* d_bf16 = nullptr;           // BF16 W2, W2^T, W3, W3^T per region
  float* d_m = nullptr;             // Adam moments
  float* d_v = nullptr;
  float4* d_norm = nullptr;         // input normalisation per region
  double* d_rect = nullptr;
  float* d_partial = nullptr;       // per-CTA gradient partials
  float* d_loss = nullptr;
  float* d_hist = nullptr;
  unsigned* d_sync = nullptr;       // persistent training: barrier counter and error word
  float* d_sched = nullptr;         // persistent training: per-step learning rate and bias corrections
  float4* d_samples = nullptr;      // training samples (x, y, target) grouped by region
  int* d_sample_off = nullptr;      // inside the d_samples allocation
  float2* d_table = nullptr;        // grad u_hat on a G x G grid per region
  int table_grid = 0;
  // the same table as a linearly filtered texture (regions stacked in y),
  // for FP32 stepping; 0 where the table's shape does not allow one
  unsigned long long d_tex = 0;
  void* d_fit = nullptr;            // output-layer refit scratch (kept across calls)
  size_t fit_bytes = 0;
  void* d_tabwork = nullptr;        // table build scratch: grid points, regions, evaluations (kept across calls)
  size_t tabwork_bytes = 0;
  size_t table_cap = 0;             // capacity of d_table (bytes)
  int tex_grid = 0;                 // grid of the table that d_tex describes
  // capacities (bytes) of the training buffers, which only grow: a training
  // call allocates nothing once they are large enough
  size_t cap_samples = 0, cap_partial = 0, cap_loss = 0, cap_hist = 0, cap_sched = 0;
  long long adam_t = 0;
  int trainer = 0;                  // fk_mlp_set_trainer: 0 auto, 1 grid-persistent, 2 per-step graph
  unsigned long long barrier_ns = 0;  // grid-barrier waits give up after this (0: 5 s)
  Mlp() = default;
  Mlp(const Mlp&) = delete;
  Mlp& operator=(const Mlp&) = delete;
  ~Mlp();
};

size_t mlp_pass_smem();
int mlp_nparam();
int mlp_init(Mlp& M, int n_regions, const double* rects, unsigned long long seed, cudaStream_t s,
             std::string& err);
int mlp_set_params(Mlp& M, const float* host, cudaStream_t s);
int mlp_train(Mlp& M, int n, const double* xy, const double* target, const int* region, int steps, int batch,
              double lr, unsigned long long seed, float* loss_hist, cudaStream_t s, std::string& err);
int mlp_loss_grad(Mlp& M, int n, const double* xy, const double* target, double* loss, float* grad, cudaStream_t s,
                  std::string& err);
int mlp_eval_host(Mlp& M, int n, const double* xy, const int* region, double* out, cudaStream_t s, std::string& err);
int mlp_build_table(Mlp& M, int G, cudaStream_t s, std::string& err);
int mlp_fit_output(Mlp& M, int n, const double* xy, const double* target, const int* region, double ridge,
                   cudaStream_t s, std::string& err);

}  // namespace fk
