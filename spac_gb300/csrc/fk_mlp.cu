// Learned control variate (MLP) -- C ABI entry points.
#include "../../include/spac_fk.h"
#include "fk_mlp.h"

namespace fk {
Mlp::~Mlp() {
  if (d_master) cudaFree(d_master);
  if (d_bf16) cudaFree(d_bf16);
  if (d_m) cudaFree(d_m);
  if (d_v) cudaFree(d_v);
}
}  // namespace fk

extern "C" {
int fk_mlp_create(fk_ctx*, int, const double*, const double*, unsigned long long, int*) { return FK_ERR_ARG; }
int fk_mlp_num_params(fk_ctx*, int, int*) { return FK_ERR_ARG; }
int fk_mlp_get_params(fk_ctx*, int, float*) { return FK_ERR_ARG; }
int fk_mlp_set_params(fk_ctx*, int, const float*) { return FK_ERR_ARG; }
int fk_mlp_train(fk_ctx*, int, int, const double*, const double*, int, int, double, unsigned long long, float*) {
  return FK_ERR_ARG;
}
int fk_mlp_eval(fk_ctx*, int, int, const double*, double*) { return FK_ERR_ARG; }
int fk_mlp_loss_grad(fk_ctx*, int, int, const double*, const double*, double*, float*) { return FK_ERR_ARG; }
}
