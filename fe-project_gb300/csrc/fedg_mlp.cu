// fedg_mlp.cu -- column-guess network (placeholder until the kernels land).
#include "fedg_mlp.cuh"
struct MlpState { int ready = 0; };
void mlp_free(MlpState* m) { delete m; }
bool mlp_ready(const MlpState* m) { return m && m->ready; }
int mlp_infer(MlpState*, const fedg::Ops&, const double*, const double*, const double*, double, float*, float*, float*,
              cudaStream_t) {
  return (int)cudaErrorNotSupported;
}
