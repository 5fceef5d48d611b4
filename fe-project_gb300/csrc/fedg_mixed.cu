// fedg_mixed.cu -- mixed-precision fused update (placeholder until the FP32 kernels land).
#include "fedg_mixed.cuh"
struct MixedState { int dummy; };
void mixed_free(MixedState* m) { delete m; }
extern "C" const char* fedg_last_error(void);
int mixed_update(fedg_ctx*, double* const*, int, const fedg_update_opts*, double*) { return -1; }
