// fedg_mixed.cuh -- the mixed-precision fused update path (declarations).
#pragma once
#include "../../include/fedg.h"
#include "fedg_common.cuh"

struct MixedState;
void mixed_free(MixedState* m);
int mixed_update(fedg_ctx* c, double* const q[5], int nsteps, const fedg_update_opts* o, double* iters_out);
