// fedg_mlp.cuh -- column-guess network (declarations).
#pragma once
#include <cuda_runtime.h>
#include "fedg_common.cuh"

struct MlpState;
void mlp_free(MlpState* m);
bool mlp_ready(const MlpState* m);
// Guess of the implicit increment Q - q* of every column from the stage input q* (DDENS, MOMZ,
// DRHOT) and impl_fac; writes three FP32 (Np, Ne) fields.
int mlp_infer(MlpState* m, const fedg::Ops& op, const double* qd, const double* qm, const double* qr, double impl_fac,
              float* gd, float* gm, float* gr, cudaStream_t s);
