// fedg_mlp.cuh -- column-guess network: a 3-layer GELU MLP that maps a column's stage input
// (DDENS', MOMZ, DRHOT' at every level + impl_fac) to the implicit increment Q - q* of the
// HEVI Newton solve.  BF16 weights, FP32 accumulation; trained on the GPU with these kernels.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "fedg_common.cuh"

struct MlpState;
void mlp_free(MlpState* m);
bool mlp_ready(const MlpState* m);
// Feature rows of the guess network, written by the producer of the stage input q* (the stage
// kernels): row c (column c) holds DDENS'(l) s[0], MOMZ(l) s[1], DRHOT'(l) s[2] at
// X[c*dinp + v*L + l] (bf16), followed by impl_fac and zero padding, which mlp_rows fills.
struct MlpRows {
  __nv_bfloat16* X;
  int dinp, L;
  float s[3];
};
int mlp_rows(MlpState* m, int ncol, double impl_fac, MlpRows* out, cudaStream_t s);
// Guess of Q - q* for every column from the rows prepared by mlp_rows and the producer: three
// GEMMs on the tensor cores, the last scattering into three FP32 (Np, Ne) fields.
int mlp_infer(MlpState* m, const fedg::Ops& op, float* gd, float* gm, float* gr, cudaStream_t s);

// 0; -1 if a tensor-core GEMM of this network gave up waiting on its barrier since the last call
// (it then drained its MMAs and skipped its stores); -2 if the drain ran out too (synchronises the
// stream; clears the flag)
int mlp_take_error(MlpState* m, cudaStream_t s);
// polls of the tensor-core GEMMs' normal-path barrier waits (the drain keeps its full limit)
int mlp_set_poll_limit(MlpState* m, int polls);

// host-side management used by the C ABI
int mlp_create(int levels, int hidden, MlpState** out);
int mlp_set_scales(MlpState* m, const float in_scale[4], const float out_scale[3]);
long long mlp_num_params(const MlpState* m);
int mlp_set_params(MlpState* m, const float* host, long long n, cudaStream_t s);
int mlp_get_params(MlpState* m, float* host, long long n, cudaStream_t s);
int mlp_train_step(MlpState* m, const float* X, const float* T, int batch, float lr, float* loss, cudaStream_t s);
int mlp_loss_grad(MlpState* m, const float* X, const float* T, int batch, float* loss, float* grad_host, cudaStream_t s);
int mlp_predict(MlpState* m, const float* X, float* Y, int n, cudaStream_t s);
int mlp_set_ready(MlpState* m, int ready);
