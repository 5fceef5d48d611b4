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
// Guess of Q - q* for every column from the stage input q* (DDENS, MOMZ, DRHOT fields, FP64) and
// impl_fac; writes three FP32 (Np, Ne) fields.  Runs the three GEMMs on the tensor cores.
int mlp_infer(MlpState* m, const fedg::Ops& op, const float2* qd, const float2* qm, const float2* qr, double impl_fac,
              float* gd, float* gm, float* gr, cudaStream_t s);

// 0, or -1 if a tensor-core GEMM of this network gave up waiting on its barrier since the last
// call (synchronises the stream; clears the flag)
int mlp_take_error(MlpState* m, cudaStream_t s);

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
