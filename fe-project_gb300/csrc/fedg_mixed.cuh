// fedg_mixed.cuh -- the mixed-precision fused update path (declarations).
#pragma once
#include "../../include/fedg.h"
#include "fedg_common.cuh"
#include "fedg_kernels.cuh"
#include <cuda_bf16.h>

namespace fedg {

// FP32 copies of the element operators for the FP32 kernels
struct OpsF {
  float D[FEDG_MAXN1 * FEDG_MAXN1];
  float F[FEDG_MAXN1 * FEDG_MAXN1];
  float Fv[FEDG_MAXN1 * FEDG_MAXN1];
  float T[FEDG_MAXN1 * FEDG_MAXN1];
  float Lb[FEDG_MAXN1], Lt[FEDG_MAXN1];
  float E11, E22, E33, FSx, FSy, FSz;
  float grav, kap, coriolis_f;
  float Uref, Vref;
  int NeX, NeY, NeZ, N1, Np, L;
  // part of a decomposed domain: the x-, x+, y-, y+ exterior face layers of the FP32 stage state
  // ([6][boundary elements][N1*N1] 8-byte slots, the value in .x); NULL where periodic
  const float2* hx[4];
};

// column profiles of the base state in FP32, [L] each
struct ProfF {
  const float* dens;
  const float* pres;
  const float* therm;
  const float* rtherm;       // 1 / THERM_hyd
  const float* sl = nullptr; // sponge-layer coefficient per level (NULL: no sponge)
  float sl_h = 0.f;          // 1: the sponge also damps MOMX/MOMY
};


// float-pair (hi, lo) copies of the column-solve operators and constants
struct OpsX {
  float2 D[FEDG_MAXN1 * FEDG_MAXN1], T[FEDG_MAXN1 * FEDG_MAXN1];
  float2 Lb[FEDG_MAXN1], Lt[FEDG_MAXN1];
  float2 E33, tmp1, grav, kap;  // tmp1 = FSz/2
  float2 Uref, Vref;
  float cb[12];  // binomial coefficients C(kappa, n+1), n = 0..11
  float rmax;    // |DRHOT/RHOT_hyd| up to which the series is used
  double kap64;
};

// column profiles as float pairs and FP32
struct ProfX {
  const float2 *dh, *ph, *rh, *rhinv;  // DENS_hyd, PRES_hyd, RHOT_hyd (from PRES_hyd), 1/RHOT_hyd
  const float *dhf, *phf, *rhf, *rthf;  // DENS_hyd, PRES_hyd, THERM_hyd, 1/THERM_hyd
};

// stage input q* as float pairs, one array per variable
struct X5 {
  const float2* v[5];
};
// the implicit operator A(var0) of DENS, MOMZ, RHOT as float pairs, written by the stage-1 kernel
struct A3 {
  const float2* v[3];
};

// controls of the mixed-precision column solve
struct MixViArgs {
  double impl_fac, inv_impl_fac, tol, cref;
  float2 impl2;     // impl_fac as a float pair
  float2 inv_impl2; // 1/impl_fac as a float pair
  int max_iter;
  int check64;  // 1: convergence judged by the float-pair residual; 0: by the split residual
  int neumann;  // > 0: corrections after an LU correction use this many Jacobian-vector products
                // of a truncated Neumann series while it contracts (0: LU corrections only)
};

// ---- float-pair precision mode (FEDG_PREC_PAIR, fedg_pair.cu) ----
struct OpsP {
  float2 D[FEDG_MAXN1 * FEDG_MAXN1], T[FEDG_MAXN1 * FEDG_MAXN1];
  float2 F[FEDG_MAXN1 * FEDG_MAXN1], Fv[FEDG_MAXN1 * FEDG_MAXN1];
  float2 Lb[FEDG_MAXN1], Lt[FEDG_MAXN1];
  float2 E11, E22, E33, FSx, FSy, FSz, grav, kap, cor, Uref, Vref;
  float cb[12];
  float rmax;
  double kap64;
  int NeX, NeY, NeZ, N1, Np, L;
  // part of a decomposed domain: the x-, x+, y-, y+ exterior face layers as deviation pairs
  // ([6][NeY*NeZ or NeX*NeZ][N1*N1], fields DDENS..DRHOT used); NULL where periodic
  const float2* hx[4];
};
// base-state profiles for the pair stage kernels, [L] each
struct ProfP {
  const float2 *dh, *ph, *th, *rth, *ptr;  // DENS_hyd, PRES_hyd, THERM_hyd, 1/THERM_hyd, THERM_hyd/DENS_hyd
  const float* phf;                         // PRES_hyd in FP32 (wave speed)
  const float2* sl = nullptr;               // sponge-layer coefficient per level (NULL: no sponge)
  float sl_h = 0.f;                         // 1: the sponge also damps MOMX/MOMY
};
struct PairCoef {
  float2 dt, a21e, a21i, a31e, a31i, a32e, a32i, b1, b2, b3;
  float2 ssp[4];  // ERK_SSP_3s3o: 3/4, 1/4, 1/3, 2/3 (HEVE)
};
struct StagePairBufs {
  const float2* qs[5];  // deviation state of the explicit tendency (q^n at stage 1, Q_s after)
  float2* qnf[5];       // stage 3: deviation copy of q^{n+1}
  double* qn[5];        // q^n; stage 3 overwrites it with q^{n+1}
  float2* qi[5];        // next stage input q*_{s+1}
  float2* S3[5];        // stage-3 input accumulator
  float2* SF[5];        // final-update accumulator
  const float2* TI[5];  // implicit tendency of the stage (stages 2, 3)
  __nv_bfloat16* X;     // stages 1, 2: feature rows of the column-guess network (NULL: none)
  int xdinp;
  float xs[3];
  double* dtrc;         // stage 3: DDENS before the modal filter (DDENS_TRC of the tracer flux; NULL: none)
  float2* a0[3];        // stage 1 (HEVI): A(q^n) of DENS, MOMZ, RHOT for the column solves' first residual
  double* qh[5];        // stage 3: also store q^{n+1} here (mapped page-locked host memory; NULL: none)
};
int launch_stage_pair_heve(int N1, int stage, const OpsP& op, const ProfP& pf, const double* dens64,
                           const StagePairBufs& B, const PairCoef& cf, int Ne, int filt, cudaStream_t s);
// elements [ke0, Ne) (ke0 > 0: one z-range of the mesh, for the pipelined first stage)
int launch_stage_pair(int N1, int stage, const OpsP& op, const ProfP& pf, const double* dens64,
                      const StagePairBufs& B, const PairCoef& cf, int Ne, int filt, cudaStream_t s, int ke0 = 0);

// Mixed-precision column solve (fedg_vicol.cu).  qin: stage input q* (float pairs); z: var0
// (FP64; alph and the plain initial iterate); guess: FP32 increments of (DENS, MOMZ, RHOT) over
// q*, or NULL; a0: the implicit operator at var0 from the stage-1 kernel (the first residual when
// the iterate starts at var0).
// qsf: FP32 deviation copy of Q (MOMX/MOMY relative to DENS_hyd*(Uref, Vref)); tout: (Q - q*)/
// impl_fac in FP32; gsc: vi_cols_scratch_floats(n) floats of block-Thomas history; status[ncol]:
// solves used, -1 not converged, -2 non-finite; cnt[3]: failed columns, solves, converged columns.
size_t vi_cols_scratch_floats(size_t nodes);
// pair_out: qsf and tout are float-pair (float2) arrays instead of FP32 ones
int launch_vi_cols(int N1, const Ops& op, const OpsX& ox, const ProfX& px, const X5& qin, const F5c& z,
                   const A3& a0, const float* const* guess, void* const* qsf, void* const* tout, float* gsc, int* status,
                   unsigned long long* cnt, const MixViArgs& a, bool pair_out, cudaStream_t s);

}  // namespace fedg

struct MixedState;
void mixed_free(MixedState* m);
// hout (optional): device-mapped page-locked host arrays that the last step's stage-3 kernel also
// writes q^{n+1} to (fedg_update_host; float-pair paths only)
// hin (optional, float-pair HEVI on a periodic mesh): page-locked host arrays holding the state; the
// first step copies them into q in z-ranges on a second stream while the deviation split and the
// stage-1 kernel run on the ranges that have arrived
int mixed_update(fedg_ctx* c, double* const q[5], int nsteps, const fedg_update_opts* o, double* iters_out,
                 double* const* hout = nullptr, double* const* hin = nullptr);
