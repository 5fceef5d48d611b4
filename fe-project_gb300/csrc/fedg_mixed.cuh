// fedg_mixed.cuh -- the mixed-precision fused update path (declarations).
#pragma once
#include "../../include/fedg.h"
#include "fedg_common.cuh"
#include "fedg_kernels.cuh"

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
};

// column profiles of the base state in FP32, [L] each
struct ProfF {
  const float* dens;
  const float* pres;
  const float* therm;
  const float* rtherm;  // 1 / THERM_hyd
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

// controls of the mixed-precision column solve
struct MixViArgs {
  double impl_fac, inv_impl_fac, tol, cref;
  float2 impl2;  // impl_fac as a float pair
  int max_iter;
  int check64;  // 1: convergence judged by the float-pair residual; 0: by the split residual
};

// Mixed-precision column solve (fedg_vicol.cu).  qin: stage input q* (float pairs); z: var0
// (FP64; alph and the plain initial iterate); guess: FP32 increments of (DENS, MOMZ, RHOT) over
// q*, or NULL.
// qsf: FP32 deviation copy of Q (MOMX/MOMY relative to DENS_hyd*(Uref, Vref)); tout: (Q - q*)/
// impl_fac in FP32; gsc: vi_cols_scratch_floats(n) floats of block-Thomas history; status[ncol]:
// solves used, -1 not converged, -2 non-finite; cnt[3]: failed columns, solves, converged columns.
size_t vi_cols_scratch_floats(size_t nodes);
int launch_vi_cols(int N1, const Ops& op, const OpsX& ox, const ProfX& px, const X5& qin, const F5c& z,
                   const float* const* guess, float* const* qsf, float* const* tout, float* gsc, int* status,
                   unsigned long long* cnt, const MixViArgs& a, cudaStream_t s);

}  // namespace fedg

struct MixedState;
void mixed_free(MixedState* m);
int mixed_update(fedg_ctx* c, double* const q[5], int nsteps, const fedg_update_opts* o, double* iters_out);
