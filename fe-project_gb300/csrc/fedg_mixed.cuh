// fedg_mixed.cuh -- the mixed-precision fused update path (declarations).
#pragma once
#include "../../include/fedg.h"
#include "fedg_common.cuh"

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

// binomial-series coefficients of (1+r)^kappa - 1 = sum_{n>=1} c_n r^n, and 1/RHOT_hyd per level
struct PresSeries {
  double c[12];
  int nterm;
  double rmax;  // |r| above which pow() is used instead
};

}  // namespace fedg

struct MixedState;
void mixed_free(MixedState* m);
int mixed_update(fedg_ctx* c, double* const q[5], int nsteps, const fedg_update_opts* o, double* iters_out);
