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

// binomial-series coefficients of (1+r)^kappa - 1 = sum_{n>=1} c_n r^n, and 1/RHOT_hyd per level
struct PresSeries {
  double c[12];
  int nterm;
  double rmax;  // |r| above which pow() is used instead
};

// controls of the mixed-precision column solve
struct MixViArgs {
  double impl_fac, inv_impl_fac, tol, cref;
  double Uref, Vref;  // reference wind of the FP32 deviation copy of Q
  int max_iter;
  int check64;  // 1: convergence judged by the FP64 residual; 0: by the split residual
};

// Mixed-precision column solve (fedg_vicol.cu).  qin: stage input q* (FP64); z: var0 (alph and
// the plain initial iterate); guess: FP32 increments of (DENS, MOMZ, RHOT) over q*, or NULL.
// qsf: FP32 deviation copy of Q (MOMX/MOMY relative to DENS_hyd*(Uref, Vref)); tout: (Q - q*)/
// impl_fac in FP32; gsc: vi_cols_scratch_floats(n) floats of block-Thomas history; status[ncol]:
// solves used, -1 not converged, -2 non-finite; cnt[3]: failed columns, solves, converged columns.
size_t vi_cols_scratch_floats(size_t nodes);
int launch_vi_cols(int N1, const Ops& op, const Prof& pf, const ProfF& pff, const double* rhinv, const PresSeries& ps,
                   const F5c& qin, const F5c& z, const float* const* guess, float* const* qsf, float* const* tout,
                   float* gsc, int* status, unsigned long long* cnt, const MixViArgs& a, cudaStream_t s);

}  // namespace fedg

struct MixedState;
void mixed_free(MixedState* m);
int mixed_update(fedg_ctx* c, double* const q[5], int nsteps, const fedg_update_opts* o, double* iters_out);
