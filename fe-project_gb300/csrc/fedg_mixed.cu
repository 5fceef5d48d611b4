// fedg_mixed.cu -- the mixed-precision fused HEVI update (IMEX ARK232), the headline path.
//
// Per time step five launches, each stage's RK arithmetic fused into its kernel:
//   K1  stage-1 explicit tendency E(q^n) and implicit operator A(q^n) (impl_fac = 0),
//       writes the stage-2 input q*_2 (FP64) and two FP32 tendency accumulators
//   V2  column Newton solve of Q - q*_2 - impl_fac A(Q) = 0  -> Q_2 (FP64), t_im2 (FP32)
//   K2  E(Q_2), writes q*_3 (FP64), updates the final accumulator
//   V3  column Newton solve for stage 3 -> Q_3, t_im3
//   K3  E(Q_3), q^{n+1} = q^n + dt*(accumulator + b3 (t_ex3 + t_im3)) in FP64, then the modal
//       filter of the element, written in place over q^n
// (FElib: driver_nonhydro3d.F90:727-951, timeint_rk.F90:2201-2565, butcher_tab.F90:260-274.)
//
// Precision: explicit volume/face arithmetic in FP32 on deviations from the hydrostatic state
// (the pressure deviation is formed as PRES_hyd*((1 + DRHOT/THERM_hyd)^kappa - 1), never as a
// difference of totals); FP64 for the prognostic state, every RK accumulation, the Newton
// residual (DENS/MOMZ/RHOT and MOMX/MOMY) and the Newton update; the Jacobian and its LU in
// FP32 (the FP64 residual judges convergence, so the converged state is FP64-accurate).
#include <cmath>
#include <cstring>
#include <vector>

#include "fedg_ctx.cuh"
#include "fedg_mlp.cuh"

namespace fedg {

struct MixCoef {
  double dt, a21e, a21i, a31e, a31i, a32e, a32i, b1, b2, b3;
  double Uref, Vref;  // reference wind of the FP32 momentum deviations
};

struct StageBufs {
  const float* qsf[5];  // state of the explicit tendency as FP32 deviations (q^n at stage 1, Q_s after):
                        // DDENS, MOMX - DENS_hyd*Uref, MOMY - DENS_hyd*Vref, MOMZ, DRHOT
  float* qnf[5];        // stage 3: FP32 deviation copy of q^{n+1} (next step's stage-1 state)
  double* qn[5];        // q^n; stage 3 overwrites it with q^{n+1}
  double* qi[5];        // next stage input q*_{s+1} (stages 1, 2)
  float* S3[5];         // stage-3 input accumulator
  float* SF[5];         // final-update accumulator
  const float* TI[5];   // implicit tendency of the stage (stages 2, 3)
};

// PRES - PRES_hyd = PRES_hyd ((1 + DRHOT/THERM_hyd)^kappa - 1)   (nonhydro3d_common.F90:470-474)
__device__ __forceinline__ float dpres_f(float dr, float rth, float ph, float kap) {
  return ph * expm1f(kap * log1pf(dr * rth));
}

template <int N1>
__device__ __forceinline__ void face_neighbour(const OpsF& op, int f, int ke, int ex, int ey, int ez, int nxy,
                                               long& kn, int& levP, int kM) {
  constexpr int N = N1 - 1;
  levP = ez * N1 + kM;
  switch (f) {
    case 0: kn = (long)ke + (ey > 0 ? -op.NeX : (op.NeY - 1) * op.NeX); break;
    case 1: kn = (long)ke + (ex < op.NeX - 1 ? 1 : -(op.NeX - 1)); break;
    case 2: kn = (long)ke + (ey < op.NeY - 1 ? op.NeX : -(op.NeY - 1) * op.NeX); break;
    case 3: kn = (long)ke + (ex > 0 ? -1 : op.NeX - 1); break;
    case 4: kn = ez > 0 ? (long)ke - nxy : -1; levP = (ez - 1) * N1 + N; break;
    default: kn = ez < op.NeZ - 1 ? (long)ke + nxy : -1; levP = (ez + 1) * N1; break;
  }
}

template <int N1, int EPB, int STAGE>
__global__ void __launch_bounds__(EPB* N1* N1* N1)
    k_stage_mixed(const OpsF op, const ProfF pf, const double* __restrict__ dens64, const StageBufs B,
                  const MixCoef cf, int Ne, int filter_on) {
  constexpr int Np = N1 * N1 * N1, NF = N1 * N1, N = N1 - 1;
  constexpr int NW = Np / 32;  // warps per element (N1 >= 4)
  extern __shared__ float smf[];
  float* s_st = smf;                        // [EPB][6][Np]
  float* s_fl = s_st + EPB * 6 * Np;        // [EPB][15][Np]
  float* s_df = s_fl + EPB * 15 * Np;       // [EPB][5][6NF]
  float* s_di = s_df + EPB * 5 * 6 * NF;    // [EPB][5][2NF] (stage 1: implicit operator faces)
  const int tid = threadIdx.x;
  const int le = tid / Np, p = tid - le * Np;
  const int ke = blockIdx.x * EPB + le;
  const bool valid = ke < Ne;
  const int i = p % N1, j = (p / N1) % N1, k = p / NF;
  const int nxy = op.NeX * op.NeY;
  const int ez = valid ? ke / nxy : 0;
  const int ey = valid ? (ke - ez * nxy) / op.NeX : 0;
  const int ex = valid ? ke - ez * nxy - ey * op.NeX : 0;
  float* st = s_st + le * 6 * Np;
  float* fl = s_fl + le * 15 * Np;
  float* df = s_df + le * 5 * 6 * NF;
  float* di = s_di + le * 5 * 2 * NF;
  const size_t g = (size_t)ke * Np + p;
  const int lev = ez * N1 + k;
  const double dh64 = valid ? __ldg(dens64 + lev) : 1.0;

  // The state arrives as FP32 deviations: DDENS, DRHOT are deviations already; MOMX/MOMY are
  // taken relative to the horizontally uniform reference DENS_hyd(z)*(Uref, Vref) (subtracted in
  // FP64 by the producer), whose fluxes have zero divergence and cancel across every face.
  float qv[5], dp = 0.f;
#pragma unroll
  for (int v = 0; v < 5; ++v) qv[v] = valid ? __ldg(B.qsf[v] + g) : 0.f;
  const float dh = valid ? __ldg(pf.dens + lev) : 1.f;
  const float th = valid ? __ldg(pf.therm + lev) : 0.f;
  if (valid) dp = dpres_f(qv[VRT], __ldg(pf.rtherm + lev), __ldg(pf.pres + lev), op.kap);
#pragma unroll
  for (int v = 0; v < 5; ++v) st[v * Np + p] = qv[v];
  st[5 * Np + p] = dp;
  {
    const float Uf = op.Uref, Vf = op.Vref;
    const float mxd = qv[VMX], myd = qv[VMY], mz = qv[VMZ], dd = qv[VD];
    const float mxr = dh * Uf, myr = dh * Vf;
    const float rdens = 1.f / (dd + dh);
    const float ptr = th / dh;
    const float ptd = (qv[VRT] - ptr * dd) * rdens, pt = ptr + ptd;
    const float ud = (mxd - Uf * dd) * rdens, vd = (myd - Vf * dd) * rdens;
    const float u = Uf + ud, vv = Vf + vd, w = mz * rdens;
    fl[(0 * 5 + VD) * Np + p] = mxd;
    fl[(1 * 5 + VD) * Np + p] = myd;
    fl[(2 * 5 + VD) * Np + p] = mz;
    fl[(0 * 5 + VRT) * Np + p] = mxr * ptd + mxd * pt;
    fl[(1 * 5 + VRT) * Np + p] = myr * ptd + myd * pt;
    fl[(2 * 5 + VRT) * Np + p] = mz * pt;  // used by the implicit operator only (stage 1)
    fl[(0 * 5 + VMZ) * Np + p] = (mxr + mxd) * w;
    fl[(1 * 5 + VMZ) * Np + p] = (myr + myd) * w;
    fl[(2 * 5 + VMZ) * Np + p] = mz * w;
    fl[(0 * 5 + VMX) * Np + p] = mxr * ud + mxd * u + dp;
    fl[(1 * 5 + VMX) * Np + p] = myr * ud + myd * u;
    fl[(2 * 5 + VMX) * Np + p] = mz * u;
    fl[(0 * 5 + VMY) * Np + p] = mxr * vd + mxd * vv;
    fl[(1 * 5 + VMY) * Np + p] = myr * vd + myd * vv + dp;
    fl[(2 * 5 + VMY) * Np + p] = mz * vv;
  }
  __syncthreads();

  // --- HEVI Rusanov face flux (hevi_numflux.F90:232-418) in FP32 ---
  if (valid) {
    const float gamm = op.kap;
    for (int fi = p; fi < 6 * NF; fi += Np) {
      const int f = fi / NF, ab = fi - f * NF, a = ab % N1, b = ab / N1;
      int iM, jM, kM;
      face_node<N1>(f, a, b, iM, jM, kM);
      const int pM = iM + N1 * jM + NF * kM;
      long kn;
      int levP;
      face_neighbour<N1>(op, f, ke, ex, ey, ez, nxy, kn, levP, kM);
      const int levM = ez * N1 + kM;
      const float ddM = st[VD * Np + pM], mxM = st[VMX * Np + pM], myM = st[VMY * Np + pM];
      const float mzM = st[VMZ * Np + pM], drM = st[VRT * Np + pM], dpM = st[5 * Np + pM];
      float ddP, mxP, myP, mzP, drP, dpP;
      if (kn >= 0) {
        int i2, j2, k2;
        face_node<N1>(face_opp(f), a, b, i2, j2, k2);
        const size_t gP = (size_t)kn * Np + i2 + N1 * j2 + NF * k2;
        ddP = __ldg(B.qsf[VD] + gP); mxP = __ldg(B.qsf[VMX] + gP); myP = __ldg(B.qsf[VMY] + gP);
        mzP = __ldg(B.qsf[VMZ] + gP); drP = __ldg(B.qsf[VRT] + gP);
        dpP = dpres_f(drP, __ldg(pf.rtherm + levP), __ldg(pf.pres + levP), op.kap);
      } else {
        levP = levM;
        ddP = ddM; mxP = mxM; myP = myM; mzP = -mzM; drP = drM; dpP = dpM;
      }
      const float nx = (f == 1) ? 1.f : (f == 3 ? -1.f : 0.f);
      const float ny = (f == 2) ? 1.f : (f == 0 ? -1.f : 0.f);
      const float nz = (f == 5) ? 1.f : (f == 4 ? -1.f : 0.f);
      const float fs = f >= 4 ? op.FSz : ((f & 1) ? op.FSx : op.FSy);
      const float dhM = __ldg(pf.dens + levM), dhP = __ldg(pf.dens + levP);
      const float densM = ddM + dhM, densP = ddP + dhP;
      const float thM = __ldg(pf.therm + levM), thP = __ldg(pf.therm + levP);
      const float rhotM = thM + drM, rhotP = thP + drP;
      const float phM = __ldg(pf.pres + levM), phP = __ldg(pf.pres + levP);
      const float rdM = 1.f / densM, rdP = 1.f / densP;
      const float tmp1 = 0.5f * fs;
      const float Uf = op.Uref, Vf = op.Vref;
      // deviation velocities / potential temperature and full velocities
      const float udM = (mxM - Uf * ddM) * rdM, udP = (mxP - Uf * ddP) * rdP;
      const float vdM = (myM - Vf * ddM) * rdM, vdP = (myP - Vf * ddP) * rdP;
      const float ptrM = thM / dhM, ptrP = thP / dhP;
      const float ptdM = (drM - ptrM * ddM) * rdM, ptdP = (drP - ptrP * ddP) * rdP;
      const float uM = Uf + udM, uP = Uf + udP, vM = Vf + vdM, vP = Vf + vdP;
      const float wM = mzM * rdM, wP = mzP * rdP;
      const float mxrM = dhM * Uf, mxrP = dhP * Uf, myrM = dhM * Vf, myrP = dhP * Vf;
      const float velhM = uM * nx + vM * ny, velhP = uP * nx + vP * ny;
      const float velM = velhM + wM * nz, velP = velhP + wP * nz;
      const float swV = 1.f - nz * nz;
      const float csM = sqrtf(gamm * (phM + dpM) * rdM), csP = sqrtf(gamm * (phP + dpP) * rdP);
      const float alpha = swV * fmaxf(csM + fabsf(velM), csP + fabsf(velP));
      // normal flux deviations F.n (the reference parts cancel: same level on both sides)
      const float fD_M = mxM * nx + myM * ny, fD_P = mxP * nx + myP * ny;
      const float fR_M = (mxrM * ptdM + mxM * (ptrM + ptdM)) * nx + (myrM * ptdM + myM * (ptrM + ptdM)) * ny;
      const float fR_P = (mxrP * ptdP + mxP * (ptrP + ptdP)) * nx + (myrP * ptdP + myP * (ptrP + ptdP)) * ny;
      const float fZ_M = mzM * velM, fZ_P = mzP * velP;
      const float fX_M = (mxrM * udM + mxM * uM) * nx + (myrM * udM + myM * uM) * ny + mzM * uM * nz;
      const float fX_P = (mxrP * udP + mxP * uP) * nx + (myrP * udP + myP * uP) * ny + mzP * uP * nz;
      const float fY_M = (mxrM * vdM + mxM * vM) * nx + (myrM * vdM + myM * vM) * ny + mzM * vM * nz;
      const float fY_P = (mxrP * vdP + mxP * vP) * nx + (myrP * vdP + myP * vP) * ny + mzP * vP * nz;
      float* o = df + ab + f * NF;
      const int S = 6 * NF;
      o[VD * S] = tmp1 * (fD_P - fD_M - alpha * (ddP - ddM));
      o[VRT * S] = tmp1 * (fR_P - fR_M - alpha * (drP - drM));
      o[VMZ * S] = tmp1 * (fZ_P - fZ_M - alpha * (mzP - mzM));
      o[VMX * S] = tmp1 * (fX_P - fX_M + nx * (dpP - dpM) - alpha * (mxP - mxM));
      o[VMY * S] = tmp1 * (fY_P - fY_M + ny * (dpP - dpM) - alpha * (myP - myM));
      if (STAGE == 1 && f >= 4) {
        // vertical faces of the implicit operator at var0 = q^n (hevi_common_2.F90:1016-1328)
        const float al = fmaxf(fabsf(mzM * rdM) + csM, fabsf(mzP * rdP) + csP);
        const float tm = 0.5f * op.FSz;
        const float potM = rhotM * rdM, potP = rhotP * rdP;
        float* oi = di + ab + (f - 4) * NF;
        const int S2 = 2 * NF;
        oi[VD * S2] = tm * ((mzP - mzM) * nz - al * (ddP - ddM));
        oi[VMZ * S2] = tm * ((dpP - dpM) * nz - al * (mzP - mzM));
        oi[VRT * S2] = tm * ((potP * mzP - potM * mzM) * nz - al * (drP - drM));
        oi[VMX * S2] = -tm * al * (mxP - mxM);
        oi[VMY * S2] = -tm * al * (myP - myM);
      }
    }
  }
  __syncthreads();

  float tex[5], tim[5];
  if (valid) {
    const int S = 6 * NF;
    float szv[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      float sx = 0.f, sy = 0.f, sz = 0.f;
#pragma unroll
      for (int l = 0; l < N1; ++l) {
        sx = fmaf(op.D[i * N1 + l], fl[(0 * 5 + v) * Np + l + N1 * j + NF * k], sx);
        sy = fmaf(op.D[j * N1 + l], fl[(1 * 5 + v) * Np + i + N1 * l + NF * k], sy);
        sz = fmaf(op.D[k * N1 + l], fl[(2 * 5 + v) * Np + i + N1 * j + NF * l], sz);
      }
      szv[v] = sz;
      const float* d = df + v * S;
      const float lf = op.Lb[j] * d[0 * NF + i + N1 * k] + op.Lt[i] * d[1 * NF + j + N1 * k] +
                       op.Lt[j] * d[2 * NF + i + N1 * k] + op.Lb[i] * d[3 * NF + j + N1 * k] +
                       op.Lb[k] * d[4 * NF + i + N1 * j] + op.Lt[k] * d[5 * NF + i + N1 * j];
      const bool horiz_only = (v == VD || v == VRT);
      tex[v] = -(op.E11 * sx + op.E22 * sy + (horiz_only ? 0.f : op.E33 * sz) + lf);
    }
    tex[VMX] += op.coriolis_f * (qv[VMY] + dh * op.Vref);
    tex[VMY] -= op.coriolis_f * (qv[VMX] + dh * op.Uref);
    if (STAGE == 1) {
      float sdp = 0.f, drho = 0.f;
#pragma unroll
      for (int l = 0; l < N1; ++l) {
        sdp = fmaf(op.D[k * N1 + l], st[5 * Np + i + N1 * j + NF * l], sdp);
        drho = fmaf(op.T[k * N1 + l], st[VD * Np + i + N1 * j + NF * l], drho);
      }
      const int S2 = 2 * NF, fb = i + N1 * j, ft = NF + i + N1 * j;
      const float lb = op.Lb[k], lt = op.Lt[k];
      tim[VD] = -(op.E33 * szv[VD] + lb * di[VD * S2 + fb] + lt * di[VD * S2 + ft]);
      tim[VMZ] = -(op.E33 * sdp + lb * di[VMZ * S2 + fb] + lt * di[VMZ * S2 + ft]) - op.grav * drho;
      tim[VRT] = -(op.E33 * szv[VRT] + lb * di[VRT * S2 + fb] + lt * di[VRT * S2 + ft]);
      tim[VMX] = -(lb * di[VMX * S2 + fb] + lt * di[VMX * S2 + ft]);
      tim[VMY] = -(lb * di[VMY * S2 + fb] + lt * di[VMY * S2 + ft]);
    } else {
#pragma unroll
      for (int v = 0; v < 5; ++v) tim[v] = __ldg(B.TI[v] + g);
    }
  }

  // --- fused RK epilogue (FP64 accumulation of the prognostic variables) ---
  if (STAGE == 1) {
    if (valid) {
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        B.qi[v][g] = __ldg(B.qn[v] + g) + cf.dt * (double)(float(cf.a21e) * tex[v] + float(cf.a21i) * tim[v]);
        B.S3[v][g] = float(cf.a31e) * tex[v] + float(cf.a31i) * tim[v];
        B.SF[v][g] = float(cf.b1) * (tex[v] + tim[v]);
      }
    }
    return;
  }
  if (STAGE == 2) {
    if (valid) {
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        const double qn = __ldg(B.qn[v] + g);
        const float s3 = __ldg(B.S3[v] + g) + float(cf.a32e) * tex[v] + float(cf.a32i) * tim[v];
        B.qi[v][g] = qn + cf.dt * (double)s3;
        B.SF[v][g] = __ldg(B.SF[v] + g) + float(cf.b2) * (tex[v] + tim[v]);
      }
    }
    return;
  }
  // STAGE 3: q^{n+1} = q^n + dt (SF + b3 (t_ex + t_im)) in FP64, then the modal filter applied to
  // the deviation from the reference state (DENS_hyd*(Uref,Vref) for MOMX/MOMY, 0 otherwise; the
  // filter leaves that smooth reference unchanged), q^{n+1} = ref + F(deviation).
  double qnew[5];
  float dev[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    qnew[v] = 0.0;
    dev[v] = 0.f;
    if (valid) {
      qnew[v] = __ldg(B.qn[v] + g) + cf.dt * (double)(__ldg(B.SF[v] + g) + float(cf.b3) * (tex[v] + tim[v]));
      const double ref = v == VMX ? dh64 * cf.Uref : (v == VMY ? dh64 * cf.Vref : 0.0);
      dev[v] = (float)(qnew[v] - ref);
    }
  }
  if (!filter_on) {
    if (valid) {
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        B.qn[v][g] = qnew[v];
        B.qnf[v][g] = dev[v];
      }
    }
    return;
  }
  __syncthreads();  // everyone is done with the shared arrays
  float* fa = s_st + le * 6 * Np;
  float* fb = fa + Np;
  for (int v = 0; v < 5; ++v) {
    fa[p] = dev[v];
    __syncthreads();
    float sacc = 0.f;
#pragma unroll
    for (int l = 0; l < N1; ++l) sacc = fmaf(op.F[i * N1 + l], fa[l + N1 * j + NF * k], sacc);
    fb[p] = sacc;
    __syncthreads();
    sacc = 0.f;
#pragma unroll
    for (int l = 0; l < N1; ++l) sacc = fmaf(op.F[j * N1 + l], fb[i + N1 * l + NF * k], sacc);
    __syncthreads();
    fa[p] = sacc;
    __syncthreads();
    sacc = 0.f;
#pragma unroll
    for (int l = 0; l < N1; ++l) sacc = fmaf(op.Fv[k * N1 + l], fa[i + N1 * j + NF * l], sacc);
    if (valid) {
      const double ref = v == VMX ? dh64 * cf.Uref : (v == VMY ? dh64 * cf.Vref : 0.0);
      B.qn[v][g] = ref + (double)sacc;
      B.qnf[v][g] = sacc;
    }
    __syncthreads();
  }
}

// =====================================================================================
// column Newton solve, mixed precision: FP64 residual, FP32 Jacobian + LU, FP64 update
// =====================================================================================
// LU without pivoting: row k stays in lane k.  The mixed path's Jacobian is
// I + impl_fac*J_A (diagonally dominant at stable time steps); a failed factorisation shows
// up as a non-finite or non-converging FP64 residual and is reported per column.
template <typename T, int n, int nr>
__device__ __forceinline__ void warp_lu_np(T (&a)[n], T (&rhs)[nr], T* prow, int lane) {
#pragma unroll
  for (int k = 0; k < n; ++k) {
    if (lane == k) {
#pragma unroll
      for (int c = k; c < n; ++c) prow[c] = a[c];
#pragma unroll
      for (int m = 0; m < nr; ++m) prow[n + m] = rhs[m];
      prow[n + nr] = T(1) / a[k];
    }
    __syncwarp();
    if (lane > k && lane < n) {
      const T f = a[k] * prow[n + nr];
#pragma unroll
      for (int c = k + 1; c < n; ++c) a[c] = fma(-f, prow[c], a[c]);
#pragma unroll
      for (int m = 0; m < nr; ++m) rhs[m] = fma(-f, prow[n + m], rhs[m]);
    }
    __syncwarp();
  }
#pragma unroll
  for (int k = n - 1; k >= 0; --k) {
    if (lane == k) {
      const T rd = T(1) / a[k];
#pragma unroll
      for (int m = 0; m < nr; ++m) rhs[m] *= rd;
    }
#pragma unroll
    for (int m = 0; m < nr; ++m) {
      const T xk = __shfl_sync(0xffffffffu, rhs[m], k);
      if (lane < k) rhs[m] = fma(-a[k], xk, rhs[m]);
    }
  }
  __syncwarp();
}

template <typename T, int n, int nr>
__device__ __forceinline__ void warp_lu_t(T (&a)[n], T (&rhs)[nr], T* prow, int* plane, int lane, int& mypiv) {
  bool done = lane >= n;
  mypiv = -1;
#pragma unroll
  for (int k = 0; k < n; ++k) {
    float bv = done ? -1.f : fabsf((float)a[k]);
    int best = lane;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float ov = __shfl_xor_sync(0xffffffffu, bv, o);
      const int ol = __shfl_xor_sync(0xffffffffu, best, o);
      if (ov > bv || (ov == bv && ol < best)) { bv = ov; best = ol; }
    }
    const bool piv = (lane == best);
    if (piv) {
#pragma unroll
      for (int c = k; c < n; ++c) prow[c] = a[c];
#pragma unroll
      for (int m = 0; m < nr; ++m) prow[n + m] = rhs[m];
      prow[n + nr] = T(1) / a[k];
      plane[k] = lane;
      mypiv = k;
    }
    __syncwarp();
    if (!done && !piv) {
      const T f = a[k] * prow[n + nr];
#pragma unroll
      for (int c = k + 1; c < n; ++c) a[c] = fma(-f, prow[c], a[c]);
#pragma unroll
      for (int m = 0; m < nr; ++m) rhs[m] = fma(-f, prow[n + m], rhs[m]);
    }
    done = done || piv;
    __syncwarp();
  }
#pragma unroll
  for (int k = n - 1; k >= 0; --k) {
    if (mypiv == k) {
      const T rd = T(1) / a[k];
#pragma unroll
      for (int m = 0; m < nr; ++m) rhs[m] *= rd;
    }
    const int src = plane[k];
#pragma unroll
    for (int m = 0; m < nr; ++m) {
      const T xk = __shfl_sync(0xffffffffu, rhs[m], src);
      if (mypiv >= 0 && mypiv < k) rhs[m] = fma(-a[k], xk, rhs[m]);
    }
  }
  __syncwarp();
}

// (1+r)^kappa - 1 by its binomial series (|r| <= rmax), else from pow().  nt terms: the caller
// picks nt warp-uniformly from max|r| so the remainder stays below 1e-16 relative.
__device__ __forceinline__ double binom_pm1(double r, const PresSeries& ps, double kap, int nt) {
  if (fabs(r) > ps.rmax) return pow(1.0 + r, kap) - 1.0;
  double s = ps.c[nt - 1];
  for (int m = nt - 2; m >= 0; --m) s = fma(s, r, ps.c[m]);
  return s * r;
}
__device__ __forceinline__ int binom_terms(float amax) {
  return amax <= 1e-4f ? 4 : (amax <= 1e-3f ? 5 : (amax <= 1e-2f ? 8 : 12));
}

struct ColMix {
  double *P, *Q;                     // [3L] iterate and stage input, row 3l+v (v: DENS, MOMZ, RHOT)
  double *fm64, *fr64, *pot64;       // [L] FP64 level quantities of the certifying residual
  double* del64;                     // [NeZ][2][3] FP64 vertical-face fluxes
  float *fm, *fr, *pot, *wt, *dpd;   // [L] FP32 level quantities (split residual, Jacobian)
  float* del;                        // [NeZ][2][3]
  float* bf;                         // [3L] residual = right-hand side of the correction
  float *xh, *Gh;                    // [3L], [9L] block-Thomas history
  float *alB, *alT;                  // [NeZ] frozen vertical Rusanov speed
  float* prow;
  int* plane;
  int L, NeZ, lane;
  const double *dh, *ph, *rh, *rhinv;
  const float *dhf, *phf, *rhf, *rhinvf;
};

// vertical face flux of element ez, side s (0 bottom, 1 top), variable v from the level arrays
// (vi_cal_del_flux_dyn, hevi_common_2.F90:1294-1323); T = float or double
template <int N1, typename T>
__device__ __forceinline__ T mix_face(const ColMix& c, int ez, int s, int v, const T* fm, const T* pot, T tmp1) {
  constexpr int N = N1 - 1;
  const int lM = ez * N1 + (s == 0 ? 0 : N);
  const bool lid = s == 0 ? (ez == 0) : (ez == c.NeZ - 1);
  const int lP = lid ? lM : (s == 0 ? lM - 1 : lM + 1);
  const T nz = s == 0 ? T(-1) : T(1);
  const T al = (T)(s == 0 ? c.alB[ez] : c.alT[ez]);
  const T mzM = (T)c.P[3 * lM + 1];
  const T mzP = lid ? -mzM : (T)c.P[3 * lP + 1];
  if (v == 0) return tmp1 * ((mzP - mzM) * nz - al * (T)(c.P[3 * lP] - c.P[3 * lM]));
  if (v == 1) return tmp1 * ((fm[lP] - fm[lM]) * nz - al * (mzP - mzM));
  return tmp1 * ((pot[lP] * mzP - pot[lM] * mzM) * nz - al * (T)(c.P[3 * lP + 2] - c.P[3 * lM + 2]));
}

// Newton residual b = impl_fac A(P) + (q* - P) of the whole column into c.bf; returns the
// warp-wide max of |b|/scale.  fp64: the operator A in FP64 (the certifying residual);
// otherwise A in FP32 and only the difference q* - P in FP64 (the split residual).
template <int N1>
__device__ double mix_residual(const Ops& op, ColMix& c, const PresSeries& ps, double impl_fac, double cref,
                               bool fp64) {
  constexpr int n3 = 3 * N1;
  const float kap = (float)op.kap;
  // level quantities, lanes over levels (warp-uniform trip count: the FP64 branch shuffles)
  for (int base = 0; base < c.L; base += 32) {
    const bool lact = base + c.lane < c.L;
    const int l = lact ? base + c.lane : c.L - 1;
    const double Pd = c.P[3 * l], Pm = c.P[3 * l + 1], Pr = c.P[3 * l + 2];
    const float densf = __ldg(c.dhf + l) + (float)Pd;
    const float rhotf = __ldg(c.rhf + l) + (float)Pr;
    const float rdf = 1.f / densf;
    float fmf, potf;
    if (fp64) {
      const double dens = __ldg(c.dh + l) + Pd;
      const double rhot = __ldg(c.rh + l) + Pr;
      double rd = (double)rdf;  // two Newton steps on 1/dens from the FP32 reciprocal
      rd = rd * fma(-dens, rd, 2.0);
      rd = rd * fma(-dens, rd, 2.0);
      const double pot = rhot * rd;
      const double rr = Pr * __ldg(c.rhinv + l);
      float ra = fabsf((float)rr);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) ra = fmaxf(ra, __shfl_xor_sync(0xffffffffu, ra, o));
      const double fm = __ldg(c.ph + l) * binom_pm1(rr, ps, op.kap, binom_terms(ra));
      if (lact) {
        c.pot64[l] = pot;
        c.fm64[l] = fm;
        c.fr64[l] = pot * Pm;
      }
      fmf = (float)fm;
      potf = (float)pot;
    } else {
      potf = rhotf * rdf;
      fmf = __ldg(c.phf + l) * expm1f(kap * log1pf((float)Pr * __ldg(c.rhinvf + l)));
    }
    if (lact) {
      c.pot[l] = potf;
      c.fm[l] = fmf;
      c.fr[l] = potf * (float)Pm;
      c.wt[l] = (float)Pm * rdf;
      c.dpd[l] = kap * (__ldg(c.phf + l) + fmf) / rhotf;
    }
  }
  __syncwarp();
  // vertical-face fluxes, lanes over (element, side, variable)
  for (int it = c.lane; it < c.NeZ * 6; it += 32) {
    const int ez = it / 6, s = (it / 3) % 2, v = it % 3;
    if (fp64) c.del64[it] = mix_face<N1, double>(c, ez, s, v, c.fm64, c.pot64, 0.5 * op.FSz);
    else c.del[it] = mix_face<N1, float>(c, ez, s, v, c.fm, c.pot, 0.5f * (float)op.FSz);
  }
  __syncwarp();
  float errf = 0.f;
  for (int l = c.lane; l < c.L; l += 32) {
    const int ez = l / N1, k = l - ez * N1;
    double A[3];
    if (fp64) {
      double sd = 0.0, sm = 0.0, sr = 0.0, drho = 0.0;
#pragma unroll
      for (int m = 0; m < N1; ++m) {
        const int lm = ez * N1 + m;
        const double dk = op.D[k * N1 + m];
        sd = fma(dk, c.P[3 * lm + 1], sd);
        sm = fma(dk, c.fm64[lm], sm);
        sr = fma(dk, c.fr64[lm], sr);
        drho = fma(op.T[k * N1 + m], c.P[3 * lm], drho);
      }
      const double* dl = c.del64 + ez * 6;
      A[0] = -(op.E33 * sd + op.Lb[k] * dl[0] + op.Lt[k] * dl[3]);
      A[1] = -(op.E33 * sm + op.Lb[k] * dl[1] + op.Lt[k] * dl[4]) - op.grav * drho;
      A[2] = -(op.E33 * sr + op.Lb[k] * dl[2] + op.Lt[k] * dl[5]);
    } else {
      float sd = 0.f, sm = 0.f, sr = 0.f, drho = 0.f;
#pragma unroll
      for (int m = 0; m < N1; ++m) {
        const int lm = ez * N1 + m;
        const float dk = (float)op.D[k * N1 + m];
        sd = fmaf(dk, (float)c.P[3 * lm + 1], sd);
        sm = fmaf(dk, c.fm[lm], sm);
        sr = fmaf(dk, c.fr[lm], sr);
        drho = fmaf((float)op.T[k * N1 + m], (float)c.P[3 * lm], drho);
      }
      const float* dl = c.del + ez * 6;
      const float E33 = (float)op.E33, lb = (float)op.Lb[k], lt = (float)op.Lt[k];
      A[0] = -(E33 * sd + lb * dl[0] + lt * dl[3]);
      A[1] = -(E33 * sm + lb * dl[1] + lt * dl[4]) - (float)op.grav * drho;
      A[2] = -(E33 * sr + lb * dl[2] + lt * dl[5]);
    }
    const float isc[3] = {1.f / __ldg(c.dhf + l), 1.f / (__ldg(c.dhf + l) * (float)cref), 1.f / __ldg(c.rhf + l)};
#pragma unroll
    for (int v = 0; v < 3; ++v) {
      const double b = fma(impl_fac, A[v], c.Q[3 * l + v] - c.P[3 * l + v]);
      const float bfl = (float)b;
      c.bf[3 * l + v] = bfl;
      errf = fmaxf(errf, fabsf(bfl) * isc[v]);
      if (!(fabsf(bfl) < 3.0e38f)) errf = __int_as_float(0x7fc00000);
    }
  }
  __syncwarp();
  float e = errf;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float oe = __shfl_xor_sync(0xffffffffu, e, o);
    e = (e != e || oe != oe) ? __int_as_float(0x7fc00000) : fmaxf(e, oe);
  }
  return (double)e;
}

// one correction: construct_matbnd + block-Thomas + warp LU, all FP32; P += correction (FP64)
template <int N1>
__device__ void mix_solve(const Ops& op, ColMix& c, double impl_fac) {
  constexpr int N = N1 - 1, n3 = 3 * N1;
  const int lane = c.lane;
  const int v = lane % 3, pv = lane / 3;
  const bool act = lane < n3;
  const int pvr = act ? pv : 0;
  const float fi = (float)impl_fac;
  const float E33 = (float)op.E33, FSz = (float)op.FSz, gr = (float)op.grav;
  for (int ez = 0; ez < c.NeZ; ++ez) {
    float a[n3];
    float rhs[4];
    float Lc[3] = {0.f, 0.f, 0.f}, Uc[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int cc = 0; cc < n3; ++cc) {
      const int v2 = cc % 3, pv2 = cc / 3;
      const int l2 = ez * N1 + pv2;
      const float fdz = E33 * fi * (float)op.D[pvr * N1 + pv2];
      const float id = (pvr == pv2) ? 1.f : 0.f;
      float x;
      if (v == 0) x = v2 == 0 ? id : (v2 == 1 ? fdz : 0.f);
      else if (v == 1) x = v2 == 1 ? id : (v2 == 0 ? fi * gr * (float)op.T[pvr * N1 + pv2] : fdz * c.dpd[l2]);
      else x = v2 == 0 ? -fdz * c.pot[l2] * c.wt[l2] : (v2 == 1 ? fdz * c.pot[l2] : id + fdz * c.wt[l2]);
      a[cc] = x;
    }
#pragma unroll
    for (int f = 0; f < 2; ++f) {
      const bool bc = (f == 0) ? (ez == 0) : (ez == c.NeZ - 1);
      const int pv1 = f == 0 ? 0 : N;
      const int l1 = ez * N1 + pv1;
      const int ln = bc ? l1 : (f == 0 ? l1 - 1 : l1 + 1);
      const float nz = f == 0 ? -1.f : 1.f;
      const float al = f == 0 ? c.alB[ez] : c.alT[ez];
      const float fac = 0.5f * fi * (float)(f == 0 ? op.Lb[pvr] : op.Lt[pvr]) * FSz;
      const float tmp1 = fac * al, tmp2 = fac * nz;
      const float pot1 = c.pot[l1], wt1 = c.wt[l1];
      const int c0 = 3 * (f == 0 ? 0 : N);
      if (bc) {
        if (v == 2) a[c0 + 0] += 2.f * tmp2 * pot1 * wt1;
        if (v == 0) a[c0 + 1] -= 2.f * tmp2;
        if (v == 1) a[c0 + 1] += 2.f * tmp1;
        if (v == 2) a[c0 + 1] -= 2.f * tmp2 * pot1;
        if (v == 2) a[c0 + 2] -= 2.f * tmp2 * wt1;
      } else {
        if (v == 0) a[c0 + 0] += tmp1;
        if (v == 2) a[c0 + 0] += tmp2 * pot1 * wt1;
        if (v == 0) a[c0 + 1] -= tmp2;
        if (v == 1) a[c0 + 1] += tmp1;
        if (v == 2) a[c0 + 1] -= tmp2 * pot1;
        if (v == 1) a[c0 + 2] -= tmp2 * c.dpd[l1];
        if (v == 2) a[c0 + 2] += tmp1 - tmp2 * wt1;
        const float potn = c.pot[ln], wtn = c.wt[ln];
        float cc0, cc1, cc2;
        if (v == 0) { cc0 = -tmp1; cc1 = tmp2; cc2 = 0.f; }
        else if (v == 1) { cc0 = 0.f; cc1 = -tmp1; cc2 = tmp2 * c.dpd[ln]; }
        else { cc0 = -tmp2 * potn * wtn; cc1 = tmp2 * potn; cc2 = -tmp1 + tmp2 * wtn; }
        if (f == 0) { Lc[0] = cc0; Lc[1] = cc1; Lc[2] = cc2; }
        else { Uc[0] = cc0; Uc[1] = cc1; Uc[2] = cc2; }
      }
    }
    rhs[0] = act ? c.bf[ez * n3 + lane] : 0.f;
    if (ez > 0) {
      const float* Gp = c.Gh + ((ez - 1) * n3 + 3 * N) * 3;
      const float* bp = c.xh + (ez - 1) * n3 + 3 * N;
#pragma unroll
      for (int c2 = 0; c2 < 3; ++c2) a[c2] -= Lc[0] * Gp[0 * 3 + c2] + Lc[1] * Gp[1 * 3 + c2] + Lc[2] * Gp[2 * 3 + c2];
      rhs[0] -= Lc[0] * bp[0] + Lc[1] * bp[1] + Lc[2] * bp[2];
    }
    const bool last = ez == c.NeZ - 1;
    rhs[1] = last ? 0.f : Uc[0];
    rhs[2] = last ? 0.f : Uc[1];
    rhs[3] = last ? 0.f : Uc[2];
    if (!act) {
#pragma unroll
      for (int cc = 0; cc < n3; ++cc) a[cc] = 0.f;
    }
    __syncwarp();
    warp_lu_np<float, n3, 4>(a, rhs, c.prow, lane);
    if (act) {
      c.xh[ez * n3 + lane] = rhs[0];
      c.Gh[(ez * n3 + lane) * 3 + 0] = rhs[1];
      c.Gh[(ez * n3 + lane) * 3 + 1] = rhs[2];
      c.Gh[(ez * n3 + lane) * 3 + 2] = rhs[3];
    }
    __syncwarp();
  }
  for (int ez = c.NeZ - 2; ez >= 0; --ez) {
    if (act) {
      const float* bn = c.xh + (ez + 1) * n3;
      const float* G = c.Gh + (ez * n3 + lane) * 3;
      c.xh[ez * n3 + lane] -= G[0] * bn[0] + G[1] * bn[1] + G[2] * bn[2];
    }
    __syncwarp();
  }
  for (int idx = lane; idx < 3 * c.L; idx += 32) c.P[idx] += (double)c.xh[idx];
  __syncwarp();
}

struct MixViArgs {
  double impl_fac, inv_impl_fac, tol, cref;
  double Uref, Vref;  // reference wind of the FP32 deviation copy of Q
  int max_iter;
  int check64;  // 1: convergence judged by the FP64 residual; 0: by the split residual
};

// per-warp shared memory in doubles
template <int N1>
__host__ __device__ constexpr int vi_mixed_doubles(int L, int NeZ) {
  // doubles: P, Q (6L), del64 (6NeZ), G history (9L floats) shared with fm64/fr64/pot64 (3L doubles)
  // floats:  fm, fr, pot, wt, dpd (5L), bf (3L), xh (3L), del (6NeZ), alB/alT (2NeZ), prow (3N1+8)
  return 6 * L + 6 * NeZ + (9 * L + 1) / 2 + 1 + (11 * L + 8 * NeZ + 3 * N1 + 8 + 1) / 2 + 2;
}

// qin: stage input q*; z: var0 (alph and the plain initial iterate); guess: FP32 increments
// of (DENS, MOMZ, RHOT) over q*, or NULL.  qout: Q; tout: (Q - q*)/impl_fac in FP32.
template <int N1>
__global__ void __launch_bounds__(128) k_vi_mixed(const Ops op, const Prof pf, const ProfF pff,
                                                   const double* __restrict__ rhinv, const PresSeries ps,
                                                   const F5c qin, const F5c z, const float* const* guess,
                                                   float* const* qsf, float* const* tout, int* status,
                                                   unsigned long long* cnt, const MixViArgs args, int ncol) {
  constexpr int N = N1 - 1, NF = N1 * N1, Np = N1 * N1 * N1;
  extern __shared__ double sm[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int col = blockIdx.x * (blockDim.x >> 5) + wib;
  if (col >= ncol) return;
  const int L = op.L, NeZ = op.NeZ;
  double* W = sm + (size_t)wib * vi_mixed_doubles<N1>(L, NeZ);
  ColMix c;
  c.L = L; c.NeZ = NeZ; c.lane = lane;
  c.dh = pf.dens; c.ph = pf.pres; c.rh = pf.rhyd; c.rhinv = rhinv;
  c.dhf = pff.dens; c.phf = pff.pres; c.rhf = pff.therm; c.rhinvf = pff.rtherm;
  c.P = W; c.Q = c.P + 3 * L; c.del64 = c.Q + 3 * L;
  double* gbase = c.del64 + 6 * NeZ;  // 9L floats of G history == 3L doubles of FP64 level arrays
  c.Gh = reinterpret_cast<float*>(gbase);
  c.fm64 = gbase; c.fr64 = c.fm64 + L; c.pot64 = c.fr64 + L;
  float* fb = reinterpret_cast<float*>(gbase + (9 * L + 1) / 2 + 1);
  c.fm = fb; c.fr = c.fm + L; c.pot = c.fr + L; c.wt = c.pot + L; c.dpd = c.wt + L;
  c.bf = c.dpd + L; c.xh = c.bf + 3 * L; c.del = c.xh + 3 * L;
  c.alB = c.del + 6 * NeZ; c.alT = c.alB + NeZ; c.prow = c.alT + NeZ;
  c.plane = nullptr;
  const int ij = col % NF, exy = col / NF;
  const int ci = ij % N1, cj = ij / N1;
  const size_t nxy = (size_t)op.NeX * op.NeY;
  auto gidx = [&](int l) -> size_t {
    const int ez = l / N1, k = l - ez * N1;
    return ((size_t)ez * nxy + exy) * Np + ci + N1 * cj + NF * k;
  };
  const int gv[3] = {VD, VMZ, VRT};
  const double impl_fac = args.impl_fac;
  const float kap = (float)op.kap;

  for (int l = lane; l < L; l += 32) {
    const size_t g = gidx(l);
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      const double qv = __ldg(qin.v[gv[m]] + g);
      c.Q[3 * l + m] = qv;
      c.P[3 * l + m] = guess ? qv + (double)__ldg(guess[m] + g) : __ldg(z.v[gv[m]] + g);
    }
    // |w| + c of var0 in FP32: the frozen vertical Rusanov speed (hevi_common_2.F90:1149-1155)
    const float dd0 = (float)__ldg(z.v[VD] + g), dr0 = (float)__ldg(z.v[VRT] + g);
    const float rdens0 = 1.f / (__ldg(pff.dens + l) + dd0);
    const float wt0 = (float)__ldg(z.v[VMZ] + g) * rdens0;
    const float pres0 = __ldg(pff.pres + l) * (1.f + expm1f(kap * log1pf(dr0 * __ldg(pff.rtherm + l))));
    c.fm[l] = fabsf(wt0) + sqrtf(kap * pres0 * rdens0);
  }
  __syncwarp();
  for (int ez = lane; ez < NeZ; ez += 32) {
    const int lb = ez * N1, lt = ez * N1 + N;
    c.alB[ez] = fmaxf(c.fm[lb], c.fm[ez > 0 ? lb - 1 : lb]);
    c.alT[ez] = fmaxf(c.fm[lt], c.fm[ez < NeZ - 1 ? lt + 1 : lt]);
  }
  __syncwarp();

  // ---- MOMX/MOMY: linear vertical-dissipation system; FP64 residual, FP32 LU ----
  {
    // the var3 arrays are loaded already; the uv system borrows the G history (4.5L doubles)
    // for its iterate and input and the float scratch for its right-hand side / solution
    double* Pu = reinterpret_cast<double*>(c.Gh);     // [2L]
    double* Qu = Pu + 2 * L;                          // [2L]
    float* Gu = reinterpret_cast<float*>(Qu + 2 * L); // [L] (4L doubles + L floats <= 9L floats)
    float* bu = c.bf;                                 // [2L] (bf has 3L)
    float* xu = c.xh;                                 // [2L]
    for (int l = lane; l < L; l += 32) {
      const size_t g = gidx(l);
      Pu[2 * l + 0] = __ldg(z.v[VMX] + g);
      Pu[2 * l + 1] = __ldg(z.v[VMY] + g);
      Qu[2 * l + 0] = __ldg(qin.v[VMX] + g);
      Qu[2 * l + 1] = __ldg(qin.v[VMY] + g);
    }
    __syncwarp();
    const float tmf = (float)(-0.5 * op.FSz);
    for (int it = 0; it < 4; ++it) {
      float err = 0.f;
      for (int l = lane; l < L; l += 32) {
        const int ez = l / N1, pv = l - ez * N1;
        const float iscu = 1.f / (__ldg(pff.dens + l) * (float)args.cref);
        const int lb = ez * N1, lt = ez * N1 + N;
        const int lbP = ez > 0 ? lb - 1 : lb, ltP = ez < NeZ - 1 ? lt + 1 : lt;
#pragma unroll
        for (int m = 0; m < 2; ++m) {
          // the operator acts on the face jumps only: jumps in FP64, the rest in FP32
          const float jB = (float)(Pu[2 * lbP + m] - Pu[2 * lb + m]);
          const float jT = (float)(Pu[2 * ltP + m] - Pu[2 * lt + m]);
          const float Af = -((float)op.Lb[pv] * tmf * c.alB[ez] * jB + (float)op.Lt[pv] * tmf * c.alT[ez] * jT);
          const double b = fma(impl_fac, (double)Af, Qu[2 * l + m] - Pu[2 * l + m]);
          const float bfl = (float)b;
          bu[2 * l + m] = bfl;
          err = fmaxf(err, fabsf(bfl) * iscu);
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) err = fmaxf(err, __shfl_xor_sync(0xffffffffu, err, o));
      if ((double)err <= args.tol || it == 3) break;
      for (int ez = 0; ez < NeZ; ++ez) {
        float a[N1];
        float rhs[3];
        const bool act = lane < N1;
        const int pv = act ? lane : 0;
        const int l = ez * N1 + pv;
        const bool bcB = ez == 0, bcT = ez == NeZ - 1;
        const float t1b = (float)(0.5 * impl_fac * op.Lb[pv] * op.FSz) * c.alB[ez];
        const float t1t = (float)(0.5 * impl_fac * op.Lt[pv] * op.FSz) * c.alT[ez];
#pragma unroll
        for (int cc = 0; cc < N1; ++cc) a[cc] = (cc == pv) ? 1.f : 0.f;
        if (!bcB) a[0] += t1b;
        if (!bcT) a[N] += t1t;
        const float Lc = bcB ? 0.f : -t1b;
        const float Uc = bcT ? 0.f : -t1t;
        float bx = bu[2 * l], by = bu[2 * l + 1];
        if (ez > 0) {
          a[0] -= Lc * Gu[(ez - 1) * N1 + N];
          bx -= Lc * xu[2 * ((ez - 1) * N1 + N)];
          by -= Lc * xu[2 * ((ez - 1) * N1 + N) + 1];
        }
        rhs[0] = bx; rhs[1] = by; rhs[2] = bcT ? 0.f : Uc;
        if (!act) {
#pragma unroll
          for (int cc = 0; cc < N1; ++cc) a[cc] = 0.f;
          rhs[0] = rhs[1] = rhs[2] = 0.f;
        }
        __syncwarp();
        warp_lu_np<float, N1, 3>(a, rhs, c.prow, lane);
        if (act) {
          xu[2 * (ez * N1 + lane)] = rhs[0];
          xu[2 * (ez * N1 + lane) + 1] = rhs[1];
          Gu[ez * N1 + lane] = rhs[2];
        }
        __syncwarp();
      }
      for (int ez = NeZ - 2; ez >= 0; --ez) {
        if (lane < N1) {
          const int l = ez * N1 + lane;
          const float gg = Gu[l];
          xu[2 * l] -= gg * xu[2 * ((ez + 1) * N1)];
          xu[2 * l + 1] -= gg * xu[2 * ((ez + 1) * N1) + 1];
        }
        __syncwarp();
      }
      for (int idx = lane; idx < 2 * L; idx += 32) Pu[idx] += (double)xu[idx];
      __syncwarp();
    }
    for (int l = lane; l < L; l += 32) {
      const size_t g = gidx(l);
      const double dh64 = __ldg(pf.dens + l);
      qsf[VMX][g] = (float)fma(-dh64, args.Uref, Pu[2 * l]);
      qsf[VMY][g] = (float)fma(-dh64, args.Vref, Pu[2 * l + 1]);
      tout[VMX][g] = (float)(Pu[2 * l] - Qu[2 * l]) * (float)args.inv_impl_fac;
      tout[VMY][g] = (float)(Pu[2 * l + 1] - Qu[2 * l + 1]) * (float)args.inv_impl_fac;
    }
    __syncwarp();
  }

  // ---- DENS/MOMZ/RHOT Newton: first correction from the split residual, then the
  //      certifying residual before every further correction ----
  int st, nsolve = 0;
  mix_residual<N1>(op, c, ps, impl_fac, args.cref, false);
  mix_solve<N1>(op, c, impl_fac);
  nsolve = 1;
  while (true) {
    const double err = mix_residual<N1>(op, c, ps, impl_fac, args.cref, args.check64 != 0);
    if (err != err) { st = -2; break; }
    if (err <= args.tol) { st = nsolve; break; }
    if (nsolve >= args.max_iter) { st = -1; break; }
    mix_solve<N1>(op, c, impl_fac);
    ++nsolve;
  }
  for (int l = lane; l < L; l += 32) {
    const size_t g = gidx(l);
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      const double pnew = c.P[3 * l + m];
      qsf[gv[m]][g] = (float)pnew;
      tout[gv[m]][g] = (float)(pnew - c.Q[3 * l + m]) * (float)args.inv_impl_fac;
    }
  }
  if (lane == 0) {
    if (status) status[col] = st;
    if (st < 0) atomicAdd(cnt, 1ull);
    else {
      atomicAdd(cnt + 1, (unsigned long long)st);
      atomicAdd(cnt + 2, 1ull);
    }
  }
}

// FP32 deviation copy of a state (DDENS, MOMX - DENS_hyd*Uref, MOMY - DENS_hyd*Vref, MOMZ, DRHOT)
struct Dev5 { float* v[5]; };
__global__ void k_to_dev(F5c q, Dev5 out, const double* __restrict__ dens_prof, double Uref, double Vref, int Np,
                         int N1, size_t nxy, size_t n) {
  const size_t g = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n) return;
  const size_t ke = g / Np;
  const int ez = (int)(ke / nxy), k = (int)(g - ke * Np) / (N1 * N1);
  const double dh = dens_prof[ez * N1 + k];
  out.v[VD][g] = (float)q.v[VD][g];
  out.v[VMX][g] = (float)fma(-dh, Uref, q.v[VMX][g]);
  out.v[VMY][g] = (float)fma(-dh, Vref, q.v[VMY][g]);
  out.v[VMZ][g] = (float)q.v[VMZ][g];
  out.v[VRT][g] = (float)q.v[VRT][g];
}

// sums of MOMX, MOMY and DENS over the domain (FP64) for the reference wind
__global__ void k_wind_sums(const double* __restrict__ mx, const double* __restrict__ my,
                            const double* __restrict__ dd, const double* __restrict__ dens_prof, int Np, int N1,
                            size_t nxy, size_t n, double* out) {
  double s0 = 0.0, s1 = 0.0, s2 = 0.0;
  for (size_t g = (size_t)blockIdx.x * blockDim.x + threadIdx.x; g < n; g += (size_t)gridDim.x * blockDim.x) {
    const size_t ke = g / Np;
    const int ez = (int)(ke / nxy), k = (int)(g - ke * Np) / (N1 * N1);
    s0 += mx[g];
    s1 += my[g];
    s2 += dens_prof[ez * N1 + k] + dd[g];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    s0 += __shfl_xor_sync(0xffffffffu, s0, o);
    s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    s2 += __shfl_xor_sync(0xffffffffu, s2, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(out + 0, s0);
    atomicAdd(out + 1, s1);
    atomicAdd(out + 2, s2);
  }
}

// ---------------------------------------------------------------------------------------
template <int N1>
static constexpr int epb_m() { return N1 == 4 ? 4 : 1; }

template <int N1, int STAGE>
static int launch_stage_n(const OpsF& op, const ProfF& pf, const double* dens64, const StageBufs& B,
                          const MixCoef& cf, int Ne, int filt, cudaStream_t s) {
  constexpr int EPB = epb_m<N1>(), Np = N1 * N1 * N1, NF = N1 * N1;
  const size_t smem = sizeof(float) * EPB * (21 * Np + 5 * 6 * NF + 5 * 2 * NF);
  auto kfn = k_stage_mixed<N1, EPB, STAGE>;
  cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  kfn<<<(Ne + EPB - 1) / EPB, EPB * Np, smem, s>>>(op, pf, dens64, B, cf, Ne, filt);
  return (int)cudaGetLastError();
}

template <int N1>
static int launch_stage_m(int stage, const OpsF& op, const ProfF& pf, const double* dens64, const StageBufs& B,
                          const MixCoef& cf, int Ne, int filt, cudaStream_t s) {
  if (stage == 1) return launch_stage_n<N1, 1>(op, pf, dens64, B, cf, Ne, filt, s);
  if (stage == 2) return launch_stage_n<N1, 2>(op, pf, dens64, B, cf, Ne, filt, s);
  return launch_stage_n<N1, 3>(op, pf, dens64, B, cf, Ne, filt, s);
}

template <int N1>
static int launch_vi_m(const Ops& op, const Prof& pf, const ProfF& pff, const double* rhinv, const PresSeries& ps,
                       const F5c& qin, const F5c& z, const float* const* guess, float* const* qsf, float* const* tout,
                       int* status, unsigned long long* cnt, const MixViArgs& a, cudaStream_t s) {
  const int per_warp = vi_mixed_doubles<N1>(op.L, op.NeZ);
  const int ncol = op.NeX * op.NeY * N1 * N1;
  int wpb = 4;
  size_t smem = sizeof(double) * (size_t)per_warp * wpb;
  while (wpb > 1 && smem > 200 * 1024) { wpb >>= 1; smem = sizeof(double) * (size_t)per_warp * wpb; }
  if (smem > 227 * 1024) return (int)cudaErrorInvalidValue;
  auto kfn = k_vi_mixed<N1>;
  cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  kfn<<<(ncol + wpb - 1) / wpb, 32 * wpb, smem, s>>>(op, pf, pff, rhinv, ps, qin, z, guess, qsf, tout, status, cnt,
                                                       a, ncol);
  return (int)cudaGetLastError();
}

}  // namespace fedg

// =====================================================================================
struct MixedState {
  size_t n = 0;
  double* dbuf = nullptr;   // qi (5n): next stage input, FP64
  float* fbuf = nullptr;    // S3 | SF | TI (5n each) | guess (3n) | QSF (5n) | QNF (5n)
  float* prof = nullptr;    // [4][L]
  double* rhinv = nullptr;  // [L]
  float** d_ptrs = nullptr; // device arrays of float pointers: TI[5], guess[3], QSF[5]
  OpsF opf;
  PresSeries ps;
  double Uref = 0.0, Vref = 0.0;
  bool wind_set = false;
  double* qi(int v) { return dbuf + (size_t)v * n; }
  float* S3(int v) { return fbuf + (size_t)v * n; }
  float* SF(int v) { return fbuf + (size_t)(5 + v) * n; }
  float* TI(int v) { return fbuf + (size_t)(10 + v) * n; }
  float* GU(int v) { return fbuf + (size_t)(15 + v) * n; }
  float* QSF(int v) { return fbuf + (size_t)(18 + v) * n; }
  float* QNF(int v) { return fbuf + (size_t)(23 + v) * n; }
};

void mixed_free(MixedState* m) {
  if (!m) return;
  cudaFree(m->dbuf);
  cudaFree(m->fbuf);
  cudaFree(m->prof);
  cudaFree(m->rhinv);
  cudaFree(m->d_ptrs);
  delete m;
}

static int mixed_setup(fedg_ctx* c) {
  if (c->mixed) return 0;
  if (c->N1 != 4 && c->N1 != 8) return api_fail("fedg_update: the mixed-precision path is built for porder 3 and 7");
  MixedState* m = new MixedState();
  m->n = c->n;
  const int L = c->L;
  cudaError_t e;
  if ((e = cudaMalloc(&m->dbuf, sizeof(double) * 5 * c->n)) != cudaSuccess ||
      (e = cudaMalloc(&m->fbuf, sizeof(float) * 28 * c->n)) != cudaSuccess ||
      (e = cudaMalloc(&m->prof, sizeof(float) * 4 * L)) != cudaSuccess ||
      (e = cudaMalloc(&m->rhinv, sizeof(double) * L)) != cudaSuccess ||
      (e = cudaMalloc(&m->d_ptrs, sizeof(float*) * 13)) != cudaSuccess) {
    mixed_free(m);
    return api_cuda_fail(e, "fedg_update(mixed): allocation");
  }
  // FP32 operators
  const Ops& o = c->op;
  OpsF& f = m->opf;
  std::memset(&f, 0, sizeof(f));
  for (int k = 0; k < FEDG_MAXN1 * FEDG_MAXN1; ++k) {
    f.D[k] = (float)o.D[k]; f.F[k] = (float)o.F[k]; f.Fv[k] = (float)o.Fv[k]; f.T[k] = (float)o.T[k];
  }
  for (int k = 0; k < FEDG_MAXN1; ++k) { f.Lb[k] = (float)o.Lb[k]; f.Lt[k] = (float)o.Lt[k]; }
  f.E11 = (float)o.E11; f.E22 = (float)o.E22; f.E33 = (float)o.E33;
  f.FSx = (float)o.FSx; f.FSy = (float)o.FSy; f.FSz = (float)o.FSz;
  f.grav = (float)o.grav; f.kap = (float)o.kap; f.coriolis_f = (float)o.coriolis_f;
  f.NeX = o.NeX; f.NeY = o.NeY; f.NeZ = o.NeZ; f.N1 = o.N1; f.Np = o.Np; f.L = o.L;
  // binomial series of (1+r)^kappa - 1: c_n = C(kappa, n); 12 terms are exact to roundoff for |r| <= 0.03
  m->ps.nterm = 12;
  m->ps.rmax = 0.03;
  double cn = 1.0;
  for (int n = 1; n <= 12; ++n) {
    cn *= (o.kap - (n - 1)) / n;
    m->ps.c[n - 1] = cn;
  }
  // FP32 base-state profiles and 1/RHOT_hyd
  std::vector<double> hp(4 * L);
  e = cudaMemcpy(hp.data(), c->d_prof, sizeof(double) * 4 * L, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) { mixed_free(m); return api_cuda_fail(e, "fedg_update(mixed): profile copy"); }
  std::vector<float> pfh(4 * L);
  std::vector<double> rinv(L);
  for (int l = 0; l < L; ++l) {
    pfh[l] = (float)hp[l];
    pfh[L + l] = (float)hp[L + l];
    pfh[2 * L + l] = (float)hp[2 * L + l];
    pfh[3 * L + l] = (float)(1.0 / hp[2 * L + l]);
    rinv[l] = 1.0 / hp[3 * L + l];
  }
  float* hptr[13];
  for (int v = 0; v < 5; ++v) hptr[v] = m->TI(v);
  for (int v = 0; v < 3; ++v) hptr[5 + v] = m->GU(v);
  for (int v = 0; v < 5; ++v) hptr[8 + v] = m->QSF(v);
  if ((e = cudaMemcpy(m->prof, pfh.data(), sizeof(float) * 4 * L, cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(m->rhinv, rinv.data(), sizeof(double) * L, cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(m->d_ptrs, hptr, sizeof(float*) * 13, cudaMemcpyHostToDevice)) != cudaSuccess) {
    mixed_free(m);
    return api_cuda_fail(e, "fedg_update(mixed): upload");
  }
  c->mixed = m;
  return 0;
}

int mixed_update(fedg_ctx* c, double* const q[5], int nsteps, const fedg_update_opts* o, double* iters_out) {
  if (o->eqs != FEDG_HEVI) return api_fail("fedg_update: the mixed-precision path implements HEVI (IMEX ARK232)");
  if (o->max_iter < 1) return api_fail("fedg_update: max_iter must be >= 1");
  int r = mixed_setup(c);
  if (r) return r;
  MixedState* m = c->mixed;
  if (o->use_guess && !mlp_ready(c->guess)) return api_fail("fedg_update: use_guess set but no trained column-guess network is loaded (fedg_guess_load)");
  const double alp = (3.0 + 2.0 * std::sqrt(2.0)) / 6.0, gam = 1.0 - 1.0 / std::sqrt(2.0), del = 1.0 / (2.0 * std::sqrt(2.0));
  MixCoef cf{o->dt, 2.0 * gam, gam, 1.0 - alp, del, alp, del, del, del, gam, 0.0, 0.0};
  const ProfF pff{m->prof, m->prof + c->L, m->prof + 2 * c->L, m->prof + 3 * c->L};
  const Prof pf = c->prof();
  StageBufs B;
  std::memset(&B, 0, sizeof(B));
  for (int v = 0; v < 5; ++v) {
    B.qn[v] = q[v];
    B.qnf[v] = m->QNF(v);
    B.qi[v] = m->qi(v);
    B.S3[v] = m->S3(v);
    B.SF[v] = m->SF(v);
    B.TI[v] = m->TI(v);
  }
  if (!m->wind_set) {  // reference wind = domain-mean velocity of the first state seen
    double* d_s = reinterpret_cast<double*>(m->fbuf);  // TI area, free before the first step
    if (cudaMemsetAsync(d_s, 0, 3 * sizeof(double), c->stream) != cudaSuccess) return api_fail("memset");
    r = tracked(c, FEDG_K_AUX, [&] {
      k_wind_sums<<<1024, 256, 0, c->stream>>>(q[1], q[2], q[0], c->d_prof, c->Np, c->N1, c->nxy, c->n, d_s);
      return (int)cudaGetLastError();
    });
    if (r) return api_cuda_fail((cudaError_t)r, "fedg_update(mixed): wind sums");
    double hs[3];
    if (cudaMemcpyAsync(hs, d_s, sizeof(hs), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
        cudaStreamSynchronize(c->stream) != cudaSuccess)
      return api_fail("fedg_update(mixed): wind readback");
    m->Uref = hs[2] != 0.0 ? hs[0] / hs[2] : 0.0;
    m->Vref = hs[2] != 0.0 ? hs[1] / hs[2] : 0.0;
    m->opf.Uref = (float)m->Uref;
    m->opf.Vref = (float)m->Vref;
    m->wind_set = true;
  }
  cf.Uref = m->Uref;
  cf.Vref = m->Vref;
  const double impl_fac = gam * o->dt;
  MixViArgs va{impl_fac, 1.0 / impl_fac, o->tol, 340.0, m->Uref, m->Vref, o->max_iter, 1};
  {  // FP32 deviation copy of the incoming state for the first stage-1 tendency
    F5c qc{{q[0], q[1], q[2], q[3], q[4]}};
    Dev5 dv{{m->QNF(0), m->QNF(1), m->QNF(2), m->QNF(3), m->QNF(4)}};
    r = tracked(c, FEDG_K_AUX, [&] {
      k_to_dev<<<(unsigned)((c->n + 255) / 256), 256, 0, c->stream>>>(qc, dv, c->d_prof, m->Uref, m->Vref, c->Np,
                                                                     c->N1, c->nxy, c->n);
      return (int)cudaGetLastError();
    });
    if (r) return api_cuda_fail((cudaError_t)r, "fedg_update(mixed): deviation copy");
  }
  if (cudaMemsetAsync(c->d_cnt, 0, sizeof(unsigned long long) * 3, c->stream) != cudaSuccess)
    return api_fail("fedg_update: memset");
  const int filt = c->d.mf_on;
  auto stage = [&](int s) -> int {
    return tracked(c, FEDG_K_MTEND, [&] {
      switch (c->N1) {
        case 4: return launch_stage_m<4>(s, m->opf, pff, c->d_prof, B, cf, c->Ne, filt, c->stream);
        case 8: return launch_stage_m<8>(s, m->opf, pff, c->d_prof, B, cf, c->Ne, filt, c->stream);
      }
      return (int)cudaErrorInvalidValue;
    });
  };
  auto vi = [&]() -> int {
    F5c qin{{m->qi(0), m->qi(1), m->qi(2), m->qi(3), m->qi(4)}};
    F5c z{{q[0], q[1], q[2], q[3], q[4]}};
    float* const* qo = m->d_ptrs + 8;
    const float* const* gptr = nullptr;
    if (o->use_guess) {
      const int rg = tracked(c, FEDG_K_MLP, [&] {
        return mlp_infer(c->guess, c->op, m->qi(0), m->qi(3), m->qi(4), impl_fac, m->GU(0), m->GU(1), m->GU(2), c->stream);
      });
      if (rg) return rg;
      gptr = (const float* const*)(m->d_ptrs + 5);
    }
    return tracked(c, FEDG_K_MVI, [&] {
      switch (c->N1) {
        case 4: return launch_vi_m<4>(c->op, pf, pff, m->rhinv, m->ps, qin, z, gptr, qo, m->d_ptrs, c->d_status, c->d_cnt, va, c->stream);
        case 8: return launch_vi_m<8>(c->op, pf, pff, m->rhinv, m->ps, qin, z, gptr, qo, m->d_ptrs, c->d_status, c->d_cnt, va, c->stream);
      }
      return (int)cudaErrorInvalidValue;
    });
  };
  for (int step = 0; step < nsteps; ++step) {
    for (int v = 0; v < 5; ++v) B.qsf[v] = m->QNF(v);
    if ((r = stage(1))) return api_cuda_fail((cudaError_t)r, "fedg_update(mixed): stage 1");
    if ((r = vi())) return api_cuda_fail((cudaError_t)r, "fedg_update(mixed): column solve 2");
    for (int v = 0; v < 5; ++v) B.qsf[v] = m->QSF(v);
    if ((r = stage(2))) return api_cuda_fail((cudaError_t)r, "fedg_update(mixed): stage 2");
    if ((r = vi())) return api_cuda_fail((cudaError_t)r, "fedg_update(mixed): column solve 3");
    if ((r = stage(3))) return api_cuda_fail((cudaError_t)r, "fedg_update(mixed): stage 3");
  }
  if (cudaMemcpyAsync(c->h_cnt, c->d_cnt, sizeof(unsigned long long) * 3, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
      cudaStreamSynchronize(c->stream) != cudaSuccess)
    return api_fail("fedg_update(mixed): status readback");
  if (iters_out) *iters_out = c->h_cnt[2] ? double(c->h_cnt[1]) / double(c->h_cnt[2]) : 0.0;
  return (int)c->h_cnt[0];
}
