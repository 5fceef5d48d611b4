// fedg_pair.cu -- the explicit stage kernels of the float-pair precision mode (FEDG_PREC_PAIR).
//
// Same algorithm and fusion as k_stage_mixed (fedg_mixed.cu), with every quantity that carries
// the solution kept as an unevaluated float pair (hi + lo, fedg_f2.cuh):
//   - the deviation state and pressure deviation;
//   - the 15 flux components and the Rusanov face fluxes;
//   - the Dx/Dy/Dz contractions (compensated sums of exact products) and the Lift;
//   - the RK accumulators and the modal filter.
// Only the Rusanov wave speed and the reference-wind velocities inside it stay FP32: they
// multiply face jumps, which are small against the fields.
//
// Why the mode exists: in FP32, the rounding of a flux value is amplified by the DG derivative,
// whose row norms grow like N^2/h.  Relative to the tendency the error is about
// 6e-8 N^2 |F| / |dF| per stage, where dF is the flux variation across one element.  On strong
// flows (a -15 K density current at p = 7) that drifts from FP64 by ~4e-8 of the state per step.
// Pairs bring the same amplification down to ~1e-14.
//
// FElib counterparts: cal_tend for HEVI (FElib/src/atmosphere/dynamics/
// scale_atm_dyn_dgm_nonhydro3d_rhot_hevi.F90:289-482), the HEVI numerical flux
// (scale_atm_dyn_dgm_nonhydro3d_rhot_hevi_numflux.F90:232-418), the implicit operator at var0
// (scale_atm_dyn_dgm_nonhydro3d_hevi_common_2.F90:1016-1328), timeint_rk (FElib/src/common/
// scale_timeint_rk.F90:2201-2565) and the modal filter (scale_atm_dyn_dgm_modalfilter.F90:49-130);
// with HEVE = true, cal_tend for HEVE (…_rhot_heve.F90:292-489), its numerical flux
// (…_rhot_heve_numflux.F90:946-1139) and the SSP-RK3 stages (scale_timeint_rk.F90:1182-1278).
// The sponge layer (…_dgm_spongelayer.F90:134-219) is added to the explicit tendency when a
// profile is given.
#include "fedg_ctx.cuh"
#include "fedg_f2.cuh"
#include "fedg_mixed.cuh"

namespace fedg {
namespace {

__device__ __forceinline__ f2 operator+(f2 a, f2 b) { return f2_add(a, b); }
__device__ __forceinline__ f2 operator-(f2 a, f2 b) { return f2_sub(a, b); }
__device__ __forceinline__ f2 operator*(f2 a, f2 b) { return f2_mul(a, b); }
__device__ __forceinline__ f2 operator*(f2 a, float b) { return f2_mul_f(a, b); }
__device__ __forceinline__ f2 operator-(f2 a) { return f2_neg(a); }
__device__ __forceinline__ f2 ld2(const float2* p) { return f2_of(__ldg(p)); }
constexpr f2 Z2{0.f, 0.f};

// pressure deviation PRES_hyd ((1 + DRHOT/THERM_hyd)^kappa - 1): leading term in pairs, the rest
// of the binomial series in FP32 (relative size |r|), pow() in FP64 beyond rmax
__device__ __forceinline__ f2 dpres2(const OpsP& o, f2 dr, f2 rth, f2 ph) {
  const f2 r = dr * rth;
  f2 S;
  if (fabsf(r.h) <= o.rmax) {
    float tl = o.cb[11];
#pragma unroll
    for (int m = 10; m >= 1; --m) tl = fmaf(tl, r.h, o.cb[m]);
    S = f2_add_f(f2_of(o.kap) * r, __fmul_rn(__fmul_rn(r.h, r.h), tl));
  } else {
    S = f2_split(pow(1.0 + ((double)r.h + (double)r.l), o.kap64) - 1.0);
  }
  return ph * S;
}

template <int N1>
__device__ __forceinline__ void face_nb(const OpsP& op, int f, int ke, int ex, int ey, int ez, int nxy, long& kn,
                                        int& levP, int kM) {
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

// stage-3 output: modal filter (tensorprod3D_kernel.F90:2555-2618) of the five deviation fields,
// all five per pass (three barriers), then q^{n+1} = ref + F(dev) in FP64 and its deviation pair.
// fa, fb: [5][Np] float2 of this element (free shared memory at this point).
template <int N1>
__device__ __forceinline__ void filter_store(const OpsP& op, float2* fa, float2* fb, const f2 (&dev)[5],
                                             const f2 (&ref)[5], const StagePairBufs& B, size_t g, bool valid,
                                             int i, int j, int k, int p) {
  constexpr int Np = N1 * N1 * N1, NF = N1 * N1;
#pragma unroll
  for (int v = 0; v < 5; ++v) fa[v * Np + p] = f2_pack(dev[v]);
  __syncthreads();
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    f2acc s1;
#pragma unroll
    for (int l = 0; l < N1; ++l) s1.add(f2_of(op.F[i * N1 + l]), f2_of(fa[v * Np + l + N1 * j + NF * k]));
    fb[v * Np + p] = f2_pack(s1.get());
  }
  __syncthreads();
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    f2acc s2;
#pragma unroll
    for (int l = 0; l < N1; ++l) s2.add(f2_of(op.F[j * N1 + l]), f2_of(fb[v * Np + i + N1 * l + NF * k]));
    fa[v * Np + p] = f2_pack(s2.get());
  }
  __syncthreads();
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    f2acc s3;
#pragma unroll
    for (int l = 0; l < N1; ++l) s3.add(f2_of(op.Fv[k * N1 + l]), f2_of(fa[v * Np + i + N1 * j + NF * l]));
    if (valid) {
      const f2 fil = s3.get();
      const f2 out = ref[v] + fil;
      const double o64 = (double)out.h + (double)out.l;
      B.qn[v][g] = o64;
      if (B.qh[0]) B.qh[v][g] = o64;
      B.qnf[v][g] = f2_pack(fil);
    }
  }
}

// HEVE: the explicit HEVE operator (heve.F90:292-489, heve_numflux.F90:946-1139: vertical DENS/RHOT
// fluxes, the vertical pressure gradient and -g VFilterPM1(DDENS) explicit, unmasked wave speed) with
// the SSP-RK3 low-storage update (timeint_rk.F90:1182-1278) in place of the IMEX ARK232 stages
template <int N1, int EPB, int STAGE, bool HEVE = false>
__global__ void __launch_bounds__(EPB* N1* N1* N1)
    k_stage_pair(const OpsP op, const ProfP pf, const double* __restrict__ dens64, const StagePairBufs B,
                 const PairCoef cf, int Ne, int filter_on, int ke0, int pf_next) {
  constexpr int Np = N1 * N1 * N1, NF = N1 * N1;
  extern __shared__ float2 smp[];
  // One block per SM leaves the latency of an element's loads uncovered when the block starts: ask
  // L2 now for the fields of the block that will follow this one on the SM (pf_next elements on,
  // the grid's resident width), one bulk prefetch per field and element range.
  if (pf_next > 0 && threadIdx.x < 25) {
    const int kn0 = ke0 + blockIdx.x * EPB + pf_next;
    if (kn0 < Ne) {
      const size_t off = (size_t)kn0 * Np;
      const unsigned bytes = (unsigned)((Ne - kn0 < EPB ? Ne - kn0 : EPB) * Np * 8);
      const int t = threadIdx.x, f = t % 5;
      const void* src = nullptr;
      if (t < 5) src = B.qs[f] + off;
      else if (t < 10) src = B.qn[f] + off;
      else if (t < 15 && !HEVE && STAGE >= 2) src = B.TI[f] + off;
      else if (t < 20 && !HEVE && STAGE == 2) src = B.S3[f] + off;
      else if (t < 25 && !HEVE && STAGE >= 2) src = B.SF[f] + off;
      if (src) asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
    }
  }
  float2* s_st = smp;                       // [EPB][6][Np]
  float2* s_fl = s_st + EPB * 6 * Np;       // [EPB][15][Np]
  float2* s_df = s_fl + EPB * 15 * Np;      // [EPB][5][6NF]
  float2* s_di = s_df + EPB * 5 * 6 * NF;   // [EPB][5][2NF]
  const int tid = threadIdx.x;
  const int le = tid / Np, p = tid - le * Np;
  const int ke = ke0 + blockIdx.x * EPB + le;  // elements [ke0, Ne)
  const bool valid = ke < Ne;
  const int i = p % N1, j = (p / N1) % N1, k = p / NF;
  const int nxy = op.NeX * op.NeY;
  const int ez = valid ? ke / nxy : 0;
  const int ey = valid ? (ke - ez * nxy) / op.NeX : 0;
  const int ex = valid ? ke - ez * nxy - ey * op.NeX : 0;
  float2* st = s_st + le * 6 * Np;
  float2* fl = s_fl + le * 15 * Np;
  float2* df = s_df + le * 5 * 6 * NF;
  float2* di = s_di + le * 5 * 2 * NF;
  const size_t g = (size_t)ke * Np + p;
  const int lev = ez * N1 + k;
  const f2 U = f2_of(op.Uref), V = f2_of(op.Vref);

  f2 qv[5], dp = Z2;
#pragma unroll
  for (int v = 0; v < 5; ++v) qv[v] = valid ? ld2(B.qs[v] + g) : Z2;
  const f2 dh = valid ? ld2(pf.dh + lev) : f2{1.f, 0.f};
  if (valid) dp = dpres2(op, qv[VRT], ld2(pf.rth + lev), ld2(pf.ph + lev));
#pragma unroll
  for (int v = 0; v < 5; ++v) st[v * Np + p] = f2_pack(qv[v]);
  st[5 * Np + p] = f2_pack(dp);
  {
    const f2 mxd = qv[VMX], myd = qv[VMY], mz = qv[VMZ], dd = qv[VD];
    const f2 mxr = dh * U, myr = dh * V;
    const f2 rdens = f2_recip(dd + dh);
    const f2 ptr = valid ? ld2(pf.ptr + lev) : Z2;
    const f2 ptd = (qv[VRT] - ptr * dd) * rdens, pt = ptr + ptd;
    const f2 ud = (mxd - U * dd) * rdens, vd = (myd - V * dd) * rdens;
    const f2 u = U + ud, vv = V + vd, w = mz * rdens;
    fl[(0 * 5 + VD) * Np + p] = f2_pack(mxd);
    fl[(1 * 5 + VD) * Np + p] = f2_pack(myd);
    fl[(2 * 5 + VD) * Np + p] = f2_pack(mz);
    fl[(0 * 5 + VRT) * Np + p] = f2_pack(mxr * ptd + mxd * pt);
    fl[(1 * 5 + VRT) * Np + p] = f2_pack(myr * ptd + myd * pt);
    fl[(2 * 5 + VRT) * Np + p] = f2_pack(mz * pt);
    fl[(0 * 5 + VMZ) * Np + p] = f2_pack((mxr + mxd) * w);
    fl[(1 * 5 + VMZ) * Np + p] = f2_pack((myr + myd) * w);
    fl[(2 * 5 + VMZ) * Np + p] = f2_pack(HEVE ? mz * w + dp : mz * w);
    fl[(0 * 5 + VMX) * Np + p] = f2_pack(mxr * ud + mxd * u + dp);
    fl[(1 * 5 + VMX) * Np + p] = f2_pack(myr * ud + myd * u);
    fl[(2 * 5 + VMX) * Np + p] = f2_pack(mz * u);
    fl[(0 * 5 + VMY) * Np + p] = f2_pack(mxr * vd + mxd * vv);
    fl[(1 * 5 + VMY) * Np + p] = f2_pack(myr * vd + myd * vv + dp);
    fl[(2 * 5 + VMY) * Np + p] = f2_pack(mz * vv);
  }
  __syncthreads();

  // --- HEVI Rusanov face flux in pairs (wave speed in FP32) ---
  if (valid) {
    const float gamm = op.kap.x;
    for (int fi = p; fi < 6 * NF; fi += Np) {
      const int f = fi / NF, ab = fi - f * NF, a = ab % N1, b = ab / N1;
      int iM, jM, kM;
      face_node<N1>(f, a, b, iM, jM, kM);
      const int pM = iM + N1 * jM + NF * kM;
      long kn;
      int levP;
      face_nb<N1>(op, f, ke, ex, ey, ez, nxy, kn, levP, kM);
      // a boundary of a decomposed mesh: the exterior face layer comes from the halo exchange
      const int hsd = halo_side(f, ex, ey, op.NeX, op.NeY);
      const float2* hxs = hsd >= 0 ? op.hx[hsd] : nullptr;
      const int levM = ez * N1 + kM;
      const f2 ddM = f2_of(st[VD * Np + pM]), mxM = f2_of(st[VMX * Np + pM]), myM = f2_of(st[VMY * Np + pM]);
      const f2 mzM = f2_of(st[VMZ * Np + pM]), drM = f2_of(st[VRT * Np + pM]), dpM = f2_of(st[5 * Np + pM]);
      f2 ddP, mxP, myP, mzP, drP, dpP;
      if (hxs) {
        const size_t per = halo_stride(hsd, op.NeX, op.NeY, op.NeZ, NF), h = halo_index(hsd, ex, ey, ez, ab, op.NeX, op.NeY, NF);
        ddP = ld2(hxs + h); mxP = ld2(hxs + per + h); myP = ld2(hxs + 2 * per + h);
        mzP = ld2(hxs + 3 * per + h); drP = ld2(hxs + 4 * per + h);
        dpP = dpres2(op, drP, ld2(pf.rth + levP), ld2(pf.ph + levP));
      } else if (kn >= 0) {
        int i2, j2, k2;
        face_node<N1>(face_opp(f), a, b, i2, j2, k2);
        const size_t gP = (size_t)kn * Np + i2 + N1 * j2 + NF * k2;
        ddP = ld2(B.qs[VD] + gP); mxP = ld2(B.qs[VMX] + gP); myP = ld2(B.qs[VMY] + gP);
        mzP = ld2(B.qs[VMZ] + gP); drP = ld2(B.qs[VRT] + gP);
        dpP = dpres2(op, drP, ld2(pf.rth + levP), ld2(pf.ph + levP));
      } else {
        levP = levM;
        ddP = ddM; mxP = mxM; myP = myM; mzP = -mzM; drP = drM; dpP = dpM;
      }
      const float nx = (f == 1) ? 1.f : (f == 3 ? -1.f : 0.f);
      const float ny = (f == 2) ? 1.f : (f == 0 ? -1.f : 0.f);
      const float nz = (f == 5) ? 1.f : (f == 4 ? -1.f : 0.f);
      const f2 fs = f >= 4 ? f2_of(op.FSz) : ((f & 1) ? f2_of(op.FSx) : f2_of(op.FSy));
      const f2 dhM = ld2(pf.dh + levM), dhP = ld2(pf.dh + levP);
      const f2 rdM = f2_recip(ddM + dhM), rdP = f2_recip(ddP + dhP);
      const f2 ptrM = ld2(pf.ptr + levM), ptrP = ld2(pf.ptr + levP);
      const f2 udM = (mxM - U * ddM) * rdM, udP = (mxP - U * ddP) * rdP;
      const f2 vdM = (myM - V * ddM) * rdM, vdP = (myP - V * ddP) * rdP;
      const f2 ptdM = (drM - ptrM * ddM) * rdM, ptdP = (drP - ptrP * ddP) * rdP;
      const f2 uM = U + udM, uP = U + udP, vM = V + vdM, vP = V + vdP;
      const f2 wM = mzM * rdM, wP = mzP * rdP;
      const f2 mxrM = dhM * U, mxrP = dhP * U, myrM = dhM * V, myrP = dhP * V;
      // wave speed (FP32): max(|u.n| + c) over both sides, horizontal faces only (swV)
      const float velM = uM.h * nx + vM.h * ny + wM.h * nz, velP = uP.h * nx + vP.h * ny + wP.h * nz;
      const float csM = sqrtf(gamm * (__ldg(pf.phf + levM) + dpM.h) * rdM.h);
      const float csP = sqrtf(gamm * (__ldg(pf.phf + levP) + dpP.h) * rdP.h);
      const float swV = HEVE ? 1.f : 1.f - nz * nz;
      const float alpha = swV * fmaxf(csM + fabsf(velM), csP + fabsf(velP));
      // normal flux deviations F.n (the reference parts cancel: same level on both sides)
      f2 fD_M = mxM * nx + myM * ny, fD_P = mxP * nx + myP * ny;
      f2 fR_M = (mxrM * ptdM + mxM * (ptrM + ptdM)) * nx + (myrM * ptdM + myM * (ptrM + ptdM)) * ny;
      f2 fR_P = (mxrP * ptdP + mxP * (ptrP + ptdP)) * nx + (myrP * ptdP + myP * (ptrP + ptdP)) * ny;
      if (HEVE) {  // vertical mass and RHOT fluxes (the reference state has no vertical flux)
        fD_M = fD_M + mzM * nz;
        fD_P = fD_P + mzP * nz;
        fR_M = fR_M + mzM * (ptrM + ptdM) * nz;
        fR_P = fR_P + mzP * (ptrP + ptdP) * nz;
      }
      const f2 velM2 = uM * nx + vM * ny + wM * nz, velP2 = uP * nx + vP * ny + wP * nz;
      const f2 fZ_M = mzM * velM2, fZ_P = mzP * velP2;
      const f2 fX_M = (mxrM * udM + mxM * uM) * nx + (myrM * udM + myM * uM) * ny + mzM * uM * nz;
      const f2 fX_P = (mxrP * udP + mxP * uP) * nx + (myrP * udP + myP * uP) * ny + mzP * uP * nz;
      const f2 fY_M = (mxrM * vdM + mxM * vM) * nx + (myrM * vdM + myM * vM) * ny + mzM * vM * nz;
      const f2 fY_P = (mxrP * vdP + mxP * vP) * nx + (myrP * vdP + myP * vP) * ny + mzP * vP * nz;
      const f2 tmp1 = fs * 0.5f;
      float2* o = df + ab + f * NF;
      const int S = 6 * NF;
      o[VD * S] = f2_pack(tmp1 * (fD_P - fD_M - (ddP - ddM) * alpha));
      o[VRT * S] = f2_pack(tmp1 * (fR_P - fR_M - (drP - drM) * alpha));
      o[VMZ * S] = f2_pack(HEVE ? tmp1 * (fZ_P - fZ_M + (dpP - dpM) * nz - (mzP - mzM) * alpha)
                                : tmp1 * (fZ_P - fZ_M - (mzP - mzM) * alpha));
      o[VMX * S] = f2_pack(tmp1 * (fX_P - fX_M + (dpP - dpM) * nx - (mxP - mxM) * alpha));
      o[VMY * S] = f2_pack(tmp1 * (fY_P - fY_M + (dpP - dpM) * ny - (myP - myM) * alpha));
      if (!HEVE && STAGE == 1 && f >= 4) {
        // vertical faces of the implicit operator at var0 = q^n (hevi_common_2.F90:1016-1328)
        const float al = fmaxf(fabsf(wM.h) + csM, fabsf(wP.h) + csP);
        const f2 tm = f2_of(op.FSz) * 0.5f;
        const f2 potM = (ld2(pf.th + levM) + drM) * rdM, potP = (ld2(pf.th + levP) + drP) * rdP;
        float2* oi = di + ab + (f - 4) * NF;
        const int S2 = 2 * NF;
        oi[VD * S2] = f2_pack(tm * ((mzP - mzM) * nz - (ddP - ddM) * al));
        oi[VMZ * S2] = f2_pack(tm * ((dpP - dpM) * nz - (mzP - mzM) * al));
        oi[VRT * S2] = f2_pack(tm * ((potP * mzP - potM * mzM) * nz - (drP - drM) * al));
        oi[VMX * S2] = f2_pack(-(tm * ((mxP - mxM) * al)));
        oi[VMY * S2] = f2_pack(-(tm * ((myP - myM) * al)));
      }
    }
  }
  __syncthreads();

  f2 tex[5], tim[5];
  if (valid) {
    const int S = 6 * NF;
    f2 szv[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      f2acc sx, sy, sz;
#pragma unroll
      for (int l = 0; l < N1; ++l) {
        sx.add(f2_of(op.D[i * N1 + l]), f2_of(fl[(0 * 5 + v) * Np + l + N1 * j + NF * k]));
        sy.add(f2_of(op.D[j * N1 + l]), f2_of(fl[(1 * 5 + v) * Np + i + N1 * l + NF * k]));
        sz.add(f2_of(op.D[k * N1 + l]), f2_of(fl[(2 * 5 + v) * Np + i + N1 * j + NF * l]));
      }
      szv[v] = sz.get();
      const float2* d = df + v * S;
      f2acc lf;
      lf.add(f2_of(op.Lb[j]), f2_of(d[0 * NF + i + N1 * k]));
      lf.add(f2_of(op.Lt[i]), f2_of(d[1 * NF + j + N1 * k]));
      lf.add(f2_of(op.Lt[j]), f2_of(d[2 * NF + i + N1 * k]));
      lf.add(f2_of(op.Lb[i]), f2_of(d[3 * NF + j + N1 * k]));
      lf.add(f2_of(op.Lb[k]), f2_of(d[4 * NF + i + N1 * j]));
      lf.add(f2_of(op.Lt[k]), f2_of(d[5 * NF + i + N1 * j]));
      const bool horiz_only = !HEVE && (v == VD || v == VRT);
      f2 s = f2_of(op.E11) * sx.get() + f2_of(op.E22) * sy.get() + lf.get();
      if (!horiz_only) s = s + f2_of(op.E33) * szv[v];
      tex[v] = -s;
    }
    tex[VMX] = tex[VMX] + f2_of(op.cor) * (qv[VMY] + dh * V);
    tex[VMY] = tex[VMY] - f2_of(op.cor) * (qv[VMX] + dh * U);
    if (pf.sl) {  // sponge layer on the explicit tendency (driver_nonhydro3d.F90:831-841)
      const f2 cz = ld2(pf.sl + lev);
      tex[VMZ] = tex[VMZ] - cz * qv[VMZ];
      if (pf.sl_h != 0.f) {
        tex[VMX] = tex[VMX] - cz * (qv[VMX] + dh * U);
        tex[VMY] = tex[VMY] - cz * (qv[VMY] + dh * V);
      }
    }
    if (HEVE) {  // -g VFilterPM1(DDENS) (heve.F90:447-452)
      f2acc drho;
#pragma unroll
      for (int l = 0; l < N1; ++l) drho.add(f2_of(op.T[k * N1 + l]), f2_of(st[VD * Np + i + N1 * j + NF * l]));
      tex[VMZ] = tex[VMZ] - f2_of(op.grav) * drho.get();
#pragma unroll
      for (int v = 0; v < 5; ++v) tim[v] = Z2;
    } else if (STAGE == 1) {
      f2acc sdp, drho;
#pragma unroll
      for (int l = 0; l < N1; ++l) {
        sdp.add(f2_of(op.D[k * N1 + l]), f2_of(st[5 * Np + i + N1 * j + NF * l]));
        drho.add(f2_of(op.T[k * N1 + l]), f2_of(st[VD * Np + i + N1 * j + NF * l]));
      }
      const int S2 = 2 * NF, fb = i + N1 * j, ft = NF + i + N1 * j;
      const f2 lb = f2_of(op.Lb[k]), lt = f2_of(op.Lt[k]), E33 = f2_of(op.E33);
      auto dv = [&](int v, int o) { return f2_of(di[v * S2 + o]); };
      tim[VD] = -(E33 * szv[VD] + lb * dv(VD, fb) + lt * dv(VD, ft));
      tim[VMZ] = -(E33 * sdp.get() + lb * dv(VMZ, fb) + lt * dv(VMZ, ft) + f2_of(op.grav) * drho.get());
      tim[VRT] = -(E33 * szv[VRT] + lb * dv(VRT, fb) + lt * dv(VRT, ft));
      tim[VMX] = -(lb * dv(VMX, fb) + lt * dv(VMX, ft));
      tim[VMY] = -(lb * dv(VMY, fb) + lt * dv(VMY, ft));
      if (B.a0[0]) {
        B.a0[0][g] = f2_pack(tim[VD]);
        B.a0[1][g] = f2_pack(tim[VMZ]);
        B.a0[2][g] = f2_pack(tim[VRT]);
      }
    } else {
#pragma unroll
      for (int v = 0; v < 5; ++v) tim[v] = ld2(B.TI[v] + g);
    }
  }

  // --- fused RK epilogue in pairs ---
  const f2 dt = f2_of(cf.dt);
  if constexpr (HEVE) {
    // ERK_SSP_3s3o on the deviations (the reference state does not change in time): q1 = qn + dt t(qn),
    // q2 = 3/4 qn + 1/4 (q1 + dt t(q1)), q3 = 1/3 qn + 2/3 (q2 + dt t(q2)); the stage inputs and
    // outputs are deviation pairs, qn is split from the FP64 state
    f2 dev[5], ref[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      ref[v] = v == VMX ? dh * U : (v == VMY ? dh * V : Z2);
      dev[v] = Z2;
      if (valid) {
        const f2 qnd = f2_split(__ldg(B.qn[v] + g)) - ref[v];
        const f2 up = qv[v] + dt * tex[v];
        dev[v] = STAGE == 1 ? up
                            : (STAGE == 2 ? f2_of(cf.ssp[0]) * qnd + f2_of(cf.ssp[1]) * up
                                          : f2_of(cf.ssp[2]) * qnd + f2_of(cf.ssp[3]) * up);
      }
    }
    if (STAGE < 3) {
      if (valid) {
#pragma unroll
        for (int v = 0; v < 5; ++v) B.qi[v][g] = f2_pack(dev[v]);
      }
      return;
    }
    if (B.dtrc && valid) B.dtrc[g] = (double)dev[VD].h + (double)dev[VD].l;  // DDENS_TRC: before the filter
    if (!filter_on) {
      if (valid) {
#pragma unroll
        for (int v = 0; v < 5; ++v) {
          const f2 out = ref[v] + dev[v];
          const double o64 = (double)out.h + (double)out.l;
          B.qn[v][g] = o64;
          if (B.qh[0]) B.qh[v][g] = o64;
          B.qnf[v][g] = f2_pack(dev[v]);
        }
      }
      return;
    }
    __syncthreads();  // everyone is done with the shared arrays
    filter_store<N1>(op, s_st + le * 6 * Np, s_fl + le * 15 * Np, dev, ref, B, g, valid, i, j, k, p);
    return;
  }
  if (STAGE == 1 || STAGE == 2) {
    float xq[3] = {0.f, 0.f, 0.f};
    if (valid) {
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        const f2 qn = f2_split(__ldg(B.qn[v] + g));
        f2 qs;
        if (STAGE == 1) {
          qs = qn + dt * (f2_of(cf.a21e) * tex[v] + f2_of(cf.a21i) * tim[v]);
          B.S3[v][g] = f2_pack(f2_of(cf.a31e) * tex[v] + f2_of(cf.a31i) * tim[v]);
          B.SF[v][g] = f2_pack(f2_of(cf.b1) * (tex[v] + tim[v]));
        } else {
          const f2 s3 = ld2(B.S3[v] + g) + f2_of(cf.a32e) * tex[v] + f2_of(cf.a32i) * tim[v];
          qs = qn + dt * s3;
          B.SF[v][g] = f2_pack(ld2(B.SF[v] + g) + f2_of(cf.b2) * (tex[v] + tim[v]));
        }
        B.qi[v][g] = f2_pack(qs);
        if (v == VD) xq[0] = qs.h;
        if (v == VMZ) xq[1] = qs.h;
        if (v == VRT) xq[2] = qs.h;
      }
    }
    if (B.X) {  // the element's q* as feature rows of the guess network
      __syncthreads();
      __nv_bfloat16* sx = reinterpret_cast<__nv_bfloat16*>(st);  // [NF][3][N1]
#pragma unroll
      for (int v = 0; v < 3; ++v) sx[((i + N1 * j) * 3 + v) * N1 + k] = __float2bfloat16_rn(xq[v] * B.xs[v]);
      __syncthreads();
      if (valid && p < 3 * NF) {
        const int cij = p / 3, v = p - 3 * cij;
        const size_t row = (size_t)(ex + op.NeX * ey) * NF + cij;
        __nv_bfloat16* dst = B.X + row * B.xdinp + v * op.L + ez * N1;
        if constexpr (N1 == 8) *reinterpret_cast<uint4*>(dst) = *reinterpret_cast<const uint4*>(sx + (cij * 3 + v) * N1);
        else *reinterpret_cast<uint2*>(dst) = *reinterpret_cast<const uint2*>(sx + (cij * 3 + v) * N1);
      }
    }
    return;
  }
  // STAGE 3: q^{n+1} = q^n + dt (SF + b3 (t_ex + t_im)), then the modal filter of the deviation
  // from the reference state (DENS_hyd*(Uref, Vref) for MOMX/MOMY, 0 otherwise)
  f2 qnew[5], dev[5], ref[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    qnew[v] = Z2;
    dev[v] = Z2;
    ref[v] = v == VMX ? dh * U : (v == VMY ? dh * V : Z2);
    if (valid) {
      qnew[v] = f2_split(__ldg(B.qn[v] + g)) + dt * (ld2(B.SF[v] + g) + f2_of(cf.b3) * (tex[v] + tim[v]));
      dev[v] = qnew[v] - ref[v];
    }
  }
  if (B.dtrc && valid) B.dtrc[g] = (double)qnew[VD].h + (double)qnew[VD].l;  // DDENS_TRC: before the filter
  if (!filter_on) {
    if (valid) {
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        const double o64 = (double)qnew[v].h + (double)qnew[v].l;
        B.qn[v][g] = o64;
        if (B.qh[0]) B.qh[v][g] = o64;
        B.qnf[v][g] = f2_pack(dev[v]);
      }
    }
    return;
  }
  __syncthreads();  // everyone is done with the shared arrays
  filter_store<N1>(op, s_st + le * 6 * Np, s_fl + le * 15 * Np, dev, ref, B, g, valid, i, j, k, p);
}

template <int N1>
constexpr int epb_p() { return N1 == 4 ? 4 : 1; }

template <int N1, int STAGE, bool HEVE = false>
int launch_pair_n(const OpsP& op, const ProfP& pf, const double* dens64, const StagePairBufs& B, const PairCoef& cf,
                  int Ne, int filt, cudaStream_t s, int ke0 = 0) {
  constexpr int EPB = epb_p<N1>(), Np = N1 * N1 * N1, NF = N1 * N1;
  const size_t smem = sizeof(float2) * EPB * (21 * Np + 5 * 6 * NF + 5 * 2 * NF);
  auto kfn = k_stage_pair<N1, EPB, STAGE, HEVE>;
  cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (Ne <= ke0) return (int)cudaSuccess;
  // the grid's resident width in elements: the block that follows a block on its SM starts about
  // that many elements further on
  int dev = 0, nsm = 0, nb = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kfn, EPB * Np, smem);
  const int pf_next = nsm * nb * EPB;
  kfn<<<(Ne - ke0 + EPB - 1) / EPB, EPB * Np, smem, s>>>(op, pf, dens64, B, cf, Ne, filt, ke0, pf_next);
  return (int)cudaGetLastError();
}

}  // namespace

int launch_stage_pair_heve(int N1, int stage, const OpsP& op, const ProfP& pf, const double* dens64,
                           const StagePairBufs& B, const PairCoef& cf, int Ne, int filt, cudaStream_t s) {
  if (N1 == 8) {
    if (stage == 1) return launch_pair_n<8, 1, true>(op, pf, dens64, B, cf, Ne, filt, s);
    if (stage == 2) return launch_pair_n<8, 2, true>(op, pf, dens64, B, cf, Ne, filt, s);
    return launch_pair_n<8, 3, true>(op, pf, dens64, B, cf, Ne, filt, s);
  }
  if (N1 == 4) {
    if (stage == 1) return launch_pair_n<4, 1, true>(op, pf, dens64, B, cf, Ne, filt, s);
    if (stage == 2) return launch_pair_n<4, 2, true>(op, pf, dens64, B, cf, Ne, filt, s);
    return launch_pair_n<4, 3, true>(op, pf, dens64, B, cf, Ne, filt, s);
  }
  return (int)cudaErrorInvalidValue;
}

int launch_stage_pair(int N1, int stage, const OpsP& op, const ProfP& pf, const double* dens64,
                      const StagePairBufs& B, const PairCoef& cf, int Ne, int filt, cudaStream_t s, int ke0) {
  if (N1 == 8) {
    if (stage == 1) return launch_pair_n<8, 1>(op, pf, dens64, B, cf, Ne, filt, s, ke0);
    if (stage == 2) return launch_pair_n<8, 2>(op, pf, dens64, B, cf, Ne, filt, s, ke0);
    return launch_pair_n<8, 3>(op, pf, dens64, B, cf, Ne, filt, s, ke0);
  }
  if (N1 == 4) {
    if (stage == 1) return launch_pair_n<4, 1>(op, pf, dens64, B, cf, Ne, filt, s, ke0);
    if (stage == 2) return launch_pair_n<4, 2>(op, pf, dens64, B, cf, Ne, filt, s, ke0);
    return launch_pair_n<4, 3>(op, pf, dens64, B, cf, Ne, filt, s, ke0);
  }
  return (int)cudaErrorInvalidValue;
}

}  // namespace fedg
