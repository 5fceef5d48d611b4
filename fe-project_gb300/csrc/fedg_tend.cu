// fedg_tend.cu -- explicit DG tendency (volume + Rusanov face flux + Lift), the modal
// filter and DRHOT->DPRES, FP64, one thread block per element (or per few elements).
//
// Restates, on the flat cube domain (Gsqrt = 1, GI3 = 0):
//   HEVE  FElib/src/fluid_dyn_solver/scale_atm_dyn_dgm_nonhydro3d_rhot_heve.F90:292-489
//         + Rusanov flux ..._rhot_heve_numflux.F90:946-1139
//   HEVI  ..._rhot_hevi.F90:289-482 + ..._rhot_hevi_numflux.F90:232-418
//   Div_var5 / Lift / VFilterPM1 of scale_element_operation_tensorprod3D(_kernel).F90
//   modal filter ..._dgm_modalfilter.F90:49-130, DRHOT2PRES ..._nonhydro3d_common.F90:428-479
//
// Data layout in HBM: five (Np, Ne) FP64 fields, node fastest -- the FElib layout, so a
// thread block reads each field of its element as one contiguous Np*8-byte run.
// Exterior states: periodic neighbours in x/y; at the lids the element's own state with
// MOMZ reflected (what FElib's halo copy + slip ApplyBC produce, dgm_bnd.F90:323-341).
#include "fedg_common.cuh"
#include "fedg_kernels.cuh"

namespace fedg {

template <int N1, int EPB, bool HEVI>
__global__ void __launch_bounds__(EPB* N1* N1* N1)
    k_tend_fp64(const Ops op, const Prof pf, const F5c q, const double* __restrict__ dpres,
                const F5 t, int Ne) {
  constexpr int Np = N1 * N1 * N1, NF = N1 * N1, N = N1 - 1;
  extern __shared__ double sm[];
  double* s_st = sm;                      // [EPB][6][Np]   state + DPRES
  double* s_fl = s_st + EPB * 6 * Np;     // [EPB][15][Np]  fluxes, c = dir*5 + var
  double* s_df = s_fl + EPB * 15 * Np;    // [EPB][5][6*NF] del_flux
  const int tid = threadIdx.x;
  const int le = tid / Np, p = tid - le * Np;
  const int ke = blockIdx.x * EPB + le;
  const bool valid = ke < Ne;
  const int i = p % N1, j = (p / N1) % N1, k = p / NF;
  const int nxy = op.NeX * op.NeY;
  const int ez = valid ? ke / nxy : 0;
  const int ey = valid ? (ke - ez * nxy) / op.NeX : 0;
  const int ex = valid ? ke - ez * nxy - ey * op.NeX : 0;
  double* st = s_st + le * 6 * Np;
  double* fl = s_fl + le * 15 * Np;
  double* df = s_df + le * 5 * 6 * NF;
  const size_t g = (size_t)ke * Np + p;
  const int lev = ez * N1 + k;

  double qv[5], dp = 0.0;
  if (valid) {
#pragma unroll
    for (int v = 0; v < 5; ++v) qv[v] = __ldg(q.v[v] + g);
    dp = __ldg(dpres + g);
  } else {
#pragma unroll
    for (int v = 0; v < 5; ++v) qv[v] = 0.0;
  }
#pragma unroll
  for (int v = 0; v < 5; ++v) st[v * Np + p] = qv[v];
  st[5 * Np + p] = dp;

  // --- volume fluxes (heve.F90:385-418 / hevi.F90:384-413) ---
  {
    const double dh = valid ? __ldg(pf.dens + lev) : 1.0;
    const double th = valid ? __ldg(pf.therm + lev) : 0.0;
    const double mx = qv[VMX], my = qv[VMY], mz = qv[VMZ];
    const double rdens = 1.0 / (qv[VD] + dh);
    const double pt = (th + qv[VRT]) * rdens;
    const double u = mx * rdens, v = my * rdens, w = mz * rdens;
    fl[(0 * 5 + VD) * Np + p] = mx;
    fl[(1 * 5 + VD) * Np + p] = my;
    fl[(2 * 5 + VD) * Np + p] = mz;
    fl[(0 * 5 + VRT) * Np + p] = mx * pt;
    fl[(1 * 5 + VRT) * Np + p] = my * pt;
    fl[(2 * 5 + VRT) * Np + p] = HEVI ? 0.0 : mz * pt;
    fl[(0 * 5 + VMZ) * Np + p] = mx * w;
    fl[(1 * 5 + VMZ) * Np + p] = my * w;
    fl[(2 * 5 + VMZ) * Np + p] = HEVI ? mz * w : mz * w + dp;
    fl[(0 * 5 + VMX) * Np + p] = mx * u + dp;
    fl[(1 * 5 + VMX) * Np + p] = my * u;
    fl[(2 * 5 + VMX) * Np + p] = mz * u;
    fl[(0 * 5 + VMY) * Np + p] = mx * v;
    fl[(1 * 5 + VMY) * Np + p] = my * v + dp;
    fl[(2 * 5 + VMY) * Np + p] = mz * v;
  }
  __syncthreads();

  // --- Rusanov face flux, del_flux = F* - F^- (numflux get_generalvc) ---
  if (valid) {
    const double gamm = op.kap;
    for (int fi = p; fi < 6 * NF; fi += Np) {
      const int f = fi / NF, ab = fi - f * NF, a = ab % N1, b = ab / N1;
      int iM, jM, kM;
      face_node<N1>(f, a, b, iM, jM, kM);
      const int pM = iM + N1 * jM + NF * kM;
      long kn;
      int levP = ez * N1 + kM;
      switch (f) {
        case 0: kn = (long)ke + (ey > 0 ? -op.NeX : (op.NeY - 1) * op.NeX); break;
        case 1: kn = (long)ke + (ex < op.NeX - 1 ? 1 : -(op.NeX - 1)); break;
        case 2: kn = (long)ke + (ey < op.NeY - 1 ? op.NeX : -(op.NeY - 1) * op.NeX); break;
        case 3: kn = (long)ke + (ex > 0 ? -1 : op.NeX - 1); break;
        case 4: kn = ez > 0 ? (long)ke - nxy : -1; levP = (ez - 1) * N1 + N; break;
        default: kn = ez < op.NeZ - 1 ? (long)ke + nxy : -1; levP = (ez + 1) * N1; break;
      }
      const int levM = ez * N1 + kM;
      double ddM = st[VD * Np + pM], mxM = st[VMX * Np + pM], myM = st[VMY * Np + pM];
      double mzM = st[VMZ * Np + pM], drM = st[VRT * Np + pM], dpM = st[5 * Np + pM];
      double ddP, mxP, myP, mzP, drP, dpP;
      // a boundary of a decomposed mesh: the exterior face layer comes from the halo exchange
      const int hsd = halo_side(f, ex, ey, op.NeX, op.NeY);
      const double* hxs = hsd >= 0 ? op.hx[hsd] : nullptr;
      if (hxs) {
        const size_t per = halo_stride(hsd, op.NeX, op.NeY, op.NeZ, NF), h = halo_index(hsd, ex, ey, ez, ab, op.NeX, op.NeY, NF);
        ddP = __ldg(hxs + h); mxP = __ldg(hxs + per + h); myP = __ldg(hxs + 2 * per + h);
        mzP = __ldg(hxs + 3 * per + h); drP = __ldg(hxs + 4 * per + h); dpP = __ldg(hxs + 5 * per + h);
      } else if (kn >= 0) {
        int i2, j2, k2;
        face_node<N1>(face_opp(f), a, b, i2, j2, k2);
        const size_t gP = (size_t)kn * Np + i2 + N1 * j2 + NF * k2;
        ddP = __ldg(q.v[VD] + gP); mxP = __ldg(q.v[VMX] + gP); myP = __ldg(q.v[VMY] + gP);
        mzP = __ldg(q.v[VMZ] + gP); drP = __ldg(q.v[VRT] + gP); dpP = __ldg(dpres + gP);
      } else {  // slip lid
        levP = levM;
        ddP = ddM; mxP = mxM; myP = myM; mzP = -mzM; drP = drM; dpP = dpM;
      }
      const double nx = (f == 1) ? 1.0 : (f == 3 ? -1.0 : 0.0);
      const double ny = (f == 2) ? 1.0 : (f == 0 ? -1.0 : 0.0);
      const double nz = (f == 5) ? 1.0 : (f == 4 ? -1.0 : 0.0);
      const double fs = f >= 4 ? op.FSz : ((f & 1) ? op.FSx : op.FSy);
      const double densM = ddM + __ldg(pf.dens + levM), densP = ddP + __ldg(pf.dens + levP);
      const double rhotM = __ldg(pf.therm + levM) + drM, rhotP = __ldg(pf.therm + levP) + drP;
      const double phM = __ldg(pf.pres + levM), phP = __ldg(pf.pres + levP);
      const double tmp1 = 0.5 * fs;
      double* o = df + ab + f * NF;
      const int S = 6 * NF;
      if (!HEVI) {
        const double velM = (mxM * nx + myM * ny + mzM * nz) / densM;
        const double velP = (mxP * nx + myP * ny + mzP * nz) / densP;
        const double alpha = fmax(sqrt(gamm * (phM + dpM) / densM) + fabs(velM),
                                  sqrt(gamm * (phP + dpP) / densP) + fabs(velP));
        o[VD * S] = tmp1 * (densP * velP - densM * velM - alpha * (ddP - ddM));
        o[VRT * S] = tmp1 * (rhotP * velP - rhotM * velM - alpha * (drP - drM));
        o[VMZ * S] = tmp1 * (mzP * velP - mzM * velM + (dpP - dpM) * nz - alpha * (mzP - mzM));
        o[VMX * S] = tmp1 * (mxP * velP - mxM * velM + nx * (dpP - dpM) - alpha * (mxP - mxM));
        o[VMY * S] = tmp1 * (myP * velP - myM * velM + ny * (dpP - dpM) - alpha * (myP - myM));
      } else {
        const double velhM = (mxM * nx + myM * ny) / densM;
        const double velhP = (mxP * nx + myP * ny) / densP;
        const double velM = velhM + mzM * nz / densM;
        const double velP = velhP + mzP * nz / densP;
        const double swV = 1.0 - nz * nz;
        const double alpha = swV * fmax(sqrt(gamm * (phM + dpM) / densM) + fabs(velM),
                                        sqrt(gamm * (phP + dpP) / densP) + fabs(velP));
        o[VD * S] = tmp1 * (densP * velhP - densM * velhM - alpha * (ddP - ddM));
        o[VRT * S] = tmp1 * (rhotP * velhP - rhotM * velhM - alpha * (drP - drM));
        o[VMZ * S] = tmp1 * (mzP * velP - mzM * velM - alpha * (mzP - mzM));
        o[VMX * S] = tmp1 * (mxP * velP - mxM * velM + nx * (dpP - dpM) - alpha * (mxP - mxM));
        o[VMY * S] = tmp1 * (myP * velP - myM * velM + ny * (dpP - dpM) - alpha * (myP - myM));
      }
    }
  }
  __syncthreads();
  if (!valid) return;

  // --- Div_var5 (D1D along x, y, z) + tensor-product Lift, combined (heve.F90:424-465) ---
  const int S = 6 * NF;
  double out[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    double sx = 0.0, sy = 0.0, sz = 0.0;
#pragma unroll
    for (int l = 0; l < N1; ++l) {
      sx = fma(op.D[i * N1 + l], fl[(0 * 5 + v) * Np + l + N1 * j + NF * k], sx);
      sy = fma(op.D[j * N1 + l], fl[(1 * 5 + v) * Np + i + N1 * l + NF * k], sy);
      sz = fma(op.D[k * N1 + l], fl[(2 * 5 + v) * Np + i + N1 * j + NF * l], sz);
    }
    const double* d = df + v * S;
    const double lf = op.Lb[j] * d[0 * NF + i + N1 * k] + op.Lt[i] * d[1 * NF + j + N1 * k] +
                      op.Lt[j] * d[2 * NF + i + N1 * k] + op.Lb[i] * d[3 * NF + j + N1 * k] +
                      op.Lb[k] * d[4 * NF + i + N1 * j] + op.Lt[k] * d[5 * NF + i + N1 * j];
    const bool horiz_only = HEVI && (v == VD || v == VRT);
    out[v] = -(op.E11 * sx + op.E22 * sy + (horiz_only ? 0.0 : op.E33 * sz) + lf);
  }
  if (!HEVI) {  // -g * VFilterPM1(DDENS)
    double drho = 0.0;
#pragma unroll
    for (int l = 0; l < N1; ++l) drho = fma(op.T[k * N1 + l], st[VD * Np + i + N1 * j + NF * l], drho);
    out[VMZ] -= op.grav * drho;
  }
  out[VMX] += op.coriolis_f * qv[VMY];
  out[VMY] -= op.coriolis_f * qv[VMX];
#pragma unroll
  for (int v = 0; v < 5; ++v) t.v[v][g] = out[v];
}

// ---------------------------------------------------------------------------------------
// modal filter, in place: q <- Fv_z Fh_y Fh_x q  (tensorprod3D_kernel.F90:2555-2618)
// ---------------------------------------------------------------------------------------
template <int N1, int EPB>
__global__ void __launch_bounds__(EPB* N1* N1* N1) k_filter_fp64(const Ops op, F5 q, int Ne) {
  constexpr int Np = N1 * N1 * N1, NF = N1 * N1;
  extern __shared__ double sm[];
  const int tid = threadIdx.x, le = tid / Np, p = tid - le * Np;
  const int ke = blockIdx.x * EPB + le;
  const bool valid = ke < Ne;
  const int i = p % N1, j = (p / N1) % N1, k = p / NF;
  double* a = sm + le * 2 * Np;
  double* b = a + Np;
  const size_t g = (size_t)ke * Np + p;
  for (int v = 0; v < 5; ++v) {
    a[p] = valid ? q.v[v][g] : 0.0;
    __syncthreads();
    double s = 0.0;
#pragma unroll
    for (int l = 0; l < N1; ++l) s = fma(op.F[i * N1 + l], a[l + N1 * j + NF * k], s);
    b[p] = s;
    __syncthreads();
    s = 0.0;
#pragma unroll
    for (int l = 0; l < N1; ++l) s = fma(op.F[j * N1 + l], b[i + N1 * l + NF * k], s);
    __syncthreads();
    a[p] = s;
    __syncthreads();
    s = 0.0;
#pragma unroll
    for (int l = 0; l < N1; ++l) s = fma(op.Fv[k * N1 + l], a[i + N1 * j + NF * l], s);
    if (valid) q.v[v][g] = s;
    __syncthreads();
  }
}

// DRHOT -> (PRES, DPRES), FP64 (nonhydro3d_common.F90:428-479)
__global__ void k_drhot2pres(const Ops op, const Prof pf, const double* __restrict__ drhot,
                             double* __restrict__ pres, double* __restrict__ dpres, size_t n) {
  const size_t g = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n) return;
  const int p = (int)(g % op.Np);
  const size_t ke = g / op.Np;
  const int ez = (int)(ke / ((size_t)op.NeX * op.NeY));
  const int lev = ez * op.N1 + p / (op.N1 * op.N1);
  const double rhot = __ldg(pf.therm + lev) + drhot[g];
  double pr;
  dpres[g] = dpres_of(op, rhot, __ldg(pf.pres + lev), &pr);
  if (pres) pres[g] = pr;
}

// ---------------------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------------------
template <int N1>
static constexpr int epb_of() { return N1 <= 4 ? (N1 <= 2 ? 16 : (N1 == 3 ? 8 : 4)) : 1; }

template <int N1>
static int launch_tend_n(const Ops& op, const Prof& pf, const F5c& q, const double* dpres, const F5& t, int Ne,
                         int hevi, cudaStream_t s) {
  constexpr int EPB = epb_of<N1>();
  constexpr int Np = N1 * N1 * N1;
  const size_t smem = sizeof(double) * EPB * (21 * Np + 5 * 6 * N1 * N1);
  const int grid = (Ne + EPB - 1) / EPB;
  if (hevi) {
    auto kfn = k_tend_fp64<N1, EPB, true>;
    cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    kfn<<<grid, EPB * Np, smem, s>>>(op, pf, q, dpres, t, Ne);
  } else {
    auto kfn = k_tend_fp64<N1, EPB, false>;
    cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    kfn<<<grid, EPB * Np, smem, s>>>(op, pf, q, dpres, t, Ne);
  }
  return (int)cudaGetLastError();
}

int launch_tend_fp64(const Ops& op, const Prof& pf, const F5c& q, const double* dpres, const F5& t, int Ne,
                     int hevi, cudaStream_t s) {
  switch (op.N1) {
    case 2: return launch_tend_n<2>(op, pf, q, dpres, t, Ne, hevi, s);
    case 3: return launch_tend_n<3>(op, pf, q, dpres, t, Ne, hevi, s);
    case 4: return launch_tend_n<4>(op, pf, q, dpres, t, Ne, hevi, s);
    case 5: return launch_tend_n<5>(op, pf, q, dpres, t, Ne, hevi, s);
    case 6: return launch_tend_n<6>(op, pf, q, dpres, t, Ne, hevi, s);
    case 7: return launch_tend_n<7>(op, pf, q, dpres, t, Ne, hevi, s);
    case 8: return launch_tend_n<8>(op, pf, q, dpres, t, Ne, hevi, s);
  }
  return (int)cudaErrorInvalidValue;
}

template <int N1>
static int launch_filter_n(const Ops& op, const F5& q, int Ne, cudaStream_t s) {
  constexpr int EPB = epb_of<N1>();
  constexpr int Np = N1 * N1 * N1;
  const size_t smem = sizeof(double) * EPB * 2 * Np;
  k_filter_fp64<N1, EPB><<<(Ne + EPB - 1) / EPB, EPB * Np, smem, s>>>(op, q, Ne);
  return (int)cudaGetLastError();
}

int launch_filter_fp64(const Ops& op, const F5& q, int Ne, cudaStream_t s) {
  switch (op.N1) {
    case 2: return launch_filter_n<2>(op, q, Ne, s);
    case 3: return launch_filter_n<3>(op, q, Ne, s);
    case 4: return launch_filter_n<4>(op, q, Ne, s);
    case 5: return launch_filter_n<5>(op, q, Ne, s);
    case 6: return launch_filter_n<6>(op, q, Ne, s);
    case 7: return launch_filter_n<7>(op, q, Ne, s);
    case 8: return launch_filter_n<8>(op, q, Ne, s);
  }
  return (int)cudaErrorInvalidValue;
}

int launch_drhot2pres(const Ops& op, const Prof& pf, const double* drhot, double* pres, double* dpres, size_t n,
                      cudaStream_t s) {
  const int bs = 256;
  k_drhot2pres<<<(unsigned)((n + bs - 1) / bs), bs, 0, s>>>(op, pf, drhot, pres, dpres, n);
  return (int)cudaGetLastError();
}

}  // namespace fedg
