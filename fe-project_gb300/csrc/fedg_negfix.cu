// fedg_negfix.cu -- the tracer negative fixer of the coupled model, FP64, one thread block per element.
//
// Restates FElib/src/microphysics/scale_atm_phy_mp_dgm_common.F90:429-556
// (atm_phy_mp_dgm_common_negative_fixer), which the tracer driver calls after the tracer step
// (fix_negative_val, FElib/src/fluid_dyn_solver/scale_atm_dyn_dgm_driver_trcadv3d.F90:550, 596-651):
//   - per element, each water species (1 + QLA + QIA of them) has its mass DENS q clipped below at
//     TRC_EPS and rescaled to the element's mass max(M0, 0); DDENS takes the mass change and the
//     internal energy CVtot PRES / Rtot the change times the species' CV and the temperature;
//   - the new mixing ratios are the new masses over the new density; the internal energy is rescaled
//     to the element's old total, the mixture's Rtot, CVtot, CPtot follow the new mixing ratios, the
//     potential energy of the mass change (DDENS - DDENS0) g z is taken out, and
//     PRES = IntEn Rtot / CVtot;  DRHOT (optional) is rebuilt from PRES with the mixture's exponent.
// The mixture's specific heats are SCALE's ATMOS_THERMODYN_specific_heat (scale_atmos_thermodyn.F90
// of SCALE, which the reference tree does not vendor): qdry = 1 - sum_q q MASS_q, Rtot = sum_q q R_q +
// qdry Rdry, and the same for CV and CP.
// Element integrals use the LGL quadrature of the flat cube: Gsqrt J w_i w_j w_k with Gsqrt = 1.
//
// Also the driver's update_pressure_specific_heat (driver_trcadv3d.F90:653-716), which precedes the
// fixer: the mixture's Rtot, CVtot, CPtot from the tracers and PRES from DRHOT with them
// (calc_pressure -> atm_dyn_dgm_nonhydro3d_common_DRHOT2PRES, nonhydro3d_common.F90:428-479:
// PRES = P00 (Rtot (THERM_hyd + DRHOT) / P00)^(CPtot / CVtot), DPRES = PRES - PRES_hyd).
#include <algorithm>
#include <cmath>
#include <vector>

#include "fedg_ctx.cuh"

namespace fedg {
namespace {

constexpr int MAXQA = 16;

struct NegFixArgs {
  double* q[MAXQA];  // QTRC of the QA tracers (Np, Ne), in place
  double mass[MAXQA], r[MAXQA], cv[MAXQA], cp[MAXQA];  // TRACER_MASS, TRACER_R, TRACER_CV, TRACER_CP
  int QA, nwat;      // nwat = 1 + QLA + QIA: the species the fixer clips
  double* ddens;
  double* pres;
  double* cvtot;
  double* cptot;
  double* rtot;
  const double* dens_hyd;
  const double* pres_hyd;
  double* drhot;     // or NULL
  double zmin, dz;   // the element layers' bottom and height
  double xk[FEDG_MAXN1];  // LGL nodes of [-1, 1]
};

// block-wide sums of two values; every thread gets both (sh: 2 * 32 doubles)
__device__ __forceinline__ void blk_sum2(double& a, double& b, double* sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
  }
  const int w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  __syncthreads();  // the previous call's readers are done with sh
  if ((threadIdx.x & 31) == 0) { sh[w] = a; sh[32 + w] = b; }
  __syncthreads();
  a = 0.0;
  b = 0.0;
  for (int i = 0; i < nw; ++i) { a += sh[i]; b += sh[32 + i]; }
}

// SCALE's mixture specific heats of the mixing ratios qv[0..QA)
__device__ __forceinline__ void specific_heat(const NegFixArgs& A, const Ops& op, const double (&qv)[MAXQA], double& Rt,
                                              double& CVt, double& CPt) {
  double qdry = 1.0, r = 0.0, cv = 0.0, cp = 0.0;
#pragma unroll
  for (int iq = 0; iq < MAXQA; ++iq) {
    if (iq < A.QA) {
      qdry = qdry - qv[iq] * A.mass[iq];
      r = r + qv[iq] * A.r[iq];
      cv = cv + qv[iq] * A.cv[iq];
      cp = cp + qv[iq] * A.cp[iq];
    }
  }
  Rt = r + qdry * op.rdry;
  CVt = cv + qdry * op.cvdry;
  CPt = cp + qdry * op.cpdry;
}

__global__ void __launch_bounds__(512) k_negative_fixer(const Ops op, const NegFixArgs A) {
  __shared__ double sh[64];
  const int ke = blockIdx.x, p = threadIdx.x;
  const int N1 = op.N1, NF = N1 * N1;
  const bool node = p < op.Np;  // blocks are whole warps: the tail threads only join the sums
  const size_t g = (size_t)ke * op.Np + (node ? p : 0);
  const int i = p % N1, j = (p / N1) % N1, k = p / NF;
  const int ez = ke / (op.NeX * op.NeY);
  constexpr double TRC_EPS = 1e-128;

  double int_w = 0.0, dens = 0.0, ddens0 = 0.0, ien0 = 0.0, temp = 0.0;
  if (node) {
    int_w = op.Jac * op.w[i] * op.w[j] * op.w[k];
    ddens0 = A.ddens[g];
    dens = A.dens_hyd[g] + ddens0;
    ien0 = A.cvtot[g] * A.pres[g] / A.rtot[g];
    temp = ien0 / (dens * A.cvtot[g]);
  }
  double ddens = ddens0, ien = ien0;
  double m1[MAXQA];  // the new masses of the water species
#pragma unroll
  for (int iq = 0; iq < MAXQA; ++iq) m1[iq] = 0.0;
#pragma unroll
  for (int iq = 0; iq < MAXQA; ++iq) {
    if (iq < A.nwat) {
      const double m0 = node ? dens * A.q[iq][g] : 0.0;
      double m1n = node ? fmax(TRC_EPS, m0) : 0.0;
      double M0 = int_w * m0, M1 = int_w * m1n;
      blk_sum2(M0, M1, sh);
      m1n = fmax(M0, 0.0) / M1 * m1n;
      ddens = ddens + (m1n - m0);
      ien = ien + (m1n - m0) * A.cv[iq] * temp;
      m1[iq] = m1n;
    }
  }
  dens = node ? A.dens_hyd[g] + ddens : 1.0;
  double qv[MAXQA];
#pragma unroll
  for (int iq = 0; iq < MAXQA; ++iq) qv[iq] = iq < A.QA ? m1[iq] / dens : 0.0;
  double E0 = int_w * ien0, E1 = int_w * ien;
  blk_sum2(E0, E1, sh);
  if (!node) return;
  ien = E0 / E1 * ien;
  double Rt, CVt, CPt;
  specific_heat(A, op, qv, Rt, CVt, CPt);
  const double zlev = A.zmin + A.dz * (ez + 0.5 * (1.0 + A.xk[k]));
  ien = ien - (ddens - ddens0) * op.grav * zlev;
  const double pres = ien * Rt / CVt;
#pragma unroll
  for (int iq = 0; iq < MAXQA; ++iq)
    if (iq < A.QA) A.q[iq][g] = qv[iq];
  A.ddens[g] = ddens;
  A.pres[g] = pres;
  A.rtot[g] = Rt;
  A.cvtot[g] = CVt;
  A.cptot[g] = CPt;
  if (A.drhot)
    A.drhot[g] = op.pres00 / Rt * pow(pres / op.pres00, CVt / CPt) -
                 op.pres00 / op.rdry * pow(A.pres_hyd[g] / op.pres00, op.cvdry / op.cpdry);
}

struct HeatArgs {
  const double* q[MAXQA];
  double mass[MAXQA], r[MAXQA], cv[MAXQA], cp[MAXQA];
  int QA;
  const double* drhot;
  const double* pres_hyd;
  const double* therm_hyd;
  double* rtot;
  double* cvtot;
  double* cptot;
  double* pres;
  double* dpres;  // or NULL
};

// update_pressure_specific_heat, node by node: the mixture's Rtot, CVtot, CPtot, then PRES from
// RHOT = THERM_hyd + DRHOT with the mixture's exponent
__global__ void __launch_bounds__(256) k_specific_heat_pressure(const Ops op, const HeatArgs A, size_t n) {
  for (size_t g = blockIdx.x * (size_t)blockDim.x + threadIdx.x; g < n; g += (size_t)gridDim.x * blockDim.x) {
    double qdry = 1.0, r = 0.0, cv = 0.0, cp = 0.0;
#pragma unroll
    for (int iq = 0; iq < MAXQA; ++iq) {
      if (iq < A.QA) {
        const double q = A.q[iq][g];
        qdry = qdry - q * A.mass[iq];
        r = r + q * A.r[iq];
        cv = cv + q * A.cv[iq];
        cp = cp + q * A.cp[iq];
      }
    }
    const double Rt = r + qdry * op.rdry, CVt = cv + qdry * op.cvdry, CPt = cp + qdry * op.cpdry;
    A.rtot[g] = Rt;
    A.cvtot[g] = CVt;
    A.cptot[g] = CPt;
    const double rhot = A.therm_hyd[g] + A.drhot[g];
    const double pres = op.pres00 * pow(Rt * (1.0 / op.pres00) * rhot, CPt / CVt);
    A.pres[g] = pres;
    if (A.dpres) A.dpres[g] = pres - A.pres_hyd[g];
  }
}

}  // namespace
}  // namespace fedg

extern "C" int fedg_trc_specific_heat_pressure(fedg_ctx* c, const double* const* QTRC, int QA, const double* trc_mass,
                                               const double* trc_r, const double* trc_cv, const double* trc_cp,
                                               const double* DRHOT, const double* PRES_hyd, const double* THERM_hyd,
                                               double* Rtot, double* CVtot, double* CPtot, double* PRES,
                                               double* DPRES) {
  if (!c || !QTRC || !trc_mass || !trc_r || !trc_cv || !trc_cp || !DRHOT || !PRES_hyd || !THERM_hyd || !Rtot ||
      !CVtot || !CPtot || !PRES)
    return api_fail("fedg_trc_specific_heat_pressure: null argument");
  if (QA < 0 || QA > MAXQA) return api_fail("fedg_trc_specific_heat_pressure: QA must be 0..16");
  HeatArgs A{};
  for (int iq = 0; iq < QA; ++iq) {
    if (!QTRC[iq]) return api_fail("fedg_trc_specific_heat_pressure: null tracer field");
    A.q[iq] = QTRC[iq];
    A.mass[iq] = trc_mass[iq];
    A.r[iq] = trc_r[iq];
    A.cv[iq] = trc_cv[iq];
    A.cp[iq] = trc_cp[iq];
  }
  A.QA = QA;
  A.drhot = DRHOT; A.pres_hyd = PRES_hyd; A.therm_hyd = THERM_hyd;
  A.rtot = Rtot; A.cvtot = CVtot; A.cptot = CPtot; A.pres = PRES; A.dpres = DPRES;
  cudaSetDevice(c->d.device);
  const size_t n = c->n;
  const int grid = (int)std::min<size_t>((n + 255) / 256, (size_t)152 * 16);
  const int r = tracked(c, FEDG_K_TRC_AUX, [&] {
    k_specific_heat_pressure<<<grid, 256, 0, c->stream>>>(c->op, A, n);
    return (int)cudaGetLastError();
  });
  return r ? api_cuda_fail((cudaError_t)r, "fedg_trc_specific_heat_pressure") : 0;
}

extern "C" int fedg_trc_negative_fixer(fedg_ctx* c, double* const* QTRC, int QA, int QLA, int QIA,
                                       const double* trc_mass, const double* trc_r, const double* trc_cv,
                                       const double* trc_cp, double* DDENS, double* PRES, double* CVtot,
                                       double* CPtot, double* Rtot, const double* DENS_hyd, const double* PRES_hyd,
                                       double* DRHOT, double dt) {
  (void)dt;  // in FElib's argument list, unused by the fixer
  if (!c || !QTRC || !trc_mass || !trc_r || !trc_cv || !trc_cp || !DDENS || !PRES || !CVtot || !CPtot || !Rtot ||
      !DENS_hyd || !PRES_hyd)
    return api_fail("fedg_trc_negative_fixer: null argument");
  if (QA < 1 || QA > MAXQA) return api_fail("fedg_trc_negative_fixer: QA must be 1..16");
  if (QLA < 0 || QIA < 0 || 1 + QLA + QIA != QA)
    return api_fail("fedg_trc_negative_fixer: QA must equal 1 + QLA + QIA (FElib's fixer leaves the mixing ratios of "
                    "other tracers undefined)");
  NegFixArgs A{};
  for (int iq = 0; iq < QA; ++iq) {
    if (!QTRC[iq]) return api_fail("fedg_trc_negative_fixer: null tracer field");
    A.q[iq] = QTRC[iq];
    A.mass[iq] = trc_mass[iq];
    A.r[iq] = trc_r[iq];
    A.cv[iq] = trc_cv[iq];
    A.cp[iq] = trc_cp[iq];
  }
  A.QA = QA;
  A.nwat = 1 + QLA + QIA;
  A.ddens = DDENS; A.pres = PRES; A.cvtot = CVtot; A.cptot = CPtot; A.rtot = Rtot;
  A.dens_hyd = DENS_hyd; A.pres_hyd = PRES_hyd; A.drhot = DRHOT;
  A.zmin = c->d.zmin;
  A.dz = (c->d.zmax - c->d.zmin) / c->d.NeZ;
  lgl_nodes_1d(c->N1 - 1, A.xk);
  cudaSetDevice(c->d.device);
  const int threads = ((c->Np + 31) / 32) * 32;
  const int r = tracked(c, FEDG_K_TRC_AUX, [&] {
    k_negative_fixer<<<c->Ne, threads, 0, c->stream>>>(c->op, A);
    return (int)cudaGetLastError();
  });
  return r ? api_cuda_fail((cudaError_t)r, "fedg_trc_negative_fixer") : 0;
}
