// fedg_trc.cu -- tracer advection: HEVE DG transport of a mixing ratio by a (time-averaged) mass
// flux, with the nonnegativity limiter of Light and Durran (2016) -- FCT on the lowest mode, then
// truncation and mass-aware rescaling (TMAR).  FP64, one thread block per element.
//
// Restates on the flat cube domain (Gsqrt = GsqrtH = 1, G13 = G23 = 0, G11 = G22 = 1,
// J = dx dy dz / 8, J * Fscale = the face Jacobian):
//   FElib/src/fluid_dyn_solver/scale_atm_dyn_dgm_trcadvect3d_heve.F90
//     cal_alphdens_advtest :404-455; save_massflux + cal_alphdens_dyn :343-401, 460-551
//     calc_fct_coef :234-306 with get_netOutwardFlux :678-777
//     cal_tend :149-231 with get_delflux :554-674;  TMAR :311-340;  FaceIntMat :75-137
//   tracer modal filter  ..._dgm_modalfilter.F90:232-270
//   tracer RK            FElib/src/common/scale_timeint_rk.F90:1390-1498 (low-storage form)
//   one tracer's step    ..._driver_trcadv3d.F90:420-545
//
// Layout: every field is FElib's (Np, Ne) FP64 array; the Rusanov coefficients alph_dens_M/P are
// face-node arrays (NfpTot, Ne) with face f = 0..5 (y-, x+, y+, x-, z-, z+) and face node a + N1*b.
// Exterior values: the periodic neighbour's node, or at a slip lid the element's own node with the
// vertical mass flux reflected (FElib's halo copy + ApplyBC on the mass flux).
#include <cmath>
#include <cstring>
#include <vector>

#include "fedg_ctx.cuh"

namespace fedg {
namespace {

struct TrcIn {
  const double* Q;       // mixing ratio of the stage
  const double* mf[3];   // MFLX_x, MFLX_y, MFLX_z
  const double* aM;      // alph_dens_M (NfpTot, Ne)
  const double* aP;      // alph_dens_P
  const double* rhoq;    // RHOQ_tp (physics tendency of dens*q) or NULL
  const double* ddens;   // DDENS_TRC
  const double* ddens0;  // DDENS0_TRC
};

struct TrcFct {          // calc_fct_coef
  double c_ssm1;         // stage density DENS_hyd + (1 - c) DDENS0 + c DDENS
  double dt;             // dt * gam(s+1,s) / sig(s+1,s)
  double* fct_elem;      // [Ne] or NULL
  double* fct_node;      // (Np, Ne) or NULL
};

struct TrcStage {        // cal_tend + Advance_trcvar (+ last-stage filter, TMAR and rescale)
  const double* fct_elem;   // per-element coefficient (fused update) or NULL
  const double* fct_node;   // nodal coefficient field (FElib's fct_coef) or NULL; both NULL: 1
  double* tend;             // (Np, Ne) tendency output or NULL
  int advance;              // 0: tendency only
  int first, last, acc;     // first stage (store var0), last stage, varTmp accumulation active
  double sig_ss, gam_ss, sig_Ns, gam_Ns, c_ssm1, c_ss;  // gam_* include dt
  double* q_out;            // next stage's mixing ratio (not the last stage)
  double* var0;             // q^n * dens^n
  double* vtmp;             // varTmp
  int filter, tmar;         // last stage
  const double* ddens_fin;  // DDENS of the dynamics (final rescale); NULL: DDENS_TRC
  double* qtrc_out;         // last stage: QTRC
};

struct TrcFilt {
  double Fh[FEDG_MAXN1 * FEDG_MAXN1], Fv[FEDG_MAXN1 * FEDG_MAXN1];
};

// outward normal component on face f of the vector field (vx, vy, vz) at node g; the normals are
// axis-aligned, so only one component is loaded.  flip_z reflects the vertical component (the
// exterior side of a slip lid).
__device__ __forceinline__ double normal_comp(int f, const double* __restrict__ vx, const double* __restrict__ vy,
                                              const double* __restrict__ vz, size_t g, bool flip_z = false) {
  switch (f) {
    case 0: return -__ldg(vy + g);
    case 1: return __ldg(vx + g);
    case 2: return __ldg(vy + g);
    case 3: return -__ldg(vx + g);
    case 4: return flip_z ? __ldg(vz + g) : -__ldg(vz + g);
    default: return flip_z ? -__ldg(vz + g) : __ldg(vz + g);
  }
}

// Rusanov flux 0.5 ((q+ m+ + q- m-) - a+ q+ + a- q-) in FElib's operation order, without
// contraction, so that both sides of a slip lid cancel to exactly zero.
__device__ __forceinline__ double trc_numflux(double qM, double qP, double mfM, double mfP, double aM, double aP) {
  const double s = __dadd_rn(__dmul_rn(qP, mfP), __dmul_rn(qM, mfM));
  return __dmul_rn(0.5, __dadd_rn(__dsub_rn(s, __dmul_rn(aP, qP)), __dmul_rn(aM, qM)));
}

// sum of v over the Np threads of element le of the block, in a fixed order
template <int N1, int EPB>
__device__ __forceinline__ double elem_sum(double v, double* s_red, int le, int p) {
  constexpr int Np = N1 * N1 * N1;
  __syncthreads();
  if constexpr (Np % 32 == 0) {
    constexpr int NW = Np / 32;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((p & 31) == 0) s_red[le * NW + (p >> 5)] = v;
    __syncthreads();
    double s = 0.0;
#pragma unroll
    for (int w = 0; w < NW; ++w) s += s_red[le * NW + w];
    return s;
  } else {
    s_red[le * Np + p] = v;
    __syncthreads();
    double s = 0.0;
    for (int q = 0; q < Np; ++q) s += s_red[le * Np + q];
    return s;
  }
}

// ---------------------------------------------------------------------------------------
// calc_fct_coef: fct = max(0, min(1, Q_e / (sum_f max(0, outflux_f) + 1e-10)))
// ---------------------------------------------------------------------------------------
template <int N1, int EPB>
__global__ void __launch_bounds__(EPB* N1* N1* N1)
    k_trc_fct(const Ops op, const double* __restrict__ dens_prof, const TrcIn in, const TrcFct fc, int Ne) {
  constexpr int Np = N1 * N1 * N1, NF = N1 * N1;
  extern __shared__ double sm[];
  double* s_face = sm;                    // [EPB][6 NF] weighted face integrands
  double* s_out = s_face + EPB * 6 * NF;  // [EPB][6]
  double* s_red = s_out + EPB * 8;        // reduction scratch [EPB][Np]
  const int tid = threadIdx.x, le = tid / Np, p = tid - le * Np;
  const long ke = (long)blockIdx.x * EPB + le;
  const bool valid = ke < Ne;
  const int nxy = op.NeX * op.NeY;
  const int ez = valid ? (int)(ke / nxy) : 0;
  const int ey = valid ? (int)((ke - (long)ez * nxy) / op.NeX) : 0;
  const int ex = valid ? (int)(ke - (long)ez * nxy - (long)ey * op.NeX) : 0;
  const double J = op.Jac;
  double* sf = s_face + le * 6 * NF;
  if (valid) {
    for (int fi = p; fi < 6 * NF; fi += Np) {
      const int f = fi / NF, ab = fi - f * NF, a = ab % N1, b = ab / N1;
      int pM;
      size_t gP;
      long kn;
      face_exterior<N1>(op, f, a, b, ke, ex, ey, ez, nxy, pM, gP, kn);
      const size_t gM = (size_t)ke * Np + pM;
      const double mfM = normal_comp(f, in.mf[0], in.mf[1], in.mf[2], gM);
      const double mfP = normal_comp(f, in.mf[0], in.mf[1], in.mf[2], gP, kn < 0);
      const size_t fa = (size_t)ke * 6 * NF + fi;
      const double nf = trc_numflux(__ldg(in.Q + gM), __ldg(in.Q + gP), mfM, mfP, __ldg(in.aM + fa), __ldg(in.aP + fa));
      const double JF = J * (f >= 4 ? op.FSz : ((f & 1) ? op.FSx : op.FSy));
      sf[fi] = __dmul_rn(__dmul_rn(op.w[a], op.w[b]), __dmul_rn(JF, nf));
    }
  }
  // element integral of dens_ssm1 q / dt + RHOQ_tp with the LGL weights
  double v = 0.0;
  if (valid) {
    const size_t g = (size_t)ke * Np + p;
    const int i = p % N1, j = (p / N1) % N1, k = p / NF;
    const double dens = __ldg(dens_prof + ez * N1 + k) + (1.0 - fc.c_ssm1) * __ldg(in.ddens0 + g) +
                        fc.c_ssm1 * __ldg(in.ddens + g);
    v = J * (op.w[i] * op.w[j] * op.w[k]) * (dens * __ldg(in.Q + g) / fc.dt + (in.rhoq ? __ldg(in.rhoq + g) : 0.0));
  }
  const double qe = elem_sum<N1, EPB>(v, s_red, le, p);  // (synchronises: the face integrands are visible)
  if (valid && p < 6) {  // FaceIntMat row f, in face-node order
    double s = 0.0;
    for (int q = 0; q < NF; ++q) s = __dadd_rn(s, sf[p * NF + q]);
    s_out[le * 8 + p] = s;
  }
  __syncthreads();
  if (valid) {
    double net = 0.0;
#pragma unroll
    for (int f = 0; f < 6; ++f) net += fmax(0.0, s_out[le * 8 + f]);
    const double r = fmax(0.0, fmin(1.0, qe / (net + 1.0e-10)));
    if (fc.fct_elem && p == 0) fc.fct_elem[ke] = r;
    if (fc.fct_node) fc.fct_node[(size_t)ke * Np + p] = r;
  }
}

// ---------------------------------------------------------------------------------------
// last-stage post-processing of one element, value qn of node p in s_q[Np] space:
// tracer modal filter of dens*q, TMAR, rescale (dgm_modalfilter.F90:232-270, trcadvect3d_heve.F90:311-340)
// ---------------------------------------------------------------------------------------
template <int N1, int EPB>
__device__ __forceinline__ double trc_post(const Ops& op, const TrcFilt& tf, double qn, double wgt, int filter, int tmar,
                                           double* s_a, double* s_b, double* s_red, int le, int p, bool valid) {
  constexpr int Np = N1 * N1 * N1, NF = N1 * N1;
  const int i = p % N1, j = (p / N1) % N1, k = p / NF;
  double* a = s_a + le * Np;
  double* b = s_b + le * Np;
  if (filter) {
    b[p] = valid ? wgt * qn : 0.0;
    __syncthreads();
    double s = 0.0;
#pragma unroll
    for (int l = 0; l < N1; ++l) s += tf.Fh[i * N1 + l] * b[l + N1 * j + NF * k];
    a[p] = s;
    __syncthreads();
    s = 0.0;
#pragma unroll
    for (int l = 0; l < N1; ++l) s += tf.Fh[j * N1 + l] * a[i + N1 * l + NF * k];
    __syncthreads();
    b[p] = s;
    __syncthreads();
    s = 0.0;
#pragma unroll
    for (int l = 0; l < N1; ++l) s += tf.Fv[k * N1 + l] * b[i + N1 * j + NF * l];
    if (valid) qn = s / wgt;
  }
  if (tmar) {
    const double J = op.Jac;
    const double wd = valid ? J * (op.w[i] * op.w[j] * op.w[k]) * wgt : 0.0;
    const double qp = fmax(0.0, qn);
    const double q0 = elem_sum<N1, EPB>(wd * qn, s_red, le, p);
    const double q1 = elem_sum<N1, EPB>(wd * qp, s_red, le, p);
    qn = q0 / (q1 + 1.0e-32) * qp;
  }
  return qn;
}

// ---------------------------------------------------------------------------------------
// cal_tend (FCT-limited del_flux, Div, Lift) and the low-storage tracer RK advance
// ---------------------------------------------------------------------------------------
template <int N1, int EPB>
__global__ void __launch_bounds__(EPB* N1* N1* N1)
    k_trc_stage(const Ops op, const double* __restrict__ dens_prof, const TrcIn in, const TrcStage st,
                const TrcFilt tf, int Ne) {
  constexpr int Np = N1 * N1 * N1, NF = N1 * N1;
  extern __shared__ double sm[];
  double* s_fl = sm;                       // [EPB][3][Np] volume fluxes MFLX_d q
  double* s_nf = s_fl + EPB * 3 * Np;      // [EPB][6NF] numflux
  double* s_qm = s_nf + EPB * 6 * NF;      // [EPB][6NF] q- MomFlx-
  double* s_rm = s_qm + EPB * 6 * NF;      // [EPB][6NF] R-
  double* s_rp = s_rm + EPB * 6 * NF;      // [EPB][6NF] R+
  double* s_face = s_rp + EPB * 6 * NF;    // [EPB][6NF] weighted integrands; del_flux afterwards
  double* s_out = s_face + EPB * 6 * NF;   // [EPB][8]
  double* s_red = s_out + EPB * 8;         // [EPB][Np]
  double* s_b = s_red + EPB * Np;          // [EPB][Np] (filter)
  const int tid = threadIdx.x, le = tid / Np, p = tid - le * Np;
  const long ke = (long)blockIdx.x * EPB + le;
  const bool valid = ke < Ne;
  const int i = p % N1, j = (p / N1) % N1, k = p / NF;
  const int nxy = op.NeX * op.NeY;
  const int ez = valid ? (int)(ke / nxy) : 0;
  const int ey = valid ? (int)((ke - (long)ez * nxy) / op.NeX) : 0;
  const int ex = valid ? (int)(ke - (long)ez * nxy - (long)ey * op.NeX) : 0;
  const double J = op.Jac;
  const size_t g = (size_t)ke * Np + p;
  double* fl = s_fl + le * 3 * Np;
  double* nfv = s_nf + le * 6 * NF;
  double* qmv = s_qm + le * 6 * NF;
  double* rmv = s_rm + le * 6 * NF;
  double* rpv = s_rp + le * 6 * NF;
  double* sf = s_face + le * 6 * NF;

  const double q = valid ? __ldg(in.Q + g) : 0.0;
  fl[p] = valid ? __ldg(in.mf[0] + g) * q : 0.0;
  fl[Np + p] = valid ? __ldg(in.mf[1] + g) * q : 0.0;
  fl[2 * Np + p] = valid ? __ldg(in.mf[2] + g) * q : 0.0;
  if (valid) {
    const double own = st.fct_elem ? __ldg(st.fct_elem + ke) : 1.0;
    for (int fi = p; fi < 6 * NF; fi += Np) {
      const int f = fi / NF, ab = fi - f * NF, a = ab % N1, b = ab / N1;
      int pM;
      size_t gP;
      long kn;
      face_exterior<N1>(op, f, a, b, ke, ex, ey, ez, nxy, pM, gP, kn);
      const size_t gM = (size_t)ke * Np + pM;
      const double mfM = normal_comp(f, in.mf[0], in.mf[1], in.mf[2], gM);
      const double mfP = normal_comp(f, in.mf[0], in.mf[1], in.mf[2], gP, kn < 0);
      const size_t fa = (size_t)ke * 6 * NF + fi;
      const double qM = __ldg(in.Q + gM);
      const double nf = trc_numflux(qM, __ldg(in.Q + gP), mfM, mfP, __ldg(in.aM + fa), __ldg(in.aP + fa));
      const double JF = J * (f >= 4 ? op.FSz : ((f & 1) ? op.FSx : op.FSy));
      nfv[fi] = nf;
      qmv[fi] = qM * mfM;
      if (st.fct_node) {
        rmv[fi] = __ldg(st.fct_node + gM);
        rpv[fi] = __ldg(st.fct_node + gP);
      } else {
        rmv[fi] = own;
        rpv[fi] = st.fct_elem ? (kn >= 0 ? __ldg(st.fct_elem + kn) : own) : 1.0;
      }
      sf[fi] = __dmul_rn(__dmul_rn(op.w[a], op.w[b]), __dmul_rn(JF, nf));
    }
  }
  __syncthreads();
  if (valid && p < 6) {
    double s = 0.0;
    for (int qq = 0; qq < NF; ++qq) s = __dadd_rn(s, sf[p * NF + qq]);
    s_out[le * 8 + p] = s;
  }
  __syncthreads();
  if (valid) {  // del_flux = Fscale (numflux 0.5 (R+ + R- - (R+ - R-) sign(1, outflux_f)) - q- MomFlx-)
    for (int fi = p; fi < 6 * NF; fi += Np) {
      const int f = fi / NF;
      const double sg = signbit(s_out[le * 8 + f]) ? -1.0 : 1.0;
      const double RM = rmv[fi], RP = rpv[fi];
      const double fs = f >= 4 ? op.FSz : ((f & 1) ? op.FSx : op.FSy);
      sf[fi] = fs * (nfv[fi] * (0.5 * (RP + RM - (RP - RM) * sg)) - qmv[fi]);
    }
  }
  __syncthreads();

  double t = 0.0;
  if (valid) {
    double sx = 0.0, sy = 0.0, sz = 0.0;
#pragma unroll
    for (int l = 0; l < N1; ++l) {
      sx = fma(op.D[i * N1 + l], fl[l + N1 * j + NF * k], sx);
      sy = fma(op.D[j * N1 + l], fl[Np + i + N1 * l + NF * k], sy);
      sz = fma(op.D[k * N1 + l], fl[2 * Np + i + N1 * j + NF * l], sz);
    }
    const double lf = op.Lb[j] * sf[0 * NF + i + N1 * k] + op.Lt[i] * sf[1 * NF + j + N1 * k] +
                      op.Lt[j] * sf[2 * NF + i + N1 * k] + op.Lb[i] * sf[3 * NF + j + N1 * k] +
                      op.Lb[k] * sf[4 * NF + i + N1 * j] + op.Lt[k] * sf[5 * NF + i + N1 * j];
    t = -(op.E11 * sx + op.E22 * sy + op.E33 * sz + lf) + (in.rhoq ? __ldg(in.rhoq + g) : 0.0);
    if (st.tend) st.tend[g] = t;
  }
  if (!st.advance) return;  // uniform across the block

  // rk_advance_trcvar_low_storage (timeint_rk.F90:1390-1498)
  double qn = 0.0, wgt = 1.0;
  if (valid) {
    const double dh = __ldg(dens_prof + ez * N1 + k);
    const double dd = __ldg(in.ddens + g), dd0 = __ldg(in.ddens0 + g);
    const double d0 = dh + dd0;
    const double dssm1 = d0 + st.c_ssm1 * (dd - dd0);
    if (st.last) {
      qn = (st.vtmp[g] + st.sig_ss * q * dssm1 + st.gam_ss * t) / (dh + dd);
    } else {
      double v0;
      if (st.first) {
        v0 = q * d0;
        st.var0[g] = v0;
      } else {
        v0 = st.var0[g];
      }
      if (st.acc) {
        const double vt = (st.first ? 0.0 : st.vtmp[g]) + st.sig_Ns * q * dssm1 + st.gam_Ns * t;
        st.vtmp[g] = vt;
      } else if (st.first) {
        st.vtmp[g] = 0.0;
      }
      const double dss = d0 + st.c_ss * (dd - dd0);
      qn = ((1.0 - st.sig_ss) * v0 + st.sig_ss * q * dssm1 + st.gam_ss * t) / dss;
      st.q_out[g] = qn;
    }
    wgt = dh + dd;
  }
  if (!st.last) return;  // uniform across the block
  qn = trc_post<N1, EPB>(op, tf, qn, wgt, st.filter, st.tmar, s_fl, s_b, s_red, le, p, valid);
  if (valid) {
    const double dh = __ldg(dens_prof + ez * N1 + k);
    const double ddf = st.ddens_fin ? __ldg(st.ddens_fin + g) : __ldg(in.ddens + g);
    st.qtrc_out[g] = (dh + __ldg(in.ddens + g)) / (dh + ddf) * qn;
  }
}

// stand-alone tracer modal filter and/or TMAR of QTRC (in place)
template <int N1, int EPB>
__global__ void __launch_bounds__(EPB* N1* N1* N1)
    k_trc_post(const Ops op, const double* __restrict__ dens_prof, double* Q, const double* __restrict__ ddens,
               const TrcFilt tf, int filter, int tmar, int Ne) {
  constexpr int Np = N1 * N1 * N1, NF = N1 * N1;
  extern __shared__ double sm[];
  double* s_a = sm;
  double* s_b = s_a + EPB * Np;
  double* s_red = s_b + EPB * Np;
  const int tid = threadIdx.x, le = tid / Np, p = tid - le * Np;
  const long ke = (long)blockIdx.x * EPB + le;
  const bool valid = ke < Ne;
  const int nxy = op.NeX * op.NeY;
  const int ez = valid ? (int)(ke / nxy) : 0;
  const size_t g = (size_t)ke * Np + p;
  const double qn = valid ? Q[g] : 0.0;
  const double wgt = valid ? __ldg(dens_prof + ez * N1 + p / NF) + __ldg(ddens + g) : 1.0;
  const double r = trc_post<N1, EPB>(op, tf, qn, wgt, filter, tmar, s_a, s_b, s_red, le, p, valid);
  if (valid) Q[g] = r;
}

// cal_alphdens_advtest (trcadvect3d_heve.F90:404-455): one thread per face node
template <int N1>
__global__ void k_trc_alph_adv(const Ops op, const double* __restrict__ dens_prof, const double* __restrict__ ddens,
                               const double* __restrict__ mx, const double* __restrict__ my,
                               const double* __restrict__ mz, double* aM, double* aP, long Ne) {
  constexpr int Np = N1 * N1 * N1, NF = N1 * N1;
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (size_t)Ne * 6 * NF) return;
  const long ke = (long)(t / (6 * NF));
  const int fi = (int)(t - (size_t)ke * 6 * NF), f = fi / NF, ab = fi - f * NF, a = ab % N1, b = ab / N1;
  const int nxy = op.NeX * op.NeY;
  const int ez = (int)(ke / nxy), ey = (int)((ke - (long)ez * nxy) / op.NeX), ex = (int)(ke - (long)ez * nxy - (long)ey * op.NeX);
  int pM;
  size_t gP;
  long kn;
  face_exterior<N1>(op, f, a, b, ke, ex, ey, ez, nxy, pM, gP, kn);
  const size_t gM = (size_t)ke * Np + pM;
  const int kM = pM / NF, kP = (int)((gP % Np) / NF);
  const int ezP = kn >= 0 ? (int)(kn / nxy) : ez;
  const double densM = __ldg(ddens + gM) + __ldg(dens_prof + ez * N1 + kM);
  const double densP = __ldg(ddens + gP) + __ldg(dens_prof + ezP * N1 + kP);
  const double velM = normal_comp(f, mx, my, mz, gM) / densM;
  const double velP = normal_comp(f, mx, my, mz, gP, kn < 0) / densP;
  const double alpha = fmax(fabs(velM), fabs(velP));
  aM[t] = alpha * densM;
  aP[t] = alpha * densP;
}

// Stage state of save_massflux in the three representations the update paths hold it in:
// FP64 fields (FElib's), float-pair deviations and FP32 deviations (from the hydrostatic state and
// the reference-wind momentum DENS_hyd (Uref, Vref) of MOMX/MOMY).  get() returns the FP64 value.
struct StF64 {
  const double* q[5];
  __device__ double get(int v, size_t g, int) const { return __ldg(q[v] + g); }
};
struct StPair {
  const float2* q[5];
  const double* dens;  // DENS_hyd per level
  double U, V;
  __device__ double get(int v, size_t g, int lev) const {
    const float2 x = __ldg(q[v] + g);
    double d = (double)x.x + (double)x.y;
    if (v == VMX) d = fma(__ldg(dens + lev), U, d);
    if (v == VMY) d = fma(__ldg(dens + lev), V, d);
    return d;
  }
};
struct StF32 {
  const float* q[5];
  const double* dens;
  double U, V;
  __device__ double get(int v, size_t g, int lev) const {
    double d = (double)__ldg(q[v] + g);
    if (v == VMX) d = fma(__ldg(dens + lev), U, d);
    if (v == VMY) d = fma(__ldg(dens + lev), V, d);
    return d;
  }
};

template <class S>
struct MflxArgs {
  S q;                  // DDENS, MOMX, MOMY, MOMZ, DRHOT of the stage
  const double* dpres;  // DPRES or NULL (formed from DRHOT)
  double* mf[3];
  double* aM;
  double* aP;
  double w_h, w_v;
  int first, hevi;
};

template <class S>
__device__ __forceinline__ double dpres_of(const Ops& op, const Prof& pf, const MflxArgs<S>& A, size_t g, int lev) {
  if (A.dpres) return __ldg(A.dpres + g);
  const double rhot = __ldg(pf.therm + lev) + A.q.get(VRT, g, lev);
  return op.pres00 * pow(op.rdry / op.pres00 * rhot, op.kap) - __ldg(pf.pres + lev);
}

// normal momentum component (axis-aligned faces); flip_z: the exterior side of a slip lid
template <class S>
__device__ __forceinline__ double normal_mom(const S& q, int f, size_t g, int lev, bool flip_z = false) {
  switch (f) {
    case 0: return -q.get(VMY, g, lev);
    case 1: return q.get(VMX, g, lev);
    case 2: return q.get(VMY, g, lev);
    case 3: return -q.get(VMX, g, lev);
    case 4: return flip_z ? q.get(VMZ, g, lev) : -q.get(VMZ, g, lev);
    default: return flip_z ? -q.get(VMZ, g, lev) : q.get(VMZ, g, lev);
  }
}

// save_massflux (driver_nonhydro3d.F90:900-917): MFLX += w MOM of the stage
template <class S>
__global__ void k_trc_mflx(const MflxArgs<S> A, int Np, int N1, size_t nxy, size_t n) {
  const size_t g = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n) return;
  const size_t ke = g / Np;
  const int lev = (int)(ke / nxy) * N1 + (int)(g - ke * Np) / (N1 * N1);
  const double mx = A.w_h * A.q.get(VMX, g, lev), my = A.w_h * A.q.get(VMY, g, lev);
  const double mz = A.w_v * A.q.get(VMZ, g, lev);
  if (A.first) {
    A.mf[0][g] = mx;
    A.mf[1][g] = my;
    A.mf[2][g] = mz;
  } else {
    A.mf[0][g] += mx;
    A.mf[1][g] += my;
    A.mf[2][g] += mz;
  }
}

// cal_alphdens_dyn (trcadvect3d_heve.F90:460-551): one thread per face node
template <int N1, class S>
__global__ void k_trc_alph_dyn(const Ops op, const Prof pf, const MflxArgs<S> A, long Ne) {
  constexpr int Np = N1 * N1 * N1, NF = N1 * N1;
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (size_t)Ne * 6 * NF) return;
  const long ke = (long)(t / (6 * NF));
  const int fi = (int)(t - (size_t)ke * 6 * NF), f = fi / NF, ab = fi - f * NF, a = ab % N1, b = ab / N1;
  const int nxy = op.NeX * op.NeY;
  const int ez = (int)(ke / nxy), ey = (int)((ke - (long)ez * nxy) / op.NeX), ex = (int)(ke - (long)ez * nxy - (long)ey * op.NeX);
  int pM;
  size_t gP;
  long kn;
  face_exterior<N1>(op, f, a, b, ke, ex, ey, ez, nxy, pM, gP, kn);
  const size_t gM = (size_t)ke * Np + pM;
  const int levM = ez * N1 + pM / NF;
  const int levP = (kn >= 0 ? (int)(kn / nxy) : ez) * N1 + (int)((gP % Np) / NF);
  const double densM = A.q.get(VD, gM, levM) + __ldg(pf.dens + levM);
  const double densP = A.q.get(VD, gP, levP) + __ldg(pf.dens + levP);
  const double gnn = (f < 4 || !A.hevi) ? 1.0 : 0.0;  // |nx| + |ny| (+ |nz| for HEVE) on axis-aligned faces
  const double velM = normal_mom(A.q, f, gM, levM) / densM;
  const double velP = normal_mom(A.q, f, gP, levP, kn < 0) / densP;
  const double gamm = op.kap;
  const double alpha = fmax(sqrt(gnn * gamm * (__ldg(pf.pres + levM) + dpres_of(op, pf, A, gM, levM)) / densM) + fabs(velM),
                            sqrt(gnn * gamm * (__ldg(pf.pres + levP) + dpres_of(op, pf, A, gP, levP)) / densP) + fabs(velP));
  const double tw = f < 4 ? A.w_h : A.w_v;
  const double am = tw * alpha * densM, ap = tw * alpha * densP;
  if (A.first) {
    A.aM[t] = am;
    A.aP[t] = ap;
  } else {
    A.aM[t] += am;
    A.aP[t] += ap;
  }
}

template <int N1>
constexpr int trc_epb() { return N1 <= 4 ? (N1 <= 2 ? 16 : (N1 == 3 ? 8 : 4)) : 1; }

template <int N1>
size_t fct_smem() {
  constexpr int EPB = trc_epb<N1>(), Np = N1 * N1 * N1, NF = N1 * N1;
  return sizeof(double) * EPB * (6 * NF + 8 + Np);
}
template <int N1>
size_t stage_smem() {
  constexpr int EPB = trc_epb<N1>(), Np = N1 * N1 * N1, NF = N1 * N1;
  return sizeof(double) * EPB * (3 * Np + 5 * 6 * NF + 8 + 2 * Np);
}

template <int N1>
int launch_fct_n(const Ops& op, const double* dp, const TrcIn& in, const TrcFct& fc, int Ne, cudaStream_t s) {
  constexpr int EPB = trc_epb<N1>(), Np = N1 * N1 * N1;
  const size_t sm = fct_smem<N1>();
  auto kfn = k_trc_fct<N1, EPB>;
  cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  kfn<<<(Ne + EPB - 1) / EPB, EPB * Np, sm, s>>>(op, dp, in, fc, Ne);
  return (int)cudaGetLastError();
}
template <int N1>
int launch_stage_n(const Ops& op, const double* dp, const TrcIn& in, const TrcStage& st, const TrcFilt& tf, int Ne,
                   cudaStream_t s) {
  constexpr int EPB = trc_epb<N1>(), Np = N1 * N1 * N1;
  const size_t sm = stage_smem<N1>();
  auto kfn = k_trc_stage<N1, EPB>;
  cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  kfn<<<(Ne + EPB - 1) / EPB, EPB * Np, sm, s>>>(op, dp, in, st, tf, Ne);
  return (int)cudaGetLastError();
}
template <int N1>
int launch_post_n(const Ops& op, const double* dp, double* Q, const double* dd, const TrcFilt& tf, int filter, int tmar,
                  int Ne, cudaStream_t s) {
  constexpr int EPB = trc_epb<N1>(), Np = N1 * N1 * N1;
  const size_t sm = sizeof(double) * EPB * 3 * Np;
  k_trc_post<N1, EPB><<<(Ne + EPB - 1) / EPB, EPB * Np, sm, s>>>(op, dp, Q, dd, tf, filter, tmar, Ne);
  return (int)cudaGetLastError();
}
template <int N1>
int launch_alph_adv_n(const Ops& op, const double* dp, const double* dd, const double* mx, const double* my,
                      const double* mz, double* aM, double* aP, int Ne, cudaStream_t s) {
  const size_t nt = (size_t)Ne * 6 * N1 * N1;
  k_trc_alph_adv<N1><<<(unsigned)((nt + 255) / 256), 256, 0, s>>>(op, dp, dd, mx, my, mz, aM, aP, Ne);
  return (int)cudaGetLastError();
}
template <int N1, class S>
int launch_alph_dyn_n(const Ops& op, const Prof& pf, const MflxArgs<S>& A, int Ne, cudaStream_t s) {
  const size_t nt = (size_t)Ne * 6 * N1 * N1;
  k_trc_alph_dyn<N1, S><<<(unsigned)((nt + 255) / 256), 256, 0, s>>>(op, pf, A, Ne);
  return (int)cudaGetLastError();
}

#define FEDG_TRC_DISPATCH(N1, CALL)                        \
  switch (N1) {                                            \
    case 2: { constexpr int NN = 2; return CALL; }         \
    case 3: { constexpr int NN = 3; return CALL; }         \
    case 4: { constexpr int NN = 4; return CALL; }         \
    case 5: { constexpr int NN = 5; return CALL; }         \
    case 6: { constexpr int NN = 6; return CALL; }         \
    case 7: { constexpr int NN = 7; return CALL; }         \
    case 8: { constexpr int NN = 8; return CALL; }         \
  }                                                        \
  return (int)cudaErrorInvalidValue;

int launch_fct(const Ops& op, const double* dp, const TrcIn& in, const TrcFct& fc, int Ne, cudaStream_t s) {
  FEDG_TRC_DISPATCH(op.N1, launch_fct_n<NN>(op, dp, in, fc, Ne, s))
}
int launch_stage(const Ops& op, const double* dp, const TrcIn& in, const TrcStage& st, const TrcFilt& tf, int Ne,
                 cudaStream_t s) {
  FEDG_TRC_DISPATCH(op.N1, launch_stage_n<NN>(op, dp, in, st, tf, Ne, s))
}
int launch_post(const Ops& op, const double* dp, double* Q, const double* dd, const TrcFilt& tf, int filter, int tmar,
                int Ne, cudaStream_t s) {
  FEDG_TRC_DISPATCH(op.N1, launch_post_n<NN>(op, dp, Q, dd, tf, filter, tmar, Ne, s))
}
int launch_alph_adv(const Ops& op, const double* dp, const double* dd, const double* mx, const double* my,
                    const double* mz, double* aM, double* aP, int Ne, cudaStream_t s) {
  FEDG_TRC_DISPATCH(op.N1, launch_alph_adv_n<NN>(op, dp, dd, mx, my, mz, aM, aP, Ne, s))
}
template <class S>
int launch_alph_dyn(const Ops& op, const Prof& pf, const MflxArgs<S>& A, int Ne, cudaStream_t s) {
  FEDG_TRC_DISPATCH(op.N1, (launch_alph_dyn_n<NN, S>(op, pf, A, Ne, s)))
}

// both save_massflux kernels of one stage
template <class S>
int save_massflux_launch(fedg_ctx* c, const MflxArgs<S>& A) {
  int r = tracked(c, FEDG_K_TRC_AUX, [&] {
    k_trc_mflx<S><<<(unsigned)((c->n + 255) / 256), 256, 0, c->stream>>>(A, c->Np, c->N1, c->nxy, c->n);
    return (int)cudaGetLastError();
  });
  if (!r) r = tracked(c, FEDG_K_TRC_AUX, [&] { return launch_alph_dyn(c->op, c->prof(), A, c->Ne, c->stream); });
  return r;
}

TrcFilt make_filter(const fedg_ctx* c, double etac_h, double alpha_h, int ord_h, double etac_v, double alpha_v,
                    int ord_v) {
  TrcFilt tf;
  std::memset(&tf, 0, sizeof(tf));
  modal_filter_1d(c->N1 - 1, etac_h, alpha_h, ord_h, tf.Fh);
  modal_filter_1d(c->N1 - 1, etac_v, alpha_v, ord_v, tf.Fv);
  return tf;
}

int check_base(const fedg_ctx* c, const char* who) {
  if (!c->base_set) return api_fail(std::string(who) + ": the base state is not registered (fedg_set_base_state)");
  return 0;
}

// the tracer kernels read lateral neighbours of a periodic mesh only (no slab halo)
int check_periodic(const fedg_ctx* c, const char* who) {
  if (fedg::slab(c)) return api_fail(std::string(who) + ": not available on a part of a decomposed mesh (periodic_x/y = FEDG_HALO)");
  return 0;
}

}  // namespace

// save_massflux of a stage that the FP32 or float-pair update holds as deviations (qp: pairs, or
// qf: FP32), into the tracer-flux outputs registered with fedg_update_set_tracer_flux
int save_massflux_dev(fedg_ctx* c, int rkstage, const float2* const qp[5], const float* const qf[5], double U,
                      double V, double w_h, double w_v, int is_hevi) {
  double* const* tf = c->trc_flux;
  auto fill = [&](auto& A) {
    A.dpres = nullptr;
    for (int d = 0; d < 3; ++d) A.mf[d] = tf[d];
    A.aM = tf[3];
    A.aP = tf[4];
    A.w_h = w_h;
    A.w_v = w_v;
    A.first = rkstage == 1;
    A.hevi = is_hevi != 0;
  };
  if (qp) {
    MflxArgs<StPair> A;
    for (int v = 0; v < 5; ++v) A.q.q[v] = qp[v];
    A.q.dens = c->d_prof;
    A.q.U = U;
    A.q.V = V;
    fill(A);
    return save_massflux_launch(c, A);
  }
  MflxArgs<StF32> A;
  for (int v = 0; v < 5; ++v) A.q.q[v] = qf[v];
  A.q.dens = c->d_prof;
  A.q.U = U;
  A.q.V = V;
  fill(A);
  return save_massflux_launch(c, A);
}
}  // namespace fedg

// ---------------------------------------------------------------------------------------
// entry points (include/fedg.h)
// ---------------------------------------------------------------------------------------
extern "C" {

int fedg_trc_alphdens_advtest(fedg_ctx* c, const double* DDENS, const double* MOMX, const double* MOMY,
                              const double* MOMZ, double* alph_M, double* alph_P) {
  if (!c || !DDENS || !MOMX || !MOMY || !MOMZ || !alph_M || !alph_P)
    return api_fail("fedg_trc_alphdens_advtest: null argument");
  if (int r = check_base(c, "fedg_trc_alphdens_advtest")) return r;
  if (int r = check_periodic(c, "fedg_trc_alphdens_advtest")) return r;
  cudaSetDevice(c->d.device);
  const int r = tracked(c, FEDG_K_TRC_AUX, [&] {
    return launch_alph_adv(c->op, c->d_prof, DDENS, MOMX, MOMY, MOMZ, alph_M, alph_P, c->Ne, c->stream);
  });
  return r ? api_cuda_fail((cudaError_t)r, "fedg_trc_alphdens_advtest") : 0;
}

int fedg_trc_save_massflux(fedg_ctx* c, int rkstage, const double* const q[5], const double* DPRES, double w_h,
                           double w_v, int is_hevi, double* const mflx[3], double* alph_M, double* alph_P) {
  if (!c || !q || !mflx || !alph_M || !alph_P) return api_fail("fedg_trc_save_massflux: null argument");
  for (int v = 0; v < 5; ++v)
    if (!q[v]) return api_fail("fedg_trc_save_massflux: null state field");
  for (int d = 0; d < 3; ++d)
    if (!mflx[d]) return api_fail("fedg_trc_save_massflux: null mass-flux field");
  if (rkstage < 1) return api_fail("fedg_trc_save_massflux: rkstage is 1-based");
  if (int r = check_base(c, "fedg_trc_save_massflux")) return r;
  if (int r = check_periodic(c, "fedg_trc_save_massflux")) return r;
  cudaSetDevice(c->d.device);
  MflxArgs<StF64> A;
  for (int v = 0; v < 5; ++v) A.q.q[v] = q[v];
  A.dpres = DPRES;
  for (int d = 0; d < 3; ++d) A.mf[d] = mflx[d];
  A.aM = alph_M;
  A.aP = alph_P;
  A.w_h = w_h;
  A.w_v = w_v;
  A.first = rkstage == 1;
  A.hevi = is_hevi != 0;
  const int r = save_massflux_launch(c, A);
  return r ? api_cuda_fail((cudaError_t)r, "fedg_trc_save_massflux") : 0;
}

int fedg_trc_fct_coef(fedg_ctx* c, const double* QTRC, const double* const mflx[3], const double* RHOQ_tp,
                      const double* alph_M, const double* alph_P, const double* DDENS_TRC, const double* DDENS0_TRC,
                      double rk_c_ssm1, double dt, double* fct_coef) {
  if (!c || !QTRC || !mflx || !mflx[0] || !mflx[1] || !mflx[2] || !alph_M || !alph_P || !DDENS_TRC || !DDENS0_TRC ||
      !fct_coef)
    return api_fail("fedg_trc_fct_coef: null argument");
  if (!(dt > 0.0)) return api_fail("fedg_trc_fct_coef: dt must be positive");
  if (int r = check_base(c, "fedg_trc_fct_coef")) return r;
  if (int r = check_periodic(c, "fedg_trc_fct_coef")) return r;
  cudaSetDevice(c->d.device);
  const TrcIn in{QTRC, {mflx[0], mflx[1], mflx[2]}, alph_M, alph_P, RHOQ_tp, DDENS_TRC, DDENS0_TRC};
  const TrcFct fc{rk_c_ssm1, dt, nullptr, fct_coef};
  const int r = tracked(c, FEDG_K_TRC_FCT, [&] { return launch_fct(c->op, c->d_prof, in, fc, c->Ne, c->stream); });
  return r ? api_cuda_fail((cudaError_t)r, "fedg_trc_fct_coef") : 0;
}

int fedg_trc_cal_tend(fedg_ctx* c, const double* QTRC, const double* const mflx[3], const double* alph_M,
                      const double* alph_P, const double* fct_coef, const double* RHOQ_tp, double* QTRC_dt) {
  if (!c || !QTRC || !mflx || !mflx[0] || !mflx[1] || !mflx[2] || !alph_M || !alph_P || !QTRC_dt)
    return api_fail("fedg_trc_cal_tend: null argument");
  if (int r = check_periodic(c, "fedg_trc_cal_tend")) return r;
  cudaSetDevice(c->d.device);
  const TrcIn in{QTRC, {mflx[0], mflx[1], mflx[2]}, alph_M, alph_P, RHOQ_tp, nullptr, nullptr};
  TrcStage st;
  std::memset(&st, 0, sizeof(st));
  st.fct_node = fct_coef;
  st.tend = QTRC_dt;
  TrcFilt tf;
  std::memset(&tf, 0, sizeof(tf));
  const int r = tracked(c, FEDG_K_TRC_TEND, [&] { return launch_stage(c->op, c->d_prof, in, st, tf, c->Ne, c->stream); });
  return r ? api_cuda_fail((cudaError_t)r, "fedg_trc_cal_tend") : 0;
}

int fedg_trc_tmar(fedg_ctx* c, double* QTRC, const double* DDENS) {
  if (!c || !QTRC || !DDENS) return api_fail("fedg_trc_tmar: null argument");
  if (int r = check_base(c, "fedg_trc_tmar")) return r;
  cudaSetDevice(c->d.device);
  TrcFilt tf;
  std::memset(&tf, 0, sizeof(tf));
  const int r = tracked(c, FEDG_K_TRC_AUX, [&] { return launch_post(c->op, c->d_prof, QTRC, DDENS, tf, 0, 1, c->Ne, c->stream); });
  return r ? api_cuda_fail((cudaError_t)r, "fedg_trc_tmar") : 0;
}

int fedg_trc_modalfilter(fedg_ctx* c, double* QTRC, const double* DDENS, double etac_h, double alpha_h, int order_h,
                         double etac_v, double alpha_v, int order_v) {
  if (!c || !QTRC || !DDENS) return api_fail("fedg_trc_modalfilter: null argument");
  if (int r = check_base(c, "fedg_trc_modalfilter")) return r;
  cudaSetDevice(c->d.device);
  const TrcFilt tf = make_filter(c, etac_h, alpha_h, order_h, etac_v, alpha_v, order_v);
  const int r = tracked(c, FEDG_K_TRC_AUX, [&] { return launch_post(c->op, c->d_prof, QTRC, DDENS, tf, 1, 0, c->Ne, c->stream); });
  return r ? api_cuda_fail((cudaError_t)r, "fedg_trc_modalfilter") : 0;
}

int fedg_trc_update(fedg_ctx* c, double* QTRC, const double* const mflx[3], const double* alph_M,
                    const double* alph_P, const double* DDENS_TRC, const double* DDENS0_TRC, const double* DDENS,
                    const double* RHOQ_tp, const fedg_trc_opts* o) {
  if (!c || !QTRC || !mflx || !mflx[0] || !mflx[1] || !mflx[2] || !alph_M || !alph_P || !DDENS_TRC || !DDENS0_TRC || !o)
    return api_fail("fedg_trc_update: null argument");
  if (o->scheme != FEDG_SSP_RK3) return api_fail("fedg_trc_update: the tracer scheme must be FEDG_SSP_RK3 (ERK_SSP_3s3o)");
  if (o->prec != FEDG_PREC_FP64 && o->prec != FEDG_PREC_PAIR)
    return api_fail("fedg_trc_update: prec must be FEDG_PREC_FP64 or FEDG_PREC_PAIR");
  if (!(o->dt > 0.0) || o->nsteps < 0) return api_fail("fedg_trc_update: dt must be positive and nsteps >= 0");
  if (int r = check_base(c, "fedg_trc_update")) return r;
  if (int r = check_periodic(c, "fedg_trc_update")) return r;
  cudaSetDevice(c->d.device);
  // ERK_SSP_3s3o in Shu-Osher form (scale_timeint_rk_butcher_tab.F90:200-210) and its stage nodes
  constexpr int ns = 3;
  const double sig[4][3] = {{0, 0, 0}, {1, 0, 0}, {0.75, 0.25, 0}, {1.0 / 3.0, 0, 2.0 / 3.0}};
  const double gam[4][3] = {{0, 0, 0}, {1, 0, 0}, {0, 0.25, 0}, {0, 0, 2.0 / 3.0}};
  const double cn[3] = {0.0, 1.0, 0.5};
  const size_t n = c->n;
  if (!c->trc_buf) {
    if (cudaMalloc(&c->trc_buf, sizeof(double) * (4 * n + (size_t)c->Ne)) != cudaSuccess) {
      c->trc_buf = nullptr;
      return api_fail("fedg_trc_update: out of device memory (4 tracer fields of scratch)");
    }
  }
  if (o->prec == FEDG_PREC_PAIR)
    return trc_update_pair(c, QTRC, mflx, alph_M, alph_P, DDENS_TRC, DDENS0_TRC, DDENS, RHOQ_tp, o, c->trc_buf);
  double* bufA = c->trc_buf;
  double* bufB = bufA + n;
  double* var0 = bufB + n;
  double* vtmp = var0 + n;
  double* fct = vtmp + n;
  const TrcFilt tf = o->filter ? make_filter(c, o->mf_etac_h, o->mf_alpha_h, o->mf_order_h, o->mf_etac_v,
                                             o->mf_alpha_v, o->mf_order_v)
                               : TrcFilt{};
  for (int step = 0; step < o->nsteps; ++step) {
    const double* qs = QTRC;
    for (int s = 1; s <= ns; ++s) {
      double* qo = (s == ns) ? QTRC : ((s & 1) ? bufA : bufB);
      const TrcIn in{qs, {mflx[0], mflx[1], mflx[2]}, alph_M, alph_P, RHOQ_tp, DDENS_TRC, DDENS0_TRC};
      const double sig_ss = sig[s][s - 1], gam_ss = gam[s][s - 1];
      if (o->limiter) {
        const TrcFct fc{cn[s - 1], o->dt * gam_ss / sig_ss, fct, nullptr};
        const int r = tracked(c, FEDG_K_TRC_FCT, [&] { return launch_fct(c->op, c->d_prof, in, fc, c->Ne, c->stream); });
        if (r) return api_cuda_fail((cudaError_t)r, "fedg_trc_update: FCT coefficient");
      }
      TrcStage st;
      std::memset(&st, 0, sizeof(st));
      st.fct_elem = o->limiter ? fct : nullptr;
      st.advance = 1;
      st.first = s == 1;
      st.last = s == ns;
      const double sig_Ns = sig[ns][s - 1], gam_Ns = o->dt * gam[ns][s - 1];
      st.acc = !st.last && (std::fabs(sig_Ns) > 1.0e-16 || std::fabs(gam_Ns) > 1.0e-16);
      st.sig_ss = sig_ss;
      st.gam_ss = o->dt * gam_ss;
      st.sig_Ns = sig_Ns;
      st.gam_Ns = gam_Ns;
      st.c_ssm1 = cn[s - 1];
      st.c_ss = s < ns ? cn[s] : 0.0;
      st.q_out = qo;
      st.var0 = var0;
      st.vtmp = vtmp;
      st.filter = o->filter != 0;
      st.tmar = o->limiter && o->tmar;
      st.ddens_fin = DDENS;
      st.qtrc_out = QTRC;
      const int r = tracked(c, FEDG_K_TRC_TEND, [&] { return launch_stage(c->op, c->d_prof, in, st, tf, c->Ne, c->stream); });
      if (r) return api_cuda_fail((cudaError_t)r, "fedg_trc_update: stage");
      qs = qo;
    }
  }
  return 0;
}

}  // extern "C"
