// fedg_trc_pair.cu -- the tracer step of fedg_trc_update in float pairs (FEDG_PREC_PAIR).
//
// Same algorithm, fusion and launch structure as the FP64 kernels of fedg_trc.cu (FElib's
// trcadvect3d_heve.F90 FCT coefficient :234-306, cal_tend :149-231, TMAR :311-340, the tracer filter
// ..._dgm_modalfilter.F90:232-270 and rk_advance_trcvar_low_storage2D, scale_timeint_rk.F90:1390-1498),
// with every value carried as an unevaluated float pair (hi + lo, about 48 bits; fedg_f2.cuh):
//   - FP64 inputs are split with integer instructions on load; the stage fields, var0 and varTmp
//     stay pairs between launches; the final QTRC is converted back to FP64;
//   - the face and element integrals are pair sums, the D_x/D_y/D_z contractions and the Lift are
//     compensated sums of exact products, divisions are pair reciprocals.
// Why: the FP64 kernels keep GB300's FP64 pipe ~86 % busy at ~80 FP64 instructions per node and
// launch; the FP32 pipe has 64x its issue rate.  The pair path is FP64-class (relative rounding
// ~1e-14), not bit-identical: the reciprocal replaces FP64 division, and the FCT face selection
// 0.5 (R+ + R- - (R+ - R-) sign) is taken exactly as R- or R+.
#include <cmath>
#include <cstring>
#include <vector>

#include "fedg_ctx.cuh"
#include "fedg_f2.cuh"

namespace fedg {
namespace {

__device__ __forceinline__ f2 operator+(f2 a, f2 b) { return f2_add(a, b); }
__device__ __forceinline__ f2 operator-(f2 a, f2 b) { return f2_sub(a, b); }
__device__ __forceinline__ f2 operator*(f2 a, f2 b) { return f2_mul(a, b); }
__device__ __forceinline__ f2 operator-(f2 a) { return f2_neg(a); }
__device__ __forceinline__ f2 zero2() { return f2{0.f, 0.f}; }

__device__ __forceinline__ f2 ld64(const double* p, size_t g) { return f2_split(__ldg(p + g)); }
__device__ __forceinline__ f2 ldp(const float2* p, size_t g) { return f2_of(__ldg(p + g)); }
__device__ __forceinline__ f2 pos_part(f2 x) { return x.h > 0.f ? x : zero2(); }
__device__ __forceinline__ f2 clamp01(f2 x) {
  if (!(x.h > 0.f)) return zero2();
  if (x.h > 1.f || (x.h == 1.f && x.l > 0.f)) return f2{1.f, 0.f};
  return x;
}

struct TrcOpsP {
  float2 D[FEDG_MAXN1 * FEDG_MAXN1];
  float2 Fh[FEDG_MAXN1 * FEDG_MAXN1], Fv[FEDG_MAXN1 * FEDG_MAXN1];
  float2 Lb[FEDG_MAXN1], Lt[FEDG_MAXN1], w[FEDG_MAXN1];
  float2 E11, E22, E33, FSx, FSy, FSz, J, JFx, JFy, JFz;
  int NeX, NeY, NeZ;
};

struct InP {
  const double* Q64;   // stage input as FP64 (first stage: QTRC) ...
  const float2* Qp;    // ... or as pairs (later stages)
  const double* mf[3];
  const double* aM;
  const double* aP;
  const double* rhoq;
  const double* ddens;
  const double* ddens0;
};

struct StageP {
  float2 c_ssm1, c_ss, sig_ss, one_m_sig, gam_ss, sig_Ns, gam_Ns, rdt_fct;
  int first, last, acc, limiter, filter, tmar;
  const float2* fct;   // per element (limiter)
  float2* fct_out;     // FCT kernel output
  float2* q_out;
  float2* var0;
  float2* vtmp;
  const double* ddens_fin;
  double* qtrc_out;
};

template <int N1>
__device__ __forceinline__ f2 q_at(const InP& in, size_t g) {
  return in.Qp ? ldp(in.Qp, g) : ld64(in.Q64, g);
}

__device__ __forceinline__ f2 normal_comp_p(int f, const InP& in, size_t g, bool flip_z) {
  switch (f) {
    case 0: return -ld64(in.mf[1], g);
    case 1: return ld64(in.mf[0], g);
    case 2: return ld64(in.mf[1], g);
    case 3: return -ld64(in.mf[0], g);
    case 4: return flip_z ? ld64(in.mf[2], g) : -ld64(in.mf[2], g);
    default: return flip_z ? -ld64(in.mf[2], g) : ld64(in.mf[2], g);
  }
}

__device__ __forceinline__ f2 shfl_xor(f2 v, int o) {
  return f2{__shfl_xor_sync(0xffffffffu, v.h, o), __shfl_xor_sync(0xffffffffu, v.l, o)};
}

// sum over the Np threads of element le, in a fixed order, every thread gets the result
template <int N1, int EPB>
__device__ __forceinline__ f2 elem_sum_p(f2 v, float2* s_red, int le, int p) {
  constexpr int Np = N1 * N1 * N1;
  __syncthreads();
  if constexpr (Np % 32 == 0) {
    constexpr int NW = Np / 32;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = v + shfl_xor(v, o);
    if ((p & 31) == 0) s_red[le * NW + (p >> 5)] = f2_pack(v);
    __syncthreads();
    if (p == 0) {
      f2 s = zero2();
      for (int w = 0; w < NW; ++w) s = s + f2_of(s_red[le * NW + w]);
      s_red[EPB * Np + le] = f2_pack(s);
    }
    __syncthreads();
    return f2_of(s_red[EPB * Np + le]);
  } else {
    s_red[le * Np + p] = f2_pack(v);
    __syncthreads();
    if (p == 0) {
      f2 s = zero2();
      for (int q = 0; q < Np; ++q) s = s + f2_of(s_red[le * Np + q]);
      s_red[EPB * Np + le] = f2_pack(s);
    }
    __syncthreads();
    return f2_of(s_red[EPB * Np + le]);
  }
}

// per-face sums of the weighted integrands sf[6][NF] of element le into s_out[le][0..5]: one warp
// per face when the element has at least 6 warps, else one thread per face (the caller synchronises)
template <int N1>
__device__ __forceinline__ void face_sums_p(const float2* sf, float2* s_out, int le, int p, bool valid) {
  constexpr int Np = N1 * N1 * N1, NF = N1 * N1;
  if constexpr (Np >= 6 * 32) {
    const int f = p >> 5, lane = p & 31;
    if (f < 6) {
      f2 s = zero2();
      for (int q = lane; q < NF; q += 32) s = s + f2_of(sf[f * NF + q]);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s = s + shfl_xor(s, o);
      if (valid && lane == 0) s_out[le * 8 + f] = f2_pack(s);
    }
  } else {
    if (valid && p < 6) {
      f2 s = zero2();
      for (int q = 0; q < NF; ++q) s = s + f2_of(sf[p * NF + q]);
      s_out[le * 8 + p] = f2_pack(s);
    }
  }
}

template <int N1>
__device__ __forceinline__ void face_nodes_p(const TrcOpsP& op, int f, int a, int b, long ke, int ex, int ey, int ez,
                                             int nxy, int& pM, size_t& gP, long& kn) {
  constexpr int Np = N1 * N1 * N1, NF = N1 * N1;
  int iM, jM, kM;
  face_node<N1>(f, a, b, iM, jM, kM);
  pM = iM + N1 * jM + NF * kM;
  switch (f) {
    case 0: kn = ke + (ey > 0 ? -op.NeX : (long)(op.NeY - 1) * op.NeX); break;
    case 1: kn = ke + (ex < op.NeX - 1 ? 1 : -(op.NeX - 1)); break;
    case 2: kn = ke + (ey < op.NeY - 1 ? op.NeX : -(long)(op.NeY - 1) * op.NeX); break;
    case 3: kn = ke + (ex > 0 ? -1 : op.NeX - 1); break;
    case 4: kn = ez > 0 ? ke - nxy : -1; break;
    default: kn = ez < op.NeZ - 1 ? ke + nxy : -1; break;
  }
  if (kn >= 0) {
    int i2, j2, k2;
    face_node<N1>(face_opp(f), a, b, i2, j2, k2);
    gP = (size_t)kn * Np + i2 + N1 * j2 + NF * k2;
  } else {
    gP = (size_t)ke * Np + pM;
  }
}

// Rusanov flux of face node fi of element ke; returns numflux, sets q- m- and the weighted
// integrand (w_a w_b J Fscale numflux) of the face integral
template <int N1>
__device__ __forceinline__ f2 face_flux_p(const TrcOpsP& op, const InP& in, long ke, int ex, int ey, int ez, int nxy,
                                          int fi, f2& qm, f2& wint, long& kn) {
  constexpr int Np = N1 * N1 * N1, NF = N1 * N1;
  const int f = fi / NF, ab = fi - f * NF, a = ab % N1, b = ab / N1;
  int pM;
  size_t gP;
  face_nodes_p<N1>(op, f, a, b, ke, ex, ey, ez, nxy, pM, gP, kn);
  const size_t gM = (size_t)ke * Np + pM;
  const f2 mfM = normal_comp_p(f, in, gM, false);
  const f2 mfP = normal_comp_p(f, in, gP, kn < 0);
  const f2 qM = q_at<N1>(in, gM), qP = q_at<N1>(in, gP);
  const size_t fa = (size_t)ke * 6 * NF + fi;
  const f2 nf = f2_mul_f((qP * mfP + qM * mfM) - ld64(in.aP, fa) * qP + ld64(in.aM, fa) * qM, 0.5f);
  qm = qM * mfM;
  const f2 JF = f2_of(f >= 4 ? op.JFz : ((f & 1) ? op.JFx : op.JFy));
  wint = (f2_of(op.w[a]) * f2_of(op.w[b])) * (JF * nf);
  return nf;
}

template <int N1, int EPB>
__global__ void __launch_bounds__(EPB* N1* N1* N1)
    k_trc_fct_p(const TrcOpsP op, const double* __restrict__ dens_prof, const InP in, const StageP st, int Ne) {
  constexpr int Np = N1 * N1 * N1, NF = N1 * N1;
  extern __shared__ float2 smp[];
  float2* s_face = smp;                    // [EPB][6NF]
  float2* s_out = s_face + EPB * 6 * NF;   // [EPB][8]
  float2* s_red = s_out + EPB * 8;         // [EPB][Np] + [EPB]
  const int tid = threadIdx.x, le = tid / Np, p = tid - le * Np;
  const long ke = (long)blockIdx.x * EPB + le;
  const bool valid = ke < Ne;
  const int nxy = op.NeX * op.NeY;
  const int ez = valid ? (int)(ke / nxy) : 0;
  const int ey = valid ? (int)((ke - (long)ez * nxy) / op.NeX) : 0;
  const int ex = valid ? (int)(ke - (long)ez * nxy - (long)ey * op.NeX) : 0;
  float2* sf = s_face + le * 6 * NF;
  if (valid) {
    for (int fi = p; fi < 6 * NF; fi += Np) {
      f2 qm, wint;
      long kn;
      face_flux_p<N1>(op, in, ke, ex, ey, ez, nxy, fi, qm, wint, kn);
      sf[fi] = f2_pack(wint);
    }
  }
  f2 v = zero2();
  if (valid) {
    const size_t g = (size_t)ke * Np + p;
    const int i = p % N1, j = (p / N1) % N1, k = p / NF;
    const f2 dens = f2_split(__ldg(dens_prof + ez * N1 + k)) + (f2{1.f, 0.f} - f2_of(st.c_ssm1)) * ld64(in.ddens0, g) +
                    f2_of(st.c_ssm1) * ld64(in.ddens, g);
    f2 m = dens * q_at<N1>(in, g) * f2_of(st.rdt_fct);
    if (in.rhoq) m = m + ld64(in.rhoq, g);
    v = f2_of(op.J) * ((f2_of(op.w[i]) * f2_of(op.w[j])) * f2_of(op.w[k])) * m;
  }
  const f2 qe = elem_sum_p<N1, EPB>(v, s_red, le, p);
  face_sums_p<N1>(sf, s_out, le, p, valid);
  __syncthreads();
  if (valid && p == 0) {
    f2 net = zero2();
#pragma unroll
    for (int f = 0; f < 6; ++f) net = net + pos_part(f2_of(s_out[le * 8 + f]));
    net = f2_add_f(net, 1.0e-10f);
    st.fct_out[ke] = f2_pack(clamp01(qe * f2_recip(net)));
  }
}

template <int N1, int EPB>
__global__ void __launch_bounds__(EPB* N1* N1* N1, (N1 == 8 ? 3 : 1))
    k_trc_stage_p(const TrcOpsP op, const double* __restrict__ dens_prof, const InP in, const StageP st, int Ne) {
  constexpr int Np = N1 * N1 * N1, NF = N1 * N1;
  extern __shared__ float2 smp[];
  float2* s_fl = smp;                       // [EPB][3][Np]
  float2* s_nf = s_fl + EPB * 3 * Np;       // [EPB][6NF]
  float2* s_qm = s_nf + EPB * 6 * NF;       // [EPB][6NF]
  float2* s_rr = s_qm + EPB * 6 * NF;       // [EPB][6NF] FCT coefficient of the exterior side
  float2* s_face = s_rr + EPB * 6 * NF;     // [EPB][6NF]
  float2* s_out = s_face + EPB * 6 * NF;    // [EPB][8]
  float2* s_red = s_out + EPB * 8;          // [EPB][Np] + [EPB]
  float2* s_b = s_red + EPB * (Np + 1);     // [EPB][Np]
  const int tid = threadIdx.x, le = tid / Np, p = tid - le * Np;
  const long ke = (long)blockIdx.x * EPB + le;
  const bool valid = ke < Ne;
  const int i = p % N1, j = (p / N1) % N1, k = p / NF;
  const int nxy = op.NeX * op.NeY;
  const int ez = valid ? (int)(ke / nxy) : 0;
  const int ey = valid ? (int)((ke - (long)ez * nxy) / op.NeX) : 0;
  const int ex = valid ? (int)(ke - (long)ez * nxy - (long)ey * op.NeX) : 0;
  const size_t g = (size_t)ke * Np + p;
  float2* fl = s_fl + le * 3 * Np;
  float2* nfv = s_nf + le * 6 * NF;
  float2* qmv = s_qm + le * 6 * NF;
  float2* rpv = s_rr + le * 6 * NF;
  float2* sf = s_face + le * 6 * NF;

  const f2 q = valid ? q_at<N1>(in, g) : zero2();
  fl[p] = f2_pack(valid ? ld64(in.mf[0], g) * q : zero2());
  fl[Np + p] = f2_pack(valid ? ld64(in.mf[1], g) * q : zero2());
  fl[2 * Np + p] = f2_pack(valid ? ld64(in.mf[2], g) * q : zero2());
  const f2 one{1.f, 0.f};
  const f2 own = (valid && st.limiter) ? ldp(st.fct, ke) : one;
  if (valid) {
    for (int fi = p; fi < 6 * NF; fi += Np) {
      f2 qm, wint;
      long kn;
      const f2 nf = face_flux_p<N1>(op, in, ke, ex, ey, ez, nxy, fi, qm, wint, kn);
      nfv[fi] = f2_pack(nf);
      qmv[fi] = f2_pack(qm);
      rpv[fi] = f2_pack(st.limiter ? (kn >= 0 ? ldp(st.fct, kn) : own) : one);
      sf[fi] = f2_pack(wint);
    }
  }
  __syncthreads();
  face_sums_p<N1>(sf, s_out, le, p, valid);
  __syncthreads();
  if (valid) {  // del_flux = Fscale (numflux R - q- m-), R = R- on outflow faces, R+ on inflow faces
    for (int fi = p; fi < 6 * NF; fi += Np) {
      const int f = fi / NF;
      const f2 R = signbit(s_out[le * 8 + f].x) ? f2_of(rpv[fi]) : own;
      const f2 fs = f2_of(f >= 4 ? op.FSz : ((f & 1) ? op.FSx : op.FSy));
      sf[fi] = f2_pack(fs * (f2_of(nfv[fi]) * R - f2_of(qmv[fi])));
    }
  }
  __syncthreads();

  f2 t = zero2();
  if (valid) {
    f2acc sx, sy, sz, lf;
#pragma unroll
    for (int l = 0; l < N1; ++l) {
      sx.add(f2_of(op.D[i * N1 + l]), f2_of(fl[l + N1 * j + NF * k]));
      sy.add(f2_of(op.D[j * N1 + l]), f2_of(fl[Np + i + N1 * l + NF * k]));
      sz.add(f2_of(op.D[k * N1 + l]), f2_of(fl[2 * Np + i + N1 * j + NF * l]));
    }
    lf.add(f2_of(op.Lb[j]), f2_of(sf[0 * NF + i + N1 * k]));
    lf.add(f2_of(op.Lt[i]), f2_of(sf[1 * NF + j + N1 * k]));
    lf.add(f2_of(op.Lt[j]), f2_of(sf[2 * NF + i + N1 * k]));
    lf.add(f2_of(op.Lb[i]), f2_of(sf[3 * NF + j + N1 * k]));
    lf.add(f2_of(op.Lb[k]), f2_of(sf[4 * NF + i + N1 * j]));
    lf.add(f2_of(op.Lt[k]), f2_of(sf[5 * NF + i + N1 * j]));
    t = -(f2_of(op.E11) * sx.get() + f2_of(op.E22) * sy.get() + f2_of(op.E33) * sz.get() + lf.get());
    if (in.rhoq) t = t + ld64(in.rhoq, g);
  }

  // rk_advance_trcvar_low_storage in pairs
  f2 qn = zero2(), wgt = one;
  if (valid) {
    const f2 dh = f2_split(__ldg(dens_prof + ez * N1 + k));
    const f2 dd = ld64(in.ddens, g), dd0 = ld64(in.ddens0, g);
    const f2 d0 = dh + dd0;
    const f2 dssm1 = d0 + f2_of(st.c_ssm1) * (dd - dd0);
    if (st.last) {
      qn = (ldp(st.vtmp, g) + f2_of(st.sig_ss) * q * dssm1 + f2_of(st.gam_ss) * t) * f2_recip(dh + dd);
    } else {
      f2 v0;
      if (st.first) {
        v0 = q * d0;
        st.var0[g] = f2_pack(v0);
      } else {
        v0 = ldp(st.var0, g);
      }
      if (st.acc) {
        const f2 vt = (st.first ? zero2() : ldp(st.vtmp, g)) + f2_of(st.sig_Ns) * q * dssm1 + f2_of(st.gam_Ns) * t;
        st.vtmp[g] = f2_pack(vt);
      } else if (st.first) {
        st.vtmp[g] = make_float2(0.f, 0.f);
      }
      const f2 dss = d0 + f2_of(st.c_ss) * (dd - dd0);
      qn = (f2_of(st.one_m_sig) * v0 + f2_of(st.sig_ss) * q * dssm1 + f2_of(st.gam_ss) * t) * f2_recip(dss);
      st.q_out[g] = f2_pack(qn);
    }
    wgt = dh + dd;
  }
  if (!st.last) return;  // uniform across the block

  // tracer filter of dens q, TMAR, rescale (FP64 output)
  if (st.filter) {
    float2* a = s_fl + le * 3 * Np;  // the flux arrays are free after the contractions above
    float2* b = s_b + le * Np;
    __syncthreads();
    b[p] = f2_pack(valid ? wgt * qn : zero2());
    __syncthreads();
    f2acc s1;
#pragma unroll
    for (int l = 0; l < N1; ++l) s1.add(f2_of(op.Fh[i * N1 + l]), f2_of(b[l + N1 * j + NF * k]));
    a[p] = f2_pack(s1.get());
    __syncthreads();
    f2acc s2;
#pragma unroll
    for (int l = 0; l < N1; ++l) s2.add(f2_of(op.Fh[j * N1 + l]), f2_of(a[i + N1 * l + NF * k]));
    __syncthreads();
    b[p] = f2_pack(s2.get());
    __syncthreads();
    f2acc s3;
#pragma unroll
    for (int l = 0; l < N1; ++l) s3.add(f2_of(op.Fv[k * N1 + l]), f2_of(b[i + N1 * j + NF * l]));
    if (valid) qn = s3.get() * f2_recip(wgt);
  }
  if (st.tmar) {
    const f2 wd = valid ? f2_of(op.J) * ((f2_of(op.w[i]) * f2_of(op.w[j])) * f2_of(op.w[k])) * wgt : zero2();
    const f2 qp = pos_part(qn);
    const f2 q0 = elem_sum_p<N1, EPB>(wd * qn, s_red, le, p);
    const f2 q1 = elem_sum_p<N1, EPB>(wd * qp, s_red, le, p);
    qn = q0 * f2_recip(f2_add_f(q1, 1.0e-32f)) * qp;
  }
  if (valid) {
    const f2 dh = f2_split(__ldg(dens_prof + ez * N1 + k));
    const f2 ddf = st.ddens_fin ? ld64(st.ddens_fin, g) : ld64(in.ddens, g);
    const f2 r = (dh + ld64(in.ddens, g)) * f2_recip(dh + ddf) * qn;
    st.qtrc_out[g] = (double)r.h + (double)r.l;
  }
}

float2 hsplit(double x) {
  const float h = (float)x;
  return make_float2(h, (float)(x - (double)h));
}

template <int N1>
constexpr int epb_p() { return N1 <= 4 ? (N1 <= 2 ? 16 : (N1 == 3 ? 8 : 4)) : 1; }

template <int N1>
int launch_pair_n(bool fct, const TrcOpsP& op, const double* dp, const InP& in, const StageP& st, int Ne,
                  cudaStream_t s) {
  constexpr int EPB = epb_p<N1>(), Np = N1 * N1 * N1, NF = N1 * N1;
  const int grid = (Ne + EPB - 1) / EPB;
  if (fct) {
    const size_t sm = sizeof(float2) * (EPB * (6 * NF + 8 + Np) + EPB);
    auto kf = k_trc_fct_p<N1, EPB>;
    cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    kf<<<grid, EPB * Np, sm, s>>>(op, dp, in, st, Ne);
  } else {
    const size_t sm = sizeof(float2) * (EPB * (3 * Np + 4 * 6 * NF + 8 + Np + 1 + Np));
    auto kf = k_trc_stage_p<N1, EPB>;
    cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    kf<<<grid, EPB * Np, sm, s>>>(op, dp, in, st, Ne);
  }
  return (int)cudaGetLastError();
}

int launch_pair(int N1, bool fct, const TrcOpsP& op, const double* dp, const InP& in, const StageP& st, int Ne,
                cudaStream_t s) {
  switch (N1) {
    case 2: return launch_pair_n<2>(fct, op, dp, in, st, Ne, s);
    case 3: return launch_pair_n<3>(fct, op, dp, in, st, Ne, s);
    case 4: return launch_pair_n<4>(fct, op, dp, in, st, Ne, s);
    case 5: return launch_pair_n<5>(fct, op, dp, in, st, Ne, s);
    case 6: return launch_pair_n<6>(fct, op, dp, in, st, Ne, s);
    case 7: return launch_pair_n<7>(fct, op, dp, in, st, Ne, s);
    case 8: return launch_pair_n<8>(fct, op, dp, in, st, Ne, s);
  }
  return (int)cudaErrorInvalidValue;
}

}  // namespace

// the fused tracer step in float pairs (fedg_trc_update with opts->prec == FEDG_PREC_PAIR); buffers
// are the FP64 path's scratch reinterpreted as pairs (same bytes)
int trc_update_pair(fedg_ctx* c, double* QTRC, const double* const mflx[3], const double* aM, const double* aP,
                    const double* ddens_trc, const double* ddens0_trc, const double* ddens, const double* rhoq,
                    const fedg_trc_opts* o, double* scratch) {
  const Ops& d = c->op;
  TrcOpsP op;
  std::memset(&op, 0, sizeof(op));
  const int N1 = c->N1;
  for (int a = 0; a < N1 * N1; ++a) op.D[a] = hsplit(d.D[a]);
  for (int a = 0; a < N1; ++a) {
    op.Lb[a] = hsplit(d.Lb[a]);
    op.Lt[a] = hsplit(d.Lt[a]);
    op.w[a] = hsplit(d.w[a]);
  }
  if (o->filter) {
    std::vector<double> Fh(N1 * N1), Fv(N1 * N1);
    modal_filter_1d(N1 - 1, o->mf_etac_h, o->mf_alpha_h, o->mf_order_h, Fh.data());
    modal_filter_1d(N1 - 1, o->mf_etac_v, o->mf_alpha_v, o->mf_order_v, Fv.data());
    for (int a = 0; a < N1 * N1; ++a) {
      op.Fh[a] = hsplit(Fh[a]);
      op.Fv[a] = hsplit(Fv[a]);
    }
  }
  op.E11 = hsplit(d.E11);
  op.E22 = hsplit(d.E22);
  op.E33 = hsplit(d.E33);
  op.FSx = hsplit(d.FSx);
  op.FSy = hsplit(d.FSy);
  op.FSz = hsplit(d.FSz);
  op.J = hsplit(d.Jac);
  op.JFx = hsplit(d.Jac * d.FSx);
  op.JFy = hsplit(d.Jac * d.FSy);
  op.JFz = hsplit(d.Jac * d.FSz);
  op.NeX = d.NeX;
  op.NeY = d.NeY;
  op.NeZ = d.NeZ;
  const size_t n = c->n;
  float2* bufA = reinterpret_cast<float2*>(scratch);
  float2* bufB = bufA + n;
  float2* var0 = bufB + n;
  float2* vtmp = var0 + n;
  float2* fct = vtmp + n;
  constexpr int ns = 3;  // ERK_SSP_3s3o (scale_timeint_rk_butcher_tab.F90:200-210)
  const double sig[4][3] = {{0, 0, 0}, {1, 0, 0}, {0.75, 0.25, 0}, {1.0 / 3.0, 0, 2.0 / 3.0}};
  const double gam[4][3] = {{0, 0, 0}, {1, 0, 0}, {0, 0.25, 0}, {0, 0, 2.0 / 3.0}};
  const double cn[3] = {0.0, 1.0, 0.5};
  for (int step = 0; step < o->nsteps; ++step) {
    const float2* qsp = nullptr;
    for (int s = 1; s <= ns; ++s) {
      InP in{s == 1 ? QTRC : nullptr, qsp, {mflx[0], mflx[1], mflx[2]}, aM, aP, rhoq, ddens_trc, ddens0_trc};
      StageP st;
      std::memset(&st, 0, sizeof(st));
      const double sig_ss = sig[s][s - 1], gam_ss = gam[s][s - 1];
      const double sig_Ns = sig[ns][s - 1], gam_Ns = o->dt * gam[ns][s - 1];
      st.c_ssm1 = hsplit(cn[s - 1]);
      st.c_ss = hsplit(s < ns ? cn[s] : 0.0);
      st.sig_ss = hsplit(sig_ss);
      st.one_m_sig = hsplit(1.0 - sig_ss);
      st.gam_ss = hsplit(o->dt * gam_ss);
      st.sig_Ns = hsplit(sig_Ns);
      st.gam_Ns = hsplit(gam_Ns);
      st.rdt_fct = hsplit(sig_ss / (o->dt * gam_ss));
      st.first = s == 1;
      st.last = s == ns;
      st.acc = !st.last && (std::fabs(sig_Ns) > 1.0e-16 || std::fabs(gam_Ns) > 1.0e-16);
      st.limiter = o->limiter != 0;
      st.filter = o->filter != 0;
      st.tmar = o->limiter && o->tmar;
      st.fct = fct;
      st.fct_out = fct;
      st.q_out = (s & 1) ? bufA : bufB;
      st.var0 = var0;
      st.vtmp = vtmp;
      st.ddens_fin = ddens;
      st.qtrc_out = QTRC;
      int r = 0;
      if (o->limiter)
        r = tracked(c, FEDG_K_TRC_FCT, [&] { return launch_pair(N1, true, op, c->d_prof, in, st, c->Ne, c->stream); });
      if (!r)
        r = tracked(c, FEDG_K_TRC_TEND, [&] { return launch_pair(N1, false, op, c->d_prof, in, st, c->Ne, c->stream); });
      if (r) return api_cuda_fail((cudaError_t)r, "fedg_trc_update (pair)");
      qsp = st.q_out;
    }
  }
  return 0;
}

}  // namespace fedg
