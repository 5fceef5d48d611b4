// fedg_nd_pair.cu -- the numerical diffusion of fedg_nd.cu in float pairs (FEDG_PREC_PAIR).
//
// Same passes, fluxes and lid values as the FP64 kernels (FElib's nonhydro3d_numdiff.F90:214-721,
// ..._dgm_bnd.F90:370-508), with every intermediate an unevaluated float pair (fedg_f2.cuh): the
// FP64 fields are split with integer instructions on load, the gradient and Laplacian fields stay
// pairs between passes, contractions and Lift are compensated sums of exact products, divisions are
// pair reciprocals.  The update adds the pair increment dt*tend to the FP64 field in FP64 (two
// adds), so the field keeps all of its bits.
// Why: the FP64 passes keep GB300's FP64 pipe ~87 % busy; the FP32 pipe issues 64x faster.
#include <cmath>
#include <cstring>

#include "fedg_ctx.cuh"
#include "fedg_f2.cuh"

namespace fedg {
namespace {

__device__ __forceinline__ f2 operator+(f2 a, f2 b) { return f2_add(a, b); }
__device__ __forceinline__ f2 operator-(f2 a, f2 b) { return f2_sub(a, b); }
__device__ __forceinline__ f2 operator*(f2 a, f2 b) { return f2_mul(a, b); }
__device__ __forceinline__ f2 z2() { return f2{0.f, 0.f}; }
__device__ __forceinline__ f2 ld64(const double* p, size_t g) { return f2_split(__ldg(p + g)); }
__device__ __forceinline__ f2 ldp(const float2* p, size_t g) { return f2_of(__ldg(p + g)); }

struct NdOpsP {
  float2 D[FEDG_MAXN1 * FEDG_MAXN1];
  float2 Lb[FEDG_MAXN1], Lt[FEDG_MAXN1];
  float2 E[3], FS[3];  // E11, E22, E33; Fscale of x, y, z faces
  int NeX, NeY, NeZ;
};

__device__ __forceinline__ int face_dir_p(int f) { return f >= 4 ? 2 : ((f & 1) ? 0 : 1); }
__device__ __forceinline__ float face_n_p(int f) { return (f == 1 || f == 2 || f == 5) ? 1.f : -1.f; }

// lid exteriors (even: wall-normal momentum reflected; odd: normal gradient reflected except for the
// wall-normal momentum); the normals are +-1, so the reflection is an exact sign change
__device__ __forceinline__ f2 even_ext_p(int var, int dir, f2 vM) {
  const bool refl = (var == VMX && dir == 0) || (var == VMY && dir == 1) || (var == VMZ && dir == 2);
  return refl ? f2_neg(vM) : vM;
}
__device__ __forceinline__ f2 odd_ext_p(int var, int dir, f2 gM) {
  const bool keep = (var == VMX && dir == 0) || (var == VMY && dir == 1) || (var == VMZ && dir == 2);
  return keep ? gM : f2_neg(gM);
}

template <int N1>
__device__ __forceinline__ void face_nodes_nd(const NdOpsP& op, int f, int a, int b, long ke, int ex, int ey, int ez,
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

template <int N1>
__device__ __forceinline__ f2 dsum_p(const NdOpsP& op, const float2* u, int dir, int i, int j, int k) {
  constexpr int NF = N1 * N1;
  f2acc s;
#pragma unroll
  for (int l = 0; l < N1; ++l) {
    const int p = dir == 0 ? l + N1 * j + NF * k : (dir == 1 ? i + N1 * l + NF * k : i + N1 * j + NF * l);
    s.add(f2_of(op.D[(dir == 0 ? i : (dir == 1 ? j : k)) * N1 + l]), f2_of(u[p]));
  }
  return s.get();
}
// Lift of the faces of one direction (x: faces 1, 3; y: 0, 2; z: 4, 5)
template <int N1>
__device__ __forceinline__ void lift_dir_p(f2acc& s, const NdOpsP& op, const float2* fv, int dir, int i, int j, int k) {
  constexpr int NF = N1 * N1;
  if (dir == 0) {
    s.add(f2_of(op.Lt[i]), f2_of(fv[1 * NF + j + N1 * k]));
    s.add(f2_of(op.Lb[i]), f2_of(fv[3 * NF + j + N1 * k]));
  } else if (dir == 1) {
    s.add(f2_of(op.Lb[j]), f2_of(fv[0 * NF + i + N1 * k]));
    s.add(f2_of(op.Lt[j]), f2_of(fv[2 * NF + i + N1 * k]));
  } else {
    s.add(f2_of(op.Lb[k]), f2_of(fv[4 * NF + i + N1 * j]));
    s.add(f2_of(op.Lt[k]), f2_of(fv[5 * NF + i + N1 * j]));
  }
}

struct NdIdx {
  long ke;
  int p, le, i, j, k, ex, ey, ez, nxy;
  bool valid;
};
template <int N1, int EPB>
__device__ __forceinline__ NdIdx nd_idx(const NdOpsP& op, int Ne) {
  constexpr int Np = N1 * N1 * N1, NF = N1 * N1;
  NdIdx e;
  const int tid = threadIdx.x;
  e.le = tid / Np;
  e.p = tid - e.le * Np;
  e.ke = (long)blockIdx.x * EPB + e.le;
  e.valid = e.ke < Ne;
  e.i = e.p % N1;
  e.j = (e.p / N1) % N1;
  e.k = e.p / NF;
  e.nxy = op.NeX * op.NeY;
  e.ez = e.valid ? (int)(e.ke / e.nxy) : 0;
  e.ey = e.valid ? (int)((e.ke - (long)e.ez * e.nxy) / op.NeX) : 0;
  e.ex = e.valid ? (int)(e.ke - (long)e.ez * e.nxy - (long)e.ey * op.NeX) : 0;
  return e;
}

// a field read either as FP64 (the prognostic variable) or as pairs (an intermediate)
struct Src {
  const double* d;
  const float2* p;
  __device__ __forceinline__ f2 at(size_t g) const { return d ? ld64(d, g) : ldp(p, g); }
};

// gradient pass: G = (d/dx Vh, d/dy Vh, d/dz Vv), divided by the density when dens_div; the even
// routine's lid exterior of Vh (and of Vv when bc_v)
template <int N1, int EPB>
__global__ void __launch_bounds__(EPB* N1* N1* N1)
    k_nd_grad_p(const NdOpsP op, const double* __restrict__ dens_prof, const Src Vh, const Src Vv,
                const double* __restrict__ ddens, int var, int dens_div, int bc_v, float2* __restrict__ Gx,
                float2* __restrict__ Gy, float2* __restrict__ Gz, int Ne) {
  constexpr int Np = N1 * N1 * N1, NF = N1 * N1;
  extern __shared__ float2 smp[];
  const NdIdx e = nd_idx<N1, EPB>(op, Ne);
  float2* vh = smp + e.le * (2 * Np + 6 * NF);
  float2* vv = vh + Np;
  float2* df = vv + Np;
  const size_t g = (size_t)e.ke * Np + e.p;
  if (e.valid) {
    const f2 rd = dens_div ? f2_recip(ld64(ddens, g) + f2_split(__ldg(dens_prof + e.ez * N1 + e.k))) : f2{1.f, 0.f};
    vh[e.p] = f2_pack(Vh.at(g) * rd);
    vv[e.p] = f2_pack(Vv.at(g) * rd);
    for (int fi = e.p; fi < 6 * NF; fi += Np) {
      const int f = fi / NF, ab = fi - f * NF, a = ab % N1, b = ab / N1;
      int pM;
      size_t gP;
      long kn;
      face_nodes_nd<N1>(op, f, a, b, e.ke, e.ex, e.ey, e.ez, e.nxy, pM, gP, kn);
      const size_t gM = (size_t)e.ke * Np + pM;
      const int dir = face_dir_p(f);
      const float n = face_n_p(f);
      f2 wM{1.f, 0.f}, wP{1.f, 0.f};
      if (dens_div) {
        const int levM = e.ez * N1 + pM / NF;
        const int levP = (kn >= 0 ? (int)(kn / e.nxy) : e.ez) * N1 + (int)((gP % Np) / NF);
        wP = f2_recip(ld64(ddens, gP) + f2_split(__ldg(dens_prof + levP)));
        wM = f2_recip(ld64(ddens, gM) + f2_split(__ldg(dens_prof + levM)));
      }
      const bool lid = kn < 0;
      const Src& S = dir == 2 ? Vv : Vh;
      const f2 sM = S.at(gM);
      f2 sP = S.at(gP);
      if (lid && (dir != 2 || bc_v)) sP = even_ext_p(var, dir, sM);
      const f2 d = f2_mul_f(sP * wP - sM * wM, 0.5f);
      // (1 - sign n) on interior faces: 2 on faces with n = -1, 0 with n = +1; 1 at a lid
      const float fac = lid ? n : (n < 0.f ? -2.f : 0.f);
      df[fi] = f2_pack(f2_mul_f(f2_of(op.FS[dir]) * d, fac));
    }
  }
  __syncthreads();
  if (!e.valid) return;
  f2acc sx, sy, sz;
  sx.add(f2_of(op.E[0]), dsum_p<N1>(op, vh, 0, e.i, e.j, e.k));
  lift_dir_p<N1>(sx, op, df, 0, e.i, e.j, e.k);
  sy.add(f2_of(op.E[1]), dsum_p<N1>(op, vh, 1, e.i, e.j, e.k));
  lift_dir_p<N1>(sy, op, df, 1, e.i, e.j, e.k);
  sz.add(f2_of(op.E[2]), dsum_p<N1>(op, vv, 2, e.i, e.j, e.k));
  lift_dir_p<N1>(sz, op, df, 2, e.i, e.j, e.k);
  Gx[g] = f2_pack(sx.get());
  Gy[g] = f2_pack(sy.get());
  Gz[g] = f2_pack(sz.get());
}

// Laplacian pass with the odd routine's lid exterior of G: horizontal and vertical parts
template <int N1, int EPB>
__global__ void __launch_bounds__(EPB* N1* N1* N1)
    k_nd_lap_p(const NdOpsP op, const float2* __restrict__ Gx, const float2* __restrict__ Gy,
               const float2* __restrict__ Gz, int var, float2* __restrict__ lh, float2* __restrict__ lv, int Ne) {
  constexpr int Np = N1 * N1 * N1, NF = N1 * N1;
  extern __shared__ float2 smp[];
  const NdIdx e = nd_idx<N1, EPB>(op, Ne);
  float2* gx = smp + e.le * (3 * Np + 6 * NF);
  float2* gy = gx + Np;
  float2* gz = gy + Np;
  float2* df = gz + Np;
  const size_t g = (size_t)e.ke * Np + e.p;
  if (e.valid) {
    gx[e.p] = __ldg(Gx + g);
    gy[e.p] = __ldg(Gy + g);
    gz[e.p] = __ldg(Gz + g);
    for (int fi = e.p; fi < 6 * NF; fi += Np) {
      const int f = fi / NF, ab = fi - f * NF, a = ab % N1, b = ab / N1;
      int pM;
      size_t gP;
      long kn;
      face_nodes_nd<N1>(op, f, a, b, e.ke, e.ex, e.ey, e.ez, e.nxy, pM, gP, kn);
      const size_t gM = (size_t)e.ke * Np + pM;
      const int dir = face_dir_p(f);
      const float n = face_n_p(f);
      const float2* Gd = dir == 0 ? Gx : (dir == 1 ? Gy : Gz);
      const f2 gMc = ldp(Gd, gM);
      const bool lid = kn < 0;
      const f2 gPc = lid ? odd_ext_p(var, dir, gMc) : ldp(Gd, gP);
      // 0.5 (1 + sign n) (g+ - g-) n on interior faces; 0.5 (g+ - g-) n at a lid
      const float fac = lid ? 0.5f * n : (n > 0.f ? 1.f : 0.f);
      df[fi] = f2_pack(f2_mul_f(f2_of(op.FS[dir]) * (gPc - gMc), fac));
    }
  }
  __syncthreads();
  if (!e.valid) return;
  f2acc sh, sv;
  sh.add(f2_of(op.E[0]), dsum_p<N1>(op, gx, 0, e.i, e.j, e.k));
  sh.add(f2_of(op.E[1]), dsum_p<N1>(op, gy, 1, e.i, e.j, e.k));
  lift_dir_p<N1>(sh, op, df, 0, e.i, e.j, e.k);
  lift_dir_p<N1>(sh, op, df, 1, e.i, e.j, e.k);
  sv.add(f2_of(op.E[2]), dsum_p<N1>(op, gz, 2, e.i, e.j, e.k));
  lift_dir_p<N1>(sv, op, df, 2, e.i, e.j, e.k);
  lh[g] = f2_pack(sh.get());
  lv[g] = f2_pack(sv.get());
}

// tendency pass with the odd routine's lid exterior of G, then V += dt tend (the increment in pairs,
// added to the FP64 field in FP64)
template <int N1, int EPB>
__global__ void __launch_bounds__(EPB* N1* N1* N1)
    k_nd_tend_p(const NdOpsP op, const double* __restrict__ dens_prof, const float2* __restrict__ Gx,
                const float2* __restrict__ Gy, const float2* __restrict__ Gz, const double* ddens, int var, int mul_dens,
                float2 ch, float2 cv, float2 dt, double* V, int Ne) {
  constexpr int Np = N1 * N1 * N1, NF = N1 * N1;
  extern __shared__ float2 smp[];
  const NdIdx e = nd_idx<N1, EPB>(op, Ne);
  float2* fx = smp + e.le * (3 * Np + 6 * NF);
  float2* fy = fx + Np;
  float2* fz = fy + Np;
  float2* df = fz + Np;
  const size_t g = (size_t)e.ke * Np + e.p;
  if (e.valid) {
    // DDENS is read only when it weights the variable (for DDENS itself V aliases it)
    const f2 dens = mul_dens ? f2_split(__ldg(dens_prof + e.ez * N1 + e.k)) + ld64(ddens, g) : f2{1.f, 0.f};
    const f2 h = f2_of(ch) * dens, v = f2_of(cv) * dens;
    fx[e.p] = f2_pack(h * ldp(Gx, g));
    fy[e.p] = f2_pack(h * ldp(Gy, g));
    fz[e.p] = f2_pack(v * ldp(Gz, g));
    for (int fi = e.p; fi < 6 * NF; fi += Np) {
      const int f = fi / NF, ab = fi - f * NF, a = ab % N1, b = ab / N1;
      int pM;
      size_t gP;
      long kn;
      face_nodes_nd<N1>(op, f, a, b, e.ke, e.ex, e.ey, e.ez, e.nxy, pM, gP, kn);
      const size_t gM = (size_t)e.ke * Np + pM;
      const int dir = face_dir_p(f);
      const float n = face_n_p(f);
      const float2* Gd = dir == 0 ? Gx : (dir == 1 ? Gy : Gz);
      const f2 gMc = ldp(Gd, gM);
      const bool lid = kn < 0;
      const f2 gPc = lid ? odd_ext_p(var, dir, gMc) : ldp(Gd, gP);
      f2 wM{0.5f, 0.f}, wP{0.5f, 0.f};
      if (mul_dens) {
        const int levM = e.ez * N1 + pM / NF;
        const int levP = (kn >= 0 ? (int)(kn / e.nxy) : e.ez) * N1 + (int)((gP % Np) / NF);
        wM = f2_mul_f(f2_split(__ldg(dens_prof + levM)) + ld64(ddens, gM), 0.5f);
        wP = f2_mul_f(f2_split(__ldg(dens_prof + levP)) + ld64(ddens, gP), 0.5f);
      }
      const f2 c = f2_of(dir == 2 ? cv : ch);
      // (1 + sign n) on interior faces: 2 with n = +1, 0 with n = -1; 1 at a lid
      const float fac = lid ? n : (n > 0.f ? 2.f : 0.f);
      df[fi] = f2_pack(f2_mul_f(f2_of(op.FS[dir]) * (c * (wP * gPc - wM * gMc)), fac));
    }
  }
  __syncthreads();
  if (!e.valid) return;
  f2acc s;
  s.add(f2_of(op.E[0]), dsum_p<N1>(op, fx, 0, e.i, e.j, e.k));
  s.add(f2_of(op.E[1]), dsum_p<N1>(op, fy, 1, e.i, e.j, e.k));
  s.add(f2_of(op.E[2]), dsum_p<N1>(op, fz, 2, e.i, e.j, e.k));
  lift_dir_p<N1>(s, op, df, 0, e.i, e.j, e.k);
  lift_dir_p<N1>(s, op, df, 1, e.i, e.j, e.k);
  lift_dir_p<N1>(s, op, df, 2, e.i, e.j, e.k);
  const f2 inc = f2_of(dt) * s.get();
  V[g] = (V[g] + (double)inc.h) + (double)inc.l;
}

float2 hsplit_nd(double x) {
  const float h = (float)x;
  return make_float2(h, (float)(x - (double)h));
}

template <int N1>
constexpr int nd_epb_p() { return N1 <= 4 ? (N1 <= 2 ? 16 : (N1 == 3 ? 8 : 4)) : 1; }

template <int N1>
int nd_pass_p_n(int pass, const NdOpsP& op, const double* dp, Src a, Src b, const float2* G0, const float2* G1,
                const float2* G2, const double* ddens, int var, int f1, int f2, float2 ch, float2 cv, float2 dt,
                float2* o1, float2* o2, float2* o3, double* V, int Ne, cudaStream_t s) {
  constexpr int EPB = nd_epb_p<N1>(), Np = N1 * N1 * N1, NF = N1 * N1;
  const int grid = (Ne + EPB - 1) / EPB;
  if (pass == 0) {
    const size_t sm = sizeof(float2) * EPB * (2 * Np + 6 * NF);
    auto kf = k_nd_grad_p<N1, EPB>;
    cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    kf<<<grid, EPB * Np, sm, s>>>(op, dp, a, b, ddens, var, f1, f2, o1, o2, o3, Ne);
  } else if (pass == 1) {
    const size_t sm = sizeof(float2) * EPB * (3 * Np + 6 * NF);
    auto kf = k_nd_lap_p<N1, EPB>;
    cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    kf<<<grid, EPB * Np, sm, s>>>(op, G0, G1, G2, var, o1, o2, Ne);
  } else {
    const size_t sm = sizeof(float2) * EPB * (3 * Np + 6 * NF);
    auto kf = k_nd_tend_p<N1, EPB>;
    cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    kf<<<grid, EPB * Np, sm, s>>>(op, dp, G0, G1, G2, ddens, var, f1, ch, cv, dt, V, Ne);
  }
  return (int)cudaGetLastError();
}

int nd_pass_p(int N1, int pass, const NdOpsP& op, const double* dp, Src a, Src b, const float2* G0, const float2* G1,
              const float2* G2, const double* ddens, int var, int f1, int f2, float2 ch, float2 cv, float2 dt,
              float2* o1, float2* o2, float2* o3, double* V, int Ne, cudaStream_t s) {
  switch (N1) {
    case 2: return nd_pass_p_n<2>(pass, op, dp, a, b, G0, G1, G2, ddens, var, f1, f2, ch, cv, dt, o1, o2, o3, V, Ne, s);
    case 3: return nd_pass_p_n<3>(pass, op, dp, a, b, G0, G1, G2, ddens, var, f1, f2, ch, cv, dt, o1, o2, o3, V, Ne, s);
    case 4: return nd_pass_p_n<4>(pass, op, dp, a, b, G0, G1, G2, ddens, var, f1, f2, ch, cv, dt, o1, o2, o3, V, Ne, s);
    case 5: return nd_pass_p_n<5>(pass, op, dp, a, b, G0, G1, G2, ddens, var, f1, f2, ch, cv, dt, o1, o2, o3, V, Ne, s);
    case 6: return nd_pass_p_n<6>(pass, op, dp, a, b, G0, G1, G2, ddens, var, f1, f2, ch, cv, dt, o1, o2, o3, V, Ne, s);
    case 7: return nd_pass_p_n<7>(pass, op, dp, a, b, G0, G1, G2, ddens, var, f1, f2, ch, cv, dt, o1, o2, o3, V, Ne, s);
    case 8: return nd_pass_p_n<8>(pass, op, dp, a, b, G0, G1, G2, ddens, var, f1, f2, ch, cv, dt, o1, o2, o3, V, Ne, s);
  }
  return (int)cudaErrorInvalidValue;
}

}  // namespace

// fedg_numdiff_apply_prec with prec == FEDG_PREC_PAIR; scratch = 5 Np*Ne doubles reused as pairs
int numdiff_apply_pair(fedg_ctx* c, double* const q[5], int nlap, double coef_h, double coef_v, double dt,
                       double* scratch) {
  const Ops& d = c->op;
  NdOpsP op;
  std::memset(&op, 0, sizeof(op));
  const int N1 = c->N1;
  for (int a = 0; a < N1 * N1; ++a) op.D[a] = hsplit_nd(d.D[a]);
  for (int a = 0; a < N1; ++a) {
    op.Lb[a] = hsplit_nd(d.Lb[a]);
    op.Lt[a] = hsplit_nd(d.Lt[a]);
  }
  op.E[0] = hsplit_nd(d.E11);
  op.E[1] = hsplit_nd(d.E22);
  op.E[2] = hsplit_nd(d.E33);
  op.FS[0] = hsplit_nd(d.FSx);
  op.FS[1] = hsplit_nd(d.FSy);
  op.FS[2] = hsplit_nd(d.FSz);
  op.NeX = d.NeX;
  op.NeY = d.NeY;
  op.NeZ = d.NeZ;
  const size_t n = c->n;
  float2* Gx = reinterpret_cast<float2*>(scratch);
  float2* Gy = Gx + n;
  float2* Gz = Gy + n;
  float2* lh = Gz + n;
  float2* lv = lh + n;
  const double sgn = ((nlap + 1) % 2 == 0) ? 1.0 : -1.0;
  const float2 ch = hsplit_nd(sgn * coef_h), cv = hsplit_nd(sgn * coef_v), dtp = hsplit_nd(dt), zero = make_float2(0.f, 0.f);
  const int order[5] = {VRT, VMZ, VMX, VMY, VD};
  for (int vi = 0; vi < 5; ++vi) {
    const int var = order[vi];
    const int dw = var != VD;
    const Src qv{q[var], nullptr};
    int r = tracked(c, FEDG_K_ND, [&] {
      return nd_pass_p(N1, 0, op, c->d_prof, qv, qv, nullptr, nullptr, nullptr, q[VD], var, dw, 1, zero, zero, zero,
                       Gx, Gy, Gz, nullptr, c->Ne, c->stream);
    });
    for (int it = 1; it < nlap && !r; ++it) {
      r = tracked(c, FEDG_K_ND, [&] {
        return nd_pass_p(N1, 1, op, c->d_prof, Src{}, Src{}, Gx, Gy, Gz, nullptr, var, 0, 0, zero, zero, zero, lh, lv,
                         nullptr, nullptr, c->Ne, c->stream);
      });
      if (!r)
        r = tracked(c, FEDG_K_ND, [&] {
          return nd_pass_p(N1, 0, op, c->d_prof, Src{nullptr, lh}, Src{nullptr, lv}, nullptr, nullptr, nullptr, q[VD], var,
                           0, 0, zero, zero, zero, Gx, Gy, Gz, nullptr, c->Ne, c->stream);
        });
    }
    if (!r)
      r = tracked(c, FEDG_K_ND, [&] {
        return nd_pass_p(N1, 2, op, c->d_prof, Src{}, Src{}, Gx, Gy, Gz, q[VD], var, dw, 0, ch, cv, dtp, nullptr, nullptr,
                         nullptr, q[var], c->Ne, c->stream);
      });
    if (r) return api_cuda_fail((cudaError_t)r, "fedg_numdiff_apply (pair)");
  }
  return 0;
}

}  // namespace fedg
