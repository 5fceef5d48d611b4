// fedg_nd.cu -- numerical diffusion (FElib's hyperdiffusion filter) and the sponge layer, FP64.
//
// Numerical diffusion: each prognostic variable q gets q += dt (-1)^(n+1) coef nabla^(2n) q after
// the dynamics step, the Laplacian built from one-sided LDG fluxes (the gradient takes the exterior
// value on faces with a negative normal, the divergence on faces with a positive one), with
// horizontal and vertical coefficients, density weighting of all variables but DDENS, and the lid
// values of FElib's boundary routines (centred fluxes there).
//   FElib/src/fluid_dyn_solver/scale_atm_dyn_dgm_nonhydro3d_numdiff.F90
//     Apply / apply_numfilter :214-376; numdiff_tend :379-440; cal_del_flux_lap_with_coef :443-500
//     numdiff_cal_laplacian :505-558; cal_del_flux_lap :561-601; numdiff_cal_flx :606-665
//     cal_del_gradDiffVar :668-721
//   lid values  ..._dgm_bnd.F90:370-508 (ApplyBC_numdiff_odd_lc / _even_lc), slip + adiabatic lids
// Sponge layer: Rayleigh damping of MOMZ (and optionally MOMX, MOMY) added to the explicit tendency,
// coefficient 0.25/tau (1 + sign(z - h)) (1 - cos(pi (z - h)/(z_top - h)))
//   ..._dgm_spongelayer.F90:134-219
//
// One thread block per element (EPB elements for p <= 3), one launch per pass and variable.  On the
// axis-aligned faces of the flat cube only the normal component of each face flux is nonzero, so
// each face node carries one value.
#include <cmath>
#include <cstring>
#include <vector>

#include "fedg_ctx.cuh"

namespace fedg {
namespace {

__device__ __forceinline__ double sgn1(double x) { return signbit(x) ? -1.0 : 1.0; }  // Fortran sign(1, x)
__device__ __forceinline__ double face_n(int f) { return (f == 1 || f == 2 || f == 5) ? 1.0 : -1.0; }
__device__ __forceinline__ int face_dir(int f) { return f >= 4 ? 2 : ((f & 1) ? 0 : 1); }

// exterior of a scalar at a lid (even routine): the wall-normal momentum is reflected
__device__ __forceinline__ double even_ext(int var, int dir, double vM, double n) {
  const bool refl = (var == VMX && dir == 0) || (var == VMY && dir == 1) || (var == VMZ && dir == 2);
  if (!refl) return vM;
  const double g = vM * n;
  return vM - 2.0 * g * n;
}
// exterior normal gradient component at a lid (odd routine): the normal component is reflected for
// DENS/RHOT (adiabatic) and for the tangential momenta (slip); kept for the wall-normal momentum
__device__ __forceinline__ double odd_ext_n(int var, int dir, double gMn_comp, double n) {
  const bool keep = (var == VMX && dir == 0) || (var == VMY && dir == 1) || (var == VMZ && dir == 2);
  if (keep) return gMn_comp;
  const double gn = gMn_comp * n;
  return gMn_comp - 2.0 * gn * n;
}

template <int N1>
__device__ __forceinline__ double lift(const Ops& op, const double* fv, int i, int j, int k) {
  constexpr int NF = N1 * N1;
  return op.Lb[j] * fv[0 * NF + i + N1 * k] + op.Lt[i] * fv[1 * NF + j + N1 * k] + op.Lt[j] * fv[2 * NF + i + N1 * k] +
         op.Lb[i] * fv[3 * NF + j + N1 * k] + op.Lb[k] * fv[4 * NF + i + N1 * j] + op.Lt[k] * fv[5 * NF + i + N1 * j];
}
// Lift of the faces of one direction only (the others carry zeros)
template <int N1>
__device__ __forceinline__ double lift_dir(const Ops& op, const double* fv, int dir, int i, int j, int k) {
  constexpr int NF = N1 * N1;
  if (dir == 0) return op.Lt[i] * fv[1 * NF + j + N1 * k] + op.Lb[i] * fv[3 * NF + j + N1 * k];
  if (dir == 1) return op.Lb[j] * fv[0 * NF + i + N1 * k] + op.Lt[j] * fv[2 * NF + i + N1 * k];
  return op.Lb[k] * fv[4 * NF + i + N1 * j] + op.Lt[k] * fv[5 * NF + i + N1 * j];
}
template <int N1>
__device__ __forceinline__ double dsum(const Ops& op, const double* u, int dir, int i, int j, int k) {
  constexpr int NF = N1 * N1;
  double s = 0.0;
#pragma unroll
  for (int l = 0; l < N1; ++l) {
    const int p = dir == 0 ? l + N1 * j + NF * k : (dir == 1 ? i + N1 * l + NF * k : i + N1 * j + NF * l);
    s = fma(op.D[(dir == 0 ? i : (dir == 1 ? j : k)) * N1 + l], u[p], s);
  }
  return s;
}

struct ElemIdx {
  long ke;
  int p, le, i, j, k, ex, ey, ez, nxy;
  bool valid;
};
template <int N1, int EPB>
__device__ __forceinline__ ElemIdx elem_idx(const Ops& op, int Ne) {
  constexpr int Np = N1 * N1 * N1, NF = N1 * N1;
  ElemIdx e;
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

__device__ __forceinline__ double fscale(const Ops& op, int f) { return f >= 4 ? op.FSz : ((f & 1) ? op.FSx : op.FSy); }

// numdiff_cal_flx: G = (d/dx Vh, d/dy Vh, d/dz Vv) (each divided by the density when dens_div),
// with the even routine's lid exterior of Vh (and of Vv when bc_v)
template <int N1, int EPB>
__global__ void __launch_bounds__(EPB* N1* N1* N1)
    k_nd_grad(const Ops op, const double* __restrict__ dens_prof, const double* __restrict__ Vh,
              const double* __restrict__ Vv, const double* __restrict__ ddens, int var, int dens_div, int bc_v,
              double* __restrict__ Gx, double* __restrict__ Gy, double* __restrict__ Gz, int Ne) {
  constexpr int Np = N1 * N1 * N1, NF = N1 * N1;
  extern __shared__ double sm[];
  const ElemIdx e = elem_idx<N1, EPB>(op, Ne);
  double* vh = sm + e.le * (2 * Np + 6 * NF);
  double* vv = vh + Np;
  double* df = vv + Np;
  const size_t g = (size_t)e.ke * Np + e.p;
  if (e.valid) {
    const double dens = dens_div ? __ldg(ddens + g) + __ldg(dens_prof + e.ez * N1 + e.k) : 1.0;
    vh[e.p] = dens_div ? __ldg(Vh + g) / dens : __ldg(Vh + g);
    vv[e.p] = dens_div ? __ldg(Vv + g) / dens : __ldg(Vv + g);
    for (int fi = e.p; fi < 6 * NF; fi += Np) {
      const int f = fi / NF, ab = fi - f * NF, a = ab % N1, b = ab / N1;
      int pM;
      size_t gP;
      long kn;
      face_exterior<N1>(op, f, a, b, e.ke, e.ex, e.ey, e.ez, e.nxy, pM, gP, kn);
      const size_t gM = (size_t)e.ke * Np + pM;
      const int dir = face_dir(f);
      const double n = face_n(f);
      double wM = 1.0, wP = 1.0;
      if (dens_div) {
        const int levM = e.ez * N1 + pM / NF;
        const int levP = (kn >= 0 ? (int)(kn / e.nxy) : e.ez) * N1 + (int)((gP % Np) / NF);
        wP = 1.0 / (__ldg(ddens + gP) + __ldg(dens_prof + levP));
        wM = 1.0 / (__ldg(ddens + gM) + __ldg(dens_prof + levM));
      }
      const bool lid = kn < 0;
      const double src_M = dir == 2 ? __ldg(Vv + gM) : __ldg(Vh + gM);
      double src_P = dir == 2 ? __ldg(Vv + gP) : __ldg(Vh + gP);
      if (lid && (dir != 2 || bc_v)) src_P = even_ext(var, dir, src_M, n);
      const double d = 0.5 * (src_P * wP - src_M * wM);
      df[fi] = fscale(op, f) * (lid ? d * n : (1.0 - sgn1(n)) * d * n);
    }
  }
  __syncthreads();
  if (!e.valid) return;
  Gx[g] = op.E11 * dsum<N1>(op, vh, 0, e.i, e.j, e.k) + lift_dir<N1>(op, df, 0, e.i, e.j, e.k);
  Gy[g] = op.E22 * dsum<N1>(op, vh, 1, e.i, e.j, e.k) + lift_dir<N1>(op, df, 1, e.i, e.j, e.k);
  Gz[g] = op.E33 * dsum<N1>(op, vv, 2, e.i, e.j, e.k) + lift_dir<N1>(op, df, 2, e.i, e.j, e.k);
}

// numdiff_cal_laplacian with the odd routine's lid exterior of G: horizontal and vertical parts
template <int N1, int EPB>
__global__ void __launch_bounds__(EPB* N1* N1* N1)
    k_nd_lap(const Ops op, const double* __restrict__ Gx, const double* __restrict__ Gy,
             const double* __restrict__ Gz, int var, double* __restrict__ lh, double* __restrict__ lv, int Ne) {
  constexpr int Np = N1 * N1 * N1, NF = N1 * N1;
  extern __shared__ double sm[];
  const ElemIdx e = elem_idx<N1, EPB>(op, Ne);
  double* gx = sm + e.le * (3 * Np + 6 * NF);
  double* gy = gx + Np;
  double* gz = gy + Np;
  double* df = gz + Np;
  const size_t g = (size_t)e.ke * Np + e.p;
  const double* G[3] = {Gx, Gy, Gz};
  if (e.valid) {
    gx[e.p] = __ldg(Gx + g);
    gy[e.p] = __ldg(Gy + g);
    gz[e.p] = __ldg(Gz + g);
    for (int fi = e.p; fi < 6 * NF; fi += Np) {
      const int f = fi / NF, ab = fi - f * NF, a = ab % N1, b = ab / N1;
      int pM;
      size_t gP;
      long kn;
      face_exterior<N1>(op, f, a, b, e.ke, e.ex, e.ey, e.ez, e.nxy, pM, gP, kn);
      const size_t gM = (size_t)e.ke * Np + pM;
      const int dir = face_dir(f);
      const double n = face_n(f);
      const double gMc = __ldg(G[dir] + gM);
      const bool lid = kn < 0;
      const double gPc = lid ? odd_ext_n(var, dir, gMc, n) : __ldg(G[dir] + gP);
      df[fi] = fscale(op, f) * (lid ? 0.5 * (gPc - gMc) * n : 0.5 * (1.0 + sgn1(n)) * (gPc - gMc) * n);
    }
  }
  __syncthreads();
  if (!e.valid) return;
  lh[g] = op.E11 * dsum<N1>(op, gx, 0, e.i, e.j, e.k) + op.E22 * dsum<N1>(op, gy, 1, e.i, e.j, e.k) +
          (lift_dir<N1>(op, df, 1, e.i, e.j, e.k) + lift_dir<N1>(op, df, 0, e.i, e.j, e.k));
  lv[g] = op.E33 * dsum<N1>(op, gz, 2, e.i, e.j, e.k) + lift_dir<N1>(op, df, 2, e.i, e.j, e.k);
}

// numdiff_tend with the odd routine's lid exterior of G, then V += dt tend
template <int N1, int EPB>
__global__ void __launch_bounds__(EPB* N1* N1* N1)
    k_nd_tend(const Ops op, const double* __restrict__ dens_prof, const double* __restrict__ Gx,
              const double* __restrict__ Gy, const double* __restrict__ Gz, const double* ddens, int var,
              int mul_dens, double ch, double cv, double dt, double* V, int Ne) {
  constexpr int Np = N1 * N1 * N1, NF = N1 * N1;
  extern __shared__ double sm[];
  const ElemIdx e = elem_idx<N1, EPB>(op, Ne);
  double* fx = sm + e.le * (3 * Np + 6 * NF);
  double* fy = fx + Np;
  double* fz = fy + Np;
  double* df = fz + Np;
  const size_t g = (size_t)e.ke * Np + e.p;
  const double* G[3] = {Gx, Gy, Gz};
  if (e.valid) {
    // DDENS is read only when it weights the variable (for DDENS itself V aliases it)
    const double dens = mul_dens ? __ldg(dens_prof + e.ez * N1 + e.k) + __ldg(ddens + g) : 1.0;
    const double h = mul_dens ? ch * dens : ch, v = mul_dens ? cv * dens : cv;
    fx[e.p] = h * __ldg(Gx + g);
    fy[e.p] = h * __ldg(Gy + g);
    fz[e.p] = v * __ldg(Gz + g);
    for (int fi = e.p; fi < 6 * NF; fi += Np) {
      const int f = fi / NF, ab = fi - f * NF, a = ab % N1, b = ab / N1;
      int pM;
      size_t gP;
      long kn;
      face_exterior<N1>(op, f, a, b, e.ke, e.ex, e.ey, e.ez, e.nxy, pM, gP, kn);
      const size_t gM = (size_t)e.ke * Np + pM;
      const int dir = face_dir(f);
      const double n = face_n(f);
      const double gMc = __ldg(G[dir] + gM);
      const bool lid = kn < 0;
      const double gPc = lid ? odd_ext_n(var, dir, gMc, n) : __ldg(G[dir] + gP);
      double wM = 0.5, wP = 0.5;
      if (mul_dens) {
        const int levM = e.ez * N1 + pM / NF;
        const int levP = (kn >= 0 ? (int)(kn / e.nxy) : e.ez) * N1 + (int)((gP % Np) / NF);
        wM = 0.5 * (__ldg(dens_prof + levM) + __ldg(ddens + gM));
        wP = 0.5 * (__ldg(dens_prof + levP) + __ldg(ddens + gP));
      }
      const double c = dir == 2 ? cv : ch;
      const double d = lid ? c * (wP * gPc - wM * gMc) * n : (1.0 + sgn1(n)) * c * (wP * gPc - wM * gMc) * n;
      df[fi] = fscale(op, f) * d;
    }
  }
  __syncthreads();
  if (!e.valid) return;
  const double t = op.E11 * dsum<N1>(op, fx, 0, e.i, e.j, e.k) + op.E22 * dsum<N1>(op, fy, 1, e.i, e.j, e.k) +
                   op.E33 * dsum<N1>(op, fz, 2, e.i, e.j, e.k) + lift<N1>(op, df, e.i, e.j, e.k);
  V[g] = V[g] + dt * t;
}

// sponge layer: tend -= c(z) (s MOMX, s MOMY, MOMZ), c per level
__global__ void k_sponge(const double* __restrict__ coef, double* __restrict__ tx, double* __restrict__ ty,
                         double* __restrict__ tz, const double* __restrict__ mx, const double* __restrict__ my,
                         const double* __restrict__ mz, double s, int N1, int Np, size_t nxy, size_t n) {
  const size_t g = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n) return;
  const size_t ke = g / Np;
  const int lev = (int)(ke / nxy) * N1 + (int)(g - ke * Np) / (N1 * N1);
  const double c = __ldg(coef + lev);
  tx[g] = tx[g] - s * c * __ldg(mx + g);
  ty[g] = ty[g] - s * c * __ldg(my + g);
  tz[g] = tz[g] - c * __ldg(mz + g);
}

template <int N1>
constexpr int nd_epb() { return N1 <= 4 ? (N1 <= 2 ? 16 : (N1 == 3 ? 8 : 4)) : 1; }

template <int N1>
int nd_pass_n(int pass, const Ops& op, const double* dp, const double* a, const double* b, const double* c,
              const double* ddens, int var, int flag1, int flag2, double ch, double cv, double dt, double* o1,
              double* o2, double* o3, int Ne, cudaStream_t s) {
  constexpr int EPB = nd_epb<N1>(), Np = N1 * N1 * N1, NF = N1 * N1;
  const int grid = (Ne + EPB - 1) / EPB;
  if (pass == 0) {
    const size_t sm = sizeof(double) * EPB * (2 * Np + 6 * NF);
    auto kf = k_nd_grad<N1, EPB>;
    cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    kf<<<grid, EPB * Np, sm, s>>>(op, dp, a, b, ddens, var, flag1, flag2, o1, o2, o3, Ne);
  } else if (pass == 1) {
    const size_t sm = sizeof(double) * EPB * (3 * Np + 6 * NF);
    auto kf = k_nd_lap<N1, EPB>;
    cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    kf<<<grid, EPB * Np, sm, s>>>(op, a, b, c, var, o1, o2, Ne);
  } else {
    const size_t sm = sizeof(double) * EPB * (3 * Np + 6 * NF);
    auto kf = k_nd_tend<N1, EPB>;
    cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    kf<<<grid, EPB * Np, sm, s>>>(op, dp, a, b, c, ddens, var, flag1, ch, cv, dt, o1, Ne);
  }
  return (int)cudaGetLastError();
}

int nd_pass(int pass, const Ops& op, const double* dp, const double* a, const double* b, const double* c,
            const double* ddens, int var, int flag1, int flag2, double ch, double cv, double dt, double* o1,
            double* o2, double* o3, int Ne, cudaStream_t s) {
  switch (op.N1) {
    case 2: return nd_pass_n<2>(pass, op, dp, a, b, c, ddens, var, flag1, flag2, ch, cv, dt, o1, o2, o3, Ne, s);
    case 3: return nd_pass_n<3>(pass, op, dp, a, b, c, ddens, var, flag1, flag2, ch, cv, dt, o1, o2, o3, Ne, s);
    case 4: return nd_pass_n<4>(pass, op, dp, a, b, c, ddens, var, flag1, flag2, ch, cv, dt, o1, o2, o3, Ne, s);
    case 5: return nd_pass_n<5>(pass, op, dp, a, b, c, ddens, var, flag1, flag2, ch, cv, dt, o1, o2, o3, Ne, s);
    case 6: return nd_pass_n<6>(pass, op, dp, a, b, c, ddens, var, flag1, flag2, ch, cv, dt, o1, o2, o3, Ne, s);
    case 7: return nd_pass_n<7>(pass, op, dp, a, b, c, ddens, var, flag1, flag2, ch, cv, dt, o1, o2, o3, Ne, s);
    case 8: return nd_pass_n<8>(pass, op, dp, a, b, c, ddens, var, flag1, flag2, ch, cv, dt, o1, o2, o3, Ne, s);
  }
  return (int)cudaErrorInvalidValue;
}

}  // namespace
}  // namespace fedg

namespace fedg {
void sponge_coef_host(const fedg_ctx* c, double tau, double height, double* coef) {
  std::vector<double> xs(c->N1);
  lgl_nodes_1d(c->N1 - 1, xs.data());
  const double dz = (c->d.zmax - c->d.zmin) / c->d.NeZ, rt = 1.0 / tau, ztop = c->d.zmax;
  for (int l = 0; l < c->L; ++l) {
    const int ez = l / c->N1, k = l - ez * c->N1;
    const double z = c->d.zmin + (ez + 0.5 * (xs[k] + 1.0)) * dz;
    coef[l] = 0.25 * rt * (1.0 + (std::signbit(z - height) ? -1.0 : 1.0)) *
              (1.0 - std::cos(M_PI * (z - height) / (ztop - height)));
  }
}
}  // namespace fedg

extern "C" {

int fedg_numdiff_apply(fedg_ctx* c, double* const q[5], int nlap, double coef_h, double coef_v, double dt) {
  return fedg_numdiff_apply_prec(c, q, nlap, coef_h, coef_v, dt, FEDG_PREC_FP64);
}

int fedg_numdiff_apply_prec(fedg_ctx* c, double* const q[5], int nlap, double coef_h, double coef_v, double dt,
                            int prec) {
  if (!c || !q) return api_fail("fedg_numdiff_apply: null argument");
  if (fedg::slab(c)) return api_fail("fedg_numdiff_apply: not available on a part of a decomposed mesh (periodic_x/y = FEDG_HALO)");
  if (prec != FEDG_PREC_FP64 && prec != FEDG_PREC_PAIR)
    return api_fail("fedg_numdiff_apply: prec must be FEDG_PREC_FP64 or FEDG_PREC_PAIR");
  for (int v = 0; v < 5; ++v)
    if (!q[v]) return api_fail("fedg_numdiff_apply: null field");
  if (nlap < 1) return api_fail("fedg_numdiff_apply: ND_LAPLACIAN_NUM must be >= 1");
  if (!c->base_set) return api_fail("fedg_numdiff_apply: the base state is not registered (fedg_set_base_state)");
  cudaSetDevice(c->d.device);
  const size_t n = c->n;
  if (!c->nd_buf) {
    if (cudaMalloc(&c->nd_buf, sizeof(double) * 5 * n) != cudaSuccess) {
      c->nd_buf = nullptr;
      return api_fail("fedg_numdiff_apply: out of device memory (5 fields of scratch)");
    }
  }
  if (prec == FEDG_PREC_PAIR) return numdiff_apply_pair(c, q, nlap, coef_h, coef_v, dt, c->nd_buf);
  double* Gx = c->nd_buf;
  double* Gy = Gx + n;
  double* Gz = Gy + n;
  double* lh = Gz + n;
  double* lv = lh + n;
  const double sgn = ((nlap + 1) % 2 == 0) ? 1.0 : -1.0;  // (-1)^mod(n+1, 2)
  const int order[5] = {VRT, VMZ, VMX, VMY, VD};         // apply_numfilter's order: DDENS changes last
  for (int vi = 0; vi < 5; ++vi) {
    const int var = order[vi];
    const int dw = var != VD;
    int r = tracked(c, FEDG_K_ND, [&] {
      return nd_pass(0, c->op, c->d_prof, q[var], q[var], nullptr, q[VD], var, dw, 1, 0, 0, 0, Gx, Gy, Gz, c->Ne,
                     c->stream);
    });
    for (int it = 1; it < nlap && !r; ++it) {
      r = tracked(c, FEDG_K_ND, [&] {
        return nd_pass(1, c->op, c->d_prof, Gx, Gy, Gz, nullptr, var, 0, 0, 0, 0, 0, lh, lv, nullptr, c->Ne, c->stream);
      });
      if (!r)
        r = tracked(c, FEDG_K_ND, [&] {
          return nd_pass(0, c->op, c->d_prof, lh, lv, nullptr, q[VD], var, 0, 0, 0, 0, 0, Gx, Gy, Gz, c->Ne, c->stream);
        });
    }
    if (!r)
      r = tracked(c, FEDG_K_ND, [&] {
        return nd_pass(2, c->op, c->d_prof, Gx, Gy, Gz, q[VD], var, dw, 0, sgn * coef_h, sgn * coef_v, dt, q[var],
                       nullptr, nullptr, c->Ne, c->stream);
      });
    if (r) return api_cuda_fail((cudaError_t)r, "fedg_numdiff_apply");
  }
  return 0;
}

int fedg_sponge_add_tend(fedg_ctx* c, double* const tend[3], const double* const mom[3], double tau, double height,
                         int hveldamp) {
  if (!c || !tend || !mom) return api_fail("fedg_sponge_add_tend: null argument");
  for (int d = 0; d < 3; ++d)
    if (!tend[d] || !mom[d]) return api_fail("fedg_sponge_add_tend: null field");
  if (!(tau > 0.0)) return api_fail("fedg_sponge_add_tend: tau must be positive");
  if (!(height < c->d.zmax)) return api_fail("fedg_sponge_add_tend: the damping height must be below the top");
  cudaSetDevice(c->d.device);
  std::vector<double> coef(c->L);
  sponge_coef_host(c, tau, height, coef.data());
  if (!c->sponge_coef && cudaMalloc(&c->sponge_coef, sizeof(double) * c->L) != cudaSuccess) {
    c->sponge_coef = nullptr;
    return api_fail("fedg_sponge_add_tend: out of device memory");
  }
  const bool upload = !(c->sponge_key[0] == tau && c->sponge_key[1] == height);
  if (upload) {  // the profile is uploaded only when (tau, height) change
    if (cudaMemcpyAsync(c->sponge_coef, coef.data(), sizeof(double) * c->L, cudaMemcpyHostToDevice, c->stream) !=
        cudaSuccess)
      return api_fail("fedg_sponge_add_tend: coefficient upload");
    c->sponge_key[0] = tau;
    c->sponge_key[1] = height;
  }
  const int r = tracked(c, FEDG_K_ND, [&] {
    k_sponge<<<(unsigned)((c->n + 255) / 256), 256, 0, c->stream>>>(c->sponge_coef, tend[0], tend[1], tend[2], mom[0],
                                                                   mom[1], mom[2], hveldamp ? 1.0 : 0.0, c->N1, c->Np,
                                                                   c->nxy, c->n);
    return (int)cudaGetLastError();
  });
  if (r) return api_cuda_fail((cudaError_t)r, "fedg_sponge_add_tend");
  // the host coefficient array must outlive the asynchronous copy
  if (upload && cudaStreamSynchronize(c->stream) != cudaSuccess) return api_fail("fedg_sponge_add_tend: synchronise");
  return 0;
}

}  // extern "C"
