// fedg_vi.cu -- vertical-implicit column solve of the HEVI scheme (cal_vi), FP64.
//
// Restates FElib/src/fluid_dyn_solver/scale_atm_dyn_dgm_nonhydro3d_rhot_hevi.F90:772-965
// with its column operators ..._rhot_hevi_common_2.F90:
//   eval_Ax_uv + solve_uv + construct_matbnd_uv      :482-689, 904-1011, 1016-1168
//   eval_Ax + solve + construct_matbnd               :111-479, 693-901, 1171-1328
//   block LU with partial pivoting of the (3 N1)^2 diagonal blocks
//                                      ..._hevi_common_linalgebra.F90:2296-2445
//
// GB300 mapping: one warp per horizontal-node column (FElib's (i,j) inside an element
// column, all NeZ*N1 levels).  Lane r < 3*N1 owns row r = var + 3*node of the current
// element block in registers; the pivot row is broadcast through shared memory; the
// block-Thomas history (G = D^-1 U and the eliminated right-hand side) and the iterate
// live in the warp's shared-memory slice.  Columns are independent, so there is no
// inter-warp synchronisation at all.
//
// Newton: max_iter == 1 is FElib's single linearised solve from the guess; max_iter > 1
// evaluates the FP64 residual b = impl_fac*A(P) - P + q* before every solve and stops once
// max |b| / scale <= tol (scale: DENS_hyd, DENS_hyd*cref, RHOT_hyd per level).
#include "fedg_common.cuh"
#include "fedg_kernels.cuh"

namespace fedg {

// Warp LU with partial pivoting: lane r < n holds row r of A (a[]) and of the right-hand
// sides (rhs[]).  On return the lane that served as pivot for unknown k holds x_k in rhs[]
// and mypiv == k.  prow: n + nr + 1 doubles of shared scratch; plane: n ints.
template <int n, int nr>
__device__ __forceinline__ void warp_lu(double (&a)[n], double (&rhs)[nr], double* prow, int* plane, int lane,
                                        int& mypiv) {
  bool done = lane >= n;
  mypiv = -1;
#pragma unroll
  for (int k = 0; k < n; ++k) {
    // |a| compared as the integer bit pattern of a non-negative double: no FP64 instructions
    long long bv = done ? -1LL : (__double_as_longlong(a[k]) & 0x7fffffffffffffffLL);
    int best = lane;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const long long ov = __shfl_xor_sync(0xffffffffu, bv, o);
      const int ol = __shfl_xor_sync(0xffffffffu, best, o);
      if (ov > bv || (ov == bv && ol < best)) { bv = ov; best = ol; }
    }
    const bool piv = (lane == best);
    if (piv) {
#pragma unroll
      for (int c = k; c < n; ++c) prow[c] = a[c];
#pragma unroll
      for (int m = 0; m < nr; ++m) prow[n + m] = rhs[m];
      prow[n + nr] = 1.0 / a[k];
      plane[k] = lane;
      mypiv = k;
    }
    __syncwarp();
    if (!done && !piv) {
      const double f = a[k] * prow[n + nr];
#pragma unroll
      for (int c = k + 1; c < n; ++c) a[c] = fma(-f, prow[c], a[c]);
#pragma unroll
      for (int m = 0; m < nr; ++m) rhs[m] = fma(-f, prow[n + m], rhs[m]);
    }
    done = done || piv;
    __syncwarp();
  }
  // column-oriented back substitution on the pivoted upper triangle
#pragma unroll
  for (int k = n - 1; k >= 0; --k) {
    if (mypiv == k) {
      const double rd = 1.0 / a[k];
#pragma unroll
      for (int m = 0; m < nr; ++m) rhs[m] *= rd;
    }
    const int src = plane[k];
#pragma unroll
    for (int m = 0; m < nr; ++m) {
      const double xk = __shfl_sync(0xffffffffu, rhs[m], src);
      if (mypiv >= 0 && mypiv < k) rhs[m] = fma(-a[k], xk, rhs[m]);
    }
  }
  __syncwarp();
}

// Element-block LU of the column Newton solve in FP64: lane r < 3*N1 holds row r (DENS, MOMZ, RHOT
// of node r/3) and its nr right-hand sides.  Pivot order PivOrder<N1> (fedg_common.cuh): the DENS
// columns first, each pivoted on its own DENS row without a search (the DENS block is the identity
// plus the small Lift face terms), then the MOMZ/RHOT columns of the dense Schur complement with
// partial pivoting over the remaining rows.  The pivot search compares |a| as the bit pattern of a
// non-negative double (monotonic as an integer), so it runs on the integer pipes, not on GB300's
// scarce FP64 pipe; only the structurally nonzero columns of a pivot row are broadcast and
// eliminated; each pivot's reciprocal is formed once and kept for the back substitution.
// On return the lane that pivoted step s (plane[s]) holds x of column PivOrder::col(s) in rhs[].
template <int N1, int nr, int s>
__device__ __forceinline__ void lu_d_fwd(double (&a)[3 * N1], double (&rhs)[nr], double* prow, int* plane, int lane,
                                         bool& done, int& mypiv, double& rpiv) {
  constexpr int n = 3 * N1;
  using O = PivOrder<N1>;
  if constexpr (s < n) {
    constexpr int pc = O::col(s);
    int best;
    if constexpr (s < N1) {
      best = 3 * s;
    } else {
      long long bv = done ? -1LL : (__double_as_longlong(a[pc]) & 0x7fffffffffffffffLL);
      best = lane;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const long long ov = __shfl_xor_sync(0xffffffffu, bv, o);
        const int ol = __shfl_xor_sync(0xffffffffu, best, o);
        if (ov > bv || (ov == bv && ol < best)) { bv = ov; best = ol; }
      }
    }
    const bool piv = lane == best;
    if (piv) {
#pragma unroll
      for (int c = 0; c < n; ++c)
        if (O::nz(s, c)) prow[c] = a[c];
#pragma unroll
      for (int m = 0; m < nr; ++m) prow[n + m] = rhs[m];
      rpiv = 1.0 / a[pc];
      prow[n + nr] = rpiv;
      plane[s] = lane;
      mypiv = s;
    }
    __syncwarp();
    if (!done && !piv) {
      const double f = a[pc] * prow[n + nr];
#pragma unroll
      for (int c = 0; c < n; ++c)
        if (O::nz(s, c)) a[c] = fma(-f, prow[c], a[c]);
#pragma unroll
      for (int m = 0; m < nr; ++m) rhs[m] = fma(-f, prow[n + m], rhs[m]);
    }
    done = done || piv;
    __syncwarp();
    lu_d_fwd<N1, nr, s + 1>(a, rhs, prow, plane, lane, done, mypiv, rpiv);
  }
}
template <int N1, int nr, int s>
__device__ __forceinline__ void lu_d_bwd(const double (&a)[3 * N1], double (&rhs)[nr], const int* plane, int mypiv,
                                         double rpiv) {
  using O = PivOrder<N1>;
  if constexpr (s >= 0) {
    constexpr int pc = O::col(s);
    if (mypiv == s) {
#pragma unroll
      for (int m = 0; m < nr; ++m) rhs[m] *= rpiv;
    }
    const int src = plane[s];
#pragma unroll
    for (int m = 0; m < nr; ++m) {
      const double xk = __shfl_sync(0xffffffffu, rhs[m], src);
      if (mypiv >= 0 && mypiv < s) rhs[m] = fma(-a[pc], xk, rhs[m]);
    }
    lu_d_bwd<N1, nr, s - 1>(a, rhs, plane, mypiv, rpiv);
  }
}
template <int N1, int nr>
__device__ __forceinline__ void warp_lu_dfirst(double (&a)[3 * N1], double (&rhs)[nr], double* prow, int* plane,
                                               int lane, int& mypiv) {
  bool done = lane >= 3 * N1;
  double rpiv = 0.0;
  mypiv = -1;
  lu_d_fwd<N1, nr, 0>(a, rhs, prow, plane, lane, done, mypiv, rpiv);
  lu_d_bwd<N1, nr, 3 * N1 - 1>(a, rhs, plane, mypiv, rpiv);
  __syncwarp();
}

template <int N1>
struct ColCtx {
  static constexpr int N = N1 - 1, n3 = 3 * N1, NF = N1 * N1, Np = N1 * N1 * N1;
  const Ops& op;
  const Prof& pf;
  int L, NeZ, lane;
  double *P, *Q, *bh, *Gh, *fr, *fm, *pot, *wt, *dpd, *alB, *alT, *prow;
  int* plane;
};

// per-level linearisation quantities at the iterate P (eval_Ax :236-295)
template <int N1>
__device__ void col_levels(ColCtx<N1>& c) {
  const Ops& op = c.op;
  for (int l = c.lane; l < c.L; l += 32) {
    const double dens = __ldg(c.pf.dens + l) + c.P[3 * l + 0];
    const double rhot = __ldg(c.pf.rhyd + l) + c.P[3 * l + 2];
    const double pot = rhot / dens;
    const double pr = op.pres00 * pow(op.rdry / op.pres00 * rhot, op.kap);
    c.pot[l] = pot;
    c.fm[l] = pr - __ldg(c.pf.pres + l);
    c.fr[l] = pot * c.P[3 * l + 1];
    c.wt[l] = c.P[3 * l + 1] / dens;
    c.dpd[l] = op.kap * pr / rhot;
  }
  __syncwarp();
}

// vertical face flux of element ez for variable v (vi_cal_del_flux_dyn :1294-1323)
template <int N1>
__device__ __forceinline__ void col_face(const ColCtx<N1>& c, int ez, int v, double& dB, double& dT) {
  constexpr int N = N1 - 1;
  const double tmp1 = 0.5 * c.op.FSz;
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    const int lM = ez * N1 + (s == 0 ? 0 : N);
    const bool lid = s == 0 ? (ez == 0) : (ez == c.NeZ - 1);
    const int lP = lid ? lM : (s == 0 ? lM - 1 : lM + 1);
    const double nz = s == 0 ? -1.0 : 1.0;
    const double al = s == 0 ? c.alB[ez] : c.alT[ez];
    const double mzM = c.P[3 * lM + 1];
    const double mzP = lid ? -mzM : c.P[3 * lP + 1];
    double r;
    if (v == 0) r = tmp1 * ((mzP - mzM) * nz - al * (c.P[3 * lP] - c.P[3 * lM]));
    else if (v == 1) r = tmp1 * ((c.fm[lP] - c.fm[lM]) * nz - al * (mzP - mzM));
    else r = tmp1 * ((c.pot[lP] * mzP - c.pot[lM] * mzM) * nz - al * (c.P[3 * lP + 2] - c.P[3 * lM + 2]));
    if (s == 0) dB = r; else dT = r;
  }
}

// residual (or the operator A itself when want_A) for every level -> bh; returns the
// warp-wide max of the scaled residual
template <int N1>
__device__ double col_residual(ColCtx<N1>& c, double impl_fac, double cref, bool want_A) {
  constexpr int n3 = 3 * N1;
  const Ops& op = c.op;
  col_levels<N1>(c);
  double err = 0.0;
  for (int ez = 0; ez < c.NeZ; ++ez) {
    if (c.lane < n3) {
      const int v = c.lane % 3, pv = c.lane / 3;
      const int l = ez * N1 + pv;
      double dB, dT;
      col_face<N1>(c, ez, v, dB, dT);
      double sz = 0.0, drho = 0.0;
#pragma unroll
      for (int m = 0; m < N1; ++m) {
        const int lm = ez * N1 + m;
        const double fx = v == 0 ? c.P[3 * lm + 1] : (v == 1 ? c.fm[lm] : c.fr[lm]);
        sz = fma(op.D[pv * N1 + m], fx, sz);
        drho = fma(op.T[pv * N1 + m], c.P[3 * lm], drho);
      }
      double A = -(op.E33 * sz + op.Lb[pv] * dB + op.Lt[pv] * dT);
      if (v == 1) A -= op.grav * drho;
      double b;
      if (want_A) {
        b = A;
      } else {
        b = impl_fac * A - c.P[3 * l + v] + c.Q[3 * l + v];
        const double sc = v == 0 ? __ldg(c.pf.dens + l) : (v == 1 ? __ldg(c.pf.dens + l) * cref : __ldg(c.pf.rhyd + l));
        err = fmax(err, fabs(b) / sc);
        if (!(fabs(b) < 1e300)) err = __longlong_as_double(0x7ff8000000000000LL);  // NaN propagates
      }
      c.bh[3 * l + v] = b;
    }
  }
  __syncwarp();
  double e = err;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double oe = __shfl_xor_sync(0xffffffffu, e, o);
    e = (e != e || oe != oe) ? __longlong_as_double(0x7ff8000000000000LL) : fmax(e, oe);
  }
  return e;
}

// one linearised solve (construct_matbnd + block-Thomas + LU), result added to P
template <int N1>
__device__ void col_solve(ColCtx<N1>& c, double impl_fac) {
  constexpr int N = N1 - 1, n3 = 3 * N1;
  const Ops& op = c.op;
  const int lane = c.lane;
  const int v = lane % 3, pv = lane / 3;
  const bool act = lane < n3;
  for (int ez = 0; ez < c.NeZ; ++ez) {
    double a[n3];
    double rhs[4];
    double Lc[3] = {0.0, 0.0, 0.0}, Uc[3] = {0.0, 0.0, 0.0};
    const int pvr = act ? pv : 0;
#pragma unroll
    for (int cc = 0; cc < n3; ++cc) {
      const int v2 = cc % 3, pv2 = cc / 3;
      const int l2 = ez * N1 + pv2;
      const double fdz = op.E33 * impl_fac * op.D[pvr * N1 + pv2];
      const double id = (pvr == pv2) ? 1.0 : 0.0;
      double x;
      if (v == 0) x = v2 == 0 ? id : (v2 == 1 ? fdz : 0.0);
      else if (v == 1) x = v2 == 1 ? id : (v2 == 0 ? impl_fac * op.grav * op.T[pvr * N1 + pv2] : fdz * c.dpd[l2]);
      else x = v2 == 0 ? -fdz * c.pot[l2] * c.wt[l2] : (v2 == 1 ? fdz * c.pot[l2] : id + fdz * c.wt[l2]);
      a[cc] = x;
    }
#pragma unroll
    for (int f = 0; f < 2; ++f) {
      const bool bc = (f == 0) ? (ez == 0) : (ez == c.NeZ - 1);
      constexpr int dummy = 0; (void)dummy;
      const int pv1 = f == 0 ? 0 : N;
      const int l1 = ez * N1 + pv1;
      const int ln = bc ? l1 : (f == 0 ? l1 - 1 : l1 + 1);
      const double nz = f == 0 ? -1.0 : 1.0;
      const double al = f == 0 ? c.alB[ez] : c.alT[ez];
      const double fac = 0.5 * impl_fac * (f == 0 ? op.Lb[pvr] : op.Lt[pvr]) * op.FSz;
      const double tmp1 = fac * al, tmp2 = fac * nz;
      const double potw = c.pot[l1] * c.wt[l1];
      const int c0 = 3 * (f == 0 ? 0 : N);  // first column of node pv1
      if (bc) {
        if (v == 2) a[c0 + 0] += 2.0 * tmp2 * potw;
        if (v == 0) a[c0 + 1] -= 2.0 * tmp2;
        if (v == 1) a[c0 + 1] += 2.0 * tmp1;
        if (v == 2) a[c0 + 1] -= 2.0 * tmp2 * c.pot[l1];
        if (v == 2) a[c0 + 2] -= 2.0 * tmp2 * c.wt[l1];
      } else {
        if (v == 0) a[c0 + 0] += tmp1;
        if (v == 2) a[c0 + 0] += tmp2 * potw;
        if (v == 0) a[c0 + 1] -= tmp2;
        if (v == 1) a[c0 + 1] += tmp1;
        if (v == 2) a[c0 + 1] -= tmp2 * c.pot[l1];
        if (v == 1) a[c0 + 2] -= tmp2 * c.dpd[l1];
        if (v == 2) a[c0 + 2] += tmp1 - tmp2 * c.wt[l1];
        double cc0, cc1, cc2;
        if (v == 0) { cc0 = -tmp1; cc1 = tmp2; cc2 = 0.0; }
        else if (v == 1) { cc0 = 0.0; cc1 = -tmp1; cc2 = tmp2 * c.dpd[ln]; }
        else { cc0 = -tmp2 * c.pot[ln] * c.wt[ln]; cc1 = tmp2 * c.pot[ln]; cc2 = -tmp1 + tmp2 * c.wt[ln]; }
        if (f == 0) { Lc[0] = cc0; Lc[1] = cc1; Lc[2] = cc2; }
        else { Uc[0] = cc0; Uc[1] = cc1; Uc[2] = cc2; }
      }
    }
    rhs[0] = act ? c.bh[ez * n3 + lane] : 0.0;
    if (ez > 0) {
      const double* Gp = c.Gh + ((ez - 1) * n3 + 3 * N) * 3;
      const double* bp = c.bh + (ez - 1) * n3 + 3 * N;
#pragma unroll
      for (int c2 = 0; c2 < 3; ++c2)
        a[c2] -= Lc[0] * Gp[0 * 3 + c2] + Lc[1] * Gp[1 * 3 + c2] + Lc[2] * Gp[2 * 3 + c2];
      rhs[0] -= Lc[0] * bp[0] + Lc[1] * bp[1] + Lc[2] * bp[2];
    }
    const bool last = ez == c.NeZ - 1;
    rhs[1] = last ? 0.0 : Uc[0];
    rhs[2] = last ? 0.0 : Uc[1];
    rhs[3] = last ? 0.0 : Uc[2];
    if (!act) {
#pragma unroll
      for (int cc = 0; cc < n3; ++cc) a[cc] = 0.0;
    }
    __syncwarp();
    int mypiv;
    warp_lu_dfirst<N1, 4>(a, rhs, c.prow, c.plane, lane, mypiv);
    if (mypiv >= 0) {
      const int xc = PivOrder<N1>::col(mypiv);  // the unknown this lane solved for
      c.bh[ez * n3 + xc] = rhs[0];
      c.Gh[(ez * n3 + xc) * 3 + 0] = rhs[1];
      c.Gh[(ez * n3 + xc) * 3 + 1] = rhs[2];
      c.Gh[(ez * n3 + xc) * 3 + 2] = rhs[3];
    }
    __syncwarp();
  }
  // block back substitution (common_2.F90:443-458)
  for (int ez = c.NeZ - 2; ez >= 0; --ez) {
    if (act) {
      const double* bn = c.bh + (ez + 1) * n3;
      const double* G = c.Gh + (ez * n3 + lane) * 3;
      c.bh[ez * n3 + lane] -= G[0] * bn[0] + G[1] * bn[1] + G[2] * bn[2];
    }
    __syncwarp();
  }
  for (int idx = lane; idx < 3 * c.L; idx += 32) c.P[idx] += c.bh[idx];
  __syncwarp();
}

template <int N1>
__global__ void __launch_bounds__(128) k_vi_fp64(const Ops op, const Prof pf, const F5c qin, const F5c z,
                                                  const F5c guess, const F5 qout, const F5 tout, int* status,
                                                  const ViArgs args, int ncol, int per_warp) {
  constexpr int N = N1 - 1, n3 = 3 * N1, NF = N1 * N1, Np = N1 * N1 * N1;
  extern __shared__ double sm[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int col = blockIdx.x * (blockDim.x >> 5) + wib;
  if (col >= ncol) return;  // uniform per warp
  const int L = op.L, NeZ = op.NeZ;
  double* W = sm + (size_t)wib * per_warp;
  ColCtx<N1> c{op, pf};
  c.L = L; c.NeZ = NeZ; c.lane = lane;
  c.P = W; c.Q = c.P + 3 * L; c.bh = c.Q + 3 * L; c.Gh = c.bh + 3 * L;
  c.fr = c.Gh + 9 * L; c.fm = c.fr + L; c.pot = c.fm + L; c.wt = c.pot + L; c.dpd = c.wt + L;
  c.alB = c.dpd + L; c.alT = c.alB + NeZ; c.prow = c.alT + NeZ;
  c.plane = reinterpret_cast<int*>(c.prow + n3 + 8);
  const int ij = col % NF, exy = col / NF;
  const int ci = ij % N1, cj = ij / N1;
  const size_t nxy = (size_t)op.NeX * op.NeY;
  auto gidx = [&](int l) -> size_t {
    const int ez = l / N1, k = l - ez * N1;
    return ((size_t)ez * nxy + exy) * Np + ci + N1 * cj + NF * k;
  };
  const int gv[3] = {VD, VMZ, VRT};
  const double impl_fac = args.impl_fac;

  // --- load q*, the iterate (guess or var0), and alph from var0 (eval_Ax_uv :1149-1155) ---
  for (int l = lane; l < L; l += 32) {
    const size_t g = gidx(l);
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      c.Q[3 * l + m] = __ldg(qin.v[gv[m]] + g);
      c.P[3 * l + m] = guess.v[0] ? __ldg(guess.v[gv[m]] + g) : __ldg(z.v[gv[m]] + g);
    }
    // sound speed + |w| of var0 -> fr (temporary)
    const double rdens0 = 1.0 / (__ldg(pf.dens + l) + __ldg(z.v[VD] + g));
    const double wt0 = __ldg(z.v[VMZ] + g) * rdens0;
    const double pres0 = op.pres00 * pow(op.rdry / op.pres00 * (__ldg(pf.rhyd + l) + __ldg(z.v[VRT] + g)), op.kap);
    c.fr[l] = fabs(wt0) + sqrt(op.kap * pres0 * rdens0);
  }
  __syncwarp();
  for (int ez = lane; ez < NeZ; ez += 32) {
    const int lb = ez * N1, lt = ez * N1 + N;
    c.alB[ez] = fmax(c.fr[lb], c.fr[ez > 0 ? lb - 1 : lb]);
    c.alT[ez] = fmax(c.fr[lt], c.fr[ez < NeZ - 1 ? lt + 1 : lt]);
  }
  __syncwarp();

  // --- MOMX/MOMY: the linear vertical-dissipation system (eval_Ax_uv + solve_uv) ---
  {
    double* Pu = c.Gh;          // [2L]
    double* Qu = Pu + 2 * L;    // [2L]
    double* bu = Qu + 2 * L;    // [2L]
    double* Gu = bu + 2 * L;    // [L]
    for (int l = lane; l < L; l += 32) {
      const size_t g = gidx(l);
      Pu[2 * l + 0] = __ldg(z.v[VMX] + g);
      Pu[2 * l + 1] = __ldg(z.v[VMY] + g);
      Qu[2 * l + 0] = __ldg(qin.v[VMX] + g);
      Qu[2 * l + 1] = __ldg(qin.v[VMY] + g);
    }
    __syncwarp();
    const double tm = -0.5 * op.FSz;
    if (impl_fac == 0.0) {
      for (int l = lane; l < L; l += 32) {
        const int ez = l / N1, pv = l - ez * N1;
        const int lb = ez * N1, lt = ez * N1 + N;
        const int lbP = ez > 0 ? lb - 1 : lb, ltP = ez < NeZ - 1 ? lt + 1 : lt;
        const double dBx = tm * c.alB[ez] * (Pu[2 * lbP] - Pu[2 * lb]), dTx = tm * c.alT[ez] * (Pu[2 * ltP] - Pu[2 * lt]);
        const double dBy = tm * c.alB[ez] * (Pu[2 * lbP + 1] - Pu[2 * lb + 1]),
                     dTy = tm * c.alT[ez] * (Pu[2 * ltP + 1] - Pu[2 * lt + 1]);
        const size_t g = gidx(l);
        if (tout.v[0]) {
          tout.v[VMX][g] = -(op.Lb[pv] * dBx + op.Lt[pv] * dTx);
          tout.v[VMY][g] = -(op.Lb[pv] * dBy + op.Lt[pv] * dTy);
        }
        if (qout.v[0]) { qout.v[VMX][g] = Qu[2 * l]; qout.v[VMY][g] = Qu[2 * l + 1]; }
      }
    } else {
      // The element blocks are the identity plus the Lift face terms in columns 0 and N, coupled to
      // the neighbours only through those, so the system reduces exactly to a scalar tridiagonal
      // system in the interface jumps J_e = d(e, 0) - d(e-1, N), e = 1 .. NeZ-1 (J_0 = J_NeZ = 0 at the
      // slip lids):  (1 + beta(e, 0) + tau(e-1, N)) J_e - beta(e-1, N) J_{e-1} - tau(e, 0) J_{e+1}
      //            = b(e, 0) - b(e-1, N),  beta(e, p) = impl_fac Fz Lb[p] alB_e / 2, tau with Lt, alT,
      // and then d(e, p) = b(e, p) - beta(e, p) J_e + tau(e, p) J_{e+1}: the same linear solve as the
      // per-element LU of solve_Nnode8_uv (hevi_common_linalgebra.F90:2142-2294), in O(NeZ).
      for (int l = lane; l < L; l += 32) {  // b = impl_fac A_uv(P) - P + q*
        const int ez = l / N1, pv = l - ez * N1;
        const int lb = ez * N1, lt = ez * N1 + N;
        const int lbP = ez > 0 ? lb - 1 : lb, ltP = ez < NeZ - 1 ? lt + 1 : lt;
        const double dBx = tm * c.alB[ez] * (Pu[2 * lbP] - Pu[2 * lb]), dTx = tm * c.alT[ez] * (Pu[2 * ltP] - Pu[2 * lt]);
        const double dBy = tm * c.alB[ez] * (Pu[2 * lbP + 1] - Pu[2 * lb + 1]),
                     dTy = tm * c.alT[ez] * (Pu[2 * ltP + 1] - Pu[2 * lt + 1]);
        bu[2 * l] = impl_fac * (-(op.Lb[pv] * dBx + op.Lt[pv] * dTx)) - Pu[2 * l] + Qu[2 * l];
        bu[2 * l + 1] = impl_fac * (-(op.Lb[pv] * dBy + op.Lt[pv] * dTy)) - Pu[2 * l + 1] + Qu[2 * l + 1];
      }
      __syncwarp();
      const double cfs = 0.5 * impl_fac * op.FSz;
      double* J = Gu;  // [2][NeZ + 1]: the jumps of MOMX and MOMY
      if (lane < 2) {  // one Thomas sweep per momentum component
        const int m = lane;
        double* Jm = J + m * (NeZ + 1);
        double cprev = 0.0, rprev = 0.0;
        Jm[0] = 0.0;
        Jm[NeZ] = 0.0;
        for (int e = 1; e < NeZ; ++e) {
          const double aa = e >= 2 ? -cfs * op.Lb[N] * c.alB[e - 1] : 0.0;
          const double dd = 1.0 + cfs * op.Lb[0] * c.alB[e] + cfs * op.Lt[N] * c.alT[e - 1];
          const double cc = e < NeZ - 1 ? -cfs * op.Lt[0] * c.alT[e] : 0.0;
          const double ip = 1.0 / (dd - aa * cprev);
          const double rr = bu[2 * (e * N1) + m] - bu[2 * ((e - 1) * N1 + N) + m];
          cprev = cc * ip;
          rprev = (rr - aa * rprev) * ip;
          Jm[e] = rprev;
          // forward coefficients kept in the jump slots' neighbours: store c' beside J
          Gu[2 * (NeZ + 1) + m * (NeZ + 1) + e] = cprev;
        }
        for (int e = NeZ - 2; e >= 1; --e) Jm[e] -= Gu[2 * (NeZ + 1) + m * (NeZ + 1) + e] * Jm[e + 1];
      }
      __syncwarp();
      for (int l = lane; l < L; l += 32) {
        const int ez = l / N1, pv = l - ez * N1;
        const double beta = ez > 0 ? cfs * op.Lb[pv] * c.alB[ez] : 0.0;
        const double tau = ez < NeZ - 1 ? cfs * op.Lt[pv] * c.alT[ez] : 0.0;
#pragma unroll
        for (int m = 0; m < 2; ++m) {
          const double* Jm = J + m * (NeZ + 1);
          bu[2 * l + m] = bu[2 * l + m] - beta * Jm[ez] + tau * Jm[ez + 1];
        }
      }
      __syncwarp();
      for (int l = lane; l < L; l += 32) {
        const double px = Pu[2 * l] + bu[2 * l], py = Pu[2 * l + 1] + bu[2 * l + 1];
        const size_t g = gidx(l);
        if (qout.v[0]) { qout.v[VMX][g] = px; qout.v[VMY][g] = py; }
        if (tout.v[0]) {
          tout.v[VMX][g] = (px - Qu[2 * l]) / impl_fac;
          tout.v[VMY][g] = (py - Qu[2 * l + 1]) / impl_fac;
        }
      }
    }
    __syncwarp();
  }

  // --- DENS/MOMZ/RHOT: Newton on G(P) = P - q* - impl_fac A(P) ---
  int st;
  if (impl_fac == 0.0) {
    col_residual<N1>(c, 0.0, args.cref, true);
    for (int l = lane; l < L; l += 32) {
      const size_t g = gidx(l);
#pragma unroll
      for (int m = 0; m < 3; ++m) {
        if (tout.v[0]) tout.v[gv[m]][g] = c.bh[3 * l + m];
        if (qout.v[0]) qout.v[gv[m]][g] = c.Q[3 * l + m];
      }
    }
    st = 0;
  } else {
    int nsolve = 0;
    while (true) {
      const double err = col_residual<N1>(c, impl_fac, args.cref, false);
      if (err != err) { st = -2; break; }
      if (args.max_iter > 1 && err <= args.tol) { st = nsolve; break; }
      if (nsolve >= args.max_iter) { st = -1; break; }
      col_solve<N1>(c, impl_fac);
      ++nsolve;
      if (args.max_iter == 1) { st = 1; break; }
    }
    for (int l = lane; l < L; l += 32) {
      const size_t g = gidx(l);
#pragma unroll
      for (int m = 0; m < 3; ++m) {
        const double pnew = c.P[3 * l + m];
        if (qout.v[0]) qout.v[gv[m]][g] = pnew;
        if (tout.v[0]) tout.v[gv[m]][g] = (pnew - c.Q[3 * l + m]) / impl_fac;
      }
    }
  }
  if (lane == 0 && status) status[col] = st;
}

template <int N1>
static int launch_vi_n(const Ops& op, const Prof& pf, const F5c& qin, const F5c& z, const F5c& guess,
                       const F5& qout, const F5& tout, int* status, const ViArgs& a, cudaStream_t s) {
  constexpr int n3 = 3 * N1;
  const int L = op.L;
  const int per_warp = 23 * L + 2 * op.NeZ + n3 + 8 + (n3 + 1) / 2 + 1;  // doubles
  const int ncol = op.NeX * op.NeY * N1 * N1;
  int wpb = 4;
  size_t smem = sizeof(double) * (size_t)per_warp * wpb;
  while (wpb > 1 && smem > 200 * 1024) { wpb >>= 1; smem = sizeof(double) * (size_t)per_warp * wpb; }
  if (smem > 227 * 1024) return (int)cudaErrorInvalidValue;
  auto kfn = k_vi_fp64<N1>;
  cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  kfn<<<(ncol + wpb - 1) / wpb, 32 * wpb, smem, s>>>(op, pf, qin, z, guess, qout, tout, status, a, ncol, per_warp);
  return (int)cudaGetLastError();
}

int launch_vi_fp64(const Ops& op, const Prof& pf, const F5c& qin, const F5c& z, const F5c& guess, const F5& qout,
                   const F5& tout, int* status, const ViArgs& a, cudaStream_t s) {
  switch (op.N1) {
    case 2: return launch_vi_n<2>(op, pf, qin, z, guess, qout, tout, status, a, s);
    case 3: return launch_vi_n<3>(op, pf, qin, z, guess, qout, tout, status, a, s);
    case 4: return launch_vi_n<4>(op, pf, qin, z, guess, qout, tout, status, a, s);
    case 5: return launch_vi_n<5>(op, pf, qin, z, guess, qout, tout, status, a, s);
    case 6: return launch_vi_n<6>(op, pf, qin, z, guess, qout, tout, status, a, s);
    case 7: return launch_vi_n<7>(op, pf, qin, z, guess, qout, tout, status, a, s);
    case 8: return launch_vi_n<8>(op, pf, qin, z, guess, qout, tout, status, a, s);
  }
  return (int)cudaErrorInvalidValue;
}

}  // namespace fedg
