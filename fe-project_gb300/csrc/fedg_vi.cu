// fedg_vi.cu -- vertical-implicit column solve of the HEVI scheme (cal_vi), FP64.
//
// Restates FElib/src/fluid_dyn_solver/scale_atm_dyn_dgm_nonhydro3d_rhot_hevi.F90:772-965
// with its column operators ..._rhot_hevi_common_2.F90:
//   eval_Ax_uv + solve_uv + construct_matbnd_uv      :482-689, 904-1011, 1016-1168
//   eval_Ax + solve + construct_matbnd               :111-479, 693-901, 1171-1328
//   block LU with partial pivoting of the (3 N1)^2 diagonal blocks
//                                      ..._hevi_common_linalgebra.F90:2296-2445
//
// GB300 mapping: two horizontal-node columns per warp (FElib's (i,j) inside an element column, all
// NeZ*N1 levels), one per half-warp.  The kernel is bound by GB300's FP64 pipe, which spends the same
// cycles on a warp instruction whatever its active lanes, so the layout is chosen to keep lanes busy.
// Of the 3*N1 rows of an element block, the N1 DENS rows are the identity plus Lift face terms in the
// DENS columns: they are pivoted first, each on its own row (no search), and after the first step they
// eliminate nothing from one another.  The 2*N1 MOMZ/RHOT rows form the dense Schur complement that is
// pivoted with a search.  Lane hl of a half therefore holds the MOMZ (hl even) or RHOT (hl odd) row of
// node hl/2 and, for hl < N1, the DENS row of node hl as a second register row: the Schur phase runs
// on all 32 lanes (one column per warp left half of them idle there), and the DENS rows cost FP64
// instructions only where they have nonzeros.  Pivot rows are broadcast through the half's shared-memory
// slice; the iterate and the per-level linearisation quantities live in shared memory; the block-Thomas
// history (G = D^-1 U) lives in a global scratch slice of the warp, which a persistent grid keeps small
// enough to stay in L2.  Columns are independent: no synchronisation beyond the warp.
//
// Newton: max_iter == 1 is FElib's single linearised solve from the guess; max_iter > 1
// evaluates the FP64 residual b = impl_fac*A(P) - P + q* before every solve and stops once
// max |b| / scale <= tol (scale: DENS_hyd, DENS_hyd*cref, RHOT_hyd per level).  The two columns of a
// warp iterate together; a converged column skips its corrections until the other one is done.
#include "fedg_common.cuh"
#include "fedg_kernels.cuh"

namespace fedg {

// One half-warp's rows of an element block: the Schur row (MOMZ or RHOT of node hl/2) and, for
// hl < N1, the DENS row of node hl, each with its 4 right-hand sides (the residual and the three
// columns of the coupling to the next element).
template <int N1>
struct BlockRows {
  double aS[3 * N1], aD[3 * N1];
  double rS[4], rD[4];
  double rpS = 0.0, rpD = 0.0;  // reciprocal of the row's pivot
  int pvS = -1;                 // pivot step of the Schur row (-1: not yet a pivot row)
  bool doneS = false;
};

// Forward elimination of the element block in PivOrder<N1> (fedg_common.cuh): steps s < N1 pivot the
// DENS column of node s on the DENS row of node s; steps s >= N1 pivot the MOMZ/RHOT columns with
// partial pivoting over the remaining Schur rows, comparing |a| as the bit pattern of a non-negative
// double (monotonic as an integer, so the search runs on the integer pipes) and breaking ties toward
// the lower row.  Only the structurally nonzero columns of a pivot row are broadcast and eliminated.
// The DENS rows hold nonzeros only in their own DENS column, the DENS columns of the face nodes 0 and
// N, the MOMZ columns and the RHOT column of node 0, so they take part only in step 0 (column 0).
template <int N1, int s>
__device__ __forceinline__ void blk_fwd(BlockRows<N1>& R, double* prow, int* plane, int hl, bool actS, bool actD) {
  constexpr int n = 3 * N1;
  using O = PivOrder<N1>;
  if constexpr (s < n) {
    constexpr int pc = O::col(s);
    if constexpr (s < N1) {
      if (hl == s) {
#pragma unroll
        for (int c = 0; c < n; ++c)
          if (O::nz(s, c)) prow[c] = R.aD[c];
#pragma unroll
        for (int m = 0; m < 4; ++m) prow[n + m] = R.rD[m];
        if constexpr (s == 0) R.rpD = 1.0 / R.aD[pc];  // the others were formed after step 0
        prow[n + 4] = R.rpD;
      }
      __syncwarp();
      if (actS) {
        const double f = R.aS[pc] * prow[n + 4];
#pragma unroll
        for (int c = 0; c < n; ++c)
          if (O::nz(s, c)) R.aS[c] = fma(-f, prow[c], R.aS[c]);
#pragma unroll
        for (int m = 0; m < 4; ++m) R.rS[m] = fma(-f, prow[n + m], R.rS[m]);
      }
      if constexpr (s == 0) {
        if (actD && hl > 0) {
          const double f = R.aD[pc] * prow[n + 4];
#pragma unroll
          for (int c = 0; c < n; ++c)
            if (O::nz(s, c)) R.aD[c] = fma(-f, prow[c], R.aD[c]);
#pragma unroll
          for (int m = 0; m < 4; ++m) R.rD[m] = fma(-f, prow[n + m], R.rD[m]);
          // the DENS rows are final from here on: the reciprocals of their pivots all at once
          double d = R.aD[3];
#pragma unroll
          for (int k = 2; k < N1; ++k)
            if (hl == k) d = R.aD[3 * k];
          R.rpD = 1.0 / d;
        }
      }
      __syncwarp();
    } else {
      long long bv = (actS && !R.doneS) ? (__double_as_longlong(R.aS[pc]) & 0x7fffffffffffffffLL) : -1LL;
      int best = hl;
#pragma unroll
      for (int o = 8; o > 0; o >>= 1) {  // within the half-warp
        const long long ov = __shfl_xor_sync(0xffffffffu, bv, o);
        const int ol = __shfl_xor_sync(0xffffffffu, best, o);
        if (ov > bv || (ov == bv && ol < best)) { bv = ov; best = ol; }
      }
      const bool piv = hl == best;
      if (piv) {
#pragma unroll
        for (int c = 0; c < n; ++c)
          if (O::nz(s, c)) prow[c] = R.aS[c];
#pragma unroll
        for (int m = 0; m < 4; ++m) prow[n + m] = R.rS[m];
        R.rpS = 1.0 / R.aS[pc];
        prow[n + 4] = R.rpS;
        plane[s] = hl;
        R.pvS = s;
      }
      __syncwarp();
      if (actS && !R.doneS && !piv) {
        const double f = R.aS[pc] * prow[n + 4];
#pragma unroll
        for (int c = 0; c < n; ++c)
          if (O::nz(s, c)) R.aS[c] = fma(-f, prow[c], R.aS[c]);
#pragma unroll
        for (int m = 0; m < 4; ++m) R.rS[m] = fma(-f, prow[n + m], R.rS[m]);
      }
      R.doneS = R.doneS || piv;
      __syncwarp();
    }
    blk_fwd<N1, s + 1>(R, prow, plane, hl, actS, actD);
  }
}

// Column-oriented back substitution on the pivoted upper triangle.  On return the Schur row that
// pivoted step s holds x of column PivOrder::col(s) in rS[], the DENS row of node hl x of column 3 hl
// in rD[].
template <int N1, int s>
__device__ __forceinline__ void blk_bwd(BlockRows<N1>& R, const int* plane, int hl, int hbase, bool actD) {
  using O = PivOrder<N1>;
  if constexpr (s >= 0) {
    constexpr int pc = O::col(s);
    if constexpr (s >= N1) {
      if (R.pvS == s) {
#pragma unroll
        for (int m = 0; m < 4; ++m) R.rS[m] *= R.rpS;
      }
      const int src = hbase + plane[s];
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        const double xk = __shfl_sync(0xffffffffu, R.rS[m], src);
        if (R.pvS >= 0 && R.pvS < s) R.rS[m] = fma(-R.aS[pc], xk, R.rS[m]);
        if constexpr (pc % 3 == 1 || pc == 2) {
          if (actD) R.rD[m] = fma(-R.aD[pc], xk, R.rD[m]);
        }
      }
    } else if constexpr (s == N1 - 1) {
      // Among the DENS unknowns only the top node's (column 3N) enters the other DENS rows; after its
      // update every DENS row is final and is scaled by its pivot's reciprocal here, at once.
      if (hl == s) {
#pragma unroll
        for (int m = 0; m < 4; ++m) R.rD[m] *= R.rpD;
      }
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        const double xk = __shfl_sync(0xffffffffu, R.rD[m], hbase + s);
        if (hl < s) R.rD[m] = fma(-R.aD[pc], xk, R.rD[m]);
      }
      if (hl < s) {
#pragma unroll
        for (int m = 0; m < 4; ++m) R.rD[m] *= R.rpD;
      }
    }
    blk_bwd<N1, s - 1>(R, plane, hl, hbase, actD);
  }
}

template <int N1>
struct ColCtx {
  static constexpr int N = N1 - 1, n3 = 3 * N1, NF = N1 * N1, Np = N1 * N1 * N1;
  const Ops& op;
  const Prof& pf;
  const F5c& qin;
  int L, NeZ, hl, hbase;
  size_t gxy, nxyNp;  // node offset of the column in an element layer; nodes per element layer
  double *P, *bh, *fr, *fm, *pot, *wt, *dpd, *alB, *alT, *J, *prow;
  double* G;  // block-Thomas history [NeZ][3 N1][3] (global scratch)
  int* plane;
  __device__ __forceinline__ size_t g(int l) const {
    const int ez = l / N1, k = l - ez * N1;
    return (size_t)ez * nxyNp + gxy + (size_t)NF * k;
  }
};

// per-level linearisation quantities at the iterate P (eval_Ax :236-295)
template <int N1>
__device__ __forceinline__ void col_levels(ColCtx<N1>& c) {
  const Ops& op = c.op;
  for (int l = c.hl; l < c.L; l += 16) {
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

// field v (0 DENS, 1 MOMZ, 2 RHOT) of the var3 part, selected without indexing the parameter array
__device__ __forceinline__ const double* var3_field(const F5c& f, int v) {
  return v == 0 ? f.v[VD] : (v == 1 ? f.v[VMZ] : f.v[VRT]);
}

// residual (or the operator A itself when want_A) for every level -> bh; returns the half-warp's
// max of the scaled residual (NaN when any entry is not finite)
template <int N1>
__device__ __forceinline__ double col_residual(ColCtx<N1>& c, double impl_fac, double cref, bool want_A) {
  constexpr int n3 = 3 * N1;
  const Ops& op = c.op;
  col_levels<N1>(c);
  double err = 0.0;
  bool bad = false;
  for (int i = c.hl; i < c.NeZ * n3; i += 16) {
    const int ez = i / n3, r = i - ez * n3;
    const int v = r % 3, pv = r / 3;
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
      b = impl_fac * A - c.P[3 * l + v] + __ldg(var3_field(c.qin, v) + c.g(l));
      const double sc = v == 0 ? __ldg(c.pf.dens + l) : (v == 1 ? __ldg(c.pf.dens + l) * cref : __ldg(c.pf.rhyd + l));
      err = fmax(err, fabs(b) / sc);
      bad = bad || !(fabs(b) < 1e300);
    }
    c.bh[3 * l + v] = b;
  }
  __syncwarp();
  double e = bad ? __longlong_as_double(0x7ff8000000000000LL) : err;
#pragma unroll
  for (int o = 8; o > 0; o >>= 1) {
    const double oe = __shfl_xor_sync(0xffffffffu, e, o);
    e = (e != e || oe != oe) ? __longlong_as_double(0x7ff8000000000000LL) : fmax(e, oe);
  }
  return e;
}

// Row (v, pvr) of the element block of ez (construct_matbnd :1171-1328): the diagonal block in a[],
// the coupling to the element below (Lc) and above (Uc) in the three unknowns of the face node.
// DENS: v == 0 known at compile time.
template <int N1, bool DENS>
__device__ __forceinline__ void blk_row(const ColCtx<N1>& c, int ez, int v_rt, int pvr, double impl_fac,
                                        double (&a)[3 * N1], double (&Lc)[3], double (&Uc)[3]) {
  constexpr int N = N1 - 1, n3 = 3 * N1;
  const Ops& op = c.op;
  const int v = DENS ? 0 : v_rt;
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
  for (int m = 0; m < 3; ++m) { Lc[m] = 0.0; Uc[m] = 0.0; }
#pragma unroll
  for (int f = 0; f < 2; ++f) {
    const bool bc = (f == 0) ? (ez == 0) : (ez == c.NeZ - 1);
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
}

// the coupling to the element below through its eliminated face-node rows: a -= Lc G, rhs -= Lc b
template <int N1>
__device__ __forceinline__ void blk_couple(const ColCtx<N1>& c, int ez, const double (&Lc)[3], double (&a)[3 * N1],
                                           double& rhs) {
  constexpr int N = N1 - 1, n3 = 3 * N1;
  const double* Gp = c.G + ((ez - 1) * n3 + 3 * N) * 3;
  const double* bp = c.bh + (ez - 1) * n3 + 3 * N;
#pragma unroll
  for (int c2 = 0; c2 < 3; ++c2)
    a[c2] -= Lc[0] * Gp[0 * 3 + c2] + Lc[1] * Gp[1 * 3 + c2] + Lc[2] * Gp[2 * 3 + c2];
  rhs -= Lc[0] * bp[0] + Lc[1] * bp[1] + Lc[2] * bp[2];
}

// one linearised solve (construct_matbnd + block-Thomas + LU), result added to P when apply
template <int N1>
__device__ __forceinline__ void col_solve(ColCtx<N1>& c, double impl_fac, bool apply) {
  constexpr int n3 = 3 * N1;
  const int hl = c.hl;
  const bool actS = hl < 2 * N1, actD = hl < N1;
  const int vS = 1 + (hl & 1), pvS = actS ? (hl >> 1) : 0, pvD = actD ? hl : 0;
  const int rS = 3 * pvS + vS, rD = 3 * pvD;
  for (int ez = 0; ez < c.NeZ; ++ez) {
    BlockRows<N1> R;
    double LcS[3], UcS[3], LcD[3], UcD[3];
    blk_row<N1, false>(c, ez, vS, pvS, impl_fac, R.aS, LcS, UcS);
    blk_row<N1, true>(c, ez, 0, pvD, impl_fac, R.aD, LcD, UcD);
    R.rS[0] = actS ? c.bh[ez * n3 + rS] : 0.0;
    R.rD[0] = actD ? c.bh[ez * n3 + rD] : 0.0;
    if (ez > 0) {
      blk_couple<N1>(c, ez, LcS, R.aS, R.rS[0]);
      blk_couple<N1>(c, ez, LcD, R.aD, R.rD[0]);
    }
    const bool last = ez == c.NeZ - 1;
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      R.rS[1 + m] = last ? 0.0 : UcS[m];
      R.rD[1 + m] = last ? 0.0 : UcD[m];
    }
    if (!actS) {
#pragma unroll
      for (int cc = 0; cc < n3; ++cc) R.aS[cc] = 0.0;
    }
    if (!actD) {
#pragma unroll
      for (int cc = 0; cc < n3; ++cc) R.aD[cc] = 0.0;
    }
    __syncwarp();
    blk_fwd<N1, 0>(R, c.prow, c.plane, hl, actS, actD);
    blk_bwd<N1, n3 - 1>(R, c.plane, hl, c.hbase, actD);
    __syncwarp();
    if (actS) {
      const int xc = PivOrder<N1>::col(R.pvS);  // the unknown this row solved for
      c.bh[ez * n3 + xc] = R.rS[0];
#pragma unroll
      for (int m = 0; m < 3; ++m) c.G[(ez * n3 + xc) * 3 + m] = R.rS[1 + m];
    }
    if (actD) {
      c.bh[ez * n3 + rD] = R.rD[0];
#pragma unroll
      for (int m = 0; m < 3; ++m) c.G[(ez * n3 + rD) * 3 + m] = R.rD[1 + m];
    }
    __syncwarp();
  }
  // block back substitution (common_2.F90:443-458)
  for (int ez = c.NeZ - 2; ez >= 0; --ez) {
    const double* bn = c.bh + (ez + 1) * n3;
    for (int r = hl; r < n3; r += 16) {
      const double* G = c.G + (ez * n3 + r) * 3;
      c.bh[ez * n3 + r] -= G[0] * bn[0] + G[1] * bn[1] + G[2] * bn[2];
    }
    __syncwarp();
  }
  if (apply)
    for (int idx = hl; idx < 3 * c.L; idx += 16) c.P[idx] += c.bh[idx];
  __syncwarp();
}

// shared-memory doubles of one column
__host__ __device__ inline int vi_col_doubles(int N1, int L, int NeZ) {
  const int n3 = 3 * N1;
  return 11 * L + 2 * NeZ + 4 * (NeZ + 1) + n3 + 8 + (n3 + 1) / 2 + 1;
}

template <int N1>
__global__ void __launch_bounds__(128) k_vi_fp64(const Ops op, const Prof pf, const F5c qin, const F5c z,
                                                  const F5c guess, const F5 qout, const F5 tout, int* status,
                                                  const ViArgs args, int ncol, int per_col, double* gsc) {
  constexpr int N = N1 - 1, n3 = 3 * N1, NF = N1 * N1, Np = N1 * N1 * N1;
  extern __shared__ double sm[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, h = lane >> 4, hl = lane & 15;
  const int wpb = blockDim.x >> 5;
  const int slot = blockIdx.x * wpb + wib;
  const int npair = (ncol + 1) / 2;
  const int L = op.L, NeZ = op.NeZ;
  double* W = sm + (size_t)(2 * wib + h) * per_col;
  ColCtx<N1> c{op, pf, qin};
  c.L = L; c.NeZ = NeZ; c.hl = hl; c.hbase = lane & 16;
  c.P = W; c.bh = c.P + 3 * L;
  c.fr = c.bh + 3 * L; c.fm = c.fr + L; c.pot = c.fm + L; c.wt = c.pot + L; c.dpd = c.wt + L;
  c.alB = c.dpd + L; c.alT = c.alB + NeZ; c.J = c.alT + NeZ; c.prow = c.J + 4 * (NeZ + 1);
  c.plane = reinterpret_cast<int*>(c.prow + n3 + 8);
  c.G = gsc + ((size_t)slot * 2 + h) * ((size_t)NeZ * n3 * 3);
  c.nxyNp = (size_t)op.NeX * op.NeY * Np;
  const int gv[3] = {VD, VMZ, VRT};
  const double impl_fac = args.impl_fac;

  for (int pair = slot; pair < npair; pair += gridDim.x * wpb) {
    const int col_h = 2 * pair + h;
    const bool live = col_h < ncol;  // an odd column count leaves the last half-warp a copy to idle on
    const int col = live ? col_h : ncol - 1;
    const int ij = col % NF, exy = col / NF;
    c.gxy = (size_t)exy * Np + ij % N1 + N1 * (ij / N1);

    // --- the iterate (guess or var0), and alph from var0 (eval_Ax_uv :1149-1155) ---
    for (int l = hl; l < L; l += 16) {
      const size_t g = c.g(l);
#pragma unroll
      for (int m = 0; m < 3; ++m) c.P[3 * l + m] = guess.v[0] ? __ldg(guess.v[gv[m]] + g) : __ldg(z.v[gv[m]] + g);
      // sound speed + |w| of var0 -> fr (temporary)
      const double rdens0 = 1.0 / (__ldg(pf.dens + l) + __ldg(z.v[VD] + g));
      const double wt0 = __ldg(z.v[VMZ] + g) * rdens0;
      const double pres0 = op.pres00 * pow(op.rdry / op.pres00 * (__ldg(pf.rhyd + l) + __ldg(z.v[VRT] + g)), op.kap);
      c.fr[l] = fabs(wt0) + sqrt(op.kap * pres0 * rdens0);
    }
    __syncwarp();
    for (int ez = hl; ez < NeZ; ez += 16) {
      const int lb = ez * N1, lt = ez * N1 + N;
      c.alB[ez] = fmax(c.fr[lb], c.fr[ez > 0 ? lb - 1 : lb]);
      c.alT[ez] = fmax(c.fr[lt], c.fr[ez < NeZ - 1 ? lt + 1 : lt]);
    }
    __syncwarp();

    // --- MOMX/MOMY: the linear vertical-dissipation system (eval_Ax_uv + solve_uv) ---
    {
      double* Pu = c.bh;  // [2L] (bh is free until the Newton iteration)
      double* bu = c.fm;  // [2L] over fm and pot
      for (int l = hl; l < L; l += 16) {
        const size_t g = c.g(l);
        Pu[2 * l + 0] = __ldg(z.v[VMX] + g);
        Pu[2 * l + 1] = __ldg(z.v[VMY] + g);
      }
      __syncwarp();
      const double tm = -0.5 * op.FSz;
      if (impl_fac == 0.0) {
        for (int l = hl; l < L; l += 16) {
          const int ez = l / N1, pv = l - ez * N1;
          const int lb = ez * N1, lt = ez * N1 + N;
          const int lbP = ez > 0 ? lb - 1 : lb, ltP = ez < NeZ - 1 ? lt + 1 : lt;
          const double dBx = tm * c.alB[ez] * (Pu[2 * lbP] - Pu[2 * lb]), dTx = tm * c.alT[ez] * (Pu[2 * ltP] - Pu[2 * lt]);
          const double dBy = tm * c.alB[ez] * (Pu[2 * lbP + 1] - Pu[2 * lb + 1]),
                       dTy = tm * c.alT[ez] * (Pu[2 * ltP + 1] - Pu[2 * lt + 1]);
          const size_t g = c.g(l);
          if (live && tout.v[0]) {
            tout.v[VMX][g] = -(op.Lb[pv] * dBx + op.Lt[pv] * dTx);
            tout.v[VMY][g] = -(op.Lb[pv] * dBy + op.Lt[pv] * dTy);
          }
          if (live && qout.v[0]) { qout.v[VMX][g] = __ldg(qin.v[VMX] + g); qout.v[VMY][g] = __ldg(qin.v[VMY] + g); }
        }
      } else {
        // The element blocks are the identity plus the Lift face terms in columns 0 and N, coupled to
        // the neighbours only through those, so the system reduces exactly to a scalar tridiagonal
        // system in the interface jumps J_e = d(e, 0) - d(e-1, N), e = 1 .. NeZ-1 (J_0 = J_NeZ = 0 at the
        // slip lids):  (1 + beta(e, 0) + tau(e-1, N)) J_e - beta(e-1, N) J_{e-1} - tau(e, 0) J_{e+1}
        //            = b(e, 0) - b(e-1, N),  beta(e, p) = impl_fac Fz Lb[p] alB_e / 2, tau with Lt, alT,
        // and then d(e, p) = b(e, p) - beta(e, p) J_e + tau(e, p) J_{e+1}: the same linear solve as the
        // per-element LU of solve_Nnode8_uv (hevi_common_linalgebra.F90:2142-2294), in O(NeZ).
        for (int l = hl; l < L; l += 16) {  // b = impl_fac A_uv(P) - P + q*
          const int ez = l / N1, pv = l - ez * N1;
          const int lb = ez * N1, lt = ez * N1 + N;
          const int lbP = ez > 0 ? lb - 1 : lb, ltP = ez < NeZ - 1 ? lt + 1 : lt;
          const double dBx = tm * c.alB[ez] * (Pu[2 * lbP] - Pu[2 * lb]), dTx = tm * c.alT[ez] * (Pu[2 * ltP] - Pu[2 * lt]);
          const double dBy = tm * c.alB[ez] * (Pu[2 * lbP + 1] - Pu[2 * lb + 1]),
                       dTy = tm * c.alT[ez] * (Pu[2 * ltP + 1] - Pu[2 * lt + 1]);
          const size_t g = c.g(l);
          bu[2 * l] = impl_fac * (-(op.Lb[pv] * dBx + op.Lt[pv] * dTx)) - Pu[2 * l] + __ldg(qin.v[VMX] + g);
          bu[2 * l + 1] = impl_fac * (-(op.Lb[pv] * dBy + op.Lt[pv] * dTy)) - Pu[2 * l + 1] + __ldg(qin.v[VMY] + g);
        }
        __syncwarp();
        const double cfs = 0.5 * impl_fac * op.FSz;
        double* J = c.J;               // [2][NeZ + 1]: the jumps of MOMX and MOMY
        double* cp = c.J + 2 * (NeZ + 1);  // [2][NeZ + 1]: the forward-sweep coefficients
        if (hl < 2) {  // one Thomas sweep per momentum component
          const int m = hl;
          double* Jm = J + m * (NeZ + 1);
          double* cm = cp + m * (NeZ + 1);
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
            cm[e] = cprev;
          }
          for (int e = NeZ - 2; e >= 1; --e) Jm[e] -= cm[e] * Jm[e + 1];
        }
        __syncwarp();
        for (int l = hl; l < L; l += 16) {
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
        if (live) {
          for (int l = hl; l < L; l += 16) {
            const double px = Pu[2 * l] + bu[2 * l], py = Pu[2 * l + 1] + bu[2 * l + 1];
            const size_t g = c.g(l);
            if (qout.v[0]) { qout.v[VMX][g] = px; qout.v[VMY][g] = py; }
            if (tout.v[0]) {
              tout.v[VMX][g] = (px - __ldg(qin.v[VMX] + g)) / impl_fac;
              tout.v[VMY][g] = (py - __ldg(qin.v[VMY] + g)) / impl_fac;
            }
          }
        }
      }
      __syncwarp();
    }

    // --- DENS/MOMZ/RHOT: Newton on G(P) = P - q* - impl_fac A(P) ---
    int st = 0;
    if (impl_fac == 0.0) {
      col_residual<N1>(c, 0.0, args.cref, true);
      if (live) {
        for (int l = hl; l < L; l += 16) {
          const size_t g = c.g(l);
#pragma unroll
          for (int m = 0; m < 3; ++m) {
            if (tout.v[0]) tout.v[gv[m]][g] = c.bh[3 * l + m];
            if (qout.v[0]) qout.v[gv[m]][g] = __ldg(qin.v[gv[m]] + g);
          }
        }
      }
    } else {
      int nsolve = 0;
      bool done = !live;
      while (true) {
        const double err = col_residual<N1>(c, impl_fac, args.cref, false);
        if (!done) {
          if (err != err) { st = -2; done = true; }
          else if (args.max_iter > 1 && err <= args.tol) { st = nsolve; done = true; }
          else if (nsolve >= args.max_iter) { st = -1; done = true; }
        }
        if (__all_sync(0xffffffffu, done)) break;
        col_solve<N1>(c, impl_fac, !done);
        ++nsolve;
        if (args.max_iter == 1) {
          if (!done) st = 1;
          break;
        }
      }
      if (live) {
        for (int l = hl; l < L; l += 16) {
          const size_t g = c.g(l);
#pragma unroll
          for (int m = 0; m < 3; ++m) {
            const double pnew = c.P[3 * l + m];
            if (qout.v[0]) qout.v[gv[m]][g] = pnew;
            if (tout.v[0]) tout.v[gv[m]][g] = (pnew - __ldg(qin.v[gv[m]] + g)) / impl_fac;
          }
        }
      }
    }
    if (hl == 0 && live && status) status[col] = st;
    __syncwarp();
  }
}

namespace {
struct ViPlan {
  int wpb = 0, grid = 0, per_col = 0;
  size_t smem = 0, scratch = 0;  // bytes of shared memory per block, doubles of global scratch
};

// Persistent grid: warps per block chosen for the most resident warps per SM under the shared-memory
// need of the column height, one grid-wide wave of blocks.
template <int N1>
int plan_vi_n(const Ops& op, ViPlan& p) {
  const int n3 = 3 * N1;
  p.per_col = vi_col_doubles(N1, op.L, op.NeZ);
  const int ncol = op.NeX * op.NeY * N1 * N1;
  const int npair = (ncol + 1) / 2;
  int dev = 0, nsm = 0, optin = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e != cudaSuccess) return (int)e;
  auto kfn = k_vi_fp64<N1>;
  // the device's limit, the same value from every caller: contexts planning in several host threads
  // never lower it under one another's launch
  if ((e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, optin)) != cudaSuccess) return (int)e;
  int best = 0, best_nb = 0;
  for (int wpb = 4; wpb >= 1; wpb >>= 1) {
    const size_t smem = sizeof(double) * 2 * (size_t)p.per_col * wpb;
    if (smem > (size_t)optin) continue;
    int nb = 0;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kfn, 32 * wpb, smem)) != cudaSuccess) return (int)e;
    if (nb * wpb > best) { best = nb * wpb; best_nb = nb; p.wpb = wpb; p.smem = smem; }
  }
  if (best == 0) return (int)cudaErrorInvalidValue;  // one column does not fit in shared memory
  p.grid = std::max(1, std::min((npair + p.wpb - 1) / p.wpb, best_nb * nsm));
  p.scratch = (size_t)p.grid * p.wpb * 2 * op.NeZ * n3 * 3;
  return 0;
}

int plan_vi(const Ops& op, ViPlan& p) {
  switch (op.N1) {
    case 2: return plan_vi_n<2>(op, p);
    case 3: return plan_vi_n<3>(op, p);
    case 4: return plan_vi_n<4>(op, p);
    case 5: return plan_vi_n<5>(op, p);
    case 6: return plan_vi_n<6>(op, p);
    case 7: return plan_vi_n<7>(op, p);
    case 8: return plan_vi_n<8>(op, p);
  }
  return (int)cudaErrorInvalidValue;
}

template <int N1>
int launch_vi_n(const ViPlan& p, const Ops& op, const Prof& pf, const F5c& qin, const F5c& z, const F5c& guess,
                const F5& qout, const F5& tout, int* status, const ViArgs& a, double* gsc, cudaStream_t s) {
  const int ncol = op.NeX * op.NeY * N1 * N1;
  auto kfn = k_vi_fp64<N1>;
  kfn<<<p.grid, 32 * p.wpb, p.smem, s>>>(op, pf, qin, z, guess, qout, tout, status, a, ncol, p.per_col, gsc);
  return (int)cudaGetLastError();
}
}  // namespace

size_t vi_fp64_scratch_doubles(const Ops& op) {
  ViPlan p;
  return plan_vi(op, p) ? 0 : p.scratch;
}

int launch_vi_fp64(const Ops& op, const Prof& pf, const F5c& qin, const F5c& z, const F5c& guess, const F5& qout,
                   const F5& tout, int* status, const ViArgs& a, double* gsc, size_t gsc_doubles, cudaStream_t s) {
  ViPlan p;
  if (const int r = plan_vi(op, p)) return r;
  if (!gsc || gsc_doubles < p.scratch) return (int)cudaErrorInvalidValue;
  switch (op.N1) {
    case 2: return launch_vi_n<2>(p, op, pf, qin, z, guess, qout, tout, status, a, gsc, s);
    case 3: return launch_vi_n<3>(p, op, pf, qin, z, guess, qout, tout, status, a, gsc, s);
    case 4: return launch_vi_n<4>(p, op, pf, qin, z, guess, qout, tout, status, a, gsc, s);
    case 5: return launch_vi_n<5>(p, op, pf, qin, z, guess, qout, tout, status, a, gsc, s);
    case 6: return launch_vi_n<6>(p, op, pf, qin, z, guess, qout, tout, status, a, gsc, s);
    case 7: return launch_vi_n<7>(p, op, pf, qin, z, guess, qout, tout, status, a, gsc, s);
    case 8: return launch_vi_n<8>(p, op, pf, qin, z, guess, qout, tout, status, a, gsc, s);
  }
  return (int)cudaErrorInvalidValue;
}

}  // namespace fedg
