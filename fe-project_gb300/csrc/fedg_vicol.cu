// fedg_vicol.cu -- HEVI column Newton solve of the mixed-precision path (cal_vi), N1 lanes per
// column and 32/N1 columns per warp.
//
// FElib's cal_vi (FElib/src/atmosphere/dynamics/scale_atm_dyn_dgm_nonhydro3d_rhot_hevi.F90:
// 772-965, the operators of scale_atm_dyn_dgm_nonhydro3d_hevi_common_2.F90) solves, column by
// column, Q - q* - impl_fac A(Q) = 0 for the vertical acoustic/buoyancy operator A with the
// vertical Rusanov speed frozen at var0:
//   MOMX, MOMY: a linear system (vertical face dissipation only, eval_Ax_uv/solve_uv)
//   DENS, MOMZ, RHOT: Newton on a block-tridiagonal system with 3*N1 x 3*N1 element blocks
//   (construct_matbnd, block-Thomas, block LU).
//
// Thread layout: lane k of a column group owns node k of every element of the column (level
// l = ez*N1 + k) and, in the solve, the three rows (DENS, MOMZ, RHOT) of that node in each
// element block.  The columns of one warp are neighbours in x (same element, consecutive i),
// so every global load of a level touches whole 32-byte sectors.
//
// Precision (see fedg_mixed.cu for the whole path):
//   - the iterate P and the stage input q* are float pairs (hi + lo, about 48 significant bits,
//     fedg_f2.cuh); the convergence test is on the residual b = impl_fac A(P) + q* - P with the
//     operator evaluated in float pairs ("certifying" residual), so the column reaches the
//     FP64-class Newton solution while the kernel issues no FP64 arithmetic on its main path;
//   - from var0, the first residual comes from the stage-1 kernel's A(var0) (no operator pass);
//   - Jacobian, block-Thomas and the element LU (no pivoting: I + impl_fac J is diagonally
//     dominant at stable time steps; a failure shows as a non-converging or non-finite certifying
//     residual, reported per column) are FP32; after an LU correction, Neumann corrections;
//   - MOMX/MOMY: the element blocks are I plus two rank-one face terms, so the system reduces
//     exactly to a scalar tridiagonal system in the NeZ-1 interface jumps, solved in FP32 and
//     accumulated into E = P - q* in pairs; the residual (the jumps of q* formed in pairs, E in
//     pairs, the operator in FP32) is accurate far below the tolerance because the operator only
//     sees the jumps.
//
// Memory: per column in shared memory the leading parts of P, the FP32 work vector and the
// per-phase scratch (4.26 KB at p = 7, NeZ = 16: 12 warps per SM); in global memory, L2-resident
// while the column is in flight and discarded from L2 after their last use, the block-Thomas
// history and the trailing parts of P.  Data read or written once per launch carries an L2
// evict-first policy.
#include <algorithm>

#include "fedg_ctx.cuh"
#include "fedg_f2.cuh"
#include "fedg_mixed.cuh"

namespace fedg {
namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr f2 Z2F{0.f, 0.f};

// per-column shared-memory layout (bytes).  Three scratch areas whose phases never overlap share
// one region: the residual's ring of level quantities, the correction's Jacobian quantities and
// block coupling, and the MOMX/MOMY phase's tridiagonal arrays.  The column stride is the
// smallest one whose residue puts the C columns of a warp on different banks.
struct ColLayout {
  int oP, oRing, oDel, oBf, oBc, oAl, oJb, oSJ, stride;
  __host__ __device__ ColLayout(int N1, int NeZ) {
    const int L = N1 * NeZ;
    int o = 0;
    oP = o;    o += 12 * L;                    // float P[3L]: the iterate's leading parts (uv phase:
                                               // E [2L] and the face jumps of q*)
    oBf = o;   o += 12 * L;                    // float b / y / x [3L] (uv phase: [2L])
    oDel = o;  o += 48;                        // 6 face fluxes (float2) of the current element
    oAl = o;   o += ((8 * NeZ + 15) / 16) * 16; // alB, alT per element
    const int u_ring = 120 * N1;                           // 3 element slots x 5 quantities x N1 x float2
    const int u_solve = 16 * (N1 + 2) + 64;                // float4 pot, wt, dpd of the element's nodes
                                                           // + 2 neighbours; coupling from below
    const int u_jb = ((12 * (NeZ + 1) + 15) / 16) * 16;    // uv: c' and the two interface jumps
    oRing = oSJ = oJb = o;
    oBc = o + 16 * (N1 + 2);
    o += u_ring > u_solve ? (u_ring > u_jb ? u_ring : u_jb) : (u_solve > u_jb ? u_solve : u_jb);
    const int words = o / 4;
    const int C = 32 / N1, r = 32 / C, m = 2 * r;  // stride = r (mod 2r) words
    stride = 4 * (((words - r + m - 1) / m) * m + r);
  }
};

template <int N1>
struct Col {
  float* P;      // iterate: the leading parts of its float pairs, row 3l+v (v: DENS, MOMZ, RHOT)
  float4* sJ;    // Jacobian level quantities of the current element's nodes, then node N of the
                 // element below and node 0 of the element above
  void* ring;    // [3][4][N1]: slot, quantity (MOMZ, DDENS, fm, fr), node
  void* del;
  float* Bf;
  float* bc;
  float* al;
  float* jb;
  // the trailing parts of the iterate's pairs, in global memory (L2-resident while the column is in
  // flight): three planes of n nodes, node (column + element * ncol) * N1 + k, so that a warp's 32
  // nodes of an element fill one 128-byte line per plane
  float* lo;
  size_t lo_n, lo_b, lo_s;
  int k, NeZ, L;
  size_t gb, gs;  // global index of node (0, k) of this column and the element-layer stride
  __device__ float* plo(int v, int e) const { return lo + (size_t)v * lo_n + lo_b + (size_t)e * lo_s; }
  __device__ size_t g(int e) const { return gb + (size_t)e * gs; }
  __device__ float alB(int e) const { return al[2 * e]; }
  __device__ float alT(int e) const { return al[2 * e + 1]; }
};

// L2 eviction priority of the data the kernel reads or writes exactly once (var0, the stage
// kernel's A(var0), the last read of q*, the outputs): evict-first.  What a column reads again
// while the other columns stream past it (q* in every certifying residual, the block-Thomas
// history) then keeps its lines in L2 instead of going back to DRAM.
__device__ __forceinline__ unsigned long long l2_evict_first() {
  unsigned long long p;
  asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ double ld_once(const double* a, unsigned long long pol) {
  double v;
  asm("ld.global.nc.L2::cache_hint.f64 %0, [%1], %2;" : "=d"(v) : "l"(a), "l"(pol));
  return v;
}
__device__ __forceinline__ float2 ld_once(const float2* a, unsigned long long pol) {
  float2 v;
  asm("ld.global.nc.L2::cache_hint.v2.f32 {%0, %1}, [%2], %3;" : "=f"(v.x), "=f"(v.y) : "l"(a), "l"(pol));
  return v;
}
__device__ __forceinline__ void st_once(float2* a, float2 v, unsigned long long pol) {
  asm volatile("st.global.L2::cache_hint.v2.f32 [%0], {%1, %2}, %3;" ::"l"(a), "f"(v.x), "f"(v.y), "l"(pol)
               : "memory");
}
__device__ __forceinline__ void st_once(float* a, float v, unsigned long long pol) {
  asm volatile("st.global.L2::cache_hint.f32 [%0], %1, %2;" ::"l"(a), "f"(v), "l"(pol) : "memory");
}

// the pressure deviation (1 + r)^kappa - 1 in FP64 where its series is out of range (|r| > rmax):
// rare, so it is kept out of line, one copy for the whole kernel
__device__ __noinline__ f2 pres_dev_pow(float rh, float rl, double kap64) {
  return f2_split(pow(1.0 + ((double)rh + (double)rl), kap64) - 1.0);
}

__device__ __forceinline__ float grp_max_nan(float e, int width) {
  for (int o = width / 2; o > 0; o >>= 1) {
    const float oe = __shfl_xor_sync(FULL, e, o);
    e = (e != e || oe != oe) ? __int_as_float(0x7fc00000) : fmaxf(e, oe);
  }
  return e;
}

// ---------------------------------------------------------------------------------------------
// residual b = impl_fac A(P) + q* - P of the DENS/MOMZ/RHOT system into c.Bf (FP32); returns the
// column max of |b|/scale (NaN if not finite).
// The operator A in float pairs (eval_Ax, hevi_common_2.F90:1177-1292, with the vertical face flux
// vi_cal_del_flux_dyn :1294-1323).
// Element by element, with the level quantities of elements e-1, e, e+1 in a ring of 3 slots
// (MOMZ, DDENS, fm, fr and DRHOT of every node, the iterate's values as float pairs).
// The pressure deviation PRES_hyd ((1 + r)^kappa - 1), r = DRHOT/RHOT_hyd, is the binomial
// series: its leading term kappa r in pairs, the rest (relative size |r|) in FP32, which keeps
// the pair precision for |r| <= rmax; beyond that pow() in FP64.
template <int N1>
__device__ float col_residual(const OpsX& ox, const Col<N1>& c, const ProfX& px, const X5& qin, float2 impl2,
                              float cref) {
  constexpr int N = N1 - 1;
  const int k = c.k;
  float2* r2 = reinterpret_cast<float2*>(c.ring);
  auto ri = [](int s, int q, int m) { return (s * 5 + q) * N1 + m; };
  f2 Dk[N1], Tk[N1];
#pragma unroll
  for (int m = 0; m < N1; ++m) {
    Dk[m] = f2_of(ox.D[k * N1 + m]);
    Tk[m] = f2_of(ox.T[k * N1 + m]);
  }
  const f2 lbk = f2_of(ox.Lb[k]), ltk = f2_of(ox.Lt[k]);
  const f2 E33 = f2_of(ox.E33), grav = f2_of(ox.grav), tmp1 = f2_of(ox.tmp1), impl = f2_of(impl2);

  auto lo3 = [&](int e, float (&o)[3]) {
#pragma unroll
    for (int v = 0; v < 3; ++v) o[v] = *c.plo(v, e);
  };
  auto fill = [&](int e, const float (&lo)[3]) {  // level quantities of node (e, k) into slot e % 3
    const int l = e * N1 + k;
    const f2 Pd{c.P[3 * l], lo[0]}, Pm{c.P[3 * l + 1], lo[1]}, Pr{c.P[3 * l + 2], lo[2]};
    const int s = e % 3;
    const f2 dens = f2_add(f2_of(__ldg(px.dh + l)), Pd);
    const f2 rhot = f2_add(f2_of(__ldg(px.rh + l)), Pr);
    const f2 rd = f2_recip(dens);
    const f2 pot = f2_mul(rhot, rd);
    const f2 rr = f2_mul(Pr, f2_of(__ldg(px.rhinv + l)));
    f2 S;
    if (fabsf(rr.h) <= ox.rmax) {
      float tl = ox.cb[11];
#pragma unroll
      for (int m = 10; m >= 1; --m) tl = fmaf(tl, rr.h, ox.cb[m]);
      S = f2_add_f(f2_mul(f2_of(ox.kap), rr), __fmul_rn(__fmul_rn(rr.h, rr.h), tl));
    } else {
      S = pres_dev_pow(rr.h, rr.l, ox.kap64);
    }
    const f2 fm = f2_mul(f2_of(__ldg(px.ph + l)), S);
    r2[ri(s, 0, k)] = f2_pack(Pm);
    r2[ri(s, 1, k)] = f2_pack(Pd);
    r2[ri(s, 2, k)] = f2_pack(fm);
    r2[ri(s, 3, k)] = f2_pack(f2_mul(pot, Pm));
    r2[ri(s, 4, k)] = f2_pack(Pr);
  };

  float errf = 0.f;
  bool bad = false;  // a non-finite entry anywhere makes the column's error NaN (fmaxf drops NaNs)
  const int gv[3] = {VD, VMZ, VRT};
  // the stage input q* of the lane's node, loaded one element ahead so that the load latency
  // overlaps the current element's work
  float2 qcur[3], qnxt[3];
#pragma unroll
  for (int v = 0; v < 3; ++v) qcur[v] = __ldg(qin.v[gv[v]] + c.g(0));
  // iterations e = -2, -1 only fill the ring with elements 0 and 1: one call site of fill for the
  // whole loop (the kernel's code stays small for the instruction caches)
  float lon[3];  // the trailing parts of the next element to fill, loaded one iteration ahead
  lo3(0, lon);
  for (int e = -2; e < c.NeZ; ++e) {
    if (e >= 0) {
      const int sc = e % 3, sb = (e + 2) % 3, st = (e + 1) % 3;
      {
        const size_t gn = c.g(e + 1 < c.NeZ ? e + 1 : e);
#pragma unroll
        for (int v = 0; v < 3; ++v) qnxt[v] = __ldg(qin.v[gv[v]] + gn);
      }
      // vertical-face fluxes of element e: lanes over (side, variable)
      for (int t = k; t < 6; t += N1) {
        const int s = t / 3, v = t - 3 * s;
        const int nM = s == 0 ? 0 : N;
        const bool lid = s == 0 ? (e == 0) : (e == c.NeZ - 1);
        const int sP = lid ? sc : (s == 0 ? sb : st), nP = lid ? nM : (s == 0 ? N : 0);
        const float nz = s == 0 ? -1.f : 1.f;
        const float al = s == 0 ? c.alB(e) : c.alT(e);
        // jump of RHOT (the slip lid's exterior state is the interior one: no jump)
        const f2 dth = lid ? f2{0.f, 0.f} : f2_sub(f2_of(r2[ri(sP, 4, nP)]), f2_of(r2[ri(sc, 4, nM)]));
        const f2 mzM = f2_of(r2[ri(sc, 0, nM)]);
        const f2 dmz = lid ? f2_add(f2_neg(mzM), f2_neg(mzM)) : f2_sub(f2_of(r2[ri(sP, 0, nP)]), mzM);
        f2 x;
        if (v == 0) {
          const f2 dr = lid ? f2{0.f, 0.f} : f2_sub(f2_of(r2[ri(sP, 1, nP)]), f2_of(r2[ri(sc, 1, nM)]));
          x = f2_sub(f2_mul_f(dmz, nz), f2_mul_f(dr, al));
        } else if (v == 1) {
          const f2 dfm = lid ? f2{0.f, 0.f} : f2_sub(f2_of(r2[ri(sP, 2, nP)]), f2_of(r2[ri(sc, 2, nM)]));
          x = f2_sub(f2_mul_f(dfm, nz), f2_mul_f(dmz, al));
        } else {
          const f2 frM = f2_of(r2[ri(sc, 3, nM)]);
          const f2 dfr = lid ? f2_add(f2_neg(frM), f2_neg(frM)) : f2_sub(f2_of(r2[ri(sP, 3, nP)]), frM);
          x = f2_sub(f2_mul_f(dfr, nz), f2_mul_f(dth, al));
        }
        reinterpret_cast<float2*>(c.del)[t] = f2_pack(f2_mul(tmp1, x));
      }
      __syncwarp();
      {
        const int l = e * N1 + k;
        const float isc[3] = {1.f / __ldg(px.dhf + l), 1.f / (__ldg(px.dhf + l) * cref), 1.f / __ldg(px.rhf + l)};
        float bfl[3];
        f2acc sd, sm, sr, drho;
#pragma unroll
        for (int m = 0; m < N1; ++m) {
          sd.add(Dk[m], f2_of(r2[ri(sc, 0, m)]));
          drho.add(Tk[m], f2_of(r2[ri(sc, 1, m)]));
          sm.add(Dk[m], f2_of(r2[ri(sc, 2, m)]));
          sr.add(Dk[m], f2_of(r2[ri(sc, 3, m)]));
        }
        const float2* dl = reinterpret_cast<const float2*>(c.del);
        f2 A[3];
        A[0] = f2_add(f2_add(f2_mul(E33, sd.get()), f2_mul(lbk, f2_of(dl[0]))), f2_mul(ltk, f2_of(dl[3])));
        A[1] = f2_add(f2_add(f2_add(f2_mul(E33, sm.get()), f2_mul(lbk, f2_of(dl[1]))), f2_mul(ltk, f2_of(dl[4]))),
                      f2_mul(grav, drho.get()));
        A[2] = f2_add(f2_add(f2_mul(E33, sr.get()), f2_mul(lbk, f2_of(dl[2]))), f2_mul(ltk, f2_of(dl[5])));
        // this node's iterate from the ring: DDENS (quantity 1), MOMZ (0), DRHOT (4)
        const f2 Pl[3] = {f2_of(r2[ri(sc, 1, k)]), f2_of(r2[ri(sc, 0, k)]), f2_of(r2[ri(sc, 4, k)])};
#pragma unroll
        for (int v = 0; v < 3; ++v) {  // A[v] holds -A: b = q* - P - impl_fac (-A)
          const f2 qmp = f2_sub(f2_of(qcur[v]), Pl[v]);
          bfl[v] = f2_to_f(f2_sub(qmp, f2_mul(impl, A[v])));
        }
#pragma unroll
        for (int v = 0; v < 3; ++v) {
          c.Bf[3 * l + v] = bfl[v];
          errf = fmaxf(errf, fabsf(bfl[v]) * isc[v]);
          bad = bad || !(fabsf(bfl[v]) < 3.0e38f);
        }
      }
      __syncwarp();
#pragma unroll
      for (int v = 0; v < 3; ++v) qcur[v] = qnxt[v];
    }
    if (e + 2 < c.NeZ) {
      const float lcur[3] = {lon[0], lon[1], lon[2]};
      if (e + 3 < c.NeZ) lo3(e + 3, lon);
      fill(e + 2, lcur);
    }
    __syncwarp();
  }
  return grp_max_nan(bad ? __int_as_float(0x7fc00000) : errf, N1);
}

// ---------------------------------------------------------------------------------------------
// One pass over a column before its Newton solve, loads one element ahead:
//  - the frozen vertical Rusanov speed |w| + c of var0 (hevi_common_2.F90:1149-1155) at the face
//    nodes, combined over the two sides of every face into c.al (lanes 0 and N give the values,
//    passed by shuffles; the element below's top value is carried to the next element);
//  - the initial iterate P in c.P: var0, or q* plus the guess increment;
//  - with a0 (the iterate starts at var0) the first residual b = (q* - var0) + impl_fac A(var0) in
//    c.Bf, from the implicit operator the stage-1 kernel evaluated at q^n = var0 for its own
//    implicit tendency (both implicit stages of an ARK232 step start at var0).  It is formed in
//    float pairs and rounded; the first correction is never judged by it (convergence is tested
//    on the certifying residual).
template <int N1>
__device__ void col_start(const ProfX& px, float kapf, const Col<N1>& c, const F5c& z, const X5& qin,
                          const float* const* guess, const A3& a0, float2 impl2) {
  constexpr int N = N1 - 1;
  const int k = c.k, NeZ = c.NeZ;
  const int gv[3] = {VD, VMZ, VRT};
  const bool res = a0.v[0] != nullptr, useq = res || guess;
  const f2 impl = f2_of(impl2);
  const unsigned long long once = l2_evict_first();
  double zc[3];
  float2 qc[3] = {}, ac[3] = {};
  float gc[3] = {};
  {
    const size_t g0 = c.g(0);
#pragma unroll
    for (int v = 0; v < 3; ++v) {
      zc[v] = ld_once(z.v[gv[v]] + g0, once);
      if (useq) qc[v] = __ldg(qin.v[gv[v]] + g0);
      if (res) ac[v] = ld_once(a0.v[v] + g0, once);
      if (guess) gc[v] = __ldg(guess[v] + g0);
    }
  }
  float aprev = 0.f;  // |w| + c at node N of the element below
  for (int e = 0; e < NeZ; ++e) {
    const int l = e * N1 + k;
    const size_t gn = c.g(e + 1 < NeZ ? e + 1 : e);
    double zn[3];
    float2 qn[3] = {}, an[3] = {};
    float gnx[3] = {};
#pragma unroll
    for (int v = 0; v < 3; ++v) {
      zn[v] = ld_once(z.v[gv[v]] + gn, once);
      if (useq) qn[v] = __ldg(qin.v[gv[v]] + gn);
      if (res) an[v] = ld_once(a0.v[v] + gn, once);
      if (guess) gnx[v] = __ldg(guess[v] + gn);
    }
    const float dd0 = f2_split(zc[0]).h, dr0 = f2_split(zc[2]).h;
    const float rdens0 = 1.f / (__ldg(px.dhf + l) + dd0);
    const float wt0 = f2_split(zc[1]).h * rdens0;
    const float pres0 = __ldg(px.phf + l) * (1.f + expm1f(kapf * log1pf(dr0 * __ldg(px.rthf + l))));
    const float at = fabsf(wt0) + sqrtf(kapf * pres0 * rdens0);
    const float a0n = __shfl_sync(FULL, at, 0, N1), aNn = __shfl_sync(FULL, at, N, N1);
    if (k == 0) {
      c.al[2 * e] = fmaxf(a0n, e > 0 ? aprev : a0n);
      if (e > 0) c.al[2 * e - 1] = fmaxf(aprev, a0n);
      if (e == NeZ - 1) c.al[2 * e + 1] = fmaxf(aNn, aNn);
    }
    aprev = aNn;
#pragma unroll
    for (int v = 0; v < 3; ++v) {
      const f2 p = guess ? f2_add_f(f2_of(qc[v]), gc[v]) : f2_split(zc[v]);
      c.P[3 * l + v] = p.h;
      *c.plo(v, e) = p.l;
      if (res) c.Bf[3 * l + v] = f2_to_f(f2_add(f2_sub(f2_of(qc[v]), p), f2_mul(impl, f2_of(ac[v]))));
      zc[v] = zn[v];
      qc[v] = qn[v];
      ac[v] = an[v];
      gc[v] = gnx[v];
    }
  }
  __syncwarp();
}

// Element LU without pivoting of the 3*N1 rows held 3 per lane (row 3k+v in lane k: v = DENS,
// MOMZ, RHOT of node k), with four right-hand sides; on return r = A^-1 r.  Pivot rows reach the
// other lanes of the column group by shuffles (width N1); every register index is a compile-time
// constant.  The elimination follows the DENS-first order of PivOrder (fedg_common.cuh) in blocked
// form, which shortens the chain of dependent steps from 3*N1 pivots forward and back to about
// N1 + 3 (restated and checked against a dense solve in numpy: tests/test_lu_order.py,
// blocked_solve):
//   - DENS_0, then DENS_1 .. DENS_{N-1} together: once DENS_0 is eliminated their pivot rows and
//     the other rows' multipliers are final (a DENS pivot row carries only DENS_N, the MOMZ columns
//     and RHOT_0, none of which is a DENS_1 .. DENS_{N-1} column), so their updates are independent
//     sums; then DENS_N;
//   - the MOMZ/RHOT Schur complement node by node with 2x2 pivot blocks (MOMZ_k, RHOT_k), whose
//     inverse lane k forms and keeps for the back substitution;
//   - back substitution block by block, then DENS_N, then DENS_0 .. DENS_{N-1} in parallel.
// No pivoting: I + impl_fac J is diagonally dominant at stable time steps; a failure shows as a
// non-converging or non-finite certifying residual, reported per column.
template <int N1>
struct DensCols {  // the columns a DENS pivot row can hold: the MOMZ columns, RHOT_0, DENS_N
  static constexpr int count = N1 + 2;
  __host__ __device__ static constexpr int at(int i) { return i < N1 ? 3 * i + 1 : (i == N1 ? 2 : 3 * (N1 - 1)); }
};
template <int N1, int kb>
__device__ __forceinline__ void blk_fwd(float (&a)[3][3 * N1], float (&r)[3][4], int k, float (&pinv)[4]) {
  if constexpr (kb < N1) {
    constexpr int c1 = 3 * kb + 1, c2 = 3 * kb + 2;
    if (k == kb) {  // 2x2 pivot block of node kb
      const float p11 = a[1][c1], p12 = a[1][c2], p21 = a[2][c1], p22 = a[2][c2];
      const float id = __fdividef(1.f, fmaf(p11, p22, -p12 * p21));
      pinv[0] = p22 * id; pinv[1] = -p12 * id; pinv[2] = -p21 * id; pinv[3] = p11 * id;
    }
    float q[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) q[i] = __shfl_sync(FULL, pinv[i], kb, N1);
    // multipliers [f1 f2] = [a_c1 a_c2] P^-1 of this lane's MOMZ/RHOT rows (nodes after kb)
    float f1[3], f2[3];
    const bool el = k > kb;
#pragma unroll
    for (int v = 1; v < 3; ++v) {
      f1[v] = el ? fmaf(a[v][c1], q[0], a[v][c2] * q[2]) : 0.f;
      f2[v] = el ? fmaf(a[v][c1], q[1], a[v][c2] * q[3]) : 0.f;
    }
#pragma unroll
    for (int m = kb + 1; m < N1; ++m) {
#pragma unroll
      for (int u = 1; u < 3; ++u) {
        const int cc = 3 * m + u;
        const float p1 = __shfl_sync(FULL, a[1][cc], kb, N1), p2 = __shfl_sync(FULL, a[2][cc], kb, N1);
#pragma unroll
        for (int v = 1; v < 3; ++v) a[v][cc] = fmaf(-f1[v], p1, fmaf(-f2[v], p2, a[v][cc]));
      }
    }
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      const float p1 = __shfl_sync(FULL, r[1][m], kb, N1), p2 = __shfl_sync(FULL, r[2][m], kb, N1);
#pragma unroll
      for (int v = 1; v < 3; ++v) r[v][m] = fmaf(-f1[v], p1, fmaf(-f2[v], p2, r[v][m]));
    }
    blk_fwd<N1, kb + 1>(a, r, k, pinv);
  }
}
template <int N1, int kb>
__device__ __forceinline__ void blk_bwd(const float (&a)[3][3 * N1], float (&r)[3][4], int k, const float (&pinv)[4]) {
  if constexpr (kb >= 0) {
    constexpr int c1 = 3 * kb + 1, c2 = 3 * kb + 2;
    if (k == kb) {  // x of the block: P^-1 times the reduced right-hand side
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        const float y1 = r[1][m], y2 = r[2][m];
        r[1][m] = fmaf(pinv[0], y1, pinv[1] * y2);
        r[2][m] = fmaf(pinv[2], y1, pinv[3] * y2);
      }
    }
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      const float x1 = __shfl_sync(FULL, r[1][m], kb, N1), x2 = __shfl_sync(FULL, r[2][m], kb, N1);
      // DENS rows: the MOMZ columns, and RHOT_0 (column 2) for block 0
      r[0][m] = fmaf(-a[0][c1], x1, kb == 0 ? fmaf(-a[0][2], x2, r[0][m]) : r[0][m]);
      if (k < kb) {
#pragma unroll
        for (int v = 1; v < 3; ++v) r[v][m] = fmaf(-a[v][c1], x1, fmaf(-a[v][c2], x2, r[v][m]));
      }
    }
    blk_bwd<N1, kb - 1>(a, r, k, pinv);
  }
}
template <int N1>
__device__ __forceinline__ void lu_blocked(float (&a)[3][3 * N1], float (&r)[3][4], int k) {
  constexpr int N = N1 - 1;
  using DC = DensCols<N1>;
  // DENS_0: every other row, the DENS_0 pivot row's columns only
  {
    const float inv = __fdividef(1.f, __shfl_sync(FULL, a[0][0], 0, N1));
    const float f[3] = {k > 0 ? a[0][0] * inv : 0.f, a[1][0] * inv, a[2][0] * inv};
#pragma unroll
    for (int i = 0; i < DC::count; ++i) {
      const int cc = DC::at(i);
      const float p = __shfl_sync(FULL, a[0][cc], 0, N1);
#pragma unroll
      for (int v = 0; v < 3; ++v) a[v][cc] = fmaf(-f[v], p, a[v][cc]);
    }
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      const float p = __shfl_sync(FULL, r[0][m], 0, N1);
#pragma unroll
      for (int v = 0; v < 3; ++v) r[v][m] = fmaf(-f[v], p, r[v][m]);
    }
  }
  // this lane's DENS pivot reciprocal (final once DENS_0 is eliminated; lane 0's is the DENS_0 pivot)
  float dg = a[0][0];
#pragma unroll
  for (int j = 1; j < N1; ++j) dg = k == j ? a[0][3 * j] : dg;
  const float rdk = __fdividef(1.f, dg);
  // DENS_1 .. DENS_{N-1} together: MOMZ/RHOT rows only (the DENS rows hold no DENS_j, 0 < j < N)
  if constexpr (N1 > 2) {
    float f1[N1], f2[N1];
#pragma unroll
    for (int j = 1; j < N; ++j) {
      const float inv = __shfl_sync(FULL, rdk, j, N1);
      f1[j] = a[1][3 * j] * inv;
      f2[j] = a[2][3 * j] * inv;
    }
#pragma unroll
    for (int i = 0; i < DC::count; ++i) {
      const int cc = DC::at(i);
      float s1 = a[1][cc], s2 = a[2][cc];
#pragma unroll
      for (int j = 1; j < N; ++j) {
        const float p = __shfl_sync(FULL, a[0][cc], j, N1);
        s1 = fmaf(-f1[j], p, s1);
        s2 = fmaf(-f2[j], p, s2);
      }
      a[1][cc] = s1;
      a[2][cc] = s2;
    }
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      float s1 = r[1][m], s2 = r[2][m];
#pragma unroll
      for (int j = 1; j < N; ++j) {
        const float p = __shfl_sync(FULL, r[0][m], j, N1);
        s1 = fmaf(-f1[j], p, s1);
        s2 = fmaf(-f2[j], p, s2);
      }
      r[1][m] = s1;
      r[2][m] = s2;
    }
  }
  // DENS_N: MOMZ/RHOT rows, the MOMZ columns and RHOT_0
  {
    const float inv = __shfl_sync(FULL, rdk, N, N1);
    const float f1 = a[1][3 * N] * inv, f2 = a[2][3 * N] * inv;
#pragma unroll
    for (int i = 0; i < DC::count - 1; ++i) {
      const int cc = DC::at(i);
      const float p = __shfl_sync(FULL, a[0][cc], N, N1);
      a[1][cc] = fmaf(-f1, p, a[1][cc]);
      a[2][cc] = fmaf(-f2, p, a[2][cc]);
    }
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      const float p = __shfl_sync(FULL, r[0][m], N, N1);
      r[1][m] = fmaf(-f1, p, r[1][m]);
      r[2][m] = fmaf(-f2, p, r[2][m]);
    }
  }
  float pinv[4] = {0.f, 0.f, 0.f, 0.f};
  blk_fwd<N1, 0>(a, r, k, pinv);
  blk_bwd<N1, N>(a, r, k, pinv);
  // DENS_N, then the other DENS unknowns in parallel
#pragma unroll
  for (int m = 0; m < 4; ++m) {
    const float xn = __shfl_sync(FULL, r[0][m] * rdk, N, N1);
    r[0][m] = k == N ? xn : fmaf(-a[0][3 * N], xn, r[0][m]) * rdk;
  }
}

// FP32 Jacobian level quantities of level l from the iterate: pot = RHOT/DENS, wt = MOMZ/DENS,
// dpd = dP/dRHOT = kappa PRES/RHOT
__device__ __forceinline__ float4 jac_level(const ProfX& px, const float* P, int l, float kapf) {
  const float Pd = P[3 * l], Pm = P[3 * l + 1], Pr = P[3 * l + 2];
  const float rdf = 1.f / (__ldg(px.dhf + l) + Pd);
  const float rhotf = __ldg(px.rhf + l) + Pr;
  const float phf = __ldg(px.phf + l);
  const float fmf = phf * expm1f(kapf * log1pf(Pr * __ldg(px.rthf + l)));
  return make_float4(rhotf * rdf, Pm * rdf, kapf * (phf + fmf) / rhotf, 0.f);
}

// P += sgn * b (b in c.Bf) in float pairs over the lane's levels; the trailing parts come from and go
// back to their global planes, loaded four elements at a time so that their latency overlaps
template <int N1>
__device__ __forceinline__ void col_add(const Col<N1>& c, float sgn) {
  const int k = c.k;
  for (int e0 = 0; e0 < c.NeZ; e0 += 4) {
    float lv[4][3];
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int v = 0; v < 3; ++v) lv[j][v] = e0 + j < c.NeZ ? *c.plo(v, e0 + j) : 0.f;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      if (e0 + j < c.NeZ) {
        const int l = (e0 + j) * N1 + k;
#pragma unroll
        for (int v = 0; v < 3; ++v) {
          const f2 p = f2_add_f(f2{c.P[3 * l + v], lv[j][v]}, sgn * c.Bf[3 * l + v]);
          c.P[3 * l + v] = p.h;
          *c.plo(v, e0 + j) = p.l;
        }
      }
    }
  }
}

// Block-Thomas history G_e = A_e^-1 U_e of the column solve: per node the 3 rows x 3 coupling
// columns (9 floats), in three planes of n nodes (float4, float4, float) so that every lane's
// stores and loads are 16-byte vectors and a warp's 32 nodes fill whole 128-byte lines: per
// element, 4 + 4 + 1 lines.  Node index: (column + element * ncol) * N1 + k.
struct GHist {
  float* base;
  size_t n;  // nodes
  __device__ float4* p0(size_t g) const { return reinterpret_cast<float4*>(base) + g; }
  __device__ float4* p1(size_t g) const { return reinterpret_cast<float4*>(base + 4 * n) + g; }
  __device__ float* p2(size_t g) const { return base + 8 * n + g; }
  // The history is written and read back within one correction while it sits in L2.  Once the
  // back sweep has read an element's lines they are dead, and discarding them drops the dirty
  // lines without a write-back to DRAM.  g0: first node of the warp's 32 nodes of the element
  // (128-byte aligned: the warp's columns are C consecutive ones starting at a multiple of C).
  __device__ void discard(size_t g0, int lane) const {
    const char* a = nullptr;
    if (lane < 4) a = reinterpret_cast<const char*>(p0(g0)) + 128 * lane;
    else if (lane < 8) a = reinterpret_cast<const char*>(p1(g0)) + 128 * (lane - 4);
    else if (lane == 8) a = reinterpret_cast<const char*>(p2(g0));
    if (a) asm volatile("discard.global.L2 [%0], 128;" ::"l"(a) : "memory");
  }
};

// one Newton correction of the DENS/MOMZ/RHOT system from the residual in c.Bf and the Jacobian
// quantities of the iterate: construct_matbnd (hevi_common_2.F90:1325-1480), block-Thomas with the
// 3x3 couplings of the face nodes, element LU; P += correction where apply.  G history in gh.
template <int N1>
__device__ void col_solve(const Ops& op, const ProfX& px, float kapf, const Col<N1>& c, double impl_fac,
                          const GHist& gh, size_t gcol, size_t gcol0, size_t glayer, int lane, bool apply) {
  constexpr int N = N1 - 1, n3 = 3 * N1;
  const int k = c.k;
  const float fi = (float)impl_fac;
  const float fdzs = (float)op.E33 * fi;
  float Dk[N1], Tk[N1];
#pragma unroll
  for (int m = 0; m < N1; ++m) {
    Dk[m] = fdzs * (float)op.D[k * N1 + m];
    Tk[m] = fi * (float)op.grav * (float)op.T[k * N1 + m];
  }
  const float facB = 0.5f * fi * (float)op.Lb[k] * (float)op.FSz;
  const float facT = 0.5f * fi * (float)op.Lt[k] * (float)op.FSz;
  for (int e = 0; e < c.NeZ; ++e) {
    float a[3][n3];
    float r[3][4];
    {  // this element's level quantities, and the face neighbours' (lane 0: below, lane N: above)
      const int l = e * N1 + k;
      const float4 own = jac_level(px, c.P, l, kapf);
      const bool below = k == 0 && e > 0, above = k == N && e < c.NeZ - 1;
      const float4 nb = jac_level(px, c.P, below ? l - 1 : (above ? l + 1 : l), kapf);
      __syncwarp();  // the previous element's quantities have been read
      c.sJ[k] = own;
      if (below) c.sJ[N1] = nb;
      if (above) c.sJ[N1 + 1] = nb;
      __syncwarp();
    }
    float4 J[N1];
#pragma unroll
    for (int m = 0; m < N1; ++m) J[m] = c.sJ[m];
#pragma unroll
    for (int m = 0; m < N1; ++m) {
      const float fdz = Dk[m];
      const float id = (m == k) ? 1.f : 0.f;
      a[0][3 * m + 0] = id;
      a[0][3 * m + 1] = fdz;
      a[0][3 * m + 2] = 0.f;
      a[1][3 * m + 0] = Tk[m];
      a[1][3 * m + 1] = id;
      a[1][3 * m + 2] = fdz * J[m].z;
      a[2][3 * m + 0] = -fdz * J[m].x * J[m].y;
      a[2][3 * m + 1] = fdz * J[m].x;
      a[2][3 * m + 2] = id + fdz * J[m].y;
    }
    float Lc[3][3], Uc[3][3];
#pragma unroll
    for (int f = 0; f < 2; ++f) {
      const bool bnd = (f == 0) ? (e == 0) : (e == c.NeZ - 1);
      const int pv1 = f == 0 ? 0 : N;
      const float nz = f == 0 ? -1.f : 1.f;
      const float al = f == 0 ? c.alB(e) : c.alT(e);
      const float fac = f == 0 ? facB : facT;
      const float t1 = fac * al, t2 = fac * nz;
      const float pot1 = J[pv1].x, wt1 = J[pv1].y, dpd1 = J[pv1].z;
      const int c0 = 3 * pv1;
      float cc[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
      if (bnd) {  // slip lid: exterior MOMZ = -interior
        a[2][c0 + 0] += 2.f * t2 * pot1 * wt1;
        a[0][c0 + 1] -= 2.f * t2;
        a[1][c0 + 1] += 2.f * t1;
        a[2][c0 + 1] -= 2.f * t2 * pot1;
        a[2][c0 + 2] -= 2.f * t2 * wt1;
      } else {
        a[0][c0 + 0] += t1;
        a[2][c0 + 0] += t2 * pot1 * wt1;
        a[0][c0 + 1] -= t2;
        a[1][c0 + 1] += t1;
        a[2][c0 + 1] -= t2 * pot1;
        a[1][c0 + 2] -= t2 * dpd1;
        a[2][c0 + 2] += t1 - t2 * wt1;
        const float4 Jn = c.sJ[f == 0 ? N1 : N1 + 1];
        cc[0][0] = -t1; cc[0][1] = t2;
        cc[1][1] = -t1; cc[1][2] = t2 * Jn.z;
        cc[2][0] = -t2 * Jn.x * Jn.y; cc[2][1] = t2 * Jn.x; cc[2][2] = -t1 + t2 * Jn.y;
      }
#pragma unroll
      for (int v = 0; v < 3; ++v)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          if (f == 0) Lc[v][j] = cc[v][j];
          else Uc[v][j] = cc[v][j];
        }
    }
    const int l = e * N1 + k;
#pragma unroll
    for (int v = 0; v < 3; ++v) r[v][0] = c.Bf[3 * l + v];
    if (e > 0) {  // A_e -= L_e G_{e-1}, b_e -= L_e y_{e-1} (rows of node N of element e-1)
      const float4 b0 = reinterpret_cast<const float4*>(c.bc)[0];
      const float4 b1 = reinterpret_cast<const float4*>(c.bc)[1];
      const float4 b2 = reinterpret_cast<const float4*>(c.bc)[2];
      const float Gp[3][3] = {{b0.x, b0.y, b0.z}, {b1.x, b1.y, b1.z}, {b2.x, b2.y, b2.z}};
      const float yp[3] = {b0.w, b1.w, b2.w};
#pragma unroll
      for (int v = 0; v < 3; ++v) {
#pragma unroll
        for (int c2 = 0; c2 < 3; ++c2)
          a[v][c2] -= Lc[v][0] * Gp[0][c2] + Lc[v][1] * Gp[1][c2] + Lc[v][2] * Gp[2][c2];
        r[v][0] -= Lc[v][0] * yp[0] + Lc[v][1] * yp[1] + Lc[v][2] * yp[2];
      }
    }
    const bool last = e == c.NeZ - 1;
#pragma unroll
    for (int v = 0; v < 3; ++v)
#pragma unroll
      for (int j = 0; j < 3; ++j) r[v][1 + j] = last ? 0.f : Uc[v][j];
    __syncwarp();  // everyone has read c.bc
    lu_blocked<N1>(a, r, k);
#pragma unroll
    for (int v = 0; v < 3; ++v) c.Bf[3 * l + v] = r[v][0];
    if (!last) {  // the last element's G is zero and never read
      const size_t gn = (gcol + (size_t)e * glayer) * N1 + k;
      *gh.p0(gn) = make_float4(r[0][1], r[0][2], r[0][3], r[1][1]);
      *gh.p1(gn) = make_float4(r[1][2], r[1][3], r[2][1], r[2][2]);
      *gh.p2(gn) = r[2][3];
    }
    if (k == N) {
      float4* b4 = reinterpret_cast<float4*>(c.bc);
      b4[0] = make_float4(r[0][1], r[0][2], r[0][3], r[0][0]);
      b4[1] = make_float4(r[1][1], r[1][2], r[1][3], r[1][0]);
      b4[2] = make_float4(r[2][1], r[2][2], r[2][3], r[2][0]);
    }
    __syncwarp();
  }
  // back sweep: x_e = y_e - G_e x_{e+1}(node 0); the history of element e-1 is loaded while e is
  // processed
  float4 g0n = make_float4(0.f, 0.f, 0.f, 0.f), g1n = g0n;
  float g2n = 0.f;
  if (c.NeZ >= 2) {
    const size_t gn = (gcol + (size_t)(c.NeZ - 2) * glayer) * N1 + k;
    g0n = *gh.p0(gn); g1n = *gh.p1(gn); g2n = *gh.p2(gn);
  }
  for (int e = c.NeZ - 2; e >= 0; --e) {
    const int l = e * N1 + k;
    const float* x1 = c.Bf + 3 * (e + 1) * N1;
    const float xa = x1[0], xb = x1[1], xc = x1[2];
    const float4 g0 = g0n, g1 = g1n;
    const float g2 = g2n;
    if (e > 0) {
      const size_t gn = (gcol + (size_t)(e - 1) * glayer) * N1 + k;
      g0n = *gh.p0(gn); g1n = *gh.p1(gn); g2n = *gh.p2(gn);
    }
    c.Bf[3 * l + 0] -= g0.x * xa + g0.y * xb + g0.z * xc;
    c.Bf[3 * l + 1] -= g0.w * xa + g1.x * xb + g1.y * xc;
    c.Bf[3 * l + 2] -= g1.z * xa + g1.w * xb + g2 * xc;
    __syncwarp();  // every lane has read element e's history: its lines are dead
    gh.discard((gcol0 + (size_t)e * glayer) * N1, lane);
  }
  if (apply) col_add<N1>(c, 1.f);
  __syncwarp();
}

// One Newton correction by a truncated Neumann series, for a residual b (in c.Bf) that an LU
// correction has already made small.  With J = I + K (K: the Jacobian of the DENS/MOMZ/RHOT system
// without its identity, the same entries col_solve assembles), delta = (I - K + K^2 - ...) b with
// nterm products K v; its error is K^(nterm+1) J^-1 b.  At small vertical Courant numbers ||K|| is
// well below one (about 0.26 on the 128x128x16 p = 7 mesh at dt 0.005 s), so two products bring
// the residual down by ~50x at the cost of two Jacobian-vector products (no assembly, no LU), where
// an LU correction would be exact to FP32.  The caller checks the new certifying residual and
// falls back to LU corrections when the series did not contract.
// K v element by element, in place on c.Bf: lane k forms its node's three rows from the element's
// v (c.Bf), the face nodes of the neighbours (vb: node N of element e-1, saved before it was
// overwritten; node 0 of element e+1, not yet overwritten) and the level quantities of the iterate.
template <int N1>
__device__ void col_jvp(const Ops& op, const ProfX& px, float kapf, const Col<N1>& c, double impl_fac) {
  constexpr int N = N1 - 1;
  const int k = c.k;
  const float fi = (float)impl_fac;
  const float fdzs = (float)op.E33 * fi;
  float Dk[N1], Tk[N1];
#pragma unroll
  for (int m = 0; m < N1; ++m) {
    Dk[m] = fdzs * (float)op.D[k * N1 + m];
    Tk[m] = fi * (float)op.grav * (float)op.T[k * N1 + m];
  }
  const float facB = 0.5f * fi * (float)op.Lb[k] * (float)op.FSz;
  const float facT = 0.5f * fi * (float)op.Lt[k] * (float)op.FSz;
  float vb[3] = {0.f, 0.f, 0.f};  // v at node N of element e-1
  for (int e = 0; e < c.NeZ; ++e) {
    const int l = e * N1 + k;
    {
      const float4 own = jac_level(px, c.P, l, kapf);
      const bool below = k == 0 && e > 0, above = k == N && e < c.NeZ - 1;
      const float4 nb = jac_level(px, c.P, below ? l - 1 : (above ? l + 1 : l), kapf);
      __syncwarp();
      c.sJ[k] = own;
      if (below) c.sJ[N1] = nb;
      if (above) c.sJ[N1 + 1] = nb;
      __syncwarp();
    }
    const float* ve = c.Bf + 3 * e * N1;
    float y[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int m = 0; m < N1; ++m) {
      const float4 Jm = c.sJ[m];
      const float vr = ve[3 * m], vm = ve[3 * m + 1], vt = ve[3 * m + 2];
      y[0] = fmaf(Dk[m], vm, y[0]);
      y[1] = fmaf(Tk[m], vr, fmaf(Dk[m] * Jm.z, vt, y[1]));
      y[2] = fmaf(Dk[m], Jm.x * (vm - Jm.y * vr) + Jm.y * vt, y[2]);
    }
#pragma unroll
    for (int f = 0; f < 2; ++f) {
      const bool bnd = f == 0 ? (e == 0) : (e == c.NeZ - 1);
      const int pv1 = f == 0 ? 0 : N;
      const float nz = f == 0 ? -1.f : 1.f;
      const float al = f == 0 ? c.alB(e) : c.alT(e);
      const float fac = f == 0 ? facB : facT;
      const float t1 = fac * al, t2 = fac * nz;
      const float4 J1 = c.sJ[pv1];
      const float pot1 = J1.x, wt1 = J1.y, dpd1 = J1.z;
      const float r1 = ve[3 * pv1], m1 = ve[3 * pv1 + 1], h1 = ve[3 * pv1 + 2];
      if (bnd) {  // slip lid: exterior MOMZ = -interior
        y[0] -= 2.f * t2 * m1;
        y[1] += 2.f * t1 * m1;
        y[2] += 2.f * t2 * (pot1 * wt1 * r1 - pot1 * m1 - wt1 * h1);
      } else {
        const float4 Jn = c.sJ[f == 0 ? N1 : N1 + 1];
        const float* vn = f == 0 ? vb : ve + 3 * N1;  // node 0 of element e+1 (not yet overwritten)
        const float rn = vn[0], mn = vn[1], hn = vn[2];
        y[0] += t1 * (r1 - rn) - t2 * (m1 - mn);
        y[1] += t1 * (m1 - mn) - t2 * (dpd1 * h1 - Jn.z * hn);
        y[2] += t2 * (pot1 * wt1 * r1 - Jn.x * Jn.y * rn) - t2 * (pot1 * m1 - Jn.x * mn) + t1 * (h1 - hn) -
                t2 * (wt1 * h1 - Jn.y * hn);
      }
    }
    const float vN0 = ve[3 * N], vN1 = ve[3 * N + 1], vN2 = ve[3 * N + 2];
    __syncwarp();  // every lane has read element e's v
    vb[0] = vN0; vb[1] = vN1; vb[2] = vN2;
#pragma unroll
    for (int v = 0; v < 3; ++v) c.Bf[3 * l + v] = y[v];
    __syncwarp();
  }
}

// P += (I - K + K^2 - ... +- K^nterm) b for b in c.Bf (destroyed) where apply.
template <int N1>
__device__ void col_neumann(const Ops& op, const ProfX& px, float kapf, const Col<N1>& c, double impl_fac, int nterm,
                            bool apply) {
  for (int t = 0; t <= nterm; ++t) {
    if (t > 0) col_jvp<N1>(op, px, kapf, c, impl_fac);
    if (apply) col_add<N1>(c, (t & 1) ? -1.f : 1.f);
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------------------------
template <int N1, bool PO>
__global__ void __launch_bounds__(64, 6) k_vi_cols(const Ops op, const OpsX ox, const ProfX px, const X5 qin, const F5c z,
                                                const A3 a0, const float* const* guess, void* const* qsf, void* const* tout,
                                                float* __restrict__ gsc, int* status, unsigned long long* cnt,
                                                const MixViArgs args, int ncol) {
  static_assert(32 / N1 * N1 == 32, "a warp's columns cover 32 nodes of a level (whole G-history lines)");
  constexpr int N = N1 - 1, C = 32 / N1, NF = N1 * N1, Np = N1 * N1 * N1;
  extern __shared__ __align__(16) unsigned char smraw[];
  // two warps per block (C columns each): with the one-warp blocks the per-block shared-memory
  // reservation cost a whole warp of occupancy per SM
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int grp = lane / N1, k = lane % N1;
  const int col0 = (blockIdx.x * 2 + wib) * C;
  if (col0 >= ncol) return;  // ncol is a multiple of C: warps are all-valid or all-invalid (no block barriers)
  const int col = col0 + grp;
  const int NeZ = op.NeZ, L = op.L;
  const ColLayout lay(N1, NeZ);
  unsigned char* base = smraw + (size_t)(wib * C + grp) * lay.stride;
  Col<N1> c;
  c.P = reinterpret_cast<float*>(base + lay.oP);
  c.sJ = reinterpret_cast<float4*>(base + lay.oSJ);
  c.ring = base + lay.oRing;
  c.del = base + lay.oDel;
  c.Bf = reinterpret_cast<float*>(base + lay.oBf);
  c.bc = reinterpret_cast<float*>(base + lay.oBc);
  c.al = reinterpret_cast<float*>(base + lay.oAl);
  c.jb = reinterpret_cast<float*>(base + lay.oJb);
  c.k = k; c.NeZ = NeZ; c.L = L;
  c.lo_n = (size_t)ncol * L;
  c.lo = gsc + 9 * c.lo_n;  // after the block-Thomas history planes
  c.lo_b = (size_t)col * N1 + k;
  c.lo_s = (size_t)ncol * N1;
  {
    const int ij = col % NF, exy = col / NF;
    const int ci = ij % N1, cj = ij / N1;
    const size_t nxy = (size_t)op.NeX * op.NeY;
    c.gb = (size_t)exy * Np + ci + N1 * cj + NF * k;
    c.gs = nxy * Np;
  }
  const float kapf = ox.kap.x;
  const float iif = (float)args.inv_impl_fac;

  // ---- one pass over the column: alph, the initial iterate, the first residual ----
  // (the MOMX/MOMY solve runs after the DENS/MOMZ/RHOT Newton: it reuses the Newton's shared memory)
  const bool first_a0 = !guess && a0.v[0];
  col_start<N1>(px, kapf, c, z, qin, guess, first_a0 ? a0 : A3{{nullptr, nullptr, nullptr}}, args.impl2);

  // ---- DENS/MOMZ/RHOT Newton ----
  const int gv[3] = {VD, VMZ, VRT};
  const size_t gcolumn = (size_t)col, glayer = (size_t)ncol;  // G history rows of this column
  const GHist gh{gsc, (size_t)ncol * (size_t)L};
  const float cref = (float)args.cref;
  // One call site per routine, which keeps the kernel's code small enough for the instruction
  // caches.  The first residual is not tested (every column takes the first correction); from
  // var0 it was formed by col_start from the stage kernel's A(var0), not by an operator evaluation.
  // Corrections: the first is an LU correction (col_solve); after an LU correction the next one
  // is a truncated Neumann series (col_neumann, when args.neumann > 0), which keeps going while
  // each one cuts the certifying residual at least fourfold; a column whose residual did not
  // contract asks for LU corrections again.  The warp runs an LU correction if any of its active
  // columns asks for one.
  int nsolve = 0, st = 0;
  bool active = true, want_lu = true, last_lu = true;
  float err_prev = 0.f;
  while (true) {
    // the first residual comes from the stage's A(var0) when the iterate starts at var0; every
    // other one is the certifying float-pair residual
    float err = 0.f;
    if (!(nsolve == 0 && first_a0)) err = col_residual<N1>(ox, c, px, qin, args.impl2, cref);
    if (active && nsolve > 0) {
      if (err != err) { st = -2; active = false; }
      else if ((double)err <= args.tol) { st = nsolve; active = false; }
      else if (nsolve >= args.max_iter) { st = -1; active = false; }
    }
    if (!__any_sync(FULL, active)) break;
    if (nsolve > 0) want_lu = args.neumann <= 0 || (!last_lu && !(err <= 0.25f * err_prev));
    err_prev = err;
    last_lu = __any_sync(FULL, active && want_lu);
    if (last_lu) col_solve<N1>(op, px, kapf, c, args.impl_fac, gh, gcolumn, (size_t)col0, glayer, lane, active);
    else col_neumann<N1>(op, px, kapf, c, args.impl_fac, args.neumann, active);
    ++nsolve;
  }
  const unsigned long long once = l2_evict_first();
  float2 qo[3];
  float po[3];  // the trailing parts of the iterate, one element ahead like q*
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    qo[m] = ld_once(qin.v[gv[m]] + c.g(0), once);
    po[m] = *c.plo(m, 0);
  }
  for (int e = 0; e < NeZ; ++e) {
    const int l = e * N1 + k;
    const size_t gi = c.g(e);
    const float2 qc[3] = {qo[0], qo[1], qo[2]};
    const float pc[3] = {po[0], po[1], po[2]};
    {
      const int en = e + 1 < NeZ ? e + 1 : e;
      const size_t gn = c.g(en);
#pragma unroll
      for (int m = 0; m < 3; ++m) {
        qo[m] = ld_once(qin.v[gv[m]] + gn, once);
        po[m] = *c.plo(m, en);
      }
    }
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      const f2 pnew{c.P[3 * l + m], pc[m]};
      const f2 inc = f2_sub(pnew, f2_of(qc[m]));
      if constexpr (PO) {
        st_once(static_cast<float2*>(qsf[gv[m]]) + gi, f2_pack(pnew), once);
        st_once(static_cast<float2*>(tout[gv[m]]) + gi, f2_pack(f2_mul(inc, f2_of(args.inv_impl2))), once);
      } else {
        st_once(static_cast<float*>(qsf[gv[m]]) + gi, f2_to_f(pnew), once);
        st_once(static_cast<float*>(tout[gv[m]]) + gi, f2_to_f(inc) * iif, once);
      }
    }
  }
  // ---- MOMX/MOMY (eval_Ax_uv / solve_uv), after the Newton: its scratch is the Newton's ----
  __syncwarp();  // every lane has stored its DENS/MOMZ/RHOT nodes (c.P is overwritten below)
  // The operator is linear and acts on the face jumps only.  The unknown is E = P - q*, a float
  // pair per node, starting from var0 - q*: b(P) = impl_fac A(q* + E) - E.  The face jumps of q*
  // are formed in pairs once per column; the corrections are FP32 and accumulate into E in pairs,
  // so repeated corrections refine E to pair accuracy.
  {
    float* Eh = c.P;          // [2L] P - q* (float pair): the leading parts; the trailing ones in the
                              // iterate's global planes 0 and 1, free once DENS/MOMZ/RHOT are stored
    float* jq = c.P + 2 * L;  // [4 NeZ] face jumps of q*
    float* bu = c.Bf;                                   // [2L] residual
    // E = var0 - q* at every node; the bottom/top jumps (neighbour - own) of q* MOMX/MOMY from the
    // face nodes' values, passed between lanes by shuffles: jq[4e + m] = q*(e-1, N) - q*(e, 0),
    // jq[4e + 2 + m] = q*(e+1, 0) - q*(e, N), zero at the lids
    double zu[2] = {ld_once(z.v[VMX] + c.g(0), once), ld_once(z.v[VMY] + c.g(0), once)};
    float2 qu[2] = {__ldg(qin.v[VMX] + c.g(0)), __ldg(qin.v[VMY] + c.g(0))};
    f2 qtop[2] = {Z2F, Z2F};  // q*(e-1, N)
    for (int e = 0; e < NeZ; ++e) {
      const int l = e * N1 + k;
      const size_t gn = c.g(e + 1 < NeZ ? e + 1 : e);
      const double zn[2] = {ld_once(z.v[VMX] + gn, once), ld_once(z.v[VMY] + gn, once)};
      const float2 qnx[2] = {__ldg(qin.v[VMX] + gn), __ldg(qin.v[VMY] + gn)};
#pragma unroll
      for (int m = 0; m < 2; ++m) {
        const f2 qs = f2_of(qu[m]);
        const f2 ev = f2_sub(f2_split(zu[m]), qs);
        Eh[2 * l + m] = ev.h;
        *c.plo(m, e) = ev.l;
        const f2 q0{__shfl_sync(FULL, qs.h, 0, N1), __shfl_sync(FULL, qs.l, 0, N1)};
        const f2 qN{__shfl_sync(FULL, qs.h, N, N1), __shfl_sync(FULL, qs.l, N, N1)};
        if (k == 0) {
          jq[4 * e + m] = e == 0 ? 0.f : f2_to_f(f2_sub(qtop[m], q0));
          if (e > 0) jq[4 * (e - 1) + 2 + m] = f2_to_f(f2_sub(q0, qtop[m]));
          if (e == NeZ - 1) jq[4 * e + 2 + m] = 0.f;
        }
        qtop[m] = qN;
        zu[m] = zn[m];
        qu[m] = qnx[m];
      }
    }
    __syncwarp();
    const float cfs = (float)(0.5 * args.impl_fac * op.FSz);
    const float lbk = ox.Lb[k].x, ltk = ox.Lt[k].x;
    const float lb0 = ox.Lb[0].x, lbN = ox.Lb[N].x, lt0 = ox.Lt[0].x, ltN = ox.Lt[N].x;
    const float iscu_c = 1.f / (float)args.cref;
    float* jdel = reinterpret_cast<float*>(c.del);  // 4 jumps of the current element
    bool active = true;
    for (int it = 0; it < 4; ++it) {
      float err = 0.f;
      bool bad = false;
      float el[2] = {*c.plo(0, 0), *c.plo(1, 0)};  // trailing parts of E, one element ahead
      for (int e = 0; e < NeZ; ++e) {
        const float ec[2] = {el[0], el[1]};
        if (e + 1 < NeZ) {
          el[0] = *c.plo(0, e + 1);
          el[1] = *c.plo(1, e + 1);
        }
        for (int t = k; t < 4; t += N1) {
          const int s = t >> 1, m = t & 1;
          const int lM = e * N1 + (s == 0 ? 0 : N);
          const bool lid = s == 0 ? (e == 0) : (e == NeZ - 1);
          const int lP = lid ? lM : (s == 0 ? lM - 1 : lM + 1);
          jdel[t] = jq[4 * e + t] + (Eh[2 * lP + m] - Eh[2 * lM + m]);
        }
        __syncwarp();
        const int l = e * N1 + k;
        const float iscu = iscu_c / __ldg(px.dhf + l);
        const float aB = lbk * c.alB(e), aT = ltk * c.alT(e);
#pragma unroll
        for (int m = 0; m < 2; ++m) {
          const float Af = cfs * (aB * jdel[m] + aT * jdel[2 + m]);  // impl_fac * A(P)
          const float b = (Af - Eh[2 * l + m]) - ec[m];
          bu[2 * l + m] = b;
          err = fmaxf(err, fabsf(b) * iscu);
          bad = bad || !(fabsf(b) < 3.0e38f);
        }
        __syncwarp();
      }
      err = grp_max_nan(bad ? __int_as_float(0x7fc00000) : err, N1);
      const bool need = active && !(err <= args.tol) && it < 3;
      if (!__any_sync(FULL, need)) break;
      // interface jumps J_e = d_e0 - d_{e-1,N} (e = 1..NeZ-1) from the scalar tridiagonal system
      //   (1 + beta_e0 + tau_{e-1,N}) J_e - tau_e0 J_{e+1} - beta_{e-1,N} J_{e-1} = b_e0 - b_{e-1,N}
      // with beta_ep = cfs Lb[p] alB_e, tau_ep = cfs Lt[p] alT_e; then
      //   d_ep = b_ep - beta_ep J_e + tau_ep J_{e+1}   (J_0 = J_NeZ = 0: slip lids)
      float* cp = c.jb;             // [NeZ+1]
      float* Jx = c.jb + (NeZ + 1); // [NeZ+1]
      float* Jy = Jx + (NeZ + 1);   // [NeZ+1]
      if (k == 0) {
        Jx[0] = Jy[0] = 0.f;
        Jx[NeZ] = Jy[NeZ] = 0.f;
        float cprev = 0.f, rxp = 0.f, ryp = 0.f;
        for (int e = 1; e < NeZ; ++e) {
          const float aa = e >= 2 ? -cfs * lbN * c.alB(e - 1) : 0.f;  // -beta_{e-1,N}
          const float dd = 1.f + cfs * lb0 * c.alB(e) + cfs * ltN * c.alT(e - 1);
          const float cc = e < NeZ - 1 ? -cfs * lt0 * c.alT(e) : 0.f;  // -tau_{e,0}
          const float ip = __fdividef(1.f, dd - aa * cprev);
          const float rx = bu[2 * (e * N1)] - bu[2 * ((e - 1) * N1 + N)];
          const float ry = bu[2 * (e * N1) + 1] - bu[2 * ((e - 1) * N1 + N) + 1];
          cprev = cc * ip;
          rxp = (rx - aa * rxp) * ip;
          ryp = (ry - aa * ryp) * ip;
          cp[e] = cprev;
          Jx[e] = rxp;
          Jy[e] = ryp;
        }
        for (int e = NeZ - 2; e >= 1; --e) {
          Jx[e] -= cp[e] * Jx[e + 1];
          Jy[e] -= cp[e] * Jy[e + 1];
        }
      }
      __syncwarp();
      if (need) {
        for (int e0 = 0; e0 < NeZ; e0 += 4) {  // trailing parts loaded four elements at a time
          float lv[4][2];
#pragma unroll
          for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int m = 0; m < 2; ++m) lv[j][m] = e0 + j < NeZ ? *c.plo(m, e0 + j) : 0.f;
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const int e = e0 + j;
            if (e < NeZ) {
              const int l = e * N1 + k;
              const float beta = e > 0 ? cfs * lbk * c.alB(e) : 0.f;
              const float tau = e < NeZ - 1 ? cfs * ltk * c.alT(e) : 0.f;
              const f2 ex = f2_add_f(f2{Eh[2 * l], lv[j][0]}, bu[2 * l] - beta * Jx[e] + tau * Jx[e + 1]);
              const f2 ey = f2_add_f(f2{Eh[2 * l + 1], lv[j][1]}, bu[2 * l + 1] - beta * Jy[e] + tau * Jy[e + 1]);
              Eh[2 * l] = ex.h;
              *c.plo(0, e) = ex.l;
              Eh[2 * l + 1] = ey.h;
              *c.plo(1, e) = ey.l;
            }
          }
        }
      }
      active = need;
      __syncwarp();
    }
    float2 qo[2] = {ld_once(qin.v[VMX] + c.g(0), once), ld_once(qin.v[VMY] + c.g(0), once)};
    float eo[2] = {*c.plo(0, 0), *c.plo(1, 0)};
    for (int e = 0; e < NeZ; ++e) {
      const int l = e * N1 + k;
      const size_t gi = c.g(e);
      const float2 qc[2] = {qo[0], qo[1]};
      const float ec[2] = {eo[0], eo[1]};
      {
        const int en = e + 1 < NeZ ? e + 1 : e;
        const size_t gn = c.g(en);
        qo[0] = ld_once(qin.v[VMX] + gn, once);
        qo[1] = ld_once(qin.v[VMY] + gn, once);
        eo[0] = *c.plo(0, en);
        eo[1] = *c.plo(1, en);
      }
      const f2 dh = f2_of(__ldg(px.dh + l));
#pragma unroll
      for (int m = 0; m < 2; ++m) {
        const f2 ref = f2_mul(dh, f2_of(m == 0 ? ox.Uref : ox.Vref));
        const f2 inc{Eh[2 * l + m], ec[m]};  // P - q*
        const f2 pdev = f2_add(f2_sub(f2_of(qc[m]), ref), inc);
        if constexpr (PO) {
          st_once(static_cast<float2*>(qsf[VMX + m]) + gi, f2_pack(pdev), once);
          st_once(static_cast<float2*>(tout[VMX + m]) + gi, f2_pack(f2_mul(inc, f2_of(args.inv_impl2))), once);
        } else {
          st_once(static_cast<float*>(qsf[VMX + m]) + gi, f2_to_f(pdev), once);
          st_once(static_cast<float*>(tout[VMX + m]) + gi, f2_to_f(inc) * iif, once);
        }
      }
    }
    __syncwarp();
  }
  // the iterate's trailing-part lines of this warp's columns are dead: drop them from L2 without a
  // write-back (one 128-byte line per plane and element)
  for (int i = lane; i < 3 * NeZ; i += 32) {
    const int v = i / NeZ, e = i - v * NeZ;
    const float* a = c.lo + (size_t)v * c.lo_n + ((size_t)col0 + (size_t)e * ncol) * N1;
    asm volatile("discard.global.L2 [%0], 128;" ::"l"(a) : "memory");
  }

  if (k == 0 && status) status[col] = st;
  const unsigned nfail = __reduce_add_sync(FULL, (k == 0 && st < 0) ? 1u : 0u);
  const unsigned nsol = __reduce_add_sync(FULL, (k == 0 && st >= 0) ? (unsigned)st : 0u);
  const unsigned nok = __reduce_add_sync(FULL, (k == 0 && st >= 0) ? 1u : 0u);
  if (lane == 0) {
    if (nfail) atomicAdd(cnt, (unsigned long long)nfail);
    if (nok) {
      atomicAdd(cnt + 1, (unsigned long long)nsol);
      atomicAdd(cnt + 2, (unsigned long long)nok);
    }
  }
}

template <int N1, bool PO>
int launch_n(const Ops& op, const OpsX& ox, const ProfX& px, const X5& qin, const F5c& z, const A3& a0,
             const float* const* guess,
             void* const* qsf, void* const* tout, float* gsc, int* status, unsigned long long* cnt,
             const MixViArgs& a, cudaStream_t s) {
  constexpr int C = 32 / N1;
  const ColLayout lay(N1, op.NeZ);
  const size_t smem = (size_t)lay.stride * 2 * C;
  if (smem > 227 * 1024) return (int)cudaErrorInvalidValue;
  const int ncol = op.NeX * op.NeY * N1 * N1;
  auto kfn = k_vi_cols<N1, PO>;
  // the limit is raised to 227 KB, the same value from every caller: contexts of different column
  // heights launching from several host threads never lower it under one another's launch
  cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
  kfn<<<(ncol + 2 * C - 1) / (2 * C), 64, smem, s>>>(op, ox, px, qin, z, a0, guess, qsf, tout, gsc, status, cnt, a,
                                                     ncol);
  return (int)cudaGetLastError();
}

}  // namespace

size_t vi_cols_scratch_floats(size_t nodes) { return (size_t)12 * nodes; }  // G history 9, iterate 3

int launch_vi_cols(int N1, const Ops& op, const OpsX& ox, const ProfX& px, const X5& qin, const F5c& z,
                   const A3& a0, const float* const* guess, void* const* qsf, void* const* tout, float* gsc, int* status,
                   unsigned long long* cnt, const MixViArgs& a, bool pair_out, cudaStream_t s) {
  switch (N1 * 2 + (pair_out ? 1 : 0)) {
    case 8: return launch_n<4, false>(op, ox, px, qin, z, a0, guess, qsf, tout, gsc, status, cnt, a, s);
    case 9: return launch_n<4, true>(op, ox, px, qin, z, a0, guess, qsf, tout, gsc, status, cnt, a, s);
    case 16: return launch_n<8, false>(op, ox, px, qin, z, a0, guess, qsf, tout, gsc, status, cnt, a, s);
    case 17: return launch_n<8, true>(op, ox, px, qin, z, a0, guess, qsf, tout, gsc, status, cnt, a, s);
  }
  return (int)cudaErrorInvalidValue;
}

}  // namespace fedg
