// fedg_oracle.cpp -- FP64 CPU restatement of the SCALE-DG 3D nonhydrostatic DG
// dynamics step of FElib (ywkawai/FE-Project), used ONLY as test infrastructure:
// the parity checker of the CUDA path and the timed CPU baseline.  Nothing in the
// product library links or calls this file.
//
// Scope (flat cube domain: Gsqrt = 1, GI3 = 0, periodic in x/y, slip lids in z;
// dry air: Rtot = Rdry, CVtot = CVdry, CPtot = CPdry; PRES_hyd_ref = 0 so
// DPhydDx = DPhydDy = 0; constant Coriolis parameter f):
//   * reference element: LGL nodes, orthonormal Legendre Vandermonde, D1D, exact
//     (non-lumped) mass matrix -> tensor-product Lift, VPOrdM1 truncation,
//     exponential modal filter
//       FElib/src/element/scale_element_hexahedral.F90:102-404
//       FElib/src/element/scale_element_operation_tensorprod3D.F90:5464-5569
//       FElib/src/element/scale_element_modalfilter.F90:204-236
//       FElib/src/common/scale_polynomial.F90:250-373
//   * DRHOT -> PRES/DPRES      FElib/src/fluid_dyn_solver/scale_atm_dyn_dgm_nonhydro3d_common.F90:428-479
//   * HEVE cal_tend            ..._nonhydro3d_rhot_heve.F90:292-489
//     HEVE Rusanov face flux   ..._nonhydro3d_rhot_heve_numflux.F90:946-1139
//   * HEVI cal_tend            ..._nonhydro3d_rhot_hevi.F90:289-482
//     HEVI Rusanov face flux   ..._nonhydro3d_rhot_hevi_numflux.F90:232-418
//   * HEVI cal_vi              ..._nonhydro3d_rhot_hevi.F90:772-965
//     eval_Ax / solve / matbnd ..._nonhydro3d_rhot_hevi_common_2.F90:111-1328
//     batched LU (partial piv) ..._hevi_common_linalgebra.F90:2296-2445
//   * slip lid BC              ..._dgm_bnd.F90:270-367
//   * modal filter apply       ..._dgm_modalfilter.F90:49-130
//   * SSP-RK3 / IMEX ARK232    FElib/src/common/scale_timeint_rk.F90:1182-1278, 2201-2565
//                              FElib/src/common/scale_timeint_rk_butcher_tab.F90:200-274
//   * driver stage loop        ..._driver_nonhydro3d.F90:614-963
//   * tracer advection (FCT + TMAR, mass-flux averaging, tracer RK, tracer filter)
//                              ..._trcadvect3d_heve.F90, ..._driver_trcadv3d.F90:330-560
//   * numerical diffusion      ..._nonhydro3d_numdiff.F90:214-721, ..._dgm_bnd.F90:370-508
//   * sponge layer             ..._dgm_spongelayer.F90:134-219
//   * part of a domain split along x and/or y (orc_set_halo): the faces of the boundary elements
//     read the exchanged face layers, filled by a callback before every tendency, as the
//     driver's MeshFieldComm_Exchange does (..._driver_nonhydro3d.F90:768-787,
//     FElib/src/data/scale_meshfieldcomm_base.F90:340-470)
//
// Layout: every field is column-major (Np, Ne) like FElib, node n = i + N1*j + N1^2*k,
// element ke = ex + NeX*ey + NeX*NeY*ez.  Exterior (halo) values are produced in place
// from the neighbour element (periodic) or from the element itself with MOMZ reflected
// (slip lid), which is what FElib's halo exchange + ApplyBC produce on one rank.
//
// The Newton solve of cal_vi has two modes: max_iter = 1 restates FElib exactly (one
// linearised solve from the guess var0); max_iter > 1 iterates the same Newton step
// until the scaled update is below tol (an iterated mode beyond FElib's single solve).

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

enum { VD = 0, VMX = 1, VMY = 2, VMZ = 3, VRT = 4 };  // argument order of cal_tend_ex

struct Const {
  double grav = 9.80616, rdry = 287.04, cpdry = 1004.64, cvdry = 717.6, pres00 = 100000.0;
};

// ---------------------------------------------------------------------------------
// 1D reference element on LGL nodes
// ---------------------------------------------------------------------------------
static double legendre(int n, double x) {
  if (n == 0) return 1.0;
  double p0 = 1.0, p1 = x;
  for (int m = 1; m < n; ++m) {
    double p2 = ((2.0 * m + 1.0) * x * p1 - m * p0) / (m + 1.0);
    p0 = p1; p1 = p2;
  }
  return p1;
}
// derivative of P_n
static double dlegendre(int n, double x) {
  if (n == 0) return 0.0;
  // (1-x^2) P_n' = n (P_{n-1} - x P_n); at interior points only
  return n * (legendre(n - 1, x) - x * legendre(n, x)) / (1.0 - x * x);
}

// LGL nodes: +-1 and the zeros of P_N' (FElib obtains them as Jacobi(1,1) Gauss points by
// dstev, scale_polynomial.F90:250-373); here by Newton iteration on P_N'.
static void lgl_nodes(int N, std::vector<double>& x, std::vector<double>& w) {
  x.assign(N + 1, 0.0); w.assign(N + 1, 0.0);
  x[0] = -1.0; x[N] = 1.0;
  for (int i = 1; i < N; ++i) {
    double xi = -std::cos(M_PI * i / N);
    for (int it = 0; it < 100; ++it) {
      // f = P_N'(x); f' = P_N''(x) = (2x P_N' - N(N+1) P_N)/(1-x^2)
      double f = dlegendre(N, xi);
      double fp = (2.0 * xi * f - N * (N + 1.0) * legendre(N, xi)) / (1.0 - xi * xi);
      double dx = f / fp;
      xi -= dx;
      if (std::fabs(dx) < 1e-17) break;
    }
    x[i] = xi;
  }
  for (int i = 0; i <= N; ++i) {
    double pn = legendre(N, x[i]);
    w[i] = 2.0 / (N * (N + 1.0) * pn * pn);  // scale_polynomial.F90:271-287
  }
}

static void mat_inverse(int n, std::vector<double> a, std::vector<double>& inv) {
  inv.assign(n * n, 0.0);
  for (int i = 0; i < n; ++i) inv[i * n + i] = 1.0;
  for (int c = 0; c < n; ++c) {
    int piv = c;
    for (int r = c + 1; r < n; ++r)
      if (std::fabs(a[r * n + c]) > std::fabs(a[piv * n + c])) piv = r;
    if (piv != c)
      for (int k = 0; k < n; ++k) { std::swap(a[c * n + k], a[piv * n + k]); std::swap(inv[c * n + k], inv[piv * n + k]); }
    double d = 1.0 / a[c * n + c];
    for (int k = 0; k < n; ++k) { a[c * n + k] *= d; inv[c * n + k] *= d; }
    for (int r = 0; r < n; ++r) {
      if (r == c) continue;
      double f = a[r * n + c];
      if (f == 0.0) continue;
      for (int k = 0; k < n; ++k) { a[r * n + k] -= f * a[c * n + k]; inv[r * n + k] -= f * inv[c * n + k]; }
    }
  }
}

struct Elem1D {
  int N = 0, N1 = 0;
  std::vector<double> x, w;
  std::vector<double> V, invV;   // V(i,m) = P_m(x_i) sqrt(m+1/2)   (row-major, [i*N1+m])
  std::vector<double> D;         // D(i,l) = l_l'(x_i)
  std::vector<double> Minv;      // inverse of the exact 1D mass matrix = V V^T
  std::vector<double> F;         // modal filter V diag(sigma) V^-1
  std::vector<double> T;         // truncation of the highest mode V diag(1..1,0) V^-1

  void init(int porder, double etac, double alpha, int ord) {
    N = porder; N1 = porder + 1;
    lgl_nodes(N, x, w);
    V.assign(N1 * N1, 0.0);
    for (int i = 0; i < N1; ++i)
      for (int m = 0; m < N1; ++m) V[i * N1 + m] = legendre(m, x[i]) * std::sqrt(m + 0.5);
    mat_inverse(N1, V, invV);
    // derivative of the Lagrange basis at the LGL nodes (scale_element_hexahedral.F90:256-258)
    D.assign(N1 * N1, 0.0);
    for (int i = 0; i < N1; ++i)
      for (int l = 0; l < N1; ++l) {
        if (i != l) D[i * N1 + l] = legendre(N, x[i]) / (legendre(N, x[l]) * (x[i] - x[l]));
      }
    D[0] = -N * (N + 1.0) / 4.0;
    D[N * N1 + N] = N * (N + 1.0) / 4.0;
    // exact mass matrix M = (V V^T)^-1 (scale_element_base.F90:221-239), so M^-1 = V V^T
    Minv.assign(N1 * N1, 0.0);
    for (int i = 0; i < N1; ++i)
      for (int j = 0; j < N1; ++j) {
        double s = 0.0;
        for (int m = 0; m < N1; ++m) s += V[i * N1 + m] * V[j * N1 + m];
        Minv[i * N1 + j] = s;
      }
    // exponential filter (scale_element_modalfilter.F90:204-236, 60-95)
    std::vector<double> sig(N1, 1.0);
    for (int m = 0; m < N1; ++m) {
      double eta = double(m) / double(N);
      if (eta > etac && m != 0) sig[m] = std::exp(-alpha * std::pow((eta - etac) / (1.0 - etac), ord));
    }
    F.assign(N1 * N1, 0.0);
    T.assign(N1 * N1, 0.0);
    for (int i = 0; i < N1; ++i)
      for (int j = 0; j < N1; ++j) {
        double s = 0.0, t = 0.0;
        for (int m = 0; m < N1; ++m) {
          s += V[i * N1 + m] * sig[m] * invV[m * N1 + j];
          if (m < N1 - 1) t += V[i * N1 + m] * invV[m * N1 + j];  // tensorprod3D.F90:5560-5563
        }
        F[i * N1 + j] = s;
        T[i * N1 + j] = t;
      }
  }
};

// ---------------------------------------------------------------------------------
// the oracle context
// ---------------------------------------------------------------------------------
struct Oracle {
  Const c;
  Elem1D e;
  int N1, Np, Nfp, NfpTot;
  int NeX, NeY, NeZ, Ne;
  double xmin, xmax, ymin, ymax, zmin, zmax, dx, dy, dz;
  double coriolis_f = 0.0;
  int filter_on = 1;
  // base state, (Np, Ne)
  std::vector<double> dens_hyd, pres_hyd, therm_hyd;
  double newton_cref = 340.0;  // velocity scale of the MOMZ convergence test
  // tracer transport outputs of the dynamics step when set (save_massflux, driver_nonhydro3d.F90:900-935):
  // MFLX_x/y/z, alph_dens_M/P, DDENS_TRC, DDENS0_TRC
  double* trc_out[7] = {};
  // sponge layer in the dynamics step when tau > 0 (driver_nonhydro3d.F90:831-841)
  double sl_tau = 0.0, sl_height = 0.0;
  int sl_hvel = 0;
  // part of a domain decomposed along x and/or y (FElib's MeshFieldComm exchange,
  // scale_meshfieldcomm_base.F90:340-470, called by the driver before each tendency,
  // driver_nonhydro3d.F90:768-787): the x-, x+, y-, y+ exterior face layers [6 fields: DDENS, MOMX,
  // MOMY, MOMZ, DRHOT, DPRES][NeY*NeZ (x sides) or NeX*NeZ (y sides)][Nfp], filled by halo_cb before
  // every tendency of a step; NULL on a side whose direction is periodic
  const double* hx[4] = {nullptr, nullptr, nullptr, nullptr};
  void (*halo_cb)(void* user, int stage, const double* const* q, const double* dpres) = nullptr;
  void* halo_user = nullptr;

  size_t nid(int i, int j, int k) const { return (size_t)i + (size_t)N1 * j + (size_t)N1 * N1 * k; }
  size_t eid(int ex, int ey, int ez) const { return (size_t)ex + (size_t)NeX * ey + (size_t)NeX * NeY * ez; }
};

// face node -> (i,j,k) in the element; a,b are the face-local indices
static inline void face_node(int N1, int f, int a, int b, int& i, int& j, int& k) {
  const int N = N1 - 1;
  switch (f) {
    case 0: i = a; j = 0; k = b; break;      // y- (south)
    case 1: i = N; j = a; k = b; break;      // x+ (east)
    case 2: i = a; j = N; k = b; break;      // y+ (north)
    case 3: i = 0; j = a; k = b; break;      // x- (west)
    case 4: i = a; j = b; k = 0; break;      // z- (bottom)
    default: i = a; j = b; k = N; break;     // z+ (top)
  }
}
static const double NX[6] = {0, 1, 0, -1, 0, 0};
static const double NY[6] = {-1, 0, 1, 0, 0, 0};
static const double NZ[6] = {0, 0, 0, 0, -1, 1};

// neighbour element across face f (periodic x/y); returns -1 at a lid
static inline long neighbour(const Oracle& o, int ex, int ey, int ez, int f) {
  switch (f) {
    case 0: return (long)o.eid(ex, (ey - 1 + o.NeY) % o.NeY, ez);
    case 1: return (long)o.eid((ex + 1) % o.NeX, ey, ez);
    case 2: return (long)o.eid(ex, (ey + 1) % o.NeY, ez);
    case 3: return (long)o.eid((ex - 1 + o.NeX) % o.NeX, ey, ez);
    case 4: return ez > 0 ? (long)o.eid(ex, ey, ez - 1) : -1;
    default: return ez < o.NeZ - 1 ? (long)o.eid(ex, ey, ez + 1) : -1;
  }
}
static inline int opposite_face(int f) {
  static const int opp[6] = {2, 3, 0, 1, 5, 4};
  return opp[f];
}

// ---------------------------------------------------------------------------------
// DRHOT -> DPRES (nonhydro3d_common.F90:428-479, CPU branch)
// ---------------------------------------------------------------------------------
static void drhot2pres(const Oracle& o, const double* drhot, double* pres, double* dpres) {
  const double rP0 = 1.0 / o.c.pres00, kap = o.c.cpdry / o.c.cvdry;
  const size_t n = (size_t)o.Np * o.Ne;
#pragma omp parallel for
  for (size_t p = 0; p < n; ++p) {
    double rhot = o.therm_hyd[p] + drhot[p];
    double pr = o.c.pres00 * std::pow(o.c.rdry * rP0 * rhot, kap);
    if (pres) pres[p] = pr;
    dpres[p] = pr - o.pres_hyd[p];
  }
}

// ---------------------------------------------------------------------------------
// explicit tendency: HEVE (hevi = 0) or HEVI (hevi = 1)
// ---------------------------------------------------------------------------------
static void cal_tend(const Oracle& o, int hevi, const double* const q[5], const double* dpres, double* const t[5]) {
  const int N1 = o.N1, Np = o.Np, Nfp = o.Nfp;
  const double gamm = o.c.cpdry / o.c.cvdry;
  const double E11 = 2.0 / o.dx, E22 = 2.0 / o.dy, E33 = 2.0 / o.dz;
  const double FS[6] = {2.0 / o.dy, 2.0 / o.dx, 2.0 / o.dy, 2.0 / o.dx, 2.0 / o.dz, 2.0 / o.dz};
  const std::vector<double>& D = o.e.D;
  const std::vector<double>& Mi = o.e.Minv;
  const std::vector<double>& T = o.e.T;
  const int N = N1 - 1;

#pragma omp parallel
  {
    std::vector<double> flux((size_t)Np * 3 * 5), dfl((size_t)Np * 4 * 5), delf((size_t)Nfp * 6 * 5);
#pragma omp for schedule(static)
    for (long ke = 0; ke < o.Ne; ++ke) {
      const int ex = ke % o.NeX, ey = (ke / o.NeX) % o.NeY, ez = ke / (o.NeX * o.NeY);
      const size_t off = (size_t)ke * Np;
      // --- face flux (numflux get_generalvc) ---
      for (int f = 0; f < 6; ++f) {
        const long kn = neighbour(o, ex, ey, ez, f);
        const int fo = opposite_face(f);
        const double nx = NX[f], ny = NY[f], nz = NZ[f];
        for (int b = 0; b < N1; ++b)
          for (int a = 0; a < N1; ++a) {
            int i, j, k; face_node(N1, f, a, b, i, j, k);
            const size_t iM = off + o.nid(i, j, k);
            size_t iP; double msign = 1.0;
            if (kn >= 0) { int i2, j2, k2; face_node(N1, fo, a, b, i2, j2, k2); iP = (size_t)kn * Np + o.nid(i2, j2, k2); }
            else { iP = iM; msign = -1.0; }  // slip lid: MOMZ reflected (dgm_bnd.F90:323-341)
            // a slab's x boundary: the exterior values come from the exchanged face layer (the base
            // state is horizontally homogeneous, so the exterior node's base values are the own node's)
            const int hsd = (f == 3 && ex == 0) ? 0 : (f == 1 && ex == o.NeX - 1) ? 1 : (f == 0 && ey == 0) ? 2
                          : (f == 2 && ey == o.NeY - 1) ? 3 : -1;
            const double* hs = hsd >= 0 ? o.hx[hsd] : nullptr;
            const size_t hper = (size_t)(hsd < 2 ? o.NeY : o.NeX) * o.NeZ * Nfp;
            const size_t hi = (size_t)(hsd < 2 ? ey + o.NeY * ez : ex + o.NeX * ez) * Nfp + a + N1 * b;
            if (hs) iP = iM;
            const double ddM = q[VD][iM], ddP = hs ? hs[hi] : q[VD][iP];
            const double mxM = q[VMX][iM], mxP = hs ? hs[hper + hi] : q[VMX][iP];
            const double myM = q[VMY][iM], myP = hs ? hs[2 * hper + hi] : q[VMY][iP];
            const double mzM = q[VMZ][iM], mzP = hs ? hs[3 * hper + hi] : msign * q[VMZ][iP];
            const double drM = q[VRT][iM], drP = hs ? hs[4 * hper + hi] : q[VRT][iP];
            const double dpM = dpres[iM], dpP = hs ? hs[5 * hper + hi] : dpres[iP];
            const double densM = ddM + o.dens_hyd[iM], densP = ddP + o.dens_hyd[iP];
            const double rhotM = o.therm_hyd[iM] + drM, rhotP = o.therm_hyd[iP] + drP;
            const double phM = o.pres_hyd[iM], phP = o.pres_hyd[iP];
            const double tmp1 = FS[f] * 0.5;
            const int fp = a + N1 * b;
            double* df = &delf[(size_t)(f * Nfp + fp) * 5];
            if (!hevi) {
              const double velM = (mxM * nx + myM * ny + mzM * nz) / densM;
              const double velP = (mxP * nx + myP * ny + mzP * nz) / densP;
              const double gnn = std::fabs(nx) + std::fabs(ny) + std::fabs(nz);
              const double alpha = std::max(std::sqrt(gnn * gamm * (phM + dpM) / densM) + std::fabs(velM),
                                            std::sqrt(gnn * gamm * (phP + dpP) / densP) + std::fabs(velP));
              df[VD] = tmp1 * (densP * velP - densM * velM - alpha * (ddP - ddM));
              df[VRT] = tmp1 * (rhotP * velP - rhotM * velM - alpha * (drP - drM));
              df[VMZ] = tmp1 * (mzP * velP - mzM * velM + (dpP - dpM) * nz - alpha * (mzP - mzM));
              df[VMX] = tmp1 * (mxP * velP - mxM * velM + nx * (dpP - dpM) - alpha * (mxP - mxM));
              df[VMY] = tmp1 * (myP * velP - myM * velM + ny * (dpP - dpM) - alpha * (myP - myM));
            } else {
              const double velhM = (mxM * nx + myM * ny) / densM;
              const double velhP = (mxP * nx + myP * ny) / densP;
              const double velM = velhM + mzM * nz / densM;
              const double velP = velhP + mzP * nz / densP;
              const double swV = 1.0 - nz * nz;
              const double alpha = swV * std::max(std::sqrt(gamm * (phM + dpM) / densM) + std::fabs(velM),
                                                  std::sqrt(gamm * (phP + dpP) / densP) + std::fabs(velP));
              df[VD] = tmp1 * (densP * velhP - densM * velhM - alpha * (ddP - ddM));
              df[VRT] = tmp1 * (rhotP * velhP - rhotM * velhM - alpha * (drP - drM));
              df[VMZ] = tmp1 * (mzP * velP - mzM * velM - alpha * (mzP - mzM));
              df[VMX] = tmp1 * (mxP * velP - mxM * velM + nx * (dpP - dpM) - alpha * (mxP - mxM));
              df[VMY] = tmp1 * (myP * velP - myM * velM + ny * (dpP - dpM) - alpha * (myP - myM));
            }
          }
      }
      // --- volume fluxes (cal_tend flux build) ---
      for (int p = 0; p < Np; ++p) {
        const size_t g = off + p;
        const double dd = q[VD][g], mx = q[VMX][g], my = q[VMY][g], mz = q[VMZ][g], dr = q[VRT][g], dp = dpres[g];
        const double rdens = 1.0 / (dd + o.dens_hyd[g]);
        double* F = &flux[(size_t)p * 15];  // [dir*5 + var]
        F[0 * 5 + VD] = mx; F[1 * 5 + VD] = my; F[2 * 5 + VD] = mz;
        const double pt = (o.therm_hyd[g] + dr) * rdens;
        F[0 * 5 + VRT] = mx * pt; F[1 * 5 + VRT] = my * pt; F[2 * 5 + VRT] = hevi ? 0.0 : mz * pt;
        const double w = mz * rdens;
        F[0 * 5 + VMZ] = mx * w; F[1 * 5 + VMZ] = my * w; F[2 * 5 + VMZ] = mz * w + (hevi ? 0.0 : dp);
        const double u = mx * rdens, v = my * rdens;
        F[0 * 5 + VMX] = mx * u + dp; F[1 * 5 + VMX] = my * u; F[2 * 5 + VMX] = mz * u;
        F[0 * 5 + VMY] = mx * v; F[1 * 5 + VMY] = my * v + dp; F[2 * 5 + VMY] = mz * v;
      }
      // --- Div_var5: D1D along x, y, z; tensor-product Lift ---
      for (int k = 0; k < N1; ++k)
        for (int j = 0; j < N1; ++j)
          for (int i = 0; i < N1; ++i) {
            const int p = (int)o.nid(i, j, k);
            for (int v = 0; v < 5; ++v) {
              double sx = 0, sy = 0, sz = 0;
              for (int l = 0; l < N1; ++l) {
                sx += D[i * N1 + l] * flux[(size_t)o.nid(l, j, k) * 15 + 0 * 5 + v];
                sy += D[j * N1 + l] * flux[(size_t)o.nid(i, l, k) * 15 + 1 * 5 + v];
                sz += D[k * N1 + l] * flux[(size_t)o.nid(i, j, l) * 15 + 2 * 5 + v];
              }
              // Lift_hexahedral (tensorprod3D_kernel.F90:2316-2339 with Lift_mat of :5512-5569)
              const double lf =
                  Mi[j * N1 + 0] * delf[(size_t)(0 * Nfp + i + N1 * k) * 5 + v] +
                  Mi[i * N1 + N] * delf[(size_t)(1 * Nfp + j + N1 * k) * 5 + v] +
                  Mi[j * N1 + N] * delf[(size_t)(2 * Nfp + i + N1 * k) * 5 + v] +
                  Mi[i * N1 + 0] * delf[(size_t)(3 * Nfp + j + N1 * k) * 5 + v] +
                  Mi[k * N1 + 0] * delf[(size_t)(4 * Nfp + i + N1 * j) * 5 + v] +
                  Mi[k * N1 + N] * delf[(size_t)(5 * Nfp + i + N1 * j) * 5 + v];
              double* d = &dfl[(size_t)p * 20 + v * 4];
              d[0] = sx; d[1] = sy; d[2] = sz; d[3] = lf;
            }
          }
      // --- combine (heve.F90:424-465, hevi.F90:416-478) ---
      for (int k = 0; k < N1; ++k)
        for (int j = 0; j < N1; ++j)
          for (int i = 0; i < N1; ++i) {
            const int p = (int)o.nid(i, j, k);
            const size_t g = off + p;
            const double* d = &dfl[(size_t)p * 20];
            auto full = [&](int v) { return E11 * d[v * 4 + 0] + E22 * d[v * 4 + 1] + E33 * d[v * 4 + 2] + d[v * 4 + 3]; };
            auto horiz = [&](int v) { return E11 * d[v * 4 + 0] + E22 * d[v * 4 + 1] + d[v * 4 + 3]; };
            if (!hevi) {
              t[VD][g] = -full(VD);
              t[VRT][g] = -full(VRT);
              double drho = 0.0;  // VFilterPM1(DDENS) along z
              for (int l = 0; l < N1; ++l) drho += T[k * N1 + l] * q[VD][off + o.nid(i, j, l)];
              t[VMZ][g] = -full(VMZ) - o.c.grav * drho;
            } else {
              t[VD][g] = -horiz(VD);
              t[VRT][g] = -horiz(VRT);
              t[VMZ][g] = -full(VMZ);
            }
            t[VMX][g] = o.coriolis_f * q[VMY][g] - full(VMX);
            t[VMY][g] = -o.coriolis_f * q[VMX][g] - full(VMY);
          }
    }
  }
}

// ---------------------------------------------------------------------------------
// modal filter (dgm_modalfilter.F90:49-130, Gsqrt = 1)
// ---------------------------------------------------------------------------------
static void modal_filter(const Oracle& o, double* const q[5]) {
  const int N1 = o.N1, Np = o.Np;
  const std::vector<double>& F = o.e.F;
#pragma omp parallel
  {
    std::vector<double> a(Np), b(Np);
#pragma omp for schedule(static)
    for (long ke = 0; ke < o.Ne; ++ke)
      for (int v = 0; v < 5; ++v) {
        double* x = q[v] + (size_t)ke * Np;
        for (int k = 0; k < N1; ++k)
          for (int j = 0; j < N1; ++j)
            for (int i = 0; i < N1; ++i) {
              double s = 0;
              for (int l = 0; l < N1; ++l) s += F[i * N1 + l] * x[o.nid(l, j, k)];
              a[o.nid(i, j, k)] = s;
            }
        for (int k = 0; k < N1; ++k)
          for (int j = 0; j < N1; ++j)
            for (int i = 0; i < N1; ++i) {
              double s = 0;
              for (int l = 0; l < N1; ++l) s += F[j * N1 + l] * a[o.nid(i, l, k)];
              b[o.nid(i, j, k)] = s;
            }
        for (int k = 0; k < N1; ++k)
          for (int j = 0; j < N1; ++j)
            for (int i = 0; i < N1; ++i) {
              double s = 0;
              for (int l = 0; l < N1; ++l) s += F[k * N1 + l] * b[o.nid(i, j, l)];
              x[o.nid(i, j, k)] = s;
            }
      }
  }
}

// ---------------------------------------------------------------------------------
// HEVI vertical-implicit solve, one horizontal node column at a time.
// ---------------------------------------------------------------------------------
// LU with partial pivoting of an n x n row-major matrix, solving nrhs right-hand sides
// stored row-major in R (n x nrhs)  (linalgebra.F90:2296-2445 does the same per column).
static void lu_solve(int n, double* A, double* R, int nrhs) {
  for (int k = 0; k < n; ++k) {
    int piv = k;
    double amax = std::fabs(A[k * n + k]);
    for (int r = k + 1; r < n; ++r)
      if (std::fabs(A[r * n + k]) > amax) { amax = std::fabs(A[r * n + k]); piv = r; }
    if (piv != k) {
      for (int c = 0; c < n; ++c) std::swap(A[k * n + c], A[piv * n + c]);
      for (int c = 0; c < nrhs; ++c) std::swap(R[k * nrhs + c], R[piv * nrhs + c]);
    }
    const double rd = 1.0 / A[k * n + k];
    for (int r = k + 1; r < n; ++r) {
      const double f = A[r * n + k] * rd;
      if (f == 0.0) continue;
      A[r * n + k] = f;
      for (int c = k + 1; c < n; ++c) A[r * n + c] -= f * A[k * n + c];
      for (int c = 0; c < nrhs; ++c) R[r * nrhs + c] -= f * R[k * nrhs + c];
    }
  }
  for (int k = n - 1; k >= 0; --k) {
    const double rd = 1.0 / A[k * n + k];
    for (int c = 0; c < nrhs; ++c) {
      double s = R[k * nrhs + c];
      for (int m = k + 1; m < n; ++m) s -= A[k * n + m] * R[m * nrhs + c];
      R[k * nrhs + c] = s * rd;
    }
  }
}

struct ColumnWork {
  // per level (L = NeZ*N1): prognostic iterate, stage input, guess var0, base state
  std::vector<double> P[5], Q[5], Z[5], dh, ph, rh;
  std::vector<double> alphB, alphT;      // vertical-face alph per element (bottom, top)
  std::vector<double> A3;                // eval_Ax output (3, L)
  std::vector<double> b, G, D, Lm, Um, Guv, Duv, Luv, Uuv, buv;
  std::vector<double> W, WT, POT, DPDRHOT;
};

struct ColumnParams {
  double impl_fac, dt, tol;
  int max_iter;
};

// eval_Ax (var3) for the whole column at the current iterate P; fills A3 (-> tendencies),
// and the linearisation fields.  common_2.F90:111-326 and vi_cal_del_flux_dyn :1171-1328.
static void column_eval_Ax(const Oracle& o, ColumnWork& w) {
  const int N1 = o.N1, NeZ = o.NeZ, L = NeZ * N1, N = N1 - 1;
  const double E33 = 2.0 / o.dz, FSz = 2.0 / o.dz;
  const double rP0 = 1.0 / o.c.pres00, kap = o.c.cpdry / o.c.cvdry;
  const std::vector<double>& D = o.e.D;
  const std::vector<double>& Mi = o.e.Minv;
  const std::vector<double>& T = o.e.T;
  std::vector<double> fd(L), fr(L), fm(L), pot(L), dens(L);
  for (int l = 0; l < L; ++l) {
    dens[l] = w.dh[l] + w.P[VD][l];
    const double rhot = w.rh[l] + w.P[VRT][l];
    pot[l] = rhot / dens[l];
    fd[l] = w.P[VMZ][l];                       // MOMW (flat)
    fr[l] = pot[l] * fd[l];
    const double pr = o.c.pres00 * std::pow(o.c.rdry * rP0 * rhot, kap);
    fm[l] = pr - w.ph[l];                      // DPRES
    w.POT[l] = pot[l];
    w.W[l] = w.P[VMZ][l] / dens[l];
    w.WT[l] = fd[l] / dens[l];
    w.DPDRHOT[l] = kap * pr / rhot;
  }
  for (int ez = 0; ez < NeZ; ++ez) {
    // face values: 0 = bottom (nz=-1), 1 = top (nz=+1)
    double del[2][3];
    for (int s = 0; s < 2; ++s) {
      const int lM = ez * N1 + (s == 0 ? 0 : N);
      int lP; bool lid = false;
      if (s == 0) { if (ez > 0) lP = (ez - 1) * N1 + N; else { lP = lM; lid = true; } }
      else { if (ez < NeZ - 1) lP = (ez + 1) * N1; else { lP = lM; lid = true; } }
      const double nz = s == 0 ? -1.0 : 1.0;
      const double alph = s == 0 ? w.alphB[ez] : w.alphT[ez];
      const double ddM = w.P[VD][lM], ddP = w.P[VD][lP];
      const double mzM = w.P[VMZ][lM];
      const double mzP = lid ? -mzM : w.P[VMZ][lP];
      const double mwM = mzM, mwP = lid ? -mzM : w.P[VMZ][lP];
      const double drM = w.P[VRT][lM], drP = w.P[VRT][lP];
      const double tmp1 = 0.5 * FSz;
      del[s][0] = tmp1 * ((mwP - mwM) * nz - alph * (ddP - ddM));
      del[s][1] = tmp1 * ((fm[lP] - fm[lM]) * nz - alph * (mzP - mzM));
      del[s][2] = tmp1 * ((pot[lP] * mwP - pot[lM] * mwM) * nz - alph * (drP - drM));
    }
    for (int k = 0; k < N1; ++k) {
      const int l = ez * N1 + k;
      double sd = 0, sr = 0, sm = 0, drho = 0;
      for (int m = 0; m < N1; ++m) {
        sd += D[k * N1 + m] * fd[ez * N1 + m];
        sr += D[k * N1 + m] * fr[ez * N1 + m];
        sm += D[k * N1 + m] * fm[ez * N1 + m];
        drho += T[k * N1 + m] * w.P[VD][ez * N1 + m];
      }
      const double lb = Mi[k * N1 + 0], lt = Mi[k * N1 + N];
      w.A3[0 * L + l] = -(E33 * sd + lb * del[0][0] + lt * del[1][0]);
      w.A3[1 * L + l] = -(E33 * sm + lb * del[0][1] + lt * del[1][1]) - o.c.grav * drho;
      w.A3[2 * L + l] = -(E33 * sr + lb * del[0][2] + lt * del[1][2]);
    }
  }
}

// MOMX/MOMY implicit tendency -Lift(del_flux_uv) at iterate P (eval_Ax_uv, common_2.F90:482-586)
static void column_eval_Ax_uv(const Oracle& o, ColumnWork& w, std::vector<double>& tx, std::vector<double>& ty) {
  const int N1 = o.N1, NeZ = o.NeZ, N = N1 - 1;
  const double FSz = 2.0 / o.dz;
  const std::vector<double>& Mi = o.e.Minv;
  for (int ez = 0; ez < NeZ; ++ez) {
    double dx_[2], dy_[2];
    for (int s = 0; s < 2; ++s) {
      const int lM = ez * N1 + (s == 0 ? 0 : N);
      int lP;
      if (s == 0) lP = ez > 0 ? (ez - 1) * N1 + N : lM;
      else lP = ez < NeZ - 1 ? (ez + 1) * N1 : lM;
      const double alph = s == 0 ? w.alphB[ez] : w.alphT[ez];
      const double tmp1 = -0.5 * FSz * alph;
      dx_[s] = tmp1 * (w.P[VMX][lP] - w.P[VMX][lM]);
      dy_[s] = tmp1 * (w.P[VMY][lP] - w.P[VMY][lM]);
    }
    for (int k = 0; k < N1; ++k) {
      const double lb = Mi[k * N1 + 0], lt = Mi[k * N1 + N];
      tx[ez * N1 + k] = -(lb * dx_[0] + lt * dx_[1]);
      ty[ez * N1 + k] = -(lb * dy_[0] + lt * dy_[1]);
    }
  }
}

// vertical-face Rusanov speed alph frozen at the guess var0 (w.Z) (vi_cal_del_flux_dyn_uv,
// common_2.F90:1149-1155; Gnn = |nz| = 1 on vertical faces)
static void column_alph(const Oracle& o, ColumnWork& w, int L) {
  const int N1 = o.N1, NeZ = o.NeZ, N = N1 - 1;
  const double rP0 = 1.0 / o.c.pres00, kap = o.c.cpdry / o.c.cvdry;
  std::vector<double> s0(L);
  for (int l = 0; l < L; ++l) {
    const double rdens0 = 1.0 / (w.dh[l] + w.Z[VD][l]);
    const double wt0 = w.Z[VMZ][l] * rdens0;
    const double pres0 = o.c.pres00 * std::pow(o.c.rdry * rP0 * (w.rh[l] + w.Z[VRT][l]), kap);
    s0[l] = std::fabs(wt0) + std::sqrt(kap * pres0 * rdens0);
  }
  for (int ez = 0; ez < NeZ; ++ez) {
    const int lb = ez * N1, lt = ez * N1 + N;
    const int lbP = ez > 0 ? (ez - 1) * N1 + N : lb;
    const int ltP = ez < NeZ - 1 ? (ez + 1) * N1 : lt;
    w.alphB[ez] = std::max(s0[lb], s0[lbP]);
    w.alphT[ez] = std::max(s0[lt], s0[ltP]);
  }
}

// returns the number of Newton iterations used (or -1 if not converged within max_iter)
static int column_solve(const Oracle& o, ColumnWork& w, const ColumnParams& cp, double* tend_out[5], int L) {
  const int N1 = o.N1, NeZ = o.NeZ, N = N1 - 1, n3 = 3 * N1;
  const double E33 = 2.0 / o.dz, FSz = 2.0 / o.dz;
  const double rP0 = 1.0 / o.c.pres00, kap = o.c.cpdry / o.c.cvdry;
  const std::vector<double>& Dm = o.e.D;
  const std::vector<double>& Mi = o.e.Minv;
  const std::vector<double>& T = o.e.T;
  const double impl_fac = cp.impl_fac;

  column_alph(o, w, L);
  for (int v = 0; v < 5; ++v) w.P[v] = w.Z[v];  // PROG_VARS = var0 (hevi.F90:852-872)

  std::vector<double> tx(L), ty(L);
  if (impl_fac == 0.0) {  // hevi.F90:943-961: tendencies of the implicit operator at var0
    column_eval_Ax_uv(o, w, tx, ty);
    column_eval_Ax(o, w);
    for (int l = 0; l < L; ++l) {
      tend_out[VD][l] = w.A3[0 * L + l];
      tend_out[VMZ][l] = w.A3[1 * L + l];
      tend_out[VRT][l] = w.A3[2 * L + l];
      tend_out[VMX][l] = tx[l];
      tend_out[VMY][l] = ty[l];
    }
    return 0;
  }

  // ---- MOMX/MOMY: one linear solve (eval_Ax_uv + solve_uv, common_2.F90:482-689) ----
  column_eval_Ax_uv(o, w, tx, ty);
  {
    const int n = N1;
    std::vector<double>& buv = w.buv;   // (L, 2)
    for (int l = 0; l < L; ++l) {
      buv[l * 2 + 0] = impl_fac * tx[l] - w.P[VMX][l] + w.Q[VMX][l];
      buv[l * 2 + 1] = impl_fac * ty[l] - w.P[VMY][l] + w.Q[VMY][l];
    }
    std::vector<double> Dd(n * n), R(n * 3), Lc(n), Uc(n);
    std::vector<double>& Guv = w.Guv;   // (NeZ, n)
    for (int ez = 0; ez < NeZ; ++ez) {
      std::fill(Dd.begin(), Dd.end(), 0.0);
      for (int p = 0; p < n; ++p) Dd[p * n + p] = 1.0;
      for (int f = 0; f < 2; ++f) {
        const bool bc = (ez == 0 && f == 0) || (ez == NeZ - 1 && f == 1);
        const int pv1 = f == 0 ? 0 : N;
        const double alph = f == 0 ? w.alphB[ez] : w.alphT[ez];
        for (int p = 0; p < n; ++p) {
          const double lift = f == 0 ? Mi[p * N1 + 0] : Mi[p * N1 + N];
          const double tmp1 = 0.5 * impl_fac * lift * FSz * alph;
          if (!bc) {
            Dd[p * n + pv1] += tmp1;
            if (f == 0) Lc[p] = -tmp1; else Uc[p] = -tmp1;
          }
        }
      }
      for (int p = 0; p < n; ++p) {
        const int l = ez * N1 + p;
        if (ez > 0) {
          const double Lv = Lc[p];
          Dd[p * n + 0] -= Lv * Guv[(ez - 1) * n + N];
          buv[l * 2 + 0] -= Lv * buv[((ez - 1) * N1 + N) * 2 + 0];
          buv[l * 2 + 1] -= Lv * buv[((ez - 1) * N1 + N) * 2 + 1];
        }
        R[p * 3 + 0] = buv[l * 2 + 0];
        R[p * 3 + 1] = buv[l * 2 + 1];
        R[p * 3 + 2] = (ez < NeZ - 1) ? Uc[p] : 0.0;
      }
      lu_solve(n, Dd.data(), R.data(), 3);
      for (int p = 0; p < n; ++p) {
        const int l = ez * N1 + p;
        buv[l * 2 + 0] = R[p * 3 + 0];
        buv[l * 2 + 1] = R[p * 3 + 1];
        Guv[ez * n + p] = R[p * 3 + 2];
      }
    }
    for (int ez = NeZ - 2; ez >= 0; --ez)
      for (int p = 0; p < n; ++p) {
        const int l = ez * N1 + p;
        const double g = Guv[ez * n + p];
        buv[l * 2 + 0] -= g * buv[((ez + 1) * N1) * 2 + 0];
        buv[l * 2 + 1] -= g * buv[((ez + 1) * N1) * 2 + 1];
      }
    for (int l = 0; l < L; ++l) { w.P[VMX][l] += buv[l * 2 + 0]; w.P[VMY][l] += buv[l * 2 + 1]; }
  }

  // ---- DENS/MOMZ/RHOT: Newton iterations (eval_Ax + solve, common_2.F90:111-479) ----
  // The FP64 residual b = impl_fac*A(P) - P + q* is evaluated before every solve; with
  // max_iter > 1 the iteration stops once max |b|/scale <= tol (scale: DENS_hyd,
  // DENS_hyd*cref, RHOT_hyd).  max_iter == 1 is FElib's single solve without a test.
  int iters_used = -1;
  int nsolve = 0;
  for (;;) {
    column_eval_Ax(o, w);
    std::vector<double>& b = w.b;  // (NeZ, n3) row index v + 3*pv
    double err = 0.0;
    for (int ez = 0; ez < NeZ; ++ez)
      for (int k = 0; k < N1; ++k) {
        const int l = ez * N1 + k;
        const double bd = impl_fac * w.A3[0 * L + l] - w.P[VD][l] + w.Q[VD][l];
        const double bm = impl_fac * w.A3[1 * L + l] - w.P[VMZ][l] + w.Q[VMZ][l];
        const double br = impl_fac * w.A3[2 * L + l] - w.P[VRT][l] + w.Q[VRT][l];
        b[ez * n3 + 3 * k + 0] = bd;
        b[ez * n3 + 3 * k + 1] = bm;
        b[ez * n3 + 3 * k + 2] = br;
        err = std::max(err, std::fabs(bd) / w.dh[l]);
        err = std::max(err, std::fabs(bm) / (w.dh[l] * o.newton_cref));
        err = std::max(err, std::fabs(br) / w.rh[l]);
      }
    if (!std::isfinite(err)) { iters_used = -2; break; }
    if (cp.max_iter > 1 && err <= cp.tol) { iters_used = nsolve; break; }
    if (nsolve >= cp.max_iter) { iters_used = -1; break; }
    std::vector<double>& G = w.G;           // (NeZ, n3, 3)
    std::vector<double> Dd(n3 * n3), R(n3 * 4), Lc(n3 * 3), Uc(n3 * 3);
    for (int ez = 0; ez < NeZ; ++ez) {
      // construct_matbnd (common_2.F90:693-901)
      std::fill(Dd.begin(), Dd.end(), 0.0);
      std::fill(Lc.begin(), Lc.end(), 0.0);
      std::fill(Uc.begin(), Uc.end(), 0.0);
      auto Dat = [&](int v, int pv, int v2, int pv2) -> double& { return Dd[(v + 3 * pv) * n3 + v2 + 3 * pv2]; };
      for (int pv = 0; pv < N1; ++pv)
        for (int pv2 = 0; pv2 < N1; ++pv2) {
          const int l2 = ez * N1 + pv2;
          const double fdz = E33 * impl_fac * Dm[pv * N1 + pv2];
          const double id = pv == pv2 ? 1.0 : 0.0;
          Dat(0, pv, 0, pv2) = id;
          Dat(0, pv, 1, pv2) = fdz;
          Dat(0, pv, 2, pv2) = 0.0;
          Dat(1, pv, 1, pv2) = id;
          Dat(1, pv, 0, pv2) = impl_fac * o.c.grav * T[pv * N1 + pv2];
          Dat(1, pv, 2, pv2) = fdz * w.DPDRHOT[l2];
          Dat(2, pv, 0, pv2) = -fdz * w.POT[l2] * w.WT[l2];
          Dat(2, pv, 1, pv2) = fdz * w.POT[l2];
          Dat(2, pv, 2, pv2) = id + fdz * w.WT[l2];
        }
      for (int f = 0; f < 2; ++f) {
        const bool bc = (ez == 0 && f == 0) || (ez == NeZ - 1 && f == 1);
        const int pv1 = f == 0 ? 0 : N;
        const int ezn = f == 0 ? std::max(ez - 1, 0) : std::min(ez + 1, NeZ - 1);
        const int pvn = bc ? pv1 : (f == 0 ? N : 0);
        const int l1 = ez * N1 + pv1, ln = ezn * N1 + pvn;
        const double nz = f == 0 ? -1.0 : 1.0;
        const double alph = f == 0 ? w.alphB[ez] : w.alphT[ez];
        for (int pv = 0; pv < N1; ++pv) {
          const double lift = f == 0 ? Mi[pv * N1 + 0] : Mi[pv * N1 + N];
          const double fac = 0.5 * impl_fac * lift * FSz;
          const double tmp1 = fac * alph, tmp2 = fac * nz;
          if (bc) {
            Dat(2, pv, 0, pv1) += 2.0 * tmp2 * w.POT[l1] * w.WT[l1];
            Dat(0, pv, 1, pv1) -= 2.0 * tmp2;
            Dat(1, pv, 1, pv1) += 2.0 * tmp1;
            Dat(2, pv, 1, pv1) -= 2.0 * tmp2 * w.POT[l1];
            Dat(2, pv, 2, pv1) -= 2.0 * tmp2 * w.WT[l1];
          } else {
            Dat(0, pv, 0, pv1) += tmp1;
            Dat(2, pv, 0, pv1) += tmp2 * w.POT[l1] * w.WT[l1];
            Dat(0, pv, 1, pv1) -= tmp2;
            Dat(1, pv, 1, pv1) += tmp1;
            Dat(2, pv, 1, pv1) -= tmp2 * w.POT[l1];
            Dat(1, pv, 2, pv1) -= tmp2 * w.DPDRHOT[l1];
            Dat(2, pv, 2, pv1) += tmp1 - tmp2 * w.WT[l1];
            std::vector<double>& C = f == 0 ? Lc : Uc;  // (n3, 3): [row*3 + var of the neighbour node]
            C[(0 + 3 * pv) * 3 + 0] = -tmp1;
            C[(1 + 3 * pv) * 3 + 0] = 0.0;
            C[(2 + 3 * pv) * 3 + 0] = -tmp2 * w.POT[ln] * w.WT[ln];
            C[(0 + 3 * pv) * 3 + 1] = tmp2;
            C[(1 + 3 * pv) * 3 + 1] = -tmp1;
            C[(2 + 3 * pv) * 3 + 1] = tmp2 * w.POT[ln];
            C[(0 + 3 * pv) * 3 + 2] = 0.0;
            C[(1 + 3 * pv) * 3 + 2] = tmp2 * w.DPDRHOT[ln];
            C[(2 + 3 * pv) * 3 + 2] = -tmp1 + tmp2 * w.WT[ln];
          }
        }
      }
      // block-Thomas forward elimination (common_2.F90:390-430)
      if (ez > 0) {
        const int p1 = 3 * N;
        for (int r = 0; r < n3; ++r) {
          for (int c2 = 0; c2 < 3; ++c2) {
            double s = 0;
            for (int m = 0; m < 3; ++m) s += Lc[r * 3 + m] * G[((ez - 1) * n3 + p1 + m) * 3 + c2];
            Dd[r * n3 + c2] -= s;
          }
          double s = 0;
          for (int m = 0; m < 3; ++m) s += Lc[r * 3 + m] * b[(ez - 1) * n3 + p1 + m];
          b[ez * n3 + r] -= s;
        }
      }
      for (int r = 0; r < n3; ++r) {
        R[r * 4 + 0] = b[ez * n3 + r];
        for (int m = 0; m < 3; ++m) R[r * 4 + 1 + m] = (ez < NeZ - 1) ? Uc[r * 3 + m] : 0.0;
      }
      lu_solve(n3, Dd.data(), R.data(), 4);
      for (int r = 0; r < n3; ++r) {
        b[ez * n3 + r] = R[r * 4 + 0];
        for (int m = 0; m < 3; ++m) G[(ez * n3 + r) * 3 + m] = R[r * 4 + 1 + m];
      }
    }
    for (int ez = NeZ - 2; ez >= 0; --ez)  // back substitution (common_2.F90:443-458)
      for (int r = 0; r < n3; ++r) {
        double s = 0;
        for (int m = 0; m < 3; ++m) s += G[(ez * n3 + r) * 3 + m] * b[(ez + 1) * n3 + m];
        b[ez * n3 + r] -= s;
      }
    for (int ez = 0; ez < NeZ; ++ez)
      for (int k = 0; k < N1; ++k) {
        const int l = ez * N1 + k;
        w.P[VD][l] += b[ez * n3 + 3 * k + 0];
        w.P[VMZ][l] += b[ez * n3 + 3 * k + 1];
        w.P[VRT][l] += b[ez * n3 + 3 * k + 2];
      }
    ++nsolve;
    if (cp.max_iter == 1) { iters_used = 1; break; }
  }
  // tend_im = (PROG - q)/impl_fac  (hevi.F90:931-942)
  for (int v = 0; v < 5; ++v)
    for (int l = 0; l < L; ++l) tend_out[v][l] = (w.P[v][l] - w.Q[v][l]) / impl_fac;
  return iters_used;
}

// cal_vi over all columns; returns #non-converged columns; iters histogram optional
static long cal_vi(const Oracle& o, const double* const q[5], const double* const q0[5], double impl_fac,
                   double dt, int max_iter, double tol, double* const tend[5], int* col_iters) {
  const int N1 = o.N1, NeZ = o.NeZ, L = NeZ * N1, n3 = 3 * N1;
  const double rgamm = o.c.cvdry / o.c.cpdry;
  const long ncol = (long)o.NeX * o.NeY * N1 * N1;
  long nfail = 0;
  ColumnParams cp{impl_fac, dt, tol, max_iter};
#pragma omp parallel reduction(+ : nfail)
  {
    ColumnWork w;
    for (int v = 0; v < 5; ++v) { w.P[v].resize(L); w.Q[v].resize(L); w.Z[v].resize(L); }
    w.dh.resize(L); w.ph.resize(L); w.rh.resize(L);
    w.alphB.resize(NeZ); w.alphT.resize(NeZ);
    w.A3.resize(3 * L); w.b.resize(NeZ * n3); w.G.resize(NeZ * n3 * 3);
    w.buv.resize(L * 2); w.Guv.resize(NeZ * N1);
    w.W.resize(L); w.WT.resize(L); w.POT.resize(L); w.DPDRHOT.resize(L);
    std::vector<double> tout[5];
    for (int v = 0; v < 5; ++v) tout[v].resize(L);
    double* tp[5];
    for (int v = 0; v < 5; ++v) tp[v] = tout[v].data();
    std::vector<size_t> gidx(L);
#pragma omp for schedule(dynamic, 16)
    for (long c = 0; c < ncol; ++c) {
      const int ij = c % (N1 * N1);
      const long exy = c / (N1 * N1);
      const int i = ij % N1, j = ij / N1;
      const int ex = exy % o.NeX, ey = exy / o.NeX;
      for (int ez = 0; ez < NeZ; ++ez)
        for (int k = 0; k < N1; ++k) gidx[ez * N1 + k] = o.eid(ex, ey, ez) * o.Np + o.nid(i, j, k);
      for (int l = 0; l < L; ++l) {
        const size_t g = gidx[l];
        for (int v = 0; v < 5; ++v) { w.Q[v][l] = q[v][g]; w.Z[v][l] = q0[v][g]; }
        w.dh[l] = o.dens_hyd[g];
        w.ph[l] = o.pres_hyd[g];
        w.rh[l] = o.c.pres00 / o.c.rdry * std::pow(w.ph[l] / o.c.pres00, rgamm);
      }
      const int its = column_solve(o, w, cp, tp, L);
      if (its < 0) ++nfail;
      if (col_iters) col_iters[c] = its;
      for (int l = 0; l < L; ++l)
        for (int v = 0; v < 5; ++v) tend[v][gidx[l]] = tout[v][l];
    }
  }
  return nfail;
}

// The implicit operator A(P) of every column (eval_Ax for DENS/MOMZ/RHOT, eval_Ax_uv for MOMX/MOMY,
// common_2.F90:111-326, 482-586) with the vertical Rusanov speed frozen at q0 and the iterate P free.
// Test infrastructure for checking the Newton solve against a finite-difference Jacobian of A.
static void vi_operator(const Oracle& o, const double* const P[5], const double* const q0[5], double* const out[5]) {
  const int N1 = o.N1, NeZ = o.NeZ, L = NeZ * N1;
  const double rgamm = o.c.cvdry / o.c.cpdry;
  const long ncol = (long)o.NeX * o.NeY * N1 * N1;
#pragma omp parallel
  {
    ColumnWork w;
    for (int v = 0; v < 5; ++v) { w.P[v].resize(L); w.Z[v].resize(L); }
    w.dh.resize(L); w.ph.resize(L); w.rh.resize(L);
    w.alphB.resize(NeZ); w.alphT.resize(NeZ);
    w.A3.resize(3 * L);
    w.W.resize(L); w.WT.resize(L); w.POT.resize(L); w.DPDRHOT.resize(L);
    std::vector<double> tx(L), ty(L);
    std::vector<size_t> gidx(L);
#pragma omp for schedule(dynamic, 16)
    for (long c = 0; c < ncol; ++c) {
      const int ij = c % (N1 * N1);
      const long exy = c / (N1 * N1);
      const int i = ij % N1, j = ij / N1;
      const int ex = exy % o.NeX, ey = exy / o.NeX;
      for (int ez = 0; ez < NeZ; ++ez)
        for (int k = 0; k < N1; ++k) gidx[ez * N1 + k] = o.eid(ex, ey, ez) * o.Np + o.nid(i, j, k);
      for (int l = 0; l < L; ++l) {
        const size_t g = gidx[l];
        for (int v = 0; v < 5; ++v) { w.P[v][l] = P[v][g]; w.Z[v][l] = q0[v][g]; }
        w.dh[l] = o.dens_hyd[g];
        w.ph[l] = o.pres_hyd[g];
        w.rh[l] = o.c.pres00 / o.c.rdry * std::pow(w.ph[l] / o.c.pres00, rgamm);
      }
      column_alph(o, w, L);
      column_eval_Ax_uv(o, w, tx, ty);
      column_eval_Ax(o, w);
      for (int l = 0; l < L; ++l) {
        const size_t g = gidx[l];
        out[VD][g] = w.A3[0 * L + l];
        out[VMZ][g] = w.A3[1 * L + l];
        out[VRT][g] = w.A3[2 * L + l];
        out[VMX][g] = tx[l];
        out[VMY][g] = ty[l];
      }
    }
  }
}

// ---------------------------------------------------------------------------------
// Tracer advection: HEVE DG transport of a mixing ratio by a (time-averaged) mass flux, with the
// nonnegativity limiter of Light and Durran (2016): FCT on the lowest mode, then truncation and
// mass-aware rescaling (TMAR).
//   alphDens (advection test)  FElib/src/fluid_dyn_solver/scale_atm_dyn_dgm_trcadvect3d_heve.F90:404-455
//   save_massflux + alphDens   ..._trcadvect3d_heve.F90:343-401, 460-551
//   FCT coefficient            ..._trcadvect3d_heve.F90:234-306, net outward flux :678-777
//   cal_tend + del_flux        ..._trcadvect3d_heve.F90:149-231, 554-674
//   TMAR                       ..._trcadvect3d_heve.F90:311-340
//   face integration weights   ..._trcadvect3d_heve.F90:75-137
//   tracer modal filter        ..._dgm_modalfilter.F90:232-270
//   tracer RK (low storage)    FElib/src/common/scale_timeint_rk.F90:1390-1498
//   driver (one tracer)        ..._driver_trcadv3d.F90:420-545
// Flat cube: Gsqrt = GsqrtH = 1, G13 = G23 = 0, G11 = G22 = 1, J = dx dy dz / 8, and
// J * Fscale = the face Jacobian (dy dz / 4 on x faces, ...).  Face-node arrays are FElib's
// (NfpTot, Ne): face f, node a + N1*b (the face_node order above).  At a slip lid the exterior
// node is the element's own node with the vertical mass flux / momentum reflected.
// ---------------------------------------------------------------------------------
struct TrcFilter {
  std::vector<double> Fh, Fv;  // 1D tracer modal filters (horizontal, vertical)
};

static void exp_filter_matrix(const Elem1D& e, double etac, double alpha, int ord, std::vector<double>& F) {
  const int N1 = e.N1, N = e.N;
  std::vector<double> sig(N1, 1.0);
  for (int m = 0; m < N1; ++m) {
    const double eta = double(m) / double(N);
    if (eta > etac && m != 0) sig[m] = std::exp(-alpha * std::pow((eta - etac) / (1.0 - etac), ord));
  }
  F.assign(N1 * N1, 0.0);
  for (int i = 0; i < N1; ++i)
    for (int j = 0; j < N1; ++j) {
      double s = 0.0;
      for (int m = 0; m < N1; ++m) s += e.V[i * N1 + m] * sig[m] * e.invV[m * N1 + j];
      F[i * N1 + j] = s;
    }
}

// exterior node of face node (f, a, b) of element ke; lid = slip lid (own node, reflected)
static inline size_t ext_node(const Oracle& o, long ke, int f, int a, int b, bool& lid) {
  const int ex = (int)(ke % o.NeX), ey = (int)((ke / o.NeX) % o.NeY), ez = (int)(ke / ((long)o.NeX * o.NeY));
  const long kn = neighbour(o, ex, ey, ez, f);
  int i, j, k;
  if (kn >= 0) {
    lid = false;
    face_node(o.N1, opposite_face(f), a, b, i, j, k);
    return (size_t)kn * o.Np + o.nid(i, j, k);
  }
  lid = true;
  face_node(o.N1, f, a, b, i, j, k);
  return (size_t)ke * o.Np + o.nid(i, j, k);
}

// cal_alphdens_advtest: alph_dens = max(|v_n^-|, |v_n^+|) * dens * Gsqrt on each side
static void trc_alphdens_advtest(const Oracle& o, const double* ddens, const double* momx, const double* momy,
                                 const double* momz, double* aM, double* aP) {
  const int N1 = o.N1, Nfp = o.Nfp;
#pragma omp parallel for schedule(static)
  for (long ke = 0; ke < o.Ne; ++ke)
    for (int f = 0; f < 6; ++f)
      for (int b = 0; b < N1; ++b)
        for (int a = 0; a < N1; ++a) {
          int i, j, k; face_node(N1, f, a, b, i, j, k);
          const size_t iM = (size_t)ke * o.Np + o.nid(i, j, k);
          bool lid; const size_t iP = ext_node(o, ke, f, a, b, lid);
          const double densM = ddens[iM] + o.dens_hyd[iM], densP = ddens[iP] + o.dens_hyd[iP];
          const double mzP = lid ? -momz[iP] : momz[iP];
          const double velM = (momx[iM] * NX[f] + momy[iM] * NY[f] + momz[iM] * NZ[f]) / densM;
          const double velP = (momx[iP] * NX[f] + momy[iP] * NY[f] + mzP * NZ[f]) / densP;
          const double alpha = std::max(std::fabs(velM), std::fabs(velP));
          const size_t fi = (size_t)ke * 6 * Nfp + f * Nfp + a + N1 * b;
          aM[fi] = alpha * densM;
          aP[fi] = alpha * densP;
        }
}

// save_massflux: time average of the mass flux over the dynamics RK stages and of the Rusanov
// coefficient of the dynamics (alphdens_dyn), weights w_h (horizontal) and w_v (vertical)
static void trc_save_massflux(const Oracle& o, int rkstage, const double* const q[5], const double* dpres,
                              double w_h, double w_v, int is_hevi, double* const mflx[3], double* aM, double* aP) {
  const int N1 = o.N1, Nfp = o.Nfp;
  const size_t n = (size_t)o.Np * o.Ne;
  const double gamm = o.c.cpdry / o.c.cvdry;
#pragma omp parallel for schedule(static)
  for (size_t p = 0; p < n; ++p) {
    if (rkstage == 1) {
      mflx[0][p] = w_h * q[VMX][p]; mflx[1][p] = w_h * q[VMY][p]; mflx[2][p] = w_v * q[VMZ][p];
    } else {
      mflx[0][p] += w_h * q[VMX][p]; mflx[1][p] += w_h * q[VMY][p]; mflx[2][p] += w_v * q[VMZ][p];
    }
  }
#pragma omp parallel for schedule(static)
  for (long ke = 0; ke < o.Ne; ++ke)
    for (int f = 0; f < 6; ++f)
      for (int b = 0; b < N1; ++b)
        for (int a = 0; a < N1; ++a) {
          int i, j, k; face_node(N1, f, a, b, i, j, k);
          const size_t iM = (size_t)ke * o.Np + o.nid(i, j, k);
          bool lid; const size_t iP = ext_node(o, ke, f, a, b, lid);
          const double nx = NX[f], ny = NY[f], nz = NZ[f];
          const double densM = q[VD][iM] + o.dens_hyd[iM], densP = q[VD][iP] + o.dens_hyd[iP];
          const double gnn = std::fabs(nx) + std::fabs(ny) + (is_hevi ? 0.0 : std::fabs(nz));
          const double mzP = lid ? -q[VMZ][iP] : q[VMZ][iP];
          const double velM = (q[VMX][iM] * nx + q[VMY][iM] * ny + q[VMZ][iM] * nz) / densM;
          const double velP = (q[VMX][iP] * nx + q[VMY][iP] * ny + mzP * nz) / densP;
          const double alpha = std::max(std::sqrt(gnn * gamm * (o.pres_hyd[iM] + dpres[iM]) / densM) + std::fabs(velM),
                                        std::sqrt(gnn * gamm * (o.pres_hyd[iP] + dpres[iP]) / densP) + std::fabs(velP));
          const double tw = w_h * (std::fabs(nx) + std::fabs(ny)) + w_v * std::fabs(nz);
          const size_t fi = (size_t)ke * 6 * Nfp + f * Nfp + a + N1 * b;
          if (rkstage == 1) { aM[fi] = 0.0; aP[fi] = 0.0; }
          aM[fi] += tw * alpha * densM;
          aP[fi] += tw * alpha * densP;
        }
}

// Rusanov numerical flux of the tracer at every face node of element ke, the outward normal mass
// flux of the interior side, and the face integrals of J*Fscale*numflux (FaceIntMat)
static void trc_face(const Oracle& o, long ke, const double* Q, const double* const mflx[3], const double* aM,
                     const double* aP, double* numflux, double* momflxM, double* outflux) {
  const int N1 = o.N1, Nfp = o.Nfp;
  const double J = o.dx * o.dy * o.dz / 8.0;
  const double FS[6] = {2.0 / o.dy, 2.0 / o.dx, 2.0 / o.dy, 2.0 / o.dx, 2.0 / o.dz, 2.0 / o.dz};
  const std::vector<double>& w = o.e.w;
  for (int f = 0; f < 6; ++f) {
    double s = 0.0;
    for (int b = 0; b < N1; ++b)
      for (int a = 0; a < N1; ++a) {
        int i, j, k; face_node(N1, f, a, b, i, j, k);
        const size_t iM = (size_t)ke * o.Np + o.nid(i, j, k);
        bool lid; const size_t iP = ext_node(o, ke, f, a, b, lid);
        const double mzP = lid ? -mflx[2][iP] : mflx[2][iP];
        const double mfM = mflx[0][iM] * NX[f] + mflx[1][iM] * NY[f] + mflx[2][iM] * NZ[f];
        const double mfP = mflx[0][iP] * NX[f] + mflx[1][iP] * NY[f] + mzP * NZ[f];
        const int fp = f * Nfp + a + N1 * b;
        const size_t fi = (size_t)ke * 6 * Nfp + fp;
        const double qM = Q[iM], qP = Q[iP];
        const double nf = 0.5 * ((qP * mfP + qM * mfM) - aP[fi] * qP + aM[fi] * qM);
        numflux[fp] = nf;
        momflxM[fp] = mfM;
        s += w[a] * w[b] * (J * FS[f] * nf);
      }
    outflux[f] = s;
  }
}

// calc_fct_coef: the largest fraction of the element's outflow its own mass can supply in one
// stage, written to all Np nodes of the element (a nodal field, as in FElib)
static void trc_fct_coef(const Oracle& o, const double* Q, const double* const mflx[3], const double* rhoq_tp,
                         const double* aM, const double* aP, const double* ddens, const double* ddens0, double c_ssm1,
                         double dt, double* fct) {
  const int N1 = o.N1, Np = o.Np, Nfp = o.Nfp;
  const double J = o.dx * o.dy * o.dz / 8.0;
  const std::vector<double>& w = o.e.w;
#pragma omp parallel
  {
    std::vector<double> nf(6 * Nfp), mf(6 * Nfp);
    double out[6];
#pragma omp for schedule(static)
    for (long ke = 0; ke < o.Ne; ++ke) {
      trc_face(o, ke, Q, mflx, aM, aP, nf.data(), mf.data(), out);
      double net = 0.0;
      for (int f = 0; f < 6; ++f) net += std::max(0.0, out[f]);
      double qe = 0.0;
      for (int k = 0; k < N1; ++k)
        for (int j = 0; j < N1; ++j)
          for (int i = 0; i < N1; ++i) {
            const size_t g = (size_t)ke * Np + o.nid(i, j, k);
            const double dens = o.dens_hyd[g] + (1.0 - c_ssm1) * ddens0[g] + c_ssm1 * ddens[g];
            qe += J * (w[i] * w[j] * w[k]) * (dens * Q[g] / dt + (rhoq_tp ? rhoq_tp[g] : 0.0));
          }
      const double r = std::max(0.0, std::min(1.0, qe / (net + 1.0e-10)));
      for (int p = 0; p < Np; ++p) fct[(size_t)ke * Np + p] = r;
    }
  }
}

// cal_tend with the FCT-limited del_flux: d(dens q)/dt.  fct is the nodal coefficient field; the
// face value on each side is read at the face node (at a lid both sides are the element's own node)
static void trc_cal_tend(const Oracle& o, const double* Q, const double* const mflx[3], const double* aM,
                         const double* aP, const double* fct, const double* rhoq_tp, double* Qdt) {
  const int N1 = o.N1, Np = o.Np, Nfp = o.Nfp, N = N1 - 1;
  const double E11 = 2.0 / o.dx, E22 = 2.0 / o.dy, E33 = 2.0 / o.dz;
  const double FS[6] = {2.0 / o.dy, 2.0 / o.dx, 2.0 / o.dy, 2.0 / o.dx, 2.0 / o.dz, 2.0 / o.dz};
  const std::vector<double>& D = o.e.D;
  const std::vector<double>& Mi = o.e.Minv;
#pragma omp parallel
  {
    std::vector<double> nf(6 * Nfp), mf(6 * Nfp), delf(6 * Nfp), fl(3 * (size_t)Np);
    double out[6];
#pragma omp for schedule(static)
    for (long ke = 0; ke < o.Ne; ++ke) {
      trc_face(o, ke, Q, mflx, aM, aP, nf.data(), mf.data(), out);
      for (int f = 0; f < 6; ++f) {
        // 0.5 (R+ + R- - (R+ - R-) sign(1, outflux)): R- on outflow faces, R+ on inflow faces
        const double sg = std::signbit(out[f]) ? -1.0 : 1.0;
        for (int b = 0; b < N1; ++b)
          for (int a = 0; a < N1; ++a) {
            int i, j, k; face_node(N1, f, a, b, i, j, k);
            const size_t iM = (size_t)ke * Np + o.nid(i, j, k);
            bool lid; const size_t iP = ext_node(o, ke, f, a, b, lid);
            const double RM = fct[iM], RP = fct[iP];
            const int fp = f * Nfp + a + N1 * b;
            delf[fp] = FS[f] * (nf[fp] * (0.5 * (RP + RM - (RP - RM) * sg)) - Q[iM] * mf[fp]);
          }
      }
      for (int p = 0; p < Np; ++p) {
        const size_t g = (size_t)ke * Np + p;
        fl[p] = mflx[0][g] * Q[g];
        fl[Np + p] = mflx[1][g] * Q[g];
        fl[2 * Np + p] = mflx[2][g] * Q[g];
      }
      for (int k = 0; k < N1; ++k)
        for (int j = 0; j < N1; ++j)
          for (int i = 0; i < N1; ++i) {
            double sx = 0, sy = 0, sz = 0;
            for (int l = 0; l < N1; ++l) {
              sx += D[i * N1 + l] * fl[o.nid(l, j, k)];
              sy += D[j * N1 + l] * fl[Np + o.nid(i, l, k)];
              sz += D[k * N1 + l] * fl[2 * Np + o.nid(i, j, l)];
            }
            const double lf = Mi[j * N1 + 0] * delf[0 * Nfp + i + N1 * k] + Mi[i * N1 + N] * delf[1 * Nfp + j + N1 * k] +
                              Mi[j * N1 + N] * delf[2 * Nfp + i + N1 * k] + Mi[i * N1 + 0] * delf[3 * Nfp + j + N1 * k] +
                              Mi[k * N1 + 0] * delf[4 * Nfp + i + N1 * j] + Mi[k * N1 + N] * delf[5 * Nfp + i + N1 * j];
            const size_t g = (size_t)ke * Np + o.nid(i, j, k);
            Qdt[g] = -(E11 * sx + E22 * sy + E33 * sz + lf) + (rhoq_tp ? rhoq_tp[g] : 0.0);
          }
    }
  }
}

// TMAR: truncate negative values, rescale to keep the element's tracer mass
static void trc_tmar(const Oracle& o, double* Q, const double* ddens) {
  const int N1 = o.N1, Np = o.Np;
  const std::vector<double>& w = o.e.w;
  const double J = o.dx * o.dy * o.dz / 8.0;
#pragma omp parallel for schedule(static)
  for (long ke = 0; ke < o.Ne; ++ke) {
    double q0 = 0.0, q1 = 0.0;
    for (int k = 0; k < N1; ++k)
      for (int j = 0; j < N1; ++j)
        for (int i = 0; i < N1; ++i) {
          const size_t g = (size_t)ke * Np + o.nid(i, j, k);
          const double wd = J * (w[i] * w[j] * w[k]) * (o.dens_hyd[g] + ddens[g]);
          q0 += wd * Q[g];
          q1 += wd * std::max(0.0, Q[g]);
        }
    const double r = q0 / (q1 + 1.0e-32);
    for (int p = 0; p < Np; ++p) {
      const size_t g = (size_t)ke * Np + p;
      Q[g] = r * std::max(0.0, Q[g]);
    }
  }
}

// tracer modal filter: Q <- F(dens Q) / dens with dens = Gsqrt (DENS_hyd + DDENS)
static void trc_filter(const Oracle& o, const TrcFilter& tf, double* Q, const double* ddens) {
  const int N1 = o.N1, Np = o.Np;
#pragma omp parallel
  {
    std::vector<double> a(Np), b(Np), wt(Np);
#pragma omp for schedule(static)
    for (long ke = 0; ke < o.Ne; ++ke) {
      double* x = Q + (size_t)ke * Np;
      for (int p = 0; p < Np; ++p) {
        const size_t g = (size_t)ke * Np + p;
        wt[p] = o.dens_hyd[g] + ddens[g];
        b[p] = wt[p] * x[p];
      }
      for (int k = 0; k < N1; ++k)
        for (int j = 0; j < N1; ++j)
          for (int i = 0; i < N1; ++i) {
            double s = 0;
            for (int l = 0; l < N1; ++l) s += tf.Fh[i * N1 + l] * b[o.nid(l, j, k)];
            a[o.nid(i, j, k)] = s;
          }
      for (int k = 0; k < N1; ++k)
        for (int j = 0; j < N1; ++j)
          for (int i = 0; i < N1; ++i) {
            double s = 0;
            for (int l = 0; l < N1; ++l) s += tf.Fh[j * N1 + l] * a[o.nid(i, l, k)];
            b[o.nid(i, j, k)] = s;
          }
      for (int k = 0; k < N1; ++k)
        for (int j = 0; j < N1; ++j)
          for (int i = 0; i < N1; ++i) {
            double s = 0;
            for (int l = 0; l < N1; ++l) s += tf.Fv[k * N1 + l] * b[o.nid(i, j, l)];
            x[o.nid(i, j, k)] = s / wt[o.nid(i, j, k)];
          }
    }
  }
}

// One tracer time step of the tracer driver with a low-storage explicit RK scheme given by its
// Shu-Osher coefficients sig(s+1, s'), gam(s+1, s') (row-major [(nstage+1) x nstage], rows 1..nstage
// used) and nodes c(s): the FCT coefficient, the tendency, the density-weighted advance
// (rk_advance_trcvar_low_storage), then after the last stage the tracer filter and TMAR, and the
// final rescale QTRC = (DENS_hyd + DDENS_TRC) / (DENS_hyd + DDENS) QTRC_tmp.
struct TrcStepArgs {
  int nstage;
  const double* sig;  // [(nstage+1)*nstage]
  const double* gam;
  const double* c;    // [nstage]
  double dt;
  int limiter, tmar, filter;
};

static void trc_step(const Oracle& o, const TrcFilter& tf, const TrcStepArgs& A, double* QTRC,
                     const double* const mflx[3], const double* aM, const double* aP, const double* ddens_trc,
                     const double* ddens0_trc, const double* ddens, const double* rhoq_tp) {
  const size_t n = (size_t)o.Np * o.Ne;
  const int ns = A.nstage;
  auto SIG = [&](int r, int s) { return A.sig[(size_t)(r - 1) * ns + (s - 1)]; };  // 1-based (row, col)
  auto GAM = [&](int r, int s) { return A.gam[(size_t)(r - 1) * ns + (s - 1)]; };
  std::vector<double> q(QTRC, QTRC + n), var0(n), vtmp(n), tend(n), fct(n, 1.0);
  for (int s = 1; s <= ns; ++s) {
    const double c_ssm1 = A.c[s - 1];
    if (A.limiter) {
      const double dttmp = A.dt * GAM(s + 1, s) / SIG(s + 1, s);
      trc_fct_coef(o, q.data(), mflx, rhoq_tp, aM, aP, ddens_trc, ddens0_trc, c_ssm1, dttmp, fct.data());
    }
    trc_cal_tend(o, q.data(), mflx, aM, aP, fct.data(), rhoq_tp, tend.data());
    const double sig_ss = SIG(s + 1, s), gam_ss = A.dt * GAM(s + 1, s);
    if (s == ns) {
#pragma omp parallel for
      for (size_t p = 0; p < n; ++p) {
        const double d0 = o.dens_hyd[p] + ddens0_trc[p];
        const double dssm1 = d0 + c_ssm1 * (ddens_trc[p] - ddens0_trc[p]);
        q[p] = (vtmp[p] + sig_ss * q[p] * dssm1 + gam_ss * tend[p]) / (o.dens_hyd[p] + ddens_trc[p]);
      }
    } else {
      const double sig_Ns = SIG(ns + 1, s), gam_Ns = A.dt * GAM(ns + 1, s);
      const double c_ss = A.c[s];
      const bool acc = std::fabs(sig_Ns) > 1.0e-16 || std::fabs(gam_Ns) > 1.0e-16;  // CONST_EPS
#pragma omp parallel for
      for (size_t p = 0; p < n; ++p) {
        const double d0 = o.dens_hyd[p] + ddens0_trc[p];
        if (s == 1) { var0[p] = q[p] * d0; vtmp[p] = 0.0; }
        const double dssm1 = d0 + c_ssm1 * (ddens_trc[p] - ddens0_trc[p]);
        const double dss = d0 + c_ss * (ddens_trc[p] - ddens0_trc[p]);
        if (acc) vtmp[p] = vtmp[p] + sig_Ns * q[p] * dssm1 + gam_Ns * tend[p];
        q[p] = ((1.0 - sig_ss) * var0[p] + sig_ss * q[p] * dssm1 + gam_ss * tend[p]) / dss;
      }
    }
  }
  if (A.filter) trc_filter(o, tf, q.data(), ddens_trc);
  if (A.limiter && A.tmar) trc_tmar(o, q.data(), ddens_trc);
  const double* dd = ddens ? ddens : ddens_trc;
#pragma omp parallel for
  for (size_t p = 0; p < n; ++p)
    QTRC[p] = (o.dens_hyd[p] + ddens_trc[p]) / (o.dens_hyd[p] + dd[p]) * q[p];
}

// ---------------------------------------------------------------------------------
// Numerical diffusion: the hyperdiffusion filter of FElib, (-1)^(n+1) coef nabla^(2n) applied to each
// prognostic variable after the dynamics step with LDG-type alternating one-sided fluxes.
//   Apply / apply_numfilter     ..._nonhydro3d_numdiff.F90:214-376
//   numdiff_tend                :379-440;  cal_del_flux_lap_with_coef :443-500
//   numdiff_cal_laplacian       :505-558;  cal_del_flux_lap           :561-601
//   numdiff_cal_flx             :606-665;  cal_del_gradDiffVar        :668-721
//   lid boundary values         ..._dgm_bnd.F90:370-508 (ApplyBC_numdiff_odd_lc / _even_lc) for
//                               slip velocity and adiabatic thermal lids
// Flat cube: periodic faces take the neighbour's values; at a lid the exterior value is the own
// node's, reflected as FElib's boundary routines do, and the face flux is centred (is_bound).
// ---------------------------------------------------------------------------------
static inline double fsign1(double x) { return std::signbit(x) ? -1.0 : 1.0; }  // Fortran sign(1, x)

// exterior value of a scalar at a lid under the even boundary routine (slip: the wall-normal
// momentum component is reflected; the other variables keep the own value)
static inline double nd_even_ext(int var, double vM, double nx, double ny, double nz) {
  switch (var) {
    case VMX: { const double g = vM * nx; return vM - 2.0 * g * nx; }
    case VMY: { const double g = vM * ny; return vM - 2.0 * g * ny; }
    case VMZ: { const double g = vM * nz; return vM - 2.0 * g * nz; }
    default: return vM;
  }
}
// exterior gradient at a lid under the odd boundary routine
static inline void nd_odd_ext(int var, const double gM[3], double nx, double ny, double nz, double gP[3]) {
  const double gn = gM[0] * nx + gM[1] * ny + gM[2] * nz;
  gP[0] = gM[0]; gP[1] = gM[1]; gP[2] = gM[2];
  switch (var) {
    case VMX: gP[1] = gM[1] - 2.0 * gn * ny; gP[2] = gM[2] - 2.0 * gn * nz; break;
    case VMY: gP[0] = gM[0] - 2.0 * gn * nx; gP[2] = gM[2] - 2.0 * gn * nz; break;
    case VMZ: gP[0] = gM[0] - 2.0 * gn * nx; gP[1] = gM[1] - 2.0 * gn * ny; break;
    default:  // DENS, RHOT: adiabatic
      gP[0] = gM[0] - 2.0 * gn * nx; gP[1] = gM[1] - 2.0 * gn * ny; gP[2] = gM[2] - 2.0 * gn * nz; break;
  }
}

// tensor-product Lift of per-face values fv[6][Nfp] at node (i, j, k)
static inline double nd_lift(const Oracle& o, const double* fv, int i, int j, int k) {
  const int N1 = o.N1, Nfp = o.Nfp, N = N1 - 1;
  const std::vector<double>& Mi = o.e.Minv;
  return Mi[j * N1 + 0] * fv[0 * Nfp + i + N1 * k] + Mi[i * N1 + N] * fv[1 * Nfp + j + N1 * k] +
         Mi[j * N1 + N] * fv[2 * Nfp + i + N1 * k] + Mi[i * N1 + 0] * fv[3 * Nfp + j + N1 * k] +
         Mi[k * N1 + 0] * fv[4 * Nfp + i + N1 * j] + Mi[k * N1 + N] * fv[5 * Nfp + i + N1 * j];
}
static inline double nd_dx(const Oracle& o, const double* u, int dir, int i, int j, int k) {
  const int N1 = o.N1;
  const std::vector<double>& D = o.e.D;
  double s = 0.0;
  for (int l = 0; l < N1; ++l) {
    const size_t p = dir == 0 ? o.nid(l, j, k) : (dir == 1 ? o.nid(i, l, k) : o.nid(i, j, l));
    s += D[(dir == 0 ? i : (dir == 1 ? j : k)) * N1 + l] * u[p];
  }
  return s;
}

// numdiff_cal_flx: G = grad(Vh, Vh, Vv) (divided by the density if dens_div); the even boundary
// routine supplies the lid exterior of Vh (and of Vv when bc_v)
static void nd_grad(const Oracle& o, int var, const double* Vh, const double* Vv, const double* ddens, bool dens_div,
                    bool bc_v, double* Gx, double* Gy, double* Gz) {
  const int N1 = o.N1, Np = o.Np, Nfp = o.Nfp;
  const double E[3] = {2.0 / o.dx, 2.0 / o.dy, 2.0 / o.dz};
  const double FS[6] = {2.0 / o.dy, 2.0 / o.dx, 2.0 / o.dy, 2.0 / o.dx, 2.0 / o.dz, 2.0 / o.dz};
#pragma omp parallel
  {
    std::vector<double> df(3 * 6 * Nfp), vh(Np), vv(Np);
#pragma omp for schedule(static)
    for (long ke = 0; ke < o.Ne; ++ke) {
      for (int f = 0; f < 6; ++f)
        for (int b = 0; b < N1; ++b)
          for (int a = 0; a < N1; ++a) {
            int i, j, k; face_node(N1, f, a, b, i, j, k);
            const size_t iM = (size_t)ke * Np + o.nid(i, j, k);
            bool lid; const size_t iP = ext_node(o, ke, f, a, b, lid);
            const double nx = NX[f], ny = NY[f], nz = NZ[f];
            double wP = 1.0, wM = 1.0;
            if (dens_div) { wP = 1.0 / (ddens[iP] + o.dens_hyd[iP]); wM = 1.0 / (ddens[iM] + o.dens_hyd[iM]); }
            double hP = Vh[iP], vP = Vv[iP];
            if (lid) { hP = nd_even_ext(var, Vh[iM], nx, ny, nz); if (bc_v) vP = nd_even_ext(var, Vv[iM], nx, ny, nz); }
            const double dh = 0.5 * (hP * wP - Vh[iM] * wM);
            const double dv = 0.5 * (vP * wP - Vv[iM] * wM);
            const int fp = f * Nfp + a + N1 * b;
            if (lid) {
              df[0 * 6 * Nfp + fp] = FS[f] * (dh * nx);
              df[1 * 6 * Nfp + fp] = FS[f] * (dh * ny);
              df[2 * 6 * Nfp + fp] = FS[f] * (dv * nz);
            } else {
              df[0 * 6 * Nfp + fp] = FS[f] * ((1.0 - fsign1(nx)) * dh * nx);
              df[1 * 6 * Nfp + fp] = FS[f] * ((1.0 - fsign1(ny)) * dh * ny);
              df[2 * 6 * Nfp + fp] = FS[f] * ((1.0 - fsign1(nz)) * dv * nz);
            }
          }
      for (int p = 0; p < Np; ++p) {
        const size_t g = (size_t)ke * Np + p;
        if (dens_div) { vh[p] = Vh[g] / (ddens[g] + o.dens_hyd[g]); vv[p] = Vv[g] / (ddens[g] + o.dens_hyd[g]); }
        else { vh[p] = Vh[g]; vv[p] = Vv[g]; }
      }
      for (int k = 0; k < N1; ++k)
        for (int j = 0; j < N1; ++j)
          for (int i = 0; i < N1; ++i) {
            const size_t g = (size_t)ke * Np + o.nid(i, j, k);
            Gx[g] = E[0] * nd_dx(o, vh.data(), 0, i, j, k) + nd_lift(o, &df[0], i, j, k);
            Gy[g] = E[1] * nd_dx(o, vh.data(), 1, i, j, k) + nd_lift(o, &df[6 * Nfp], i, j, k);
            Gz[g] = E[2] * nd_dx(o, vv.data(), 2, i, j, k) + nd_lift(o, &df[12 * Nfp], i, j, k);
          }
    }
  }
}

// numdiff_cal_laplacian with the odd boundary routine on G: horizontal and vertical parts
static void nd_lap(const Oracle& o, int var, const double* Gx, const double* Gy, const double* Gz, double* lh,
                   double* lv) {
  const int N1 = o.N1, Np = o.Np, Nfp = o.Nfp;
  const double E[3] = {2.0 / o.dx, 2.0 / o.dy, 2.0 / o.dz};
  const double FS[6] = {2.0 / o.dy, 2.0 / o.dx, 2.0 / o.dy, 2.0 / o.dx, 2.0 / o.dz, 2.0 / o.dz};
#pragma omp parallel
  {
    std::vector<double> dfh(6 * Nfp), dfv(6 * Nfp);
#pragma omp for schedule(static)
    for (long ke = 0; ke < o.Ne; ++ke) {
      for (int f = 0; f < 6; ++f)
        for (int b = 0; b < N1; ++b)
          for (int a = 0; a < N1; ++a) {
            int i, j, k; face_node(N1, f, a, b, i, j, k);
            const size_t iM = (size_t)ke * Np + o.nid(i, j, k);
            bool lid; const size_t iP = ext_node(o, ke, f, a, b, lid);
            const double nx = NX[f], ny = NY[f], nz = NZ[f];
            double gM[3] = {Gx[iM], Gy[iM], Gz[iM]}, gP[3] = {Gx[iP], Gy[iP], Gz[iP]};
            if (lid) nd_odd_ext(var, gM, nx, ny, nz, gP);
            const int fp = f * Nfp + a + N1 * b;
            if (lid) {
              dfh[fp] = FS[f] * (0.5 * ((gP[0] - gM[0]) * nx + (gP[1] - gM[1]) * ny));
              dfv[fp] = FS[f] * (0.5 * (gP[2] - gM[2]) * nz);
            } else {
              dfh[fp] = FS[f] * (0.5 * ((1.0 + fsign1(nx)) * (gP[0] - gM[0]) * nx + (1.0 + fsign1(ny)) * (gP[1] - gM[1]) * ny));
              dfv[fp] = FS[f] * (0.5 * (1.0 + fsign1(nz)) * (gP[2] - gM[2]) * nz);
            }
          }
      const double* gx = Gx + (size_t)ke * Np;
      const double* gy = Gy + (size_t)ke * Np;
      const double* gz = Gz + (size_t)ke * Np;
      for (int k = 0; k < N1; ++k)
        for (int j = 0; j < N1; ++j)
          for (int i = 0; i < N1; ++i) {
            const size_t g = (size_t)ke * Np + o.nid(i, j, k);
            lh[g] = E[0] * nd_dx(o, gx, 0, i, j, k) + E[1] * nd_dx(o, gy, 1, i, j, k) + nd_lift(o, dfh.data(), i, j, k);
            lv[g] = E[2] * nd_dx(o, gz, 2, i, j, k) + nd_lift(o, dfv.data(), i, j, k);
          }
    }
  }
}

// numdiff_tend with the odd boundary routine on G, then var += dt tend
static void nd_tend_update(const Oracle& o, int var, const double* Gx, const double* Gy, const double* Gz,
                           const double* ddens, bool mul_dens, double ch, double cv, double dt, double* V) {
  const int N1 = o.N1, Np = o.Np, Nfp = o.Nfp;
  const double E[3] = {2.0 / o.dx, 2.0 / o.dy, 2.0 / o.dz};
  const double FS[6] = {2.0 / o.dy, 2.0 / o.dx, 2.0 / o.dy, 2.0 / o.dx, 2.0 / o.dz, 2.0 / o.dz};
#pragma omp parallel
  {
    std::vector<double> df(6 * Nfp), fx(Np), fy(Np), fz(Np);
#pragma omp for schedule(static)
    for (long ke = 0; ke < o.Ne; ++ke) {
      for (int f = 0; f < 6; ++f)
        for (int b = 0; b < N1; ++b)
          for (int a = 0; a < N1; ++a) {
            int i, j, k; face_node(N1, f, a, b, i, j, k);
            const size_t iM = (size_t)ke * Np + o.nid(i, j, k);
            bool lid; const size_t iP = ext_node(o, ke, f, a, b, lid);
            const double nx = NX[f], ny = NY[f], nz = NZ[f];
            double gM[3] = {Gx[iM], Gy[iM], Gz[iM]}, gP[3] = {Gx[iP], Gy[iP], Gz[iP]};
            if (lid) nd_odd_ext(var, gM, nx, ny, nz, gP);
            double wM = 0.5, wP = 0.5;
            if (mul_dens) { wM = 0.5 * (o.dens_hyd[iM] + ddens[iM]); wP = 0.5 * (o.dens_hyd[iP] + ddens[iP]); }
            double d;
            if (lid) {
              d = ch * (wP * gP[0] - wM * gM[0]) * nx + ch * (wP * gP[1] - wM * gM[1]) * ny + cv * (wP * gP[2] - wM * gM[2]) * nz;
            } else {
              d = (1.0 + fsign1(nx)) * ch * (wP * gP[0] - wM * gM[0]) * nx +
                  (1.0 + fsign1(ny)) * ch * (wP * gP[1] - wM * gM[1]) * ny +
                  (1.0 + fsign1(nz)) * cv * (wP * gP[2] - wM * gM[2]) * nz;
            }
            df[f * Nfp + a + N1 * b] = FS[f] * d;
          }
      for (int p = 0; p < Np; ++p) {
        const size_t g = (size_t)ke * Np + p;
        double h = ch, v = cv;
        if (mul_dens) { h = ch * (o.dens_hyd[g] + ddens[g]); v = cv * (o.dens_hyd[g] + ddens[g]); }
        fx[p] = h * Gx[g]; fy[p] = h * Gy[g]; fz[p] = v * Gz[g];
      }
      for (int k = 0; k < N1; ++k)
        for (int j = 0; j < N1; ++j)
          for (int i = 0; i < N1; ++i) {
            const size_t g = (size_t)ke * Np + o.nid(i, j, k);
            const double t = E[0] * nd_dx(o, fx.data(), 0, i, j, k) + E[1] * nd_dx(o, fy.data(), 1, i, j, k) +
                             E[2] * nd_dx(o, fz.data(), 2, i, j, k) + nd_lift(o, df.data(), i, j, k);
            V[g] = V[g] + dt * t;
          }
    }
  }
}

// Apply: THERM, MOMZ, MOMX, MOMY, DENS in FElib's order (DDENS, the density weight of the others,
// changes last); nlap = ND_LAPLACIAN_NUM, coef_h/v = ND_COEF_H/V, dt = the dynamics step
static void numdiff_apply(const Oracle& o, double* const q[5], int nlap, double coef_h, double coef_v, double dt) {
  const size_t n = (size_t)o.Np * o.Ne;
  std::vector<double> Gx(n), Gy(n), Gz(n), lh(n), lv(n);
  const double sgn = ((nlap + 1) % 2 == 0) ? 1.0 : -1.0;  // (-1)^mod(nlap+1, 2)
  const int order[5] = {VRT, VMZ, VMX, VMY, VD};
  for (int vi = 0; vi < 5; ++vi) {
    const int var = order[vi];
    const bool dw = var != VD;
    nd_grad(o, var, q[var], q[var], q[VD], dw, true, Gx.data(), Gy.data(), Gz.data());
    for (int it = 1; it < nlap; ++it) {
      nd_lap(o, var, Gx.data(), Gy.data(), Gz.data(), lh.data(), lv.data());
      nd_grad(o, var, lh.data(), lv.data(), q[VD], false, false, Gx.data(), Gy.data(), Gz.data());
    }
    nd_tend_update(o, var, Gx.data(), Gy.data(), Gz.data(), q[VD], dw, sgn * coef_h, sgn * coef_v, dt, q[var]);
  }
}

// ---------------------------------------------------------------------------------
// Sponge layer: Rayleigh damping of w (and optionally u, v) towards zero above a height
//   ..._dgm_spongelayer.F90:134-219 (add_tend, calc_wdampcoef)
// ---------------------------------------------------------------------------------
static void sponge_add_tend(const Oracle& o, double* const tend[3], const double* const mom[3], double tau,
                            double height, int hvel) {
  const int N1 = o.N1, Np = o.Np;
  const double s = hvel ? 1.0 : 0.0;
  const double ztop = o.zmax, rt = 1.0 / tau;
#pragma omp parallel for schedule(static)
  for (long ke = 0; ke < o.Ne; ++ke) {
    const int ez = (int)(ke / ((long)o.NeX * o.NeY));
    for (int k = 0; k < N1; ++k) {
      const double z = o.zmin + (ez + 0.5 * (o.e.x[k] + 1.0)) * o.dz;
      const double c = 0.25 * rt * (1.0 + fsign1(z - height)) * (1.0 - std::cos(M_PI * (z - height) / (ztop - height)));
      for (int p = k * N1 * N1; p < (k + 1) * N1 * N1; ++p) {
        const size_t g = (size_t)ke * Np + p;
        tend[0][g] = tend[0][g] - s * c * mom[0][g];
        tend[1][g] = tend[1][g] - s * c * mom[1][g];
        tend[2][g] = tend[2][g] - c * mom[2][g];
      }
    }
  }
}

}  // namespace

// =================================================================================
// C API (ctypes)
// =================================================================================
extern "C" {

typedef struct {
  int porder;
  int NeX, NeY, NeZ;
  double xmin, xmax, ymin, ymax, zmin, zmax;
  double grav, rdry, cpdry, cvdry, pres00;
  double coriolis_f;
  int filter_on;
  double mf_etac, mf_alpha;
  int mf_order;
  double newton_cref;
} orc_desc;

void* orc_create(const orc_desc* d) {
  if (!d || d->porder < 1 || d->porder > 15 || d->NeX < 1 || d->NeY < 1 || d->NeZ < 1) return nullptr;
  Oracle* o = new Oracle();
  o->c.grav = d->grav; o->c.rdry = d->rdry; o->c.cpdry = d->cpdry; o->c.cvdry = d->cvdry; o->c.pres00 = d->pres00;
  o->e.init(d->porder, d->mf_etac, d->mf_alpha, d->mf_order);
  o->N1 = d->porder + 1; o->Np = o->N1 * o->N1 * o->N1; o->Nfp = o->N1 * o->N1; o->NfpTot = 6 * o->Nfp;
  o->NeX = d->NeX; o->NeY = d->NeY; o->NeZ = d->NeZ; o->Ne = d->NeX * d->NeY * d->NeZ;
  o->xmin = d->xmin; o->xmax = d->xmax; o->ymin = d->ymin; o->ymax = d->ymax; o->zmin = d->zmin; o->zmax = d->zmax;
  o->dx = (d->xmax - d->xmin) / d->NeX; o->dy = (d->ymax - d->ymin) / d->NeY; o->dz = (d->zmax - d->zmin) / d->NeZ;
  o->coriolis_f = d->coriolis_f;
  o->filter_on = d->filter_on;
  o->newton_cref = d->newton_cref > 0 ? d->newton_cref : 340.0;
  const size_t n = (size_t)o->Np * o->Ne;
  o->dens_hyd.assign(n, 0.0); o->pres_hyd.assign(n, 0.0); o->therm_hyd.assign(n, 0.0);
  return o;
}

void orc_destroy(void* h) { delete static_cast<Oracle*>(h); }

// a part of a domain decomposed along x and/or y: the exterior face layers recv[4] (x-, x+, y-, y+;
// NULL on the sides of a periodic direction), and the exchange the step functions call before every
// tendency (after DPRES is formed)
void orc_set_halo(void* h, const double* const* recv,
                  void (*cb)(void* user, int stage, const double* const* q, const double* dpres), void* user) {
  Oracle* o = static_cast<Oracle*>(h);
  for (int s = 0; s < 4; ++s) o->hx[s] = recv[s];
  o->halo_cb = cb;
  o->halo_user = user;
}

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
void orc_set_num_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

// 1D operators: x, w (N1); D, Minv, F, T, V, invV (N1*N1 row-major)
void orc_get_1d(void* h, double* x, double* w, double* D, double* Minv, double* F, double* T, double* V, double* invV) {
  Oracle* o = static_cast<Oracle*>(h);
  const int n = o->N1;
  if (x) std::memcpy(x, o->e.x.data(), n * sizeof(double));
  if (w) std::memcpy(w, o->e.w.data(), n * sizeof(double));
  if (D) std::memcpy(D, o->e.D.data(), n * n * sizeof(double));
  if (Minv) std::memcpy(Minv, o->e.Minv.data(), n * n * sizeof(double));
  if (F) std::memcpy(F, o->e.F.data(), n * n * sizeof(double));
  if (T) std::memcpy(T, o->e.T.data(), n * n * sizeof(double));
  if (V) std::memcpy(V, o->e.V.data(), n * n * sizeof(double));
  if (invV) std::memcpy(invV, o->e.invV.data(), n * n * sizeof(double));
}

// node coordinates (Np, Ne)
void orc_node_coords(void* h, double* x, double* y, double* z) {
  Oracle* o = static_cast<Oracle*>(h);
  for (int ez = 0; ez < o->NeZ; ++ez)
    for (int ey = 0; ey < o->NeY; ++ey)
      for (int ex = 0; ex < o->NeX; ++ex) {
        const size_t ke = o->eid(ex, ey, ez);
        for (int k = 0; k < o->N1; ++k)
          for (int j = 0; j < o->N1; ++j)
            for (int i = 0; i < o->N1; ++i) {
              const size_t g = ke * o->Np + o->nid(i, j, k);
              if (x) x[g] = o->xmin + (ex + 0.5 * (o->e.x[i] + 1.0)) * o->dx;
              if (y) y[g] = o->ymin + (ey + 0.5 * (o->e.x[j] + 1.0)) * o->dy;
              if (z) z[g] = o->zmin + (ez + 0.5 * (o->e.x[k] + 1.0)) * o->dz;
            }
      }
}

// base state (Np, Ne): DENS_hyd, PRES_hyd; THERM_hyd = P00/Rd (PRES_hyd/P00)^(cv/cp)
void orc_set_base_state(void* h, const double* dens_hyd, const double* pres_hyd) {
  Oracle* o = static_cast<Oracle*>(h);
  const size_t n = (size_t)o->Np * o->Ne;
  const double rgamm = o->c.cvdry / o->c.cpdry;
  for (size_t p = 0; p < n; ++p) {
    o->dens_hyd[p] = dens_hyd[p];
    o->pres_hyd[p] = pres_hyd[p];
    o->therm_hyd[p] = o->c.pres00 / o->c.rdry * std::pow(pres_hyd[p] / o->c.pres00, rgamm);
  }
}

void orc_get_therm_hyd(void* h, double* out) {
  Oracle* o = static_cast<Oracle*>(h);
  std::memcpy(out, o->therm_hyd.data(), o->therm_hyd.size() * sizeof(double));
}

void orc_drhot2pres(void* h, const double* drhot, double* pres, double* dpres) {
  drhot2pres(*static_cast<Oracle*>(h), drhot, pres, dpres);
}

// q = {DDENS, MOMX, MOMY, MOMZ, DRHOT}; dpres may be NULL (computed here)
void orc_cal_tend(void* h, int hevi, const double* const* q, const double* dpres, double* const* tend) {
  Oracle* o = static_cast<Oracle*>(h);
  std::vector<double> dp;
  if (!dpres) { dp.resize((size_t)o->Np * o->Ne); drhot2pres(*o, q[VRT], nullptr, dp.data()); dpres = dp.data(); }
  cal_tend(*o, hevi, q, dpres, tend);
}

long orc_cal_vi(void* h, const double* const* q, const double* const* q0, double impl_fac, double dt,
                int max_iter, double tol, double* const* tend, int* col_iters) {
  return cal_vi(*static_cast<Oracle*>(h), q, q0, impl_fac, dt, max_iter, tol, tend, col_iters);
}

void orc_vi_operator(void* h, const double* const* P, const double* const* q0, double* const* out) {
  vi_operator(*static_cast<Oracle*>(h), P, q0, out);
}

void orc_modalfilter(void* h, double* const* q) { modal_filter(*static_cast<Oracle*>(h), q); }

// HEVE + SSP-RK3 (ERK_SSP_3s3o), modal filter after each step if enabled
void orc_step_heve(void* h, double* const* q, double dt, int nsteps) {
  Oracle* o = static_cast<Oracle*>(h);
  const size_t n = (size_t)o->Np * o->Ne;
  std::vector<double> q0[5], tmp[5], t[5], dp(n);
  for (int v = 0; v < 5; ++v) { q0[v].resize(n); tmp[v].resize(n); t[v].resize(n); }
  double* tp[5]; for (int v = 0; v < 5; ++v) tp[v] = t[v].data();
  for (int s = 0; s < nsteps; ++s) {
    for (int v = 0; v < 5; ++v) std::memcpy(q0[v].data(), q[v], n * sizeof(double));
    for (int st = 1; st <= 3; ++st) {
      drhot2pres(*o, q[VRT], nullptr, dp.data());
      if (o->halo_cb) o->halo_cb(o->halo_user, st, q, dp.data());
      cal_tend(*o, 0, q, dp.data(), tp);
      if (o->sl_tau > 0.0) {
        double* const tm[3] = {tp[VMX], tp[VMY], tp[VMZ]};
        const double* const mm[3] = {q[VMX], q[VMY], q[VMZ]};
        sponge_add_tend(*o, tm, mm, o->sl_tau, o->sl_height, o->sl_hvel);
      }
      if (o->trc_out[0]) {  // ERK_SSP_3s3o weights b = (1/6, 1/6, 2/3)
        const double w = st == 3 ? 2.0 / 3.0 : 1.0 / 6.0;
        trc_save_massflux(*o, st, q, dp.data(), w, w, 0, o->trc_out, o->trc_out[3], o->trc_out[4]);
      }
      for (int v = 0; v < 5; ++v) {
        double* x = q[v]; const double* x0 = q0[v].data(); double* vt = tmp[v].data(); const double* tt = t[v].data();
#pragma omp parallel for
        for (size_t p = 0; p < n; ++p) {
          if (st == 1) { vt[p] = x0[p] / 3.0; x[p] = x[p] + dt * tt[p]; }
          else if (st == 2) { x[p] = 0.75 * x0[p] + 0.25 * x[p] + 0.25 * dt * tt[p]; }
          else { x[p] = vt[p] + (2.0 / 3.0) * x[p] + (2.0 / 3.0) * dt * tt[p]; }
        }
      }
    }
    if (o->trc_out[0]) {
      std::memcpy(o->trc_out[5], q[VD], n * sizeof(double));
      std::memcpy(o->trc_out[6], q0[VD].data(), n * sizeof(double));
    }
    if (o->filter_on) modal_filter(*o, q);
  }
}

// HEVI + IMEX ARK(2,3,2); returns #non-converged column solves; iteration stats optional
long orc_step_hevi(void* h, double* const* q, double dt, int nsteps, int max_iter, double tol, double* mean_iters) {
  Oracle* o = static_cast<Oracle*>(h);
  const size_t n = (size_t)o->Np * o->Ne;
  const double alp = (3.0 + 2.0 * std::sqrt(2.0)) / 6.0, gam = 1.0 - 1.0 / std::sqrt(2.0), del = 1.0 / (2.0 * std::sqrt(2.0));
  const double aex[4][4] = {{0, 0, 0, 0}, {0, 0, 0, 0}, {0, 2 * gam, 0, 0}, {0, 1 - alp, alp, 0}};
  const double aim[4][4] = {{0, 0, 0, 0}, {0, 0, 0, 0}, {0, gam, gam, 0}, {0, del, del, gam}};
  const double bb[4] = {0, del, del, gam};
  std::vector<double> var0[5], vtmp[5], tex[4][5], tim[4][5], dp(n);
  for (int v = 0; v < 5; ++v) {
    var0[v].resize(n); vtmp[v].resize(n);
    for (int s = 1; s <= 3; ++s) { tex[s][v].resize(n); tim[s][v].resize(n); }
  }
  const long ncol = (long)o->NeX * o->NeY * o->N1 * o->N1;
  std::vector<int> its(ncol);
  long nfail = 0; double itsum = 0; long itcnt = 0;
  for (int step = 0; step < nsteps; ++step) {
    for (int v = 0; v < 5; ++v) std::memcpy(var0[v].data(), q[v], n * sizeof(double));  // StoreVar0
    for (int st = 1; st <= 3; ++st) {
      const double impl_fac = aim[st][st] * dt;
      const double* qc[5]; const double* z0[5]; double* tip[5]; double* tep[5];
      for (int v = 0; v < 5; ++v) { qc[v] = q[v]; z0[v] = var0[v].data(); tip[v] = tim[st][v].data(); tep[v] = tex[st][v].data(); }
      nfail += cal_vi(*o, qc, z0, impl_fac, dt, max_iter, tol, tip, its.data());
      if (impl_fac != 0.0) { for (long c = 0; c < ncol; ++c) if (its[c] >= 0) { itsum += its[c]; ++itcnt; } }
      for (int v = 0; v < 5; ++v) {  // StoreImplicit (timeint_rk.F90:2510-2565)
        double* x = q[v];
        if (st == 1) { std::memcpy(var0[v].data(), x, n * sizeof(double)); std::memcpy(vtmp[v].data(), x, n * sizeof(double)); }
        const double* ti = tim[st][v].data();
#pragma omp parallel for
        for (size_t p = 0; p < n; ++p) x[p] = x[p] + impl_fac * ti[p];
      }
      drhot2pres(*o, q[VRT], nullptr, dp.data());
      if (o->halo_cb) o->halo_cb(o->halo_user, st, q, dp.data());
      cal_tend(*o, 1, q, dp.data(), tep);
      if (o->sl_tau > 0.0) {
        double* const tm[3] = {tep[VMX], tep[VMY], tep[VMZ]};
        const double* const mm[3] = {q[VMX], q[VMY], q[VMZ]};
        sponge_add_tend(*o, tm, mm, o->sl_tau, o->sl_height, o->sl_hvel);
      }
      if (o->trc_out[0])  // IMEX: horizontal weight b_ex, vertical b_im (driver_nonhydro3d.F90:900-917)
        trc_save_massflux(*o, st, q, dp.data(), bb[st], bb[st], 1, o->trc_out, o->trc_out[3], o->trc_out[4]);
      for (int v = 0; v < 5; ++v) {  // Advance (rk_advance_general2D, timeint_rk.F90:2201-2360)
        double* x = q[v]; double* vt = vtmp[v].data(); const double* x0 = var0[v].data();
        const double* te = tex[st][v].data(); const double* ti = tim[st][v].data();
        if (st == 3) {
#pragma omp parallel for
          for (size_t p = 0; p < n; ++p) x[p] = vt[p] + bb[3] * dt * te[p] + bb[3] * dt * ti[p];
        } else {
#pragma omp parallel for
          for (size_t p = 0; p < n; ++p) {
            vt[p] = vt[p] + bb[st] * dt * te[p] + bb[st] * dt * ti[p];
            double s = x0[p];
            for (int j = 1; j <= st; ++j) s = s + aex[st + 1][j] * dt * tex[j][v][p] + aim[st + 1][j] * dt * tim[j][v][p];
            x[p] = s;
          }
        }
      }
    }
    if (o->trc_out[0]) {
      std::memcpy(o->trc_out[5], q[VD], n * sizeof(double));
      std::memcpy(o->trc_out[6], var0[VD].data(), n * sizeof(double));
    }
    if (o->filter_on) modal_filter(*o, q);
  }
  if (mean_iters) *mean_iters = itcnt ? itsum / itcnt : 0.0;
  return nfail;
}


// ---- tracer advection ----
// face-node arrays are (NfpTot, Ne); mflx = {MFLX_x, MFLX_y, MFLX_z}; fct is a nodal (Np, Ne) field
void orc_trc_alphdens_advtest(void* h, const double* ddens, const double* momx, const double* momy,
                              const double* momz, double* aM, double* aP) {
  trc_alphdens_advtest(*static_cast<Oracle*>(h), ddens, momx, momy, momz, aM, aP);
}
// q = {DDENS, MOMX, MOMY, MOMZ, DRHOT}; dpres may be NULL (formed from DRHOT)
void orc_trc_save_massflux(void* h, int rkstage, const double* const* q, const double* dpres, double w_h,
                           double w_v, int is_hevi, double* const* mflx, double* aM, double* aP) {
  Oracle* o = static_cast<Oracle*>(h);
  std::vector<double> dp;
  if (!dpres) { dp.resize((size_t)o->Np * o->Ne); drhot2pres(*o, q[VRT], nullptr, dp.data()); dpres = dp.data(); }
  trc_save_massflux(*o, rkstage, q, dpres, w_h, w_v, is_hevi, mflx, aM, aP);
}
void orc_trc_fct_coef(void* h, const double* Q, const double* const* mflx, const double* rhoq_tp, const double* aM,
                      const double* aP, const double* ddens, const double* ddens0, double c_ssm1, double dt,
                      double* fct) {
  trc_fct_coef(*static_cast<Oracle*>(h), Q, mflx, rhoq_tp, aM, aP, ddens, ddens0, c_ssm1, dt, fct);
}
void orc_trc_cal_tend(void* h, const double* Q, const double* const* mflx, const double* aM, const double* aP,
                      const double* fct, const double* rhoq_tp, double* Qdt) {
  trc_cal_tend(*static_cast<Oracle*>(h), Q, mflx, aM, aP, fct, rhoq_tp, Qdt);
}
void orc_trc_tmar(void* h, double* Q, const double* ddens) { trc_tmar(*static_cast<Oracle*>(h), Q, ddens); }
void orc_trc_filter(void* h, double* Q, const double* ddens, double etac_h, double alpha_h, int ord_h,
                    double etac_v, double alpha_v, int ord_v) {
  Oracle* o = static_cast<Oracle*>(h);
  TrcFilter tf;
  exp_filter_matrix(o->e, etac_h, alpha_h, ord_h, tf.Fh);
  exp_filter_matrix(o->e, etac_v, alpha_v, ord_v, tf.Fv);
  trc_filter(*o, tf, Q, ddens);
}
// nsteps tracer steps with fixed mass flux, Rusanov coefficients and densities (the advection-test
// configuration, ONLY_TRACERADV_FLAG); filt = {etac_h, alpha_h, ord_h, etac_v, alpha_v, ord_v}
void orc_trc_step(void* h, double* QTRC, const double* const* mflx, const double* aM, const double* aP,
                  const double* ddens_trc, const double* ddens0_trc, const double* ddens, const double* rhoq_tp,
                  int nstage, const double* sig, const double* gam, const double* c, double dt, int limiter,
                  int tmar, int filter, const double* filt, int nsteps) {
  Oracle* o = static_cast<Oracle*>(h);
  TrcFilter tf;
  if (filter) {
    exp_filter_matrix(o->e, filt[0], filt[1], (int)filt[2], tf.Fh);
    exp_filter_matrix(o->e, filt[3], filt[4], (int)filt[5], tf.Fv);
  }
  TrcStepArgs A{nstage, sig, gam, c, dt, limiter, tmar, filter};
  for (int s = 0; s < nsteps; ++s) trc_step(*o, tf, A, QTRC, mflx, aM, aP, ddens_trc, ddens0_trc, ddens, rhoq_tp);
}


// ---- numerical diffusion and sponge layer ----
// q = {DDENS, MOMX, MOMY, MOMZ, DRHOT}, updated in place
void orc_numdiff_apply(void* h, double* const* q, int nlap, double coef_h, double coef_v, double dt) {
  numdiff_apply(*static_cast<Oracle*>(h), q, nlap, coef_h, coef_v, dt);
}
// tend = {MOMX_dt, MOMY_dt, MOMZ_dt} (in/out), mom = {MOMX, MOMY, MOMZ}
void orc_sponge_add_tend(void* h, double* const* tend, const double* const* mom, double tau, double height,
                         int hvel) {
  sponge_add_tend(*static_cast<Oracle*>(h), tend, mom, tau, height, hvel);
}


// tracer transport outputs of orc_step_heve/orc_step_hevi (NULL clears): out = {MFLX_x, MFLX_y, MFLX_z,
// alph_dens_M, alph_dens_P, DDENS_TRC, DDENS0_TRC}
void orc_set_trc_flux(void* h, double* const* out) {
  Oracle* o = static_cast<Oracle*>(h);
  for (int i = 0; i < 7; ++i) o->trc_out[i] = out ? out[i] : nullptr;
}


// sponge layer inside orc_step_heve/orc_step_hevi (tau <= 0: off)
void orc_set_sponge(void* h, double tau, double height, int hvel) {
  Oracle* o = static_cast<Oracle*>(h);
  o->sl_tau = tau; o->sl_height = height; o->sl_hvel = hvel;
}

}  // extern "C"
