// fedg_common.cuh -- shared definitions of the GB300 SCALE-DG dynamics kernels.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

#define FEDG_MAXN1 8

namespace fedg {

enum { VD = 0, VMX = 1, VMY = 2, VMZ = 3, VRT = 4 };  // cal_tend_ex argument order

// Everything a kernel needs about the element and the mesh, passed by value (it lands in the
// kernel-parameter constant bank, so every thread of a warp reads the same word: broadcast).
struct Ops {
  double D[FEDG_MAXN1 * FEDG_MAXN1];  // D1D(i,l) = l_l'(x_i), row-major [i*N1+l]
  double F[FEDG_MAXN1 * FEDG_MAXN1];  // modal filter (h == v parameters by default)
  double Fv[FEDG_MAXN1 * FEDG_MAXN1]; // vertical modal filter
  double T[FEDG_MAXN1 * FEDG_MAXN1];  // VPOrdM1 truncation
  double Lb[FEDG_MAXN1];              // Lift coefficient from the -1 face: Minv(k,0)
  double Lt[FEDG_MAXN1];              // Lift coefficient from the +1 face: Minv(k,N)
  double w[FEDG_MAXN1];               // LGL quadrature weights (scale_polynomial.F90:271-287)
  double E11, E22, E33;               // Escale of the flat cube
  double FSx, FSy, FSz;               // Fscale per face orientation
  double Jac;                         // volume Jacobian J = dx dy dz / 8
  double grav, rdry, cpdry, cvdry, pres00;
  double kap;    // cp/cv
  double rgamm;  // cv/cp
  double coriolis_f;
  int NeX, NeY, NeZ;
  int N1, Np, L;  // L = NeZ*N1 levels
  // part of a decomposed domain: the exterior face layers of the x-, x+, y-, y+ boundaries (receive
  // buffers of the halo exchange, [6 fields][NeY*NeZ or NeX*NeZ][N1*N1] doubles); NULL where the
  // mesh is periodic in that direction
  const double* hx[4];
};

// halo side of face f of element (ex, ey) on a decomposed mesh: 0 x-, 1 x+, 2 y-, 3 y+, or -1 for a
// face inside the mesh or a lid; the buffer index of face node ab of that side; the side's field stride
__device__ __forceinline__ int halo_side(int f, int ex, int ey, int NeX, int NeY) {
  return (f == 3 && ex == 0) ? 0 : (f == 1 && ex == NeX - 1) ? 1 : (f == 0 && ey == 0) ? 2 : (f == 2 && ey == NeY - 1) ? 3 : -1;
}
__device__ __forceinline__ size_t halo_index(int side, int ex, int ey, int ez, int ab, int NeX, int NeY, int NF) {
  return (size_t)(side < 2 ? ey + NeY * ez : ex + NeX * ez) * NF + ab;
}
__device__ __forceinline__ size_t halo_stride(int side, int NeX, int NeY, int NeZ, int NF) {
  return (size_t)(side < 2 ? NeY : NeX) * NeZ * NF;
}

// column profiles of the horizontally homogeneous base state, [L] each
struct Prof {
  const double* dens;   // DENS_hyd
  const double* pres;   // PRES_hyd
  const double* therm;  // THERM_hyd (cal_tend_ex)
  const double* rhyd;   // P00/Rd (PRES_hyd/P00)^(cv/cp) (cal_vi recomputes it, hevi_common_2.F90:236-237)
};

__host__ __device__ inline int face_opp(int f) { return f ^ ((f < 4) ? 2 : 1); }

// DPRES of one node (nonhydro3d_common.F90:428-479): PRES = P00 (Rd/P00 RHOT)^(cp/cv), minus
// PRES_hyd; explicit roundings, so every kernel that forms it (the field, a slab's halo) agrees
__device__ __forceinline__ double dpres_of(const Ops& op, double rhot, double pres_hyd, double* pres = nullptr) {
  const double pr = __dmul_rn(op.pres00, pow(__dmul_rn(op.rdry / op.pres00, rhot), op.kap));
  if (pres) *pres = pr;
  return __dsub_rn(pr, pres_hyd);
}

template <int N1>
__device__ __forceinline__ void face_node(int f, int a, int b, int& i, int& j, int& k) {
  constexpr int N = N1 - 1;
  switch (f) {
    case 0: i = a; j = 0; k = b; break;   // y-
    case 1: i = N; j = a; k = b; break;   // x+
    case 2: i = a; j = N; k = b; break;   // y+
    case 3: i = 0; j = a; k = b; break;   // x-
    case 4: i = a; j = b; k = 0; break;   // z-
    default: i = a; j = b; k = N; break;  // z+
  }
}

// Exterior node of face node (f, a, b) of element ke on the flat cube: the periodic neighbour's
// matching node (kn >= 0), or at a lid (kn = -1) the element's own node.  pM: the face node's index
// in the element; gP: the exterior node's global index.
template <int N1>
__device__ __forceinline__ void face_exterior(const Ops& op, int f, int a, int b, long ke, int ex, int ey, int ez,
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

// Pivot order of the column solves' element LU (3*N1 rows: DENS, MOMZ, RHOT of node k are rows
// 3k, 3k+1, 3k+2).
// Pivot order and sparsity.  The DENS rows of an element block are
//   I + (Lift face terms in the DENS columns of nodes 0 and N)
//     + impl_fac E33 D (MOMZ columns) + (block-Thomas update: node-0 columns, RHOT_0 included),
// so a DENS row has nonzeros only in DENS_k, DENS_0, DENS_N, the MOMZ columns and RHOT_0.  The
// DENS pivots go first (DENS_0 .. DENS_N), then MOMZ/RHOT node by node.  A DENS pivot row then
// carries at most DENS_N, the N1 MOMZ columns and RHOT_0 to the right, and eliminating DENS_i
// (0 < i < N) leaves the other DENS rows untouched (their DENS_i entry is zero); what remains is
// the dense 2*N1 system of the MOMZ/RHOT Schur complement.
template <int N1>
struct PivOrder {
  // column (3 node + var) of pivot step s, and the step at which column c is pivoted
  __host__ __device__ static constexpr int col(int s) { return s < N1 ? 3 * s : 3 * ((s - N1) / 2) + 1 + ((s - N1) & 1); }
  __host__ __device__ static constexpr int pos(int c) { return c % 3 == 0 ? c / 3 : N1 + 2 * (c / 3) + (c % 3 - 1); }
  // can the pivot row of step s hold a nonzero in column c (c not yet pivoted)?
  __host__ __device__ static constexpr bool nz(int s, int c) {
    if (pos(c) <= s) return false;
    if (s >= N1) return true;  // MOMZ/RHOT phase: dense
    return c == 3 * (N1 - 1) || c % 3 == 1 || c == 2;
  }
};


__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

}  // namespace fedg
