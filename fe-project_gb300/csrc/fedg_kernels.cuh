// fedg_kernels.cuh -- launcher declarations shared by the translation units.
#pragma once
#include "fedg_common.cuh"

namespace fedg {

struct F5 { double* v[5]; };
struct F5c { const double* v[5]; };

// column-solve controls
struct ViArgs {
  double impl_fac, dt, tol;
  int max_iter;
  double cref;  // velocity scale of the MOMZ convergence test [m/s]
};

// host: 1D exponential modal filter matrix (row-major N1 x N1) of order N
void modal_filter_1d(int N, double etac, double alpha, int ord, double* F);
// host: the N+1 LGL nodes on [-1, 1]
void lgl_nodes_1d(int N, double* x);

int launch_tend_fp64(const Ops& op, const Prof& pf, const F5c& q, const double* dpres, const F5& t, int Ne,
                     int hevi, cudaStream_t s);
int launch_filter_fp64(const Ops& op, const F5& q, int Ne, cudaStream_t s);
int launch_drhot2pres(const Ops& op, const Prof& pf, const double* drhot, double* pres, double* dpres, size_t n,
                      cudaStream_t s);

// Vertical-implicit column solve (cal_vi).  qin: stage input q*, z: guess/var0 (also the
// state alph is frozen at).  qout (may be NULL): new state; tout (may be NULL): tendency
// (qout - qin)/impl_fac, or A(z) when impl_fac == 0.  status[ncol]: solves used, -1 not
// converged, -2 non-finite.  guess (may be NULL): initial Newton iterate of the var3 part
// (DDENS, MOMZ, DRHOT), overriding z for the iterate but not for alph.  gsc: block-Thomas scratch of
// at least vi_fp64_scratch_doubles(op) doubles (0 when the column does not fit in shared memory).
size_t vi_fp64_scratch_doubles(const Ops& op);
int launch_vi_fp64(const Ops& op, const Prof& pf, const F5c& qin, const F5c& z, const F5c& guess, const F5& qout,
                   const F5& tout, int* status, const ViArgs& a, double* gsc, size_t gsc_doubles, cudaStream_t s);

}  // namespace fedg
