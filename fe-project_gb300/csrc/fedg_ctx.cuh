// fedg_ctx.cuh -- context and RK objects shared by the translation units.
#pragma once
#include <string>
#include <vector>

#include "../../include/fedg.h"
#include "fedg_common.cuh"
#include "fedg_kernels.cuh"
#include "fedg_mixed.cuh"
#include "fedg_mlp.cuh"

namespace fedg {
int api_fail(const std::string& m);
int api_cuda_fail(cudaError_t e, const char* where);
}  // namespace fedg
using namespace fedg;

struct fedg_ctx {
  fedg_mesh_desc d;
  Ops op;
  int N1, Np, Ne, L, ncol;
  size_t nxy, n;  // n = Np*Ne
  cudaStream_t stream = nullptr;
  double* d_prof = nullptr;  // [4][L]: dens, pres, therm, rhyd
  bool base_set = false;
  const void* base_ptr[10] = {};
  int* d_status = nullptr;
  unsigned long long* d_cnt = nullptr;
  unsigned long long* h_cnt = nullptr;  // pinned [3]
  // fused-update scratch
  double* work = nullptr;
  size_t work_doubles = 0;
  double* vi_gsc = nullptr;  // block-Thomas scratch of the FP64 column solve
  size_t vi_gsc_doubles = 0;
  MixedState* mixed = nullptr;
  fedg_tint* upd_tint = nullptr;  // RK buffers of fedg_update, kept between calls
  MlpState* guess = nullptr;      // column-guess network attached with fedg_guess_load (not owned)
  double* host_state = nullptr;   // device copy of the state of fedg_update_host (5 Np*Ne doubles)
  cudaStream_t copy_stream = nullptr;  // fedg_update_host's H2D copies, in z-ranges
  cudaEvent_t chunk_ev[4] = {};        // one per z-range: the range has arrived
  double* trc_buf = nullptr;      // tracer update scratch: two stage fields, var0, varTmp, FCT per element
  double* nd_buf = nullptr;       // numerical-diffusion scratch: gradient (3 fields), Laplacian (2 fields)
  double* sponge_coef = nullptr;  // sponge-layer coefficient per level
  double sponge_key[2] = {-1.0, -1.0};  // (tau, height) of the uploaded profile
  // tracer transport outputs of fedg_update (fedg_update_set_tracer_flux): MFLX_x/y/z, alph_dens_M/P,
  // DDENS_TRC, DDENS0_TRC (caller's device arrays; none when trc_flux[0] is null)
  double* trc_flux[7] = {};
  // sponge layer inside fedg_update (fedg_update_set_sponge; off when sl_tau <= 0)
  double sl_tau = 0.0, sl_height = 0.0;
  int sl_hvel = 0;
  // Jacobian-vector products of the Neumann corrections of the float-pair/FP32 column solve
  // (fedg_update_set_vi_neumann; 0: LU corrections only)
  int vi_neumann = 2;
  // poll limit of the update path's tensor-core barrier waits (fedg_update_set_wait_limit)
  int tc_polls = 1 << 20;
  // reference wind of the fast paths given by a restart file (fedg_restart_read) instead of taken
  // from the first state they see
  bool wind_given = false;
  double wind[2] = {0.0, 0.0};
  // part of a decomposed domain (periodic_x and/or periodic_y = FEDG_HALO): the caller's halo
  // buffers of the x-, x+, y-, y+ sides and its exchange (fedg_update_set_halo)
  void* hsend[4] = {};
  void* hrecv[4] = {};
  fedg_halo_fn hfn = nullptr;
  void* huser = nullptr;
  // kernel timers / launch counters
  bool prof_on = false;
  long long nlaunch[FEDG_K_COUNT] = {};
  struct Rec { int id; cudaEvent_t a, b; };
  std::vector<Rec> recs;
  Prof prof() const { return Prof{d_prof, d_prof + L, d_prof + 2 * L, d_prof + 3 * L}; }
};

namespace fedg {
// fedg_trc_update's tracer steps in float pairs (fedg_trc_pair.cu); scratch: 4 Np*Ne + Ne doubles
int trc_update_pair(fedg_ctx* c, double* QTRC, const double* const mflx[3], const double* aM, const double* aP,
                    const double* ddens_trc, const double* ddens0_trc, const double* ddens, const double* rhoq,
                    const fedg_trc_opts* o, double* scratch);
// fedg_numdiff_apply_prec in float pairs (fedg_nd_pair.cu); scratch: 5 Np*Ne doubles
int numdiff_apply_pair(fedg_ctx* c, double* const q[5], int nlap, double coef_h, double coef_v, double dt,
                       double* scratch);
// sponge-layer coefficient at the L LGL levels of the column (dgm_spongelayer.F90): 0.25/tau
// (1 + sign(z - h)) (1 - cos(pi (z - h) / (z_top - h)))
void sponge_coef_host(const fedg_ctx* c, double tau, double height, double* coef);
// the fast update paths' reference wind (fedg_mixed.cu): false if none has been fixed yet
bool ref_wind(const fedg_ctx* c, double out[2]);
// fixes the reference wind of the fast update paths (from a restart file)
void set_ref_wind_given(fedg_ctx* c, double U, double V);
// slab of a decomposed domain (fedg_halo.cu): packs the stage state's x face layers, synchronises
// and calls the caller's exchange; FP64 fields (+ DPRES, NULL: formed) or float-pair deviations
bool slab(const fedg_ctx* c);  // true if either lateral direction exchanges a halo
bool halo_dir(const fedg_ctx* c, int side);  // side 0..3 (x-, x+, y-, y+) is a halo side
int halo_exchange_fp64(fedg_ctx* c, const double* const q[5], const double* dpres, int stage);
int halo_exchange_pair(fedg_ctx* c, const float2* const qs[5], int stage);
int halo_exchange_f32(fedg_ctx* c, const float* const qs[5], int stage);  // FP32 stage state, value in .x
// fedg_cal_tend_ex_noalloc's set-up (fedg_static.cu): looks up its static scratch array on device `dev`,
// the current device, which loads the module holding it; called by fedg_ctx_create
void noalloc_setup(int dev);
// save_massflux of a stage held as float-pair (qp) or FP32 (qf) deviations from the hydrostatic
// state and the reference-wind momentum (fedg_trc.cu), into the registered tracer-flux outputs
int save_massflux_dev(fedg_ctx* c, int rkstage, const float2* const qp[5], const float* const qf[5], double U,
                      double V, double w_h, double w_v, int is_hevi);
}  // namespace fedg

// Runs one launch f() of kernel class id on the context stream, counting it and, when the
// timers are on, bracketing it with a pair of CUDA events.
template <class Fn>
static int tracked(fedg_ctx* c, int id, Fn&& f) {
  c->nlaunch[id]++;
  if (!c->prof_on) return f();
  fedg_ctx::Rec r{id, nullptr, nullptr};
  cudaEventCreate(&r.a);
  cudaEventCreate(&r.b);
  cudaEventRecord(r.a, c->stream);
  const int rc = f();
  cudaEventRecord(r.b, c->stream);
  c->recs.push_back(r);
  return rc;
}

struct fedg_tint {
  fedg_ctx* ctx;
  int scheme, nstage;
  double dt;
  double a_ex[3][3], a_im[3][3], b_ex[3], b_im[3];
  double sig[4][3], gam[4][3];
  double* buf = nullptr;  // var0, vtmp, tex[ns], tim[ns] : each 5*n
  double* var0(int v) { return buf + (size_t)v * ctx->n; }
  double* vtmp(int v) { return buf + (size_t)(5 + v) * ctx->n; }
  double* tex(int s, int v) { return buf + (size_t)(10 + 5 * s + v) * ctx->n; }
  double* tim(int s, int v) { return buf + (size_t)(10 + 5 * nstage + 5 * s + v) * ctx->n; }
};

