/*
 * fedg.h -- C ABI of the GB300-native SCALE-DG nonhydrostatic 3D DG dynamics step.
 *
 * Drop-in boundary for FElib's dynamics hot path (ywkawai/FE-Project):
 *   - explicit tendency      atm_dyn_nonhydro3d_cal_tend_ex
 *                            FElib/src/fluid_dyn_solver/scale_atm_dyn_dgm_driver_nonhydro3d.F90:152-199
 *                            implementations ..._nonhydro3d_rhot_heve.F90:292-489 (HEVE),
 *                            ..._nonhydro3d_rhot_hevi.F90:289-482 (HEVI)
 *   - vertical-implicit solve atm_dyn_nonhydro3d_cal_vi
 *                            ..._driver_nonhydro3d.F90:201-250, ..._rhot_hevi.F90:772-965
 *   - RK stage methods       timeint_rk%StoreVar0 / StoreImplicit / Advance / Get_implicit_diagfac
 *                            FElib/src/common/scale_timeint_rk.F90:81-104, 304-317, 536-585, 2201-2565
 *   - modal filter           atm_dyn_dgm_modalfilter_apply, ..._dgm_modalfilter.F90:49-130
 *   - pressure               atm_dyn_dgm_nonhydro3d_common_DRHOT2PRES, ..._nonhydro3d_common.F90:428-479
 *   - driver stage loop      AtmDynDGMDriver_nonhydro3d_update, ..._driver_nonhydro3d.F90:614-963
 *
 * Conventions
 *   - Every field is an FElib array real(RP) :: q(Np, NeA), column-major, passed as a
 *     DEVICE pointer (the Fortran side passes it under `!$acc host_data use_device`).
 *     Only the first Np*Ne entries (the local elements) are read or written: exterior
 *     values of periodic faces and of the slip lids are formed inside the kernels, so no
 *     halo exchange is needed on one GPU; a part of a decomposed domain exchanges its boundary
 *     faces through caller-owned buffers (fedg_update_set_halo).
 *   - Element order ke = i + (j-1)*NeX + (k-1)*NeX*NeY, node order p = i + (j-1)*N1 + (k-1)*N1^2.
 *   - Return codes: 0 ok; > 0 number of columns whose Newton iteration did not converge;
 *     < 0 error (fedg_last_error() gives the text).  No entry point traps the GPU.
 *   - One CUDA stream per context; every call is stream-ordered and returns without a
 *     device synchronisation unless it has to read a result back (status counts).
 */
#ifndef FEDG_H
#define FEDG_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fedg_ctx fedg_ctx;
typedef struct fedg_tint fedg_tint;

/* Flat cube domain: the MeshCubeDom3D parameters FElib reads from &PARAM_ATMOS_MESH
 * (scale_mesh_cubedom3d.F90) plus the SCALE constants (&PARAM_CONST) and the modal
 * filter parameters (&PARAM_ATMOS_DYN_MODALFILTER, ..._driver_nonhydro3d.F90:1249-1294). */
typedef struct {
  int porder;                 /* PolyOrder_h == PolyOrder_v, 1..7                         */
  int NeX, NeY, NeZ;          /* local elements per direction                            */
  double xmin, xmax, ymin, ymax, zmin, zmax;
  int periodic_x, periodic_y; /* 1: periodic; FEDG_HALO: the mesh is one part of a domain */
                              /* decomposed in that direction (see below)                */
  double grav, rdry, cpdry, cvdry, pres00;
  int mf_on;                  /* MODALFILTER_FLAG                                        */
  double mf_etac_h, mf_alpha_h; int mf_order_h;
  double mf_etac_v, mf_alpha_v; int mf_order_v;
  int device;                 /* CUDA device ordinal                                     */
} fedg_mesh_desc;

enum { FEDG_HEVE = 0, FEDG_HEVI = 1 };
enum { FEDG_SSP_RK3 = 0, FEDG_IMEX_ARK232 = 1 };
/* precision of the fused update path (fedg_update) */
enum { FEDG_PREC_FP64 = 0, FEDG_PREC_MIXED = 1, FEDG_PREC_PAIR = 2 };

const char* fedg_last_error(void);

/* Context: builds the reference-element operators (D1D, exact-mass Lift, filters, VPOrdM1
 * truncation) and owns one CUDA stream and the scratch of the fused paths.
 * Replaces MeshCubeDom3D + HexahedralElement + ElementOperationTensorProd3D set-up
 * (scale_element_hexahedral.F90:102-404, scale_element_operation_tensorprod3D.F90:5512-5569). */
int fedg_ctx_create(const fedg_mesh_desc* desc, fedg_ctx** out);
void fedg_ctx_destroy(fedg_ctx* ctx);
/* the CUDA stream (cudaStream_t) every call of this context is ordered on */
void* fedg_ctx_stream(fedg_ctx* ctx);
int fedg_synchronize(fedg_ctx* ctx);

/* Base state (AUX_VARS DENS_hyd, PRES_hyd, THERM_hyd, Rtot, CVtot, CPtot, DPhydDx, DPhydDy and
 * the 2D CORIOLIS(Np2D, NeA2D)); device pointers in FElib layout.  The library keeps the
 * state as per-level column profiles: it checks on the GPU that the fields are horizontally
 * homogeneous, that Rtot/CVtot/CPtot are the dry constants, DPhydDx/DPhydDy vanish and
 * CORIOLIS is constant, and returns < 0 otherwise.  CORIOLIS and DPhyd* may be NULL (zero). */
int fedg_set_base_state(fedg_ctx* ctx, const double* DENS_hyd, const double* PRES_hyd,
                        const double* THERM_hyd, const double* Rtot, const double* CVtot,
                        const double* CPtot, const double* DPhydDx, const double* DPhydDy,
                        const double* CORIOLIS);

/* atm_dyn_dgm_nonhydro3d_common_DRHOT2PRES (nonhydro3d_common.F90:428-479). */
int fedg_drhot2pres(fedg_ctx* ctx, const double* DRHOT, double* PRES, double* DPRES);

/* atm_dyn_nonhydro3d_cal_tend_ex (driver_nonhydro3d.F90:152-199).
 *   in[16]  = DDENS_, MOMX_, MOMY_, MOMZ_, DRHOT_, DPRES_, DENS_hyd, PRES_hyd, PRES_hyd_ref,
 *             THERM_hyd, CORIOLIS, Rtot, CVtot, CPtot, DPhydDx, DPhydDy
 *   out[5]  = DENS_dt, MOMX_dt, MOMY_dt, MOMZ_dt, RHOT_dt
 *   eqs     = FEDG_HEVE (rhot_heve_cal_tend) or FEDG_HEVI (rhot_hevi_cal_tend)
 * The base-state inputs are registered with fedg_set_base_state when their pointers differ
 * from the registered ones.  DPRES_ may be NULL: it is then formed from DRHOT_ inside the kernel. */
int fedg_cal_tend_ex(fedg_ctx* ctx, const double* const in[16], double* const out[5], int eqs);

/* fedg_cal_tend_ex without any device allocation.  No counterpart in the reference: FElib
 * passes DPRES in, and fedg_cal_tend_ex allocates a scratch field on first use when it forms
 * DPRES itself.  This variant is for callers that cannot allow a cudaMalloc once their set-up is
 * over (a Fortran model whose device memory belongs to its OpenACC runtime, or any host whose
 * device allocator has already claimed the memory): it forms DPRES in a static device array of
 * 2,097,152 doubles (16 MiB, held by every GPU that loads the library) and returns < 0 with a
 * message if Np*Ne exceeds that.  Same arguments as fedg_cal_tend_ex (in[5] is ignored); the
 * base state must already be registered with fedg_set_base_state.  The array's device address
 * is looked up (cudaGetSymbolAddress) when the first context on a device is created: with CUDA's
 * lazy module loading that lookup loads the library module that holds the array and reserves its
 * 16 MiB, so it happens in fedg_ctx_create, during the caller's set-up, and the entry point only
 * reads the recorded address.  If that lookup failed, the entry point returns < 0 with the error.
 * The caller's current device is restored before returning.  All calls share the one array:
 * calls whose kernels overlap on the GPU (two contexts, two streams) race on it and must be
 * ordered by the caller. */
int fedg_cal_tend_ex_noalloc(fedg_ctx* ctx, const double* const in[16], double* const out[5], int eqs);

/* atm_dyn_nonhydro3d_cal_vi (driver_nonhydro3d.F90:201-250; rhot_hevi.F90:772-965).
 *   in[12]  = DDENS_, MOMX_, MOMY_, MOMZ_, DRHOT_, DENS_hyd, PRES_hyd,
 *             DDENS0_, MOMX0_, MOMY0_, MOMZ0_, DRHOT0_       (Rtot/CVtot/CPtot: registered)
 *   out[5]  = DENS_dt, MOMX_dt, MOMY_dt, MOMZ_dt, RHOT_dt  = (q_new - q)/impl_fac, or A(var0)
 *             when impl_fac == 0 (rhot_hevi.F90:943-961)
 *   max_iter = 1 reproduces FElib's single linearised solve from the guess var0;
 *   max_iter > 1 iterates Newton until the scaled residual is below tol.
 *   col_status (optional, device, NeX*NeY*N1*N1 ints): Newton solves used per column,
 *   -1 = not converged, -2 = non-finite.  Returns the number of non-converged columns. */
int fedg_cal_vi(fedg_ctx* ctx, const double* const in[12], double impl_fac, double dt,
                int max_iter, double tol, double* const out[5], int* col_status);

/* atm_dyn_dgm_modalfilter_apply with do_weight_Gsqrt (dgm_modalfilter.F90:49-130), in place. */
int fedg_modalfilter(fedg_ctx* ctx, double* const q[5]);

/* timeint_rk (scale_timeint_rk.F90).  The object owns var0, varTmp and the explicit and
 * implicit tendency buffers tend_buf2D_ex/im(Np, Ne, 5, nstage) on the device. */
int fedg_tint_create(fedg_ctx* ctx, int scheme, double dt, fedg_tint** out);
void fedg_tint_destroy(fedg_tint* t);
int fedg_tint_nstage(const fedg_tint* t);
double fedg_tint_implicit_diagfac(const fedg_tint* t, int stage);           /* :304-317   */
/* device pointer of tend_buf2D_ex/_im(:, :, var, stage) (var in out[] order, stage 1-based) */
double* fedg_tint_tend_ex(fedg_tint* t, int stage, int var);
double* fedg_tint_tend_im(fedg_tint* t, int stage, int var);
double* fedg_tint_var0(fedg_tint* t, int var);
int fedg_tint_store_var0(fedg_tint* t, double* const q[5]);                   /* driver :703-713 */
int fedg_tint_store_implicit(fedg_tint* t, int stage, double* const q[5]);    /* :2510-2565 */
int fedg_tint_advance(fedg_tint* t, int stage, double* const q[5]);           /* :536-585, 1182-1278, 2201-2360 */

/* AtmDynDGMDriver_nonhydro3d_update (driver_nonhydro3d.F90:614-963): nsteps full time steps
 * of q (5 device fields) with the fused GPU stage kernels.  eqs FEDG_HEVE uses SSP-RK3,
 * FEDG_HEVI uses IMEX ARK232 with the column Newton solve (max_iter, tol).
 * prec (FEDG_PREC_MIXED: HEVI only):
 *   FEDG_PREC_FP64: FElib's arithmetic in FP64.
 *   FEDG_PREC_MIXED: FP32 explicit arithmetic on deviations from the hydrostatic state and the
 *     reference wind; the Newton iterate, its certifying residual and the RK accumulation in
 *     float pairs (about 48 bits); FP32 Jacobian and LU.
 *   FEDG_PREC_PAIR: as FEDG_PREC_MIXED with the explicit operator also in float pairs.
 *     It is FP64-class end to end; use it with a Newton tol near 1e-13, so the FP32
 *     corrections are refined to pair accuracy.  With eqs FEDG_HEVE: the three SSP-RK3 stages in
 *     float pairs (no implicit solve; use_guess must be 0, iters_out is 0).
 * use_guess != 0 takes the initial Newton iterate from the column-guess network loaded with
 * fedg_guess_load.
 * iters_out (optional, host): mean Newton solves per implicit column solve. */
typedef struct {
  int eqs, prec, max_iter, use_guess;
  double dt, tol;
} fedg_update_opts;
int fedg_update(fedg_ctx* ctx, double* const q[5], int nsteps, const fedg_update_opts* opts,
                double* iters_out);

/* fedg_update for a caller whose fields live in host memory (FElib's CPU build keeps its MeshField
 * arrays on the host): host_q[5] (DDENS, MOMX, MOMY, MOMZ, DRHOT in FElib layout) must be page-locked
 * (cudaHostAlloc, or host memory registered with cudaHostRegister).  The fields are copied into the
 * context's device copy of the state (allocated on first use), nsteps steps are taken, and the result
 * is written back to host_q before the call returns.  With FEDG_PREC_PAIR the last stage kernel
 * stores the result into host_q through its device mapping while it runs, so the device-to-host
 * transfer overlaps its arithmetic, and (HEVI on a periodic mesh, once the reference wind is fixed,
 * without tracer-flux outputs) the host-to-device copies run in z-ranges on a second stream while
 * the first stage works on the ranges that have arrived; the other paths copy the state in before
 * and out after the step. */
int fedg_update_host(fedg_ctx* ctx, double* const host_q[5], int nsteps, const fedg_update_opts* opts,
                     double* iters_out);

/* Newton corrections of the FEDG_PREC_MIXED / FEDG_PREC_PAIR column solve.  Every column's first
 * correction solves the FP32 Jacobian by block-Thomas and element LU, like FElib's solve
 * (hevi_common_2.F90:329-479).  Later corrections, which only refine that FP32 solution, use a
 * truncated Neumann series of the same Jacobian J = I + K: delta = (I - K + K^2 - ...) b with nterm
 * products K v (default 2), as long as each one cuts the certifying residual fourfold; a column
 * whose residual does not contract (large vertical Courant numbers, where ||K|| is not small) goes
 * back to LU corrections.  The converged state is the same: convergence is judged by the
 * float-pair residual to tol either way.  nterm = 0: LU corrections only.  No counterpart in
 * FElib, whose solve is a single LU correction. */
int fedg_update_set_vi_neumann(fedg_ctx* ctx, int nterm);

/* Bounded waits of the update path's tensor-core contractions (the FEDG_PREC_MIXED stage kernels):
 * each wait on the MMA completion barrier polls at most `polls` times (default 1048576) before the
 * kernel gives up, drains its MMAs with the default limit and raises an error flag; fedg_update then
 * returns < 0 with fedg_last_error text.  No counterpart in FElib (no GPU waits there); a small
 * limit makes the wait run out on purpose, which is how the error path is tested. */
int fedg_update_set_wait_limit(fedg_ctx* ctx, int polls);

/* ---- Horizontal domain decomposition -------------------------------------------------------
 * FElib distributes its domain over MPI ranks and, before each tendency evaluation, exchanges the
 * face values of the prognostic fields (PROG_VARS%MeshFieldComm_Exchange, driver_nonhydro3d.F90:
 * 768-771) and of DPRES (AUXDYNVAR3D_manager%MeshFieldComm_Exchange, :783-787) through
 * MeshFieldCommBase_exchange_core / _wait_core (scale_meshfieldcomm_base.F90:340-470).
 * Here the domain is split along x and/or y into parts with full-height columns (the column solves
 * stay local): a context whose mesh has periodic_x = FEDG_HALO (periodic_y = FEDG_HALO) is one part
 * whose x (y) boundaries take their exterior values from halo buffers that the caller's transport
 * (MPI, NCCL, peer copies) fills; a direction left at 1 stays periodic inside the part, and z has
 * the slip lids.  Sides: 0 x-, 1 x+, 2 y-, 3 y+.
 *   recv[0] holds the x- neighbour's x+ face layer, which that neighbour packs into its send[1];
 *   recv[1] holds the x+ neighbour's x- face layer (its send[0]); recv[2] and recv[3] the same in y.
 * Layout of each buffer: [6 fields][boundary elements][N1*N1 face nodes] of 8-byte values; the
 * fields are DDENS, MOMX, MOMY, MOMZ, DRHOT, DPRES, the boundary elements are numbered ey + NeY*ez on
 * the x sides and ex + NeX*ez on the y sides, and face node a + N1*b is node (i, a, b) of the element
 * on an x face (i = 0 or N) and node (a, j, b) on a y face (j = 0 or N).  FEDG_PREC_FP64 exchanges
 * doubles; FEDG_PREC_PAIR exchanges float pairs (hi, lo) of the deviations from the hydrostatic
 * state and the reference wind and leaves the DPRES slot unused (the receiving side forms it from
 * DRHOT); FEDG_PREC_MIXED exchanges its FP32 deviations in the first 4 bytes of each slot.  The
 * tracer, numerical-diffusion and tracer-flux entry points need a periodic mesh and refuse a
 * decomposed one. */
enum { FEDG_HALO = 2 };
/* bytes of the halo buffer of one side (0 for a side whose direction is periodic) */
size_t fedg_halo_bytes(const fedg_ctx* ctx, int side);
/* The exchange fedg_update calls before every tendency evaluation of a part: the library has
 * packed the stage state into the send buffers of the halo sides and synchronised its stream; the
 * function moves send[1] to the x+ neighbour's recv[0], send[0] to the x- neighbour's recv[1],
 * send[3] to the y+ neighbour's recv[2] and send[2] to the y- neighbour's recv[3] (the halo sides
 * only), and returns 0 once this part's receive buffers hold the neighbours' data (nonzero:
 * fedg_update returns < 0).  stage: the RK stage (1..3) of the tendency about to be evaluated. */
typedef int (*fedg_halo_fn)(void* user, int stage);
/* Registers the part's halo buffers (device, fedg_halo_bytes(ctx, side) each, NULL on periodic
 * sides; the caller owns them, so its transport can use them directly) and the exchange (fn may be
 * NULL for callers that only use fedg_halo_pack and fedg_cal_tend_ex). */
int fedg_update_set_halo(fedg_ctx* ctx, void* const send[4], void* const recv[4], fedg_halo_fn fn, void* user);
/* Packs the FP64 face layers of q (5 fields) and DPRES (NULL: formed from DRHOT) into the send
 * buffers and synchronises: FElib's MeshFieldComm put before an exchange, for callers of
 * fedg_cal_tend_ex on a part, which reads the receive buffers as they are when it runs. */
int fedg_halo_pack(fedg_ctx* ctx, const double* const q[5], const double* DPRES);
/* The reference wind (U, V) of the FP32 and float-pair paths' momentum deviations.  A periodic
 * context takes it from the domain mean of the first state it sees; slabs must share one, so a slab
 * needs it set (any value is valid: it only shifts what the deviations are taken from).
 * fedg_update_get_ref_wind returns 0 and leaves u, v unchanged if none is fixed yet. */
int fedg_update_set_ref_wind(fedg_ctx* ctx, double u, double v);
int fedg_update_get_ref_wind(const fedg_ctx* ctx, double* u, double* v);

/* Column-guess network for the HEVI Newton solve (the learned initial iterate): a GELU MLP
 * (3L+1) -> hidden -> hidden -> 3L mapping a column's stage input (DDENS', MOMZ, DRHOT' at its
 * L = NeZ*N1 levels, then impl_fac, each times in_scale[var]) to the implicit increment
 * Q - q* (times out_scale[var]).  BF16 weights, FP32 accumulation; trained on the GPU by the
 * library's own forward/backward/Adam kernels.  No counterpart in FElib: FElib's guess is
 * var0 (rhot_hevi.F90:857-861); with fedg_update(use_guess) the plain Newton solve still
 * runs to tol from this iterate, so the network only changes how many solves are needed.
 * X, T, Y are device arrays (row per sample, FP32); parameters in host memory, logical order
 * W1 (hidden x din) | b1 | W2 | b2 | W3 (dout x hidden) | b3. */
typedef struct fedg_guess fedg_guess;
int fedg_guess_create(int levels, int hidden, fedg_guess** out);
void fedg_guess_destroy(fedg_guess* g);
long long fedg_guess_num_params(const fedg_guess* g);
int fedg_guess_set_scales(fedg_guess* g, const float in_scale[4], const float out_scale[3]);
int fedg_guess_set_params(fedg_guess* g, const float* host, long long n);
int fedg_guess_get_params(fedg_guess* g, float* host, long long n);
/* one Adam step (beta 0.9/0.999, eps 1e-8) on the mean-square loss of a batch */
int fedg_guess_train_step(fedg_guess* g, const float* X, const float* T, int batch, float lr, float* loss);
/* loss and gradient (host, logical order) without updating the parameters */
int fedg_guess_loss_grad(fedg_guess* g, const float* X, const float* T, int batch, float* loss, float* grad);
/* inference through the BF16 tensor-core GEMM path */
int fedg_guess_predict(fedg_guess* g, const float* X, float* Y, int n);
/* Bounded waits of the network's tensor-core GEMMs: each wait on the MMA completion barrier polls
 * at most `polls` times (default 1048576) before the kernel gives up, drains the MMAs it issued
 * (with the default limit), skips its stores and raises an error flag that the calling entry point
 * returns as < 0 with fedg_last_error text.  No counterpart in FElib (no GPU waits there); a small
 * limit makes the wait run out on purpose, which is how the error path is tested. */
int fedg_guess_set_wait_limit(fedg_guess* g, int polls);
/* attach (g != NULL) or detach (g == NULL) the network used by fedg_update(use_guess = 1) */
int fedg_guess_load(fedg_ctx* ctx, fedg_guess* g);

/* ---- Tracer advection -------------------------------------------------------------------
 * HEVE DG transport of a tracer mixing ratio q by a mass flux, with the nonnegativity limiter of
 * Light and Durran (2016): FCT on the lowest mode, then truncation and mass-aware rescaling (TMAR).
 * FElib/src/fluid_dyn_solver/scale_atm_dyn_dgm_trcadvect3d_heve.F90 and the tracer driver
 * ..._driver_trcadv3d.F90.  FP64, device pointers in FElib layout like every other entry point;
 * the base state (DENS_hyd) must be registered with fedg_set_base_state.
 *   mflx[3]        = MFLX_x_tavg, MFLX_y_tavg, MFLX_z_tavg (Np, NeA)
 *   alph_M/alph_P  = alphaDensM/P face values (NfpTot, Ne): face f = 1..6 (south, east, north,
 *                    west, bottom, top), face node i + (k-1) N1 on the lateral faces and
 *                    i + (j-1) N1 on the bottom/top faces
 *   fct_coef       = AUX_TRCVARS3D TRCADV_FCTCOEF (Np, NeA), one value per element */

/* atm_dyn_dgm_trcadvect3d_heve_cal_alphdens_advtest (trcadvect3d_heve.F90:404-455): the Rusanov
 * coefficients of the advection test (ONLY_TRACERADV_FLAG), max(|v_n-|, |v_n+|) dens on each side. */
int fedg_trc_alphdens_advtest(fedg_ctx* ctx, const double* DDENS, const double* MOMX, const double* MOMY,
                              const double* MOMZ, double* alph_M, double* alph_P);
/* atm_dyn_dgm_trcadvect3d_save_massflux (trcadvect3d_heve.F90:343-401, called from the dynamics
 * stage loop, driver_nonhydro3d.F90:900-917): rkstage 1 sets, later stages add
 * MFLX += w_h (MOMX, MOMY), w_v MOMZ and the dynamics' Rusanov coefficients
 * (w_h (|nx|+|ny|) + w_v |nz|) alpha dens (cal_alphdens_dyn, :460-551).
 *   q[5] = DDENS, MOMX, MOMY, MOMZ, DRHOT; DPRES may be NULL (formed from DRHOT). */
int fedg_trc_save_massflux(fedg_ctx* ctx, int rkstage, const double* const q[5], const double* DPRES, double w_h,
                           double w_v, int is_hevi, double* const mflx[3], double* alph_M, double* alph_P);
/* atm_dyn_dgm_trcadvect3d_heve_calc_fct_coef (trcadvect3d_heve.F90:234-306).  RHOQ_tp may be NULL. */
int fedg_trc_fct_coef(fedg_ctx* ctx, const double* QTRC, const double* const mflx[3], const double* RHOQ_tp,
                      const double* alph_M, const double* alph_P, const double* DDENS_TRC,
                      const double* DDENS0_TRC, double rk_c_ssm1, double dt, double* fct_coef);
/* atm_dyn_dgm_trcadvect3d_heve_cal_tend (trcadvect3d_heve.F90:149-231): QTRC_dt = d(dens q)/dt.
 * fct_coef NULL means no limiter (coefficient 1); RHOQ_tp may be NULL. */
int fedg_trc_cal_tend(fedg_ctx* ctx, const double* QTRC, const double* const mflx[3], const double* alph_M,
                      const double* alph_P, const double* fct_coef, const double* RHOQ_tp, double* QTRC_dt);
/* atm_dyn_dgm_trcadvect3d_TMAR (trcadvect3d_heve.F90:311-340), in place; DDENS = DDENS_TRC. */
int fedg_trc_tmar(fedg_ctx* ctx, double* QTRC, const double* DDENS);
/* atm_dyn_dgm_tracer_modalfilter_apply (dgm_modalfilter.F90:232-270) with the tracer filter
 * parameters (&PARAM_ATMOS_DYN_TRACER_MODALFILTER, driver_trcadv3d.F90:720-765), in place. */
int fedg_trc_modalfilter(fedg_ctx* ctx, double* QTRC, const double* DDENS, double etac_h, double alpha_h,
                         int order_h, double etac_v, double alpha_v, int order_v);
/* AtmDynDGMDriver_trcadv3d_update for one tracer (driver_trcadv3d.F90:420-545): nsteps tracer
 * steps with the mass flux, Rusanov coefficients and densities held fixed.  Each stage: the FCT
 * coefficient (limiter), the tendency and the density-weighted low-storage advance
 * (rk_advance_trcvar_low_storage2D, timeint_rk.F90:1390-1498); after the last stage the tracer
 * filter (filter), TMAR (limiter && tmar: FElib's ONLY_TRACERADV_FLAG) and the rescale
 * QTRC = (DENS_hyd + DDENS_TRC) / (DENS_hyd + DDENS) QTRC (DDENS NULL: DDENS_TRC).  In place on QTRC. */
typedef struct {
  int scheme;          /* FEDG_SSP_RK3 (ERK_SSP_3s3o, FElib's default TINTEG_TYPE_TRACER) */
  double dt;
  int nsteps;
  int limiter;         /* !TRACERADV_DISABLE_LIMITER */
  int tmar;
  int filter;          /* MODALFILTER_FLAG */
  double mf_etac_h, mf_alpha_h; int mf_order_h;
  double mf_etac_v, mf_alpha_v; int mf_order_v;
  int prec;            /* FEDG_PREC_FP64 (FElib's arithmetic, default) or FEDG_PREC_PAIR (float pairs on
                          the FP32 pipe: FP64-class, relative rounding ~1e-14) */
} fedg_trc_opts;
int fedg_trc_update(fedg_ctx* ctx, double* QTRC, const double* const mflx[3], const double* alph_M,
                    const double* alph_P, const double* DDENS_TRC, const double* DDENS0_TRC, const double* DDENS,
                    const double* RHOQ_tp, const fedg_trc_opts* opts);

/* update_pressure_specific_heat (FElib/src/fluid_dyn_solver/scale_atm_dyn_dgm_driver_trcadv3d.F90:653-716),
 * which the tracer driver runs after the tracer step and before the negative fixer: the mixture's Rtot,
 * CVtot, CPtot from the QA tracers (SCALE's mixing rule, as for the fixer) and, through calc_pressure
 * (atm_dyn_dgm_nonhydro3d_common_DRHOT2PRES, nonhydro3d_common.F90:428-479),
 * PRES = P00 (Rtot (THERM_hyd + DRHOT) / P00)^(CPtot / CVtot) and DPRES = PRES - PRES_hyd (DPRES may be
 * NULL).  QA <= 16 (0: the dry constants); tracer tables as for fedg_trc_negative_fixer; device arrays. */
int fedg_trc_specific_heat_pressure(fedg_ctx* ctx, const double* const* QTRC, int QA, const double* trc_mass,
                                    const double* trc_r, const double* trc_cv, const double* trc_cp,
                                    const double* DRHOT, const double* PRES_hyd, const double* THERM_hyd,
                                    double* Rtot, double* CVtot, double* CPtot, double* PRES, double* DPRES);

/* atm_phy_mp_dgm_common_negative_fixer (FElib/src/microphysics/scale_atm_phy_mp_dgm_common.F90:429-556),
 * which the tracer driver runs after the tracer step (fix_negative_val, driver_trcadv3d.F90:550,
 * 596-651), in place, FP64.  Per element, each water species iq = 0 .. QLA+QIA has its mass DENS q
 * clipped below at 1e-128 and rescaled to the element's mass max(M, 0); DDENS takes the mass change,
 * the internal energy CVtot PRES / Rtot the change times TRACER_CV and the temperature; then the
 * internal energy is rescaled to the element's old total, Rtot/CVtot/CPtot follow the new mixing
 * ratios (SCALE's mixture specific heats: qdry = 1 - sum q TRACER_MASS, Rtot = sum q TRACER_R +
 * qdry Rdry, likewise CV and CP), the potential energy of the mass change (DDENS - DDENS0) g z is taken
 * out and PRES = IntEn Rtot / CVtot.  DRHOT (may be NULL: FElib's non-RHOT thermodynamic variable)
 * is rebuilt as P00/Rtot (PRES/P00)^(CVtot/CPtot) - P00/Rdry (PRES_hyd/P00)^(CVdry/CPdry).
 *   QTRC[QA]        device pointers of the tracers (Np, Ne); QA = 1 + QLA + QIA (<= 16): FElib's routine
 *                   leaves the mixing ratios of any further tracer undefined, so it is refused here
 *   trc_mass/r/cv/cp host arrays of QA: TRACER_MASS, TRACER_R, TRACER_CV, TRACER_CP (scale_tracer)
 *   DENS_hyd, PRES_hyd (Np, Ne) device arrays; dt as in FElib's argument list (unused there too).
 * Element integrals: the LGL quadrature of the flat cube; z of a node from the mesh descriptor. */
int fedg_trc_negative_fixer(fedg_ctx* ctx, double* const* QTRC, int QA, int QLA, int QIA, const double* trc_mass,
                            const double* trc_r, const double* trc_cv, const double* trc_cp, double* DDENS,
                            double* PRES, double* CVtot, double* CPtot, double* Rtot, const double* DENS_hyd,
                            const double* PRES_hyd, double* DRHOT, double dt);

/* Tracer transport outputs of fedg_update (every prec), the coupling of FElib's dynamics driver to
 * its tracer driver (driver_nonhydro3d.F90:900-935): during each step, after every stage's explicit
 * tendency, the stage-weighted mass flux and the dynamics' Rusanov coefficients are accumulated into
 * mflx/alph_M/alph_P (fedg_trc_save_massflux with the scheme's b weights); DDENS0_TRC receives DDENS at
 * the step's start and DDENS_TRC the DDENS before the modal filter.  After fedg_update they hold the
 * last step's values, ready for fedg_trc_update.  The FP32 and float-pair paths accumulate them from
 * the stage states they hold as deviations, and their fused stage-3 kernel writes DDENS_TRC before
 * its filter.  mflx == NULL clears the registration.  The caller owns the arrays (FElib layout,
 * device). */
int fedg_update_set_tracer_flux(fedg_ctx* ctx, double* const mflx[3], double* alph_M, double* alph_P,
                                double* DDENS_TRC, double* DDENS0_TRC);

/* The sponge layer inside fedg_update (every prec): after every stage's explicit tendency, the
 * damping of fedg_sponge_add_tend on MOMX/MOMY/MOMZ_dt (SPONGELAYER_FLAG, driver_nonhydro3d.F90:
 * 831-841); the FP32 and float-pair paths apply it inside their fused stage kernels.
 * tau <= 0 turns it off (the default). */
int fedg_update_set_sponge(fedg_ctx* ctx, double tau, double height, int hveldamp);

/* ---- Numerical diffusion and sponge layer ---------------------------------------------------
 * atm_dyn_dgm_nonhydro3d_numdiff_Apply (FElib/src/fluid_dyn_solver/scale_atm_dyn_dgm_nonhydro3d_numdiff.F90:
 * 214-376), applied by the model after the dynamics and tracer updates (mod_atmos_dyn.F90:340-348):
 * q += dt (-1)^(nlap+1) nabla^(2 nlap) q with coefficients coef_h (horizontal) and coef_v (vertical),
 * for DRHOT, MOMZ, MOMX, MOMY, DDENS in that order; all but DDENS are differentiated as q/dens and
 * weighted by dens.  nlap = ND_LAPLACIAN_NUM, coef_h/v = ND_COEF_H/V, dt = the dynamics step.
 * q[5] = DDENS, MOMX, MOMY, MOMZ, DRHOT, in place; lids are slip and adiabatic (dgm_bnd.F90:370-508). */
int fedg_numdiff_apply(fedg_ctx* ctx, double* const q[5], int nlap, double coef_h, double coef_v, double dt);
/* the same with a precision: FEDG_PREC_FP64 (fedg_numdiff_apply) or FEDG_PREC_PAIR (the passes in float
 * pairs on the FP32 pipe, FP64-class; the increment is added to the FP64 fields in FP64) */
int fedg_numdiff_apply_prec(fedg_ctx* ctx, double* const q[5], int nlap, double coef_h, double coef_v, double dt,
                            int prec);
/* atm_dyn_dgm_spongelayer_add_tend (..._dgm_spongelayer.F90:134-219): Rayleigh damping of MOMZ (and of
 * MOMX, MOMY when hveldamp) above `height`, rate 0.25/tau (1 + sign(z - h)) (1 - cos(pi (z - h)/(z_top - h))),
 * subtracted from the explicit tendencies.  tend[3] = MOMX_dt, MOMY_dt, MOMZ_dt (in/out); mom[3] = MOMX,
 * MOMY, MOMZ.  FElib's defaults: tau = 10 dt when SL_WDAMP_TAU < 0; height from SL_WDAMP_LAYER. */
int fedg_sponge_add_tend(fedg_ctx* ctx, double* const tend[3], const double* const mom[3], double tau,
                         double height, int hveldamp);

/* ---- Restart files -------------------------------------------------------------------------
 * The restart state FElib writes through NetCDF (FElib/src/file/scale_file_restart_meshfield.F90:
 * 136-186; read back by model/atm_nonhydro3d/src/atmos/mod_atmos_vars.F90:580-633), in a flat
 * little-endian file: a header (mesh, step, time, dt, time-integration scheme name, the fast paths'
 * reference wind) and the fields DDENS, MOMX, MOMY, MOMZ, DRHOT, DENS_hyd, PRES_hyd, THERM_hyd in
 * FElib's (Np, Ne) order as float64.  fedg_restart_write takes the five prognostic fields (device)
 * and writes the registered base state with them; fedg_restart_read checks the mesh, fills the five
 * fields and, when base is not NULL, DENS_hyd, PRES_hyd, THERM_hyd (device arrays; register them with
 * fedg_set_base_state), and fixes the context's reference wind, so that a run restored into a new
 * context continues bit for bit.  The layout is documented in fe-project_gb300/csrc/fedg_restart.cu
 * and read and written by fe-project_gb300/fedg/restart.py. */
typedef struct {
  long long step;   /* time steps taken */
  double time;      /* simulated time [s] */
  double dt;        /* time step [s] */
  char scheme[32];  /* time-integration scheme (FElib's TINTEG_TYPE, e.g. "IMEX_ARK232") */
} fedg_restart_info;
int fedg_restart_write(fedg_ctx* ctx, const char* path, const double* const q[5], const fedg_restart_info* info);
int fedg_restart_read(fedg_ctx* ctx, const char* path, double* const q[5], double* const base[3],
                      fedg_restart_info* info);

/* Kernel timers: the analogue of FElib's PROF_rapstart/PROF_rapend regions
 * (e.g. 'ATM_DYN_cal_vi', 'cal_dyn_tend_interior'; scale_prof of the SCALE library).
 * When enabled, every launch of the context records a pair of CUDA events on the context
 * stream; fedg_prof_read synchronises and returns the summed device time and the launch
 * count of one kernel class.  Launch counts are kept even when timing is off. */
enum {
  FEDG_K_TEND = 0,      /* explicit tendency (volume + face + Lift), FP64          */
  FEDG_K_VI = 1,        /* column Newton solve, FP64                                */
  FEDG_K_RK = 2,        /* RK stage arithmetic                                      */
  FEDG_K_FILTER = 3,    /* modal filter                                             */
  FEDG_K_PRES = 4,      /* DRHOT -> DPRES                                           */
  FEDG_K_MTEND = 5,     /* fused mixed-precision stage kernel (tendency + RK)       */
  FEDG_K_MVI = 6,       /* mixed-precision column solve                             */
  FEDG_K_MLP = 7,       /* column-guess network (inference / training)              */
  FEDG_K_AUX = 8,       /* status reductions, base-state checks                     */
  FEDG_K_TRC_FCT = 9,   /* tracer FCT coefficient (calc_fct_coef)                   */
  FEDG_K_TRC_TEND = 10, /* tracer tendency + RK stage (cal_tend, Advance_trcvar)    */
  FEDG_K_TRC_AUX = 11,  /* tracer Rusanov coefficients, mass flux, TMAR, filter     */
  FEDG_K_ND = 12,       /* numerical diffusion passes, sponge layer                 */
  FEDG_K_COUNT = 13
};
int fedg_prof_enable(fedg_ctx* ctx, int on);
int fedg_prof_reset(fedg_ctx* ctx);
int fedg_prof_read(fedg_ctx* ctx, int kernel, double* total_ms, long long* launches);

#ifdef __cplusplus
}
#endif
#endif /* FEDG_H */
