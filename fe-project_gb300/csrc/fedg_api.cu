// fedg_api.cu -- context, base state, RK stage methods, the driver update loop and the
// extern "C" entry points declared in include/fedg.h.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/fedg.h"
#include "fedg_common.cuh"
#include "fedg_kernels.cuh"
#include "fedg_mixed.cuh"
#include "fedg_ctx.cuh"

using namespace fedg;

namespace {
thread_local std::string g_err;
int fail(const std::string& m) {
  g_err = m;
  return -1;
}
int cuda_fail(cudaError_t e, const char* where) {
  g_err = std::string(where) + ": " + cudaGetErrorString(e);
  return -2;
}
}  // namespace
namespace fedg {
int api_fail(const std::string& m) { return fail(m); }
int api_cuda_fail(cudaError_t e, const char* where) { return cuda_fail(e, where); }
}  // namespace fedg
namespace {
#define CK(call)                                              \
  do {                                                        \
    cudaError_t e_ = (call);                                  \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call);       \
  } while (0)

// ---------------- reference element (host) ----------------
double legendre(int n, double x) {
  if (n == 0) return 1.0;
  double p0 = 1.0, p1 = x;
  for (int m = 1; m < n; ++m) {
    const double p2 = ((2.0 * m + 1.0) * x * p1 - m * p0) / (m + 1.0);
    p0 = p1;
    p1 = p2;
  }
  return p1;
}

// LGL nodes: +-1 and the roots of P_N' (Newton), scale_polynomial.F90:250-373
std::vector<double> lgl(int N) {
  std::vector<double> x(N + 1);
  x[0] = -1.0;
  x[N] = 1.0;
  for (int i = 1; i < N; ++i) {
    double xi = -std::cos(M_PI * i / N);
    for (int it = 0; it < 100; ++it) {
      const double pn = legendre(N, xi), pn1 = legendre(N - 1, xi);
      const double f = N * (pn1 - xi * pn) / (1.0 - xi * xi);
      const double fp = (2.0 * xi * f - N * (N + 1.0) * pn) / (1.0 - xi * xi);
      const double d = f / fp;
      xi -= d;
      if (std::fabs(d) < 1e-17) break;
    }
    x[i] = xi;
  }
  return x;
}

void invert(int n, std::vector<double> a, std::vector<double>& inv) {
  inv.assign(n * n, 0.0);
  for (int i = 0; i < n; ++i) inv[i * n + i] = 1.0;
  for (int c = 0; c < n; ++c) {
    int p = c;
    for (int r = c + 1; r < n; ++r)
      if (std::fabs(a[r * n + c]) > std::fabs(a[p * n + c])) p = r;
    for (int k = 0; k < n; ++k) {
      std::swap(a[c * n + k], a[p * n + k]);
      std::swap(inv[c * n + k], inv[p * n + k]);
    }
    const double d = 1.0 / a[c * n + c];
    for (int k = 0; k < n; ++k) {
      a[c * n + k] *= d;
      inv[c * n + k] *= d;
    }
    for (int r = 0; r < n; ++r) {
      if (r == c) continue;
      const double f = a[r * n + c];
      for (int k = 0; k < n; ++k) {
        a[r * n + k] -= f * a[c * n + k];
        inv[r * n + k] -= f * inv[c * n + k];
      }
    }
  }
}

// exponential modal filter V diag(sigma) V^-1, sigma_m = exp(-alpha ((m/N - etac)/(1 - etac))^ord) for
// m/N > etac (scale_element_modalfilter.F90:204-236)
void filter_1d(int N, const std::vector<double>& V, const std::vector<double>& iV, double etac, double alpha, int ord,
               double* F) {
  const int n1 = N + 1;
  std::vector<double> sig(n1, 1.0);
  for (int m = 1; m < n1; ++m) {
    const double eta = double(m) / N;
    if (eta > etac) sig[m] = std::exp(-alpha * std::pow((eta - etac) / (1.0 - etac), ord));
  }
  for (int i = 0; i < n1; ++i)
    for (int j = 0; j < n1; ++j) {
      double s = 0.0;
      for (int m = 0; m < n1; ++m) s += V[i * n1 + m] * sig[m] * iV[m * n1 + j];
      F[i * n1 + j] = s;
    }
}

// 1D operators of the tensor-product element (scale_element_hexahedral.F90:102-404,
// scale_element_operation_tensorprod3D.F90:5464-5569, scale_element_modalfilter.F90:204-236)
void build_ops_1d(int N, double etac_h, double alpha_h, int ord_h, double etac_v, double alpha_v, int ord_v,
                  Ops& op) {
  const int n1 = N + 1;
  const std::vector<double> x = lgl(N);
  std::vector<double> V(n1 * n1), iV;
  for (int i = 0; i < n1; ++i)
    for (int m = 0; m < n1; ++m) V[i * n1 + m] = legendre(m, x[i]) * std::sqrt(m + 0.5);
  invert(n1, V, iV);
  for (int i = 0; i < n1; ++i)
    for (int l = 0; l < n1; ++l)
      op.D[i * n1 + l] = (i != l) ? legendre(N, x[i]) / (legendre(N, x[l]) * (x[i] - x[l])) : 0.0;
  op.D[0] = -N * (N + 1.0) / 4.0;
  op.D[N * n1 + N] = N * (N + 1.0) / 4.0;
  for (int k = 0; k < n1; ++k) {  // M^-1 = V V^T: Lift coefficients of the -1 and +1 faces
    double sb = 0.0, st = 0.0;
    for (int m = 0; m < n1; ++m) {
      sb += V[k * n1 + m] * V[0 * n1 + m];
      st += V[k * n1 + m] * V[N * n1 + m];
    }
    op.Lb[k] = sb;
    op.Lt[k] = st;
  }
  for (int i = 0; i < n1; ++i) {
    const double pn = legendre(N, x[i]);
    op.w[i] = 2.0 / (N * (N + 1.0) * pn * pn);
  }
  filter_1d(N, V, iV, etac_h, alpha_h, ord_h, op.F);
  filter_1d(N, V, iV, etac_v, alpha_v, ord_v, op.Fv);
  for (int i = 0; i < n1; ++i)
    for (int j = 0; j < n1; ++j) {
      double s = 0.0;
      for (int m = 0; m < N; ++m) s += V[i * n1 + m] * iV[m * n1 + j];
      op.T[i * n1 + j] = s;
    }
}

}  // namespace
namespace fedg {
void lgl_nodes_1d(int N, double* x) {
  const std::vector<double> v = lgl(N);
  for (int i = 0; i <= N; ++i) x[i] = v[i];
}
void modal_filter_1d(int N, double etac, double alpha, int ord, double* F) {
  const int n1 = N + 1;
  const std::vector<double> x = lgl(N);
  std::vector<double> V(n1 * n1), iV;
  for (int i = 0; i < n1; ++i)
    for (int m = 0; m < n1; ++m) V[i * n1 + m] = legendre(m, x[i]) * std::sqrt(m + 0.5);
  invert(n1, V, iV);
  filter_1d(N, V, iV, etac, alpha, ord, F);
}
}  // namespace fedg
namespace {

// ---------------- small device kernels ----------------
__global__ void k_extract_profile(const double* __restrict__ a, double* __restrict__ prof, int N1, int Np, int L,
                                  size_t nxy) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= L) return;
  const int ez = l / N1, k = l - ez * N1;
  prof[l] = a[((size_t)ez * nxy) * Np + (size_t)N1 * N1 * k];
}

// counts entries of a (Np, Ne) field differing from the profile (or from a constant if prof == NULL)
__global__ void k_check_field(const double* __restrict__ a, const double* __restrict__ prof, double cval, int N1,
                              int Np, size_t nxy, size_t n, double rtol, double atol, unsigned long long* bad) {
  const size_t g = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n) return;
  double ref = cval;
  if (prof) {
    const size_t ke = g / Np;
    const int p = (int)(g - ke * Np);
    const int ez = (int)(ke / nxy);
    ref = prof[ez * N1 + p / (N1 * N1)];
  }
  const double d = fabs(a[g] - ref);
  if (!(d <= rtol * fabs(ref) + atol)) atomicAdd(bad, 1ull);
}

__global__ void k_count_status(const int* __restrict__ st, int n, unsigned long long* bad, unsigned long long* sum,
                               unsigned long long* cnt) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const int s = st[c];
  if (s < 0) atomicAdd(bad, 1ull);
  else {
    atomicAdd(sum, (unsigned long long)s);
    atomicAdd(cnt, 1ull);
  }
}

// ---- timeint_rk stage arithmetic on five fields (scale_timeint_rk.F90) ----
struct RKC {
  double c[8];
};
// kind 0: store_var0   var0 = q
// kind 1: store_implicit (stage 1 also copies var0 = varTmp = q); q += c0 * tim_s
// kind 2: IMEX/general advance, non-final stage s: q = var0 + sum_j (aex_j tex_j + aim_j tim_j)*dt,
//         varTmp += dt (b_ex tex_s + b_im tim_s)
// kind 3: IMEX final stage: q = varTmp + dt (b_ex tex_s + b_im tim_s)
// kind 4: low-storage advance (SSP)
struct RKPtrs {
  double* q[5];
  double* var0[5];
  double* vtmp[5];
  const double* tex[3][5];
  const double* tim[3][5];
};

__global__ void k_rk(RKPtrs P, int kind, int stage, int nst, RKC c, size_t n, int first_stage) {
  const size_t g = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n) return;
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    double q = P.q[v][g];
    if (kind == 0) {
      P.var0[v][g] = q;
    } else if (kind == 1) {
      if (first_stage) {
        P.var0[v][g] = q;
        P.vtmp[v][g] = q;
      }
      P.q[v][g] = q + c.c[0] * P.tim[stage - 1][v][g];
    } else if (kind == 2) {
      double s = P.var0[v][g];
      P.vtmp[v][g] = P.vtmp[v][g] + c.c[6] * P.tex[stage - 1][v][g] + c.c[7] * P.tim[stage - 1][v][g];
      for (int j = 0; j < stage; ++j) {
        s = s + c.c[j] * P.tex[j][v][g];
        if (P.tim[j][v]) s = s + c.c[3 + j] * P.tim[j][v][g];
      }
      P.q[v][g] = s;
    } else if (kind == 3) {
      double s = P.vtmp[v][g] + c.c[6] * P.tex[stage - 1][v][g];
      if (P.tim[stage - 1][v]) s = s + c.c[7] * P.tim[stage - 1][v][g];
      P.q[v][g] = s;
    } else {  // low storage: c0 = sig_ss, c1 = gam_ss, c2 = sig_Ns, c3 = gam_Ns, c4 = final flag, c5 = use Ns
      const double t = P.tex[0][v][g];
      if (c.c[4] != 0.0) {
        P.q[v][g] = P.vtmp[v][g] + c.c[0] * q + c.c[1] * t;
      } else {
        if (first_stage) {
          P.var0[v][g] = q;
          P.vtmp[v][g] = 0.0;
        }
        if (c.c[5] != 0.0) P.vtmp[v][g] = P.vtmp[v][g] + c.c[2] * q + c.c[3] * t;
        P.q[v][g] = (1.0 - c.c[0]) * P.var0[v][g] + c.c[0] * q + c.c[1] * t;
      }
    }
  }
}

}  // namespace

extern "C" {

const char* fedg_last_error(void) { return g_err.c_str(); }

int fedg_ctx_create(const fedg_mesh_desc* d, fedg_ctx** out) {
  if (!d || !out) return fail("fedg_ctx_create: null argument");
  if (d->porder < 1 || d->porder > FEDG_MAXN1 - 1) return fail("fedg_ctx_create: porder must be 1..7");
  if (d->NeX < 1 || d->NeY < 1 || d->NeZ < 1) return fail("fedg_ctx_create: element counts must be >= 1");
  if ((d->periodic_x != 1 && d->periodic_x != FEDG_HALO) || (d->periodic_y != 1 && d->periodic_y != FEDG_HALO))
    return fail("fedg_ctx_create: lateral boundaries must be periodic (1) or halo-exchanged parts of a decomposed domain (FEDG_HALO)");
  if (!(d->xmax > d->xmin && d->ymax > d->ymin && d->zmax > d->zmin)) return fail("fedg_ctx_create: empty domain");
  if (d->NeZ > 64) return fail("fedg_ctx_create: NeZ > 64 is not supported by the column solver");
  CK(cudaSetDevice(d->device));
  fedg_ctx* c = new fedg_ctx();
  c->d = *d;
  c->N1 = d->porder + 1;
  c->Np = c->N1 * c->N1 * c->N1;
  c->Ne = d->NeX * d->NeY * d->NeZ;
  c->L = d->NeZ * c->N1;
  c->ncol = d->NeX * d->NeY * c->N1 * c->N1;
  c->nxy = (size_t)d->NeX * d->NeY;
  c->n = (size_t)c->Np * c->Ne;
  Ops& op = c->op;
  std::memset(&op, 0, sizeof(op));
  build_ops_1d(d->porder, d->mf_etac_h, d->mf_alpha_h, d->mf_order_h, d->mf_etac_v, d->mf_alpha_v, d->mf_order_v, op);
  const double dx = (d->xmax - d->xmin) / d->NeX, dy = (d->ymax - d->ymin) / d->NeY, dz = (d->zmax - d->zmin) / d->NeZ;
  op.E11 = 2.0 / dx; op.E22 = 2.0 / dy; op.E33 = 2.0 / dz;
  op.FSx = 2.0 / dx; op.FSy = 2.0 / dy; op.FSz = 2.0 / dz;
  op.Jac = dx * dy * dz / 8.0;
  op.grav = d->grav; op.rdry = d->rdry; op.cpdry = d->cpdry; op.cvdry = d->cvdry; op.pres00 = d->pres00;
  op.kap = d->cpdry / d->cvdry;
  op.rgamm = d->cvdry / d->cpdry;
  op.NeX = d->NeX; op.NeY = d->NeY; op.NeZ = d->NeZ;
  op.N1 = c->N1; op.Np = c->Np; op.L = c->L;
  cudaError_t e;
  if ((e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) != cudaSuccess ||
      (e = cudaMalloc(&c->d_prof, sizeof(double) * 4 * c->L)) != cudaSuccess ||
      (e = cudaMalloc(&c->d_status, sizeof(int) * c->ncol)) != cudaSuccess ||
      (e = cudaMalloc(&c->d_cnt, sizeof(unsigned long long) * 4)) != cudaSuccess ||
      (e = cudaMallocHost(&c->h_cnt, sizeof(unsigned long long) * 4)) != cudaSuccess) {
    fedg_ctx_destroy(c);
    return cuda_fail(e, "fedg_ctx_create");
  }
  // set-up of fedg_cal_tend_ex_noalloc on this device (loads its static scratch now, not at call time)
  noalloc_setup(d->device);
  *out = c;
  return 0;
}

void fedg_ctx_destroy(fedg_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->d.device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  mixed_free(c->mixed);
  if (c->upd_tint) fedg_tint_destroy(c->upd_tint);
  cudaFree(c->d_prof);
  cudaFree(c->d_status);
  cudaFree(c->d_cnt);
  cudaFree(c->work);
  cudaFree(c->vi_gsc);
  cudaFree(c->host_state);
  cudaFree(c->trc_buf);
  cudaFree(c->nd_buf);
  cudaFree(c->sponge_coef);
  if (c->h_cnt) cudaFreeHost(c->h_cnt);
  for (cudaEvent_t ev : c->chunk_ev)
    if (ev) cudaEventDestroy(ev);
  if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

void* fedg_ctx_stream(fedg_ctx* c) { return c ? (void*)c->stream : nullptr; }

int fedg_synchronize(fedg_ctx* c) {
  if (!c) return fail("null ctx");
  CK(cudaStreamSynchronize(c->stream));
  return 0;
}

int fedg_set_base_state(fedg_ctx* c, const double* DENS_hyd, const double* PRES_hyd, const double* THERM_hyd,
                        const double* Rtot, const double* CVtot, const double* CPtot, const double* DPhydDx,
                        const double* DPhydDy, const double* CORIOLIS) {
  if (!c || !DENS_hyd || !PRES_hyd || !THERM_hyd) return fail("fedg_set_base_state: null argument");
  CK(cudaSetDevice(c->d.device));
  const int L = c->L, bs = 256;
  const unsigned gb = (unsigned)((c->n + bs - 1) / bs);
  const double* src[3] = {DENS_hyd, PRES_hyd, THERM_hyd};
  for (int m = 0; m < 3; ++m)
    k_extract_profile<<<(L + 127) / 128, 128, 0, c->stream>>>(src[m], c->d_prof + m * L, c->N1, c->Np, L, c->nxy);
  CK(cudaMemsetAsync(c->d_cnt, 0, sizeof(unsigned long long), c->stream));
  for (int m = 0; m < 3; ++m)
    k_check_field<<<gb, bs, 0, c->stream>>>(src[m], c->d_prof + m * L, 0.0, c->N1, c->Np, c->nxy, c->n, 1e-12, 0.0,
                                            c->d_cnt);
  const double cst[3] = {c->op.rdry, c->op.cvdry, c->op.cpdry};
  const double* cf[3] = {Rtot, CVtot, CPtot};
  for (int m = 0; m < 3; ++m)
    if (cf[m]) k_check_field<<<gb, bs, 0, c->stream>>>(cf[m], nullptr, cst[m], c->N1, c->Np, c->nxy, c->n, 1e-12, 0.0, c->d_cnt);
  if (DPhydDx) k_check_field<<<gb, bs, 0, c->stream>>>(DPhydDx, nullptr, 0.0, c->N1, c->Np, c->nxy, c->n, 0.0, 1e-12, c->d_cnt);
  if (DPhydDy) k_check_field<<<gb, bs, 0, c->stream>>>(DPhydDy, nullptr, 0.0, c->N1, c->Np, c->nxy, c->n, 0.0, 1e-12, c->d_cnt);
  double f = 0.0;
  if (CORIOLIS) {
    CK(cudaMemcpyAsync(&f, CORIOLIS, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    const size_t n2 = (size_t)c->N1 * c->N1 * c->nxy;
    k_check_field<<<(unsigned)((n2 + bs - 1) / bs), bs, 0, c->stream>>>(CORIOLIS, nullptr, f, c->N1, c->Np, c->nxy, n2,
                                                                       1e-12, 0.0, c->d_cnt);
  }
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(c->h_cnt, c->d_cnt, sizeof(unsigned long long), cudaMemcpyDeviceToHost, c->stream));
  std::vector<double> hp(2 * L);
  CK(cudaMemcpyAsync(hp.data(), c->d_prof + L, sizeof(double) * L, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  if (c->h_cnt[0] != 0)
    return fail("fedg_set_base_state: base state is not horizontally homogeneous dry air with DPhyd = 0 and constant "
                "CORIOLIS (" + std::to_string(c->h_cnt[0]) + " mismatching entries)");
  for (int l = 0; l < L; ++l)  // RHOT_hyd recomputed from PRES_hyd as cal_vi does (hevi_common_2.F90:236-237)
    hp[L + l] = c->op.pres00 / c->op.rdry * std::pow(hp[l] / c->op.pres00, c->op.rgamm);
  CK(cudaMemcpyAsync(c->d_prof + 3 * L, hp.data() + L, sizeof(double) * L, cudaMemcpyHostToDevice, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  c->op.coriolis_f = f;
  c->base_set = true;
  mixed_free(c->mixed);  // FP32 profiles of the mixed path are rebuilt from the new base state
  c->mixed = nullptr;
  const void* ptrs[10] = {DENS_hyd, PRES_hyd, THERM_hyd, Rtot, CVtot, CPtot, DPhydDx, DPhydDy, CORIOLIS, nullptr};
  std::memcpy(c->base_ptr, ptrs, sizeof(ptrs));
  return 0;
}

int fedg_drhot2pres(fedg_ctx* c, const double* DRHOT, double* PRES, double* DPRES) {
  if (!c || !DRHOT || !DPRES) return fail("fedg_drhot2pres: null argument");
  if (!c->base_set) return fail("fedg_drhot2pres: base state not set");
  CK(cudaSetDevice(c->d.device));
  CK((cudaError_t)tracked(c, FEDG_K_PRES, [&] { return launch_drhot2pres(c->op, c->prof(), DRHOT, PRES, DPRES, c->n, c->stream); }));
  return 0;
}

// the FP64 column solve's block-Thomas scratch (sized by its launch plan for this mesh)
static double* vi_scratch(fedg_ctx* c, size_t* ndouble) {
  const size_t need = vi_fp64_scratch_doubles(c->op);
  *ndouble = need;
  if (need == 0) return nullptr;
  if (c->vi_gsc_doubles >= need) return c->vi_gsc;
  cudaFree(c->vi_gsc);
  c->vi_gsc = nullptr;
  c->vi_gsc_doubles = 0;
  if (cudaMalloc(&c->vi_gsc, sizeof(double) * need) != cudaSuccess) return nullptr;
  c->vi_gsc_doubles = need;
  return c->vi_gsc;
}

static double* ensure_work(fedg_ctx* c, size_t ndouble) {
  if (c->work_doubles >= ndouble) return c->work;
  cudaFree(c->work);
  c->work = nullptr;
  c->work_doubles = 0;
  if (cudaMalloc(&c->work, sizeof(double) * ndouble) != cudaSuccess) return nullptr;
  c->work_doubles = ndouble;
  return c->work;
}

int fedg_cal_tend_ex(fedg_ctx* c, const double* const in[16], double* const out[5], int eqs) {
  if (!c || !in || !out) return fail("fedg_cal_tend_ex: null argument");
  for (int v = 0; v < 5; ++v)
    if (!in[v] || !out[v]) return fail("fedg_cal_tend_ex: null field");
  if (eqs != FEDG_HEVE && eqs != FEDG_HEVI) return fail("fedg_cal_tend_ex: eqs must be FEDG_HEVE or FEDG_HEVI");
  CK(cudaSetDevice(c->d.device));
  const bool same = c->base_set && in[6] == c->base_ptr[0] && in[7] == c->base_ptr[1] && in[9] == c->base_ptr[2];
  if (!same && in[6] && in[7] && in[9]) {
    const int r = fedg_set_base_state(c, in[6], in[7], in[9], in[11], in[12], in[13], in[14], in[15], in[10]);
    if (r) return r;
  }
  if (!c->base_set) return fail("fedg_cal_tend_ex: base state not set");
  if (fedg::slab(c) && !c->hrecv[fedg::halo_dir(c, 0) ? 0 : 2])
    return fail("fedg_cal_tend_ex: a decomposed mesh (periodic_x/y = FEDG_HALO) needs its halo buffers (fedg_update_set_halo)");
  const double* dpres = in[5];
  if (!dpres) {
    double* w = ensure_work(c, c->n);
    if (!w) return fail("fedg_cal_tend_ex: out of device memory");
    CK((cudaError_t)tracked(c, FEDG_K_PRES, [&] { return launch_drhot2pres(c->op, c->prof(), in[4], nullptr, w, c->n, c->stream); }));
    dpres = w;
  }
  F5c q{{in[0], in[1], in[2], in[3], in[4]}};
  F5 t{{out[0], out[1], out[2], out[3], out[4]}};
  CK((cudaError_t)tracked(c, FEDG_K_TEND, [&] { return launch_tend_fp64(c->op, c->prof(), q, dpres, t, c->Ne, eqs, c->stream); }));
  return 0;
}

static int count_status(fedg_ctx* c, long long* sum, long long* cnt) {
  CK(cudaMemsetAsync(c->d_cnt, 0, sizeof(unsigned long long) * 3, c->stream));
  CK((cudaError_t)tracked(c, FEDG_K_AUX, [&] {
    k_count_status<<<(c->ncol + 255) / 256, 256, 0, c->stream>>>(c->d_status, c->ncol, c->d_cnt, c->d_cnt + 1,
                                                                 c->d_cnt + 2);
    return (int)cudaGetLastError();
  }));
  CK(cudaMemcpyAsync(c->h_cnt, c->d_cnt, sizeof(unsigned long long) * 3, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  if (sum) *sum += (long long)c->h_cnt[1];
  if (cnt) *cnt += (long long)c->h_cnt[2];
  return (int)c->h_cnt[0];
}

int fedg_cal_vi(fedg_ctx* c, const double* const in[12], double impl_fac, double dt, int max_iter, double tol,
                double* const out[5], int* col_status) {
  if (!c || !in || !out) return fail("fedg_cal_vi: null argument");
  for (int v = 0; v < 5; ++v)
    if (!in[v] || !in[7 + v] || !out[v]) return fail("fedg_cal_vi: null field");
  if (max_iter < 1) return fail("fedg_cal_vi: max_iter must be >= 1");
  CK(cudaSetDevice(c->d.device));
  if (!c->base_set) return fail("fedg_cal_vi: base state not set (fedg_set_base_state or fedg_cal_tend_ex first)");
  if (in[5] != c->base_ptr[0] || in[6] != c->base_ptr[1]) {
    // DENS_hyd/PRES_hyd differ from the registered ones: re-register with the registered THERM_hyd
    const int r = fedg_set_base_state(c, in[5], in[6], (const double*)c->base_ptr[2], nullptr, nullptr, nullptr,
                                      nullptr, nullptr, (const double*)c->base_ptr[8]);
    if (r) return r;
  }
  F5c q{{in[0], in[1], in[2], in[3], in[4]}};
  F5c z{{in[7], in[8], in[9], in[10], in[11]}};
  F5c none{{nullptr, nullptr, nullptr, nullptr, nullptr}};
  F5 t{{out[0], out[1], out[2], out[3], out[4]}};
  F5 qo{{nullptr, nullptr, nullptr, nullptr, nullptr}};
  ViArgs a{impl_fac, dt, tol, max_iter, 340.0};
  int* st = col_status ? col_status : c->d_status;
  size_t ngsc = 0;
  double* gsc = vi_scratch(c, &ngsc);
  if (!gsc) return fail(ngsc ? "fedg_cal_vi: out of device memory" : "fedg_cal_vi: the column does not fit in shared memory");
  CK((cudaError_t)tracked(c, FEDG_K_VI, [&] {
    return launch_vi_fp64(c->op, c->prof(), q, z, none, qo, t, st, a, gsc, ngsc, c->stream);
  }));
  if (st != c->d_status) CK(cudaMemcpyAsync(c->d_status, st, sizeof(int) * c->ncol, cudaMemcpyDeviceToDevice, c->stream));
  return count_status(c, nullptr, nullptr);
}

int fedg_modalfilter(fedg_ctx* c, double* const q[5]) {
  if (!c || !q) return fail("fedg_modalfilter: null argument");
  CK(cudaSetDevice(c->d.device));
  F5 f{{q[0], q[1], q[2], q[3], q[4]}};
  CK((cudaError_t)tracked(c, FEDG_K_FILTER, [&] { return launch_filter_fp64(c->op, f, c->Ne, c->stream); }));
  return 0;
}

// ---------------- timeint_rk ----------------
int fedg_tint_create(fedg_ctx* c, int scheme, double dt, fedg_tint** out) {
  if (!c || !out) return fail("fedg_tint_create: null argument");
  if (scheme != FEDG_SSP_RK3 && scheme != FEDG_IMEX_ARK232) return fail("fedg_tint_create: unknown scheme");
  CK(cudaSetDevice(c->d.device));
  fedg_tint* t = new fedg_tint();
  std::memset(t->a_ex, 0, sizeof(t->a_ex));
  std::memset(t->a_im, 0, sizeof(t->a_im));
  std::memset(t->sig, 0, sizeof(t->sig));
  std::memset(t->gam, 0, sizeof(t->gam));
  t->ctx = c;
  t->scheme = scheme;
  t->dt = dt;
  t->nstage = 3;
  if (scheme == FEDG_IMEX_ARK232) {  // scale_timeint_rk_butcher_tab.F90:260-274
    const double alp = (3.0 + 2.0 * std::sqrt(2.0)) / 6.0, gam = 1.0 - 1.0 / std::sqrt(2.0),
                 del = 1.0 / (2.0 * std::sqrt(2.0));
    t->a_ex[1][0] = 2.0 * gam;
    t->a_ex[2][0] = 1.0 - alp;
    t->a_ex[2][1] = alp;
    t->a_im[1][0] = gam;
    t->a_im[1][1] = gam;
    t->a_im[2][0] = del;
    t->a_im[2][1] = del;
    t->a_im[2][2] = gam;
    t->b_ex[0] = t->b_im[0] = del;
    t->b_ex[1] = t->b_im[1] = del;
    t->b_ex[2] = t->b_im[2] = gam;
  } else {  // ERK_SSP_3s3o, butcher_tab.F90:200-210
    t->sig[1][0] = 1.0;
    t->sig[2][0] = 0.75;
    t->sig[2][1] = 0.25;
    t->sig[3][0] = 1.0 / 3.0;
    t->sig[3][2] = 2.0 / 3.0;
    t->gam[1][0] = 1.0;
    t->gam[2][1] = 0.25;
    t->gam[3][2] = 2.0 / 3.0;
  }
  const size_t nb = (size_t)(10 + 10 * t->nstage) * c->n;
  if (cudaMalloc(&t->buf, sizeof(double) * nb) != cudaSuccess) {
    delete t;
    return fail("fedg_tint_create: out of device memory");
  }
  CK(cudaMemsetAsync(t->buf, 0, sizeof(double) * nb, c->stream));
  *out = t;
  return 0;
}

void fedg_tint_destroy(fedg_tint* t) {
  if (!t) return;
  cudaSetDevice(t->ctx->d.device);
  cudaStreamSynchronize(t->ctx->stream);
  cudaFree(t->buf);
  delete t;
}

int fedg_tint_nstage(const fedg_tint* t) { return t ? t->nstage : -1; }

double fedg_tint_implicit_diagfac(const fedg_tint* t, int stage) {
  if (!t || stage < 1 || stage > t->nstage || t->scheme != FEDG_IMEX_ARK232) return 0.0;
  return t->a_im[stage - 1][stage - 1] * t->dt;
}

double* fedg_tint_tend_ex(fedg_tint* t, int stage, int var) {
  if (!t || stage < 1 || stage > t->nstage || var < 0 || var > 4) return nullptr;
  return t->tex(t->scheme == FEDG_IMEX_ARK232 ? stage - 1 : 0, var);
}
double* fedg_tint_tend_im(fedg_tint* t, int stage, int var) {
  if (!t || stage < 1 || stage > t->nstage || var < 0 || var > 4) return nullptr;
  return t->tim(stage - 1, var);
}
double* fedg_tint_var0(fedg_tint* t, int var) { return (t && var >= 0 && var < 5) ? t->var0(var) : nullptr; }

static int rk_launch(fedg_tint* t, double* const q[5], int kind, int stage, RKC cc, int first) {
  fedg_ctx* c = t->ctx;
  CK(cudaSetDevice(c->d.device));
  RKPtrs P;
  std::memset(&P, 0, sizeof(P));
  for (int v = 0; v < 5; ++v) {
    if (!q[v]) return fail("fedg_tint: null field");
    P.q[v] = q[v];
    P.var0[v] = t->var0(v);
    P.vtmp[v] = t->vtmp(v);
    for (int s = 0; s < t->nstage; ++s) {
      P.tex[s][v] = t->tex(s, v);
      P.tim[s][v] = t->scheme == FEDG_IMEX_ARK232 ? t->tim(s, v) : nullptr;
    }
  }
  const int bs = 256;
  CK((cudaError_t)tracked(c, FEDG_K_RK, [&] {
    k_rk<<<(unsigned)((c->n + bs - 1) / bs), bs, 0, c->stream>>>(P, kind, stage, t->nstage, cc, c->n, first);
    return (int)cudaGetLastError();
  }));
  return 0;
}

int fedg_tint_store_var0(fedg_tint* t, double* const q[5]) {
  if (!t || !q) return fail("fedg_tint_store_var0: null argument");
  RKC cc{};
  return rk_launch(t, q, 0, 1, cc, 0);
}

int fedg_tint_store_implicit(fedg_tint* t, int stage, double* const q[5]) {
  if (!t || !q || stage < 1 || stage > t->nstage) return fail("fedg_tint_store_implicit: bad argument");
  if (t->scheme != FEDG_IMEX_ARK232) return 0;  // rk_storeimpl: explicit schemes return at once
  RKC cc{};
  cc.c[0] = t->dt * t->a_im[stage - 1][stage - 1];
  return rk_launch(t, q, 1, stage, cc, stage == 1);
}

int fedg_tint_advance(fedg_tint* t, int stage, double* const q[5]) {
  if (!t || !q || stage < 1 || stage > t->nstage) return fail("fedg_tint_advance: bad argument");
  RKC cc{};
  const double dt = t->dt;
  if (t->scheme == FEDG_IMEX_ARK232) {
    cc.c[6] = t->b_ex[stage - 1] * dt;
    cc.c[7] = t->b_im[stage - 1] * dt;
    if (stage == t->nstage) return rk_launch(t, q, 3, stage, cc, 0);
    for (int j = 0; j < stage; ++j) {
      cc.c[j] = dt * t->a_ex[stage][j];
      cc.c[3 + j] = dt * t->a_im[stage][j];
    }
    return rk_launch(t, q, 2, stage, cc, 0);
  }
  const int ns = t->nstage;
  cc.c[0] = t->sig[stage][stage - 1];
  cc.c[1] = dt * t->gam[stage][stage - 1];
  cc.c[2] = t->sig[ns][stage - 1];
  cc.c[3] = dt * t->gam[ns][stage - 1];
  cc.c[4] = stage == ns ? 1.0 : 0.0;
  cc.c[5] = (std::fabs(cc.c[2]) > 1e-16 || std::fabs(cc.c[3]) > 1e-16) ? 1.0 : 0.0;
  return rk_launch(t, q, 4, stage, cc, stage == 1);
}

// ---------------- driver update loop (driver_nonhydro3d.F90:614-963) ----------------
// hout: device-mapped page-locked host arrays that the float-pair path's last stage kernel also
// writes the result to (fedg_update_host), or NULL
static int update_impl(fedg_ctx* c, double* const q[5], int nsteps, const fedg_update_opts* o, double* iters_out,
                       double* const* hout, double* const* hin = nullptr) {
  if (!c || !q || !o) return fail("fedg_update: null argument");
  if (!c->base_set) return fail("fedg_update: base state not set");
  if (o->eqs != FEDG_HEVE && o->eqs != FEDG_HEVI) return fail("fedg_update: bad eqs");
  CK(cudaSetDevice(c->d.device));
  if (o->prec == FEDG_PREC_MIXED || o->prec == FEDG_PREC_PAIR) {
    return mixed_update(c, q, nsteps, o, iters_out, hout, hin);
  }
  if (o->prec != FEDG_PREC_FP64) return fail("fedg_update: bad prec");
  const int scheme = o->eqs == FEDG_HEVE ? FEDG_SSP_RK3 : FEDG_IMEX_ARK232;
  int r = 0;
  if (c->upd_tint && (c->upd_tint->scheme != scheme || c->upd_tint->dt != o->dt)) {
    fedg_tint_destroy(c->upd_tint);
    c->upd_tint = nullptr;
  }
  if (!c->upd_tint) {
    r = fedg_tint_create(c, scheme, o->dt, &c->upd_tint);
    if (r) return r;
  }
  fedg_tint* t = c->upd_tint;
  double* dp = ensure_work(c, c->n);
  if (!dp) return fail("fedg_update: out of device memory");
  size_t ngsc = 0;
  double* gsc = nullptr;
  if (o->eqs == FEDG_HEVI && !(gsc = vi_scratch(c, &ngsc)))
    return fail(ngsc ? "fedg_update: out of device memory" : "fedg_update: the column does not fit in shared memory");
  const double* base[16] = {};
  long long nsum = 0, ncnt = 0;
  int nfail = 0;
  double* const* tf = c->trc_flux;
  const size_t nb64 = sizeof(double) * c->n;
  for (int step = 0; step < nsteps && r >= 0; ++step) {
    if (tf[0] && cudaMemcpyAsync(tf[6], q[0], nb64, cudaMemcpyDeviceToDevice, c->stream) != cudaSuccess)
      return fail("fedg_update: DDENS0_TRC copy");
    if (o->eqs == FEDG_HEVI) r = fedg_tint_store_var0(t, q);
    for (int s = 1; s <= t->nstage && r >= 0; ++s) {
      if (o->eqs == FEDG_HEVI) {
        const double fac = fedg_tint_implicit_diagfac(t, s);
        F5c qc{{q[0], q[1], q[2], q[3], q[4]}};
        F5c z{{t->var0(0), t->var0(1), t->var0(2), t->var0(3), t->var0(4)}};
        F5c none{{nullptr, nullptr, nullptr, nullptr, nullptr}};
        F5 tim{{t->tim(s - 1, 0), t->tim(s - 1, 1), t->tim(s - 1, 2), t->tim(s - 1, 3), t->tim(s - 1, 4)}};
        F5 qo{{nullptr, nullptr, nullptr, nullptr, nullptr}};
        // stage 1: var0 is the state itself (StoreImplicit copies it at stage 1)
        if (s == 1) z = qc;
        ViArgs a{fac, o->dt, o->tol, o->max_iter, 340.0};
        r = tracked(c, FEDG_K_VI, [&] {
          return launch_vi_fp64(c->op, c->prof(), qc, z, none, qo, tim, c->d_status, a, gsc, ngsc, c->stream);
        });
        if (r) return cuda_fail((cudaError_t)r, "fedg_update: cal_vi");
        if (fac != 0.0) {
          const int nb = count_status(c, &nsum, &ncnt);
          if (nb < 0) return nb;
          nfail += nb;
        }
        r = fedg_tint_store_implicit(t, s, q);
        if (r) break;
      }
      r = tracked(c, FEDG_K_PRES, [&] { return launch_drhot2pres(c->op, c->prof(), q[4], nullptr, dp, c->n, c->stream); });
      if (r) return cuda_fail((cudaError_t)r, "fedg_update: drhot2pres");
      // a slab exchanges the face layers of the stage state and DPRES (driver_nonhydro3d.F90:768-787)
      if (fedg::slab(c) && (r = fedg::halo_exchange_fp64(c, q, dp, s))) return r;
      F5c qc{{q[0], q[1], q[2], q[3], q[4]}};
      F5 tex{{fedg_tint_tend_ex(t, s, 0), fedg_tint_tend_ex(t, s, 1), fedg_tint_tend_ex(t, s, 2),
              fedg_tint_tend_ex(t, s, 3), fedg_tint_tend_ex(t, s, 4)}};
      r = tracked(c, FEDG_K_TEND, [&] { return launch_tend_fp64(c->op, c->prof(), qc, dp, tex, c->Ne, o->eqs, c->stream); });
      if (r) return cuda_fail((cudaError_t)r, "fedg_update: cal_tend");
      if (c->sl_tau > 0.0) {  // sponge layer on the explicit tendency (driver_nonhydro3d.F90:831-841)
        double* const tm[3] = {tex.v[1], tex.v[2], tex.v[3]};
        const double* const mm[3] = {q[1], q[2], q[3]};
        r = fedg_sponge_add_tend(c, tm, mm, c->sl_tau, c->sl_height, c->sl_hvel);
        if (r) return r;
      }
      if (tf[0]) {  // save_massflux of the stage state (driver_nonhydro3d.F90:900-917)
        static const double b_ssp3[3] = {1.0 / 6.0, 1.0 / 6.0, 2.0 / 3.0};
        const double w_h = o->eqs == FEDG_HEVI ? t->b_ex[s - 1] : b_ssp3[s - 1];
        const double w_v = o->eqs == FEDG_HEVI ? t->b_im[s - 1] : b_ssp3[s - 1];
        double* const mf[3] = {tf[0], tf[1], tf[2]};
        r = fedg_trc_save_massflux(c, s, q, dp, w_h, w_v, o->eqs == FEDG_HEVI, mf, tf[3], tf[4]);
        if (r) return r;
      }
      r = fedg_tint_advance(t, s, q);
    }
    // DENS_TRC: the density before the modal filter (driver_nonhydro3d.F90:920-935)
    if (r >= 0 && tf[0] && cudaMemcpyAsync(tf[5], q[0], nb64, cudaMemcpyDeviceToDevice, c->stream) != cudaSuccess)
      return fail("fedg_update: DDENS_TRC copy");
    if (r >= 0 && c->d.mf_on) r = fedg_modalfilter(c, q);
  }
  (void)base;
  if (r < 0) return r;
  if (iters_out) *iters_out = ncnt ? double(nsum) / double(ncnt) : 0.0;
  return nfail;
}

int fedg_update(fedg_ctx* c, double* const q[5], int nsteps, const fedg_update_opts* o, double* iters_out) {
  return update_impl(c, q, nsteps, o, iters_out, nullptr);
}

// fedg_update for fields in page-locked host memory: H2D into the context's device copy of the
// state, the steps, and the result back into the host arrays.  In the float-pair paths the last
// stage kernel stores q^{n+1} through the arrays' device mapping while it runs (the device-to-host
// transfer overlaps its arithmetic); the FP64 and FP32 paths copy the result back after the step.
int fedg_update_host(fedg_ctx* c, double* const host_q[5], int nsteps, const fedg_update_opts* o,
                     double* iters_out) {
  if (!c || !host_q || !o) return fail("fedg_update_host: null argument");
  CK(cudaSetDevice(c->d.device));
  double* hd[5];
  for (int v = 0; v < 5; ++v) {
    unsigned flags = 0;
    void* dp = nullptr;
    if (!host_q[v] || cudaHostGetFlags(&flags, host_q[v]) != cudaSuccess ||
        cudaHostGetDevicePointer(&dp, host_q[v], 0) != cudaSuccess || !dp) {
      cudaGetLastError();  // clear the lookup's error
      return fail("fedg_update_host: the fields must be page-locked host memory (cudaHostAlloc or cudaHostRegister)");
    }
    hd[v] = static_cast<double*>(dp);
  }
  const size_t nb = sizeof(double) * c->n;
  if (!c->host_state && cudaMalloc(&c->host_state, 5 * nb) != cudaSuccess) {
    c->host_state = nullptr;
    return fail("fedg_update_host: out of device memory");
  }
  double* dq[5];
  for (int v = 0; v < 5; ++v) dq[v] = c->host_state + (size_t)v * c->n;
  const bool direct = o->prec == FEDG_PREC_PAIR && nsteps > 0;
  // the float-pair HEVI path on a periodic mesh overlaps the H2D copies with its first stage, once the
  // reference wind is fixed (the first call takes it from the state) and when no tracer-flux outputs
  // read the state at the step's start
  double wref[2];
  const bool piped = direct && o->eqs == FEDG_HEVI && !fedg::slab(c) && fedg::ref_wind(c, wref) && !c->trc_flux[0];
  if (!piped)
    for (int v = 0; v < 5; ++v) CK(cudaMemcpyAsync(dq[v], host_q[v], nb, cudaMemcpyHostToDevice, c->stream));
  const int r = update_impl(c, dq, nsteps, o, iters_out, direct ? hd : nullptr, piped ? host_q : nullptr);
  if (r < 0) return r;
  if (!direct)  // the FP64 and FP32 paths copy the result back after the step
    for (int v = 0; v < 5; ++v) CK(cudaMemcpyAsync(host_q[v], dq[v], nb, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return r;
}

int fedg_update_set_sponge(fedg_ctx* c, double tau, double height, int hveldamp) {
  if (!c) return fail("fedg_update_set_sponge: null context");
  if (tau > 0.0 && !(height < c->d.zmax)) return fail("fedg_update_set_sponge: the damping height must be below the top");
  c->sl_tau = tau > 0.0 ? tau : 0.0;
  c->sl_height = height;
  c->sl_hvel = hveldamp != 0;
  return 0;
}

int fedg_update_set_tracer_flux(fedg_ctx* c, double* const mflx[3], double* alph_M, double* alph_P,
                                double* DDENS_TRC, double* DDENS0_TRC) {
  if (!c) return fail("fedg_update_set_tracer_flux: null context");
  if (!mflx) {
    for (int i = 0; i < 7; ++i) c->trc_flux[i] = nullptr;
    return 0;
  }
  if (fedg::slab(c)) return fail("fedg_update_set_tracer_flux: not available on a part of a decomposed mesh (periodic_x/y = FEDG_HALO)");
  if (!mflx[0] || !mflx[1] || !mflx[2] || !alph_M || !alph_P || !DDENS_TRC || !DDENS0_TRC)
    return fail("fedg_update_set_tracer_flux: null field");
  double* const v[7] = {mflx[0], mflx[1], mflx[2], alph_M, alph_P, DDENS_TRC, DDENS0_TRC};
  for (int i = 0; i < 7; ++i) c->trc_flux[i] = v[i];
  return 0;
}

// ---------------- column-guess network ----------------
int fedg_guess_create(int levels, int hidden, fedg_guess** out) {
  if (!out) return fail("fedg_guess_create: null argument");
  MlpState* m = nullptr;
  const int r = mlp_create(levels, hidden, &m);
  if (r) return r == (int)cudaErrorInvalidValue ? fail("fedg_guess_create: levels >= 1 and hidden % 64 == 0 required")
                                                 : cuda_fail((cudaError_t)r, "fedg_guess_create");
  *out = reinterpret_cast<fedg_guess*>(m);
  return 0;
}
void fedg_guess_destroy(fedg_guess* g) { mlp_free(reinterpret_cast<MlpState*>(g)); }
long long fedg_guess_num_params(const fedg_guess* g) {
  return g ? mlp_num_params(reinterpret_cast<const MlpState*>(g)) : -1;
}
int fedg_guess_set_scales(fedg_guess* g, const float in_scale[4], const float out_scale[3]) {
  if (!g || !in_scale || !out_scale) return fail("fedg_guess_set_scales: null argument");
  return mlp_set_scales(reinterpret_cast<MlpState*>(g), in_scale, out_scale);
}
int fedg_guess_set_params(fedg_guess* g, const float* host, long long n) {
  if (!g || !host) return fail("fedg_guess_set_params: null argument");
  const int r = mlp_set_params(reinterpret_cast<MlpState*>(g), host, n, 0);
  return r ? (r == (int)cudaErrorInvalidValue ? fail("fedg_guess_set_params: wrong parameter count")
                                              : cuda_fail((cudaError_t)r, "fedg_guess_set_params"))
           : 0;
}
int fedg_guess_get_params(fedg_guess* g, float* host, long long n) {
  if (!g || !host) return fail("fedg_guess_get_params: null argument");
  const int r = mlp_get_params(reinterpret_cast<MlpState*>(g), host, n, 0);
  return r ? (r == (int)cudaErrorInvalidValue ? fail("fedg_guess_get_params: wrong parameter count")
                                              : cuda_fail((cudaError_t)r, "fedg_guess_get_params"))
           : 0;
}
int fedg_guess_train_step(fedg_guess* g, const float* X, const float* T, int batch, float lr, float* loss) {
  if (!g || !X || !T || batch < 1) return fail("fedg_guess_train_step: bad argument");
  const int r = mlp_train_step(reinterpret_cast<MlpState*>(g), X, T, batch, lr, loss, 0);
  return r ? cuda_fail((cudaError_t)r, "fedg_guess_train_step") : 0;
}
int fedg_guess_loss_grad(fedg_guess* g, const float* X, const float* T, int batch, float* loss, float* grad) {
  if (!g || !X || !T || batch < 1 || !loss) return fail("fedg_guess_loss_grad: bad argument");
  const int r = mlp_loss_grad(reinterpret_cast<MlpState*>(g), X, T, batch, loss, grad, 0);
  return r ? cuda_fail((cudaError_t)r, "fedg_guess_loss_grad") : 0;
}
int fedg_guess_predict(fedg_guess* g, const float* X, float* Y, int n) {
  if (!g || !X || !Y || n < 1) return fail("fedg_guess_predict: bad argument");
  const int r = mlp_predict(reinterpret_cast<MlpState*>(g), X, Y, n, 0);
  return r ? cuda_fail((cudaError_t)r, "fedg_guess_predict") : 0;
}
int fedg_update_set_vi_neumann(fedg_ctx* c, int nterm) {
  if (!c || nterm < 0 || nterm > 8) return fail("fedg_update_set_vi_neumann: nterm must be 0..8");
  c->vi_neumann = nterm;
  return 0;
}
int fedg_update_set_wait_limit(fedg_ctx* c, int polls) {
  if (!c || polls < 0) return fail("fedg_update_set_wait_limit: bad argument");
  c->tc_polls = polls;
  return 0;
}
int fedg_guess_set_wait_limit(fedg_guess* g, int polls) {
  if (!g || polls < 0) return fail("fedg_guess_set_wait_limit: bad argument");
  return mlp_set_poll_limit(reinterpret_cast<MlpState*>(g), polls) ? fail("fedg_guess_set_wait_limit") : 0;
}
int fedg_guess_load(fedg_ctx* c, fedg_guess* g) {
  if (!c) return fail("fedg_guess_load: null ctx");
  MlpState* m = reinterpret_cast<MlpState*>(g);
  if (m) {
    if (mlp_num_params(m) <= 0) return fail("fedg_guess_load: empty network");
    mlp_set_ready(m, 1);
  }
  c->guess = m;
  return 0;
}

int fedg_prof_enable(fedg_ctx* c, int on) {
  if (!c) return fail("null ctx");
  c->prof_on = on != 0;
  return 0;
}

int fedg_prof_reset(fedg_ctx* c) {
  if (!c) return fail("null ctx");
  CK(cudaStreamSynchronize(c->stream));
  for (auto& r : c->recs) {
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  c->recs.clear();
  for (int k = 0; k < FEDG_K_COUNT; ++k) c->nlaunch[k] = 0;
  return 0;
}

int fedg_prof_read(fedg_ctx* c, int kernel, double* total_ms, long long* launches) {
  if (!c || kernel < 0 || kernel >= FEDG_K_COUNT) return fail("fedg_prof_read: bad argument");
  CK(cudaStreamSynchronize(c->stream));
  double t = 0.0;
  for (auto& r : c->recs) {
    if (r.id != kernel) continue;
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, r.a, r.b));
    t += ms;
  }
  if (total_ms) *total_ms = t;
  if (launches) *launches = c->nlaunch[kernel];
  return 0;
}

}  // extern "C"
