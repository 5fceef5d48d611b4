// fedg_static.cu -- an explicit-tendency entry point that allocates no device memory.
//
// fedg_cal_tend_ex() forms the pressure deviation DPRES in a scratch field that the context
// allocates with cudaMalloc on first use.  Some callers cannot allow that: a Fortran model whose
// device memory is owned by its OpenACC runtime (FElib's GPU build keeps every field in
// `!$acc enter data` regions and sizes the device pool when the run starts), or any host that
// forbids device allocation once its set-up phase is over, because a late cudaMalloc can fail or
// fragment memory that another allocator has already claimed.  fedg_cal_tend_ex_noalloc() runs
// the same two kernels (DRHOT -> DPRES, then the tendency) with DPRES held in the file-scope
// device array below instead.
//
// The array is part of the library image: every GPU that loads the library holds its
// FEDG_NOALLOC_MAX_NODES doubles (16 MiB) until the process exits.  Host code cannot use the
// symbol name as a device address; the device address is looked up with cudaGetSymbolAddress,
// once per device, with that device current.  With CUDA's lazy module loading that lookup is what
// loads this translation unit's module onto the device, and loading it reserves the 16 MiB.  So the
// lookup runs during set-up: fedg_ctx_create calls noalloc_setup() on the context's device, and
// the entry point itself only reads the address recorded then.
#include <mutex>

#include "fedg_ctx.cuh"

#define FEDG_NOALLOC_MAX_NODES (2 * 1024 * 1024)  // Np*Ne limit of fedg_cal_tend_ex_noalloc
#define FEDG_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) double g_noalloc_dpres[FEDG_NOALLOC_MAX_NODES];

namespace {
std::mutex g_noalloc_mu;
double* g_noalloc_ptr[FEDG_NOALLOC_MAX_DEVICES] = {};
cudaError_t g_noalloc_err[FEDG_NOALLOC_MAX_DEVICES] = {};  // outcome of a failed set-up lookup

// Makes `dev` current for the lifetime of the guard and restores the caller's device afterwards.
struct DeviceGuard {
  int prev = -1;
  cudaError_t err = cudaSuccess;
  explicit DeviceGuard(int dev) {
    if ((err = cudaGetDevice(&prev)) == cudaSuccess && prev != dev) err = cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    int now = -1;
    if (prev >= 0 && cudaGetDevice(&now) == cudaSuccess && now != prev) cudaSetDevice(prev);
  }
};
}  // namespace

namespace fedg {
// Looks up the static array's device address on `dev` (the current device) and records it.  Called
// by fedg_ctx_create.  A failure is recorded, not returned: the context stays usable, and
// fedg_cal_tend_ex_noalloc reports the recorded error instead of trying again at call time.
void noalloc_setup(int dev) {
  if (dev < 0 || dev >= FEDG_NOALLOC_MAX_DEVICES) return;
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (g_noalloc_ptr[dev]) return;
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_dpres);
  if (e != cudaSuccess) {
    g_noalloc_err[dev] = e;
    cudaGetLastError();  // the failure is reported by the entry point, not by the next call
    return;
  }
  g_noalloc_ptr[dev] = static_cast<double*>(p);
  g_noalloc_err[dev] = cudaSuccess;
}
}  // namespace fedg

extern "C" int fedg_cal_tend_ex_noalloc(fedg_ctx* c, const double* const in[16], double* const out[5], int eqs) {
  if (!c || !in || !out) return api_fail("fedg_cal_tend_ex_noalloc: null argument");
  for (int v = 0; v < 5; ++v)
    if (!in[v] || !out[v]) return api_fail("fedg_cal_tend_ex_noalloc: null field");
  if (eqs != FEDG_HEVE && eqs != FEDG_HEVI) return api_fail("fedg_cal_tend_ex_noalloc: eqs must be FEDG_HEVE or FEDG_HEVI");
  if (c->n > (size_t)FEDG_NOALLOC_MAX_NODES)
    return api_fail("fedg_cal_tend_ex_noalloc: Np*Ne = " + std::to_string(c->n) + " exceeds the static scratch of " +
                    std::to_string(FEDG_NOALLOC_MAX_NODES) + " nodes; use fedg_cal_tend_ex");
  // the base state must already be registered (fedg_set_base_state allocates host scratch)
  if (!c->base_set || in[6] != c->base_ptr[0] || in[7] != c->base_ptr[1] || in[9] != c->base_ptr[2])
    return api_fail("fedg_cal_tend_ex_noalloc: register this base state with fedg_set_base_state first");
  const int dev = c->d.device;
  if (dev < 0 || dev >= FEDG_NOALLOC_MAX_DEVICES) return api_fail("fedg_cal_tend_ex_noalloc: device ordinal out of range");
  double* scratch = nullptr;
  cudaError_t setup_err = cudaSuccess;
  {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    scratch = g_noalloc_ptr[dev];
    setup_err = g_noalloc_err[dev];
  }
  if (!scratch)
    return api_fail(std::string("fedg_cal_tend_ex_noalloc: the static scratch was not loaded on this device when the "
                                "context was created (") +
                    (setup_err != cudaSuccess ? cudaGetErrorString(setup_err) : "no lookup") + ")");
  DeviceGuard guard(dev);
  if (guard.err != cudaSuccess) return api_cuda_fail(guard.err, "fedg_cal_tend_ex_noalloc: cudaSetDevice");
  // Every entry the tendency kernel reads (own and face-neighbour nodes, all inside [0, Np*Ne))
  // is written by the DPRES kernel first, so nothing needs clearing between calls.
  int r = tracked(c, FEDG_K_PRES, [&] { return launch_drhot2pres(c->op, c->prof(), in[4], nullptr, scratch, c->n, c->stream); });
  if (r) return api_cuda_fail((cudaError_t)r, "fedg_cal_tend_ex_noalloc: DRHOT2PRES");
  F5c q{{in[0], in[1], in[2], in[3], in[4]}};
  F5 t{{out[0], out[1], out[2], out[3], out[4]}};
  r = tracked(c, FEDG_K_TEND, [&] { return launch_tend_fp64(c->op, c->prof(), q, scratch, t, c->Ne, eqs, c->stream); });
  if (r) return api_cuda_fail((cudaError_t)r, "fedg_cal_tend_ex_noalloc: tendency");
  return 0;
}
