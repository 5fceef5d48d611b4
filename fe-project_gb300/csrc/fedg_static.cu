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
// once per device, with that device current, on the first call on that device.
#include <mutex>

#include "fedg_ctx.cuh"

#define FEDG_NOALLOC_MAX_NODES (2 * 1024 * 1024)  // Np*Ne limit of fedg_cal_tend_ex_noalloc
#define FEDG_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) double g_noalloc_dpres[FEDG_NOALLOC_MAX_NODES];

namespace {
std::mutex g_noalloc_mu;
double* g_noalloc_ptr[FEDG_NOALLOC_MAX_DEVICES] = {};
}  // namespace

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
  cudaError_t e = cudaSetDevice(dev);
  if (e != cudaSuccess) return api_cuda_fail(e, "fedg_cal_tend_ex_noalloc: cudaSetDevice");
  double* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {  // first call on this device: look up the array's device address
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_noalloc_dpres);
      if (e != cudaSuccess) return api_cuda_fail(e, "fedg_cal_tend_ex_noalloc: cudaGetSymbolAddress");
      g_noalloc_ptr[dev] = static_cast<double*>(p);
    }
    scratch = g_noalloc_ptr[dev];
  }
  // Every entry the tendency kernel reads (own and face-neighbour nodes, all inside [0, Np*Ne))
  // is written by the DPRES kernel first, so nothing needs clearing between calls.
  c->nlaunch[FEDG_K_PRES]++;
  int r = launch_drhot2pres(c->op, c->prof(), in[4], nullptr, scratch, c->n, c->stream);
  if (r) return api_cuda_fail((cudaError_t)r, "fedg_cal_tend_ex_noalloc: DRHOT2PRES");
  F5c q{{in[0], in[1], in[2], in[3], in[4]}};
  F5 t{{out[0], out[1], out[2], out[3], out[4]}};
  c->nlaunch[FEDG_K_TEND]++;
  r = launch_tend_fp64(c->op, c->prof(), q, scratch, t, c->Ne, eqs, c->stream);
  if (r) return api_cuda_fail((cudaError_t)r, "fedg_cal_tend_ex_noalloc: tendency");
  return 0;
}
