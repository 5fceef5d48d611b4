// fedg_halo.cu -- the face-layer exchange of a slab of a decomposed domain.
//
// FElib runs one local mesh per MPI rank and, before each tendency evaluation, exchanges the face
// values of the prognostic fields (PROG_VARS%MeshFieldComm_Exchange, FElib/src/fluid_dyn_solver/
// scale_atm_dyn_dgm_driver_nonhydro3d.F90:768-771) and of DPRES (:783-787); the exchange posts
// one send and one receive per neighbouring rank and waits for them (MeshFieldCommBase_exchange_core
// / _wait_core, FElib/src/data/scale_meshfieldcomm_base.F90:340-470).  Here the domain is split
// along x into slabs of full y extent with full-height columns: the column solves need no data of
// other slabs, and only the x faces of the first and last element layer cross a slab boundary.
//
// Per stage a slab packs the face nodes of those two layers into its send buffers (one small
// gather kernel), synchronises its stream and hands the buffers to the caller's exchange function
// (MPI, NCCL or a peer copy: the library has no transport of its own); the stage kernels then read
// the x- and x+ exterior values of the boundary elements from the receive buffers.  Buffer layout,
// per side: [6 fields][NeY*NeZ elements][N1*N1 face nodes] of 8-byte values (doubles in the FP64
// path, float pairs of the deviations in the float-pair path), face node a + N1*b of an x face
// being node (i, a, b) of the element.
#include "fedg_ctx.cuh"

namespace fedg {
namespace {

// one thread per (side, boundary element, face node); side 0 packs the x- face (i = 0) of the
// elements ex = 0, side 1 the x+ face (i = N) of the elements ex = NeX-1
__global__ void k_halo_pack_f64(const Ops op, const Prof pf, const F5c q, const double* __restrict__ dpres,
                                double* __restrict__ s0, double* __restrict__ s1) {
  const int NF = op.N1 * op.N1, nyz = op.NeY * op.NeZ;
  const size_t per = (size_t)nyz * NF;
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 2 * per) return;
  const int side = (int)(t / per);
  const size_t r = t - (size_t)side * per;
  const int eyz = (int)(r / NF), ab = (int)(r - (size_t)eyz * NF);
  const int ey = eyz % op.NeY, ez = eyz / op.NeY;
  const int ex = side == 0 ? 0 : op.NeX - 1, i = side == 0 ? 0 : op.N1 - 1;
  const int a = ab % op.N1, b = ab / op.N1;
  const size_t ke = (size_t)ex + (size_t)op.NeX * ey + (size_t)op.NeX * op.NeY * ez;
  const size_t g = ke * op.Np + i + op.N1 * a + (size_t)NF * b;
  double* out = side == 0 ? s0 : s1;
#pragma unroll
  for (int v = 0; v < 5; ++v) out[(size_t)v * per + r] = __ldg(q.v[v] + g);
  double dp;
  if (dpres) {
    dp = __ldg(dpres + g);
  } else {  // DRHOT -> DPRES as k_drhot2pres forms it
    const int lev = ez * op.N1 + b;
    dp = dpres_of(op, __ldg(pf.therm + lev) + __ldg(q.v[4] + g), __ldg(pf.pres + lev));
  }
  out[5 * per + r] = dp;
}

// the same for the float-pair stage state (deviation pairs); the DPRES slot is left alone
__global__ void k_halo_pack_pair(int NeX, int NeY, int NeZ, int N1, const X5 qs, float2* __restrict__ s0,
                                 float2* __restrict__ s1) {
  const int NF = N1 * N1, Np = NF * N1, nyz = NeY * NeZ;
  const size_t per = (size_t)nyz * NF;
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 2 * per) return;
  const int side = (int)(t / per);
  const size_t r = t - (size_t)side * per;
  const int eyz = (int)(r / NF), ab = (int)(r - (size_t)eyz * NF);
  const int ey = eyz % NeY, ez = eyz / NeY;
  const int ex = side == 0 ? 0 : NeX - 1, i = side == 0 ? 0 : N1 - 1;
  const int a = ab % N1, b = ab / N1;
  const size_t ke = (size_t)ex + (size_t)NeX * ey + (size_t)NeX * NeY * ez;
  const size_t g = ke * Np + i + N1 * a + (size_t)NF * b;
  float2* out = side == 0 ? s0 : s1;
#pragma unroll
  for (int v = 0; v < 5; ++v) out[(size_t)v * per + r] = __ldg(qs.v[v] + g);
}

unsigned halo_blocks(const fedg_ctx* c) {
  const size_t per = (size_t)c->d.NeY * c->d.NeZ * c->N1 * c->N1;
  return (unsigned)((2 * per + 255) / 256);
}

}  // namespace

bool slab(const fedg_ctx* c) { return c->d.periodic_x == FEDG_HALO; }

int halo_exchange_fp64(fedg_ctx* c, const double* const q[5], const double* dpres, int stage) {
  if (!c->hsend[0] || !c->hfn) return api_fail("fedg_update: a slab (periodic_x = FEDG_HALO) needs its halo buffers and exchange (fedg_update_set_halo)");
  const F5c qc{{q[0], q[1], q[2], q[3], q[4]}};
  int r = tracked(c, FEDG_K_AUX, [&] {
    k_halo_pack_f64<<<halo_blocks(c), 256, 0, c->stream>>>(c->op, c->prof(), qc, dpres, (double*)c->hsend[0],
                                                           (double*)c->hsend[1]);
    return (int)cudaGetLastError();
  });
  if (r) return api_cuda_fail((cudaError_t)r, "fedg_update: halo pack");
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return api_cuda_fail(e, "fedg_update: halo pack");
  if (c->hfn(c->huser, stage) != 0) return api_fail("fedg_update: the halo exchange function failed");
  return 0;
}

int halo_exchange_pair(fedg_ctx* c, const float2* const qs[5], int stage) {
  if (!c->hsend[0] || !c->hfn) return api_fail("fedg_update: a slab (periodic_x = FEDG_HALO) needs its halo buffers and exchange (fedg_update_set_halo)");
  const X5 x{{qs[0], qs[1], qs[2], qs[3], qs[4]}};
  int r = tracked(c, FEDG_K_AUX, [&] {
    k_halo_pack_pair<<<halo_blocks(c), 256, 0, c->stream>>>(c->d.NeX, c->d.NeY, c->d.NeZ, c->N1, x,
                                                            (float2*)c->hsend[0], (float2*)c->hsend[1]);
    return (int)cudaGetLastError();
  });
  if (r) return api_cuda_fail((cudaError_t)r, "fedg_update: halo pack");
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return api_cuda_fail(e, "fedg_update: halo pack");
  if (c->hfn(c->huser, stage) != 0) return api_fail("fedg_update: the halo exchange function failed");
  return 0;
}

}  // namespace fedg

extern "C" {

size_t fedg_halo_bytes(const fedg_ctx* c) {
  if (!c) return 0;
  return (size_t)6 * c->d.NeY * c->d.NeZ * c->N1 * c->N1 * 8;
}

int fedg_update_set_halo(fedg_ctx* c, void* const send[2], void* const recv[2], fedg_halo_fn fn, void* user) {
  if (!c || !send || !recv) return api_fail("fedg_update_set_halo: null argument");
  if (!fedg::slab(c)) return api_fail("fedg_update_set_halo: the context's mesh is periodic in x (periodic_x != FEDG_HALO)");
  for (int s = 0; s < 2; ++s) {
    if (!send[s] || !recv[s]) return api_fail("fedg_update_set_halo: null buffer");
    if (((uintptr_t)send[s] | (uintptr_t)recv[s]) & 7) return api_fail("fedg_update_set_halo: buffers must be 8-byte aligned");
    c->hsend[s] = send[s];
    c->hrecv[s] = recv[s];
  }
  c->hfn = fn;
  c->huser = user;
  c->op.hx[0] = (const double*)recv[0];
  c->op.hx[1] = (const double*)recv[1];
  return 0;
}

int fedg_halo_pack(fedg_ctx* c, const double* const q[5], const double* dpres) {
  if (!c || !q) return api_fail("fedg_halo_pack: null argument");
  for (int v = 0; v < 5; ++v)
    if (!q[v]) return api_fail("fedg_halo_pack: null field");
  if (!fedg::slab(c) || !c->hsend[0]) return api_fail("fedg_halo_pack: not a slab with registered halo buffers (fedg_update_set_halo)");
  if (!c->base_set) return api_fail("fedg_halo_pack: base state not set");
  cudaError_t e = cudaSetDevice(c->d.device);
  if (e != cudaSuccess) return api_cuda_fail(e, "fedg_halo_pack: cudaSetDevice");
  const F5c qc{{q[0], q[1], q[2], q[3], q[4]}};
  int r = tracked(c, FEDG_K_AUX, [&] {
    k_halo_pack_f64<<<fedg::halo_blocks(c), 256, 0, c->stream>>>(c->op, c->prof(), qc, dpres, (double*)c->hsend[0],
                                                                 (double*)c->hsend[1]);
    return (int)cudaGetLastError();
  });
  if (r) return api_cuda_fail((cudaError_t)r, "fedg_halo_pack");
  if ((e = cudaStreamSynchronize(c->stream)) != cudaSuccess) return api_cuda_fail(e, "fedg_halo_pack: synchronize");
  return 0;
}

int fedg_update_set_ref_wind(fedg_ctx* c, double u, double v) {
  if (!c) return api_fail("fedg_update_set_ref_wind: null context");
  if (!(u == u) || !(v == v)) return api_fail("fedg_update_set_ref_wind: not a number");
  fedg::set_ref_wind_given(c, u, v);
  return 0;
}

int fedg_update_get_ref_wind(const fedg_ctx* c, double* u, double* v) {
  if (!c || !u || !v) return api_fail("fedg_update_get_ref_wind: null argument");
  double w[2];
  if (!fedg::ref_wind(c, w)) return 0;
  *u = w[0];
  *v = w[1];
  return 1;
}

}  // extern "C"
