// fedg_halo.cu -- the face-layer exchange of one part of a decomposed domain.
//
// FElib runs one local mesh per MPI rank and, before each tendency evaluation, exchanges the face
// values of the prognostic fields (PROG_VARS%MeshFieldComm_Exchange, FElib/src/fluid_dyn_solver/
// scale_atm_dyn_dgm_driver_nonhydro3d.F90:768-771) and of DPRES (:783-787); the exchange posts
// one send and one receive per neighbouring rank and waits for them (MeshFieldCommBase_exchange_core
// / _wait_core, FElib/src/data/scale_meshfieldcomm_base.F90:340-470).  Here the domain is split
// along x into slabs of full y extent with full-height columns: the column solves need no data of
// other slabs, and only the x faces of the first and last element layer cross a slab boundary.
//
// The domain may also be split along y (a 2D grid of parts, periodic_y = FEDG_HALO), with the y
// faces of the first and last element rows exchanged the same way.
//
// Per stage a part packs the face nodes of its boundary layers into its send buffers (one small
// gather kernel), synchronises its stream and hands the buffers to the caller's exchange function
// (MPI, NCCL or a peer copy: the library has no transport of its own); the stage kernels then read
// the exterior values of the boundary faces from the receive buffers.  Sides 0..3 are x-, x+, y-,
// y+; buffer layout per side: [6 fields][boundary elements][N1*N1 face nodes] of 8-byte values
// (doubles in the FP64 path, float pairs of the deviations in the float-pair path, FP32 deviations
// in .x in the FP32 mode), the boundary
// elements numbered ey + NeY*ez on the x sides and ex + NeX*ez on the y sides, face node a + N1*b
// being node (i, a, b) of the element on an x face and (a, j, b) on a y face.
#include "fedg_ctx.cuh"

namespace fedg {
namespace {

struct HaloGeom {  // the halo sides of a part and their sizes
  int NeX, NeY, NeZ, N1;
  bool side[4];
  __host__ __device__ size_t per(int sd) const { return (size_t)(sd < 2 ? NeY : NeX) * NeZ * N1 * N1; }
};

// one thread per (side, boundary element, face node) over the halo sides in order
__device__ __forceinline__ bool halo_locate(const HaloGeom& hg, size_t t, int& sd, size_t& r, size_t& g) {
  for (sd = 0; sd < 4; ++sd) {
    if (!hg.side[sd]) continue;
    const size_t per = hg.per(sd);
    if (t < per) break;
    t -= per;
  }
  if (sd == 4) return false;
  r = t;
  const int N1 = hg.N1, NF = N1 * N1, Np = NF * N1;
  const int eb = (int)(t / NF), ab = (int)(t - (size_t)eb * NF), a = ab % N1, b = ab / N1;
  int ex, ey, ez, i, j;
  if (sd < 2) {
    ey = eb % hg.NeY; ez = eb / hg.NeY; ex = sd == 0 ? 0 : hg.NeX - 1;
    i = sd == 0 ? 0 : N1 - 1; j = a;
  } else {
    ex = eb % hg.NeX; ez = eb / hg.NeX; ey = sd == 2 ? 0 : hg.NeY - 1;
    i = a; j = sd == 2 ? 0 : N1 - 1;
  }
  const size_t ke = (size_t)ex + (size_t)hg.NeX * ey + (size_t)hg.NeX * hg.NeY * ez;
  g = ke * Np + i + N1 * j + (size_t)NF * b;
  return true;
}

struct Send4 { void* s[4]; };
struct F5f { const float* v[5]; };

__global__ void k_halo_pack_f64(const Ops op, const Prof pf, const HaloGeom hg, const F5c q,
                                const double* __restrict__ dpres, Send4 out) {
  int sd;
  size_t r, g;
  if (!halo_locate(hg, (size_t)blockIdx.x * blockDim.x + threadIdx.x, sd, r, g)) return;
  double* o = static_cast<double*>(out.s[sd]);
  const size_t per = hg.per(sd);
#pragma unroll
  for (int v = 0; v < 5; ++v) o[(size_t)v * per + r] = __ldg(q.v[v] + g);
  double dp;
  if (dpres) {
    dp = __ldg(dpres + g);
  } else {  // DRHOT -> DPRES as k_drhot2pres forms it
    const int N1 = hg.N1, NF = N1 * N1;
    const int lev = (int)((g / ((size_t)NF * N1)) / ((size_t)hg.NeX * hg.NeY)) * N1 + (int)(g % ((size_t)NF * N1)) / NF;
    dp = dpres_of(op, __ldg(pf.therm + lev) + __ldg(q.v[4] + g), __ldg(pf.pres + lev));
  }
  o[5 * per + r] = dp;
}

// the same for the float-pair stage state (deviation pairs); the DPRES slot is left alone
__global__ void k_halo_pack_pair(const HaloGeom hg, const X5 qs, Send4 out) {
  int sd;
  size_t r, g;
  if (!halo_locate(hg, (size_t)blockIdx.x * blockDim.x + threadIdx.x, sd, r, g)) return;
  float2* o = static_cast<float2*>(out.s[sd]);
  const size_t per = hg.per(sd);
#pragma unroll
  for (int v = 0; v < 5; ++v) o[(size_t)v * per + r] = __ldg(qs.v[v] + g);
}

// the same for the FP32 stage state of the FP32 mode: the value in .x of each 8-byte slot
__global__ void k_halo_pack_f32(const HaloGeom hg, const F5f qs, Send4 out) {
  int sd;
  size_t r, g;
  if (!halo_locate(hg, (size_t)blockIdx.x * blockDim.x + threadIdx.x, sd, r, g)) return;
  float2* o = static_cast<float2*>(out.s[sd]);
  const size_t per = hg.per(sd);
#pragma unroll
  for (int v = 0; v < 5; ++v) o[(size_t)v * per + r] = make_float2(__ldg(qs.v[v] + g), 0.f);
}

HaloGeom halo_geom(const fedg_ctx* c) {
  HaloGeom hg{c->d.NeX, c->d.NeY, c->d.NeZ, c->N1, {false, false, false, false}};
  for (int sd = 0; sd < 4; ++sd) hg.side[sd] = halo_dir(c, sd);
  return hg;
}

unsigned halo_blocks(const HaloGeom& hg) {
  size_t n = 0;
  for (int sd = 0; sd < 4; ++sd)
    if (hg.side[sd]) n += hg.per(sd);
  return (unsigned)((n + 255) / 256);
}

Send4 send4(const fedg_ctx* c) { return Send4{{c->hsend[0], c->hsend[1], c->hsend[2], c->hsend[3]}}; }

bool halo_ready(const fedg_ctx* c) {
  for (int sd = 0; sd < 4; ++sd)
    if (halo_dir(c, sd) && (!c->hsend[sd] || !c->hrecv[sd])) return false;
  return true;
}

}  // namespace

bool slab(const fedg_ctx* c) { return c->d.periodic_x == FEDG_HALO || c->d.periodic_y == FEDG_HALO; }
bool halo_dir(const fedg_ctx* c, int side) {
  return side < 2 ? c->d.periodic_x == FEDG_HALO : c->d.periodic_y == FEDG_HALO;
}

int halo_exchange_fp64(fedg_ctx* c, const double* const q[5], const double* dpres, int stage) {
  if (!halo_ready(c) || !c->hfn)
    return api_fail("fedg_update: a decomposed mesh (periodic_x/y = FEDG_HALO) needs its halo buffers and exchange (fedg_update_set_halo)");
  const F5c qc{{q[0], q[1], q[2], q[3], q[4]}};
  const HaloGeom hg = halo_geom(c);
  int r = tracked(c, FEDG_K_AUX, [&] {
    k_halo_pack_f64<<<halo_blocks(hg), 256, 0, c->stream>>>(c->op, c->prof(), hg, qc, dpres, send4(c));
    return (int)cudaGetLastError();
  });
  if (r) return api_cuda_fail((cudaError_t)r, "fedg_update: halo pack");
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return api_cuda_fail(e, "fedg_update: halo pack");
  if (c->hfn(c->huser, stage) != 0) return api_fail("fedg_update: the halo exchange function failed");
  return 0;
}

int halo_exchange_pair(fedg_ctx* c, const float2* const qs[5], int stage) {
  if (!halo_ready(c) || !c->hfn)
    return api_fail("fedg_update: a decomposed mesh (periodic_x/y = FEDG_HALO) needs its halo buffers and exchange (fedg_update_set_halo)");
  const X5 x{{qs[0], qs[1], qs[2], qs[3], qs[4]}};
  const HaloGeom hg = halo_geom(c);
  int r = tracked(c, FEDG_K_AUX, [&] {
    k_halo_pack_pair<<<halo_blocks(hg), 256, 0, c->stream>>>(hg, x, send4(c));
    return (int)cudaGetLastError();
  });
  if (r) return api_cuda_fail((cudaError_t)r, "fedg_update: halo pack");
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return api_cuda_fail(e, "fedg_update: halo pack");
  if (c->hfn(c->huser, stage) != 0) return api_fail("fedg_update: the halo exchange function failed");
  return 0;
}

int halo_exchange_f32(fedg_ctx* c, const float* const qs[5], int stage) {
  if (!halo_ready(c) || !c->hfn)
    return api_fail("fedg_update: a decomposed mesh (periodic_x/y = FEDG_HALO) needs its halo buffers and exchange (fedg_update_set_halo)");
  const F5f x{{qs[0], qs[1], qs[2], qs[3], qs[4]}};
  const HaloGeom hg = halo_geom(c);
  int r = tracked(c, FEDG_K_AUX, [&] {
    k_halo_pack_f32<<<halo_blocks(hg), 256, 0, c->stream>>>(hg, x, send4(c));
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

size_t fedg_halo_bytes(const fedg_ctx* c, int side) {
  if (!c || side < 0 || side > 3 || !fedg::halo_dir(c, side)) return 0;
  return (size_t)6 * (side < 2 ? c->d.NeY : c->d.NeX) * c->d.NeZ * c->N1 * c->N1 * 8;
}

int fedg_update_set_halo(fedg_ctx* c, void* const send[4], void* const recv[4], fedg_halo_fn fn, void* user) {
  if (!c || !send || !recv) return api_fail("fedg_update_set_halo: null argument");
  if (!fedg::slab(c)) return api_fail("fedg_update_set_halo: the context's mesh is periodic in x and y (no FEDG_HALO side)");
  for (int s = 0; s < 4; ++s) {
    if (!fedg::halo_dir(c, s)) {
      c->hsend[s] = c->hrecv[s] = nullptr;
      c->op.hx[s] = nullptr;
      continue;
    }
    if (!send[s] || !recv[s]) return api_fail("fedg_update_set_halo: null buffer on a halo side");
    if (((uintptr_t)send[s] | (uintptr_t)recv[s]) & 7) return api_fail("fedg_update_set_halo: buffers must be 8-byte aligned");
    c->hsend[s] = send[s];
    c->hrecv[s] = recv[s];
    c->op.hx[s] = static_cast<const double*>(recv[s]);
  }
  c->hfn = fn;
  c->huser = user;
  return 0;
}

int fedg_halo_pack(fedg_ctx* c, const double* const q[5], const double* dpres) {
  if (!c || !q) return api_fail("fedg_halo_pack: null argument");
  for (int v = 0; v < 5; ++v)
    if (!q[v]) return api_fail("fedg_halo_pack: null field");
  if (!fedg::slab(c) || !fedg::halo_ready(c))
    return api_fail("fedg_halo_pack: not a decomposed mesh with registered halo buffers (fedg_update_set_halo)");
  if (!c->base_set) return api_fail("fedg_halo_pack: base state not set");
  cudaError_t e = cudaSetDevice(c->d.device);
  if (e != cudaSuccess) return api_cuda_fail(e, "fedg_halo_pack: cudaSetDevice");
  const F5c qc{{q[0], q[1], q[2], q[3], q[4]}};
  const fedg::HaloGeom hg = fedg::halo_geom(c);
  int r = tracked(c, FEDG_K_AUX, [&] {
    fedg::k_halo_pack_f64<<<fedg::halo_blocks(hg), 256, 0, c->stream>>>(c->op, c->prof(), hg, qc, dpres, fedg::send4(c));
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
