// fedg_restart.cu -- restart files of the dynamics state.
//
// FElib writes and reads its restart state through NetCDF (FElib/src/file/scale_file_restart_meshfield.F90:
// 136-186 defines and writes the prognostic and auxiliary mesh fields; model/atm_nonhydro3d/src/atmos/
// mod_atmos_vars.F90:580-633 reads DDENS, MOMX, MOMY, MOMZ, DRHOT and the hydrostatic DENS_hyd, PRES_hyd
// back).  This image has no NetCDF library, so the same content goes into a flat little-endian file:
//
//   offset  0  char[8]   "FEDGRST1"
//           8  int32     porder, NeX, NeY, NeZ, Np, nfields (= 8), has_ref_wind, reserved
//          40  int64     step
//          48  float64   time, dt, ref_wind_u, ref_wind_v
//          80  char[32]  time-integration scheme name (FElib's TINTEG_TYPE, NUL-padded)
//         112  float64   fields, each Np * Ne values in FElib's column-major (Np, Ne) order:
//                        DDENS, MOMX, MOMY, MOMZ, DRHOT, DENS_hyd, PRES_hyd, THERM_hyd
//
// The hydrostatic fields are written from the context's registered base state (its per-level
// profiles expanded to every node: the library accepts only horizontally homogeneous base states).
// The reference wind is the one hidden quantity of the fast update paths (FEDG_PREC_MIXED/PAIR
// express MOMX/MOMY relative to DENS_hyd (U, V), fixed from the first state they see): a restart
// that carries it lets a restored run continue bit for bit.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "fedg_ctx.cuh"

namespace {

constexpr char kMagic[8] = {'F', 'E', 'D', 'G', 'R', 'S', 'T', '1'};
constexpr int kFields = 8;
constexpr size_t kHeader = 112;

bool host_is_little_endian() {
  const unsigned int one = 1;
  unsigned char b;
  std::memcpy(&b, &one, 1);
  return b == 1;
}

struct File {
  FILE* f = nullptr;
  ~File() {
    if (f) std::fclose(f);
  }
};

}  // namespace

extern "C" int fedg_restart_write(fedg_ctx* c, const char* path, const double* const q[5],
                                  const fedg_restart_info* info) {
  if (!c || !path || !q || !info) return api_fail("fedg_restart_write: null argument");
  for (int v = 0; v < 5; ++v)
    if (!q[v]) return api_fail("fedg_restart_write: null field");
  if (!c->base_set) return api_fail("fedg_restart_write: no base state registered (fedg_set_base_state)");
  if (!host_is_little_endian()) return api_fail("fedg_restart_write: big-endian host");
  cudaError_t e = cudaSetDevice(c->d.device);
  if (e != cudaSuccess) return api_cuda_fail(e, "fedg_restart_write: cudaSetDevice");
  e = cudaStreamSynchronize(c->stream);  // the fields are complete once the context's work is
  if (e != cudaSuccess) return api_cuda_fail(e, "fedg_restart_write: synchronize");
  double wind[2] = {0.0, 0.0};
  const int has_wind = fedg::ref_wind(c, wind) ? 1 : 0;

  unsigned char head[kHeader];
  std::memset(head, 0, sizeof(head));
  std::memcpy(head, kMagic, 8);
  const int ints[8] = {c->d.porder, c->d.NeX, c->d.NeY, c->d.NeZ, c->Np, kFields, has_wind, 0};
  std::memcpy(head + 8, ints, sizeof(ints));
  const long long step = info->step;
  std::memcpy(head + 40, &step, 8);
  const double dbl[4] = {info->time, info->dt, wind[0], wind[1]};
  std::memcpy(head + 48, dbl, sizeof(dbl));
  std::memcpy(head + 80, info->scheme, sizeof(info->scheme));
  head[80 + 31] = 0;

  File fh;
  fh.f = std::fopen(path, "wb");
  if (!fh.f) return api_fail(std::string("fedg_restart_write: cannot open ") + path);
  if (std::fwrite(head, 1, kHeader, fh.f) != kHeader) return api_fail("fedg_restart_write: write failed");
  std::vector<double> h(c->n);
  for (int v = 0; v < 5; ++v) {
    if ((e = cudaMemcpy(h.data(), q[v], sizeof(double) * c->n, cudaMemcpyDeviceToHost)) != cudaSuccess)
      return api_cuda_fail(e, "fedg_restart_write: field copy");
    if (std::fwrite(h.data(), sizeof(double), c->n, fh.f) != c->n) return api_fail("fedg_restart_write: write failed");
  }
  // the base state from the registered per-level profiles: DENS_hyd, PRES_hyd, THERM_hyd
  std::vector<double> prof(4 * (size_t)c->L);
  if ((e = cudaMemcpy(prof.data(), c->d_prof, sizeof(double) * 4 * c->L, cudaMemcpyDeviceToHost)) != cudaSuccess)
    return api_cuda_fail(e, "fedg_restart_write: profile copy");
  const size_t nxy = c->nxy;
  for (int m = 0; m < 3; ++m) {
    for (size_t g = 0; g < c->n; ++g) {
      const size_t ke = g / c->Np;
      const int k = (int)(g % c->Np) / (c->N1 * c->N1), ez = (int)(ke / nxy);
      h[g] = prof[(size_t)m * c->L + ez * c->N1 + k];
    }
    if (std::fwrite(h.data(), sizeof(double), c->n, fh.f) != c->n) return api_fail("fedg_restart_write: write failed");
  }
  if (std::fclose(fh.f) != 0) {
    fh.f = nullptr;
    return api_fail("fedg_restart_write: close failed");
  }
  fh.f = nullptr;
  return 0;
}

extern "C" int fedg_restart_read(fedg_ctx* c, const char* path, double* const q[5], double* const base[3],
                                 fedg_restart_info* info) {
  if (!c || !path || !q) return api_fail("fedg_restart_read: null argument");
  for (int v = 0; v < 5; ++v)
    if (!q[v]) return api_fail("fedg_restart_read: null field");
  if (!host_is_little_endian()) return api_fail("fedg_restart_read: big-endian host");
  File fh;
  fh.f = std::fopen(path, "rb");
  if (!fh.f) return api_fail(std::string("fedg_restart_read: cannot open ") + path);
  unsigned char head[kHeader];
  if (std::fread(head, 1, kHeader, fh.f) != kHeader || std::memcmp(head, kMagic, 8) != 0)
    return api_fail("fedg_restart_read: not a restart file of this library");
  int ints[8];
  std::memcpy(ints, head + 8, sizeof(ints));
  if (ints[0] != c->d.porder || ints[1] != c->d.NeX || ints[2] != c->d.NeY || ints[3] != c->d.NeZ ||
      ints[4] != c->Np || ints[5] != kFields)
    return api_fail("fedg_restart_read: the file's mesh (porder " + std::to_string(ints[0]) + ", " +
                    std::to_string(ints[1]) + "x" + std::to_string(ints[2]) + "x" + std::to_string(ints[3]) +
                    ") does not match the context's");
  long long step;
  double dbl[4];
  std::memcpy(&step, head + 40, 8);
  std::memcpy(dbl, head + 48, sizeof(dbl));
  cudaError_t e = cudaSetDevice(c->d.device);
  if (e != cudaSuccess) return api_cuda_fail(e, "fedg_restart_read: cudaSetDevice");
  if ((e = cudaStreamSynchronize(c->stream)) != cudaSuccess)
    return api_cuda_fail(e, "fedg_restart_read: synchronize");
  std::vector<double> h(c->n);
  for (int v = 0; v < kFields; ++v) {
    if (std::fread(h.data(), sizeof(double), c->n, fh.f) != c->n) return api_fail("fedg_restart_read: file too short");
    double* dst = v < 5 ? q[v] : (base ? base[v - 5] : nullptr);
    if (dst && (e = cudaMemcpy(dst, h.data(), sizeof(double) * c->n, cudaMemcpyHostToDevice)) != cudaSuccess)
      return api_cuda_fail(e, "fedg_restart_read: field copy");
  }
  if (ints[6]) fedg::set_ref_wind_given(c, dbl[2], dbl[3]);
  if (info) {
    info->step = step;
    info->time = dbl[0];
    info->dt = dbl[1];
    std::memcpy(info->scheme, head + 80, sizeof(info->scheme));
    info->scheme[sizeof(info->scheme) - 1] = 0;
  }
  return 0;
}
