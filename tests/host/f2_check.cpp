// Host check of the float-pair arithmetic of fe-project_gb300/csrc/fedg_f2.cuh: the header is
// compiled for the CPU with host stand-ins for the CUDA rounding intrinsics (IEEE single
// precision, no contraction), and every operation is compared with long double references.
// Prints one line per operation: name, max relative error, samples.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>

#include <cuda_runtime.h>

static inline float __fadd_rn(float a, float b) { volatile float r = a + b; return r; }
static inline float __fsub_rn(float a, float b) { volatile float r = a - b; return r; }
static inline float __fmul_rn(float a, float b) { volatile float r = a * b; return r; }
static inline float __fmaf_rn(float a, float b, float c) { return std::fmaf(a, b, c); }
static inline float __fdividef(float a, float b) { volatile float r = a / b; return r; }
static inline float __uint_as_float(unsigned u) { float f; std::memcpy(&f, &u, 4); return f; }
static inline long long __double_as_longlong(double d) { long long u; std::memcpy(&u, &d, 8); return u; }
static inline float __uint2float_rn(unsigned u) { return (float)u; }

#include "fedg_f2.cuh"

using namespace fedg;
typedef long double LD;
static LD val(f2 a) { return (LD)a.h + (LD)a.l; }

int main() {
  std::mt19937_64 rng(12345);
  std::normal_distribution<double> nd(0.0, 1.0);
  std::uniform_real_distribution<double> ex(-12.0, 12.0);
  auto rnd = [&]() { return nd(rng) * std::pow(10.0, ex(rng)); };
  const int S = 200000;
  LD e_split = 0, e_add = 0, e_mul = 0, e_mulf = 0, e_recip = 0, e_addf = 0, e_dot = 0;
  for (int s = 0; s < S; ++s) {
    const double x = rnd(), y = rnd();
    const f2 a = f2_split(x), b = f2_split(y);
    e_split = std::fmax(e_split, std::fabs(val(a) - (LD)x) / std::fabs((LD)x));
    const LD A = val(a), B = val(b);
    const f2 s2 = f2_add(a, b);
    const LD sref = A + B;
    if (sref != 0) e_add = std::fmax(e_add, std::fabs(val(s2) - sref) / (std::fabs(A) + std::fabs(B)));
    e_mul = std::fmax(e_mul, std::fabs(val(f2_mul(a, b)) - A * B) / std::fabs(A * B));
    const float fy = (float)y;
    e_mulf = std::fmax(e_mulf, std::fabs(val(f2_mul_f(a, fy)) - A * (LD)fy) / std::fabs(A * (LD)fy));
    e_addf = std::fmax(e_addf, std::fabs(val(f2_add_f(a, fy)) - (A + (LD)fy)) / (std::fabs(A) + std::fabs((LD)fy)));
    if (std::fabs(x) > 1e-30 && std::fabs(x) < 1e30)
      e_recip = std::fmax(e_recip, std::fabs(val(f2_recip(a)) * A - 1.0L));
    // dot product with cancellation: derivative-like weights summing to zero
    if (s % 10 == 0) {
      f2acc acc;
      LD ref = 0, mag = 0;
      const double base = rnd();
      for (int m = 0; m < 8; ++m) {
        const double w = (m < 7) ? nd(rng) : 0.0;
        const double xm = base * (1.0 + 1e-6 * nd(rng));
        const f2 wp = f2_split(w), xp = f2_split(xm);
        acc.add(wp, xp);
        ref += val(wp) * val(xp);
        mag += std::fabs(val(wp) * val(xp));
      }
      if (mag > 0) e_dot = std::fmax(e_dot, std::fabs(val(acc.get()) - ref) / mag);
    }
  }
  std::printf("split %.3Le %d\nadd %.3Le %d\nmul %.3Le %d\nmul_f %.3Le %d\nadd_f %.3Le %d\nrecip %.3Le %d\ndot %.3Le %d\n",
              e_split, S, e_add, S, e_mul, S, e_mulf, S, e_addf, S, e_recip, S, e_dot, S / 10);
  return 0;
}
