// fedg_mlp.cu -- column-guess network kernels: BF16 inference GEMMs on the 5th-generation tensor
// cores (tcgen05, TMEM accumulators) with the column gather/scatter between (Np, Ne) fields and
// feature rows fused into the first and last layer, FP32 training forward/backward, Adam.
//
// Network: x (3L+1) -> 256 -> 256 -> 3L, GELU (erf form) after the two hidden layers.
// Features (var-major): DDENS'(l), MOMZ(l), DRHOT'(l) for the L levels of the column, then
// impl_fac, each multiplied by its scale; targets: (Q - q*)(l) per variable times its scale.
#include <cmath>
#include <cstring>
#include <vector>

#include "fedg_mlp.cuh"
#include "fedg_umma.cuh"

using bf16 = __nv_bfloat16;

namespace {

using fedg::DRAIN_POLLS;
using fedg::mbar_wait_bounded;
using fedg::smem_u32;
using fedg::umma_desc;

// padding of the inference buffers: rows to the 128-row GEMM tile, inputs to the 32-wide K chunk,
// outputs to a multiple of 64 columns
constexpr int PAD_ROWS = 128, PAD_OUT = 64, PAD_K = 32;

__host__ __device__ inline int rup(int x, int a) { return (x + a - 1) / a * a; }

__device__ __forceinline__ float gelu_f(float x) { return 0.5f * x * (1.f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_d(float x) {
  return 0.5f * (1.f + erff(x * 0.70710678118654752f)) + x * 0.39894228040143268f * expf(-0.5f * x * x);
}

struct ColMap {
  int N1, Np, NeX, NeY, L;
  int lgN1;  // log2(N1): N1 is a power of two
};
// column scatter of the last inference layer: outputs (Q - q*)(l) per variable (var-major over the
// column's L levels) divided by its scale, written into (Np, Ne) fields
struct ColIO {
  ColMap cm;
  float *gd, *gm, *gr;  // guess fields
  float r0, r1, r2;     // 1 / output scales
};

// ---------------------------------------------------------------------------------------------
// Inference GEMM on the 5th-generation tensor cores:
//   C[M x Np] = act(A[M x Kp] . W[Np x Kp]^T + bias), bf16 operands (both K-major), FP32 accumulate.
// One CTA of 4 warps per 128 x BN output tile.  Each K chunk of 32 is prefetched into registers
// while the previous chunk's MMAs run, then staged in one of two shared-memory buffers in
// the no-swizzle K-major canonical layout, in 8-row x 16-byte core matrices.  K-adjacent core
// matrices are 128 B apart (leading byte offset), 8-row groups 512 B apart (stride byte
// offset).
// One elected thread issues tcgen05.mma (M = 128, N = BN, K = 16) into a TMEM accumulator of
// 128 lanes x BN columns and commits to an mbarrier.  Every wait on that barrier is bounded.
// The waits of the normal path poll at most `poll_limit` times; when one runs out the kernel
// raises *err (1), skips the epilogue's TMEM reads and stores, and drains: it waits for the
// last commit, which arrives once every MMA issued before it has completed, with the full
// limit DRAIN_POLLS.  If the drain runs out as well it raises *err (2) and still releases its
// TMEM: a CTA that exits holding TMEM can leave later allocations on its SM waiting for ever,
// while a release behind MMAs still in flight can only disturb accumulators of this launch,
// whose outputs the raised flag has already discarded.  The epilogue reads the accumulator
// with tcgen05.ld (warp w owns lanes 32w..32w+31, one output row per thread), adds the bias,
// applies GELU and stores the row.
// element offset of level l of column c within an (Np, Ne) field, from the column's base index
__device__ __forceinline__ size_t col_base(const ColMap& cm, int c) {
  const int ij = c & ((1 << (2 * cm.lgN1)) - 1), exy = c >> (2 * cm.lgN1);
  return (size_t)exy * cm.Np + (ij & (cm.N1 - 1)) + cm.N1 * (ij >> cm.lgN1);
}
__device__ __forceinline__ size_t col_off(const ColMap& cm, int l) {
  return (size_t)(l >> cm.lgN1) * ((size_t)cm.NeX * cm.NeY * cm.Np) + (size_t)((l & (cm.N1 - 1)) << (2 * cm.lgN1));
}

template <int BN, int OMODE, bool GELU>
__global__ void __launch_bounds__(128) k_gemm_tc(const bf16* __restrict__ A, const bf16* __restrict__ W,
                                                 const float* __restrict__ bias, void* __restrict__ out, int M, int Np,
                                                 int Kp, const ColIO io, int* err, int poll_limit) {
  constexpr int TM = 128, TK = 32, NA = TM * (TK / 8) / 128, NB = BN * (TK / 8) / 128;
  constexpr uint32_t TCOLS = BN <= 32 ? 32 : (BN <= 64 ? 64 : (BN <= 128 ? 128 : 256));
  static_assert(BN % 32 == 0 && BN <= 256, "tcgen05 M=128 tile: N % 32 == 0 (16 for the MMA), N <= 256");
  extern __shared__ __align__(1024) unsigned char gsm[];
  bf16* sA = reinterpret_cast<bf16*>(gsm);                // [2][TM*TK]
  bf16* sB = sA + 2 * TM * TK;                            // [2][BN*TK]
  uint64_t* mbar = reinterpret_cast<uint64_t*>(sB + 2 * BN * TK);  // [2]
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mbar + 2);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * TM, n0 = blockIdx.y * BN;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(tmem_slot)),
                 "r"(TCOLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(mbar)) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(mbar + 1)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  // instruction descriptor: D f32, A/B bf16, both K-major, N/8, M/16
  constexpr uint32_t idesc = fedg::umma_idesc_bf16(TM, BN);

  // one K chunk of this thread's A and B pieces in registers: prefetched while the previous
  // chunk's MMAs run
  uint4 ra[NA], rb[NB];
  auto load_chunk = [&](int k0) {
#pragma unroll
    for (int q = 0; q < NA; ++q) {
      const int i = tid + 128 * q, r = i >> 2, kc = i & 3;
      uint4 v = make_uint4(0, 0, 0, 0);
      if (m0 + r < M) v = *reinterpret_cast<const uint4*>(A + (size_t)(m0 + r) * Kp + k0 + kc * 8);
      ra[q] = v;
    }
#pragma unroll
    for (int q = 0; q < NB; ++q) {
      const int i = tid + 128 * q, r = i >> 2, kc = i & 3;
      rb[q] = *reinterpret_cast<const uint4*>(W + (size_t)(n0 + r) * Kp + k0 + kc * 8);
    }
  };
  auto store_chunk = [&](int buf) {  // 16-byte pieces to their core-matrix slots
#pragma unroll
    for (int q = 0; q < NA; ++q) {
      const int i = tid + 128 * q, r = i >> 2, kc = i & 3;
      *reinterpret_cast<uint4*>(sA + buf * TM * TK + ((r >> 3) * 4 + kc) * 64 + (r & 7) * 8) = ra[q];
    }
#pragma unroll
    for (int q = 0; q < NB; ++q) {
      const int i = tid + 128 * q, r = i >> 2, kc = i & 3;
      *reinterpret_cast<uint4*>(sB + buf * BN * TK + ((r >> 3) * 4 + kc) * 64 + (r & 7) * 8) = rb[q];
    }
  };

  const int nch = Kp / TK;
  bool ok = true;
  int last = -1;  // last chunk whose MMAs were committed
  load_chunk(0);
  for (int c = 0; c < nch; ++c) {
    const int buf = c & 1;
    if (c >= 2) {  // the MMAs of chunk c-2 must have read this buffer
      const bool got = mbar_wait_bounded(smem_u32(mbar + buf), (uint32_t)(((c - 2) >> 1) & 1), poll_limit);
      ok = __syncthreads_and(got) != 0;
      if (!ok) break;
    }
    store_chunk(buf);
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");  // generic stores -> tensor-core reads
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
#pragma unroll
      for (int ks = 0; ks < TK / 16; ++ks) {
        const uint64_t ad = umma_desc(smem_u32(sA + buf * TM * TK) + ks * 256, 128, 512);
        const uint64_t bd = umma_desc(smem_u32(sB + buf * BN * TK) + ks * 256, 128, 512);
        const uint32_t acc = (c > 0 || ks > 0) ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
            : "memory");
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                       smem_u32(mbar + buf))
                   : "memory");
    }
    last = c;
    if (c + 1 < nch) load_chunk((c + 1) * TK);
  }
  // the last commit arrives once every MMA before it has completed
  if (last >= 0 && ok) {
    const bool got = mbar_wait_bounded(smem_u32(mbar + (last & 1)), (uint32_t)((last >> 1) & 1), poll_limit);
    ok = __syncthreads_and(got) != 0;
  }
  if (!ok) {  // drain the MMAs in flight with the full limit before the TMEM is released
    bool drained = true;
    if (last >= 0) {
      const bool got = mbar_wait_bounded(smem_u32(mbar + (last & 1)), (uint32_t)((last >> 1) & 1), DRAIN_POLLS);
      drained = __syncthreads_and(got) != 0;
    }
    if (tid == 0) atomicMax(err, drained ? 1 : 2);
  }
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const int row = m0 + 32 * warp + lane;
  const uint32_t tl = tmem + ((uint32_t)(32 * warp) << 16);
  size_t rbase = 0;
  if constexpr (OMODE == 2) rbase = col_base(io.cm, row < M ? row : 0);
#pragma unroll 1
  for (int c0 = 0; ok && c0 < BN; c0 += 16) {  // ok is uniform over the CTA (__syncthreads_and)
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(tl + (uint32_t)c0)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
    if (row < M) {
      if constexpr (OMODE == 2) {  // scatter: output feature -> (variable, level) of column `row`
        const int L = io.cm.L;
        int f = n0 + c0;
        int vv = f / L, l = f - vv * L;
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          if (vv < 3) {
            const float y = __uint_as_float(r[j]) + bias[n0 + c0 + j];
            const size_t g = rbase + col_off(io.cm, l);
            if (vv == 0) io.gd[g] = y * io.r0;
            else if (vv == 1) io.gm[g] = y * io.r1;
            else io.gr[g] = y * io.r2;
          }
          if (++l == L) { l = 0; ++vv; }
        }
      } else {
#pragma unroll
        for (int j = 0; j < 16; j += 2) {
          const int col = n0 + c0 + j;
          float v0 = __uint_as_float(r[j]) + bias[col], v1 = __uint_as_float(r[j + 1]) + bias[col + 1];
          if (GELU) { v0 = gelu_f(v0); v1 = gelu_f(v1); }
          if constexpr (OMODE == 0) {
            *reinterpret_cast<__nv_bfloat162*>(reinterpret_cast<bf16*>(out) + (size_t)row * Np + col) =
                __floats2bfloat162_rn(v0, v1);
          } else {
            *reinterpret_cast<float2*>(reinterpret_cast<float*>(out) + (size_t)row * Np + col) = make_float2(v0, v1);
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TCOLS) : "memory");
}

template <int BN, int OMODE, bool GELU>
static void launch_tc_n(const bf16* A, const bf16* W, const float* bias, void* out, int M, int Np, int Kp,
                        const ColIO& io, int* err, int poll_limit, cudaStream_t s) {
  const size_t smem = 2 * sizeof(bf16) * (128 * 32 + BN * 32) + 2 * sizeof(uint64_t) + 16;
  auto kfn = k_gemm_tc<BN, OMODE, GELU>;
  cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  kfn<<<dim3((unsigned)((M + 127) / 128), (unsigned)(Np / BN)), 128, smem, s>>>(A, W, bias, out, M, Np, Kp, io, err,
                                                                                  poll_limit);
}

template <int OMODE, bool GELU>
static void launch_gemm_tc(const bf16* A, const bf16* W, const float* bias, void* out, int M, int Np, int Kp,
                           const ColIO& io, int* err, int poll_limit, cudaStream_t s) {
  if (Np % 256 == 0) launch_tc_n<256, OMODE, GELU>(A, W, bias, out, M, Np, Kp, io, err, poll_limit, s);
  else if (Np % 192 == 0) launch_tc_n<192, OMODE, GELU>(A, W, bias, out, M, Np, Kp, io, err, poll_limit, s);
  else if (Np % 128 == 0) launch_tc_n<128, OMODE, GELU>(A, W, bias, out, M, Np, Kp, io, err, poll_limit, s);
  else launch_tc_n<64, OMODE, GELU>(A, W, bias, out, M, Np, Kp, io, err, poll_limit, s);
}

// Generic FP32 SIMT GEMM for training: C(m,n) (+)= sum_k A(m,k) B(k,n) (+ bias[n]),
// A(m,k) = A[m*sam + k*sak], B(k,n) = B[k*sbk + n*sbn] (float or bf16), C row-major, ldc.
template <typename TB>
__global__ void __launch_bounds__(256) k_gemm_f32(const float* __restrict__ A, long sam, long sak,
                                                  const TB* __restrict__ B, long sbk, long sbn,
                                                  const float* __restrict__ bias, float* __restrict__ C, int ldc,
                                                  int M, int N, int K) {
  __shared__ float As[16][64 + 1];
  __shared__ float Bs[16][64 + 1];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int m0 = blockIdx.x * 64, n0 = blockIdx.y * 64;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += 16) {
    for (int i = threadIdx.x; i < 16 * 64; i += 256) {
      const int kk = i / 64, mm = i % 64;
      const int gm = m0 + mm, gk = k0 + kk;
      As[kk][mm] = (gm < M && gk < K) ? A[gm * sam + gk * sak] : 0.f;
      const int gn = n0 + mm;
      Bs[kk][mm] = (gn < N && gk < K) ? (float)B[gk * sbk + gn * sbn] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 16; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) a[r] = As[kk][ty * 4 + r];
#pragma unroll
      for (int c = 0; c < 4; ++c) b[c] = Bs[kk][tx * 4 + c];
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[r][c] = fmaf(a[r], b[c], acc[r][c]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int gm = m0 + ty * 4 + r, gn = n0 + tx * 4 + c;
      if (gm < M && gn < N) C[(size_t)gm * ldc + gn] = acc[r][c] + (bias ? bias[gn] : 0.f);
    }
}

__global__ void k_gelu_fwd(const float* __restrict__ z, float* __restrict__ a, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] = gelu_f(z[i]);
}
__global__ void k_gelu_bwd(const float* __restrict__ z, float* __restrict__ d, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) d[i] *= gelu_d(z[i]);
}
// dY = 2 (Y - T) / (B * dout) on the valid outputs; loss = mean (Y - T)^2
__global__ void k_mse(const float* __restrict__ Y, const float* __restrict__ T, float* __restrict__ dY, int B,
                      int dout, int doutp, float* loss) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  float l = 0.f;
  if (i < (size_t)B * doutp) {
    const int b = (int)(i / doutp), n = (int)(i % doutp);
    float g = 0.f;
    if (n < dout) {
      const float e = Y[i] - T[(size_t)b * dout + n];
      l = e * e;
      g = 2.f * e / (float(B) * float(dout));
    }
    dY[i] = g;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, l / (float(B) * float(dout)));
}
// column sums: g[n] = sum_b d[b*ld + n]
__global__ void k_colsum(const float* __restrict__ d, int B, int N, int ld, float* __restrict__ g) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  float s = 0.f;
  for (int b = 0; b < B; ++b) s += d[(size_t)b * ld + n];
  g[n] = s;
}
__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, size_t n, float lr, float b1, float b2, float eps, float c1, float c2) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}
__global__ void k_to_bf16(const float* __restrict__ a, bf16* __restrict__ b, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = __float2bfloat16_rn(a[i]);
}
__global__ void k_f32_to_bf16_rows(const float* __restrict__ X, int din, bf16* __restrict__ Xh, int dinp, int n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (size_t)n * dinp) return;
  const int r = (int)(i / dinp), c = (int)(i % dinp);
  Xh[i] = __float2bfloat16_rn(c < din ? X[(size_t)r * din + c] : 0.f);
}
__global__ void k_copy_rows(const float* __restrict__ Yp, int doutp, float* __restrict__ Y, int dout, int n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (size_t)n * dout) return;
  const int r = (int)(i / dout), c = (int)(i % dout);
  Y[i] = Yp[(size_t)r * doutp + c];
}

inline unsigned nblk(size_t n, int bs) { return (unsigned)((n + bs - 1) / bs); }

}  // namespace

struct MlpState {
  int L = 0, din = 0, h = 0, dout = 0, dinp = 0, hp = 0, doutp = 0;
  float* P = nullptr;  // FP32 master params: W1 | b1 | W2 | b2 | W3 | b3 (padded)
  float* G = nullptr;  // gradients (same layout)
  float* Mo = nullptr;
  float* Vo = nullptr;
  bf16* Wh = nullptr;  // bf16 copies of W1 | W2 | W3
  size_t oW1, ob1, oW2, ob2, oW3, ob3, np;
  size_t hW1, hW2, hW3, nh;
  int step = 0;
  float in_scale[4] = {1, 1, 1, 1};
  float out_scale[3] = {1, 1, 1};
  // training scratch
  int cap = 0;
  float *Z1 = nullptr, *A1 = nullptr, *Z2 = nullptr, *A2 = nullptr, *Y = nullptr, *dY = nullptr, *dA = nullptr;
  float* loss = nullptr;
  // inference scratch
  size_t icap = 0;
  bf16 *Xh = nullptr, *H1 = nullptr, *H2 = nullptr;
  float* Yf = nullptr;
  int* err = nullptr;  // raised by a tensor-core GEMM whose barrier wait ran out (1), or whose drain did too (2)
  int poll_limit = DRAIN_POLLS;  // polls of the tensor-core GEMMs' normal-path barrier waits
  int ready = 0;
};

void mlp_free(MlpState* m) {
  if (!m) return;
  cudaFree(m->P); cudaFree(m->G); cudaFree(m->Mo); cudaFree(m->Vo); cudaFree(m->Wh);
  cudaFree(m->Z1); cudaFree(m->A1); cudaFree(m->Z2); cudaFree(m->A2); cudaFree(m->Y); cudaFree(m->dY);
  cudaFree(m->dA); cudaFree(m->loss);
  cudaFree(m->Xh); cudaFree(m->H1); cudaFree(m->H2); cudaFree(m->Yf); cudaFree(m->err);
  delete m;
}

bool mlp_ready(const MlpState* m) { return m && m->ready; }
int mlp_set_ready(MlpState* m, int r) {
  if (!m) return (int)cudaErrorInvalidValue;
  m->ready = r;
  return 0;
}

int mlp_create(int levels, int hidden, MlpState** out) {
  if (levels < 1 || hidden < 1 || hidden % 64) return (int)cudaErrorInvalidValue;
  MlpState* m = new MlpState();
  m->L = levels;
  m->din = 3 * levels + 1;
  m->h = hidden;
  m->dout = 3 * levels;
  m->dinp = rup(m->din, PAD_K);
  m->hp = hidden;
  m->doutp = rup(m->dout, PAD_OUT);
  m->oW1 = 0;
  m->ob1 = m->oW1 + (size_t)m->hp * m->dinp;
  m->oW2 = m->ob1 + m->hp;
  m->ob2 = m->oW2 + (size_t)m->hp * m->hp;
  m->oW3 = m->ob2 + m->hp;
  m->ob3 = m->oW3 + (size_t)m->doutp * m->hp;
  m->np = m->ob3 + m->doutp;
  m->hW1 = 0;
  m->hW2 = m->hW1 + (size_t)m->hp * m->dinp;
  m->hW3 = m->hW2 + (size_t)m->hp * m->hp;
  m->nh = m->hW3 + (size_t)m->doutp * m->hp;
  cudaError_t e;
  if ((e = cudaMalloc(&m->P, sizeof(float) * m->np)) != cudaSuccess ||
      (e = cudaMalloc(&m->G, sizeof(float) * m->np)) != cudaSuccess ||
      (e = cudaMalloc(&m->Mo, sizeof(float) * m->np)) != cudaSuccess ||
      (e = cudaMalloc(&m->Vo, sizeof(float) * m->np)) != cudaSuccess ||
      (e = cudaMalloc(&m->Wh, sizeof(bf16) * m->nh)) != cudaSuccess ||
      (e = cudaMalloc(&m->loss, sizeof(float))) != cudaSuccess ||
      (e = cudaMalloc(&m->err, sizeof(int))) != cudaSuccess) {
    mlp_free(m);
    return (int)e;
  }
  cudaMemset(m->err, 0, sizeof(int));
  cudaMemset(m->P, 0, sizeof(float) * m->np);
  cudaMemset(m->G, 0, sizeof(float) * m->np);
  cudaMemset(m->Mo, 0, sizeof(float) * m->np);
  cudaMemset(m->Vo, 0, sizeof(float) * m->np);
  cudaMemset(m->Wh, 0, sizeof(bf16) * m->nh);
  *out = m;
  return 0;
}

int mlp_set_scales(MlpState* m, const float in_scale[4], const float out_scale[3]) {
  for (int k = 0; k < 4; ++k) m->in_scale[k] = in_scale[k];
  for (int k = 0; k < 3; ++k) m->out_scale[k] = out_scale[k];
  return 0;
}

long long mlp_num_params(const MlpState* m) {
  return (long long)m->h * m->din + m->h + (long long)m->h * m->h + m->h + (long long)m->dout * m->h + m->dout;
}

static void refresh_bf16(MlpState* m, cudaStream_t s) {
  const size_t n1 = (size_t)m->hp * m->dinp, n2 = (size_t)m->hp * m->hp, n3 = (size_t)m->doutp * m->hp;
  k_to_bf16<<<nblk(n1, 256), 256, 0, s>>>(m->P + m->oW1, m->Wh + m->hW1, n1);
  k_to_bf16<<<nblk(n2, 256), 256, 0, s>>>(m->P + m->oW2, m->Wh + m->hW2, n2);
  k_to_bf16<<<nblk(n3, 256), 256, 0, s>>>(m->P + m->oW3, m->Wh + m->hW3, n3);
}

// logical order: W1 (h x din) | b1 | W2 (h x h) | b2 | W3 (dout x h) | b3
static void layout_copy(const MlpState* m, const float* src, float* dst, bool to_padded) {
  size_t q = 0;
  auto blk = [&](size_t off, int rows, int cols, int ldp) {
    for (int r = 0; r < rows; ++r)
      for (int c = 0; c < cols; ++c) {
        if (to_padded) dst[off + (size_t)r * ldp + c] = src[q++];
        else dst[q++] = src[off + (size_t)r * ldp + c];
      }
  };
  blk(m->oW1, m->h, m->din, m->dinp);
  blk(m->ob1, 1, m->h, m->h);
  blk(m->oW2, m->h, m->h, m->hp);
  blk(m->ob2, 1, m->h, m->h);
  blk(m->oW3, m->dout, m->h, m->hp);
  blk(m->ob3, 1, m->dout, m->dout);
}

int mlp_set_params(MlpState* m, const float* host, long long n, cudaStream_t s) {
  if (n != mlp_num_params(m)) return (int)cudaErrorInvalidValue;
  std::vector<float> pad(m->np, 0.f);
  layout_copy(m, host, pad.data(), true);
  cudaError_t e = cudaMemcpyAsync(m->P, pad.data(), sizeof(float) * m->np, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return (int)e;
  cudaMemsetAsync(m->Mo, 0, sizeof(float) * m->np, s);
  cudaMemsetAsync(m->Vo, 0, sizeof(float) * m->np, s);
  m->step = 0;
  refresh_bf16(m, s);
  e = cudaStreamSynchronize(s);
  return (int)e;
}

int mlp_get_params(MlpState* m, float* host, long long n, cudaStream_t s) {
  if (n != mlp_num_params(m)) return (int)cudaErrorInvalidValue;
  std::vector<float> pad(m->np);
  cudaError_t e = cudaMemcpyAsync(pad.data(), m->P, sizeof(float) * m->np, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return (int)e;
  layout_copy(m, pad.data(), host, false);
  return 0;
}

static int ensure_train(MlpState* m, int B) {
  if (B <= m->cap) return 0;
  cudaFree(m->Z1); cudaFree(m->A1); cudaFree(m->Z2); cudaFree(m->A2); cudaFree(m->Y); cudaFree(m->dY); cudaFree(m->dA);
  m->cap = 0;
  cudaError_t e;
  if ((e = cudaMalloc(&m->Z1, sizeof(float) * (size_t)B * m->hp)) != cudaSuccess ||
      (e = cudaMalloc(&m->A1, sizeof(float) * (size_t)B * m->hp)) != cudaSuccess ||
      (e = cudaMalloc(&m->Z2, sizeof(float) * (size_t)B * m->hp)) != cudaSuccess ||
      (e = cudaMalloc(&m->A2, sizeof(float) * (size_t)B * m->hp)) != cudaSuccess ||
      (e = cudaMalloc(&m->Y, sizeof(float) * (size_t)B * m->doutp)) != cudaSuccess ||
      (e = cudaMalloc(&m->dY, sizeof(float) * (size_t)B * m->doutp)) != cudaSuccess ||
      (e = cudaMalloc(&m->dA, sizeof(float) * (size_t)B * m->hp)) != cudaSuccess)
    return (int)e;
  m->cap = B;
  return 0;
}

template <typename TB>
static void gemm_f32(const float* A, long sam, long sak, const TB* B, long sbk, long sbn, const float* bias, float* C,
                     int ldc, int M, int N, int K, cudaStream_t s) {
  dim3 g((M + 63) / 64, (N + 63) / 64);
  k_gemm_f32<TB><<<g, 256, 0, s>>>(A, sam, sak, B, sbk, sbn, bias, C, ldc, M, N, K);
}

// forward + backward on a batch; X: B x din (FP32, scaled features), T: B x dout (scaled targets).
// Fills m->G with the gradient of the mean-square loss; returns the loss in *loss (device scalar).
static int forward_backward(MlpState* m, const float* X, const float* T, int B, cudaStream_t s) {
  int r = ensure_train(m, B);
  if (r) return r;
  const int hp = m->hp, dinp = m->dinp, doutp = m->doutp, din = m->din;
  const bf16* W1 = m->Wh + m->hW1;
  const bf16* W2 = m->Wh + m->hW2;
  const bf16* W3 = m->Wh + m->hW3;
  float* P = m->P;
  // forward with the BF16 weights (FP32 accumulate)
  gemm_f32<bf16>(X, din, 1, W1, 1, dinp, P + m->ob1, m->Z1, hp, B, hp, din, s);
  k_gelu_fwd<<<nblk((size_t)B * hp, 256), 256, 0, s>>>(m->Z1, m->A1, (size_t)B * hp);
  gemm_f32<bf16>(m->A1, hp, 1, W2, 1, hp, P + m->ob2, m->Z2, hp, B, hp, hp, s);
  k_gelu_fwd<<<nblk((size_t)B * hp, 256), 256, 0, s>>>(m->Z2, m->A2, (size_t)B * hp);
  gemm_f32<bf16>(m->A2, hp, 1, W3, 1, hp, P + m->ob3, m->Y, doutp, B, doutp, hp, s);
  cudaMemsetAsync(m->loss, 0, sizeof(float), s);
  k_mse<<<nblk((size_t)B * doutp, 256), 256, 0, s>>>(m->Y, T, m->dY, B, m->dout, doutp, m->loss);
  // backward (straight-through for the BF16 rounding)
  float* G = m->G;
  cudaMemsetAsync(G, 0, sizeof(float) * m->np, s);
  gemm_f32<float>(m->dY, 1, doutp, m->A2, hp, 1, nullptr, G + m->oW3, hp, doutp, hp, B, s);   // dW3 = dY^T A2
  k_colsum<<<nblk(doutp, 128), 128, 0, s>>>(m->dY, B, doutp, doutp, G + m->ob3);
  gemm_f32<bf16>(m->dY, doutp, 1, W3, hp, 1, nullptr, m->dA, hp, B, hp, doutp, s);              // dA2 = dY W3
  k_gelu_bwd<<<nblk((size_t)B * hp, 256), 256, 0, s>>>(m->Z2, m->dA, (size_t)B * hp);          // dZ2
  gemm_f32<float>(m->dA, 1, hp, m->A1, hp, 1, nullptr, G + m->oW2, hp, hp, hp, B, s);          // dW2 = dZ2^T A1
  k_colsum<<<nblk(hp, 128), 128, 0, s>>>(m->dA, B, hp, hp, G + m->ob2);
  gemm_f32<bf16>(m->dA, hp, 1, W2, hp, 1, nullptr, m->Z2, hp, B, hp, hp, s);                    // dA1 -> Z2 (reuse)
  k_gelu_bwd<<<nblk((size_t)B * hp, 256), 256, 0, s>>>(m->Z1, m->Z2, (size_t)B * hp);          // dZ1 in Z2
  gemm_f32<float>(m->Z2, 1, hp, X, din, 1, nullptr, G + m->oW1, dinp, hp, din, B, s);          // dW1 = dZ1^T X
  k_colsum<<<nblk(hp, 128), 128, 0, s>>>(m->Z2, B, hp, hp, G + m->ob1);
  return (int)cudaGetLastError();
}

int mlp_train_step(MlpState* m, const float* X, const float* T, int B, float lr, float* loss, cudaStream_t s) {
  int r = forward_backward(m, X, T, B, s);
  if (r) return r;
  m->step += 1;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float c1 = 1.f - powf(b1, (float)m->step), c2 = 1.f - powf(b2, (float)m->step);
  k_adam<<<nblk(m->np, 256), 256, 0, s>>>(m->P, m->G, m->Mo, m->Vo, m->np, lr, b1, b2, eps, c1, c2);
  refresh_bf16(m, s);
  if (loss) {
    cudaError_t e = cudaMemcpyAsync(loss, m->loss, sizeof(float), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return (int)e;
  }
  return (int)cudaGetLastError();
}

int mlp_loss_grad(MlpState* m, const float* X, const float* T, int B, float* loss, float* grad_host, cudaStream_t s) {
  int r = forward_backward(m, X, T, B, s);
  if (r) return r;
  std::vector<float> pad(m->np);
  cudaError_t e = cudaMemcpyAsync(pad.data(), m->G, sizeof(float) * m->np, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(loss, m->loss, sizeof(float), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return (int)e;
  if (grad_host) layout_copy(m, pad.data(), grad_host, false);
  return 0;
}

static int ensure_infer(MlpState* m, size_t n) {
  if (n <= m->icap) return 0;
  cudaFree(m->Xh); cudaFree(m->H1); cudaFree(m->H2); cudaFree(m->Yf);
  m->icap = 0;
  const size_t nr = (size_t)rup((int)std::min<size_t>(n, 1u << 30), PAD_ROWS);
  cudaError_t e;
  if ((e = cudaMalloc(&m->Xh, sizeof(bf16) * nr * m->dinp)) != cudaSuccess ||
      (e = cudaMalloc(&m->H1, sizeof(bf16) * nr * m->hp)) != cudaSuccess ||
      (e = cudaMalloc(&m->H2, sizeof(bf16) * nr * m->hp)) != cudaSuccess ||
      (e = cudaMalloc(&m->Yf, sizeof(float) * nr * m->doutp)) != cudaSuccess)
    return (int)e;
  m->icap = nr;
  return 0;
}

// the three layers on the tensor cores over the feature rows in m->Xh; with io the last layer
// scatters its outputs to the guess fields, otherwise it writes FP32 rows to m->Yf
static int run_layers(MlpState* m, int n, const ColIO* io, cudaStream_t s) {
  const ColIO none{};
  const int pl = m->poll_limit;
  launch_gemm_tc<0, true>(m->Xh, m->Wh + m->hW1, m->P + m->ob1, m->H1, n, m->hp, m->dinp, none, m->err, pl, s);
  launch_gemm_tc<0, true>(m->H1, m->Wh + m->hW2, m->P + m->ob2, m->H2, n, m->hp, m->hp, none, m->err, pl, s);
  if (io) launch_gemm_tc<2, false>(m->H2, m->Wh + m->hW3, m->P + m->ob3, nullptr, n, m->doutp, m->hp, *io, m->err, pl, s);
  else launch_gemm_tc<1, false>(m->H2, m->Wh + m->hW3, m->P + m->ob3, m->Yf, n, m->doutp, m->hp, none, m->err, pl, s);
  return (int)cudaGetLastError();
}

// impl_fac feature (times its scale) and zero padding of every feature row
__global__ void k_rows_tail(bf16* __restrict__ X, int dinp, int f0, float fac, int ncol) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int w = dinp - f0;
  if (i >= (size_t)ncol * w) return;
  const int r = (int)(i / w), f = f0 + (int)(i % w);
  X[(size_t)r * dinp + f] = __float2bfloat16_rn(f == f0 ? fac : 0.f);
}

int mlp_rows(MlpState* m, int ncol, double impl_fac, MlpRows* out, cudaStream_t s) {
  if (!m || !m->ready) return (int)cudaErrorNotReady;
  int r = ensure_infer(m, (size_t)ncol);
  if (r) return r;
  k_rows_tail<<<nblk((size_t)ncol * (m->dinp - 3 * m->L), 256), 256, 0, s>>>(m->Xh, m->dinp, 3 * m->L,
                                                                             (float)impl_fac * m->in_scale[3], ncol);
  out->X = m->Xh;
  out->dinp = m->dinp;
  out->L = m->L;
  for (int v = 0; v < 3; ++v) out->s[v] = m->in_scale[v];
  return (int)cudaGetLastError();
}

int mlp_take_error(MlpState* m, cudaStream_t s) {
  int h = 0;
  cudaError_t e = cudaMemcpyAsync(&h, m->err, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return (int)e;
  if (h) cudaMemsetAsync(m->err, 0, sizeof(int), s);
  return h ? -h : 0;
}

int mlp_set_poll_limit(MlpState* m, int polls) {
  if (!m || polls < 0) return (int)cudaErrorInvalidValue;
  m->poll_limit = polls;
  return 0;
}

int mlp_predict(MlpState* m, const float* X, float* Y, int n, cudaStream_t s) {
  int r = ensure_infer(m, (size_t)n);
  if (r) return r;
  k_f32_to_bf16_rows<<<nblk((size_t)n * m->dinp, 256), 256, 0, s>>>(X, m->din, m->Xh, m->dinp, n);
  if ((r = run_layers(m, n, nullptr, s))) return r;
  k_copy_rows<<<nblk((size_t)n * m->dout, 256), 256, 0, s>>>(m->Yf, m->doutp, Y, m->dout, n);
  if ((r = (int)cudaGetLastError())) return r;
  return mlp_take_error(m, s) ? (int)cudaErrorLaunchTimeout : 0;
}

int mlp_infer(MlpState* m, const fedg::Ops& op, float* gd, float* gm, float* gr, cudaStream_t s) {
  if (!m || !m->ready) return (int)cudaErrorNotReady;
  if (m->L != op.L) return (int)cudaErrorInvalidValue;
  const int ncol = op.NeX * op.NeY * op.N1 * op.N1;
  if ((size_t)ncol > m->icap) return (int)cudaErrorInvalidValue;  // mlp_rows prepares the rows first
  ColIO io{};
  io.cm = ColMap{op.N1, op.Np, op.NeX, op.NeY, op.L, op.N1 == 8 ? 3 : (op.N1 == 4 ? 2 : (op.N1 == 2 ? 1 : 0))};
  if ((1 << io.cm.lgN1) != op.N1) return (int)cudaErrorInvalidValue;
  io.gd = gd; io.gm = gm; io.gr = gr;
  io.r0 = 1.f / m->out_scale[0]; io.r1 = 1.f / m->out_scale[1]; io.r2 = 1.f / m->out_scale[2];
  return run_layers(m, ncol, &io, s);
}
