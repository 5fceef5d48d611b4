// fedg_mlp.cu -- column-guess network kernels: BF16 tensor-core inference GEMMs, FP32 training
// forward/backward, Adam, and the column gather/scatter between (Np, Ne) fields and feature rows.
//
// Network: x (3L+1) -> 256 -> 256 -> 3L, GELU (erf form) after the two hidden layers.
// Features (var-major): DDENS'(l), MOMZ(l), DRHOT'(l) for the L levels of the column, then
// impl_fac, each multiplied by its scale; targets: (Q - q*)(l) per variable times its scale.
#include <cmath>
#include <cstring>
#include <vector>

#include "fedg_mlp.cuh"

using bf16 = __nv_bfloat16;

namespace {

constexpr int BM = 128, BN = 64, BK = 32;

__host__ __device__ inline int rup(int x, int a) { return (x + a - 1) / a * a; }

__device__ __forceinline__ float gelu_f(float x) { return 0.5f * x * (1.f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_d(float x) {
  return 0.5f * (1.f + erff(x * 0.70710678118654752f)) + x * 0.39894228040143268f * expf(-0.5f * x * x);
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// C[M x Np] = act(A[M x Kp] . W[Np x Kp]^T + bias), A/W bf16 row-major, Kp % 32 == 0, Np % 64 == 0.
// Block tile 128 x 64 x 32, four warps of 64 x 32, m16n8k16 BF16 tensor-core MMAs, FP32 accumulate.
template <bool GELU, bool OUTBF16>
__global__ void __launch_bounds__(128) k_gemm_bf16(const bf16* __restrict__ A, const bf16* __restrict__ W,
                                                   const float* __restrict__ bias, void* __restrict__ out, int M,
                                                   int Np, int Kp) {
  __shared__ __align__(16) bf16 As[BM][BK + 8];
  __shared__ __align__(16) bf16 Ws[BN][BK + 8];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wm = warp >> 1, wn = warp & 1;
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
  float acc[4][4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b)
#pragma unroll
      for (int c = 0; c < 4; ++c) acc[a][b][c] = 0.f;
  for (int k0 = 0; k0 < Kp; k0 += BK) {
    for (int i = threadIdx.x; i < BM * BK / 8; i += 128) {
      const int r = i / (BK / 8), cv = i % (BK / 8);
      const int gr = m0 + r;
      uint4 v = make_uint4(0, 0, 0, 0);
      if (gr < M) v = *reinterpret_cast<const uint4*>(A + (size_t)gr * Kp + k0 + cv * 8);
      *reinterpret_cast<uint4*>(&As[r][cv * 8]) = v;
    }
    for (int i = threadIdx.x; i < BN * BK / 8; i += 128) {
      const int r = i / (BK / 8), cv = i % (BK / 8);
      *reinterpret_cast<uint4*>(&Ws[r][cv * 8]) =
          *reinterpret_cast<const uint4*>(W + (size_t)(n0 + r) * Kp + k0 + cv * 8);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; kk += 16) {
      uint32_t af[4][4], bfr[4][2];
      const int ar = lane >> 2, ac = kk + (lane & 3) * 2;
#pragma unroll
      for (int mt = 0; mt < 4; ++mt) {
        const int row = wm * 64 + mt * 16 + ar;
        af[mt][0] = *reinterpret_cast<const uint32_t*>(&As[row][ac]);
        af[mt][1] = *reinterpret_cast<const uint32_t*>(&As[row + 8][ac]);
        af[mt][2] = *reinterpret_cast<const uint32_t*>(&As[row][ac + 8]);
        af[mt][3] = *reinterpret_cast<const uint32_t*>(&As[row + 8][ac + 8]);
      }
#pragma unroll
      for (int nt = 0; nt < 4; ++nt) {
        const int n = wn * 32 + nt * 8 + ar;
        bfr[nt][0] = *reinterpret_cast<const uint32_t*>(&Ws[n][ac]);
        bfr[nt][1] = *reinterpret_cast<const uint32_t*>(&Ws[n][ac + 8]);
      }
#pragma unroll
      for (int mt = 0; mt < 4; ++mt)
#pragma unroll
        for (int nt = 0; nt < 4; ++nt) mma_bf16(acc[mt][nt], af[mt], bfr[nt]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int mt = 0; mt < 4; ++mt)
#pragma unroll
    for (int nt = 0; nt < 4; ++nt) {
      const int col = n0 + wn * 32 + nt * 8 + (lane & 3) * 2;
      const float b0 = bias[col], b1 = bias[col + 1];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int row = m0 + wm * 64 + mt * 16 + (lane >> 2) + h * 8;
        if (row >= M) continue;
        float v0 = acc[mt][nt][2 * h] + b0, v1 = acc[mt][nt][2 * h + 1] + b1;
        if (GELU) { v0 = gelu_f(v0); v1 = gelu_f(v1); }
        if (OUTBF16) {
          *reinterpret_cast<__nv_bfloat162*>(reinterpret_cast<bf16*>(out) + (size_t)row * Np + col) =
              __floats2bfloat162_rn(v0, v1);
        } else {
          *reinterpret_cast<float2*>(reinterpret_cast<float*>(out) + (size_t)row * Np + col) = make_float2(v0, v1);
        }
      }
    }
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

// column c = (ex, ey, i, j): level l of variable v lives at ((ez*nxy + exy)*Np + i + N1 j + N1^2 k)
struct ColMap {
  int N1, Np, NeX, NeY, L;
};
__device__ __forceinline__ size_t col_gidx(const ColMap& cm, int c, int l) {
  const int NF = cm.N1 * cm.N1;
  const int ij = c % NF, exy = c / NF, ci = ij % cm.N1, cj = ij / cm.N1;
  const int ez = l / cm.N1, k = l - ez * cm.N1;
  return ((size_t)ez * cm.NeX * cm.NeY + exy) * cm.Np + ci + cm.N1 * cj + NF * k;
}
__global__ void k_gather_x(ColMap cm, const double* __restrict__ qd, const double* __restrict__ qm,
                           const double* __restrict__ qr, float fac, float s0, float s1, float s2, bf16* __restrict__ X,
                           int dinp, int ncol) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (size_t)ncol * dinp) return;
  const int c = (int)(i / dinp), f = (int)(i % dinp);
  float x = 0.f;
  if (f < 3 * cm.L) {
    const int v = f / cm.L, l = f - v * cm.L;
    const size_t g = col_gidx(cm, c, l);
    x = v == 0 ? (float)qd[g] * s0 : (v == 1 ? (float)qm[g] * s1 : (float)qr[g] * s2);
  } else if (f == 3 * cm.L) {
    x = fac;
  }
  X[i] = __float2bfloat16_rn(x);
}
__global__ void k_scatter_y(ColMap cm, const float* __restrict__ Y, int doutp, float r0, float r1, float r2,
                            float* __restrict__ gd, float* __restrict__ gm, float* __restrict__ gr, int ncol) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (size_t)ncol * 3 * cm.L) return;
  const int c = (int)(i / (3 * cm.L)), f = (int)(i % (3 * cm.L));
  const int v = f / cm.L, l = f - v * cm.L;
  const float y = Y[(size_t)c * doutp + f];
  const size_t g = col_gidx(cm, c, l);
  if (v == 0) gd[g] = y * r0;
  else if (v == 1) gm[g] = y * r1;
  else gr[g] = y * r2;
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
  int ready = 0;
};

void mlp_free(MlpState* m) {
  if (!m) return;
  cudaFree(m->P); cudaFree(m->G); cudaFree(m->Mo); cudaFree(m->Vo); cudaFree(m->Wh);
  cudaFree(m->Z1); cudaFree(m->A1); cudaFree(m->Z2); cudaFree(m->A2); cudaFree(m->Y); cudaFree(m->dY);
  cudaFree(m->dA); cudaFree(m->loss);
  cudaFree(m->Xh); cudaFree(m->H1); cudaFree(m->H2); cudaFree(m->Yf);
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
  m->dinp = rup(m->din, BK);
  m->hp = hidden;
  m->doutp = rup(m->dout, BN);
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
      (e = cudaMalloc(&m->loss, sizeof(float))) != cudaSuccess) {
    mlp_free(m);
    return (int)e;
  }
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
  const size_t nr = (size_t)rup((int)std::min<size_t>(n, 1u << 30), BM);
  cudaError_t e;
  if ((e = cudaMalloc(&m->Xh, sizeof(bf16) * nr * m->dinp)) != cudaSuccess ||
      (e = cudaMalloc(&m->H1, sizeof(bf16) * nr * m->hp)) != cudaSuccess ||
      (e = cudaMalloc(&m->H2, sizeof(bf16) * nr * m->hp)) != cudaSuccess ||
      (e = cudaMalloc(&m->Yf, sizeof(float) * nr * m->doutp)) != cudaSuccess)
    return (int)e;
  m->icap = nr;
  return 0;
}

static int run_layers(MlpState* m, int n, cudaStream_t s) {
  const dim3 g1((n + BM - 1) / BM, m->hp / BN), g3((n + BM - 1) / BM, m->doutp / BN);
  k_gemm_bf16<true, true><<<g1, 128, 0, s>>>(m->Xh, m->Wh + m->hW1, m->P + m->ob1, m->H1, n, m->hp, m->dinp);
  k_gemm_bf16<true, true><<<g1, 128, 0, s>>>(m->H1, m->Wh + m->hW2, m->P + m->ob2, m->H2, n, m->hp, m->hp);
  k_gemm_bf16<false, false><<<g3, 128, 0, s>>>(m->H2, m->Wh + m->hW3, m->P + m->ob3, m->Yf, n, m->doutp, m->hp);
  return (int)cudaGetLastError();
}

int mlp_predict(MlpState* m, const float* X, float* Y, int n, cudaStream_t s) {
  int r = ensure_infer(m, (size_t)n);
  if (r) return r;
  k_f32_to_bf16_rows<<<nblk((size_t)n * m->dinp, 256), 256, 0, s>>>(X, m->din, m->Xh, m->dinp, n);
  if ((r = run_layers(m, n, s))) return r;
  k_copy_rows<<<nblk((size_t)n * m->dout, 256), 256, 0, s>>>(m->Yf, m->doutp, Y, m->dout, n);
  return (int)cudaGetLastError();
}

int mlp_infer(MlpState* m, const fedg::Ops& op, const double* qd, const double* qm, const double* qr, double impl_fac,
              float* gd, float* gm, float* gr, cudaStream_t s) {
  if (!m || !m->ready) return (int)cudaErrorNotReady;
  if (m->L != op.L) return (int)cudaErrorInvalidValue;
  const int ncol = op.NeX * op.NeY * op.N1 * op.N1;
  int r = ensure_infer(m, (size_t)ncol);
  if (r) return r;
  ColMap cm{op.N1, op.Np, op.NeX, op.NeY, op.L};
  k_gather_x<<<nblk((size_t)ncol * m->dinp, 256), 256, 0, s>>>(cm, qd, qm, qr, (float)impl_fac * m->in_scale[3],
                                                               m->in_scale[0], m->in_scale[1], m->in_scale[2], m->Xh,
                                                               m->dinp, ncol);
  if ((r = run_layers(m, ncol, s))) return r;
  k_scatter_y<<<nblk((size_t)ncol * 3 * m->L, 256), 256, 0, s>>>(cm, m->Yf, m->doutp, 1.f / m->out_scale[0],
                                                                 1.f / m->out_scale[1], 1.f / m->out_scale[2], gd, gm,
                                                                 gr, ncol);
  return (int)cudaGetLastError();
}
