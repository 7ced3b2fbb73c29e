// Learned T2 starting amplitudes: a small MLP trained on converged amplitudes.
//
// For every doubles element (i,j,a,b) of a Hamiltonian the network maps MP2-level pair
// features to the difference between the converged CCSD amplitude and the MP2 guess
// (ccwfn.cc:75-87 gives the MP2 guess t2 = <ij|ab>/D).  The plain CCSD iteration then
// starts from t2 = t2_mp2 + prediction; its own convergence test decides the answer.
//
//   features (kFeat = 15), D = e_i + e_j - e_a - e_b, S = kScale:
//     0: S*<ij|ab>/D   1: S*<ij|ba>/D   2: S*<ij|ab>   3: -1/D
//     4: (e_i+e_j)/2   5: (e_a+e_b)/2   6: [i==j]      7: [a==b]
//     8: S*<ab|ab>     9: S*<ij|ij>    10: S*(<ia|ia> + <jb|jb>)   11: S*(<ia|ai> + <jb|bj>)
//    12: |e_i-e_j|/2  13: |e_a-e_b|/2  14: (e_i-e_j)(e_a-e_b)/4
//   (8-11 are the diagonal ladder and ring elements that dress the MP2 denominator; every
//   feature is invariant under (i,j,a,b) -> (j,i,b,a), so the guess keeps the symmetry
//   of the exact amplitudes)
//   target: T*(t2_ccsd - t2_mp2),   T = kTarget
//   network: 12 -> 256 -> 256 -> 1, SiLU; weights stored in FP16 for the forward and
//   backward passes, FP32 master copies for the Adam update, FP32 accumulation.
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <random>
#include <vector>

#include "cc.h"
#include "tc_ptx.h"

namespace ucc {
void count_kernel_launch();
Ctx& ctx_of(ucc_ctx* h);               // capi.cpp
void mlp_guess(Ctx& c, ucc_mlp* net);  // t2 guess of the network into the context's T_guess
// pair features (and, with targets, the scaled t2 - t2_mp2 of converged amplitudes) to host
void mlp_features(Ctx& c, float* out, size_t rows, float* targets, bool with_targets);

namespace mlp {

constexpr int kFeat = 15, kHid = 256;
constexpr double kScale = 100.0, kTarget = 1000.0;

__device__ __forceinline__ float silu(float z) { return z / (1.0f + __expf(-z)); }
__device__ __forceinline__ float dsilu(float z) {
  const float s = 1.0f / (1.0f + __expf(-z));
  return s * (1.0f + z * (1.0f - s));
}

template <typename T>
__device__ __forceinline__ float ld(const T* p, int64_t i);
template <>
__device__ __forceinline__ float ld<float>(const float* p, int64_t i) {
  return p[i];
}
template <>
__device__ __forceinline__ float ld<__half>(const __half* p, int64_t i) {
  return __half2float(p[i]);
}

// C[m][n] (+)= sum_k A[m*sAm + k*sAk] * B[k*sBk + n*sBn]; 64x64 tiles, 4x4 per thread,
// FP32 accumulation, B in FP32 or FP16
template <typename TB>
__global__ void __launch_bounds__(256) gemm_f32(int M, int N, int K, const float* A, int64_t sAm, int64_t sAk,
                                                const TB* B, int64_t sBk, int64_t sBn, float* C, int64_t ldc,
                                                int accumulate) {
  __shared__ float As[16][65];
  __shared__ float Bs[16][65];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const int m0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += 16) {
    for (int e = threadIdx.x; e < 64 * 16; e += 256) {
      const int mm = e % 64, kk = e / 64;
      const int m = m0 + mm, k = k0 + kk;
      As[kk][mm] = (m < M && k < K) ? A[(int64_t)m * sAm + (int64_t)k * sAk] : 0.f;
      const int n = n0 + mm;
      Bs[kk][mm] = (n < N && k < K) ? ld<TB>(B, (int64_t)k * sBk + (int64_t)n * sBn) : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 16; kk++) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; i++) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; j++) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const int m = m0 + ty + 16 * i;
    if (m >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const int n = n0 + tx + 16 * j;
      if (n >= N) continue;
      float* c = C + (int64_t)m * ldc + n;
      *c = accumulate ? *c + acc[i][j] : acc[i][j];
    }
  }
}

// Z += bias (per column); A = silu(Z)
__global__ void bias_act(int64_t n, int h, float* Z, const float* b, float* A) {
  for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < n * h; x += (int64_t)gridDim.x * blockDim.x) {
    const float z = Z[x] + b[x % h];
    Z[x] = z;
    if (A) A[x] = silu(z);
  }
}
// y = y + b3 (scalar)
__global__ void add_scalar(int64_t n, float* y, const float* b) {
  for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < n; x += (int64_t)gridDim.x * blockDim.x)
    y[x] += b[0];
}
// dy = 2 (y - t) / n ; loss partial sums
__global__ void mse_grad(int64_t n, const float* y, const float* t, float* dy, float* loss_part) {
  float s = 0.f;
  for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < n; x += (int64_t)gridDim.x * blockDim.x) {
    const float d = y[x] - t[x];
    dy[x] = 2.f * d / (float)n;
    s += d * d;
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if (threadIdx.x % 32 == 0) atomicAdd(loss_part, s / (float)n);
}
// dA (in) -> dZ = dA * silu'(Z), in place
__global__ void act_grad(int64_t n, const float* Z, float* dA) {
  for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < n; x += (int64_t)gridDim.x * blockDim.x)
    dA[x] *= dsilu(Z[x]);
}
// column sums of an n x h matrix (bias gradients), one thread per column
__global__ void col_sum(int64_t n, int h, const float* X, float* out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= h) return;
  float s = 0.f;
  for (int64_t r = 0; r < n; r++) s += X[r * h + j];
  out[j] = s;
}
// Adam on FP32 masters, then the FP16 working copy
__global__ void adam(int64_t n, float* w, const float* g, float* m, float* v, __half* wh, float lr, float b1, float b2,
                     float c1, float c2) {
  for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < n; x += (int64_t)gridDim.x * blockDim.x) {
    const float gi = g[x];
    const float mi = b1 * m[x] + (1.f - b1) * gi;
    const float vi = b2 * v[x] + (1.f - b2) * gi * gi;
    m[x] = mi;
    v[x] = vi;
    const float wi = w[x] - lr * (mi / c1) / (sqrtf(vi / c2) + 1e-8f);
    w[x] = wi;
    if (wh) wh[x] = __float2half(wi);
  }
}
__global__ void to_half(int64_t n, const float* w, __half* wh) {
  for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < n; x += (int64_t)gridDim.x * blockDim.x)
    wh[x] = __float2half(w[x]);
}
// gather rows idx[r] of X (n x f) and t
__global__ void gather_rows(int64_t nb, int f, const int64_t* idx, const float* X, const float* t, float* Xb,
                            float* tb) {
  for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < nb * f; x += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = x / f, c = x % f;
    Xb[x] = X[idx[r] * f + c];
    if (c == 0) tb[r] = t[idx[r]];
  }
}

// features of every (i,j,a,b) of the loaded Hamiltonian
__global__ void features_kernel(int no, int nv, const double* Voovv, const double* Voooo, const double* Vovov,
                                const double* Vvvvv, const double* eps, float* X) {
  const int64_t n = (int64_t)no * no * nv * nv;
  const int64_t o = no, v = nv;
  for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < n; x += (int64_t)gridDim.x * blockDim.x) {
    const int b = (int)(x % nv);
    int64_t r = x / nv;
    const int a = (int)(r % nv);
    r /= nv;
    const int j = (int)(r % no), i = (int)(r / no);
    const double D = ((eps[i] + eps[j]) - eps[no + a]) - eps[no + b];
    const double vij = Voovv[x];
    const double vx = Voovv[(((int64_t)i * no + j) * nv + b) * nv + a];
    float* f = X + x * kFeat;
    f[0] = (float)(kScale * vij / D);
    f[1] = (float)(kScale * vx / D);
    f[2] = (float)(kScale * vij);
    f[3] = (float)(-1.0 / D);
    f[4] = (float)(0.5 * (eps[i] + eps[j]));
    f[5] = (float)(0.5 * (eps[no + a] + eps[no + b]));
    f[6] = i == j ? 1.f : 0.f;
    f[7] = a == b ? 1.f : 0.f;
    f[8] = (float)(kScale * Vvvvv[((a * v + b) * v + a) * v + b]);                                // <ab|ab>
    f[9] = (float)(kScale * Voooo[((i * o + j) * o + i) * o + j]);                                // <ij|ij>
    f[10] = (float)(kScale * (Vovov[((i * v + a) * o + i) * v + a] + Vovov[((j * v + b) * o + j) * v + b]));
    f[11] = (float)(kScale * (Voovv[((i * o + i) * v + a) * v + a] + Voovv[((j * o + j) * v + b) * v + b]));
    const double dij = eps[i] - eps[j], dab = eps[no + a] - eps[no + b];
    f[12] = (float)(0.5 * fabs(dij));
    f[13] = (float)(0.5 * fabs(dab));
    f[14] = (float)(0.25 * dij * dab);
  }
}
// target = T * (t2 - t2_mp2)
__global__ void targets_kernel(int no, int nv, const double* Voovv, const double* eps, const double* t2, float* y) {
  const int64_t n = (int64_t)no * no * nv * nv;
  for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < n; x += (int64_t)gridDim.x * blockDim.x) {
    const int b = (int)(x % nv);
    int64_t r = x / nv;
    const int a = (int)(r % nv);
    r /= nv;
    const int j = (int)(r % no), i = (int)(r / no);
    const double D = ((eps[i] + eps[j]) - eps[no + a]) - eps[no + b];
    y[x] = (float)(kTarget * (t2[x] - Voovv[x] / D));
  }
}
unsigned grid1(int64_t n) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 16)); }

// ------------------------------------------------------------------------------------
// The guess in one pass on the tensor cores: for 128 doubles elements per tile, the pair
// features and the first layer (15 -> 256, FP32 on the CUDA cores), the second layer
// (256 -> 256) as one tcgen05 MMA chain with FP16 operands and an FP32 accumulator in
// tensor memory, and the output layer with the guess t2 = t2_mp2 + y / kTarget in the
// epilogue.  No feature or activation array reaches global memory.
//
// Shared memory (1024-aligned): the second layer's weights as the MMA's B operand, W2^T
// [256 n][256 k] in four 64-wide K blocks (K-major, 128-byte swizzle: the 16-byte chunk c
// of row r sits at chunk c ^ (r & 7)); the tile's activations as the A operand [128][256]
// in the same layout; the tile's features [128][16] and MP2 amplitudes; b1, b2, w3 in
// FP32; the partial outputs of the column halves.  The first layer runs register-blocked:
// lane l of warp w holds W1 for the hidden units 8l .. 8l+7 for the whole kernel and
// computes them for the rows 16w .. 16w+15, reading each row's features once as a
// broadcast (one shared-memory load per 8 multiply-adds; loading W1 from shared memory per
// multiply-add made the pass load-bound, 107 ms at no=32/nv=320).
// SiLU is z * sigmoid(z) with sigmoid(z) = (1 + tanh(z/2)) / 2 (one tanh.approx).
// ------------------------------------------------------------------------------------
constexpr int kGuessRows = 128, kGuessThreads = 256, kGFeatStride = 16;
constexpr size_t kGW2 = 0, kGA1 = kGW2 + 4 * 256 * 128, kGF = kGA1 + 4 * 128 * 128;
constexpr size_t kGT2 = kGF + (size_t)kGuessRows * kGFeatStride * 4, kGB1 = kGT2 + (size_t)kGuessRows * 8;
constexpr size_t kGB2 = kGB1 + kHid * 4, kGW3 = kGB2 + kHid * 4;
constexpr size_t kGYP = kGW3 + kHid * 4, kGBAR = kGYP + kGuessRows * 4;
constexpr size_t kGuessSmem = 1024 + kGBAR + 64;
// instruction descriptor, kind::f16: D f32 (bit 4), A and B f16 (format 0 at bits 7-9 and
// 10-12), both K-major, N = 256 (N >> 3 at bits 17-22), M = 128 (M >> 4 at bits 24-28)
constexpr uint32_t kGuessIdesc = (1u << 4) | ((uint32_t)(256 >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);

__device__ __forceinline__ float silu_tanh(float z) {
  float t;
  asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(0.5f * z));
  return z * fmaf(0.5f, t, 0.5f);
}

// diagonal integral tables the features read: vv[a][b] = <ab|ab>, oo[i][j] = <ij|ij>,
// ov1[i][a] = <ia|ia>, ov2[i][a] = <ii|aa> (= <ia|ai>), in FP32
__global__ void guess_diag_kernel(int no, int nv, const double* Voovv, const double* Voooo, const double* Vovov,
                                  const double* Vvvvv, float* vv, float* oo, float* ov1, float* ov2) {
  const int64_t o = no, v = nv;
  const int64_t tot = v * v + o * o + 2 * o * v;
  for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < tot; x += (int64_t)gridDim.x * blockDim.x) {
    if (x < v * v) {
      const int64_t a = x / v, b = x % v;
      vv[x] = (float)Vvvvv[((a * v + b) * v + a) * v + b];
    } else if (x < v * v + o * o) {
      const int64_t y = x - v * v, i = y / o, j = y % o;
      oo[y] = (float)Voooo[((i * o + j) * o + i) * o + j];
    } else if (x < v * v + o * o + o * v) {
      const int64_t y = x - v * v - o * o, i = y / v, a = y % v;
      ov1[y] = (float)Vovov[((i * v + a) * o + i) * v + a];
    } else {
      const int64_t y = x - v * v - o * o - o * v, i = y / v, a = y % v;
      ov2[y] = (float)Voovv[((i * o + i) * v + a) * v + a];
    }
  }
}

__global__ void __launch_bounds__(kGuessThreads, 1)
    guess_tc_kernel(int no, int nv, int64_t n, const double* __restrict__ Voovv, const double* __restrict__ eps,
                    const float* __restrict__ vv, const float* __restrict__ oo, const float* __restrict__ ov1,
                    const float* __restrict__ ov2, const __half* __restrict__ wh, const float* __restrict__ w,
                    int64_t oW1, int64_t oW2, int64_t ow3, int64_t ob1, int64_t ob2, int64_t ob3,
                    double* __restrict__ t2out, int* err) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  float* Fs = reinterpret_cast<float*>(smem + kGF);
  double* T2m = reinterpret_cast<double*>(smem + kGT2);
  float* b1s = reinterpret_cast<float*>(smem + kGB1);
  float* b2s = reinterpret_cast<float*>(smem + kGB2);
  float* w3s = reinterpret_cast<float*>(smem + kGW3);
  float* yp = reinterpret_cast<float*>(smem + kGYP);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + kGBAR);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + kGBAR + 8);
  int* stop = reinterpret_cast<int*>(smem + kGBAR + 16);
  const int tid = threadIdx.x, warp = tid / 32, lane = tid % 32;

  // weights: W2^T into the swizzled B operand, 8 k-consecutive FP16 values per 16-byte chunk
  for (int ch = tid; ch < kHid * (kHid / 8); ch += kGuessThreads) {
    const int nn = ch / (kHid / 8), c8 = ch % (kHid / 8), kb = c8 / 8, c = c8 % 8;
    __align__(16) __half hv[8];
#pragma unroll
    for (int e = 0; e < 8; e++) hv[e] = wh[oW2 + (int64_t)(c8 * 8 + e) * kHid + nn];
    *reinterpret_cast<uint4*>(smem + kGW2 + (size_t)kb * 256 * 128 + (size_t)nn * 128 + ((c ^ (nn & 7)) << 4)) =
        *reinterpret_cast<const uint4*>(hv);
  }
  // this thread's first-layer weights, held for the whole kernel
  const int u0 = 8 * lane, rg = warp;  // hidden units u0 .. u0+7, tile rows 16 rg .. 16 rg + 15
  float w1r[kFeat][8], b1r[8];
#pragma unroll
  for (int k = 0; k < kFeat; k++)
#pragma unroll
    for (int e = 0; e < 8; e++) w1r[k][e] = __half2float(wh[oW1 + (int64_t)k * kHid + u0 + e]);
#pragma unroll
  for (int e = 0; e < 8; e++) b1r[e] = w[ob1 + u0 + e];
  for (int x = tid; x < kHid; x += kGuessThreads) {
    b1s[x] = w[ob1 + x];
    b2s[x] = w[ob2 + x];
    w3s[x] = __half2float(wh[ow3 + x]);
  }
  const float b3 = w[ob3];
  if (tid == 0) {
    tc::mbar_init(bar, 1);
    *stop = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc::smem_u32(tslot)),
                 "r"(256));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc::fence_proxy_async();
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = *tslot;
  const int lr = tid & (kGuessRows - 1), half = tid / kGuessRows;  // row of the tile, hidden-unit half
  const int q = warp & 3;                                          // TMEM lane quarter (rows q*32..q*32+31)
  const int64_t ntiles = (n + kGuessRows - 1) / kGuessRows;
  const int64_t o = no, v = nv;
  uint32_t phase = 0;
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t x = tile * kGuessRows + lr;
    const bool valid = x < n;
    if (half == 0) {  // the features and MP2 amplitude of row lr
    float f[kFeat];
    double t2mp2 = 0.0;
    if (valid) {
      const int b = (int)(x % v), a = (int)((x / v) % v), j = (int)((x / (v * v)) % o), i = (int)(x / (v * v * o));
      const double D = ((eps[i] + eps[j]) - eps[no + a]) - eps[no + b];
      const double vij = Voovv[x];
      t2mp2 = vij / D;
      const float rD = 1.0f / (float)D, S = (float)kScale;
      const float vx = (float)Voovv[((int64_t)(i * o + j) * v + b) * v + a];
      const float ei = (float)eps[i], ej = (float)eps[j], ea = (float)eps[no + a], eb = (float)eps[no + b];
      f[0] = S * (float)vij * rD;
      f[1] = S * vx * rD;
      f[2] = S * (float)vij;
      f[3] = -rD;
      f[4] = 0.5f * (ei + ej);
      f[5] = 0.5f * (ea + eb);
      f[6] = i == j ? 1.f : 0.f;
      f[7] = a == b ? 1.f : 0.f;
      f[8] = S * vv[(int64_t)a * v + b];
      f[9] = S * oo[(int64_t)i * o + j];
      f[10] = S * (ov1[(int64_t)i * v + a] + ov1[(int64_t)j * v + b]);
      f[11] = S * (ov2[(int64_t)i * v + a] + ov2[(int64_t)j * v + b]);
      f[12] = 0.5f * fabsf(ei - ej);
      f[13] = 0.5f * fabsf(ea - eb);
      f[14] = 0.25f * (ei - ej) * (ea - eb);
    } else {
#pragma unroll
      for (int k = 0; k < kFeat; k++) f[k] = 0.f;
    }
#pragma unroll
    for (int k = 0; k < kFeat; k++) Fs[lr * kGFeatStride + k] = f[k];
    Fs[lr * kGFeatStride + kFeat] = valid ? 1.f : 0.f;
    T2m[lr] = t2mp2;
    }
    __syncthreads();
    // layer 1: units u0 .. u0+7 of rows 16 rg .. 16 rg + 15, SiLU, FP16, into the A operand
    // (unit u is K index u of the second layer: K block u / 64, chunk (u % 64) / 8)
    {
      const int kb = u0 / 64, c = (u0 % 64) / 8;
#pragma unroll 2
      for (int rr = 0; rr < 16; rr++) {
        const int row = 16 * rg + rr;
        const float* fr = Fs + row * kGFeatStride;
        float z[8];
#pragma unroll
        for (int e = 0; e < 8; e++) z[e] = b1r[e];
#pragma unroll
        for (int k = 0; k < kFeat; k++) {
          const float fk = fr[k];
#pragma unroll
          for (int e = 0; e < 8; e++) z[e] = fmaf(fk, w1r[k][e], z[e]);
        }
        const bool rv = fr[kFeat] != 0.f;
        __align__(16) __half hv[8];
#pragma unroll
        for (int e = 0; e < 8; e++) hv[e] = __float2half_rn(rv ? silu_tanh(z[e]) : 0.f);
        *reinterpret_cast<uint4*>(smem + kGA1 + (size_t)kb * 128 * 128 + (size_t)row * 128 +
                                  ((c ^ (row & 7)) << 4)) = *reinterpret_cast<const uint4*>(hv);
      }
    }
    tc::fence_proxy_async();
    tc::fence_before();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after();
#pragma unroll
      for (int kb = 0; kb < 4; kb++) {
        const uint64_t ad = tc::sdesc(smem + kGA1 + (size_t)kb * 128 * 128);
        const uint64_t bd = tc::sdesc(smem + kGW2 + (size_t)kb * 256 * 128);
#pragma unroll
        for (int k = 0; k < 4; k++)  // +32 bytes along K per 16-element step
          tc::mma_i(tmem, ad + (uint64_t)(k * 2), bd + (uint64_t)(k * 2), kGuessIdesc, (kb | k) != 0);
      }
      tc::mma_commit(bar);
      if (!tc::mbar_wait(bar, phase, err)) *stop = 1;
    }
    __syncthreads();
    if (*stop) break;
    phase ^= 1u;
    tc::fence_after();
    // output layer: warp w reads TMEM lanes (w % 4) * 32.. (its rows) and columns of its half
    float part = 0.f;
#pragma unroll 1
    for (int ch = 0; ch < 4; ch++) {
      uint32_t r[32];
      tc::tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(half * 128 + ch * 32), r);
#pragma unroll
      for (int jj = 0; jj < 32; jj++) {
        const int u = half * 128 + ch * 32 + jj;
        part = fmaf(silu_tanh(__uint_as_float(r[jj]) + b2s[u]), w3s[u], part);
      }
    }
    if (half == 1) yp[lr] = part;
    tc::fence_before();
    __syncthreads();
    if (half == 0 && valid) t2out[x] = T2m[lr] + (double)(part + yp[lr] + b3) / kTarget;
  }
  if (tid == 0 && *stop) tc::mbar_wait_deadline(bar, phase);  // no MMA in flight when TMEM is released
  tc::fence_before();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(256));
  }
}

}  // namespace mlp
}  // namespace ucc

using namespace ucc;
using namespace ucc::mlp;

struct ucc_mlp {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string last_error;
  // FP32 masters, Adam moments, FP16 copies: W1 [8][256], b1 [256], W2 [256][256], b2, w3 [256], b3 [1]
  int64_t nparam = 0;
  float* w = nullptr;  // all parameters, contiguous
  float* g = nullptr;
  float* m = nullptr;
  float* v = nullptr;
  __half* wh = nullptr;
  int64_t adam_t = 0;
  int64_t cap = 0;   // activation buffers sized for this many rows
  int64_t ycap = 0;  // output / output-gradient buffers
  float *Z1 = nullptr, *A1 = nullptr, *Z2 = nullptr, *A2 = nullptr, *y = nullptr, *dy = nullptr, *loss = nullptr;
  int64_t oW1() const { return 0; }
  int64_t ob1() const { return (int64_t)kFeat * kHid; }
  int64_t oW2() const { return ob1() + kHid; }
  int64_t ob2() const { return oW2() + (int64_t)kHid * kHid; }
  int64_t ow3() const { return ob2() + kHid; }
  int64_t ob3() const { return ow3() + kHid; }
  ~ucc_mlp() {
    for (void* p : {(void*)w, (void*)g, (void*)m, (void*)v, (void*)wh, (void*)Z1, (void*)A1, (void*)Z2, (void*)A2,
                    (void*)y, (void*)dy, (void*)loss})
      if (p) cudaFree(p);
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace {
template <typename F>
ucc_status mguard(ucc_mlp* n, F&& f) {
  if (!n) return UCC_BAD_ARGS;
  n->last_error.clear();
  try {
    UCC_CUDA(cudaSetDevice(n->device));
    f(*n);
    return UCC_OK;
  } catch (const Error& e) {
    n->last_error = e.what();
    return e.status;
  } catch (const std::exception& e) {
    n->last_error = e.what();
    return UCC_CUDA_ERROR;
  }
}

constexpr int64_t kChunk = 1 << 20;  // rows per forward pass (activation buffers)

void ensure_rows(ucc_mlp& n, int64_t rows) {
  const int64_t act = std::min(rows, kChunk);
  if (act > n.cap) {
    for (float** p : {&n.Z1, &n.A1, &n.Z2, &n.A2}) {
      if (*p) cudaFree(*p);
      UCC_CUDA(cudaMalloc(p, sizeof(float) * act * kHid));
    }
    n.cap = act;
  }
  if (rows > n.ycap) {
    for (float** p : {&n.y, &n.dy}) {
      if (*p) cudaFree(*p);
      UCC_CUDA(cudaMalloc(p, sizeof(float) * rows));
    }
    n.ycap = rows;
  }
}

template <typename TB>
void gemm(ucc_mlp& n, int M, int N, int K, const float* A, int64_t sAm, int64_t sAk, const TB* B, int64_t sBk,
          int64_t sBn, float* C, int64_t ldc, bool acc) {
  dim3 grid((N + 63) / 64, (M + 63) / 64);
  gemm_f32<TB><<<grid, 256, 0, n.stream>>>(M, N, K, A, sAm, sAk, B, sBk, sBn, C, ldc, acc ? 1 : 0);
  count_kernel_launch();
  UCC_CUDA(cudaGetLastError());
}

// forward pass for rows X[rows][8] -> n.y (chunks of kChunk rows through the activations)
void forward(ucc_mlp& n, const float* X, int64_t rows) {
  const __half* W1 = n.wh + n.oW1();
  const __half* W2 = n.wh + n.oW2();
  const __half* w3 = n.wh + n.ow3();
  for (int64_t r0 = 0; r0 < rows; r0 += kChunk) {
    const int64_t len = std::min(kChunk, rows - r0);
    const float* Xc = X + r0 * kFeat;
    float* yc = n.y + r0;
    gemm(n, (int)len, kHid, kFeat, Xc, kFeat, 1, W1, kHid, 1, n.Z1, kHid, false);
    bias_act<<<grid1(len * kHid), 256, 0, n.stream>>>(len, kHid, n.Z1, n.w + n.ob1(), n.A1);
    gemm(n, (int)len, kHid, kHid, n.A1, kHid, 1, W2, kHid, 1, n.Z2, kHid, false);
    bias_act<<<grid1(len * kHid), 256, 0, n.stream>>>(len, kHid, n.Z2, n.w + n.ob2(), n.A2);
    gemm(n, (int)len, 1, kHid, n.A2, kHid, 1, w3, 1, 1, yc, 1, false);
    add_scalar<<<grid1(len), 256, 0, n.stream>>>(len, yc, n.w + n.ob3());
    for (int k = 0; k < 3; k++) count_kernel_launch();
    UCC_CUDA(cudaGetLastError());
  }
}

// loss and gradients (into n.g) for rows X, targets t; returns mean squared error
float backward(ucc_mlp& n, const float* X, const float* t, int64_t rows) {
  UCC_REQUIRE(rows <= kChunk, UCC_BAD_ARGS, "training batch larger than the activation chunk");
  forward(n, X, rows);
  UCC_CUDA(cudaMemsetAsync(n.loss, 0, sizeof(float), n.stream));
  mse_grad<<<grid1(rows), 256, 0, n.stream>>>(rows, n.y, t, n.dy, n.loss);
  float* g = n.g;
  // w3, b3
  gemm(n, kHid, 1, (int)rows, n.A2, 1, kHid, n.dy, 1, 1, g + n.ow3(), 1, false);
  col_sum<<<1, 32, 0, n.stream>>>(rows, 1, n.dy, g + n.ob3());
  // dA2 = dy w3^T -> dZ2 (reuse A2 as dZ2 after its use above)
  gemm(n, (int)rows, kHid, 1, n.dy, 1, 1, n.wh + n.ow3(), 1, 1, n.A2, kHid, false);
  act_grad<<<grid1(rows * kHid), 256, 0, n.stream>>>(rows * kHid, n.Z2, n.A2);
  // W2, b2
  gemm(n, kHid, kHid, (int)rows, n.A1, 1, kHid, n.A2, kHid, 1, g + n.oW2(), kHid, false);
  col_sum<<<(kHid + 127) / 128, 128, 0, n.stream>>>(rows, kHid, n.A2, g + n.ob2());
  // dA1 = dZ2 W2^T -> dZ1 (into A1)
  gemm(n, (int)rows, kHid, kHid, n.A2, kHid, 1, n.wh + n.oW2(), 1, kHid, n.A1, kHid, false);
  act_grad<<<grid1(rows * kHid), 256, 0, n.stream>>>(rows * kHid, n.Z1, n.A1);
  // W1, b1
  gemm(n, kFeat, kHid, (int)rows, X, 1, kFeat, n.A1, kHid, 1, g + n.oW1(), kHid, false);
  col_sum<<<(kHid + 127) / 128, 128, 0, n.stream>>>(rows, kHid, n.A1, g + n.ob1());
  for (int k = 0; k < 6; k++) count_kernel_launch();
  UCC_CUDA(cudaGetLastError());
  float loss = 0.f;
  UCC_CUDA(cudaMemcpyAsync(&loss, n.loss, sizeof(float), cudaMemcpyDeviceToHost, n.stream));
  UCC_CUDA(cudaStreamSynchronize(n.stream));
  return loss;
}
}  // namespace

extern "C" {

ucc_status ucc_mlp_create(ucc_mlp** out, int device, uint64_t seed) {
  if (!out) return UCC_BAD_ARGS;
  *out = nullptr;
  int nd = 0;
  if (cudaGetDeviceCount(&nd) != cudaSuccess || device < 0 || device >= nd) return UCC_CUDA_ERROR;
  ucc_mlp* n = new (std::nothrow) ucc_mlp;
  if (!n) return UCC_OUT_OF_MEMORY;
  n->device = device;
  ucc_status st = mguard(n, [&](ucc_mlp& m) {
    UCC_CUDA(cudaStreamCreateWithFlags(&m.stream, cudaStreamNonBlocking));
    m.nparam = m.ob3() + 1;
    UCC_CUDA(cudaMalloc(&m.w, sizeof(float) * m.nparam));
    UCC_CUDA(cudaMalloc(&m.g, sizeof(float) * m.nparam));
    UCC_CUDA(cudaMalloc(&m.m, sizeof(float) * m.nparam));
    UCC_CUDA(cudaMalloc(&m.v, sizeof(float) * m.nparam));
    UCC_CUDA(cudaMalloc(&m.wh, sizeof(__half) * m.nparam));
    UCC_CUDA(cudaMalloc(&m.loss, sizeof(float)));
    UCC_CUDA(cudaMemset(m.m, 0, sizeof(float) * m.nparam));
    UCC_CUDA(cudaMemset(m.v, 0, sizeof(float) * m.nparam));
    // He-style initialisation, deterministic in the seed
    std::vector<float> h(m.nparam, 0.f);
    std::mt19937_64 rng(seed);
    std::normal_distribution<float> nd1(0.f, std::sqrt(2.f / kFeat)), nd2(0.f, std::sqrt(2.f / kHid));
    for (int64_t k = m.oW1(); k < m.ob1(); k++) h[k] = nd1(rng);
    for (int64_t k = m.oW2(); k < m.ob2(); k++) h[k] = nd2(rng);
    for (int64_t k = m.ow3(); k < m.ob3(); k++) h[k] = 0.1f * nd2(rng);
    UCC_CUDA(cudaMemcpy(m.w, h.data(), sizeof(float) * m.nparam, cudaMemcpyHostToDevice));
    to_half<<<grid1(m.nparam), 256, 0, m.stream>>>(m.nparam, m.w, m.wh);
    count_kernel_launch();
    UCC_CUDA(cudaStreamSynchronize(m.stream));
  });
  if (st != UCC_OK) {
    delete n;
    return st;
  }
  *out = n;
  return UCC_OK;
}

ucc_status ucc_mlp_destroy(ucc_mlp* n) {
  if (!n) return UCC_BAD_ARGS;
  cudaSetDevice(n->device);
  delete n;
  return UCC_OK;
}

const char* ucc_mlp_last_error(ucc_mlp* n) { return n ? n->last_error.c_str() : "null network"; }

int ucc_mlp_num_params(void) {
  return kFeat * kHid + kHid + kHid * kHid + kHid + kHid + 1;
}

ucc_status ucc_mlp_get_params(ucc_mlp* n, float* out, size_t count) {
  return mguard(n, [&](ucc_mlp& m) {
    UCC_REQUIRE(out && (int64_t)count == m.nparam, UCC_BAD_ARGS, "parameter count mismatch");
    UCC_CUDA(cudaMemcpy(out, m.w, sizeof(float) * count, cudaMemcpyDeviceToHost));
  });
}

ucc_status ucc_mlp_set_params(ucc_mlp* n, const float* in, size_t count) {
  return mguard(n, [&](ucc_mlp& m) {
    UCC_REQUIRE(in && (int64_t)count == m.nparam, UCC_BAD_ARGS, "parameter count mismatch");
    UCC_CUDA(cudaMemcpy(m.w, in, sizeof(float) * count, cudaMemcpyHostToDevice));
    to_half<<<grid1(m.nparam), 256, 0, m.stream>>>(m.nparam, m.w, m.wh);
    count_kernel_launch();
    UCC_CUDA(cudaStreamSynchronize(m.stream));
  });
}

ucc_status ucc_mlp_predict(ucc_mlp* n, const float* X, int64_t rows, float* y) {
  return mguard(n, [&](ucc_mlp& m) {
    UCC_REQUIRE(X && y && rows >= 1, UCC_BAD_ARGS, "bad arguments");
    ensure_rows(m, rows);
    float* dX = nullptr;
    UCC_CUDA(cudaMallocAsync(&dX, sizeof(float) * rows * kFeat, m.stream));
    UCC_CUDA(cudaMemcpyAsync(dX, X, sizeof(float) * rows * kFeat, cudaMemcpyHostToDevice, m.stream));
    forward(m, dX, rows);
    UCC_CUDA(cudaMemcpyAsync(y, m.y, sizeof(float) * rows, cudaMemcpyDeviceToHost, m.stream));
    UCC_CUDA(cudaFreeAsync(dX, m.stream));
    UCC_CUDA(cudaStreamSynchronize(m.stream));
  });
}

ucc_status ucc_mlp_loss_grad(ucc_mlp* n, const float* X, const float* t, int64_t rows, float* loss, float* grad,
                             size_t count) {
  return mguard(n, [&](ucc_mlp& m) {
    UCC_REQUIRE(X && t && loss && rows >= 1, UCC_BAD_ARGS, "bad arguments");
    UCC_REQUIRE(!grad || (int64_t)count == m.nparam, UCC_BAD_ARGS, "gradient count mismatch");
    ensure_rows(m, rows);
    float *dX = nullptr, *dt = nullptr;
    UCC_CUDA(cudaMallocAsync(&dX, sizeof(float) * rows * kFeat, m.stream));
    UCC_CUDA(cudaMallocAsync(&dt, sizeof(float) * rows, m.stream));
    UCC_CUDA(cudaMemcpyAsync(dX, X, sizeof(float) * rows * kFeat, cudaMemcpyHostToDevice, m.stream));
    UCC_CUDA(cudaMemcpyAsync(dt, t, sizeof(float) * rows, cudaMemcpyHostToDevice, m.stream));
    *loss = backward(m, dX, dt, rows);
    if (grad) UCC_CUDA(cudaMemcpy(grad, m.g, sizeof(float) * count, cudaMemcpyDeviceToHost));
    UCC_CUDA(cudaFreeAsync(dX, m.stream));
    UCC_CUDA(cudaFreeAsync(dt, m.stream));
    UCC_CUDA(cudaStreamSynchronize(m.stream));
  });
}

ucc_status ucc_mlp_train(ucc_mlp* n, const float* X, const float* t, int64_t rows, int epochs, int batch, float lr,
                         uint64_t seed, float* final_loss) {
  return mguard(n, [&](ucc_mlp& m) {
    UCC_REQUIRE(X && t && rows >= 1 && epochs >= 1 && batch >= 1 && lr > 0, UCC_BAD_ARGS, "bad arguments");
    const int64_t nb = std::min<int64_t>(batch, rows);
    ensure_rows(m, nb);
    float *dX = nullptr, *dt = nullptr, *Xb = nullptr, *tb = nullptr;
    int64_t* didx = nullptr;
    UCC_CUDA(cudaMallocAsync(&dX, sizeof(float) * rows * kFeat, m.stream));
    UCC_CUDA(cudaMallocAsync(&dt, sizeof(float) * rows, m.stream));
    UCC_CUDA(cudaMallocAsync(&Xb, sizeof(float) * nb * kFeat, m.stream));
    UCC_CUDA(cudaMallocAsync(&tb, sizeof(float) * nb, m.stream));
    UCC_CUDA(cudaMallocAsync(&didx, sizeof(int64_t) * rows, m.stream));
    UCC_CUDA(cudaMemcpyAsync(dX, X, sizeof(float) * rows * kFeat, cudaMemcpyHostToDevice, m.stream));
    UCC_CUDA(cudaMemcpyAsync(dt, t, sizeof(float) * rows, cudaMemcpyHostToDevice, m.stream));
    std::vector<int64_t> idx(rows);
    for (int64_t k = 0; k < rows; k++) idx[k] = k;
    std::mt19937_64 rng(seed);
    const float b1 = 0.9f, b2 = 0.999f;
    double epoch_loss = 0.0;
    for (int ep = 0; ep < epochs; ep++) {
      std::shuffle(idx.begin(), idx.end(), rng);
      UCC_CUDA(cudaMemcpyAsync(didx, idx.data(), sizeof(int64_t) * rows, cudaMemcpyHostToDevice, m.stream));
      UCC_CUDA(cudaStreamSynchronize(m.stream));
      epoch_loss = 0.0;
      int64_t steps = 0;
      for (int64_t s = 0; s + nb <= rows; s += nb, steps++) {
        gather_rows<<<grid1(nb * kFeat), 256, 0, m.stream>>>(nb, kFeat, didx + s, dX, dt, Xb, tb);
        count_kernel_launch();
        epoch_loss += backward(m, Xb, tb, nb);
        m.adam_t++;
        const float c1 = 1.f - std::pow(b1, (float)m.adam_t), c2 = 1.f - std::pow(b2, (float)m.adam_t);
        adam<<<grid1(m.nparam), 256, 0, m.stream>>>(m.nparam, m.w, m.g, m.m, m.v, m.wh, lr, b1, b2, c1, c2);
        count_kernel_launch();
      }
      if (steps) epoch_loss /= (double)steps;
    }
    UCC_CUDA(cudaStreamSynchronize(m.stream));
    for (void* p : {(void*)dX, (void*)dt, (void*)Xb, (void*)tb, (void*)didx}) UCC_CUDA(cudaFreeAsync(p, m.stream));
    UCC_CUDA(cudaStreamSynchronize(m.stream));
    if (final_loss) *final_loss = (float)epoch_loss;
  });
}

// features / targets of the Hamiltonian loaded in ctx (targets need converged CCSD)
ucc_status ucc_mlp_features(ucc_ctx* ctx, float* out, size_t rows, int with_targets, float* targets) {
  if (!ctx || !out) return UCC_BAD_ARGS;
  Ctx& c = ctx_of(ctx);
  try {
    UCC_CUDA(cudaSetDevice(c.device));
    mlp_features(c, out, rows, with_targets ? targets : nullptr, with_targets != 0);
    return UCC_OK;
  } catch (const Error& e) {
    c.last_error = e.what();
    return e.status;
  }
}

// next ucc_ccsd starts from t1 = f_ia/D1 and t2 = t2_mp2 + network prediction
ucc_status ucc_mlp_guess(ucc_ctx* ctx, ucc_mlp* net) {
  if (!ctx || !net) return UCC_BAD_ARGS;
  Ctx& c = ctx_of(ctx);
  try {
    UCC_CUDA(cudaSetDevice(c.device));
    mlp_guess(c, net);
    return UCC_OK;
  } catch (const Error& e) {
    c.last_error = e.what();
    return e.status;
  }
}

}  // extern "C"

namespace ucc {
void mlp_features(Ctx& c, float* out, size_t rows, float* targets, bool with_targets) {
  UCC_REQUIRE(out, UCC_BAD_ARGS, "null argument");
  UCC_REQUIRE(c.loaded, UCC_BAD_STATE, "no Hamiltonian loaded");
  const int64_t n = (int64_t)c.no * c.no * c.nv * c.nv;
  UCC_REQUIRE((int64_t)rows == n, UCC_BAD_ARGS, "rows must be no*no*nv*nv");
  Scratch X(c, sizeof(float) * n * kFeat);
  features_kernel<<<grid1(n), 256, 0, c.stream>>>(c.no, c.nv, c.get("Voovv").p, c.get("Voooo").p, c.get("Vovov").p,
                                                  c.get("Vvvvv").p, c.get("eps").p, static_cast<float*>(X.p));
  count_kernel_launch();
  UCC_CUDA(cudaMemcpyAsync(out, X.p, sizeof(float) * n * kFeat, cudaMemcpyDeviceToHost, c.stream));
  if (with_targets) {
    UCC_REQUIRE(targets && c.have_ccsd, UCC_BAD_STATE, "targets need converged CCSD amplitudes");
    Scratch y(c, sizeof(float) * n);
    targets_kernel<<<grid1(n), 256, 0, c.stream>>>(c.no, c.nv, c.get("Voovv").p, c.get("eps").p,
                                                   amp2(c, c.get("T").p).p, static_cast<float*>(y.p));
    count_kernel_launch();
    UCC_CUDA(cudaMemcpyAsync(targets, y.p, sizeof(float) * n, cudaMemcpyDeviceToHost, c.stream));
  }
  UCC_CUDA(cudaStreamSynchronize(c.stream));
}

// the network's T2 guess into the context's T_guess (t1 = f_ia / D1): one fused
// tensor-core pass over the doubles elements on the context's stream; the weights are
// read on that stream after the network's own stream has finished updating them
void mlp_guess(Ctx& c, ucc_mlp* net) {
  UCC_REQUIRE(c.loaded, UCC_BAD_STATE, "no Hamiltonian loaded");
  UCC_REQUIRE(net->device == c.device, UCC_BAD_ARGS, "network and context on different devices");
  const int no = c.no, nv = c.nv;
  const int64_t n = (int64_t)no * no * nv * nv, n1 = (int64_t)no * nv;
  UCC_CUDA(cudaStreamSynchronize(net->stream));
  if (!c.has("T_guess")) c.alloc("T_guess", {n1 + n}, true);
  double* g = c.get("T_guess").p;
  // t1 part: f_ia / (f_ii - f_aa) on the host (small)
  std::vector<double> t1(n1);
  const int nact = no + nv;
  for (int i = 0; i < no; i++)
    for (int a = 0; a < nv; a++)
      t1[(size_t)i * nv + a] = c.fock[(size_t)i * nact + no + a] / (c.eps[i] - c.eps[no + a]);
  UCC_CUDA(cudaMemcpyAsync(g, t1.data(), sizeof(double) * n1, cudaMemcpyHostToDevice, c.stream));
  const int64_t ndiag = (int64_t)nv * nv + (int64_t)no * no + 2LL * no * nv;
  Scratch diag(c, sizeof(float) * ndiag);
  float* vv = static_cast<float*>(diag.p);
  float* oo = vv + (int64_t)nv * nv;
  float* ov1 = oo + (int64_t)no * no;
  float* ov2 = ov1 + (int64_t)no * nv;
  guess_diag_kernel<<<grid1(ndiag), 256, 0, c.stream>>>(no, nv, c.get("Voovv").p, c.get("Voooo").p,
                                                        c.get("Vovov").p, c.get("Vvvvv").p, vv, oo, ov1, ov2);
  count_kernel_launch();
  UCC_CUDA(cudaFuncSetAttribute(guess_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGuessSmem));
  int sms = 0;
  UCC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c.device));
  const int64_t ntiles = (n + kGuessRows - 1) / kGuessRows;
  Scratch errflag(c, sizeof(int));
  UCC_CUDA(cudaMemsetAsync(errflag.p, 0, sizeof(int), c.stream));
  Timer timer(c.stream);
  timer.start();
  guess_tc_kernel<<<(unsigned)std::min<int64_t>(ntiles, sms), kGuessThreads, kGuessSmem, c.stream>>>(
      no, nv, n, c.get("Voovv").p, c.get("eps").p, vv, oo, ov1, ov2, net->wh, net->w, net->oW1(), net->oW2(),
      net->ow3(), net->ob1(), net->ob2(), net->ob3(), g + n1, static_cast<int*>(errflag.p));
  count_kernel_launch();
  UCC_CUDA(cudaGetLastError());
  int herr = 0;
  UCC_CUDA(cudaMemcpyAsync(&herr, errflag.p, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
  c.stats.guess_ms += timer.stop_ms();
  UCC_REQUIRE(!herr, UCC_DEVICE_TIMEOUT, "guess network: a tensor-core wait timed out");
}
}  // namespace ucc
