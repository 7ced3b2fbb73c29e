// Batched CCSD over many small, uneven-size Hamiltonians (one graph launch per sweep).
//
// Each member keeps its own context (integral blocks, amplitudes, intermediates).  The
// residual build of ccwfn.cc:311-539 is recorded once per member through the launcher
// hooks (core.h: Recorder) instead of being launched: every member yields the same
// sequence of GEMM / permute / fill operations with its own sizes and pointers, its
// scratch placed in a per-member arena.  Operation k of all members then becomes ONE
// grouped launch:
//
//   grouped_gemm<BM,BN>  -- FP64 DFMA tiles of every member's GEMM k, a flat tile space
//                           (prefix sums over members), the tile shape chosen per
//                           operation by timing the candidates on the real operands;
//   grouped_perm         -- every member's permute / axpby / fill k, in 2048-element chunks.
//
// The rest of a sweep (Jacobi update, residual norm, convergence mask, DIIS with its
// B-matrix rows, subspace solve and extrapolation, tau/ttau, energy) is written directly
// as grouped kernels over (member, chunk).  The whole solve is ONE graph launch: a CUDA
// graph whose while-node repeats the captured sweep on the device; the sweep's last
// kernel sets the loop condition from the count of members still iterating, so the host
// neither launches nor waits per sweep.  A member whose ||R|| drops below R_CONVERGENCE is
// masked out of every later kernel, so it ends exactly where the one-member solver would
// (ccwfn.cc:188-258).  The loop is bounded twice on the device: by MAXITER (members stop
// iterating) and by a time limit on the globaltimer, after which the loop ends and the
// call reports UCC_DEVICE_TIMEOUT with the batch still usable.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "cc.h"
#include "engine.h"
#include "pert.h"

namespace ucc {
void count_kernel_launch();
void mlp_guess(Ctx& c, ucc_mlp* net);  // mlp.cu
void mlp_features(Ctx& c, float* out, size_t rows, float* targets, bool with_targets);

namespace batch {

constexpr int kDiis = 8;
constexpr int64_t kChunk = 2048;  // elements per work item of the elementwise kernels

struct GemmDesc {
  int64_t M, N, K, sAm, sAk, sBk, sBn, sCm, sCn;
  const double* A;
  const double* B;
  double* C;
  double alpha, beta;
  int prob;
};

struct PermDesc {
  int rank, prob, fill;
  int64_t total;
  int64_t d[kMaxRank], si[kMaxRank], so[kMaxRank];
  const double* in;
  double* out;
  double alpha, beta;
};

struct Member {  // device view of one member for the sweep kernels
  int no, nv;
  int64_t n1, np;
  const double* eps;
  double* T;
  double* Told;
  const double* R;
  double* tau;
  double* ttau;
  const double* Loovv;
  double* err;  // [kDiis][np]
  double* vec;  // [kDiis][np]
  double fock_last;  // f[no-1][nact-1] (one-electron energy term, ccwfn.cc:270-273)
};

struct SweepState {  // device-side bookkeeping shared by all members
  int iter;
  int count;   // DIIS vectors held after this sweep's add
  int slot;    // slot written by this sweep's add
  int nadded;
  int active_count;
  double r_conv;
  int maxiter;
  unsigned long long t0;        // globaltimer at the start of the solve
  unsigned long long limit_ns;  // device time limit of the sweep loop
  int timed_out;                // the loop ended on the time limit with members still iterating
};

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// first node of the solve graph: the clock of the time limit
__global__ void solve_start_kernel(SweepState* st) {
  st->t0 = global_ns();
  st->timed_out = 0;
}

// last node of every sweep: repeat while members are iterating and time is left
__global__ void loop_control_kernel(cudaGraphConditionalHandle loop, SweepState* st) {
  unsigned int again = st->active_count > 0 ? 1u : 0u;
  if (again && global_ns() - st->t0 > st->limit_ns) {
    st->timed_out = 1;
    again = 0u;
  }
  cudaGraphSetConditional(loop, again);
}

__device__ __forceinline__ int find_item(const int64_t* __restrict__ prefix, int n, int64_t t) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (prefix[mid] <= t)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// ---------------------------------------------------------------------------------------
// Grouped GEMM: 16x16 threads, each (BM/16) x (BN/16) outputs, K in steps of 16 through
// shared memory; operand loads follow whichever index is contiguous.
// ---------------------------------------------------------------------------------------
template <int BM_, int BN_>
__global__ void __launch_bounds__(256) grouped_gemm(const GemmDesc* __restrict__ desc,
                                                    const int64_t* __restrict__ prefix, int nd, int64_t total,
                                                    const int* __restrict__ active) {
  constexpr int TM = BM_ / 16, TN = BN_ / 16, BK = 16;
  __shared__ double As[BK][BM_ + 1];
  __shared__ double Bs[BK][BN_ + 1];
  const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
  for (int64_t t = blockIdx.x; t < total; t += gridDim.x) {
    const int di = find_item(prefix, nd, t);
    const GemmDesc g = desc[di];
    if (!active[g.prob]) continue;
    const int64_t local = t - prefix[di];
    const int64_t ntn = (g.N + BN_ - 1) / BN_;
    const int64_t m0 = local / ntn * BM_, n0 = local % ntn * BN_;
    double acc[TM][TN];
#pragma unroll
    for (int i = 0; i < TM; i++)
#pragma unroll
      for (int j = 0; j < TN; j++) acc[i][j] = 0.0;
    const bool a_kfast = g.sAk == 1, b_nfast = g.sBn == 1;
    for (int64_t k0 = 0; k0 < g.K; k0 += BK) {
      for (int e = tid; e < BM_ * BK; e += 256) {
        const int mm = a_kfast ? e / BK : e % BM_, kk = a_kfast ? e % BK : e / BM_;
        const int64_t m = m0 + mm, k = k0 + kk;
        As[kk][mm] = (m < g.M && k < g.K) ? g.A[m * g.sAm + k * g.sAk] : 0.0;
      }
      for (int e = tid; e < BN_ * BK; e += 256) {
        const int nn = b_nfast ? e % BN_ : e / BK, kk = b_nfast ? e / BN_ : e % BK;
        const int64_t n = n0 + nn, k = k0 + kk;
        Bs[kk][nn] = (n < g.N && k < g.K) ? g.B[k * g.sBk + n * g.sBn] : 0.0;
      }
      __syncthreads();
#pragma unroll
      for (int kk = 0; kk < BK; kk++) {
        double a[TM], b[TN];
#pragma unroll
        for (int i = 0; i < TM; i++) a[i] = As[kk][ty + 16 * i];
#pragma unroll
        for (int j = 0; j < TN; j++) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
        for (int i = 0; i < TM; i++)
#pragma unroll
          for (int j = 0; j < TN; j++) acc[i][j] = fma(a[i], b[j], acc[i][j]);
      }
      __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < TM; i++) {
      const int64_t m = m0 + ty + 16 * i;
      if (m >= g.M) continue;
#pragma unroll
      for (int j = 0; j < TN; j++) {
        const int64_t n = n0 + tx + 16 * j;
        if (n >= g.N) continue;
        double* c = g.C + m * g.sCm + n * g.sCn;
        const double v = g.alpha * acc[i][j];
        *c = (g.beta == 0.0) ? v : fma(g.beta, *c, v);
      }
    }
  }
}

struct TileShape {
  int bm, bn;
};
constexpr TileShape kShapes[] = {{64, 64}, {32, 32}, {64, 32}, {32, 64}};
constexpr int kNumShapes = 4;

__global__ void grouped_perm(const PermDesc* __restrict__ desc, const int64_t* __restrict__ prefix, int nd,
                             int64_t total, const int* __restrict__ active) {
  for (int64_t t = blockIdx.x; t < total; t += gridDim.x) {
    const int di = find_item(prefix, nd, t);
    const PermDesc& p = desc[di];
    if (!active[p.prob]) continue;
    const int64_t e0 = (t - prefix[di]) * kChunk, e1 = min(e0 + kChunk, p.total);
    for (int64_t e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
      int64_t r = e, oi = 0, oo = 0;
      for (int k = p.rank - 1; k >= 0; k--) {
        const int64_t x = r % p.d[k];
        r /= p.d[k];
        oi += x * p.si[k];
        oo += x * p.so[k];
      }
      if (p.fill) {
        p.out[oo] = p.alpha;
      } else {
        const double v = p.alpha * p.in[oi];
        p.out[oo] = (p.beta == 0.0) ? v : fma(p.beta, p.out[oo], v);
      }
    }
  }
}

// ---------------------------------------------------------------------------------------
// Sweep kernels over (member, chunk of its packed amplitudes)
// ---------------------------------------------------------------------------------------
__device__ double block_sum(double v) {
  __shared__ double sh[32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x / 32, l = threadIdx.x % 32;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  const int nw = (blockDim.x + 31) / 32;
  v = (threadIdx.x < nw) ? sh[threadIdx.x] : 0.0;
  if (w == 0)
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double denom(const Member& m, int64_t x) {
  const double* e = m.eps;
  if (x < m.n1) return e[x / m.nv] - e[m.no + x % m.nv];
  int64_t y = x - m.n1;
  const int b = (int)(y % m.nv);
  y /= m.nv;
  const int a = (int)(y % m.nv);
  y /= m.nv;
  const int j = (int)(y % m.no), i = (int)(y / m.no);
  return ((e[i] + e[j]) - e[m.no + a]) - e[m.no + b];
}

// Told = T (start of a sweep)
__global__ void save_kernel(const Member* __restrict__ mem, const int64_t* __restrict__ prefix, int nm, int64_t total,
                            const int* __restrict__ active) {
  for (int64_t t = blockIdx.x; t < total; t += gridDim.x) {
    const int b = find_item(prefix, nm, t);
    if (!active[b]) continue;
    const Member& m = mem[b];
    const int64_t e0 = (t - prefix[b]) * kChunk, e1 = min(e0 + kChunk, m.np);
    for (int64_t x = e0 + threadIdx.x; x < e1; x += blockDim.x) m.Told[x] = m.T[x];
  }
}

// T = Told + R / D; partial[t] = sum of R^2 over the chunk
__global__ void jacobi_kernel(const Member* __restrict__ mem, const int64_t* __restrict__ prefix, int nm,
                              int64_t total, const int* __restrict__ active, double* partial) {
  for (int64_t t = blockIdx.x; t < total; t += gridDim.x) {
    const int b = find_item(prefix, nm, t);
    if (!active[b]) continue;
    const Member& m = mem[b];
    const int64_t e0 = (t - prefix[b]) * kChunk, e1 = min(e0 + kChunk, m.np);
    double s = 0.0;
    for (int64_t x = e0 + threadIdx.x; x < e1; x += blockDim.x) {
      const double r = m.R[x];
      s += r * r;
      m.T[x] = m.Told[x] + r / denom(m, x);
    }
    s = block_sum(s);
    if (threadIdx.x == 0) partial[t] = s;
  }
}

// per member: sum of its chunk partials in a fixed order (one block per member)
__global__ void reduce_kernel(const int64_t* __restrict__ prefix, int nm, int64_t total, const int* __restrict__ active,
                              const double* __restrict__ partial, double* out) {
  const int b = blockIdx.x;
  if (b >= nm || !active[b]) return;
  const int64_t t0 = prefix[b], t1 = (b + 1 < nm) ? prefix[b + 1] : total;
  double s = 0.0;
  for (int64_t t = t0 + threadIdx.x; t < t1; t += blockDim.x) s += partial[t];
  s = block_sum(s);
  if (threadIdx.x == 0) out[b] = s;
}

// convergence test (ccwfn.cc:216) and the DIIS slot of this sweep's add
__global__ void converge_kernel(int nm, SweepState* st, int* active, const double* __restrict__ sumsq, double* rms,
                                int* iterations, int* converged) {
  const int iter = st->iter + 1;
  int left = 0;
  for (int b = threadIdx.x; b < nm; b += blockDim.x) {
    if (!active[b]) continue;
    const double r = sqrt(sumsq[b]);
    rms[b] = r;
    iterations[b] = iter;
    if (r < st->r_conv) {
      active[b] = 0;
      converged[b] = 1;
    } else if (iter >= st->maxiter) {
      active[b] = 0;
    } else {
      left++;
    }
  }
  for (int o = 16; o > 0; o >>= 1) left += __shfl_down_sync(0xffffffffu, left, o);
  __shared__ int sh[32];
  if (threadIdx.x % 32 == 0) sh[threadIdx.x / 32] = left;
  __syncthreads();
  if (threadIdx.x == 0) {
    int tot = 0;
    for (int w = 0; w < (int)(blockDim.x + 31) / 32; w++) tot += sh[w];
    st->active_count = tot;
    st->iter = iter;
    st->slot = st->count < kDiis ? st->count : st->nadded % kDiis;
    st->count = min(st->count + 1, kDiis);
    st->nadded++;
  }
}

// err[slot] = T - Told, vec[slot] = T
__global__ void diis_add_kernel(const Member* __restrict__ mem, const int64_t* __restrict__ prefix, int nm,
                                int64_t total, const int* __restrict__ active, const SweepState* __restrict__ st) {
  const int slot = st->slot;
  for (int64_t t = blockIdx.x; t < total; t += gridDim.x) {
    const int b = find_item(prefix, nm, t);
    if (!active[b]) continue;
    const Member& m = mem[b];
    double* e = m.err + (int64_t)slot * m.np;
    double* v = m.vec + (int64_t)slot * m.np;
    const int64_t e0 = (t - prefix[b]) * kChunk, e1 = min(e0 + kChunk, m.np);
    for (int64_t x = e0 + threadIdx.x; x < e1; x += blockDim.x) {
      const double tn = m.T[x];
      e[x] = tn - m.Told[x];
      v[x] = tn;
    }
  }
}

// partial[p * total + t] = <err_p, err_slot> over chunk t (blockIdx.y = p)
__global__ void diis_dot_kernel(const Member* __restrict__ mem, const int64_t* __restrict__ prefix, int nm,
                                int64_t total, const int* __restrict__ active, const SweepState* __restrict__ st,
                                double* partial) {
  const int p = blockIdx.y;
  if (p >= st->count) return;
  const int slot = st->slot;
  for (int64_t t = blockIdx.x; t < total; t += gridDim.x) {
    const int b = find_item(prefix, nm, t);
    if (!active[b]) continue;
    const Member& m = mem[b];
    const double* ep = m.err + (int64_t)p * m.np;
    const double* es = m.err + (int64_t)slot * m.np;
    const int64_t e0 = (t - prefix[b]) * kChunk, e1 = min(e0 + kChunk, m.np);
    double s = 0.0;
    for (int64_t x = e0 + threadIdx.x; x < e1; x += blockDim.x) s += ep[x] * es[x];
    s = block_sum(s);
    if (threadIdx.x == 0) partial[(int64_t)p * total + t] = s;
  }
}

// B-matrix row of this sweep's add, then the bordered solve (the elimination of
// diis_coefficients in cc_ground.cpp), one thread per member
__global__ void diis_solve_kernel(const int64_t* __restrict__ prefix, int nm, int64_t total,
                                  const int* __restrict__ active, const SweepState* __restrict__ st,
                                  const double* __restrict__ partial, double* Bmat, double* coef, int* status) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nm || !active[b]) return;
  const int cnt = st->count, slot = st->slot;
  double* Bb = Bmat + (int64_t)b * kDiis * kDiis;
  const int64_t t0 = prefix[b], t1 = (b + 1 < nm) ? prefix[b + 1] : total;
  for (int p = 0; p < cnt; p++) {
    double s = 0.0;
    for (int64_t t = t0; t < t1; t++) s += partial[(int64_t)p * total + t];
    Bb[slot * kDiis + p] = s;
    Bb[p * kDiis + slot] = s;
  }
  double* cb = coef + (int64_t)b * kDiis;
  if (cnt <= 2) return;  // ccwfn.cc:220: extrapolate only with more than two vectors
  const int n = cnt, mdim = n + 1;
  double B[(kDiis + 1) * (kDiis + 1)], c[kDiis + 1];
  double mx = 0.0;
  for (int p = 0; p < n; p++)
    for (int q = 0; q < n; q++) {
      B[p * mdim + q] = Bb[p * kDiis + q];
      mx = fmax(mx, fabs(B[p * mdim + q]));
    }
  if (mx > 0.0)
    for (int p = 0; p < n; p++)
      for (int q = 0; q < n; q++) B[p * mdim + q] /= mx;
  for (int p = 0; p < n; p++) B[p * mdim + n] = B[n * mdim + p] = -1.0;
  B[n * mdim + n] = 0.0;
  for (int p = 0; p < mdim; p++) c[p] = 0.0;
  c[n] = -1.0;
  for (int col = 0; col < mdim; col++) {
    int piv = col;
    for (int r = col + 1; r < mdim; r++)
      if (fabs(B[r * mdim + col]) > fabs(B[piv * mdim + col])) piv = r;
    if (piv != col) {
      for (int k = 0; k < mdim; k++) {
        const double tmp = B[col * mdim + k];
        B[col * mdim + k] = B[piv * mdim + k];
        B[piv * mdim + k] = tmp;
      }
      const double tmp = c[col];
      c[col] = c[piv];
      c[piv] = tmp;
    }
    const double d = B[col * mdim + col];
    if (d == 0.0) {
      status[b] = 1;  // singular subspace: the member keeps its Jacobi step
      return;
    }
    for (int r = col + 1; r < mdim; r++) {
      const double f = B[r * mdim + col] / d;
      if (f == 0.0) continue;
      for (int k = col; k < mdim; k++) B[r * mdim + k] -= f * B[col * mdim + k];
      c[r] -= f * c[col];
    }
  }
  for (int r = mdim - 1; r >= 0; r--) {
    double s = c[r];
    for (int k = r + 1; k < mdim; k++) s -= B[r * mdim + k] * c[k];
    c[r] = s / B[r * mdim + r];
  }
  for (int p = 0; p < n; p++) cb[p] = c[p];
}

// T = sum_p coef[p] vec[p] (when the member extrapolates), then tau and ttau from T
__global__ void extrapolate_tau_kernel(const Member* __restrict__ mem, const int64_t* __restrict__ prefix, int nm,
                                       int64_t total, const int* __restrict__ active,
                                       const SweepState* __restrict__ st, const double* __restrict__ coef,
                                       const int* __restrict__ status, int use_diis) {
  const int cnt = st->count;
  for (int64_t t = blockIdx.x; t < total; t += gridDim.x) {
    const int b = find_item(prefix, nm, t);
    if (!active[b]) continue;
    const Member& m = mem[b];
    const bool ex = use_diis && cnt > 2 && !status[b];
    const double* cb = coef + (int64_t)b * kDiis;
    const int64_t e0 = (t - prefix[b]) * kChunk, e1 = min(e0 + kChunk, m.np);
    if (ex)
      for (int64_t x = e0 + threadIdx.x; x < e1; x += blockDim.x) {
        double s = 0.0;
        for (int p = 0; p < cnt; p++) s += cb[p] * m.vec[(int64_t)p * m.np + x];
        m.T[x] = s;
      }
  }
}

// tau = t2 + t1 t1, ttau = t2 + t1 t1 / 2 from T, and the energy partials sum tau * L
__global__ void tau_energy_kernel(const Member* __restrict__ mem, const int64_t* __restrict__ prefix2, int nm,
                                  int64_t total, const int* __restrict__ active, double* partial) {
  for (int64_t t = blockIdx.x; t < total; t += gridDim.x) {
    const int b = find_item(prefix2, nm, t);
    if (!active[b]) continue;
    const Member& m = mem[b];
    const int64_t n2 = m.np - m.n1;
    const int64_t e0 = (t - prefix2[b]) * kChunk, e1 = min(e0 + kChunk, n2);
    const double* t1 = m.T;
    const double* t2 = m.T + m.n1;
    double s = 0.0;
    for (int64_t x = e0 + threadIdx.x; x < e1; x += blockDim.x) {
      int64_t y = x;
      const int bb = (int)(y % m.nv);
      y /= m.nv;
      const int a = (int)(y % m.nv);
      y /= m.nv;
      const int j = (int)(y % m.no), i = (int)(y / m.no);
      const double tt = t1[(int64_t)i * m.nv + a] * t1[(int64_t)j * m.nv + bb];
      const double v = t2[x];
      const double tau = v + tt;
      m.tau[x] = tau;
      m.ttau[x] = v + 0.5 * tt;
      s += tau * m.Loovv[x];
    }
    s = block_sum(s);
    if (threadIdx.x == 0) partial[t] = s;
  }
}

__global__ void energy_kernel(const Member* __restrict__ mem, const int64_t* __restrict__ prefix2, int nm,
                              int64_t total, const int* __restrict__ active, const double* __restrict__ partial,
                              double* energy) {
  const int b = blockIdx.x;
  if (b >= nm || !active[b]) return;
  const int64_t t0 = prefix2[b], t1 = (b + 1 < nm) ? prefix2[b + 1] : total;
  double s = 0.0;
  for (int64_t t = t0 + threadIdx.x; t < t1; t += blockDim.x) s += partial[t];
  s = block_sum(s);
  if (threadIdx.x == 0) {
    const Member& m = mem[b];
    energy[b] = 2.0 * m.fock_last * m.T[m.n1 - 1] + s;
  }
}

// ---------------------------------------------------------------------------------------
template <typename T>
struct DevArray {
  T* p = nullptr;
  size_t n = 0;
  DevArray() = default;
  DevArray(DevArray&& o) noexcept : p(o.p), n(o.n) {
    o.p = nullptr;
    o.n = 0;
  }
  DevArray(const DevArray&) = delete;
  DevArray& operator=(const DevArray&) = delete;
  ~DevArray() {
    if (p) cudaFree(p);
  }
  void upload(const std::vector<T>& h, cudaStream_t s) {
    if (h.size() > n) {
      if (p) cudaFree(p);
      p = nullptr;
      UCC_CUDA(cudaMalloc(&p, sizeof(T) * std::max<size_t>(1, h.size())));
      n = h.size();
    }
    if (!h.empty()) UCC_CUDA(cudaMemcpyAsync(p, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice, s));
  }
  void zeros(size_t count, cudaStream_t s) {
    if (count > n) {
      if (p) cudaFree(p);
      p = nullptr;
      UCC_CUDA(cudaMalloc(&p, sizeof(T) * std::max<size_t>(1, count)));
      n = count;
    }
    UCC_CUDA(cudaMemsetAsync(p, 0, sizeof(T) * std::max<size_t>(1, count), s));
  }
};

struct GroupOp {
  int kind = 0;  // RecordedOp::Kind (fill is a permute descriptor with fill = 1)
  int shape = 0;  // GEMM tile shape (index into kShapes)
  DevArray<GemmDesc> gdesc;
  DevArray<PermDesc> pdesc;
  DevArray<int64_t> prefix[kNumShapes];
  int64_t total[kNumShapes] = {};
  int nd = 0;
  double flops = 0.0;
};

}  // namespace batch
}  // namespace ucc

using namespace ucc;
using namespace ucc::batch;

struct ucc_batch {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string last_error;
  std::vector<std::unique_ptr<Ctx>> members;
  std::vector<int> has_guess;
  // recorded sweep
  bool built = false;
  std::vector<std::unique_ptr<DeviceBuffer>> arenas;
  std::vector<GroupOp> ops;
  DevArray<Member> mem;
  DevArray<int64_t> prefix_np, prefix_t2;
  int64_t total_np = 0, total_t2 = 0;
  DevArray<int> active, iterations, converged, status;
  DevArray<double> partial, dpartial, sumsq, rms, energy, Bmat, coef, epartial;
  DevArray<SweepState> state;
  std::vector<std::unique_ptr<DeviceBuffer>> diis_store;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int graph_kernels = 0;
  int use_diis = -1;
  double time_limit_s = 600.0;  // device time limit of one solve's sweep loop
  ucc_batch_info info{};

  ~ucc_batch() {
    if (stream) cudaStreamSynchronize(stream);
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    for (auto& m : members) m->stream = nullptr;  // the batch owns the stream
    members.clear();
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace {

template <typename F>
ucc_status bguard(ucc_batch* b, F&& f) {
  if (!b) return UCC_BAD_ARGS;
  b->last_error.clear();
  try {
    UCC_CUDA(cudaSetDevice(b->device));
    f(*b);
    return UCC_OK;
  } catch (const Error& e) {
    b->last_error = e.what();
    return e.status;
  } catch (const std::exception& e) {
    b->last_error = e.what();
    return UCC_CUDA_ERROR;
  }
}

unsigned grid_for(int64_t items) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>(items, 152 * 8)); }

void launch_gemm(ucc_batch& B, GroupOp& op, int shape) {
  const int64_t total = op.total[shape];
  if (total == 0) return;
  const unsigned grid = grid_for(total);
  const GemmDesc* d = op.gdesc.p;
  const int64_t* pf = op.prefix[shape].p;
  switch (shape) {
    case 0:
      grouped_gemm<64, 64><<<grid, 256, 0, B.stream>>>(d, pf, op.nd, total, B.active.p);
      break;
    case 1:
      grouped_gemm<32, 32><<<grid, 256, 0, B.stream>>>(d, pf, op.nd, total, B.active.p);
      break;
    case 2:
      grouped_gemm<64, 32><<<grid, 256, 0, B.stream>>>(d, pf, op.nd, total, B.active.p);
      break;
    default:
      grouped_gemm<32, 64><<<grid, 256, 0, B.stream>>>(d, pf, op.nd, total, B.active.p);
      break;
  }
  UCC_CUDA(cudaGetLastError());
}

void launch_op(ucc_batch& B, GroupOp& op) {
  if (op.kind == RecordedOp::kGemm) {
    launch_gemm(B, op, op.shape);
  } else if (op.total[0] > 0) {
    grouped_perm<<<grid_for(op.total[0]), 256, 0, B.stream>>>(op.pdesc.p, op.prefix[0].p, op.nd, op.total[0],
                                                              B.active.p);
    UCC_CUDA(cudaGetLastError());
  }
}

// record every member's residual build and group the operations
void build(ucc_batch& B) {
  const int nm = (int)B.members.size();
  UCC_REQUIRE(nm >= 1, UCC_BAD_STATE, "empty batch");
  std::vector<std::vector<RecordedOp>> traces(nm);
  std::vector<std::string> tape;
  B.arenas.clear();
  B.diis_store.clear();
  double arena_bytes = 0.0;
  for (int b = 0; b < nm; b++) {
    Ctx& c = *B.members[b];
    ccsd_alloc(c);
    const double* to = c.get("Told").p;
    double* r = c.get("R").p;
    size_t need = 0;
    for (int pass = 0; pass < 2; pass++) {
      Recorder rec;
      const bool first = b == 0 && pass == 0;
      if (!first) {
        rec.tape = tape;
        rec.replay_tape = true;
      }
      if (pass == 1) {
        B.arenas.push_back(std::make_unique<DeviceBuffer>(need / sizeof(double) + 1));
        rec.arena = reinterpret_cast<char*>(B.arenas.back()->p);
        arena_bytes += (double)need;
      }
      recorder() = &rec;
      try {
        ccsd_residual(c, to, r);
      } catch (...) {
        recorder() = nullptr;
        throw;
      }
      recorder() = nullptr;
      if (first) tape = rec.tape;
      UCC_REQUIRE(first || rec.tape_pos == tape.size(), UCC_BAD_STATE, "recorded contraction sequence diverged");
      if (pass == 0)
        need = rec.peak;
      else
        traces[b] = std::move(rec.ops);
    }
  }
  const size_t nops = traces[0].size();
  for (int b = 1; b < nm; b++) {
    UCC_REQUIRE(traces[b].size() == nops, UCC_BAD_STATE, "members recorded different operation counts");
    for (size_t k = 0; k < nops; k++)
      UCC_REQUIRE(traces[b][k].kind == traces[0][k].kind && traces[b][k].rank == traces[0][k].rank, UCC_BAD_STATE,
                  "members recorded different operation kinds");
  }
  B.ops.clear();
  B.ops.resize(nops);
  for (size_t k = 0; k < nops; k++) {
    GroupOp& g = B.ops[k];
    g.kind = traces[0][k].kind;
    g.nd = nm;
    if (g.kind == RecordedOp::kGemm) {
      std::vector<GemmDesc> d(nm);
      for (int b = 0; b < nm; b++) {
        const RecordedOp& o = traces[b][k];
        d[b] = GemmDesc{o.M, o.N, o.K, o.sAm, o.sAk, o.sBk, o.sBn, o.sCm, o.sCn, o.A, o.B, o.C, o.alpha, o.beta, b};
        g.flops += 2.0 * (double)o.M * (double)o.N * (double)o.K;
      }
      g.gdesc.upload(d, B.stream);
      for (int s = 0; s < kNumShapes; s++) {
        std::vector<int64_t> pf(nm);
        int64_t run = 0;
        for (int b = 0; b < nm; b++) {
          pf[b] = run;
          run += ((d[b].M + kShapes[s].bm - 1) / kShapes[s].bm) * ((d[b].N + kShapes[s].bn - 1) / kShapes[s].bn);
        }
        g.total[s] = run;
        g.prefix[s].upload(pf, B.stream);
      }
    } else {
      std::vector<PermDesc> d(nm);
      std::vector<int64_t> pf(nm);
      int64_t run = 0;
      for (int b = 0; b < nm; b++) {
        const RecordedOp& o = traces[b][k];
        PermDesc& p = d[b];
        std::memset(&p, 0, sizeof p);
        p.rank = o.rank;
        p.prob = b;
        p.fill = o.kind == RecordedOp::kFill;
        p.total = 1;
        for (int q = 0; q < o.rank; q++) {
          p.d[q] = o.d[q];
          p.si[q] = o.si[q];
          p.so[q] = o.so[q];
          p.total *= o.d[q];
        }
        p.in = o.in;
        p.out = o.out;
        p.alpha = o.alpha;
        p.beta = o.beta;
        pf[b] = run;
        run += (p.total + kChunk - 1) / kChunk;
      }
      g.total[0] = run;
      g.pdesc.upload(d, B.stream);
      g.prefix[0].upload(pf, B.stream);
    }
  }
  // sweep tables
  std::vector<Member> mh(nm);
  std::vector<int64_t> pnp(nm), pt2(nm);
  int64_t rnp = 0, rt2 = 0;
  for (int b = 0; b < nm; b++) {
    Ctx& c = *B.members[b];
    Member& m = mh[b];
    const int n = c.no + c.nv;
    m.no = c.no;
    m.nv = c.nv;
    m.n1 = (int64_t)c.no * c.nv;
    m.np = npacked(c);
    m.eps = c.get("eps").p;
    m.T = c.get("T").p;
    m.Told = c.get("Told").p;
    m.R = c.get("R").p;
    m.tau = c.get("tau").p;
    m.ttau = c.get("ttau").p;
    m.Loovv = c.get("Loovv").p;
    B.diis_store.push_back(std::make_unique<DeviceBuffer>((size_t)(2 * kDiis * m.np)));
    m.err = B.diis_store.back()->p;
    m.vec = m.err + (int64_t)kDiis * m.np;
    m.fock_last = c.fock[(size_t)(c.no - 1) * n + (n - 1)];
    pnp[b] = rnp;
    rnp += (m.np + kChunk - 1) / kChunk;
    pt2[b] = rt2;
    rt2 += (m.np - m.n1 + kChunk - 1) / kChunk;
  }
  B.mem.upload(mh, B.stream);
  B.prefix_np.upload(pnp, B.stream);
  B.prefix_t2.upload(pt2, B.stream);
  B.total_np = rnp;
  B.total_t2 = rt2;
  B.partial.zeros((size_t)rnp, B.stream);
  B.dpartial.zeros((size_t)rnp * kDiis, B.stream);
  B.epartial.zeros((size_t)rt2, B.stream);
  for (DevArray<double>* a : {&B.sumsq, &B.rms, &B.energy}) a->zeros((size_t)nm, B.stream);
  B.Bmat.zeros((size_t)nm * kDiis * kDiis, B.stream);
  B.coef.zeros((size_t)nm * kDiis, B.stream);
  for (DevArray<int>* a : {&B.active, &B.iterations, &B.converged, &B.status}) a->zeros((size_t)nm, B.stream);
  B.state.zeros(1, B.stream);
  UCC_CUDA(cudaStreamSynchronize(B.stream));
  B.info.members = nm;
  B.info.grouped_ops = (int)nops;
  B.info.arena_bytes = arena_bytes;
  B.built = true;
}

void set_all_active(ucc_batch& B) {
  std::vector<int> one(B.members.size(), 1);
  B.active.upload(one, B.stream);
}

// one residual build with the default shapes (valid data in every buffer), then each
// GEMM operation timed with every tile shape; the fastest is kept
void autotune(ucc_batch& B) {
  set_all_active(B);
  for (auto& op : B.ops) launch_op(B, op);
  UCC_CUDA(cudaStreamSynchronize(B.stream));
  cudaEvent_t e0, e1;
  UCC_CUDA(cudaEventCreate(&e0));
  UCC_CUDA(cudaEventCreate(&e1));
  for (int s = 0; s < kNumShapes; s++) B.info.shape_choice[s] = 0;
  for (auto& op : B.ops) {
    if (op.kind != RecordedOp::kGemm) continue;
    float best = 1e30f;
    int pick = 0;
    for (int s = 0; s < kNumShapes; s++) {
      if (op.total[s] == 0) continue;
      launch_gemm(B, op, s);  // warm
      cudaEventRecord(e0, B.stream);
      launch_gemm(B, op, s);
      cudaEventRecord(e1, B.stream);
      UCC_CUDA(cudaEventSynchronize(e1));
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (ms < best) {
        best = ms;
        pick = s;
      }
    }
    op.shape = pick;
    B.info.shape_choice[pick]++;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
}

// the kernels of one sweep, in order (captured into the sweep graph)
int enqueue_sweep(ucc_batch& B) {
  const int nm = (int)B.members.size();
  int k = 0;
  save_kernel<<<grid_for(B.total_np), 256, 0, B.stream>>>(B.mem.p, B.prefix_np.p, nm, B.total_np, B.active.p);
  k++;
  for (auto& op : B.ops) {
    launch_op(B, op);
    k++;
  }
  jacobi_kernel<<<grid_for(B.total_np), 256, 0, B.stream>>>(B.mem.p, B.prefix_np.p, nm, B.total_np, B.active.p,
                                                            B.partial.p);
  reduce_kernel<<<nm, 256, 0, B.stream>>>(B.prefix_np.p, nm, B.total_np, B.active.p, B.partial.p, B.sumsq.p);
  converge_kernel<<<1, 1024, 0, B.stream>>>(nm, B.state.p, B.active.p, B.sumsq.p, B.rms.p, B.iterations.p,
                                            B.converged.p);
  k += 3;
  if (B.use_diis) {
    diis_add_kernel<<<grid_for(B.total_np), 256, 0, B.stream>>>(B.mem.p, B.prefix_np.p, nm, B.total_np, B.active.p,
                                                                B.state.p);
    diis_dot_kernel<<<dim3(grid_for(B.total_np), kDiis), 256, 0, B.stream>>>(B.mem.p, B.prefix_np.p, nm, B.total_np,
                                                                             B.active.p, B.state.p, B.dpartial.p);
    diis_solve_kernel<<<(nm + 127) / 128, 128, 0, B.stream>>>(B.prefix_np.p, nm, B.total_np, B.active.p, B.state.p,
                                                              B.dpartial.p, B.Bmat.p, B.coef.p, B.status.p);
    extrapolate_tau_kernel<<<grid_for(B.total_np), 256, 0, B.stream>>>(B.mem.p, B.prefix_np.p, nm, B.total_np,
                                                                       B.active.p, B.state.p, B.coef.p, B.status.p, 1);
    k += 4;
  }
  tau_energy_kernel<<<grid_for(B.total_t2), 256, 0, B.stream>>>(B.mem.p, B.prefix_t2.p, nm, B.total_t2, B.active.p,
                                                                B.epartial.p);
  energy_kernel<<<nm, 256, 0, B.stream>>>(B.mem.p, B.prefix_t2.p, nm, B.total_t2, B.active.p, B.epartial.p,
                                          B.energy.p);
  k += 2;
  UCC_CUDA(cudaGetLastError());
  return k;
}

// the solve graph: start node -> while(members iterating) { sweep kernels; loop control }
void capture(ucc_batch& B, bool diis) {
  if (B.exec && B.use_diis == (int)diis) return;
  if (B.exec) cudaGraphExecDestroy(B.exec);
  if (B.graph) cudaGraphDestroy(B.graph);
  B.exec = nullptr;
  B.graph = nullptr;
  B.use_diis = diis;
  UCC_CUDA(cudaGraphCreate(&B.graph, 0));
  SweepState* stp = B.state.p;
  void* start_args[] = {&stp};
  cudaKernelNodeParams kp = {};
  kp.func = (void*)solve_start_kernel;
  kp.gridDim = dim3(1);
  kp.blockDim = dim3(1);
  kp.kernelParams = start_args;
  cudaGraphNode_t start = nullptr, loop = nullptr;
  UCC_CUDA(cudaGraphAddKernelNode(&start, B.graph, nullptr, 0, &kp));
  cudaGraphConditionalHandle handle;
  UCC_CUDA(cudaGraphConditionalHandleCreate(&handle, B.graph, 1, cudaGraphCondAssignDefault));
  cudaGraphNodeParams cp = {};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = handle;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  UCC_CUDA(cudaGraphAddNode(&loop, B.graph, &start, nullptr, 1, &cp));
  cudaGraph_t body = cp.conditional.phGraph_out[0];
  UCC_CUDA(cudaStreamBeginCaptureToGraph(B.stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  int k = 0;
  try {
    k = enqueue_sweep(B);
    loop_control_kernel<<<1, 1, 0, B.stream>>>(handle, B.state.p);
    UCC_CUDA(cudaGetLastError());
    k++;
  } catch (...) {
    cudaGraph_t g = nullptr;
    cudaStreamEndCapture(B.stream, &g);
    throw;
  }
  cudaGraph_t captured = nullptr;
  UCC_CUDA(cudaStreamEndCapture(B.stream, &captured));
  UCC_CUDA(cudaGraphInstantiate(&B.exec, B.graph, 0));
  B.graph_kernels = k;
  B.info.graph_kernels = k;
}

// amplitudes of every member at the start of a solve: a supplied guess, else MP2
void start_members(ucc_batch& B) {
  for (auto& mp : B.members) {
    Ctx& c = *mp;
    const int no = c.no, nv = c.nv;
    const int64_t np = npacked(c), n1 = (int64_t)no * nv;
    double* T = c.get("T").p;
    if (c.has("T_guess")) {
      UCC_CUDA(cudaMemcpyAsync(T, c.get("T_guess").p, sizeof(double) * np, cudaMemcpyDeviceToDevice, c.stream));
      UCC_CUDA(cudaStreamSynchronize(c.stream));
      c.drop("T_guess");
    } else {  // t1 = f_ia / D1, t2 = <ij|ab> / D2 (ccwfn.cc:75-87)
      double* R = c.get("R").p;
      double* Told = c.get("Told").p;
      permute_add(c, Fk(c, "ov"), 1.0, 0.0, amp1(c, R));
      permute_add(c, V(c, "oovv"), 1.0, 0.0, amp2(c, R));
      fill(c, np, 0.0, Told);
      Scratch ss(c, sizeof(double));
      const double* e = c.get("eps").p;
      jacobi_update(c, no, nv, e, e + no, 0.0, R, R + n1, Told, Told + n1, T, T + n1, ss.d());
    }
    build_tau(c, no, nv, T, T + n1, 1.0, c.get("tau").p, 0.5, c.get("ttau").p);
  }
  UCC_CUDA(cudaStreamSynchronize(B.stream));
}

}  // namespace

extern "C" {

ucc_status ucc_batch_create(ucc_batch** out, int device) {
  if (!out) return UCC_BAD_ARGS;
  *out = nullptr;
  int nd = 0;
  if (cudaGetDeviceCount(&nd) != cudaSuccess || device < 0 || device >= nd) return UCC_CUDA_ERROR;
  ucc_batch* b = new (std::nothrow) ucc_batch;
  if (!b) return UCC_OUT_OF_MEMORY;
  b->device = device;
  ucc_status st = bguard(b, [&](ucc_batch& B) { UCC_CUDA(cudaStreamCreateWithFlags(&B.stream, cudaStreamNonBlocking)); });
  if (st != UCC_OK) {
    delete b;
    return st;
  }
  *out = b;
  return UCC_OK;
}

ucc_status ucc_batch_destroy(ucc_batch* b) {
  if (!b) return UCC_BAD_ARGS;
  cudaSetDevice(b->device);
  delete b;
  return UCC_OK;
}

const char* ucc_batch_last_error(ucc_batch* b) { return b ? b->last_error.c_str() : "null batch"; }

ucc_status ucc_batch_add_df(ucc_batch* b, int no, int nv, int naux, const double* fock, const double* Bq, int* index) {
  return bguard(b, [&](ucc_batch& B) {
    UCC_REQUIRE(no >= 1 && nv >= 1 && naux >= 1 && fock && Bq, UCC_BAD_ARGS, "need no, nv, naux >= 1, fock and B");
    auto c = std::make_unique<Ctx>();
    c->device = B.device;
    c->stream = B.stream;
    ucc_options_default(&c->opt);
    try {
      load_from_df(*c, no, nv, naux, fock, Bq);
    } catch (...) {
      c->stream = nullptr;
      throw;
    }
    c->loaded = true;
    B.members.push_back(std::move(c));
    B.built = false;
    if (B.exec) cudaGraphExecDestroy(B.exec);
    if (B.graph) cudaGraphDestroy(B.graph);
    B.exec = nullptr;
    B.graph = nullptr;
    if (index) *index = (int)B.members.size() - 1;
  });
}

ucc_status ucc_batch_guess_mlp(ucc_batch* b, int index, ucc_mlp* net) {
  return bguard(b, [&](ucc_batch& B) {
    UCC_REQUIRE(net && index >= 0 && index < (int)B.members.size(), UCC_BAD_ARGS, "bad member index or network");
    mlp_guess(*B.members[index], net);
  });
}

ucc_status ucc_batch_ccsd(ucc_batch* b, const ucc_options* opt, double* e_ccsd, int* iterations, int* converged) {
  return bguard(b, [&](ucc_batch& B) {
    UCC_REQUIRE(opt && e_ccsd && iterations && converged, UCC_BAD_ARGS, "null argument");
    UCC_REQUIRE(opt->precision == UCC_FP64, UCC_UNSUPPORTED, "the batched solver runs the FP64 form");
    UCC_REQUIRE(opt->maxiter >= 1 && opt->r_convergence > 0, UCC_BAD_ARGS, "bad maxiter or r_convergence");
    const int nm = (int)B.members.size();
    UCC_REQUIRE(nm >= 1, UCC_BAD_STATE, "empty batch");
    if (!B.built) {
      build(B);
      autotune(B);
    }
    capture(B, opt->diis != 0);
    start_members(B);
    set_all_active(B);
    for (DevArray<int>* a : {&B.iterations, &B.converged, &B.status}) a->zeros((size_t)nm, B.stream);
    std::vector<SweepState> st(1);
    st[0] = SweepState{0, 0, 0, 0, nm, opt->r_convergence, opt->maxiter, 0ull,
                       (unsigned long long)(B.time_limit_s * 1e9), 0};
    B.state.upload(st, B.stream);
    // energies of the starting amplitudes (what a member that stops at once reports)
    std::vector<double> e0(nm);
    for (int k = 0; k < nm; k++) e0[k] = ccsd_energy(*B.members[k], B.members[k]->get("T").p);
    B.energy.upload(e0, B.stream);
    cudaEvent_t t0, t1;
    UCC_CUDA(cudaEventCreate(&t0));
    UCC_CUDA(cudaEventCreate(&t1));
    UCC_CUDA(cudaEventRecord(t0, B.stream));
    // the whole solve: one graph launch, the sweep loop runs on the device
    UCC_CUDA(cudaGraphLaunch(B.exec, B.stream));
    B.info.graph_launches = 1;
    UCC_CUDA(cudaEventRecord(t1, B.stream));
    UCC_CUDA(cudaEventSynchronize(t1));
    SweepState fin;
    UCC_CUDA(cudaMemcpy(&fin, B.state.p, sizeof(SweepState), cudaMemcpyDeviceToHost));
    const int sweeps = fin.iter;
    count_kernel_launch();  // the start node
    for (int k = 0; k < sweeps * B.graph_kernels; k++) count_kernel_launch();
    float ms = 0.f;
    cudaEventElapsedTime(&ms, t0, t1);
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    UCC_CUDA(cudaMemcpy(e_ccsd, B.energy.p, sizeof(double) * nm, cudaMemcpyDeviceToHost));
    UCC_CUDA(cudaMemcpy(iterations, B.iterations.p, sizeof(int) * nm, cudaMemcpyDeviceToHost));
    UCC_CUDA(cudaMemcpy(converged, B.converged.p, sizeof(int) * nm, cudaMemcpyDeviceToHost));
    double fl = 0.0;
    for (int k = 0; k < nm; k++) {
      fl += iterations[k] * flops_ccsd_iter(B.members[k]->no, B.members[k]->nv);
      B.members[k]->have_ccsd = converged[k] != 0;
    }
    B.info.sweeps = sweeps;
    B.info.solve_ms = ms;
    B.info.flops = fl;
    UCC_REQUIRE(!fin.timed_out, UCC_DEVICE_TIMEOUT,
                "batched solve: the device time limit (" + std::to_string(B.time_limit_s) + " s) ran out after " +
                    std::to_string(sweeps) + " sweeps with " + std::to_string(fin.active_count) +
                    " members still iterating");
  });
}

ucc_status ucc_batch_set_time_limit(ucc_batch* b, double seconds) {
  return bguard(b, [&](ucc_batch& B) {
    UCC_REQUIRE(seconds > 0.0 && seconds <= 86400.0, UCC_BAD_ARGS, "time limit must be in (0, 86400] s");
    B.time_limit_s = seconds;
  });
}

ucc_status ucc_batch_features(ucc_batch* b, int index, float* out, size_t rows, int with_targets, float* targets) {
  return bguard(b, [&](ucc_batch& B) {
    UCC_REQUIRE(index >= 0 && index < (int)B.members.size(), UCC_BAD_ARGS, "bad member index");
    mlp_features(*B.members[index], out, rows, targets, with_targets != 0);
  });
}

ucc_status ucc_batch_get_info(ucc_batch* b, ucc_batch_info* out) {
  return bguard(b, [&](ucc_batch& B) {
    UCC_REQUIRE(out, UCC_BAD_ARGS, "null argument");
    *out = B.info;
  });
}

ucc_status ucc_batch_get_t2(ucc_batch* b, int index, double* out, size_t count) {
  return bguard(b, [&](ucc_batch& B) {
    UCC_REQUIRE(out && index >= 0 && index < (int)B.members.size(), UCC_BAD_ARGS, "bad member index");
    Ctx& c = *B.members[index];
    UCC_REQUIRE(c.has("T"), UCC_BAD_STATE, "no amplitudes yet");
    const int64_t n1 = (int64_t)c.no * c.nv, n2 = npacked(c) - n1;
    UCC_REQUIRE((int64_t)count == n2, UCC_BAD_ARGS, "t2 size mismatch");
    UCC_CUDA(cudaMemcpy(out, c.get("T").p + n1, sizeof(double) * n2, cudaMemcpyDeviceToHost));
  });
}

}  // extern "C"
