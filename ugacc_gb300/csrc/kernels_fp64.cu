// FP64 kernels for the plain form of the RHF-CC solver (sm_103a).
//
//  * dgemm_kernel      -- register-blocked DFMA GEMM over arbitrarily strided operands,
//                         with a permuting epilogue so that a contraction result lands
//                         directly in its tensor layout (no separate transpose pass)
//  * permute_kernel_*  -- tensor transposition with alpha/beta through a 32x33 shared tile
//  * reductions        -- compensated (Neumaier) FP64 sums in two deterministic passes
//  * amplitude kernels -- tau/ttau, Jacobi update with on-the-fly denominators, DIIS
//                         linear combination
//  * triples_energy    -- the (T) energy of ccwfn.cc:795-852 for a batch of i>=j>=k
//                         tuples, reading W3 produced by the tuple GEMMs
#include <algorithm>
#include <atomic>
#include <cstdio>
#include <memory>

#include "core.h"

namespace ucc {

static std::atomic<int64_t> g_launches{0};
int64_t launches() { return g_launches.load(); }
static inline void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void count_kernel_launch() { count_launch(); }

static void check_launch(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) throw Error(UCC_CUDA_ERROR, std::string(what) + ": " + cudaGetErrorString(e));
}

// ------------------------------------------------------------------------------------
// GEMM
// ------------------------------------------------------------------------------------
namespace {
constexpr int BM = 64, BN = 64, BK = 16, GT = 256;

struct GemmArgs {
  int64_t M, N, K;
  int64_t kchunk;  // > 0: split-K, blockIdx.z selects K range [z*kchunk, min(K,(z+1)*kchunk)) and the
                   // tile goes to C + z*M*N as a plain row-major partial (alpha = 1, beta = 0)
  double alpha, beta;
  const double* A;
  int64_t sAm, sAk, bA;
  const double* B;
  int64_t sBk, sBn, bB;
  double* C;
  int64_t bC;
  GemmEpilogue epi;
  const GemmPtrs* ptrs;
};

template <bool AK, bool BN_>
__global__ void __launch_bounds__(GT) dgemm_kernel(GemmArgs g) {
  __shared__ double As[BK][BM + 1];
  __shared__ double Bs[BK][BN + 1];
  const int tid = threadIdx.x;
  const int tx = tid % 16, ty = tid / 16;
  const int64_t m0 = (int64_t)blockIdx.y * BM, n0 = (int64_t)blockIdx.x * BN;
  const double* A;
  const double* B;
  double* C;
  int64_t kbeg = 0, kend = g.K;
  if (g.ptrs) {
    A = g.ptrs[blockIdx.z].A;
    B = g.ptrs[blockIdx.z].B;
    C = g.ptrs[blockIdx.z].C;
  } else if (g.kchunk > 0) {
    A = g.A;
    B = g.B;
    C = g.C + (int64_t)blockIdx.z * g.M * g.N;
    kbeg = (int64_t)blockIdx.z * g.kchunk;
    kend = min(g.K, kbeg + g.kchunk);
  } else {
    A = g.A + (int64_t)blockIdx.z * g.bA;
    B = g.B + (int64_t)blockIdx.z * g.bB;
    C = g.C + (int64_t)blockIdx.z * g.bC;
  }
  double acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) acc[i][j] = 0.0;

  for (int64_t k0 = kbeg; k0 < kend; k0 += BK) {
#pragma unroll
    for (int r = 0; r < (BM * BK) / GT; r++) {
      const int e = tid + r * GT;
      int mm, kk;
      if (AK) { mm = e / BK; kk = e % BK; } else { kk = e / BM; mm = e % BM; }
      const int64_t m = m0 + mm, k = k0 + kk;
      As[kk][mm] = (m < g.M && k < kend) ? A[m * g.sAm + k * g.sAk] : 0.0;
    }
#pragma unroll
    for (int r = 0; r < (BN * BK) / GT; r++) {
      const int e = tid + r * GT;
      int nn, kk;
      if (BN_) { kk = e / BN; nn = e % BN; } else { nn = e / BK; kk = e % BK; }
      const int64_t n = n0 + nn, k = k0 + kk;
      Bs[kk][nn] = (n < g.N && k < kend) ? B[k * g.sBk + n * g.sBn] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; kk++) {
      double a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; i++) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; j++) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
  GemmEpilogue ep = g.epi;
  double alpha = g.alpha, beta = g.beta;
  if (g.kchunk > 0) {
    ep.msplit = 0;
    ep.s_mhi = g.N;
    ep.s_n = 1;
    alpha = 1.0;
    beta = 0.0;
  }
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const int64_t m = m0 + ty + 16 * i;
    if (m >= g.M) continue;
    const int64_t mo = ep.msplit ? (m / ep.msplit) * ep.s_mhi + (m % ep.msplit) * ep.s_mlo : m * ep.s_mhi;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const int64_t n = n0 + tx + 16 * j;
      if (n >= g.N) continue;
      double* cp = C + mo + n * ep.s_n;
      const double v = alpha * acc[i][j];
      *cp = (beta == 0.0) ? v : fma(beta, *cp, v);
    }
  }
}

// alpha * x + beta * y with the common coefficients taken off the FP64 pipe (GB300 issues
// about two FP64 operations per SM clock, so a multiply per element already competes with
// HBM): alpha = +-1 is exact (a sign flip), beta = 0 stores, beta = 1 adds once.  The
// results are bit-identical to fma(beta, y, alpha * x).
__device__ __forceinline__ double combine(double alpha, double x, double beta, const double* y) {
  double v;
  if (alpha == 1.0)
    v = x;
  else if (alpha == -1.0)
    v = __longlong_as_double(__double_as_longlong(x) ^ (long long)0x8000000000000000ULL);
  else
    v = alpha * x;
  if (beta == 0.0) return v;
  if (beta == 1.0) return *y + v;
  return fma(beta, *y, v);
}
// C(epi) = alpha * sum_z P[z][m][n] + beta * C(epi), the fixed-order split-K reduction
__global__ void splitk_reduce_kernel(int64_t M, int64_t N, int nsplit, const double* P, double alpha, double beta,
                                     double* C, GemmEpilogue ep) {
  const int64_t MN = M * N;
  for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < MN; x += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int z = 0; z < nsplit; z++) s += P[(int64_t)z * MN + x];
    const int64_t m = x / N, n = x - m * N;
    const int64_t mo = ep.msplit ? (m / ep.msplit) * ep.s_mhi + (m % ep.msplit) * ep.s_mlo : m * ep.s_mhi;
    double* cp = C + mo + n * ep.s_n;
    const double v = alpha * s;
    *cp = (beta == 0.0) ? v : fma(beta, *cp, v);
  }
}
}  // namespace

void splitk_reduce(Ctx& c, int64_t M, int64_t N, int nsplit, const double* P, double alpha, double beta, double* C,
                   const GemmEpilogue& epi);

void dgemm_strided(Ctx& c, int64_t M, int64_t N, int64_t K, double alpha, const double* A, int64_t sAm, int64_t sAk,
                   const double* B, int64_t sBk, int64_t sBn, double beta, double* C, const GemmEpilogue& epi,
                   int batch, int64_t bA, int64_t bB, int64_t bC, const GemmPtrs* ptrs) {
  if (M <= 0 || N <= 0 || batch <= 0) return;
  if (Recorder* r = recorder()) {
    UCC_REQUIRE(batch == 1 && !ptrs && epi.msplit == 0, UCC_UNSUPPORTED, "dgemm: form not recordable");
    RecordedOp o;
    o.kind = RecordedOp::kGemm;
    o.M = M, o.N = N, o.K = K, o.sAm = sAm, o.sAk = sAk, o.sBk = sBk, o.sBn = sBn, o.sCm = epi.s_mhi, o.sCn = epi.s_n;
    o.A = A, o.B = B, o.C = C, o.alpha = alpha, o.beta = beta;
    r->ops.push_back(o);
    return;
  }
  UCC_REQUIRE(batch <= 65535, UCC_BAD_ARGS, "dgemm: batch too large");
  GemmArgs g{M, N, K, 0, alpha, beta, A, sAm, sAk, bA, B, sBk, sBn, bB, C, bC, epi, ptrs};
  dim3 grid((unsigned)((N + BN - 1) / BN), (unsigned)((M + BM - 1) / BM), (unsigned)batch);
  UCC_REQUIRE(grid.y <= 65535, UCC_BAD_ARGS, "dgemm: M too large");
  // Too few output tiles to fill the GPU and a long K: split K over blockIdx.z into
  // partial tiles, then reduce them in a fixed order (deterministic).
  const int64_t tiles = (int64_t)grid.x * grid.y;
  std::unique_ptr<Scratch> part;
  int nsplit = 1;
  if (batch == 1 && !ptrs && tiles < 2 * 152 && K >= 4 * 64) {
    nsplit = (int)std::min<int64_t>({(2 * 152 + tiles - 1) / tiles, K / 64, 512});
    const int64_t kchunk = ((K + nsplit - 1) / nsplit + BK - 1) / BK * BK;
    nsplit = (int)((K + kchunk - 1) / kchunk);
    if (nsplit > 1) {
      part = std::make_unique<Scratch>(c, sizeof(double) * M * N * nsplit);
      g.kchunk = kchunk;
      g.C = part->d();
      grid.z = (unsigned)nsplit;
    }
  }
  const bool ak = (sAk == 1) || (sAm != 1 && sAk < sAm);
  const bool bn = (sBn == 1) || (sBk != 1 && sBn < sBk);
  cudaEvent_t ev0 = c.take_event(), ev1 = c.take_event();
  cudaEventRecord(ev0, c.stream);
  if (ak && bn)
    dgemm_kernel<true, true><<<grid, GT, 0, c.stream>>>(g);
  else if (ak)
    dgemm_kernel<true, false><<<grid, GT, 0, c.stream>>>(g);
  else if (bn)
    dgemm_kernel<false, true><<<grid, GT, 0, c.stream>>>(g);
  else
    dgemm_kernel<false, false><<<grid, GT, 0, c.stream>>>(g);
  count_launch();
  check_launch("dgemm");
  if (part) splitk_reduce(c, M, N, nsplit, part->d(), alpha, beta, C, epi);
  cudaEventRecord(ev1, c.stream);
  c.gemm_timers.push_back({ev0, ev1, 2.0 * (double)M * (double)N * (double)K * (double)batch});
  if (c.gemm_timers.size() >= 4096) c.resolve_timers();
}

void splitk_reduce(Ctx& c, int64_t M, int64_t N, int nsplit, const double* P, double alpha, double beta, double* C,
                   const GemmEpilogue& epi) {
  const int64_t MN = M * N;
  const unsigned blocks = (unsigned)std::min<int64_t>((MN + 255) / 256, 152 * 16);
  splitk_reduce_kernel<<<blocks, 256, 0, c.stream>>>(M, N, nsplit, P, alpha, beta, C, epi);
  count_launch();
  check_launch("split-K reduce");
}

// ------------------------------------------------------------------------------------
// GEMM with a small output (M, N <= 256, M N <= 4096) and a long K (reductions such as
// sum_nef t_inef L_mnef): block z sums the K chunk [z kc, (z+1) kc) for every output into
// P[z][m][n]; splitk_reduce adds the chunks in a fixed order.  A 64 x 64 tile would leave
// most of its multiply-adds idle on such shapes.
// ------------------------------------------------------------------------------------
namespace {
constexpr int SMT = 256, SMK = 16;  // threads, K rows staged per step
__global__ void __launch_bounds__(SMT) dgemm_smallmn_kernel(int M, int N, int64_t K, int64_t kc,
                                                           const double* __restrict__ A, int64_t sAm, int64_t sAk,
                                                           const double* __restrict__ B, int64_t sBk, int64_t sBn,
                                                           double* P) {
  extern __shared__ double sm[];
  double* As = sm;                   // [SMK][M]
  double* Bs = sm + (size_t)SMK * M;  // [SMK][N]
  const int MN = M * N, t = threadIdx.x;
  const int64_t k0 = (int64_t)blockIdx.x * kc, k1 = min(K, k0 + kc);
  double acc[16];
#pragma unroll
  for (int j = 0; j < 16; j++) acc[j] = 0.0;
  for (int64_t kb = k0; kb < k1; kb += SMK) {
    const int kn = (int)(k1 - kb < SMK ? k1 - kb : SMK);
    __syncthreads();
    for (int e = t; e < SMK * M; e += SMT) {  // A tile, k fastest when A is K-contiguous
      const int kk = sAk == 1 ? e % SMK : e / M, m = sAk == 1 ? e / SMK : e % M;
      As[kk * M + m] = kk < kn ? A[(int64_t)m * sAm + (kb + kk) * sAk] : 0.0;
    }
    for (int e = t; e < SMK * N; e += SMT) {
      const int kk = sBk == 1 ? e % SMK : e / N, n = sBk == 1 ? e / SMK : e % N;
      Bs[kk * N + n] = kk < kn ? B[(kb + kk) * sBk + (int64_t)n * sBn] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < 16; j++) {
      const int o = t + j * SMT;
      if (o < MN) {
        const int m = o / N, n = o - m * N;
        double s = acc[j];
#pragma unroll
        for (int kk = 0; kk < SMK; kk++) s = fma(As[kk * M + m], Bs[kk * N + n], s);
        acc[j] = s;
      }
    }
  }
#pragma unroll
  for (int j = 0; j < 16; j++) {
    const int o = t + j * SMT;
    if (o < MN) P[(int64_t)blockIdx.x * MN + o] = acc[j];
  }
}
}  // namespace

bool dgemm_small_output(Ctx& c, int64_t M, int64_t N, int64_t K, double alpha, const double* A, int64_t sAm,
                        int64_t sAk, const double* B, int64_t sBk, int64_t sBn, double beta, double* C,
                        const GemmEpilogue& epi) {
  if (recorder() || M > 256 || N > 256 || M * N > 16 * SMT || K < 8192) return false;
  int64_t nblk = std::min<int64_t>((K + 511) / 512, 4 * 152);
  const int64_t kc = ((K + nblk - 1) / nblk + SMK - 1) / SMK * SMK;
  nblk = (K + kc - 1) / kc;
  Scratch part(c, sizeof(double) * M * N * nblk);
  cudaEvent_t ev0 = c.take_event(), ev1 = c.take_event();
  cudaEventRecord(ev0, c.stream);
  dgemm_smallmn_kernel<<<(unsigned)nblk, SMT, sizeof(double) * SMK * (M + N), c.stream>>>(
      (int)M, (int)N, K, kc, A, sAm, sAk, B, sBk, sBn, part.d());
  count_launch();
  check_launch("dgemm_smallmn");
  splitk_reduce(c, M, N, (int)nblk, part.d(), alpha, beta, C, epi);
  cudaEventRecord(ev1, c.stream);
  c.gemm_timers.push_back({ev0, ev1, 2.0 * (double)M * N * K});
  if (c.gemm_timers.size() >= 4096) c.resolve_timers();
  return true;
}

void dgemm(Ctx& c, bool ta, bool tb, int64_t M, int64_t N, int64_t K, double alpha, const double* A, int64_t lda,
           const double* B, int64_t ldb, double beta, double* C, const GemmEpilogue& epi, int batch, int64_t sA,
           int64_t sB, int64_t sC, const GemmPtrs* ptrs) {
  const int64_t sAm = ta ? 1 : lda, sAk = ta ? lda : 1;
  const int64_t sBk = tb ? 1 : ldb, sBn = tb ? ldb : 1;
  dgemm_strided(c, M, N, K, alpha, A, sAm, sAk, B, sBk, sBn, beta, C, epi, batch, sA, sB, sC, ptrs);
}

// ------------------------------------------------------------------------------------
// Permutation: out (dense, dims od) = alpha * in(strides is, in out's axis order) + beta * out
// ------------------------------------------------------------------------------------
namespace {
struct PermArgs {
  int rank;
  int64_t od[kMaxRank];
  int64_t is[kMaxRank];
  int64_t os[kMaxRank];
  double alpha, beta;
  const double* in;
  double* out;
  int64_t total;
};

// Index arithmetic runs in 32 bits (I = uint32_t) whenever every element count and offset
// fits.  The general kernel decomposes every element's index (a division per axis); merged
// axes shorten that, and the row kernel below pays it once per row.
template <class I>
__global__ void permute_kernel_elem(PermArgs a) {
  I od[kMaxRank], is[kMaxRank], os[kMaxRank];
  for (int k = 0; k < a.rank; k++) od[k] = (I)a.od[k], is[k] = (I)a.is[k], os[k] = (I)a.os[k];
  const I total = (I)a.total;
  for (I idx = (I)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += (I)gridDim.x * blockDim.x) {
    I rem = idx, off = 0, oo = 0;
    for (int k = a.rank - 1; k >= 0; k--) {
      const I x = rem % od[k];
      rem /= od[k];
      off += x * is[k];
      oo += x * os[k];
    }
    a.out[oo] = combine(a.alpha, a.in[off], a.beta, a.out + oo);
  }
}

// Rows of the last output axis cut into 128-element segments; each warp takes a contiguous
// range of segments, decomposes a row's base offsets only when its row changes, and keeps
// four loads per lane in flight before the stores.
template <class I>
__global__ void permute_kernel_rows(PermArgs a) {
  const int r = a.rank;
  I od[kMaxRank], is[kMaxRank], os[kMaxRank];
  for (int k = 0; k < r; k++) od[k] = (I)a.od[k], is[k] = (I)a.is[k], os[k] = (I)a.os[k];
  const I dl = od[r - 1], isl = is[r - 1], osl = os[r - 1];
  const I rows = (I)(a.total / a.od[r - 1]);
  const I nseg = (dl + 127) / 128, items = rows * nseg;
  const int lane = threadIdx.x & 31;
  const I nwarps = ((I)gridDim.x * blockDim.x) >> 5;
  const I warp = ((I)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const I per = (items + nwarps - 1) / nwarps;
  const I w0 = warp * per, w1 = (w0 + per < items) ? w0 + per : items;
  const double* __restrict__ in = a.in;
  double* __restrict__ out = a.out;
  I cur = (I)-1, bi = 0, bo = 0;
  for (I w = w0; w < w1; w++) {
    const I row = w / nseg, x0 = (w - row * nseg) * 128;
    if (row != cur) {
      I rem = row;
      bi = 0, bo = 0;
      for (int k = r - 2; k >= 0; k--) {
        const I x = rem % od[k];
        rem /= od[k];
        bi += x * is[k];
        bo += x * os[k];
      }
      cur = row;
    }
    double v[4];
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const I x = x0 + (I)(u * 32 + lane);
      v[u] = x < dl ? in[bi + x * isl] : 0.0;
    }
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const I x = x0 + (I)(u * 32 + lane);
      if (x < dl) {
        double* o = out + bo + x * osl;
        *o = combine(a.alpha, v[u], a.beta, o);
      }
    }
  }
}

// Tile over output axis q (contiguous in the input) and the last output axis.
struct TileArgs {
  PermArgs p;
  int q;
  int nrest;
  int64_t rd[kMaxRank];   // dims of the remaining axes
  int64_t ris[kMaxRank];  // their input strides
  int64_t ros[kMaxRank];  // their output strides
  int64_t rest_total;
  int64_t tiles_last;
};

template <class I>
__global__ void permute_kernel_tile(TileArgs t) {
  __shared__ double tile[32][33];
  const int r = t.p.rank;
  const I dl = (I)t.p.od[r - 1], dq = (I)t.p.od[t.q];
  const I tiles_last = (I)t.tiles_last;
  const I tl = ((I)blockIdx.x % tiles_last) * 32, tq = ((I)blockIdx.x / tiles_last) * 32;
  const I isl = (I)t.p.is[r - 1], osq = (I)t.p.os[t.q], osl = (I)t.p.os[r - 1];
  I rd[kMaxRank], ris[kMaxRank], ros[kMaxRank];
  for (int k = 0; k < t.nrest; k++) rd[k] = (I)t.rd[k], ris[k] = (I)t.ris[k], ros[k] = (I)t.ros[k];
  const I rest_total = (I)t.rest_total;
  for (I rest = blockIdx.y; rest < rest_total; rest += gridDim.y) {
    I rem = rest, bi = 0, bo = 0;
    for (int k = t.nrest - 1; k >= 0; k--) {
      const I x = rem % rd[k];
      rem /= rd[k];
      bi += x * ris[k];
      bo += x * ros[k];
    }
    for (int jj = threadIdx.y; jj < 32; jj += blockDim.y) {
      const I xl = tl + jj, xq = tq + threadIdx.x;
      if (xl < dl && xq < dq) tile[jj][threadIdx.x] = t.p.in[bi + xl * isl + xq];
    }
    __syncthreads();
    for (int jj = threadIdx.y; jj < 32; jj += blockDim.y) {
      const I xq = tq + jj, xl = tl + threadIdx.x;
      if (xl < dl && xq < dq) {
        double* o = t.p.out + bo + xq * osq + xl * osl;
        *o = combine(t.p.alpha, tile[threadIdx.x][jj], t.p.beta, o);
      }
    }
    __syncthreads();
  }
}

// Drop unit axes and merge neighbours that are contiguous in both tensors, so that e.g.
// ijab <- jiab becomes a rank-3 copy with rows of nv*nv elements.
void canonical_axes(PermArgs& a) {
  int r = 0;
  for (int k = 0; k < a.rank; k++) {
    if (a.od[k] == 1) continue;
    if (r > 0 && a.is[r - 1] == a.is[k] * a.od[k] && a.os[r - 1] == a.os[k] * a.od[k]) {
      a.od[r - 1] *= a.od[k];
      a.is[r - 1] = a.is[k];
      a.os[r - 1] = a.os[k];
      continue;
    }
    a.od[r] = a.od[k], a.is[r] = a.is[k], a.os[r] = a.os[k];
    r++;
  }
  if (r == 0) a.od[0] = 1, a.is[0] = 1, a.os[0] = 1, r = 1;
  a.rank = r;
}

// True when every element count and every in/out offset of the permutation is below 2^31.
bool fits32(const PermArgs& a) {
  int64_t mi = 0, mo = 0;
  for (int k = 0; k < a.rank; k++) {
    mi += (a.od[k] - 1) * (a.is[k] < 0 ? -a.is[k] : a.is[k]);
    mo += (a.od[k] - 1) * (a.os[k] < 0 ? -a.os[k] : a.os[k]);
    if (a.is[k] < 0 || a.os[k] < 0) return false;
  }
  const int64_t lim = (int64_t)1 << 31;
  return a.total < lim && mi < lim && mo < lim;
}
}  // namespace

void permute_add(Ctx& c, const Tensor& in, double alpha, double beta, const Tensor& out) {
  UCC_REQUIRE(in.rank == out.rank, UCC_BAD_ARGS, "permute_add: rank mismatch");
  if (Recorder* r = recorder()) {
    RecordedOp o;
    o.kind = RecordedOp::kPermute;
    o.rank = out.rank;
    for (int k = 0; k < out.rank; k++) {
      UCC_REQUIRE(in.d[k] == out.d[k], UCC_BAD_ARGS, "permute_add: dim mismatch");
      o.d[k] = out.d[k];
      o.si[k] = in.s[k];
      o.so[k] = out.s[k];
    }
    o.in = in.p, o.out = out.p, o.alpha = alpha, o.beta = beta;
    if (out.size() > 0) r->ops.push_back(o);
    return;
  }
  PermArgs a{};
  a.rank = out.rank;
  a.total = out.size();
  if (a.total == 0) return;
  for (int k = 0; k < out.rank; k++) {
    UCC_REQUIRE(in.d[k] == out.d[k], UCC_BAD_ARGS, "permute_add: dim mismatch");
    a.od[k] = out.d[k];
    a.is[k] = in.s[k];
    a.os[k] = out.s[k];
  }
  a.alpha = alpha;
  a.beta = beta;
  a.in = in.p;
  a.out = out.p;
  canonical_axes(a);
  const bool narrow = fits32(a);
  const int r = a.rank;
  int q = -1;
  if (r >= 2 && a.is[r - 1] != 1 && a.os[r - 1] == 1 && a.od[r - 1] >= 8) {
    for (int k = 0; k < r - 1; k++)
      if (a.is[k] == 1 && a.od[k] >= 8) q = k;
  }
  if (q >= 0) {
    TileArgs t{};
    t.p = a;
    t.q = q;
    t.nrest = 0;
    t.rest_total = 1;
    for (int k = 0; k < r - 1; k++) {
      if (k == q) continue;
      t.rd[t.nrest] = a.od[k];
      t.ris[t.nrest] = a.is[k];
      t.ros[t.nrest] = a.os[k];
      t.rest_total *= a.od[k];
      t.nrest++;
    }
    t.tiles_last = (a.od[r - 1] + 31) / 32;
    const int64_t tiles_q = (a.od[q] + 31) / 32;
    dim3 grid((unsigned)(t.tiles_last * tiles_q), (unsigned)std::min<int64_t>(t.rest_total, 65535));
    if (narrow)
      permute_kernel_tile<uint32_t><<<grid, dim3(32, 8), 0, c.stream>>>(t);
    else
      permute_kernel_tile<int64_t><<<grid, dim3(32, 8), 0, c.stream>>>(t);
  } else if (a.od[r - 1] >= 32) {
    const int threads = 256;
    const int64_t items = (a.total / a.od[r - 1]) * ((a.od[r - 1] + 127) / 128);
    const int64_t blocks = std::min<int64_t>((items + 7) / 8, 152 * 16);
    if (narrow)
      permute_kernel_rows<uint32_t><<<(unsigned)blocks, threads, 0, c.stream>>>(a);
    else
      permute_kernel_rows<int64_t><<<(unsigned)blocks, threads, 0, c.stream>>>(a);
  } else {
    const int threads = 256;
    const int64_t blocks = std::min<int64_t>((a.total + threads - 1) / threads, 152 * 64);
    if (narrow)
      permute_kernel_elem<uint32_t><<<(unsigned)blocks, threads, 0, c.stream>>>(a);
    else
      permute_kernel_elem<int64_t><<<(unsigned)blocks, threads, 0, c.stream>>>(a);
  }
  count_launch();
  check_launch("permute");
}

// ------------------------------------------------------------------------------------
// Elementwise
// ------------------------------------------------------------------------------------
namespace {
__global__ void axpby_kernel(int64_t n, double alpha, const double* x, double beta, double* y) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    y[i] = combine(alpha, x[i], beta, y + i);
  }
}
__global__ void fill_kernel(int64_t n, double v, double* y) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = v;
}
unsigned grid_for(int64_t n, int threads = 256) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + threads - 1) / threads, 152 * 32));
}
}  // namespace

static void record_flat(Recorder* r, RecordedOp::Kind kind, int64_t n, double alpha, const double* x, double beta,
                        double* y) {
  RecordedOp o;
  o.kind = kind;
  o.rank = 1;
  o.d[0] = n;
  o.si[0] = 1;
  o.so[0] = 1;
  o.in = x, o.out = y, o.alpha = alpha, o.beta = beta;
  r->ops.push_back(o);
}

void axpby(Ctx& c, int64_t n, double alpha, const double* x, double beta, double* y) {
  if (n <= 0) return;
  if (Recorder* r = recorder()) return record_flat(r, RecordedOp::kPermute, n, alpha, x, beta, y);
  axpby_kernel<<<grid_for(n), 256, 0, c.stream>>>(n, alpha, x, beta, y);
  count_launch();
  check_launch("axpby");
}

void fill(Ctx& c, int64_t n, double v, double* y) {
  if (n <= 0) return;
  if (Recorder* r = recorder()) return record_flat(r, RecordedOp::kFill, n, v, nullptr, 0.0, y);
  fill_kernel<<<grid_for(n), 256, 0, c.stream>>>(n, v, y);
  count_launch();
  check_launch("fill");
}

// ------------------------------------------------------------------------------------
// Compensated reductions.  Pass 1: each block writes (sum, compensation) of its
// grid-stride share; pass 2: one block folds the partials.  Fixed grid => deterministic.
// ------------------------------------------------------------------------------------
namespace {
constexpr int RED_BLOCKS = 512, RED_THREADS = 256;

__device__ inline void neumaier(double& s, double& c, double x) {
  const double t = s + x;
  if (fabs(s) >= fabs(x))
    c += (s - t) + x;
  else
    c += (x - t) + s;
  s = t;
}

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

// partial[(vec * gridDim.x + block)] ; x may be indexed per vector via xs
__global__ void dot_pass1(int64_t n, const double* const* xs, const double* x0, const double* y, double* partial) {
  const double* x = xs ? xs[blockIdx.y] : x0;
  double s = 0.0, cc = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    neumaier(s, cc, y ? x[i] * y[i] : x[i]);
  const double tot = block_sum(s + cc);
  if (threadIdx.x == 0) partial[(int64_t)blockIdx.y * gridDim.x + blockIdx.x] = tot;
}

// The DIIS overlaps: one FMA per element per thread (a thread's share is ~n / 131072
// terms), the block and cross-block folds as above.  The compensated per-element form
// costs about six FP64 operations per element and bounded this kernel on GB300's FP64
// pipe; the overlaps only feed the extrapolation coefficients.
__global__ void multidot_pass1(int64_t n, const double* const* xs, const double* y, double* partial) {
  const double* __restrict__ x = xs[blockIdx.y];
  double s0 = 0.0, s1 = 0.0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (; i + stride < n; i += 2 * stride) {
    s0 = fma(x[i], y[i], s0);
    s1 = fma(x[i + stride], y[i + stride], s1);
  }
  if (i < n) s0 = fma(x[i], y[i], s0);
  const double tot = block_sum(s0 + s1);
  if (threadIdx.x == 0) partial[(int64_t)blockIdx.y * gridDim.x + blockIdx.x] = tot;
}

__global__ void sum_pass2(int nparts, const double* partial, double* out) {
  // one block per output
  const double* p = partial + (int64_t)blockIdx.x * nparts;
  double s = 0.0, cc = 0.0;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) neumaier(s, cc, p[i]);
  const double tot = block_sum(s + cc);
  if (threadIdx.x == 0) out[blockIdx.x] = tot;
}
}  // namespace

void dot_async(Ctx& c, int64_t n, const double* x, const double* y, double* d_out) {
  UCC_REQUIRE(!recorder(), UCC_UNSUPPORTED, "not recordable");
  Scratch part(c, sizeof(double) * RED_BLOCKS);
  dot_pass1<<<dim3(RED_BLOCKS, 1), RED_THREADS, 0, c.stream>>>(n, nullptr, x, y, part.d());
  sum_pass2<<<1, RED_THREADS, 0, c.stream>>>(RED_BLOCKS, part.d(), d_out);
  count_launch();
  count_launch();
  check_launch("dot");
}

double dot(Ctx& c, int64_t n, const double* x, const double* y) {
  Scratch out(c, sizeof(double));
  dot_async(c, n, x, y, out.d());
  double h = 0.0;
  UCC_CUDA(cudaMemcpyAsync(&h, out.d(), sizeof(double), cudaMemcpyDeviceToHost, c.stream));
  UCC_CUDA(cudaStreamSynchronize(c.stream));
  return h;
}

void multidot_async(Ctx& c, int nvec, const double* const* d_xs, const double* y, int64_t n, double* d_out) {
  UCC_REQUIRE(!recorder(), UCC_UNSUPPORTED, "not recordable");
  if (nvec <= 0) return;
  Scratch part(c, sizeof(double) * RED_BLOCKS * nvec);
  multidot_pass1<<<dim3(RED_BLOCKS, nvec), RED_THREADS, 0, c.stream>>>(n, d_xs, y, part.d());
  sum_pass2<<<nvec, RED_THREADS, 0, c.stream>>>(RED_BLOCKS, part.d(), d_out);
  count_launch();
  count_launch();
  check_launch("multidot");
}

// ------------------------------------------------------------------------------------
// Amplitude kernels
// ------------------------------------------------------------------------------------
namespace {
template <class I>
__global__ void tau_kernel(int no, int nv, const double* t1, const double* t2, double f1, double* tau, double f2,
                           double* ttau, double g) {
  const I n = (I)no * no * nv * nv, v_ = (I)nv, o_ = (I)no;
  for (I x = (I)blockIdx.x * blockDim.x + threadIdx.x; x < n; x += (I)gridDim.x * blockDim.x) {
    const I b = x % v_;
    I r = x / v_;
    const I a = r % v_;
    r /= v_;
    const I j = r % o_;
    const I i = r / o_;
    const double tt = t1[i * v_ + a] * t1[j * v_ + b];
    const double v = g * t2[x];  // g = 1 or 1/2: exact
    tau[x] = fma(f1, tt, v);
    if (ttau) ttau[x] = fma(f2, tt, v);
  }
}

// Sum of squares of the residuals goes to partial[block] (one FMA per element: all terms
// are non-negative, so the plain sum is accurate to the number of terms a thread folds
// times the unit roundoff).  Index arithmetic in I (32 bits when no*no*nv*nv < 2^31).
template <class I>
__global__ void jacobi_kernel(int no, int nv, const double* d_do, const double* d_dv, double shift, const double* R1,
                              const double* R2, const double* t1o, const double* t2o, double* t1n, double* t2n,
                              double* partial) {
  const I n1 = (I)no * nv, n2 = (I)no * no * nv * nv, v = (I)nv, o = (I)no;
  double s = 0.0;
  for (I x = (I)blockIdx.x * blockDim.x + threadIdx.x; x < n1 + n2; x += (I)gridDim.x * blockDim.x) {
    if (x < n1) {
      const I a = x % v, i = x / v;
      const double r = R1[x];
      s = fma(r, r, s);
      t1n[x] = t1o[x] + r / ((d_do[i] - d_dv[a]) + shift);
    } else {
      const I y = x - n1;
      const I b = y % v;
      I q = y / v;
      const I a = q % v;
      q /= v;
      const I j = q % o;
      const I i = q / o;
      const double r = R2[y];
      s = fma(r, r, s);
      const double D = ((d_do[i] + d_do[j]) - d_dv[a]) - d_dv[b];
      t2n[y] = t2o[y] + r / (D + shift);
    }
  }
  const double tot = block_sum(s);
  if (threadIdx.x == 0) partial[blockIdx.x] = tot;
}

__global__ void lincomb_kernel(int nvec, const double* const* vecs, const double* coef, int64_t n, double* out) {
  for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < n; x += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int p = 0; p < nvec; p++) s += coef[p] * vecs[p][x];
    out[x] = s;
  }
}
}  // namespace

void build_tau(Ctx& c, int no, int nv, const double* t1, const double* t2, double f1, double* tau, double f2,
               double* ttau, double g) {
  UCC_REQUIRE(!recorder(), UCC_UNSUPPORTED, "not recordable");
  UCC_REQUIRE(g == 1.0 || g == 0.5, UCC_BAD_ARGS, "build_tau: t2 scale 1 or 1/2");
  const int64_t n = (int64_t)no * no * nv * nv;
  if (n + 152 * 32 * 256 < ((int64_t)1 << 31))
    tau_kernel<uint32_t><<<grid_for(n), 256, 0, c.stream>>>(no, nv, t1, t2, f1, tau, f2, ttau, g);
  else
    tau_kernel<int64_t><<<grid_for(n), 256, 0, c.stream>>>(no, nv, t1, t2, f1, tau, f2, ttau, g);
  count_launch();
  check_launch("tau");
}

void jacobi_update(Ctx& c, int no, int nv, const double* d_do, const double* d_dv, double shift, const double* R1,
                   const double* R2, const double* t1old, const double* t2old, double* t1new, double* t2new,
                   double* d_sumsq) {
  UCC_REQUIRE(!recorder(), UCC_UNSUPPORTED, "not recordable");
  Scratch part(c, sizeof(double) * RED_BLOCKS);
  const int64_t n = (int64_t)no * nv + (int64_t)no * no * nv * nv;
  if (n + (int64_t)RED_BLOCKS * RED_THREADS < ((int64_t)1 << 31))
    jacobi_kernel<uint32_t><<<RED_BLOCKS, RED_THREADS, 0, c.stream>>>(no, nv, d_do, d_dv, shift, R1, R2, t1old, t2old,
                                                                      t1new, t2new, part.d());
  else
    jacobi_kernel<int64_t><<<RED_BLOCKS, RED_THREADS, 0, c.stream>>>(no, nv, d_do, d_dv, shift, R1, R2, t1old, t2old,
                                                                     t1new, t2new, part.d());
  sum_pass2<<<1, RED_THREADS, 0, c.stream>>>(RED_BLOCKS, part.d(), d_sumsq);
  count_launch();
  count_launch();
  check_launch("jacobi");
}

void lincomb(Ctx& c, int nvec, const double* const* d_vecs, const double* coef, int64_t n, double* out) {
  UCC_REQUIRE(!recorder(), UCC_UNSUPPORTED, "not recordable");
  Scratch dc(c, sizeof(double) * nvec);
  UCC_CUDA(cudaMemcpyAsync(dc.p, coef, sizeof(double) * nvec, cudaMemcpyHostToDevice, c.stream));
  lincomb_kernel<<<grid_for(n), 256, 0, c.stream>>>(nvec, d_vecs, dc.d(), n, out);
  count_launch();
  check_launch("lincomb");
  // the host coefficient array may go out of scope once the copy has been consumed
  UCC_CUDA(cudaStreamSynchronize(c.stream));
}

// ------------------------------------------------------------------------------------
// (T) energy, ccwfn.cc:795-852.  One block per (tuple, a); threads over (b, c) with
// a >= b >= c.  W3 holds nv^3 per tuple as W[a][b][c].
// ------------------------------------------------------------------------------------
namespace {
__global__ void triples_energy_kernel(int no, int nv, const int* tuples, const double* W3, const double* t1,
                                      const double* Voovv, const double* eps, double* partial) {
  const int t = blockIdx.y;
  const int a = blockIdx.x;
  const int i = tuples[3 * t], j = tuples[3 * t + 1], k = tuples[3 * t + 2];
  const int64_t nv2 = (int64_t)nv * nv;
  const double* W = W3 + (int64_t)t * nv2 * nv;
  const double* Vij = Voovv + ((int64_t)i * no + j) * nv2;
  const double* Vik = Voovv + ((int64_t)i * no + k) * nv2;
  const double* Vjk = Voovv + ((int64_t)j * no + k) * nv2;
  const double* t1i = t1 + (int64_t)i * nv;
  const double* t1j = t1 + (int64_t)j * nv;
  const double* t1k = t1 + (int64_t)k * nv;
  const double eijk = eps[i] + eps[j] + eps[k];
  const double fac = 2.0 - (double)((i == j) + (i == k) + (j == k));
  double s = 0.0, cc = 0.0;
  const int npair = (a + 1) * (a + 1);
  for (int q = threadIdx.x; q < npair; q += blockDim.x) {
    const int b = q / (a + 1), c = q % (a + 1);
    if (c > b) continue;
    auto Wv = [&](int x, int y, int z) { return W[(int64_t)x * nv2 + (int64_t)y * nv + z]; };
    auto Vv = [&](int x, int y, int z) {
      const double num = Wv(x, y, z) + Vij[(int64_t)x * nv + y] * t1k[z] + Vik[(int64_t)x * nv + z] * t1j[y] +
                         Vjk[(int64_t)y * nv + z] * t1i[x];
      return num / (1.0 + (double)((x == y) + (x == z) + (y == z)));
    };
    const double wabc = Wv(a, b, c), wacb = Wv(a, c, b), wbac = Wv(b, a, c);
    const double wbca = Wv(b, c, a), wcab = Wv(c, a, b), wcba = Wv(c, b, a);
    const double vabc = Vv(a, b, c), vacb = Vv(a, c, b), vbac = Vv(b, a, c);
    const double vbca = Vv(b, c, a), vcab = Vv(c, a, b), vcba = Vv(c, b, a);
    const double X3 = wabc * vabc + wacb * vacb + wbac * vbac + wbca * vbca + wcab * vcab + wcba * vcba;
    const double Y3 = vabc + vbca + vcab;
    const double Z3 = vacb + vbac + vcba;
    const double denom = eijk - (eps[no + a] + eps[no + b] + eps[no + c]);
    const double e = ((Y3 - 2.0 * Z3) * (wabc + wbca + wcab) + (Z3 - 2.0 * Y3) * (wacb + wbac + wcba) + 3.0 * X3) *
                     fac / denom;
    neumaier(s, cc, e);
  }
  const double tot = block_sum(s + cc);
  if (threadIdx.x == 0) partial[(int64_t)t * nv + a] = tot;
}

// FP32 W3 (mixed form): the per-element V3/X3/Y3/Z3 algebra in FP32, the sums in FP64.
// W3 arrives as up to three partial arrays (one per pair of W3 terms, each written without
// a read-modify-write by its tensor-core GEMM), nparts * part_stride floats apart; their
// sum is formed while staging.  Block (r, t) takes the sorted tile triple r (tiles
// A >= B >= C of edge ET along the virtual axis) of tuple t and stages the six permutation
// tiles W[A][B][C], W[A][C][B], ..., W[C][B][A] in shared memory with coalesced loads, so
// every W3 element is read from memory once; the Voovv blocks and t1 / eps pieces of the
// three tile ranges are staged too.  Roles 0, 1, 2 are the index ranges of a, b, c.
constexpr int ET = 8;
// Threads per block.  The staging and energy loops below run a compile-time number of
// iterations with closed-form local indices of (thread, iteration), which these relations
// make exact: thread t, iteration k covers element t + TNT*k of each loop.
constexpr int TNT = 128;
static_assert(TNT == 2 * ET * ET && (ET * ET * ET) % TNT == 0 && (6 * ET * ET) % TNT == 0, "tile/thread layout");
template <int NP>  // W3 partial arrays (1 or 3), a compile-time count so that all loads are in flight together
__global__ void __launch_bounds__(TNT) triples_energy_f32_tiled_kernel(int no, int nv, const int* __restrict__ tuples,
                                                                      const int* __restrict__ tri, int ntri,
                                                                      const float* __restrict__ W3, int nparts,
                                                                      int64_t part_stride,
                                                                      const double* __restrict__ t1,
                                                                      const double* __restrict__ Voovv,
                                                                      const double* __restrict__ eps, double* partial) {
  __shared__ float Ws[6][ET][ET][ET + 1];
  __shared__ float Vs[3][6][ET][ET + 1];  // Vij, Vik, Vjk on the 6 ordered role pairs
  __shared__ float s1[3][3][ET];          // t1 rows i, j, k on the 3 role ranges
  __shared__ float ev[3][ET];
  const int r = blockIdx.x, t = blockIdx.y;
  const int code = tri[r];
  const int Ra = (code & 1023) * ET, Rb = ((code >> 10) & 1023) * ET, Rc = (code >> 20) * ET;
  auto R0 = [&](int role) { return role == 0 ? Ra : (role == 1 ? Rb : Rc); };  // range start of a role
  const int i = tuples[3 * t], j = tuples[3 * t + 1], k = tuples[3 * t + 2];
  const int64_t nv2 = (int64_t)nv * nv;
  const float* W = W3 + (int64_t)t * nv2 * nv;
  // role order of each permutation tile p, two bits per role: W[x in role 0][y in 1][z in 2]
  // for (0,1,2), (0,2,1), (1,0,2), (1,2,0), (2,0,1), (2,1,0)
  constexpr uint64_t kPerm = 0x24ull | (0x18ull << 6) | (0x21ull << 12) | (0x09ull << 18) | (0x12ull << 24) |
                             (0x06ull << 30);
  // local coordinates of this thread inside an ET^3 tile: (tx + 2 it, ty, tz) at iteration it
  const int tid = threadIdx.x, tx = tid / (ET * ET), ty = (tid / ET) % ET, tz = tid % ET;
#pragma unroll
  for (int it = 0; it < 6 * ET * ET * ET / TNT; it++) {
    const int p = it / (ET * ET * ET / TNT), x = tx + 2 * (it % (ET * ET * ET / TNT));
    const uint64_t code6 = kPerm >> (6 * p);
    const int gx = R0((int)(code6 & 3)) + x, gy = R0((int)((code6 >> 2) & 3)) + ty, gz = R0((int)((code6 >> 4) & 3)) + tz;
    float w = 0.f;
    if (gx < nv && gy < nv && gz < nv) {
      const int64_t o = (int64_t)gx * nv2 + (int64_t)gy * nv + gz;
      w = W[o];
#pragma unroll
      for (int q = 1; q < NP; q++) w += W[o + q * part_stride];
    }
    Ws[p][x][ty][tz] = w;
  }
  auto Vm = [&](int m) {  // Vij, Vik, Vjk
    return Voovv + ((m == 2 ? (int64_t)j : (int64_t)i) * no + (m == 0 ? j : k)) * nv2;
  };
  // element tid + TNT*it: matrix m = it / 3, role pair pid = 2 (it % 3) + tx, row ty, column tz
#pragma unroll
  for (int it = 0; it < 3 * 6 * ET * ET / TNT; it++) {
    const int m = it / 3, u = it % 3, v0 = tx, pid = 2 * u + v0, x = ty, y = tz;
    const int v = v0 < u ? v0 : v0 + 1;  // ordered role pair (u, v), u != v
    const int gx = R0(u) + x, gy = R0(v) + y;
    Vs[m][pid][x][y] = (gx < nv && gy < nv) ? (float)Vm(m)[(int64_t)gx * nv + gy] : 0.f;
  }
  if (threadIdx.x < 3 * 3 * ET) {
    const int m = threadIdx.x / (3 * ET), role = (threadIdx.x / ET) % 3, l = threadIdx.x % ET;
    const int row = m == 0 ? i : (m == 1 ? j : k), g = R0(role) + l;
    s1[m][role][l] = g < nv ? (float)t1[(int64_t)row * nv + g] : 0.f;
  }
  if (threadIdx.x < 3 * ET) {
    const int role = threadIdx.x / ET, l = threadIdx.x % ET, g = R0(role) + l;
    ev[role][l] = g < nv ? (float)eps[no + g] : 0.f;
  }
  __syncthreads();
  const float eijk = (float)(eps[i] + eps[j] + eps[k]);
  const float fac = 2.0f - (float)((i == j) + (i == k) + (j == k));
  const float inv[4] = {1.0f, 0.5f, 0.25f, 0.25f};
  auto pid = [](int u, int v) { return u * 2 + (v > u ? v - 1 : v); };
  // V at one permutation: roles (r0, r1, r2) with local indices (l0, l1, l2), global (g0, g1, g2)
  auto Vp = [&](float w, int r0, int l0, int r1, int l1, int r2, int l2, int g0, int g1, int g2) {
    const float num = w + Vs[0][pid(r0, r1)][l0][l1] * s1[2][r2][l2] + Vs[1][pid(r0, r2)][l0][l2] * s1[1][r1][l1] +
                      Vs[2][pid(r1, r2)][l1][l2] * s1[0][r0][l0];
    return num * inv[(g0 == g1) + (g0 == g2) + (g1 == g2)];
  };
  double s = 0.0;
#pragma unroll
  for (int it = 0; it < ET * ET * ET / TNT; it++) {
    const int la = tx + 2 * it, lb = ty, lc = tz;
    const int a = Ra + la, b = Rb + lb, c = Rc + lc;
    if (a >= nv || b > a || c > b) continue;
    const float wabc = Ws[0][la][lb][lc], wacb = Ws[1][la][lc][lb], wbac = Ws[2][lb][la][lc];
    const float wbca = Ws[3][lb][lc][la], wcab = Ws[4][lc][la][lb], wcba = Ws[5][lc][lb][la];
    const float vabc = Vp(wabc, 0, la, 1, lb, 2, lc, a, b, c), vacb = Vp(wacb, 0, la, 2, lc, 1, lb, a, c, b);
    const float vbac = Vp(wbac, 1, lb, 0, la, 2, lc, b, a, c), vbca = Vp(wbca, 1, lb, 2, lc, 0, la, b, c, a);
    const float vcab = Vp(wcab, 2, lc, 0, la, 1, lb, c, a, b), vcba = Vp(wcba, 2, lc, 1, lb, 0, la, c, b, a);
    const float X3 = wabc * vabc + wacb * vacb + wbac * vbac + wbca * vbca + wcab * vcab + wcba * vcba;
    const float Y3 = vabc + vbca + vcab;
    const float Z3 = vacb + vbac + vcba;
    const float denom = eijk - (ev[0][la] + ev[1][lb] + ev[2][lc]);
    const float e = ((Y3 - 2.0f * Z3) * (wabc + wbca + wcab) + (Z3 - 2.0f * Y3) * (wacb + wbac + wcba) + 3.0f * X3) *
                    fac / denom;
    s += (double)e;
  }
  const double tot = block_sum(s);
  if (threadIdx.x == 0) partial[(int64_t)t * ntri + r] = tot;
}
// Pipelined form of the FP32 energy for nv % 4 == 0, W3 in the blocked layout of
// w3_block_offset: a persistent block walks items (tuple t, tile triple r), item =
// t * ntri + r, in steps of the grid.  While it computes item n from one shared-memory
// stage, every input of item n + G lands in the other stage by 16-byte cp.async (no
// registers held): the 18 W3 tiles (6 index orders x 3 partial arrays), each one
// contiguous 2 KB block, and FP32 copies of the Voovv blocks, t1 rows and virtual orbital
// energies (made once per (T) call; rows outside nv zero-filled).  The partial arrays stay
// separate in shared memory and are added where an element is read.  The blocks' swizzle
// and the threads' bit-permuted order over a tile make every shared-memory read of the
// energy loop conflict-free (one wavefront per warp read).  No FP64 instruction runs per
// element (the FP64 pipe of this part is narrow): the item's sum is formed in FP32 per
// warp and in FP64 across the warps.
constexpr int EP_THREADS = 256;
constexpr int EP_WTILE = ET * ET * ET;  // floats per tile (one block)
template <int NP>
struct EpStage {
  float W[NP][6][EP_WTILE];
  float V[3][6][ET * ET];  // Vij, Vik, Vjk on the 6 ordered role pairs, rows of 8
  float t1[3][3][ET];      // t1 rows i, j, k on the 3 role ranges
  float ev[3][ET];         // virtual orbital energies on the 3 role ranges
  double red[EP_THREADS / 32];
};
static_assert(sizeof(EpStage<3>) % 16 == 0 && sizeof(EpStage<1>) % 16 == 0, "16-byte stage alignment");
static_assert(offsetof(EpStage<3>, V) % 16 == 0 && offsetof(EpStage<3>, t1) % 16 == 0 &&
                  offsetof(EpStage<3>, ev) % 16 == 0 && offsetof(EpStage<1>, V) % 16 == 0 &&
                  offsetof(EpStage<1>, t1) % 16 == 0 && offsetof(EpStage<1>, ev) % 16 == 0,
              "16-byte cp.async destinations");
// the 288 + 18 + 6 chunks of the Voovv blocks, t1 rows and energies of one item
constexpr int EP_SIDE_CHUNKS = 3 * 6 * ET * 2 + 3 * 3 * 2 + 3 * 2;

__device__ __forceinline__ void ep_cp16(void* dst, const void* src, bool valid) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(src), "r"(valid ? 16 : 0) : "memory");
}
__device__ __forceinline__ void ep_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void ep_wait1() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

// FP32 copies for the pipelined energy: Voovv [no][no][nv][nv] at 0, t1 [no][nv] at off_t1,
// the virtual energies [nv] at off_ev, the occupied ones [no] at off_eo
__global__ void triples_f32_inputs_kernel(int no, int nv, const double* __restrict__ t1,
                                          const double* __restrict__ Voovv, const double* __restrict__ eps,
                                          float* __restrict__ out, int64_t off_t1, int64_t off_ev, int64_t off_eo) {
  const int64_t nV = (int64_t)no * no * nv * nv, nT = (int64_t)no * nv, n = nV + nT + nv + no;
  for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < n; x += (int64_t)gridDim.x * blockDim.x) {
    if (x < nV)
      out[x] = (float)Voovv[x];
    else if (x < nV + nT)
      out[off_t1 + (x - nV)] = (float)t1[x - nV];
    else if (x < nV + nT + nv)
      out[off_ev + (x - nV - nT)] = (float)eps[no + (x - nV - nT)];
    else
      out[off_eo + (x - nV - nT - nv)] = (float)eps[x - nV - nT - nv];
  }
}

template <int NP>
__global__ void __launch_bounds__(EP_THREADS, 2)
    triples_energy_pipe_kernel(int no, int nv, const int* __restrict__ tuples, const int* __restrict__ tri, int ntri,
                               int64_t nitems, const float* __restrict__ W3, int64_t part_stride, int T,
                               const float* __restrict__ f32, int64_t off_t1, int64_t off_ev, int64_t off_eo,
                               double* __restrict__ partial) {
  extern __shared__ __align__(16) unsigned char ep_smem[];
  EpStage<NP>* st = reinterpret_cast<EpStage<NP>*>(ep_smem);
  const int tid = threadIdx.x;
  const int64_t nv2 = (int64_t)nv * nv, per = (int64_t)T * T * T * EP_WTILE;  // W3 floats per tuple
  const float* Vf = f32;
  const float* t1f = f32 + off_t1;
  const float* evf = f32 + off_ev;
  const float* eof = f32 + off_eo;
  constexpr uint64_t kPerm = 0x24ull | (0x18ull << 6) | (0x21ull << 12) | (0x09ull << 18) | (0x12ull << 24) |
                             (0x06ull << 30);
  // this thread's W3 chunk: 16 bytes at 4 c16 floats into the blocks of tiles 3 h .. 3 h + 2
  const int c16 = tid & 127, h = tid >> 7;
  auto ranges = [&](int64_t item, int& Ra, int& Rb, int& Rc, int& t) {
    t = (int)(item / ntri);
    const int code = tri[item - (int64_t)t * ntri];
    Ra = (code & 1023) * ET;
    Rb = ((code >> 10) & 1023) * ET;
    Rc = (code >> 20) * ET;
  };
  auto issue = [&](int64_t item, int s) {
    int Ra, Rb, Rc, t;
    ranges(item, Ra, Rb, Rc, t);
    auto R0 = [&](int role) { return role == 0 ? Ra : (role == 1 ? Rb : Rc); };
    const float* Wt = W3 + (int64_t)t * per;
#pragma unroll
    for (int pp = 0; pp < 3; pp++) {
      const int p = 3 * h + pp;
      const uint64_t c6 = kPerm >> (6 * p);
      const int64_t X = R0((int)(c6 & 3)) / ET, Y = R0((int)((c6 >> 2) & 3)) / ET, Z = R0((int)((c6 >> 4) & 3)) / ET;
      const float* src = Wt + ((X * T + Y) * T + Z) * EP_WTILE + 4 * c16;
      float* dst = &st[s].W[0][p][4 * c16];
#pragma unroll
      for (int q = 0; q < NP; q++) ep_cp16(dst + q * 6 * EP_WTILE, src + q * part_stride, true);
    }
    const int i = tuples[3 * t], j = tuples[3 * t + 1], k = tuples[3 * t + 2];
    for (int c = tid; c < EP_SIDE_CHUNKS; c += EP_THREADS) {
      const float* src;
      float* dst;
      bool ok;
      if (c < 288) {  // Voovv block m on role pair pid, row x, half hf
        const int m = c / 96, pid = (c / 16) % 6, x = (c / 2) % 8, hf = c % 2;
        const int u = pid / 2, v0 = pid % 2, v = v0 < u ? v0 : v0 + 1;
        const int gx = R0(u) + x, gy = R0(v) + 4 * hf;
        ok = gx < nv && gy < nv;
        src = Vf + ((m == 2 ? (int64_t)j : (int64_t)i) * no + (m == 0 ? j : k)) * nv2 + (ok ? (int64_t)gx * nv + gy : 0);
        dst = &st[s].V[m][pid][x * ET + 4 * hf];
      } else if (c < 306) {  // t1 row m on role range
        const int d = c - 288, m = d / 6, role = (d / 2) % 3, hf = d % 2;
        const int row = m == 0 ? i : (m == 1 ? j : k), g = R0(role) + 4 * hf;
        ok = g < nv;
        src = t1f + (int64_t)row * nv + (ok ? g : 0);
        dst = &st[s].t1[m][role][4 * hf];
      } else {  // virtual energies on role range
        const int d = c - 306, role = d / 2, hf = d % 2, g = R0(role) + 4 * hf;
        ok = g < nv;
        src = evf + (ok ? g : 0);
        dst = &st[s].ev[role][4 * hf];
      }
      ep_cp16(dst, src, ok);
    }
  };

  const int64_t G = gridDim.x;
  int64_t item = blockIdx.x;
  if (item >= nitems) return;
  issue(item, 0);
  ep_commit();
  for (int s = 0; item < nitems; item += G, s ^= 1) {
    const int64_t nxt = item + G;
    if (nxt < nitems) issue(nxt, s ^ 1);
    ep_commit();  // an empty group on the last item keeps the count of one group in flight
    ep_wait1();
    __syncthreads();
    int Ra, Rb, Rc, t;
    ranges(item, Ra, Rb, Rc, t);
    const int i = tuples[3 * t], j = tuples[3 * t + 1], k = tuples[3 * t + 2];
    const float eijk = eof[i] + eof[j] + eof[k];
    const float fac = 2.0f - (float)((i == j) + (i == k) + (j == k));
    const EpStage<NP>& S = st[s];
    auto W = [&](int p, int x, int y, int z) {
      const int o = 64 * x + 8 * (y ^ x) + (z ^ ((5 * y) & 7));  // w3_block_offset within a block
      float w = S.W[0][p][o];
#pragma unroll
      for (int q = 1; q < NP; q++) w += S.W[q][p][o];
      return w;
    };
    auto pid = [](int u, int v) { return u * 2 + (v > u ? v - 1 : v); };
    auto Vp = [&](float w, int r0, int l0, int r1, int l1, int r2, int l2) {
      return w + S.V[0][pid(r0, r1)][l0 * ET + l1] * S.t1[2][r2][l2] +
             S.V[1][pid(r0, r2)][l0 * ET + l2] * S.t1[1][r1][l1] + S.V[2][pid(r1, r2)][l1 * ET + l2] * S.t1[0][r0][l0];
    };
    float sf = 0.f;
#pragma unroll
    for (int it = 0; it < ET * ET * ET / EP_THREADS; it++) {
      // the order over the tile that makes the six permuted reads conflict-free
      const int la = (tid & 1) | (((tid >> 6) & 1) << 1) | (((tid >> 7) & 1) << 2);
      const int lb = ((tid >> 2) & 1) | (((tid >> 1) & 1) << 1) | (((tid >> 5) & 1) << 2);
      const int lc = ((tid >> 4) & 1) | (((tid >> 3) & 1) << 1) | ((it & 1) << 2);
      const int a = Ra + la, b = Rb + lb, c = Rc + lc;
      if (a >= nv || b > a || c > b) continue;
      const float wabc = W(0, la, lb, lc), wacb = W(1, la, lc, lb), wbac = W(2, lb, la, lc);
      const float wbca = W(3, lb, lc, la), wcab = W(4, lc, la, lb), wcba = W(5, lc, lb, la);
      const float vabc = Vp(wabc, 0, la, 1, lb, 2, lc), vacb = Vp(wacb, 0, la, 2, lc, 1, lb);
      const float vbac = Vp(wbac, 1, lb, 0, la, 2, lc), vbca = Vp(wbca, 1, lb, 2, lc, 0, la);
      const float vcab = Vp(wcab, 2, lc, 0, la, 1, lb), vcba = Vp(wcba, 2, lc, 1, lb, 0, la);
      const float X3 = wabc * vabc + wacb * vacb + wbac * vbac + wbca * vbca + wcab * vcab + wcba * vcba;
      const float Y3 = vabc + vbca + vcab;
      const float Z3 = vacb + vbac + vcba;
      // V = numerator / (1 + number of equal index pairs), the same count for all six orders
      const int neq = (a == b) + (a == c) + (b == c);
      const float deg = neq == 0 ? 1.0f : (neq == 1 ? 0.5f : 0.25f);
      const float denom = eijk - (S.ev[0][la] + S.ev[1][lb] + S.ev[2][lc]);
      sf += ((Y3 - 2.0f * Z3) * (wabc + wbca + wcab) + (Z3 - 2.0f * Y3) * (wacb + wbac + wcba) + 3.0f * X3) * deg *
            fac / denom;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sf += __shfl_xor_sync(0xffffffffu, sf, o);
    if ((tid & 31) == 0) st[s].red[tid >> 5] = (double)sf;
    __syncthreads();
    if (tid == 0) {
      double tot = 0.0;
#pragma unroll
      for (int w = 0; w < EP_THREADS / 32; w++) tot += S.red[w];
      partial[item] = tot;
    }
  }
}

}  // namespace

int64_t triples_f32_partials(int nv) {
  const int64_t T = (nv + ET - 1) / ET;
  return T * (T + 1) * (T + 2) / 6;
}

// ------------------------------------------------------------------------------------
// Pair-symmetric particle ladder.  Pairs p <= q are numbered q(q+1)/2 + p, strict pairs
// p < q are numbered q(q-1)/2 + p.
// ------------------------------------------------------------------------------------
namespace {
__device__ __forceinline__ void pair_le(int64_t P, int& p, int& q) {
  int j = (int)((sqrt(8.0 * (double)P + 1.0) - 1.0) * 0.5);
  while ((int64_t)(j + 1) * (j + 2) / 2 <= P) j++;
  while ((int64_t)j * (j + 1) / 2 > P) j--;
  q = j;
  p = (int)(P - (int64_t)j * (j + 1) / 2);
}
__device__ __forceinline__ void pair_lt(int64_t Q, int& p, int& q) {
  int j = (int)((sqrt(8.0 * (double)Q + 1.0) + 1.0) * 0.5);
  while ((int64_t)j * (j + 1) / 2 <= Q) j++;
  while (j > 1 && (int64_t)(j - 1) * j / 2 > Q) j--;
  q = j;
  p = (int)(Q - (int64_t)j * (j - 1) / 2);
}

// the operator W_abef of a packed ladder, from a stored [nv]^4 block H:
//   mode 0: H[a][b][e][f]                          (<ab|ef>, pair-symmetric itself)
//   mode 1: H[e][f][a][b] + H[f][e][b][a]          (sum_ef Z_ijef H_efab of a Z + Z(ji,ba) residual)
//   mode 2: H[a][b][e][f] + H[b][a][f][e]          (sum_ef Z_ijef H_abef of a Z + Z(ji,ba) residual)
__device__ __forceinline__ double ladder_op(const double* H, int nv, int mode, int a, int b, int e, int f) {
  auto at = [&](int p, int q, int r, int s) { return H[(((int64_t)p * nv + q) * nv + r) * nv + s]; };
  if (mode == 1) return at(e, f, a, b) + at(f, e, b, a);
  if (mode == 2) return at(a, b, e, f) + at(b, a, f, e);
  return at(a, b, e, f);
}

// Vp[ab][ef] = W_abef + W_abfe (e < f), W_abee (e == f), a <= b;  Vm[ab][ef] = W_abef - W_abfe, a < b, e < f
__global__ void pack_vvvv_kernel(int nv, int mode, const double* __restrict__ H, double* Vp, double* Vm) {
  const int64_t np = (int64_t)nv * (nv + 1) / 2, nm = (int64_t)nv * (nv - 1) / 2;
  for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < np * np + nm * nm;
       x += (int64_t)gridDim.x * blockDim.x) {
    int a, b, e, f;
    if (x < np * np) {
      pair_le(x / np, a, b);
      pair_le(x % np, e, f);
      Vp[x] = e == f ? ladder_op(H, nv, mode, a, b, e, e)
                     : ladder_op(H, nv, mode, a, b, e, f) + ladder_op(H, nv, mode, a, b, f, e);
    } else {
      const int64_t y = x - np * np;
      pair_lt(y / nm, a, b);
      pair_lt(y % nm, e, f);
      Vm[y] = ladder_op(H, nv, mode, a, b, e, f) - ladder_op(H, nv, mode, a, b, f, e);
    }
  }
}

// Tp[ij][ef] = (tau_ijef + tau_ijfe)/2 (e < f), tau_ijee (e == f), i <= j;  Tm = (tau_ijef - tau_ijfe)/2, i < j, e < f
__global__ void pack_tau_kernel(int no, int nv, const double* __restrict__ tau, double* Tp, double* Tm) {
  const int64_t op = (int64_t)no * (no + 1) / 2, om = (int64_t)no * (no - 1) / 2;
  const int64_t vp = (int64_t)nv * (nv + 1) / 2, vm = (int64_t)nv * (nv - 1) / 2;
  const int64_t nv2 = (int64_t)nv * nv;
  for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < op * vp + om * vm;
       x += (int64_t)gridDim.x * blockDim.x) {
    int i, j, e, f;
    if (x < op * vp) {
      pair_le(x / vp, i, j);
      pair_le(x % vp, e, f);
      const double* t = tau + ((int64_t)i * no + j) * nv2;
      Tp[x] = e == f ? t[(int64_t)e * nv + e] : 0.5 * (t[(int64_t)e * nv + f] + t[(int64_t)f * nv + e]);
    } else {
      const int64_t y = x - op * vp;
      pair_lt(y / vm, i, j);
      pair_lt(y % vm, e, f);
      const double* t = tau + ((int64_t)i * no + j) * nv2;
      Tm[y] = 0.5 * (t[(int64_t)e * nv + f] - t[(int64_t)f * nv + e]);
    }
  }
}

// Tiled form of the two packings for a source whose (x, y) slice is one contiguous
// nv x nv block t = src + (x * nx + y) * nv^2 (tau: x, y = i, j; <ab|ef>: x, y = a, b):
//   P[x<=y][e<=f] = h (t[e][f] + t[f][e]) (e < f), t[e][e] (e == f)
//   M[x<y][e<f]   = h (t[e][f] - t[f][e])
// with h = 1/2 (tau) or 1 (<ab|ef>).  Block (tile pair, x<=y pair) stages the 32 x 32 tile
// (E, F) of t and the transposed tile (F, E) in shared memory, both read along rows, and
// writes the packed elements along e (contiguous in both outputs for fixed f); the pair
// indices come from a per-block decode instead of an FP64 square root per element (GB300's
// FP64 pipe made the per-element form run at 0.44-0.77 TB/s).
__global__ void pack_pairs_tiled_kernel(int nx, int nv, double h, const double* __restrict__ src, double* P,
                                        double* M) {
  __shared__ double A[32][33], B[32][33];
  const int64_t vp = (int64_t)nv * (nv + 1) / 2, vm = (int64_t)nv * (nv - 1) / 2;
  // tile pair (E <= F) from blockIdx.x: F (F + 1) / 2 + E
  int F = 0;
  while ((F + 1) * (F + 2) / 2 <= (int)blockIdx.x) F++;
  const int E = (int)blockIdx.x - F * (F + 1) / 2;
  // row pair (x <= y) from blockIdx.y: y (y + 1) / 2 + x
  const int64_t R = blockIdx.y;
  int y = (int)((sqrtf(8.0f * (float)R + 1.0f) - 1.0f) * 0.5f);
  while ((int64_t)(y + 1) * (y + 2) / 2 <= R) y++;
  while ((int64_t)y * (y + 1) / 2 > R) y--;
  const int x = (int)(R - (int64_t)y * (y + 1) / 2);
  const double* t = src + ((int64_t)x * nx + y) * (int64_t)nv * nv;
  const int e0 = E * 32, f0 = F * 32, tx = threadIdx.x, ty = threadIdx.y;
  for (int r = ty; r < 32; r += 8) {
    const int ea = e0 + r, fa = f0 + tx;  // A[r][tx] = t[e0 + r][f0 + tx]
    A[r][tx] = (ea < nv && fa < nv) ? t[(int64_t)ea * nv + fa] : 0.0;
    const int fb = f0 + r, eb = e0 + tx;  // B[tx][r] = t[f0 + r][e0 + tx]: B[e][f] = t[f][e]
    B[tx][r] = (fb < nv && eb < nv) ? t[(int64_t)fb * nv + eb] : 0.0;
  }
  __syncthreads();
  double* Prow = P + R * vp;
  double* Mrow = x < y ? M + ((int64_t)y * (y - 1) / 2 + x) * vm : nullptr;
  for (int c = ty; c < 32; c += 8) {  // f = f0 + c, e = e0 + tx along the lanes
    const int f = f0 + c, e = e0 + tx;
    if (f >= nv || e > f) continue;
    const double a = A[tx][c], b = B[tx][c];
    Prow[(int64_t)f * (f + 1) / 2 + e] = e == f ? a : h * (a + b);
    if (Mrow && e < f) Mrow[(int64_t)f * (f - 1) / 2 + e] = h * (a - b);
  }
}

// R2[ijab] += S[(i,j) sorted][(a,b) sorted] + sign * A[...], sign = (-1)^[i>j] (-1)^[a>b],
// A = 0 on i == j or a == b
template <class I>
__global__ void unpack_ladder_kernel(int no, int nv, double alpha, const double* __restrict__ S,
                                     const double* __restrict__ A, double* R2) {
  const I n = (I)no * no * nv * nv, v_ = (I)nv, o_ = (I)no;
  const I vp = v_ * (v_ + 1) / 2, vm = v_ * (v_ - 1) / 2;
  for (I x = (I)blockIdx.x * blockDim.x + threadIdx.x; x < n; x += (I)gridDim.x * blockDim.x) {
    const I b = x % v_;
    I r = x / v_;
    const I a = r % v_;
    r /= v_;
    const I j = r % o_, i = r / o_;
    const I i0 = i < j ? i : j, j0 = i < j ? j : i, a0 = a < b ? a : b, b0 = a < b ? b : a;
    double v = S[(int64_t)(j0 * (j0 + 1) / 2 + i0) * vp + b0 * (b0 + 1) / 2 + a0];
    if (i != j && a != b) {
      const double am = A[(int64_t)(j0 * (j0 - 1) / 2 + i0) * vm + b0 * (b0 - 1) / 2 + a0];
      v += ((i > j) != (a > b)) ? -am : am;
    }
    R2[x] = combine(alpha, v, 1.0, R2 + x);
  }
}
}  // namespace

void pack_vvvv(Ctx& c, int nv, int mode, const double* H, double* Vp, double* Vm) {
  UCC_REQUIRE(!recorder(), UCC_UNSUPPORTED, "not recordable");
  const int64_t np = (int64_t)nv * (nv + 1) / 2, nm = (int64_t)nv * (nv - 1) / 2;
  const int nt = (nv + 31) / 32;
  if (mode == 0 && np <= 65535) {  // <ab|ef>: the (a, b) slice is one contiguous block
    pack_pairs_tiled_kernel<<<dim3((unsigned)(nt * (nt + 1) / 2), (unsigned)np), dim3(32, 8), 0, c.stream>>>(
        nv, nv, 1.0, H, Vp, Vm);
    count_launch();
    check_launch("pack_vvvv");
    return;
  }
  pack_vvvv_kernel<<<grid_for(np * np + nm * nm), 256, 0, c.stream>>>(nv, mode, H, Vp, Vm);
  count_launch();
  check_launch("pack_vvvv");
}

void pack_tau(Ctx& c, int no, int nv, const double* tau, double* Tp, double* Tm) {
  UCC_REQUIRE(!recorder(), UCC_UNSUPPORTED, "not recordable");
  const int64_t op = (int64_t)no * (no + 1) / 2;
  const int nt = (nv + 31) / 32;
  if (op <= 65535) {
    pack_pairs_tiled_kernel<<<dim3((unsigned)(nt * (nt + 1) / 2), (unsigned)op), dim3(32, 8), 0, c.stream>>>(
        no, nv, 0.5, tau, Tp, Tm);
    count_launch();
    check_launch("pack_tau");
    return;
  }
  const int64_t n = (int64_t)no * (no + 1) / 2 * nv * (nv + 1) / 2 + (int64_t)no * (no - 1) / 2 * nv * (nv - 1) / 2;
  pack_tau_kernel<<<grid_for(n), 256, 0, c.stream>>>(no, nv, tau, Tp, Tm);
  count_launch();
  check_launch("pack_tau");
}

void unpack_ladder(Ctx& c, int no, int nv, double alpha, const double* S, const double* A, double* R2) {
  UCC_REQUIRE(!recorder(), UCC_UNSUPPORTED, "not recordable");
  const int64_t n = (int64_t)no * no * nv * nv;
  if (n + 152 * 32 * 256 < ((int64_t)1 << 31))
    unpack_ladder_kernel<uint32_t><<<grid_for(n), 256, 0, c.stream>>>(no, nv, alpha, S, A, R2);
  else
    unpack_ladder_kernel<int64_t><<<grid_for(n), 256, 0, c.stream>>>(no, nv, alpha, S, A, R2);
  count_launch();
  check_launch("unpack_ladder");
}

TriplesF32Layout triples_f32_layout(int no, int nv) {
  auto up4 = [](int64_t n) { return (n + 3) / 4 * 4; };
  TriplesF32Layout L;
  L.off_t1 = up4((int64_t)no * no * nv * nv);
  L.off_ev = L.off_t1 + up4((int64_t)no * nv);
  L.off_eo = L.off_ev + up4(nv);
  L.total = L.off_eo + up4(no);
  return L;
}

void triples_f32_inputs(Ctx& c, int no, int nv, const double* t1, const double* Voovv, const double* eps,
                        float* out) {
  const TriplesF32Layout L = triples_f32_layout(no, nv);
  const int64_t n = (int64_t)no * no * nv * nv + (int64_t)no * nv + nv + no;
  triples_f32_inputs_kernel<<<grid_for(n), 256, 0, c.stream>>>(no, nv, t1, Voovv, eps, out, L.off_t1, L.off_ev,
                                                              L.off_eo);
  count_launch();
  check_launch("triples_f32_inputs");
}

void triples_energy_f32(Ctx& c, int no, int nv, int ntuple, const int* d_tuples, const float* W3, int nparts,
                        int64_t part_stride, const double* t1, const double* Voovv, const double* eps,
                        double* d_partial, const float* f32in) {
  UCC_REQUIRE(ntuple <= 65535, UCC_BAD_ARGS, "triples_energy: too many tuples per batch");
  const int T = (nv + ET - 1) / ET;
  UCC_REQUIRE(T <= 1024, UCC_BAD_ARGS, "triples_energy: too many virtual tiles");
  std::vector<int> tri;
  for (int A = 0; A < T; A++)
    for (int B = 0; B <= A; B++)
      for (int C = 0; C <= B; C++) tri.push_back(A | (B << 10) | (C << 20));
  Scratch dtri(c, sizeof(int) * tri.size());
  UCC_CUDA(cudaMemcpyAsync(dtri.p, tri.data(), sizeof(int) * tri.size(), cudaMemcpyHostToDevice, c.stream));
  UCC_REQUIRE(nparts == 1 || nparts == 3, UCC_BAD_ARGS, "triples_energy: 1 or 3 W3 partial arrays");
  if (f32in) {  // W3 in the blocked layout
    UCC_REQUIRE(nv % 4 == 0 && part_stride % 4 == 0 && reinterpret_cast<uintptr_t>(W3) % 16 == 0 &&
                    reinterpret_cast<uintptr_t>(f32in) % 16 == 0,
                UCC_BAD_ARGS, "triples_energy: the blocked W3 form needs nv % 4 == 0 and 16-byte aligned arrays");
    const TriplesF32Layout L = triples_f32_layout(no, nv);
    // persistent blocks, as many as fit (two per SM by their two 42 KB stages)
    static thread_local int sms[64] = {0}, per_sm[2][64] = {{0}};
    const int dev = c.device & 63, np = nparts == 3 ? 0 : 1;
    const size_t smem = nparts == 3 ? 2 * sizeof(EpStage<3>) : 2 * sizeof(EpStage<1>);
    if (!sms[dev]) UCC_CUDA(cudaDeviceGetAttribute(&sms[dev], cudaDevAttrMultiProcessorCount, c.device));
    if (!per_sm[np][dev]) {
      if (nparts == 3) {
        UCC_CUDA(cudaFuncSetAttribute(triples_energy_pipe_kernel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
        UCC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm[np][dev], triples_energy_pipe_kernel<3>,
                                                               EP_THREADS, smem));
      } else {
        UCC_CUDA(cudaFuncSetAttribute(triples_energy_pipe_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
        UCC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm[np][dev], triples_energy_pipe_kernel<1>,
                                                               EP_THREADS, smem));
      }
      per_sm[np][dev] = std::max(1, per_sm[np][dev]);
    }
    const int64_t nitems = (int64_t)ntuple * (int64_t)tri.size();
    const unsigned grid = (unsigned)std::min<int64_t>(nitems, (int64_t)sms[dev] * per_sm[np][dev]);
    if (nparts == 3)
      triples_energy_pipe_kernel<3><<<grid, EP_THREADS, smem, c.stream>>>(
          no, nv, d_tuples, static_cast<const int*>(dtri.p), (int)tri.size(), nitems, W3, part_stride, T, f32in,
          L.off_t1, L.off_ev, L.off_eo, d_partial);
    else
      triples_energy_pipe_kernel<1><<<grid, EP_THREADS, smem, c.stream>>>(
          no, nv, d_tuples, static_cast<const int*>(dtri.p), (int)tri.size(), nitems, W3, part_stride, T, f32in,
          L.off_t1, L.off_ev, L.off_eo, d_partial);
    count_launch();
    check_launch("triples_energy_f32");
    UCC_CUDA(cudaStreamSynchronize(c.stream));  // the tile list is freed on return
    return;
  }
  dim3 grid((unsigned)tri.size(), (unsigned)ntuple);
  if (nparts == 3)
    triples_energy_f32_tiled_kernel<3><<<grid, TNT, 0, c.stream>>>(
        no, nv, d_tuples, static_cast<const int*>(dtri.p), (int)tri.size(), W3, nparts, part_stride, t1, Voovv, eps,
        d_partial);
  else
    triples_energy_f32_tiled_kernel<1><<<grid, TNT, 0, c.stream>>>(
        no, nv, d_tuples, static_cast<const int*>(dtri.p), (int)tri.size(), W3, nparts, part_stride, t1, Voovv, eps,
        d_partial);
  count_launch();
  check_launch("triples_energy_f32");
  UCC_CUDA(cudaStreamSynchronize(c.stream));  // the tile list is freed on return
}

void triples_energy(Ctx& c, int no, int nv, int ntuple, const int* d_tuples, const double* W3, const double* t1,
                    const double* Voovv, const double* eps, double* d_partial) {
  UCC_REQUIRE(ntuple <= 65535, UCC_BAD_ARGS, "triples_energy: too many tuples per batch");
  dim3 grid((unsigned)nv, (unsigned)ntuple);
  triples_energy_kernel<<<grid, 256, 0, c.stream>>>(no, nv, d_tuples, W3, t1, Voovv, eps, d_partial);
  count_launch();
  check_launch("triples_energy");
}


// ------------------------------------------------------------------------------------
// GEMV: y[n] = alpha * sum_k x[k] * A[k*sk + n*sn] + beta * y[n*sy]  (contractions whose
// free side is a single vector; a 64x64 GEMM tile would waste 63/64 of its work)
// ------------------------------------------------------------------------------------
namespace {
// Block (bx, z) folds the k range [z*kc, min(K, (z+1)*kc)) of 32 consecutive n; with one
// K chunk it writes y, otherwise the chunk sums go to P[z][n] for gemv_reduce (fixed order).
__global__ void gemv_ncontig(int64_t N, int64_t K, int64_t kc, double alpha, const double* x, int64_t sx,
                             const double* A, int64_t sk, int64_t sn, double beta, double* y, int64_t sy, double* P) {
  // blockDim = (32, 8): threadIdx.x over n (coalesced when sn == 1), threadIdx.y over k
  __shared__ double red[8][33];
  const int64_t n = (int64_t)blockIdx.x * 32 + threadIdx.x;
  const int64_t k0 = (int64_t)blockIdx.y * kc, k1 = k0 + kc < K ? k0 + kc : K;
  double s = 0.0;
  if (n < N)
    for (int64_t k = k0 + threadIdx.y; k < k1; k += 8) s = fma(x[k * sx], A[k * sk + n * sn], s);
  red[threadIdx.y][threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.y == 0 && n < N) {
    double t = 0.0;
    for (int r = 0; r < 8; r++) t += red[r][threadIdx.x];
    if (P)
      P[(int64_t)blockIdx.y * N + n] = t;
    else
      y[n * sy] = combine(alpha, t, beta, y + n * sy);
  }
}
__global__ void gemv_reduce(int64_t N, int nz, const double* __restrict__ P, double alpha, double beta, double* y,
                            int64_t sy) {
  for (int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; n < N; n += (int64_t)gridDim.x * blockDim.x) {
    double t = P[n];
    for (int z = 1; z < nz; z++) t += P[(int64_t)z * N + n];
    y[n * sy] = combine(alpha, t, beta, y + n * sy);
  }
}
__global__ void gemv_kcontig(int64_t N, int64_t K, double alpha, const double* x, int64_t sx, const double* A,
                             int64_t sk, int64_t sn, double beta, double* y, int64_t sy) {
  // one warp per n, lanes over k (coalesced when sk == 1)
  const int64_t n = (int64_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const int lane = threadIdx.x % 32;
  if (n >= N) return;
  double s = 0.0;
  for (int64_t k = lane; k < K; k += 32) s = fma(x[k * sx], A[k * sk + n * sn], s);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if (lane == 0) {
    double* op = y + n * sy;
    *op = (beta == 0.0) ? alpha * s : fma(beta, *op, alpha * s);
  }
}
}  // namespace

void dgemv_strided(Ctx& c, int64_t N, int64_t K, double alpha, const double* x, int64_t sx, const double* A,
                   int64_t sk, int64_t sn, double beta, double* y, int64_t sy) {
  if (N <= 0) return;
  if (Recorder* r = recorder()) {  // a GEMM with one row
    RecordedOp o;
    o.kind = RecordedOp::kGemm;
    o.M = 1, o.N = N, o.K = K, o.sAm = 0, o.sAk = sx, o.sBk = sk, o.sBn = sn, o.sCm = 0, o.sCn = sy;
    o.A = x, o.B = A, o.C = y, o.alpha = alpha, o.beta = beta;
    r->ops.push_back(o);
    return;
  }
  if (sk == 1 && sn != 1) {
    const int wpb = 8;
    gemv_kcontig<<<(unsigned)((N + wpb - 1) / wpb), 32 * wpb, 0, c.stream>>>(N, K, alpha, x, sx, A, sk, sn, beta, y,
                                                                            sy);
  } else {
    // enough blocks for ~4 per SM: split K into chunks of at least 256 when the n tiles are few
    const int64_t nb = (N + 31) / 32;
    int64_t nz = std::min<int64_t>((4 * 152 + nb - 1) / nb, K / 256);
    nz = std::max<int64_t>(1, std::min<int64_t>(nz, 256));
    const int64_t kc = nz > 1 ? (K + nz - 1) / nz : K;
    if (nz > 1) nz = (K + kc - 1) / kc;
    if (nz <= 1) {
      gemv_ncontig<<<dim3((unsigned)nb, 1), dim3(32, 8), 0, c.stream>>>(N, K, K, alpha, x, sx, A, sk, sn, beta, y, sy,
                                                                         nullptr);
    } else {
      Scratch part(c, sizeof(double) * nz * N);
      gemv_ncontig<<<dim3((unsigned)nb, (unsigned)nz), dim3(32, 8), 0, c.stream>>>(N, K, kc, alpha, x, sx, A, sk, sn,
                                                                                   beta, y, sy, part.d());
      gemv_reduce<<<grid_for(N), 256, 0, c.stream>>>(N, (int)nz, part.d(), alpha, beta, y, sy);
      count_launch();
    }
  }
  count_launch();
  check_launch("gemv");
}

}  // namespace ucc
