// Internal core of the GB300 RHF-CC library: device tensors, the context, errors,
// and the launchers of the hand-written kernels.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/ugacc_gb300.h"

namespace ucc {

constexpr int kMaxRank = 6;

// A (possibly strided) view of float64 device memory.  Dense tensors are row-major;
// views produced by permute() share the pointer and reorder dims/strides.
struct Tensor {
  double* p = nullptr;
  int rank = 0;
  int64_t d[kMaxRank] = {};
  int64_t s[kMaxRank] = {};

  int64_t size() const {
    int64_t n = 1;
    for (int k = 0; k < rank; k++) n *= d[k];
    return n;
  }
  bool dense() const {
    int64_t st = 1;
    for (int k = rank - 1; k >= 0; k--) {
      if (d[k] != 1 && s[k] != st) return false;
      st *= d[k];
    }
    return true;
  }
  // view with axes reordered: result axis k is this tensor's axis perm[k]
  Tensor permute(const std::vector<int>& perm) const;
  Tensor slice0(int64_t i) const;  // drop leading axis at index i
};

Tensor make_view(double* p, const std::vector<int64_t>& dims);

struct Error : std::runtime_error {
  ucc_status status;
  Error(ucc_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};

#define UCC_CUDA(call)                                                                     \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess)                                                                 \
      throw ::ucc::Error(e_ == cudaErrorMemoryAllocation ? UCC_OUT_OF_MEMORY : UCC_CUDA_ERROR, \
                         std::string(#call) + ": " + cudaGetErrorString(e_));             \
  } while (0)

#define UCC_REQUIRE(cond, status, msg) \
  do {                                 \
    if (!(cond)) throw ::ucc::Error(status, msg); \
  } while (0)

// An operand matrix whose row and column indices are index groups of a tensor made of up
// to two strided runs each: element (r, k) sits at p + off(r) + off(k) with
// off(r) = rsplit ? (r / rsplit) rs_hi + (r % rsplit) rs_lo : r rs_hi (columns likewise).
// The tensor-core operand readers take it directly, so such operands need no gather.
struct MatView {
  const double* p = nullptr;
  int64_t rows = 0, cols = 0;
  int64_t rsplit = 0, rs_hi = 0, rs_lo = 0;
  int64_t ksplit = 0, ks_hi = 0, ks_lo = 0;
  static MatView strided(const double* p, int64_t rows, int64_t cols, int64_t sr, int64_t sk) {
    MatView v;
    v.p = p;
    v.rows = rows;
    v.cols = cols;
    v.rs_hi = sr;
    v.ks_hi = sk;
    return v;
  }
  int64_t roff(int64_t r) const { return rsplit ? (r / rsplit) * rs_hi + (r % rsplit) * rs_lo : r * rs_hi; }
  int64_t koff(int64_t k) const { return ksplit ? (k / ksplit) * ks_hi + (k % ksplit) * ks_lo : k * ks_hi; }
  // the rows [r0, r0 + n) (columns [k0, k0 + n)) as a view; false when r0 splits a run
  bool sub_rows(int64_t r0, int64_t n, MatView& out) const {
    if (rsplit && r0 % rsplit) return false;
    out = *this;
    out.p = p + roff(r0);
    out.rows = n;
    return true;
  }
  bool sub_cols(int64_t k0, int64_t n, MatView& out) const {
    if (ksplit && k0 % ksplit) return false;
    out = *this;
    out.p = p + koff(k0);
    out.cols = n;
    return true;
  }
  bool k_contiguous() const { return (ksplit ? ks_lo : ks_hi) == 1; }  // unit stride along the columns
};

// FP64 buffer from the stream-ordered pool, freed in stream order (no device
// synchronisation): per-sweep state such as the refinement anchors.
struct PoolBuffer {
  double* p = nullptr;
  cudaStream_t stream = nullptr;
  PoolBuffer(cudaStream_t s, size_t count) : stream(s) {
    if (count) UCC_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&p), count * sizeof(double), s));
  }
  ~PoolBuffer() {
    if (p) cudaFreeAsync(p, stream);
  }
  PoolBuffer(const PoolBuffer&) = delete;
  PoolBuffer& operator=(const PoolBuffer&) = delete;
};

// Owned device buffer (cudaMalloc; freed on destruction).
struct DeviceBuffer {
  double* p = nullptr;
  size_t n = 0;
  DeviceBuffer() = default;
  explicit DeviceBuffer(size_t count);
  ~DeviceBuffer();
  DeviceBuffer(const DeviceBuffer&) = delete;
  DeviceBuffer& operator=(const DeviceBuffer&) = delete;
};

struct Ctx;

// Stream-ordered scratch allocation (CUDA's async pool on the context stream).
struct Recorder;
struct Scratch {
  Ctx* ctx = nullptr;
  void* p = nullptr;
  Recorder* rec = nullptr;  // allocated from a recorder's arena
  Scratch(Ctx& c, size_t bytes);
  ~Scratch();
  double* d() const { return static_cast<double*>(p); }
  Scratch(const Scratch&) = delete;
  Scratch& operator=(const Scratch&) = delete;
};

struct Timer {  // CUDA events on the context stream
  cudaEvent_t a = nullptr, b = nullptr;
  cudaStream_t st = nullptr;
  explicit Timer(cudaStream_t s);
  ~Timer();
  void start();
  double stop_ms();  // synchronises
};

struct Perturbation;  // cc_pert.cpp
struct Ctx;

// Scoped switch that keeps every contraction in FP64 (Hamiltonian build, refinement).
struct Fp64Scope {
  Ctx& c;
  bool saved;
  explicit Fp64Scope(Ctx& ctx, bool on = true);
  ~Fp64Scope();
};
// Scoped setting of the FP64 switch to a given value (false re-enables split products
// inside an FP64 scope when the context precision is MIXED).
struct PrecisionScope {
  Ctx& c;
  bool saved;
  PrecisionScope(Ctx& ctx, bool force_fp64);
  ~PrecisionScope();
};

struct Ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  ucc_options opt{};
  std::string last_error;

  int no = 0, nv = 0, naux = 0;
  bool loaded = false, have_ccsd = false, have_hbar = false, have_lambda = false;
  bool have_tgrad = false;  // (T) gradient pieces present: Lambda and the densities include them
  std::vector<double> eps;  // orbital energies (diagonal of the Fock matrix)
  std::vector<double> fock;  // [nact][nact]

  // named persistent device arrays (integral blocks, amplitudes, HBAR, ...)
  std::map<std::string, std::unique_ptr<DeviceBuffer>> store;
  std::map<std::string, std::vector<int64_t>> shapes;
  Tensor get(const std::string& name) const;
  Tensor alloc(const std::string& name, const std::vector<int64_t>& dims, bool zero = true);
  bool has(const std::string& name) const { return store.count(name) != 0; }
  void drop(const std::string& name);

  bool force_fp64 = false;  // integral construction and refinement sweeps stay FP64
  double e2_parts[6] = {};  // two-particle density energies OOOO VVVV OOOV VVVO OVOV OOVV

  // Anchored refinement of a mixed-precision solve.  In a record sweep (mode 1) every
  // heavy GEMM runs in FP64 and keeps its operands A0, B0 and product P0 = A0 B0; in a
  // delta sweep (mode 2) the same GEMM, found by its position in the sweep, is evaluated
  // as P0 + (A - A0) B + A0 (B - B0) with the two correction products on the tensor
  // cores, so that their rounding error scales with the distance from the anchor.
  struct AnchorTerm {
    int64_t M = 0, N = 0, K = 0;
    bool a_const = false, b_const = false;
    std::unique_ptr<PoolBuffer> a0, b0, p0;  // dense [M][K], [K][N], [M][N]
  };
  struct Anchors {
    int mode = 0;     // 0 off, 1 record, 2 delta
    int digits = 9;   // bf16 slices per operand of the record sweep's sliced products
    size_t next = 0;
    std::vector<AnchorTerm> terms;
    void begin(int m) {
      mode = m;
      next = 0;
      if (m == 1) terms.clear();
    }
    void clear() {
      mode = 0;
      next = 0;
      terms.clear();
    }
  } anchors;
  // state of the tensor-core path (split operand cache, error flag), dropped on reload
  std::shared_ptr<void> tc_cache;
  // true if p lies in a block that never changes once built (integrals, L, HBAR)
  bool is_constant(const double* p) const;
  std::vector<std::unique_ptr<Perturbation>> perts;
  ucc_stats stats{};

  // CUDA-event timing of FP64 GEMM launches, resolved into stats lazily
  struct TimedLaunch {
    cudaEvent_t a, b;
    double flops;
    int kind = 0;  // 0 FP64 GEMM, 1 split tensor-core GEMM, 2 sliced FP64 GEMM
    double products = 1.0;  // sliced: the slice products per output (S(S+1)/2 for S digits)
  };
  std::vector<TimedLaunch> gemm_timers;
  std::vector<cudaEvent_t> event_pool;
  cudaEvent_t take_event();
  void resolve_timers();  // synchronises the stream

  ~Ctx();
};

// ----------------------------------------------------------------------------------
// Operation recording for grouped replay (batched solver).  While a Recorder is
// installed on the calling thread, the GEMM / GEMV / permute / axpby / fill launchers
// append a description of their work instead of launching, Scratch allocations come
// from the recorder's arena (a stack: scoped scratch is released in reverse order), and
// contract() takes its index-group orders from a tape shared by all recorded problems,
// so that every problem yields the same operation sequence.
// ----------------------------------------------------------------------------------
struct RecordedOp {
  enum Kind { kGemm = 0, kPermute = 1, kFill = 2 } kind = kGemm;
  // GEMM: C[m*sCm + n*sCn] = alpha * sum_k A[m*sAm + k*sAk] B[k*sBk + n*sBn] + beta * C
  int64_t M = 0, N = 0, K = 0, sAm = 0, sAk = 0, sBk = 0, sBn = 0, sCm = 0, sCn = 0;
  const double* A = nullptr;
  const double* B = nullptr;
  double* C = nullptr;
  double alpha = 0.0, beta = 0.0;
  // permute: out = alpha * in + beta * out over out's dims; fill: out = alpha
  int rank = 0;
  int64_t d[kMaxRank] = {}, si[kMaxRank] = {}, so[kMaxRank] = {};
  const double* in = nullptr;
  double* out = nullptr;
};

struct Recorder {
  std::vector<RecordedOp> ops;
  char* arena = nullptr;  // null: sizing pass, the addresses handed out are never used
  size_t used = 0, peak = 0;
  struct Block {
    size_t off, bytes;
    bool freed;
  };
  std::vector<Block> blocks;
  std::vector<std::string> tape;
  size_t tape_pos = 0;
  bool replay_tape = false;
  void* alloc(size_t bytes);
  void release(void* p);
};
Recorder*& recorder();  // the calling thread's recorder (null: launch normally)

// ----------------------------------------------------------------------------------
// Kernel launchers (kernels_fp64.cu).  All are asynchronous on ctx.stream.
// ----------------------------------------------------------------------------------
struct GemmEpilogue {  // C offset of element (m, n): (m / msplit) * s_mhi + (m % msplit) * s_mlo + n * s_n
  int64_t msplit = 0;  // 0: plain, offset = m * s_mhi + n * s_n
  int64_t s_mhi = 0, s_mlo = 0, s_n = 1;
};

// Blocked W3 layout of the mixed (T) path: W[a][b][c] of one tuple in 8 x 8 x 8 blocks,
// block (a/8, b/8, c/8) at ((a/8 * T + b/8) * T + c/8) * 512 (T = ceil(nv/8) blocks per
// index), element (x, y, z) = (a%8, b%8, c%8) of a block at 64 x + 8 (y ^ x) + (z ^ (5y % 8)).
// Every tile the energy reads is then one contiguous 2 KB block, and the swizzle makes its
// six index orders conflict-free shared-memory reads for the energy kernel's thread order.
__host__ __device__ __forceinline__ int64_t w3_block_offset(int64_t a, int64_t b, int64_t c, int64_t T) {
  const int x = (int)(a & 7), y = (int)(b & 7), z = (int)(c & 7);
  return (((a >> 3) * T + (b >> 3)) * T + (c >> 3)) * 512 + 64 * x + 8 * (y ^ x) + (z ^ ((5 * y) & 7));
}

struct GemmPtrs {
  const double* A;
  const double* B;
  double* C;
};

// C = alpha * op(A) op(B) + beta * C, row-major; op(A)[m][k] = ta ? A[k*lda+m] : A[m*lda+k];
// op(B)[k][n] = tb ? B[n*ldb+k] : B[k*ldb+n].  Batched over `batch` with either strides
// or a device array of pointer triples.
void dgemm(Ctx& c, bool ta, bool tb, int64_t M, int64_t N, int64_t K, double alpha, const double* A, int64_t lda,
           const double* B, int64_t ldb, double beta, double* C, const GemmEpilogue& epi, int batch = 1,
           int64_t sA = 0, int64_t sB = 0, int64_t sC = 0, const GemmPtrs* ptrs = nullptr);

// Same with arbitrary operand strides: op(A)[m][k] = A[m*sAm + k*sAk], op(B)[k][n] = B[k*sBk + n*sBn].
// Status of the tensor-core launches since the last check (pipeline-wait timeout, sliced
// operand out of range), read after synchronising the stream; throws on either.
void tc_check(Ctx& c);
// FP64 GEMM for a small output (M, N <= 256, M N <= 4096) and a long K (>= 8192): K chunks
// per block and a fixed-order reduce.  False when the shape does not qualify.
bool dgemm_small_output(Ctx& c, int64_t M, int64_t N, int64_t K, double alpha, const double* A, int64_t sAm,
                        int64_t sAk, const double* B, int64_t sBk, int64_t sBn, double beta, double* C,
                        const GemmEpilogue& epi);
void dgemm_strided(Ctx& c, int64_t M, int64_t N, int64_t K, double alpha, const double* A, int64_t sAm, int64_t sAk,
                   const double* B, int64_t sBk, int64_t sBn, double beta, double* C, const GemmEpilogue& epi,
                   int batch, int64_t bA, int64_t bB, int64_t bC, const GemmPtrs* ptrs);
// y[n] = alpha * sum_k x[k*sx] A[k*sk + n*sn] + beta * y[n*sy]
void dgemv_strided(Ctx& c, int64_t N, int64_t K, double alpha, const double* x, int64_t sx, const double* A,
                   int64_t sk, int64_t sn, double beta, double* y, int64_t sy);

// out = alpha * in + beta * out over out's dims; both may be strided views.
void permute_add(Ctx& c, const Tensor& in, double alpha, double beta, const Tensor& out);

// y = alpha * x + beta * y, dense, n elements
void axpby(Ctx& c, int64_t n, double alpha, const double* x, double beta, double* y);
void fill(Ctx& c, int64_t n, double v, double* y);

// Sum of x[k] * y[k] (y == nullptr: sum of x) with compensated FP64 accumulation; the
// result stays on the device.
void dot_async(Ctx& c, int64_t n, const double* x, const double* y, double* d_out);
double dot(Ctx& c, int64_t n, const double* x, const double* y);
// Several dot products x_k . y at once (DIIS B-matrix row), results on the device.
void multidot_async(Ctx& c, int nvec, const double* const* d_xs, const double* y, int64_t n, double* d_out);

// tau = g t2 + f1 * t1(i,a) t1(j,b); ttau = g t2 + f2 * t1 t1  (ttau may be null; g = 1 or 1/2)
void build_tau(Ctx& c, int no, int nv, const double* t1, const double* t2, double f1, double* tau, double f2,
               double* ttau, double g = 1.0);

// Jacobi update t_new = t_old + R / (D + shift), D built on the fly from the diagonals
// do[no], dv[nv] in the reference's order ((d_i + d_j) - d_a) - d_b; the sum of R^2
// (compensated) goes to the device scalar d_sumsq.
void jacobi_update(Ctx& c, int no, int nv, const double* d_do, const double* d_dv, double shift, const double* R1,
                   const double* R2, const double* t1old, const double* t2old, double* t1new, double* t2new,
                   double* d_sumsq);

// out = sum_p coef[p] * vecs[p] (device pointers, host coefficients), n elements
void lincomb(Ctx& c, int nvec, const double* const* d_vecs, const double* coef, int64_t n, double* out);

// (T) energy over a batch of (i>=j>=k) tuples, given W3 for each tuple.
void triples_energy(Ctx& c, int no, int nv, int ntuple, const int* d_tuples, const double* W3,
                    const double* t1, const double* Voovv, const double* eps, double* d_partial);
// The same from an FP32 W3 (mixed form) held as nparts partial arrays part_stride floats
// apart (W3 = their sum): per-element arithmetic in FP32, the energy sum in FP64
// (compensated).
// With f32in (FP32 copies of Voovv, t1 and eps made once per (T) call by triples_f32_inputs,
// laid out by triples_f32_layout; nv % 4 == 0) the pipelined kernel runs on W3 in the
// blocked layout of w3_block_offset, part_stride floats per array; without it the
// padded-tile kernel on the plain [a][b][c] layout.
int64_t triples_f32_partials(int nv);  // partial sums per tuple written by triples_energy_f32
struct TriplesF32Layout {
  int64_t off_t1, off_ev, off_eo, total;  // float offsets of t1, virtual and occupied energies; total floats
};
TriplesF32Layout triples_f32_layout(int no, int nv);
void triples_f32_inputs(Ctx& c, int no, int nv, const double* t1, const double* Voovv, const double* eps,
                        float* out);
void triples_energy_f32(Ctx& c, int no, int nv, int ntuple, const int* d_tuples, const float* W3, int nparts,
                        int64_t part_stride, const double* t1, const double* Voovv, const double* eps,
                        double* d_partial, const float* f32in = nullptr);

// Pair-symmetric particle ladder (sum_ef W_abef tau_ijef = S + sign A over packed pairs,
// W and tau invariant under the simultaneous pair swap):
// Vp[a<=b][e<=f] = W_abef + W_abfe (W_abee on e == f), Vm[a<b][e<f] = W_abef - W_abfe, with
// W from a stored block by `mode` (0: H_abef; 1: H_efab + H_feba; 2: H_abef + H_bafe);
// Tp[i<=j][e<=f] = (tau_ijef + tau_ijfe)/2 (tau_ijee on e == f), Tm[i<j][e<f] = (tau_ijef - tau_ijfe)/2;
// R2[ijab] += alpha (S[ij][ab] + sign A[ij][ab]) over the sorted pairs.  Pairs p <= q are
// numbered q(q+1)/2 + p, strict pairs q(q-1)/2 + p.
void pack_vvvv(Ctx& c, int nv, int mode, const double* H, double* Vp, double* Vm);
void pack_tau(Ctx& c, int no, int nv, const double* tau, double* Tp, double* Tm);
void unpack_ladder(Ctx& c, int no, int nv, double alpha, const double* S, const double* A, double* R2);

int64_t launches();  // kernels launched by this library so far (all contexts)

}  // namespace ucc
