// Contraction engine and context plumbing (host code).
#include "engine.h"

#include <algorithm>
#include <cstring>

namespace ucc {

// mixed-precision GEMM path (tc_gemm.cu); returns false if it declines the problem
bool mixed_gemm(Ctx& c, int64_t M, int64_t N, int64_t K, double alpha, const double* A, int64_t sAm, int64_t sAk,
                const double* B, int64_t sBk, int64_t sBn, double beta, double* C, int64_t sCm, int64_t sCn);
bool tc_eligible(int64_t M, int64_t N, int64_t K);
bool mixed_gemm(Ctx& c, int64_t M, int64_t N, int64_t K, double alpha, const MatView& A, const MatView& B, double beta,
                double* C, int64_t sCm, int64_t sCn);
bool sliced_gemm(Ctx& c, int64_t M, int64_t N, int64_t K, double alpha, const MatView& A, const MatView& B,
                 double beta, double* C, int64_t sCm, int64_t sCn);
bool sliced_gemm(Ctx& c, int64_t M, int64_t N, int64_t K, double alpha, const double* A, int64_t sAm, int64_t sAk,
                 const double* B, int64_t sBk, int64_t sBn, double beta, double* C, int64_t sCm, int64_t sCn);
void tc_gemm_oriented(Ctx& c, int64_t M, int64_t N, int64_t K, double alpha, const double* A, int64_t sAm,
                      int64_t sAk, const double* B, int64_t sBk, int64_t sBn, double beta, double* C, int64_t sCm,
                      int64_t sCn, int parts, int kc);

// ---------------------------------------------------------------------------------------
Tensor make_view(double* p, const std::vector<int64_t>& dims) {
  Tensor t;
  t.p = p;
  t.rank = (int)dims.size();
  UCC_REQUIRE(t.rank <= kMaxRank, UCC_BAD_ARGS, "rank too large");
  int64_t st = 1;
  for (int k = t.rank - 1; k >= 0; k--) {
    t.d[k] = dims[k];
    t.s[k] = st;
    st *= dims[k];
  }
  return t;
}

Tensor Tensor::permute(const std::vector<int>& perm) const {
  UCC_REQUIRE((int)perm.size() == rank, UCC_BAD_ARGS, "permute: wrong length");
  Tensor r = *this;
  for (int k = 0; k < rank; k++) {
    r.d[k] = d[perm[k]];
    r.s[k] = s[perm[k]];
  }
  return r;
}

Tensor Tensor::slice0(int64_t i) const {
  Tensor r;
  r.p = p + i * s[0];
  r.rank = rank - 1;
  for (int k = 1; k < rank; k++) {
    r.d[k - 1] = d[k];
    r.s[k - 1] = s[k];
  }
  return r;
}

DeviceBuffer::DeviceBuffer(size_t count) : n(count) {
  if (count) UCC_CUDA(cudaMalloc(&p, count * sizeof(double)));
}
DeviceBuffer::~DeviceBuffer() {
  if (p) cudaFree(p);
}

Scratch::Scratch(Ctx& c, size_t bytes) : ctx(&c) {
  if (bytes == 0) bytes = 16;
  if ((rec = recorder()) != nullptr) {
    p = rec->alloc(bytes);
    return;
  }
  UCC_CUDA(cudaMallocAsync(&p, bytes, c.stream));
}
Scratch::~Scratch() {
  if (rec)
    rec->release(p);
  else if (p)
    cudaFreeAsync(p, ctx->stream);
}

Recorder*& recorder() {
  static thread_local Recorder* r = nullptr;
  return r;
}

void* Recorder::alloc(size_t bytes) {
  bytes = (bytes + 255) / 256 * 256;
  // sizing pass: offsets from a fixed non-null base; nothing is launched while recording
  char* base = arena ? arena : reinterpret_cast<char*>(uintptr_t(1) << 44);
  blocks.push_back({used, bytes, false});
  void* p = base + used;
  used += bytes;
  peak = std::max(peak, used);
  return p;
}

void Recorder::release(void* p) {
  char* base = arena ? arena : reinterpret_cast<char*>(uintptr_t(1) << 44);
  const size_t off = (size_t)(static_cast<char*>(p) - base);
  for (auto& b : blocks)
    if (b.off == off && !b.freed) b.freed = true;
  while (!blocks.empty() && blocks.back().freed) {
    used = blocks.back().off;
    blocks.pop_back();
  }
}

Timer::Timer(cudaStream_t s) : st(s) {
  cudaEventCreate(&a);
  cudaEventCreate(&b);
}
Timer::~Timer() {
  cudaEventDestroy(a);
  cudaEventDestroy(b);
}
void Timer::start() { cudaEventRecord(a, st); }
double Timer::stop_ms() {
  cudaEventRecord(b, st);
  cudaEventSynchronize(b);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  return ms;
}

Tensor Ctx::get(const std::string& name) const {
  auto it = store.find(name);
  UCC_REQUIRE(it != store.end(), UCC_BAD_STATE, "array not available: " + name);
  return make_view(it->second->p, shapes.at(name));
}

Tensor Ctx::alloc(const std::string& name, const std::vector<int64_t>& dims, bool zero) {
  size_t n = 1;
  for (auto x : dims) n *= (size_t)x;
  auto it = store.find(name);
  if (it == store.end() || it->second->n != n) {
    store[name].reset();
    store[name] = std::make_unique<DeviceBuffer>(n);
  }
  shapes[name] = dims;
  if (zero && n) UCC_CUDA(cudaMemsetAsync(store[name]->p, 0, n * sizeof(double), stream));
  return make_view(store[name]->p, dims);
}

Fp64Scope::Fp64Scope(Ctx& ctx, bool on) : c(ctx), saved(ctx.force_fp64) {
  if (on) c.force_fp64 = true;
}
Fp64Scope::~Fp64Scope() { c.force_fp64 = saved; }
PrecisionScope::PrecisionScope(Ctx& ctx, bool f) : c(ctx), saved(ctx.force_fp64) { c.force_fp64 = f; }
PrecisionScope::~PrecisionScope() { c.force_fp64 = saved; }

cudaEvent_t Ctx::take_event() {
  if (!event_pool.empty()) {
    cudaEvent_t e = event_pool.back();
    event_pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  UCC_CUDA(cudaEventCreate(&e));
  return e;
}

void Ctx::resolve_timers() {
  if (gemm_timers.empty()) return;
  UCC_CUDA(cudaStreamSynchronize(stream));
  for (auto& t : gemm_timers) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, t.a, t.b);
    if (t.kind == 1) {
      stats.tc_gemm_ms += ms;
      stats.tc_gemm_flops += t.flops;
    } else if (t.kind == 2) {
      stats.sliced_gemm_ms += ms;
      stats.sliced_gemm_flops += t.flops;
      stats.sliced_gemm_product_flops += t.flops * t.products;
    } else {
      stats.fp64_gemm_ms += ms;
      stats.fp64_gemm_flops += t.flops;
      stats.fp64_gemm_launches++;
    }
    event_pool.push_back(t.a);
    event_pool.push_back(t.b);
  }
  gemm_timers.clear();
}

bool Ctx::is_constant(const double* p) const {
  for (const auto& kv : store) {
    const std::string& n = kv.first;
    const bool block = n[0] == 'V' || (n[0] == 'H' && n != "Hdiag") || n == "Loovv" || n == "Looov" ||
                       n == "Lovvv" || n == "Lovvo";
    if (block && p >= kv.second->p && p < kv.second->p + kv.second->n) return true;
  }
  return false;
}

void Ctx::drop(const std::string& name) {
  store.erase(name);
  shapes.erase(name);
}

Temp::Temp(Ctx& c, const std::vector<int64_t>& dims, bool zero) : buf(c, [&] {
  size_t n = 1;
  for (auto x : dims) n *= (size_t)x;
  return n * sizeof(double);
}()) {
  t = make_view(buf.d(), dims);
  if (zero) {
    if (buf.rec)
      fill(c, t.size(), 0.0, buf.d());
    else
      UCC_CUDA(cudaMemsetAsync(buf.p, 0, t.size() * sizeof(double), c.stream));
  }
}

// ---------------------------------------------------------------------------------------
namespace {

// GEMMs with at least this many multiply-adds are anchored during refinement; lighter
// ones simply run in FP64 there.  The contractions over one occupied index (K = no) sit
// near 1e8 at no=16/nv=160: in FP64 they are bound by GB300's FP64 pipe (2 M N K
// operations), anchored they cost a copy, one split tensor-core product and a permute
constexpr double kAnchorMinWork = 5e7;
// the corrections of a delta sweep use the two-part split: the three-part split with
// FP64-summed K chunks (UCC_MIXED_FINE) measured 8x less noise in the delta residuals at
// no=16/nv=160 but costs ~10 % of the step and still leaves the final FP64 sweep needed
constexpr int kDeltaParts = 2, kDeltaChunk = 0;

Tensor matrix_view(const double* p, int64_t rows, int64_t cols, int64_t sr, int64_t sc) {
  Tensor t;
  t.p = const_cast<double*>(p);
  t.rank = 2;
  t.d[0] = rows;
  t.d[1] = cols;
  t.s[0] = sr;
  t.s[1] = sc;
  return t;
}

// C = alpha * A B + beta * C for one GEMM of an anchored refinement sweep
void anchored_gemm(Ctx& c, int64_t M, int64_t N, int64_t K, double alpha, const double* A, int64_t sAm, int64_t sAk,
                   bool a_const, const double* B, int64_t sBk, int64_t sBn, bool b_const, double beta, double* C,
                   int64_t sCm, int64_t sCn) {
  auto& an = c.anchors;
  const Tensor av = matrix_view(A, M, K, sAm, sAk), bv = matrix_view(B, K, N, sBk, sBn);
  const Tensor cv = matrix_view(C, M, N, sCm, sCn);
  if (an.mode == 1) {
    Ctx::AnchorTerm t;
    t.M = M;
    t.N = N;
    t.K = K;
    t.a_const = a_const;
    t.b_const = b_const;
    if (!a_const) {
      t.a0 = std::make_unique<PoolBuffer>(c.stream, (size_t)(M * K));
      permute_add(c, av, 1.0, 0.0, make_view(t.a0->p, {M, K}));
    }
    if (!b_const) {
      t.b0 = std::make_unique<PoolBuffer>(c.stream, (size_t)(K * N));
      permute_add(c, bv, 1.0, 0.0, make_view(t.b0->p, {K, N}));
    }
    t.p0 = std::make_unique<PoolBuffer>(c.stream, (size_t)(M * N));
    const double t0 = c.stats.sliced_gemm_ms;
    const bool sliced = sliced_gemm(c, M, N, K, 1.0, A, sAm, sAk, B, sBk, sBn, 0.0, t.p0->p, N, 1);
    if (sliced && c.opt.print >= 3)
      std::printf("\tsliced GEMM (anchor, %d digits)  M=%lld N=%lld K=%lld  %.3f ms\n", c.anchors.digits, (long long)M,
                  (long long)N, (long long)K, c.stats.sliced_gemm_ms - t0);
    if (!sliced) {
      GemmEpilogue epi;
      epi.s_mhi = N;
      epi.s_n = 1;
      dgemm_strided(c, M, N, K, 1.0, A, sAm, sAk, B, sBk, sBn, 0.0, t.p0->p, epi, 1, 0, 0, 0, nullptr);
    }
    permute_add(c, make_view(t.p0->p, {M, N}), alpha, beta, cv);
    an.terms.push_back(std::move(t));
    an.next++;
    return;
  }
  UCC_REQUIRE(an.next < an.terms.size(), UCC_BAD_STATE, "anchored refinement: more heavy GEMMs than recorded");
  const Ctx::AnchorTerm& t = an.terms[an.next++];
  UCC_REQUIRE(t.M == M && t.N == N && t.K == K && t.a_const == a_const && t.b_const == b_const, UCC_BAD_STATE,
              "anchored refinement: the GEMM sequence changed since the record sweep");
  Temp P(c, {M, N});
  UCC_CUDA(cudaMemcpyAsync(P->p, t.p0->p, sizeof(double) * M * N, cudaMemcpyDeviceToDevice, c.stream));
  if (!a_const) {  // P += (A - A0) B
    Temp dA(c, {M, K});
    permute_add(c, av, 1.0, 0.0, dA);
    axpby(c, M * K, -1.0, t.a0->p, 1.0, dA->p);
    tc_gemm_oriented(c, M, N, K, 1.0, dA->p, K, 1, B, sBk, sBn, 1.0, P->p, N, 1, kDeltaParts, kDeltaChunk);
  }
  if (!b_const) {  // P += A0 (B - B0)
    Temp dB(c, {K, N});
    permute_add(c, bv, 1.0, 0.0, dB);
    axpby(c, K * N, -1.0, t.b0->p, 1.0, dB->p);
    if (a_const)
      tc_gemm_oriented(c, M, N, K, 1.0, A, sAm, sAk, dB->p, N, 1, 1.0, P->p, N, 1, kDeltaParts, kDeltaChunk);
    else
      tc_gemm_oriented(c, M, N, K, 1.0, t.a0->p, K, 1, dB->p, N, 1, 1.0, P->p, N, 1, kDeltaParts, kDeltaChunk);
  }
  permute_add(c, P, alpha, beta, cv);
}

struct Parsed {
  std::string a, b, c;
};

Parsed parse(const std::string& spec) {
  Parsed p;
  auto arrow = spec.find("->");
  UCC_REQUIRE(arrow != std::string::npos, UCC_BAD_ARGS, "spec needs ->: " + spec);
  std::string lhs = spec.substr(0, arrow);
  p.c = spec.substr(arrow + 2);
  auto comma = lhs.find(',');
  if (comma == std::string::npos) {
    p.a = lhs;
  } else {
    p.a = lhs.substr(0, comma);
    p.b = lhs.substr(comma + 1);
  }
  return p;
}

int pos(const std::string& s, char ch) {
  auto k = s.find(ch);
  return k == std::string::npos ? -1 : (int)k;
}

// A group of labels, in order, addressed with one stride in tensor T (labels str)?
// Returns the innermost stride (0 = group empty / extent 1, any stride works).
bool fusable(const Tensor& T, const std::string& str, const std::string& grp, int64_t& inner) {
  inner = 0;
  int64_t expect = -1;
  for (int k = (int)grp.size() - 1; k >= 0; k--) {
    const int ax = pos(str, grp[k]);
    const int64_t d = T.d[ax], s = T.s[ax];
    if (d == 1) continue;
    if (expect < 0) {
      inner = s;
    } else if (s != expect) {
      return false;
    }
    expect = s * d;
  }
  return true;
}

int64_t extent(const Tensor& T, const std::string& str, const std::string& grp) {
  int64_t e = 1;
  for (char ch : grp) e *= T.d[pos(str, ch)];
  return e;
}

// index group grp of T as at most two strided runs, an outer one (the leading labels) and an
// inner one: offset(x) = split ? (x / split) s_hi + (x % split) s_lo : x s_hi
bool fusable2(const Tensor& T, const std::string& str, const std::string& grp, int64_t& split, int64_t& s_hi,
              int64_t& s_lo) {
  split = 0;
  s_lo = 0;
  if (fusable(T, str, grp, s_hi)) return true;
  for (size_t cut = 1; cut < grp.size(); cut++) {
    int64_t so, si;
    const std::string outer = grp.substr(0, cut), inner = grp.substr(cut);
    if (fusable(T, str, outer, so) && fusable(T, str, inner, si)) {
      split = extent(T, str, inner);
      s_hi = so;
      s_lo = si;
      return true;
    }
  }
  return false;
}

// rows (group rg) x columns (group kg) of T as a two-stride operand view
bool view2(const Tensor& T, const std::string& str, const std::string& rg, const std::string& kg, MatView& v) {
  if (!fusable2(T, str, rg, v.rsplit, v.rs_hi, v.rs_lo) || !fusable2(T, str, kg, v.ksplit, v.ks_hi, v.ks_lo))
    return false;
  v.p = T.p;
  v.rows = extent(T, str, rg);
  v.cols = extent(T, str, kg);
  return true;
}

std::string ordered(const std::string& src, const std::string& set) {
  std::string r;
  for (char ch : src)
    if (set.find(ch) != std::string::npos) r += ch;
  return r;
}

// dense copy of T relabelled into the order `target`
Tensor gather(Ctx& c, const Tensor& T, const std::string& str, const std::string& target,
              std::unique_ptr<Scratch>& holder) {
  std::vector<int> perm;
  std::vector<int64_t> dims;
  for (char ch : target) {
    perm.push_back(pos(str, ch));
    dims.push_back(T.d[pos(str, ch)]);
  }
  size_t n = 1;
  for (auto x : dims) n *= (size_t)x;
  holder = std::make_unique<Scratch>(c, n * sizeof(double));
  Tensor out = make_view(holder->d(), dims);
  Tensor src = T.permute(perm);
  permute_add(c, src, 1.0, 0.0, out);
  return out;
}

}  // namespace

Tensor view(const Tensor& T, const std::string& spec) {
  Parsed p = parse(spec);
  UCC_REQUIRE((int)p.a.size() == T.rank && p.a.size() == p.c.size(), UCC_BAD_ARGS, "view: bad spec " + spec);
  std::vector<int> perm;
  for (char ch : p.c) {
    int k = pos(p.a, ch);
    UCC_REQUIRE(k >= 0, UCC_BAD_ARGS, "view: bad spec " + spec);
    perm.push_back(k);
  }
  return T.permute(perm);
}

void transpose_add(Ctx& c, const std::string& spec, double alpha, const Tensor& A, double beta, const Tensor& C) {
  Tensor v = view(A, spec);
  permute_add(c, v, alpha, beta, C);
}

double dot_all(Ctx& c, const Tensor& A, const Tensor& B) {
  UCC_REQUIRE(A.rank == B.rank, UCC_BAD_ARGS, "dot_all: rank mismatch");
  for (int k = 0; k < A.rank; k++) UCC_REQUIRE(A.d[k] == B.d[k], UCC_BAD_ARGS, "dot_all: dim mismatch");
  std::unique_ptr<Scratch> ha, hb;
  const double* pa = A.p;
  const double* pb = B.p;
  std::string lab = std::string("abcdef").substr(0, A.rank);
  if (!A.dense()) pa = gather(c, A, lab, lab, ha).p;
  if (!B.dense()) pb = gather(c, B, lab, lab, hb).p;
  return dot(c, A.size(), pa, pb);
}

void contract(Ctx& c, const std::string& spec, double alpha, const Tensor& A, const Tensor& B, double beta,
              const Tensor& C) {
  Parsed p = parse(spec);
  UCC_REQUIRE((int)p.a.size() == A.rank && (int)p.b.size() == B.rank && (int)p.c.size() == C.rank, UCC_BAD_ARGS,
              "contract: rank/spec mismatch " + spec);
  std::string Ms, Ns, Ks;
  for (char ch : p.c) {
    const bool ia = pos(p.a, ch) >= 0, ib = pos(p.b, ch) >= 0;
    UCC_REQUIRE(ia != ib, UCC_UNSUPPORTED, "contract: batch/free label unsupported in " + spec);
    (ia ? Ms : Ns) += ch;
  }
  for (char ch : p.a) {
    if (pos(p.c, ch) >= 0) continue;
    UCC_REQUIRE(pos(p.b, ch) >= 0, UCC_UNSUPPORTED, "contract: trace label unsupported in " + spec);
    Ks += ch;
  }
  for (char ch : p.b)
    if (pos(p.c, ch) < 0) UCC_REQUIRE(pos(p.a, ch) >= 0, UCC_UNSUPPORTED, "contract: trace label in " + spec);
  // dimension checks
  for (char ch : p.c) {
    const Tensor& S = pos(p.a, ch) >= 0 ? A : B;
    const std::string& ss = pos(p.a, ch) >= 0 ? p.a : p.b;
    UCC_REQUIRE(S.d[pos(ss, ch)] == C.d[pos(p.c, ch)], UCC_BAD_ARGS, "contract: extent mismatch in " + spec);
  }
  for (char ch : Ks)
    UCC_REQUIRE(A.d[pos(p.a, ch)] == B.d[pos(p.b, ch)], UCC_BAD_ARGS, "contract: extent mismatch in " + spec);

  const int64_t M = extent(C, p.c, Ms), N = extent(C, p.c, Ns), K = extent(A, p.a, Ks);
  if (M == 0 || N == 0) return;

  // choose group orders minimising gathered bytes
  const std::string Mcand[2] = {ordered(p.c, Ms), ordered(p.a, Ms)};
  const std::string Ncand[2] = {ordered(p.c, Ns), ordered(p.b, Ns)};
  const std::string Kcand[2] = {ordered(p.a, Ks), ordered(p.b, Ks)};
  double best = 1e300;
  std::string bm, bn, bk;
  for (const auto& mo : Mcand)
    for (const auto& no_ : Ncand)
      for (const auto& ko : Kcand) {
        int64_t s1, s2;
        double cost = 0;
        if (!(fusable(A, p.a, mo, s1) && fusable(A, p.a, ko, s2))) cost += (double)A.size();
        if (!(fusable(B, p.b, ko, s1) && fusable(B, p.b, no_, s2))) cost += (double)B.size();
        if (!(fusable(C, p.c, mo, s1) && fusable(C, p.c, no_, s2))) cost += 3.0 * (double)C.size();
        if (cost < best) {
          best = cost;
          bm = mo;
          bn = no_;
          bk = ko;
        }
      }

  if (Recorder* r = recorder()) {  // every recorded problem follows the first one's choices
    if (r->replay_tape) {
      UCC_REQUIRE(r->tape_pos + 3 <= r->tape.size(), UCC_BAD_STATE, "recorded contraction sequence diverged");
      bm = r->tape[r->tape_pos++];
      bn = r->tape[r->tape_pos++];
      bk = r->tape[r->tape_pos++];
      UCC_REQUIRE(bm.size() == Ms.size() && bn.size() == Ns.size() && bk.size() == Ks.size(), UCC_BAD_STATE,
                  "recorded contraction sequence diverged at " + spec);
    } else {
      r->tape.push_back(bm);
      r->tape.push_back(bn);
      r->tape.push_back(bk);
    }
  }
  std::unique_ptr<Scratch> hA, hB, hC;
  int64_t sCm, sCn;
  const bool cdirect = fusable(C, p.c, bm, sCm) && fusable(C, p.c, bn, sCn);
  Tensor ct = C;
  if (!cdirect) {
    std::vector<int64_t> dims;
    for (char ch : bm + bn) dims.push_back(C.d[pos(p.c, ch)]);
    size_t n = 1;
    for (auto x : dims) n *= (size_t)x;
    hC = std::make_unique<Scratch>(c, n * sizeof(double));
    ct = make_view(hC->d(), dims);
    sCm = N;
    sCn = 1;
  }
  if (sCm == 0) sCm = 1;  // empty groups: any stride works
  if (sCn == 0) sCn = 1;
  const double ga = cdirect ? alpha : 1.0, gb = cdirect ? beta : 0.0;
  bool done = false;
  const bool mixed = c.opt.precision == UCC_MIXED;
  const bool anchored = c.anchors.mode != 0 && mixed && (double)M * N * K >= kAnchorMinWork && tc_eligible(M, N, K);
  const bool small_out = M <= 256 && N <= 256 && M * N <= 4096 && K >= 8192;
  // the tensor-core paths read operands whose index groups are two strided runs directly:
  // no gather
  if (M > 1 && N > 1 && mixed && !recorder() && !anchored && !small_out) {
    MatView av, bv;
    if (view2(A, p.a, bm, bk, av) && view2(B, p.b, bn, bk, bv)) {
      if (!c.force_fp64) done = mixed_gemm(c, M, N, K, ga, av, bv, gb, ct.p, sCm, sCn);
      if (!done) {
        const double t0 = c.stats.sliced_gemm_ms;
        done = sliced_gemm(c, M, N, K, ga, av, bv, gb, ct.p, sCm, sCn);
        if (done && c.opt.print >= 3)  // PRINT >= 3: every sliced FP64 GEMM with its shape and time
          std::printf("\tsliced GEMM %s  M=%lld N=%lld K=%lld  %.3f ms\n", spec.c_str(), (long long)M, (long long)N,
                      (long long)K, c.stats.sliced_gemm_ms - t0);
      }
    }
  }
  Tensor a = A, b = B;
  int64_t sAm = 1, sAk = 1, sBk = 1, sBn = 1;
  if (!done) {  // single-stride operands for the other paths: gather where needed
    std::string sa = p.a, sb = p.b;
    if (!(fusable(a, sa, bm, sAm) && fusable(a, sa, bk, sAk))) {
      a = gather(c, A, p.a, bm + bk, hA);
      sa = bm + bk;
      fusable(a, sa, bm, sAm);
      fusable(a, sa, bk, sAk);
    }
    if (!(fusable(b, sb, bk, sBk) && fusable(b, sb, bn, sBn))) {
      b = gather(c, B, p.b, bk + bn, hB);
      sb = bk + bn;
      fusable(b, sb, bk, sBk);
      fusable(b, sb, bn, sBn);
    }
    // empty groups: any stride works
    if (sAm == 0) sAm = 1;
    if (sAk == 0) sAk = 1;
    if (sBk == 0) sBk = 1;
    if (sBn == 0) sBn = 1;
  }
  if (!done && M == 1) {  // row vector times matrix
    dgemv_strided(c, N, K, ga, a.p, sAk, b.p, sBk, sBn, gb, ct.p, sCn);
    done = true;
  } else if (!done && N == 1) {  // matrix times column vector
    dgemv_strided(c, M, K, ga, b.p, sBk, a.p, sAk, sAm, gb, ct.p, sCm);
    done = true;
  }
  if (!done && anchored) {
    anchored_gemm(c, M, N, K, ga, a.p, sAm, sAk, c.is_constant(A.p), b.p, sBk, sBn, c.is_constant(B.p), gb, ct.p,
                  sCm, sCn);
    done = true;
  }
  if (!done && c.opt.precision == UCC_MIXED && !c.force_fp64)
    done = mixed_gemm(c, M, N, K, ga, a.p, sAm, sAk, b.p, sBk, sBn, gb, ct.p, sCm, sCn);
  if (!done) {  // small output, long K: a reduction rather than a GEMM (every precision)
    GemmEpilogue epi;
    epi.msplit = 0;
    epi.s_mhi = sCm;
    epi.s_n = sCn;
    done = dgemm_small_output(c, M, N, K, ga, a.p, sAm, sAk, b.p, sBk, sBn, gb, ct.p, epi);
  }
  // the FP64 work of the MIXED form (refinement sweeps, one-shot builds): sliced operands
  // on the tensor cores, FP64-accurate
  if (!done && c.opt.precision == UCC_MIXED && !recorder()) {
    const double t0 = c.stats.sliced_gemm_ms;
    done = sliced_gemm(c, M, N, K, ga, a.p, sAm, sAk, b.p, sBk, sBn, gb, ct.p, sCm, sCn);
    if (done && c.opt.print >= 3)  // PRINT >= 3: every sliced FP64 GEMM with its shape and time
      std::printf("\tsliced GEMM %s  M=%lld N=%lld K=%lld  %.3f ms\n", spec.c_str(), (long long)M, (long long)N,
                  (long long)K, c.stats.sliced_gemm_ms - t0);
  }
  if (!done) {
    GemmEpilogue epi;
    epi.msplit = 0;
    epi.s_mhi = sCm;
    epi.s_n = sCn;
    // PRINT >= 3 in the MIXED form: the FP64 (DFMA) GEMMs that remain, with their shapes
    if (c.opt.print >= 3 && c.opt.precision == UCC_MIXED && 2.0 * M * N * K >= 1e9)
      std::printf("\tFP64 GEMM %s  M=%lld N=%lld K=%lld\n", spec.c_str(), (long long)M, (long long)N, (long long)K);
    dgemm_strided(c, M, N, K, ga, a.p, sAm, sAk, b.p, sBk, sBn, gb, ct.p, epi, 1, 0, 0, 0, nullptr);
  }
  if (!cdirect) {
    // ct is laid out (bm, bn); view it with C's label order and accumulate
    std::string tl = bm + bn;
    std::vector<int> perm;
    for (char ch : p.c) perm.push_back(pos(tl, ch));
    Tensor v = ct.permute(perm);
    permute_add(c, v, alpha, beta, C);
  }
}

}  // namespace ucc
