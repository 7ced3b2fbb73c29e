// Ground state: integral blocks, DIIS and the CCSD amplitude equations
// (ugacc ccwfn.cc:12-120, :188-626).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>

#include "cc.h"

namespace ucc {

// ---------------------------------------------------------------------------------------
// Integral blocks
// ---------------------------------------------------------------------------------------
Tensor narrow(const Tensor& t, int axis, int64_t start, int64_t len) {
  Tensor r = t;
  r.p = t.p + start * t.s[axis];
  r.d[axis] = len;
  return r;
}

static void store_fock(Ctx& c, const double* fock) {
  const int no = c.no, nv = c.nv, n = no + nv;
  c.fock.assign(fock, fock + (size_t)n * n);
  c.eps.resize(n);
  for (int p = 0; p < n; p++) c.eps[p] = fock[(size_t)p * n + p];
  auto put = [&](const char* name, int r0, int nr, int c0, int nc) {
    std::vector<double> h((size_t)nr * nc);
    for (int i = 0; i < nr; i++)
      for (int j = 0; j < nc; j++) h[(size_t)i * nc + j] = fock[(size_t)(r0 + i) * n + c0 + j];
    Tensor t = c.alloc(name, {nr, nc}, false);
    UCC_CUDA(cudaMemcpyAsync(t.p, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    UCC_CUDA(cudaStreamSynchronize(c.stream));
  };
  put("foo", 0, no, 0, no);
  put("fov", 0, no, no, nv);
  put("fvo", no, nv, 0, no);
  put("fvv", no, nv, no, nv);
  Tensor e = c.alloc("eps", {n}, false);
  UCC_CUDA(cudaMemcpyAsync(e.p, c.eps.data(), n * sizeof(double), cudaMemcpyHostToDevice, c.stream));
  UCC_CUDA(cudaStreamSynchronize(c.stream));
}

static const char* kStored[] = {"oooo", "ooov", "oovv", "ovov", "ovvv", "vvvv"};

static void build_L_blocks(Ctx& c) {
  const int no = c.no, nv = c.nv;
  auto two_minus = [&](const char* name, const Tensor& X, const Tensor& Xswap) {
    std::vector<int64_t> dims(X.d, X.d + X.rank);
    Tensor out = c.alloc(name, dims, false);
    permute_add(c, Xswap, -1.0, 0.0, out);
    permute_add(c, X, 2.0, 1.0, out);
  };
  Tensor Voovv = c.get("Voovv"), Vooov = c.get("Vooov"), Vovvv = c.get("Vovvv"), Vovov = c.get("Vovov");
  two_minus("Loovv", Voovv, view(Voovv, "ijab->ijba"));
  two_minus("Looov", Vooov, view(Vooov, "mnie->nmie"));
  two_minus("Lovvv", Vovvv, view(Vovvv, "mafe->maef"));
  // L[n,a,f,i] = 2 <ni|fa> - <na|if>
  two_minus("Lovvo", view(Voovv, "nifa->nafi"), view(Vovov, "naif->nafi"));
  (void)no;
  (void)nv;
}

void load_from_ints(Ctx& c, int no, int nv, const double* fock, const double* ints) {
  c.no = no;
  c.nv = nv;
  c.naux = 0;
  store_fock(c, fock);
  const int64_t n = no + nv;
  for (const char* blk : kStored) {
    int64_t lo[4], len[4];
    for (int k = 0; k < 4; k++) {
      lo[k] = blk[k] == 'o' ? 0 : no;
      len[k] = blk[k] == 'o' ? no : nv;
    }
    std::vector<double> h((size_t)len[0] * len[1] * len[2] * len[3]);
    size_t w = 0;
    for (int64_t p = 0; p < len[0]; p++)
      for (int64_t q = 0; q < len[1]; q++)
        for (int64_t r = 0; r < len[2]; r++) {
          const double* src = ints + (((lo[0] + p) * n + lo[1] + q) * n + lo[2] + r) * n + lo[3];
          std::memcpy(&h[w], src, sizeof(double) * len[3]);
          w += len[3];
        }
    Tensor t = c.alloc(std::string("V") + blk, {len[0], len[1], len[2], len[3]}, false);
    UCC_CUDA(cudaMemcpyAsync(t.p, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    UCC_CUDA(cudaStreamSynchronize(c.stream));
  }
  build_L_blocks(c);
  UCC_CUDA(cudaStreamSynchronize(c.stream));
}

void load_from_df(Ctx& c, int no, int nv, int naux, const double* fock, const double* Bh) {
  c.no = no;
  c.nv = nv;
  c.naux = naux;
  store_fock(c, fock);
  const int64_t n = no + nv;
  Tensor B = c.alloc("Bdf", {naux, n, n}, false);
  UCC_CUDA(cudaMemcpyAsync(B.p, Bh, sizeof(double) * naux * n * n, cudaMemcpyHostToDevice, c.stream));
  const bool saved = c.force_fp64;
  c.force_fp64 = true;  // the Hamiltonian itself is always built in FP64
  for (const char* blk : kStored) {
    int64_t lo[4], len[4];
    for (int k = 0; k < 4; k++) {
      lo[k] = blk[k] == 'o' ? 0 : no;
      len[k] = blk[k] == 'o' ? no : nv;
    }
    Tensor X = c.alloc(std::string("V") + blk, {len[0], len[1], len[2], len[3]}, false);
    // <pq|rs> = (pr|qs) = sum_Q B[Q,p,r] B[Q,q,s], chunked over p to bound the scratch
    const int64_t per_p = len[1] * len[2] * len[3];
    const int64_t chunk = std::max<int64_t>(1, std::min<int64_t>(len[0], (int64_t)(256LL << 20) / per_p));
    Tensor Bqs = narrow(narrow(B, 1, lo[1], len[1]), 2, lo[3], len[3]);
    for (int64_t p0 = 0; p0 < len[0]; p0 += chunk) {
      const int64_t np = std::min(chunk, len[0] - p0);
      Tensor Bpr = narrow(narrow(B, 1, lo[0] + p0, np), 2, lo[2], len[2]);
      Tensor Xc = narrow(X, 0, p0, np);
      contract(c, "Qpr,Qqs->pqrs", 1.0, Bpr, Bqs, 0.0, Xc);
    }
  }
  c.force_fp64 = saved;
  c.drop("Bdf");
  build_L_blocks(c);
  UCC_CUDA(cudaStreamSynchronize(c.stream));
}

Tensor V(Ctx& c, const std::string& b) {
  for (const char* s : kStored)
    if (b == s) return c.get("V" + b);
  if (b == "oovo") return view(c.get("Vooov"), "nmje->mnej");
  if (b == "ovvo") return view(c.get("Voovv"), "mjeb->mbej");
  if (b == "ovoo") return view(c.get("Vooov"), "mjib->mbij");
  if (b == "vovv") return view(c.get("Vovvv"), "mafe->amef");
  if (b == "vvvo") return view(c.get("Vovvv"), "iabe->abei");
  if (b == "vovo") return view(c.get("Vovov"), "maie->amei");
  if (b == "voov") return view(c.get("Voovv"), "mieb->bmie");
  throw Error(UCC_BAD_ARGS, "no integral block " + b);
}

Tensor L(Ctx& c, const std::string& b) {
  if (b == "oovv" || b == "ooov" || b == "ovvv" || b == "ovvo") return c.get("L" + b);
  if (b == "oovo") return view(c.get("Looov"), "mnie->nmei");
  if (b == "vovv") return view(c.get("Lovvv"), "mafe->amef");
  throw Error(UCC_BAD_ARGS, "no L block " + b);
}

Tensor Fk(Ctx& c, const std::string& b) { return c.get("f" + b); }

// ---------------------------------------------------------------------------------------
// DIIS
// ---------------------------------------------------------------------------------------
Diis::Diis(Ctx& c, int64_t n, int nmax)
    : c_(c), n_(n), nmax_(nmax), err_((size_t)n * nmax), vec_((size_t)n * nmax), B_((size_t)nmax * nmax, 0.0) {
  UCC_CUDA(cudaMalloc(&d_errp_, sizeof(double*) * nmax));
  UCC_CUDA(cudaMalloc(&d_vecp_, sizeof(double*) * nmax));
  std::vector<const double*> e(nmax), v(nmax);
  for (int p = 0; p < nmax; p++) {
    e[p] = err_.p + (size_t)p * n;
    v[p] = vec_.p + (size_t)p * n;
  }
  UCC_CUDA(cudaMemcpy(d_errp_, e.data(), sizeof(double*) * nmax, cudaMemcpyHostToDevice));
  UCC_CUDA(cudaMemcpy(d_vecp_, v.data(), sizeof(double*) * nmax, cudaMemcpyHostToDevice));
}

Diis::~Diis() {
  cudaFree(d_errp_);
  cudaFree(d_vecp_);
}

void Diis::add(const double* vnew, const double* vold) {
  const int slot = count_ < nmax_ ? count_ : (int)(nadded_ % nmax_);
  double* e = err_.p + (size_t)slot * n_;
  double* v = vec_.p + (size_t)slot * n_;
  axpby(c_, n_, 1.0, vnew, 0.0, e);
  axpby(c_, n_, -1.0, vold, 1.0, e);
  UCC_CUDA(cudaMemcpyAsync(v, vnew, sizeof(double) * n_, cudaMemcpyDeviceToDevice, c_.stream));
  const int cnt = std::min(count_ + 1, nmax_);
  Scratch d(c_, sizeof(double) * nmax_);
  multidot_async(c_, cnt, d_errp_, e, n_, d.d());
  std::vector<double> row(cnt);
  UCC_CUDA(cudaMemcpyAsync(row.data(), d.p, sizeof(double) * cnt, cudaMemcpyDeviceToHost, c_.stream));
  UCC_CUDA(cudaStreamSynchronize(c_.stream));
  for (int p = 0; p < cnt; p++) B_[(size_t)slot * nmax_ + p] = B_[(size_t)p * nmax_ + slot] = row[p];
  count_ = cnt;
  nadded_++;
}

std::vector<double> diis_coefficients(const std::vector<double>& Bin, int n) {
  const int m = n + 1;
  std::vector<double> B((size_t)m * m, 0.0), c(m, 0.0);
  double mx = 0.0;
  for (int p = 0; p < n; p++)
    for (int q = 0; q < n; q++) {
      B[p * m + q] = Bin[(size_t)p * n + q];
      mx = std::max(mx, std::fabs(B[p * m + q]));
    }
  if (mx > 0.0)
    for (int p = 0; p < n; p++)
      for (int q = 0; q < n; q++) B[p * m + q] /= mx;
  for (int p = 0; p < n; p++) B[p * m + n] = B[n * m + p] = -1.0;
  B[n * m + n] = 0.0;
  c[n] = -1.0;
  for (int col = 0; col < m; col++) {
    int piv = col;
    for (int r = col + 1; r < m; r++)
      if (std::fabs(B[r * m + col]) > std::fabs(B[piv * m + col])) piv = r;
    if (piv != col) {
      for (int k = 0; k < m; k++) std::swap(B[col * m + k], B[piv * m + k]);
      std::swap(c[col], c[piv]);
    }
    const double d = B[col * m + col];
    UCC_REQUIRE(d != 0.0, UCC_NAN_DETECTED, "DIIS: singular B matrix");
    for (int r = col + 1; r < m; r++) {
      const double f = B[r * m + col] / d;
      if (f == 0.0) continue;
      for (int k = col; k < m; k++) B[r * m + k] -= f * B[col * m + k];
      c[r] -= f * c[col];
    }
  }
  for (int r = m - 1; r >= 0; r--) {
    double s = c[r];
    for (int k = r + 1; k < m; k++) s -= B[r * m + k] * c[k];
    c[r] = s / B[r * m + r];
  }
  c.resize(n);
  return c;
}

void Diis::reset() {
  count_ = 0;
  nadded_ = 0;
  std::fill(B_.begin(), B_.end(), 0.0);
}

void Diis::extrapolate(double* out) {
  const int n = count_;
  std::vector<double> Bn((size_t)n * n);
  for (int p = 0; p < n; p++)
    for (int q = 0; q < n; q++) Bn[(size_t)p * n + q] = B_[(size_t)p * nmax_ + q];
  std::vector<double> coef = diis_coefficients(Bn, n);
  lincomb(c_, n, d_vecp_, coef.data(), n_, out);
}

// ---------------------------------------------------------------------------------------
// CCSD (ccwfn.cc:188-626)
// ---------------------------------------------------------------------------------------
double flops_ccsd_iter(double no, double nv) {
  return 2.0 * (no * no * nv * nv * nv * nv + 2.0 * no * no * no * no * nv * nv + 10.0 * no * no * no * nv * nv * nv +
                8.0 * no * no * nv * nv * nv);
}

namespace {

struct Amps {  // views of the packed [t1 | t2] buffers
  Tensor t1, t2;
};

void copy_into(Ctx& c, const Tensor& src, Tensor dst) { permute_add(c, src, 1.0, 0.0, dst); }

// build_F, ccwfn.cc:311-356
void build_F(Ctx& c, const Tensor& t1, const Tensor& ttau) {
  Tensor Fvv = c.get("Fvv"), Foo = c.get("Foo"), Fov = c.get("Fov");
  copy_into(c, Fk(c, "vv"), Fvv);
  contract(c, "me,ma->ae", -0.5, Fk(c, "ov"), t1, 1.0, Fvv);
  contract(c, "mf,mafe->ae", 1.0, t1, L(c, "ovvv"), 1.0, Fvv);
  contract(c, "mnaf,mnef->ae", -1.0, ttau, L(c, "oovv"), 1.0, Fvv);
  copy_into(c, Fk(c, "oo"), Foo);
  contract(c, "ie,me->mi", 0.5, t1, Fk(c, "ov"), 1.0, Foo);
  contract(c, "ne,mnie->mi", 1.0, t1, L(c, "ooov"), 1.0, Foo);
  contract(c, "inef,mnef->mi", 1.0, ttau, L(c, "oovv"), 1.0, Foo);
  copy_into(c, Fk(c, "ov"), Fov);
  contract(c, "nf,mnef->me", 1.0, t1, L(c, "oovv"), 1.0, Fov);
}

// build_W, ccwfn.cc:358-430
void build_W(Ctx& c, const Tensor& t1, const Tensor& t2, const Tensor& tau) {
  const int no = c.no, nv = c.nv;
  Tensor Woooo = c.get("Woooo"), Wovov = c.get("Wovov"), Wovvo = c.get("Wovvo"), Zmbij = c.get("Zmbij");
  copy_into(c, V(c, "oooo"), Woooo);
  contract(c, "je,mnie->mnij", 1.0, t1, V(c, "ooov"), 1.0, Woooo);
  contract(c, "ie,mnej->mnij", 1.0, t1, V(c, "oovo"), 1.0, Woooo);
  contract(c, "ijef,mnef->mnij", 1.0, tau, V(c, "oovv"), 1.0, Woooo);
  Temp X(c, {no, no, nv, nv});
  if (!recorder()) {  // X = t2/2 + t1_jf t1_nb in one elementwise pass (as a K = 1 GEMM: DFMA tiles)
    build_tau(c, no, nv, t1.p, t2.p, 1.0, X->p, 0.0, nullptr, 0.5);
  } else {
    axpby(c, X->size(), 0.5, t2.p, 0.0, X->p);
    contract(c, "jf,nb->jnfb", 1.0, t1, t1, 1.0, X);
  }
  permute_add(c, V(c, "ovov"), -1.0, 0.0, Wovov);
  contract(c, "jf,mbfe->mbje", -1.0, t1, V(c, "ovvv"), 1.0, Wovov);
  contract(c, "nb,mnje->mbje", 1.0, t1, V(c, "ooov"), 1.0, Wovov);
  contract(c, "mnfe,jnfb->mbje", 1.0, V(c, "oovv"), X, 1.0, Wovov);
  copy_into(c, V(c, "ovvo"), Wovvo);
  contract(c, "jf,mbef->mbej", 1.0, t1, V(c, "ovvv"), 1.0, Wovvo);
  contract(c, "nb,mnej->mbej", -1.0, t1, V(c, "oovo"), 1.0, Wovvo);
  contract(c, "mnef,jnfb->mbej", -1.0, V(c, "oovv"), X, 1.0, Wovvo);
  contract(c, "mnef,njfb->mbej", 0.5, L(c, "oovv"), t2, 1.0, Wovvo);
  contract(c, "mbef,ijef->mbij", 1.0, V(c, "ovvv"), tau, 0.0, Zmbij);
}

// build_t1, ccwfn.cc:432-469 (unscaled residual)
void build_t1(Ctx& c, const Tensor& t1, const Tensor& t2, Tensor R1) {
  const int no = c.no, nv = c.nv;
  transpose_add(c, "ai->ia", 1.0, Fk(c, "vo"), 0.0, R1);
  contract(c, "ie,ae->ia", 1.0, t1, c.get("Fvv"), 1.0, R1);
  contract(c, "ma,mi->ia", -1.0, t1, c.get("Foo"), 1.0, R1);
  Temp t2x(c, {no, no, nv, nv});
  transpose_add(c, "ijab->ijba", -1.0, t2, 0.0, t2x);
  axpby(c, t2x->size(), 2.0, t2.p, 1.0, t2x->p);
  contract(c, "imae,me->ia", 1.0, t2x, c.get("Fov"), 1.0, R1);
  contract(c, "nf,nafi->ia", 1.0, t1, L(c, "ovvo"), 1.0, R1);
  contract(c, "mief,maef->ia", 1.0, t2x, V(c, "ovvv"), 1.0, R1);
  contract(c, "mnae,nmei->ia", -1.0, t2, L(c, "oovo"), 1.0, R1);
}

// build_t2, ccwfn.cc:471-539 (unscaled residual).
//
// The residual is symmetric under the simultaneous swap (i<->j, a<->b): the reference
// computes each term and its swapped partner explicitly.  Here one member of each pair
// goes into a half residual Rh and R2 = <ij|ab> + Woooo.tau + ladder + Rh + Rh(ji,ba);
// <ij|ab>, the hole ladder and the particle ladder are symmetric on their own.
//
}  // namespace

// R2 += alpha sum_ef W_abef amp_ijef on packed pairs (kernels_fp64.cu): S = Tp Vp^T over
// (i<=j, a<=b, e<=f), A = Tm Vm^T over strict pairs, a quarter of the multiply-adds of the
// plain contraction; amp must be invariant under (i,j,e,f) -> (j,i,f,e).  The packed
// operator (names vp_name / vm_name, constant blocks) is built from block `src` once.
void packed_ladder(Ctx& c, double alpha, const Tensor& amp, const char* src, int mode, const char* vp_name,
                   const char* vm_name, double* R2) {
  const int no = c.no, nv = c.nv;
  const int64_t op = (int64_t)no * (no + 1) / 2, om = (int64_t)no * (no - 1) / 2;
  const int64_t vp = (int64_t)nv * (nv + 1) / 2, vm = (int64_t)nv * (nv - 1) / 2;
  if (!c.has(vp_name)) {
    Tensor Vp = c.alloc(vp_name, {vp, vp}, false), Vm = c.alloc(vm_name, {vm, vm}, false);
    pack_vvvv(c, nv, mode, c.get(src).p, Vp.p, Vm.p);
  }
  UCC_REQUIRE(amp.dense(), UCC_BAD_ARGS, "packed ladder: dense amplitudes");
  Temp Tp(c, {op, vp}), Tm(c, {om, vm}), S(c, {op, vp}), A(c, {om, vm});
  pack_tau(c, no, nv, amp.p, Tp->p, Tm->p);
  contract(c, "pe,qe->pq", 1.0, Tp, c.get(vp_name), 0.0, S);
  contract(c, "pe,qe->pq", 1.0, Tm, c.get(vm_name), 0.0, A);
  unpack_ladder(c, no, nv, alpha, S->p, A->p, R2);
}

namespace {

// particle ladder sum_ef <ab|ef> tau_ijef, ccwfn.cc:508-510.  Outside a recorded batch it
// runs on packed pairs: S = Tp Vp^T over (i<=j, a<=b, e<=f) and A = Tm Vm^T over strict
// pairs, a quarter of the multiply-adds (the result is symmetric under the simultaneous
// swap (i,j,a,b) -> (j,i,b,a) and the integrals under (a,b,e,f) -> (b,a,f,e))
void ladder(Ctx& c, const Tensor& tau, const Tensor& R2) {
  if (recorder() || c.no < 2 || c.nv < 2) {
    contract(c, "ijef,abef->ijab", 1.0, tau, V(c, "vvvv"), 1.0, R2);
    return;
  }
  packed_ladder(c, 1.0, tau, "Vvvvv", 0, "Vpp", "Vmm", R2.p);
}

void build_t2(Ctx& c, const Tensor& t1, const Tensor& t2, const Tensor& tau, Tensor R2, std::vector<cudaEvent_t>* ev) {
  const int no = c.no, nv = c.nv;
  Tensor Fvv = c.get("Fvv"), Foo = c.get("Foo"), Fov = c.get("Fov");
  Tensor Woooo = c.get("Woooo"), Wovov = c.get("Wovov"), Wovvo = c.get("Wovvo"), Zmbij = c.get("Zmbij");
  copy_into(c, V(c, "oovv"), R2);
  contract(c, "mnab,mnij->ijab", 1.0, tau, Woooo, 1.0, R2);
  if (ev) {
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a, c.stream);
    ladder(c, tau, R2);
    cudaEventRecord(b, c.stream);
    ev->push_back(a);
    ev->push_back(b);
  } else {
    ladder(c, tau, R2);
  }
  Temp Rh(c, {no, no, nv, nv});
  contract(c, "ijae,be->ijab", 1.0, t2, Fvv, 0.0, Rh);
  {
    Temp tF(c, {nv, nv});
    contract(c, "mb,me->be", 1.0, t1, Fov, 0.0, tF);
    contract(c, "ijae,be->ijab", -0.5, t2, tF, 1.0, Rh);
    Temp tF2(c, {no, no});
    contract(c, "je,me->mj", 1.0, t1, Fov, 0.0, tF2);
    axpby(c, tF2->size(), 0.5, tF2->p, 0.0, tF2->p);
    axpby(c, Foo.size(), 1.0, Foo.p, 1.0, tF2->p);  // Foo + tF2 / 2
    contract(c, "imab,mj->ijab", -1.0, t2, tF2, 1.0, Rh);
  }
  contract(c, "ie,abej->ijab", 1.0, t1, V(c, "vvvo"), 1.0, Rh);
  contract(c, "ma,mbij->ijab", -1.0, t1, V(c, "ovoo"), 1.0, Rh);
  {
    // (t2 - t2(ba)) Wovvo + t2 (Wovvo + Wovov(..je->..ej)) = (2 t2 - t2(ba)) Wovvo + t2 Wovov^T
    Temp t2x(c, {no, no, nv, nv});
    transpose_add(c, "ijab->ijba", -1.0, t2, 0.0, t2x);
    axpby(c, t2x->size(), 2.0, t2.p, 1.0, t2x->p);
    contract(c, "imae,mbej->ijab", 1.0, t2x, Wovvo, 1.0, Rh);
    contract(c, "imae,mbje->ijab", 1.0, t2, Wovov, 1.0, Rh);
  }
  contract(c, "mjae,mbie->ijab", 1.0, t2, Wovov, 1.0, Rh);
  {
    // Za[m,b,i,j] = Zmbij + t1[i,e] <mb|ej> + t1[j,e] <mb|ie>  ->  - t1[m,a] Za[m,b,i,j]
    Temp Za(c, {no, nv, no, no});
    copy_into(c, Zmbij, Za);
    contract(c, "ie,mbej->mbij", 1.0, t1, V(c, "ovvo"), 1.0, Za);
    contract(c, "je,mbie->mbij", 1.0, t1, V(c, "ovov"), 1.0, Za);
    contract(c, "ma,mbij->ijab", -1.0, t1, Za, 1.0, Rh);
  }
  axpby(c, Rh->size(), 1.0, Rh->p, 1.0, R2.p);
  transpose_add(c, "jiba->ijab", 1.0, Rh, 1.0, R2);
}

double energy(Ctx& c, const Tensor& t1, const Tensor& tau) {
  const int no = c.no, nv = c.nv, n = no + nv;
  // ccwfn.cc:270-273 assigns instead of accumulating: only the last (i,a) pair counts
  double t1last = 0.0;
  UCC_CUDA(cudaMemcpyAsync(&t1last, t1.p + (int64_t)no * nv - 1, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
  const double two = dot_all(c, tau, L(c, "oovv"));
  const double one = 2.0 * c.fock[(size_t)(no - 1) * n + (n - 1)] * t1last;
  return one + two;
}

}  // namespace

// CCSD work arrays of one context (amplitudes packed as [t1 | t2])
void ccsd_alloc(Ctx& c) {
  const int no = c.no, nv = c.nv;
  const int64_t np = npacked(c);
  c.alloc("T", {np}, false);
  c.alloc("Told", {np}, true);
  c.alloc("R", {np}, false);
  c.alloc("tau", {no, no, nv, nv}, false);
  c.alloc("ttau", {no, no, nv, nv}, false);
  c.alloc("Fvv", {nv, nv}, false);
  c.alloc("Foo", {no, no}, false);
  c.alloc("Fov", {no, nv}, false);
  c.alloc("Woooo", {no, no, no, no}, false);
  c.alloc("Wovov", {no, nv, no, nv}, false);
  c.alloc("Wovvo", {no, nv, nv, no}, false);
  c.alloc("Zmbij", {no, nv, no, no}, false);
}

// the unscaled residual R(t_old) into r, given tau/ttau of t_old (ccwfn.cc:311-539)
void ccsd_residual(Ctx& c, const double* t_old, double* r) {
  Tensor t1 = amp1(c, const_cast<double*>(t_old)), t2 = amp2(c, const_cast<double*>(t_old));
  build_F(c, t1, c.get("ttau"));
  build_W(c, t1, t2, c.get("tau"));
  build_t1(c, t1, t2, amp1(c, r));
  build_t2(c, t1, t2, c.get("tau"), amp2(c, r), nullptr);
}

double ccsd_energy(Ctx& c, const double* t) { return energy(c, amp1(c, const_cast<double*>(t)), c.get("tau")); }

// residual norm near which BF16 hi+lo split products with FP32 accumulation stop
// resolving the update (measured ~1.5e-6 at no=16/nv=160)
constexpr double kMixedFloor = 2e-6;
// delta sweeps resolve residuals down to ~3e-5 of their anchor's residual (measured at
// no=32/nv=320: an anchor at 4.3e-5 left the delta residuals 1.3e-9 off), so an anchor
// above kReanchor * r_convergence is re-taken once the deltas reach that level
constexpr double kReanchor = 1e4;

MixedSweeps::MixedSweeps(Ctx& c)
    : c_(c),
      mixed_(c.opt.precision == UCC_MIXED),
      refine_(c.opt.precision == UCC_MIXED && c.opt.refine_sweeps > 0),
      split_phase_(c.opt.precision == UCC_MIXED) {
  c_.anchors.clear();
}

MixedSweeps::~MixedSweeps() { c_.anchors.clear(); }

// Truncating each operand to S base-2^6 digits leaves a relative error near 2^-6S in every
// product term; the digits cover the target level's bits plus a margin of kDigitMarginBits
// for the sum over K and the spread of the operands' magnitudes (an anchor error shows as a
// delta residual that stalls above the target, which re-anchors with all digits).
constexpr int kDigitMarginBits = 14;

int MixedSweeps::record_digits() const {
  if (!(record_target_ > 0.0)) return 9;
  const int d = (int)std::ceil((std::log2(1.0 / record_target_) + kDigitMarginBits) / 6.0);
  return std::min(9, std::max(4, d));
}

MixedSweeps::Kind MixedSweeps::begin() {
  kind_ = !mixed_ ? kFp64 : split_phase_ ? kSplit : record_next_ ? kRecord : kDelta;
  if (kind_ == kRecord) {
    c_.anchors.begin(1);
    digits_ = record_digits();
    c_.anchors.digits = digits_;
  }
  if (kind_ == kDelta) c_.anchors.begin(2);
  return kind_;
}

void MixedSweeps::end() {
  c_.anchors.mode = 0;
  c_.anchors.digits = 9;
}

bool MixedSweeps::after(double rms, bool* restart_diis) {
  *restart_diis = false;
  sweeps_++;
  const double rc = c_.opt.r_convergence;
  bool done = false;
  if (kind_ == kFp64) {
    done = rms < rc;
  } else if (kind_ == kSplit) {
    split++;
    if (!refine_ && rms < rc) done = true;
    // hand over near the split-product noise floor, or when the residual stops falling
    // within three decades of it: two sweeps in a row that do not halve it (one slow sweep
    // is common early on: from a learned guess at no=32/nv=320 the norm went 1.0e-2 ->
    // 5.3e-3, and handing over there left 10 delta sweeps to do instead of 7)
    const double level = std::max(rc, std::max(c_.opt.mixed_switch, kMixedFloor));
    split_slow_ = (sweeps_ > 2 && rms < 1e3 * level && rms > 0.5 * rms_prev_) ? split_slow_ + 1 : 0;
    if (!done && refine_ && (rms < level || split_slow_ >= 2)) {
      split_phase_ = false;
      record_next_ = true;
      // the deltas after this anchor run down to the re-anchoring level, or to r_convergence
      record_target_ = rms > kReanchor * rc ? kReanchor * rc : rc;
      *restart_diis = true;  // the split-sweep history extrapolates a different map
    }
  } else if (kind_ == kRecord) {
    record++;
    record_next_ = false;
    stalls_ = 0;
    anchor_rms_ = rms;
    // only a residual from products with all digits ends the solve
    done = rms < rc && record >= c_.opt.refine_sweeps && digits_ == 9;
    if (!done && rms < rc && digits_ < 9) {
      record_next_ = true;
      record_target_ = 0.0;
    }
    // the FP64 residual is well above what the last delta sweep reported: those sweeps'
    // anchor was too far away and their vectors would mislead the extrapolation
    if (!done && last_ == kDelta && rms > 2.0 * rms_prev_) *restart_diis = true;
  } else {
    delta++;
    if (rms < rc) {
      record_next_ = true;  // confirm with an FP64 residual
      record_target_ = 0.0;
    } else if (anchor_rms_ > kReanchor * rc && rms < kReanchor * rc) {
      record_next_ = true;  // the anchor is too far for the deltas to resolve rc: re-anchor here
      record_target_ = rc;
    } else if (rms > 0.7 * rms_prev_) {
      if (++stalls_ >= 2) {  // corrections no longer resolved: re-anchor
        record_next_ = true;
        record_target_ = 0.0;
      }
    } else {
      stalls_ = 0;
    }
  }
  rms_prev_ = rms;
  last_ = kind_;
  return done;
}

CCSDResult run_ccsd(Ctx& c) {
  UCC_REQUIRE(c.loaded, UCC_BAD_STATE, "no Hamiltonian loaded");
  const int no = c.no, nv = c.nv;
  const int64_t np = npacked(c);
  ccsd_alloc(c);
  Tensor T = c.get("T"), Told = c.get("Told");
  Tensor eps = c.get("eps");
  const double* d_do = eps.p;
  const double* d_dv = eps.p + no;
  Scratch sumsq(c, sizeof(double));

  // MP2 guess t1 = f_ia / D1, t2 = <ij|ab> / D2 (ccwfn.cc:75-87), unless amplitudes were given
  if (!c.has("T_guess")) {
    Temp R0(c, {np}, true);
    copy_into(c, Fk(c, "ov"), amp1(c, R0->p));
    copy_into(c, V(c, "oovv"), amp2(c, R0->p));
    jacobi_update(c, no, nv, d_do, d_dv, 0.0, R0->p, R0->p + (int64_t)no * nv, Told.p, Told.p + (int64_t)no * nv, T.p,
                  T.p + (int64_t)no * nv, sumsq.d());
  } else {  // a supplied guess (restart file, learned guess) applies to this solve only
    UCC_CUDA(cudaMemcpyAsync(T.p, c.get("T_guess").p, sizeof(double) * np, cudaMemcpyDeviceToDevice, c.stream));
    UCC_CUDA(cudaStreamSynchronize(c.stream));
    c.drop("T_guess");
  }
  auto tau_of = [&](double* buf) {
    build_tau(c, no, nv, buf, buf + (int64_t)no * nv, 1.0, c.get("tau").p, 0.5, c.get("ttau").p);
  };
  tau_of(c.get("T").p);
  CCSDResult res;
  res.e_mp2 = energy(c, amp1(c, c.get("T").p), c.get("tau"));
  if (c.opt.print) {
    std::printf("\n\tThe Coupled-Cluster Iteration:\n");
    std::printf("\t---------------------------------------------------\n");
    std::printf("\t Iter   Correlation Energy   T1 Norm      RMS   \n");
    std::printf("\t---------------------------------------------------\n");
    std::printf("\t  %3d  %20.15f\n", 0, res.e_mp2);
  }
  Diis diis(c, np, 8);
  std::vector<cudaEvent_t> ev;
  double rms = INFINITY, eccsd = NAN;
  MixedSweeps sw(c);  // mixed precision: split, record and delta sweeps (cc.h)
  const bool mixed = sw.mixed();
  bool converged = false;
  int iter = 0;
  auto t_prev = std::chrono::steady_clock::now();  // printed sweep times (the loop synchronises each sweep)
  for (iter = 1; iter <= c.opt.maxiter; iter++) {
    c.store["T"].swap(c.store["Told"]);  // amp_save, ccwfn.cc:300-309
    double* to = c.get("Told").p;
    double* tn = c.get("T").p;
    double* r = c.get("R").p;
    Tensor t1 = amp1(c, to), t2 = amp2(c, to);
    const MixedSweeps::Kind kind = sw.begin();
    {
      Fp64Scope scope(c, kind != MixedSweeps::kSplit);
      build_F(c, t1, c.get("ttau"));
      build_W(c, t1, t2, c.get("tau"));
      build_t1(c, t1, t2, amp1(c, r));
      build_t2(c, t1, t2, c.get("tau"), amp2(c, r), &ev);
    }
    sw.end();
    if (kind == MixedSweeps::kSplit || kind == MixedSweeps::kDelta) {
      // The exact residual is symmetric under (i,j,a,b) -> (j,i,b,a); rounding of the
      // tensor-core products is not.  In the antisymmetric sector the Fock terms cancel
      // and the Jacobi step does not damp, so project the noise out of R2.
      Tensor R2 = amp2(c, r);
      Temp S(c, {no, no, nv, nv});
      transpose_add(c, "ijab->jiba", 1.0, R2, 0.0, S);
      axpby(c, S->size(), 0.5, S->p, 0.5, R2.p);
    }
    double noise = -1.0, drift = -1.0;
    if (c.opt.print >= 2 && mixed) {
      // diagnostics: distance of this residual from the FP64 one at the same amplitudes,
      // and of the amplitudes from the last anchor
      if (kind == MixedSweeps::kRecord) {
        c.alloc("T_anchor", {np}, false);
        UCC_CUDA(cudaMemcpyAsync(c.get("T_anchor").p, to, sizeof(double) * np, cudaMemcpyDeviceToDevice, c.stream));
      } else {
        Temp Rx(c, {np});
        {
          Fp64Scope f(c);
          ccsd_residual(c, to, Rx->p);
        }
        axpby(c, np, -1.0, r, 1.0, Rx->p);
        noise = std::sqrt(dot(c, np, Rx->p, Rx->p));
        if (kind == MixedSweeps::kDelta) {
          axpby(c, np, 1.0, to, 0.0, Rx->p);
          axpby(c, np, -1.0, c.get("T_anchor").p, 1.0, Rx->p);
          drift = std::sqrt(dot(c, np, Rx->p, Rx->p));
        }
      }
    }
    jacobi_update(c, no, nv, d_do, d_dv, 0.0, r, r + (int64_t)no * nv, to, to + (int64_t)no * nv, tn,
                  tn + (int64_t)no * nv, sumsq.d());
    double ss = 0.0;
    UCC_CUDA(cudaMemcpyAsync(&ss, sumsq.p, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    UCC_CUDA(cudaStreamSynchronize(c.stream));
    rms = std::sqrt(ss);
    tc_check(c);
    UCC_REQUIRE(std::isfinite(rms), UCC_NAN_DETECTED, "CCSD residual is not finite");
    bool restart = false;
    if (sw.after(rms, &restart)) {
      converged = true;
      break;
    }
    if (restart) diis.reset();
    if (c.opt.diis && !restart) {
      diis.add(tn, to);
      if (diis.size() > 2) diis.extrapolate(tn);
    }
    tau_of(tn);
    eccsd = energy(c, amp1(c, tn), c.get("tau"));
    if (c.opt.print) {
      double t1n = std::sqrt(dot(c, (int64_t)no * nv, tn, tn) / (2 * no));
      static const char* tag[] = {"", " split", " record", " delta"};
      const auto t_now = std::chrono::steady_clock::now();
      const double ms = std::chrono::duration<double, std::milli>(t_now - t_prev).count();
      t_prev = t_now;
      std::printf("\t  %3d  %20.15f  %8.6f  %8.6e%s", iter, eccsd, t1n, rms, tag[kind]);
      if (mixed) std::printf("  %8.1f ms", ms);
      if (noise >= 0.0) std::printf("  |R-R64| %.3e", noise);
      if (drift >= 0.0) std::printf("  |T-T0| %.3e", drift);
      std::printf("\n");
    }
  }
  if (c.has("T_anchor")) c.drop("T_anchor");
  c.stats.mixed_iterations = sw.split;
  c.stats.anchored_iterations = sw.delta;
  const int fp64_iters = mixed ? sw.record : std::min(iter, c.opt.maxiter);
  tau_of(c.get("T").p);
  UCC_CUDA(cudaStreamSynchronize(c.stream));
  for (size_t k = 0; k + 1 < ev.size(); k += 2) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ev[k], ev[k + 1]);
    c.stats.ladder_ms += ms;
    c.stats.ladder_launches += 1;
    const double o = no, v = nv;
    c.stats.ladder_flops += 2.0 * o * o * v * v * v * v;
    c.stats.ladder_bytes += 8.0 * (v * v * v * v + 3.0 * o * o * v * v);
    cudaEventDestroy(ev[k]);
    cudaEventDestroy(ev[k + 1]);
  }
  res.iterations = std::min(iter, c.opt.maxiter);
  res.e_ccsd = eccsd;
  res.converged = converged;
  c.stats.fp64_iterations = fp64_iters;
  c.have_ccsd = res.converged;
  c.have_tgrad = false;  // new amplitudes: earlier (T) gradient pieces no longer apply
  return res;
}

}  // namespace ucc
