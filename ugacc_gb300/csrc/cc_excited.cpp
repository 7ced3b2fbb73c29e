// HBAR (hbar.cc:8-228), Lambda (cclambda.cc:13-311) and the one- and two-particle
// densities (ccdensity.cc:89-339).  Products of three or more amplitudes/integrals are
// evaluated as sequences of pairwise contractions through small intermediates, which
// turns the reference's O(no^4 nv^4) loops (e.g. Goovv, ccdensity.cc:301-325) into
// O(no^3 nv^3) work.
#include <cmath>
#include <cstdio>

#include "cc.h"

namespace ucc {

namespace {
void copy_into(Ctx& c, const Tensor& src, Tensor dst) { permute_add(c, src, 1.0, 0.0, dst); }
using V4 = std::vector<int64_t>;
}  // namespace

void run_hbar(Ctx& c) {
  UCC_REQUIRE(c.have_ccsd, UCC_BAD_STATE, "HBAR needs converged CCSD amplitudes");
  Fp64Scope fp64(c);  // HBAR, Lambda, densities and response run in FP64
  // the tensor-core operand caches key on block addresses, and the H blocks are rewritten
  // in place
  UCC_CUDA(cudaStreamSynchronize(c.stream));
  c.tc_cache.reset();
  const int no = c.no, nv = c.nv;
  double* T = c.get("T").p;
  Tensor t1 = amp1(c, T), t2 = amp2(c, T), tau = c.get("tau");
  Tensor fov = Fk(c, "ov");

  Tensor Hov = c.alloc("Hov", {no, nv}, false);  // :36-43
  copy_into(c, fov, Hov);
  contract(c, "nf,mnef->me", 1.0, t1, L(c, "oovv"), 1.0, Hov);

  Tensor Hoo = c.alloc("Hoo", {no, no}, false);  // :45-57
  copy_into(c, Fk(c, "oo"), Hoo);
  contract(c, "ie,me->mi", 1.0, t1, fov, 1.0, Hoo);
  contract(c, "ne,mnie->mi", 1.0, t1, L(c, "ooov"), 1.0, Hoo);
  contract(c, "inef,mnef->mi", 1.0, tau, L(c, "oovv"), 1.0, Hoo);

  Tensor Hvv = c.alloc("Hvv", {nv, nv}, false);  // :59-71
  copy_into(c, Fk(c, "vv"), Hvv);
  contract(c, "me,ma->ae", -1.0, fov, t1, 1.0, Hvv);
  contract(c, "mf,amef->ae", 1.0, t1, L(c, "vovv"), 1.0, Hvv);
  contract(c, "mnfa,mnfe->ae", -1.0, tau, L(c, "oovv"), 1.0, Hvv);

  Tensor Hoooo = c.alloc("Hoooo", {no, no, no, no}, false);  // :73-84
  copy_into(c, V(c, "oooo"), Hoooo);
  contract(c, "je,mnie->mnij", 2.0, t1, V(c, "ooov"), 1.0, Hoooo);
  contract(c, "ijef,mnef->mnij", 1.0, tau, V(c, "oovv"), 1.0, Hoooo);

  for (const char* k : {"Hpp1", "Hmm1", "Hpp2", "Hmm2"}) c.drop(k);  // packed ladders of the previous HBAR
  Tensor Hvvvv = c.alloc("Hvvvv", {nv, nv, nv, nv}, false);  // :86-97
  copy_into(c, V(c, "vvvv"), Hvvvv);
  contract(c, "mb,amef->abef", -2.0, t1, V(c, "vovv"), 1.0, Hvvvv);
  contract(c, "mnab,mnef->abef", 1.0, tau, V(c, "oovv"), 1.0, Hvvvv);

  Tensor Hvovv = c.alloc("Hvovv", {nv, no, nv, nv}, false);  // :99-107
  copy_into(c, V(c, "vovv"), Hvovv);
  contract(c, "na,nmef->amef", -1.0, t1, V(c, "oovv"), 1.0, Hvovv);

  Tensor Hooov = c.alloc("Hooov", {no, no, no, nv}, false);  // :109-117
  copy_into(c, V(c, "ooov"), Hooov);
  contract(c, "if,nmef->mnie", 1.0, t1, V(c, "oovv"), 1.0, Hooov);

  Tensor Hovvo = c.alloc("Hovvo", {no, nv, nv, no}, false);  // :119-135
  copy_into(c, V(c, "ovvo"), Hovvo);
  contract(c, "jf,mbef->mbej", 1.0, t1, V(c, "ovvv"), 1.0, Hovvo);
  contract(c, "nb,mnej->mbej", -1.0, t1, V(c, "oovo"), 1.0, Hovvo);
  contract(c, "mnef,njbf->mbej", -1.0, V(c, "oovv"), tau, 1.0, Hovvo);
  contract(c, "njfb,mnef->mbej", 1.0, t2, L(c, "oovv"), 1.0, Hovvo);

  Tensor Hovov = c.alloc("Hovov", {no, nv, no, nv}, false);  // :137-151
  copy_into(c, V(c, "ovov"), Hovov);
  contract(c, "jf,bmef->mbje", 1.0, t1, V(c, "vovv"), 1.0, Hovov);
  contract(c, "nb,mnje->mbje", -1.0, t1, V(c, "ooov"), 1.0, Hovov);
  contract(c, "nmef,jnfb->mbje", -1.0, V(c, "oovv"), tau, 1.0, Hovov);

  // shared intermediates of the three-amplitude terms
  Temp X1(c, {no, no, nv, no});   // X1[m,n,e,i] = <mn|ef> t1[i,f]
  contract(c, "mnef,if->mnei", 1.0, V(c, "oovv"), t1, 0.0, X1);
  Temp X2(c, {nv, no, nv, nv});   // X2[a,n,e,f] = t1[m,a] <mn|ef>
  contract(c, "ma,mnef->anef", 1.0, t1, V(c, "oovv"), 0.0, X2);
  Temp X3(c, {no, nv, nv, nv});   // X3[m,e,f,b] = <mn|ef> t1[n,b]
  contract(c, "mnef,nb->mefb", 1.0, V(c, "oovv"), t1, 0.0, X3);

  Tensor Hvvvo = c.alloc("Hvvvo", {nv, nv, nv, no}, false);  // :153-189
  copy_into(c, V(c, "vvvo"), Hvvvo);
  contract(c, "if,abef->abei", 1.0, t1, V(c, "vvvv"), 1.0, Hvvvo);
  contract(c, "mb,amei->abei", -1.0, t1, V(c, "vovo"), 1.0, Hvvvo);
  contract(c, "ma,bmie->abei", -1.0, t1, V(c, "voov"), 1.0, Hvvvo);
  contract(c, "imfa,mbef->abei", -1.0, tau, V(c, "ovvv"), 1.0, Hvvvo);
  contract(c, "imfb,amef->abei", -1.0, tau, V(c, "vovv"), 1.0, Hvvvo);
  contract(c, "mnab,mnei->abei", 1.0, tau, V(c, "oovo"), 1.0, Hvvvo);
  contract(c, "me,miab->abei", -1.0, fov, t2, 1.0, Hvvvo);
  contract(c, "mifb,amef->abei", 1.0, t2, L(c, "vovv"), 1.0, Hvvvo);
  contract(c, "mnei,mnab->abei", 1.0, X1, t2, 1.0, Hvvvo);
  contract(c, "anef,infb->abei", 1.0, X2, t2, 1.0, Hvvvo);
  contract(c, "mefb,miaf->abei", 1.0, X3, t2, 1.0, Hvvvo);
  {
    Temp X4(c, {no, nv});
    contract(c, "mf,mnfe->ne", 1.0, t1, L(c, "oovv"), 0.0, X4);
    contract(c, "niab,ne->abei", -1.0, t2, X4, 1.0, Hvvvo);
    Temp X5(c, {nv, no, nv, nv});
    contract(c, "na,mnfe->amfe", 1.0, t1, L(c, "oovv"), 0.0, X5);
    contract(c, "mifb,amfe->abei", -1.0, t2, X5, 1.0, Hvvvo);
    Temp W(c, {nv, no, nv, no});  // t1[m,a] X1[m,n,e,i]
    contract(c, "ma,mnei->anei", 1.0, t1, X1, 0.0, W);
    contract(c, "nb,anei->abei", 1.0, t1, W, 1.0, Hvvvo);
  }

  Tensor Hovoo = c.alloc("Hovoo", {no, nv, no, no}, false);  // :191-227
  copy_into(c, V(c, "ovoo"), Hovoo);
  contract(c, "je,mbie->mbij", 1.0, t1, V(c, "ovov"), 1.0, Hovoo);
  contract(c, "ie,bmje->mbij", 1.0, t1, V(c, "voov"), 1.0, Hovoo);
  contract(c, "nb,mnij->mbij", -1.0, t1, V(c, "oooo"), 1.0, Hovoo);
  contract(c, "ineb,nmje->mbij", -1.0, tau, V(c, "ooov"), 1.0, Hovoo);
  contract(c, "jneb,mnie->mbij", -1.0, tau, V(c, "ooov"), 1.0, Hovoo);
  contract(c, "mbef,ijef->mbij", 1.0, V(c, "ovvv"), tau, 1.0, Hovoo);
  contract(c, "me,ijeb->mbij", 1.0, fov, t2, 1.0, Hovoo);
  contract(c, "mnie,njeb->mbij", 1.0, L(c, "ooov"), t2, 1.0, Hovoo);
  contract(c, "mnej,ineb->mbij", -1.0, X1, t2, 1.0, Hovoo);
  {
    Temp Y2(c, {no, no, no, nv});
    contract(c, "mnef,ie->mnif", 1.0, V(c, "oovv"), t1, 0.0, Y2);
    contract(c, "mnif,jnfb->mbij", -1.0, Y2, t2, 1.0, Hovoo);
  }
  contract(c, "mefb,ijef->mbij", -1.0, X3, t2, 1.0, Hovoo);
  {
    Temp Y4(c, {no, no, nv, no});
    contract(c, "mnef,ie->mnfi", 1.0, L(c, "oovv"), t1, 0.0, Y4);
    contract(c, "mnfi,njfb->mbij", 1.0, Y4, t2, 1.0, Hovoo);
    Temp Y5(c, {no, nv});
    contract(c, "nf,mnef->me", 1.0, t1, L(c, "oovv"), 0.0, Y5);
    contract(c, "me,ijeb->mbij", 1.0, Y5, t2, 1.0, Hovoo);
    Temp Q(c, {no, no, no, no});
    contract(c, "mnej,ie->mnij", 1.0, X1, t1, 0.0, Q);
    contract(c, "mnij,nb->mbij", -1.0, Q, t1, 1.0, Hovoo);
  }
  // diagonals for the perturbed-wavefunction denominators (ccpert.cc:39-50)
  {
    std::vector<double> hoo((size_t)no * no), hvv((size_t)nv * nv), dg(no + nv);
    UCC_CUDA(cudaMemcpyAsync(hoo.data(), Hoo.p, sizeof(double) * hoo.size(), cudaMemcpyDeviceToHost, c.stream));
    UCC_CUDA(cudaMemcpyAsync(hvv.data(), Hvv.p, sizeof(double) * hvv.size(), cudaMemcpyDeviceToHost, c.stream));
    UCC_CUDA(cudaStreamSynchronize(c.stream));
    for (int i = 0; i < no; i++) dg[i] = hoo[(size_t)i * no + i];
    for (int a = 0; a < nv; a++) dg[no + a] = hvv[(size_t)a * nv + a];
    Tensor d = c.alloc("Hdiag", {no + nv}, false);
    UCC_CUDA(cudaMemcpyAsync(d.p, dg.data(), sizeof(double) * dg.size(), cudaMemcpyHostToDevice, c.stream));
  }
  // antisymmetrised combinations used by Lambda and the left-hand response
  Tensor Hovvo_x = c.alloc("Hovvo_x", {no, nv, nv, no}, false);  // 2 H[i,e,a,m] - H_ovov[i,e,m,a]
  transpose_add(c, "iema->ieam", -1.0, Hovov, 0.0, Hovvo_x);
  axpby(c, Hovvo_x.size(), 2.0, Hovvo.p, 1.0, Hovvo_x.p);
  Tensor Hvovv_x = c.alloc("Hvovv_x", {nv, no, nv, nv}, false);  // 2 H[e,i,f,a] - H[e,i,a,f]
  transpose_add(c, "eiaf->eifa", -1.0, Hvovv, 0.0, Hvovv_x);
  axpby(c, Hvovv_x.size(), 2.0, Hvovv.p, 1.0, Hvovv_x.p);
  Tensor Hooov_x = c.alloc("Hooov_x", {no, no, no, nv}, false);  // 2 H[m,i,n,a] - H[i,m,n,a]
  transpose_add(c, "imna->mina", -1.0, Hooov, 0.0, Hooov_x);
  axpby(c, Hooov_x.size(), 2.0, Hooov.p, 1.0, Hooov_x.p);
  UCC_CUDA(cudaStreamSynchronize(c.stream));
  c.have_hbar = true;
}

// ---------------------------------------------------------------------------------------
// Lambda
// ---------------------------------------------------------------------------------------
namespace {
void lambda_G(Ctx& c, const Tensor& t2, const Tensor& l2, Tensor Goo, Tensor Gvv) {  // :131-157
  contract(c, "mjab,ijab->mi", 1.0, t2, l2, 0.0, Goo);
  contract(c, "ijeb,ijab->ae", -1.0, t2, l2, 0.0, Gvv);
}

void lambda_l1(Ctx& c, const Tensor& l1, const Tensor& l2, const Tensor& Goo, const Tensor& Gvv, Tensor R1) {
  axpby(c, R1.size(), 2.0, c.get("Hov").p, 0.0, R1.p);  // :159-213
  contract(c, "ie,ea->ia", 1.0, l1, c.get("Hvv"), 1.0, R1);
  contract(c, "ma,im->ia", -1.0, l1, c.get("Hoo"), 1.0, R1);
  contract(c, "me,ieam->ia", 1.0, l1, c.get("Hovvo_x"), 1.0, R1);
  contract(c, "imef,efam->ia", 1.0, l2, c.get("Hvvvo"), 1.0, R1);
  contract(c, "mnae,iemn->ia", -1.0, l2, c.get("Hovoo"), 1.0, R1);
  contract(c, "ef,eifa->ia", -1.0, Gvv, c.get("Hvovv_x"), 1.0, R1);
  contract(c, "mn,mina->ia", -1.0, Goo, c.get("Hooov_x"), 1.0, R1);
  if (c.have_tgrad) axpby(c, R1.size(), 1.0, c.get("TS1").p, 1.0, R1.p);  // cclambda.cc:181
}

void lambda_l2(Ctx& c, const Tensor& l1, const Tensor& l2, const Tensor& Goo, const Tensor& Gvv, Tensor R2) {
  const int no = c.no, nv = c.nv;  // :215-289
  Temp Z(c, {no, no, nv, nv});
  Tensor Loovv = L(c, "oovv"), Hov = c.get("Hov");
  copy_into(c, Loovv, Z);
  if (c.have_tgrad) axpby(c, Z->size(), 0.5, c.get("TS2").p, 1.0, Z->p);  // cclambda.cc:243
  contract(c, "ia,jb->ijab", 2.0, l1, Hov, 1.0, Z);
  contract(c, "ja,ib->ijab", -1.0, l1, Hov, 1.0, Z);
  contract(c, "ijeb,ea->ijab", 1.0, l2, c.get("Hvv"), 1.0, Z);
  contract(c, "mjab,im->ijab", -1.0, l2, c.get("Hoo"), 1.0, Z);
  contract(c, "mnab,ijmn->ijab", 0.5, l2, c.get("Hoooo"), 1.0, Z);
  // 0.5 sum_ef l2_ijef Hvvvv_efab: after the (ij,ab) + (ji,ba) symmetrisation below it is the packed
  // ladder of W_abef = Hvvvv_efab + Hvvvv_feba on the symmetric l2
  const bool packed = hbar_ladder_packed(c);
  if (!packed) contract(c, "ijef,efab->ijab", 0.5, l2, c.get("Hvvvv"), 1.0, Z);
  contract(c, "ie,ejab->ijab", 1.0, l1, c.get("Hvovv_x"), 1.0, Z);
  contract(c, "mb,jima->ijab", -1.0, l1, c.get("Hooov_x"), 1.0, Z);
  contract(c, "ieam,mjeb->ijab", 1.0, c.get("Hovvo_x"), l2, 1.0, Z);
  contract(c, "jema,mibe->ijab", -1.0, c.get("Hovov"), l2, 1.0, Z);
  contract(c, "jeam,mieb->ijab", -1.0, c.get("Hovvo"), l2, 1.0, Z);
  contract(c, "ae,ijeb->ijab", 1.0, Gvv, Loovv, 1.0, Z);
  contract(c, "mi,mjab->ijab", -1.0, Goo, Loovv, 1.0, Z);
  copy_into(c, Z, R2);
  transpose_add(c, "jiba->ijab", 1.0, Z, 1.0, R2);
  if (packed) packed_ladder(c, 0.5, l2, "Hvvvv", 1, "Hpp1", "Hmm1", R2.p);
}
}  // namespace

CCSDResult run_lambda(Ctx& c) {  // :93-129
  UCC_REQUIRE(c.have_hbar, UCC_BAD_STATE, "Lambda needs HBAR");
  Fp64Scope fp64(c);  // everything outside the residual build
  const int no = c.no, nv = c.nv;
  const int64_t np = npacked(c), n1 = (int64_t)no * nv;
  Tensor Lam = c.alloc("Lam", {np}, false);
  c.alloc("Lamold", {np}, false);
  c.alloc("LR", {np}, false);
  Tensor Goo = c.alloc("Goo", {no, no}, false), Gvv = c.alloc("Gvv", {nv, nv}, false);
  double* T = c.get("T").p;
  Tensor t2 = amp2(c, T);
  if (!c.has("Lam_guess")) {  // l1 = 2 t1, l2 = 2 (2 t2 - t2(ba)), :29-41
    axpby(c, n1, 2.0, T, 0.0, Lam.p);
    Tensor l2 = amp2(c, Lam.p);
    transpose_add(c, "ijab->ijba", -2.0, t2, 0.0, l2);
    axpby(c, l2.size(), 4.0, t2.p, 1.0, l2.p);
  } else {  // a supplied guess applies to this solve only
    UCC_CUDA(cudaMemcpyAsync(Lam.p, c.get("Lam_guess").p, sizeof(double) * np, cudaMemcpyDeviceToDevice, c.stream));
    UCC_CUDA(cudaStreamSynchronize(c.stream));
    c.drop("Lam_guess");
  }
  Tensor eps = c.get("eps");
  Scratch sumsq(c, sizeof(double));
  Diis diis(c, np, 8);
  auto pseudo = [&](double* buf) { return 0.5 * dot_all(c, V(c, "oovv"), amp2(c, buf)); };
  if (c.opt.print) {
    std::printf("\n\tThe Coupled-Cluster Lambda Iteration:\n\t-------------------------------------\n");
    std::printf("\t Iter   PseudoEnergy        RMS   \n\t-------------------------------------\n");
    std::printf("\t  %3d  %20.15f\n", 0, pseudo(Lam.p));
  }
  double rms = INFINITY;
  bool converged = false;
  MixedSweeps sw(c);  // MIXED: split, record and delta sweeps; l2 is symmetrised by construction
  int iter;
  for (iter = 1; iter <= c.opt.maxiter; iter++) {
    c.store["Lam"].swap(c.store["Lamold"]);
    double* lo = c.get("Lamold").p;
    double* ln = c.get("Lam").p;
    double* r = c.get("LR").p;
    Tensor l1 = amp1(c, lo), l2 = amp2(c, lo);
    const MixedSweeps::Kind kind = sw.begin();
    {
      PrecisionScope scope(c, kind != MixedSweeps::kSplit);
      lambda_G(c, t2, l2, Goo, Gvv);
      lambda_l1(c, l1, l2, Goo, Gvv, amp1(c, r));
      lambda_l2(c, l1, l2, Goo, Gvv, amp2(c, r));
    }
    sw.end();
    jacobi_update(c, no, nv, eps.p, eps.p + no, 0.0, r, r + n1, lo, lo + n1, ln, ln + n1, sumsq.d());
    double ss = 0.0;
    UCC_CUDA(cudaMemcpyAsync(&ss, sumsq.p, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    UCC_CUDA(cudaStreamSynchronize(c.stream));
    rms = std::sqrt(ss);
    tc_check(c);
    UCC_REQUIRE(std::isfinite(rms), UCC_NAN_DETECTED, "Lambda residual is not finite");
    bool restart = false;
    if (sw.after(rms, &restart)) {
      converged = true;
      break;
    }
    if (restart) diis.reset();
    if (c.opt.diis && !restart) {
      diis.add(ln, lo);
      if (diis.size() > 2) diis.extrapolate(ln);
    }
    if (c.opt.print) {
      static const char* tag[] = {"", " split", " record", " delta"};
      std::printf("\t  %3d  %20.15f  %5.3e%s\n", iter, pseudo(ln), rms, tag[kind]);
    }
  }
  CCSDResult res;
  res.iterations = std::min(iter, c.opt.maxiter);
  res.converged = converged;
  res.e_ccsd = pseudo(c.get("Lam").p);
  c.have_lambda = res.converged;
  return res;
}

// ---------------------------------------------------------------------------------------
// Densities
// ---------------------------------------------------------------------------------------
// Gvvvv is kept for copy-out up to this many elements (256 MB)
constexpr double kKeepGvvvv = 32.0 * 1024 * 1024;

void run_density(Ctx& c, double* e1, double* e2) {
  UCC_REQUIRE(c.have_lambda, UCC_BAD_STATE, "densities need converged Lambda amplitudes");
  Fp64Scope fp64(c);
  const int no = c.no, nv = c.nv;
  double* T = c.get("T").p;
  double* Lp = c.get("Lam").p;
  Tensor t1 = amp1(c, T), t2 = amp2(c, T), tau = c.get("tau");
  Tensor l1 = amp1(c, Lp), l2 = amp2(c, Lp);

  // one-particle density, :89-151
  Tensor Doo = c.alloc("Doo", {no, no}, false);
  contract(c, "ie,je->ij", -1.0, t1, l1, 0.0, Doo);
  contract(c, "imef,jmef->ij", -1.0, t2, l2, 1.0, Doo);
  Tensor Dvv = c.alloc("Dvv", {nv, nv}, false);
  contract(c, "mb,ma->ab", 1.0, t1, l1, 0.0, Dvv);
  contract(c, "mnbe,mnae->ab", 1.0, t2, l2, 1.0, Dvv);
  Tensor Dvo = c.alloc("Dvo", {nv, no}, false);
  transpose_add(c, "ia->ai", 1.0, l1, 0.0, Dvo);
  Tensor Dov = c.alloc("Dov", {no, nv}, false);
  axpby(c, Dov.size(), 2.0, t1.p, 0.0, Dov.p);
  {
    Temp X(c, {no, no, nv, nv});  // 2 t2[i,m,a,e] - tau[m,i,a,e]
    transpose_add(c, "miae->imae", -1.0, tau, 0.0, X);
    axpby(c, X->size(), 2.0, t2.p, 1.0, X->p);
    contract(c, "me,imae->ia", 1.0, l1, X, 1.0, Dov);
    Temp Y(c, {no, no});
    contract(c, "mnef,inef->mi", 1.0, l2, t2, 0.0, Y);
    contract(c, "mi,ma->ia", -1.0, Y, t1, 1.0, Dov);
    Temp Z(c, {nv, nv});
    contract(c, "mnef,mnaf->ea", 1.0, l2, t2, 0.0, Z);
    contract(c, "ie,ea->ia", -1.0, t1, Z, 1.0, Dov);
  }
  if (c.have_tgrad) {  // the (T) pieces the densities start from, ccdensity.cc:44-69
    axpby(c, Doo.size(), 1.0, c.get("TDoo").p, 1.0, Doo.p);
    axpby(c, Dvv.size(), 1.0, c.get("TDvv").p, 1.0, Dvv.p);
    axpby(c, Dov.size(), 1.0, c.get("TDov").p, 1.0, Dov.p);
  }
  *e1 = dot_all(c, Fk(c, "oo"), Doo) + dot_all(c, Fk(c, "vv"), Dvv);

  // two-particle density blocks and energies, :153-339.  The blocks are kept in the
  // context ("Goooo", "Gooov", "Gvvvo", "Govov", "Goovv", the (T) pieces included);
  // Gvvvv (nv^4) is kept only while it is small, its energy never needs it.
  double E[6];
  {
    Tensor G = c.alloc("Goooo", {no, no, no, no}, false);
    contract(c, "ijef,klef->ijkl", 1.0, tau, l2, 0.0, G);
    E[0] = 0.5 * dot_all(c, V(c, "oooo"), G);
  }
  {
    // E = 1/2 tau[mn,ab] (sum_cd <ab|cd> l2[mn,cd]) without Gvvvv = tau . l2
    Temp Y(c, {no, no, nv, nv});
    contract(c, "mncd,abcd->mnab", 1.0, l2, V(c, "vvvv"), 0.0, Y);
    E[1] = 0.5 * dot_all(c, tau, Y);
    if ((double)nv * nv * nv * nv <= kKeepGvvvv) {
      Tensor G = c.alloc("Gvvvv", {nv, nv, nv, nv}, false);
      contract(c, "mnab,mncd->abcd", 1.0, tau, l2, 0.0, G);
    } else if (c.has("Gvvvv")) {
      c.drop("Gvvvv");
    }
  }
  Temp taux(c, {no, no, nv, nv});  // 2 tau - tau(ba)
  transpose_add(c, "ijab->ijba", -1.0, tau, 0.0, taux);
  axpby(c, taux->size(), 2.0, tau.p, 1.0, taux->p);
  Temp P(c, {no, no});  // P[k,i] = l2[k,m,e,f] t2[i,m,e,f]
  contract(c, "kmef,imef->ki", 1.0, l2, t2, 0.0, P);
  Temp Q(c, {no, no, no, nv});  // Q[k,m,i,f] = l2[k,m,e,f] t1[i,e]
  contract(c, "kmef,ie->kmif", 1.0, l2, t1, 0.0, Q);
  Temp Q3(c, {no, no, nv, no});  // Q3[k,m,e,j] = l2[k,m,e,f] t1[j,f]
  contract(c, "kmef,jf->kmej", 1.0, l2, t1, 0.0, Q3);
  {
    Tensor G = c.alloc("Gooov", {no, no, no, nv}, false);  // :206-228
    contract(c, "ke,ijea->ijka", -1.0, l1, taux, 0.0, G);
    contract(c, "ie,jkae->ijka", -1.0, t1, l2, 1.0, G);
    contract(c, "ki,ja->ijka", -2.0, P, t1, 1.0, G);
    contract(c, "kmif,jmaf->ijka", -2.0, Q, t2, 1.0, G);
    contract(c, "kj,ia->ijka", 1.0, P, t1, 1.0, G);
    contract(c, "kmjf,imaf->ijka", 1.0, Q, t2, 1.0, G);
    Temp S(c, {no, no, no, no});
    contract(c, "kmef,ijef->ijkm", 1.0, l2, t2, 0.0, S);
    contract(c, "ijkm,ma->ijka", 1.0, S, t1, 1.0, G);
    contract(c, "kmif,mjaf->ijka", 1.0, Q, t2, 1.0, G);
    contract(c, "kmej,imea->ijka", 1.0, Q3, t2, 1.0, G);
    Temp S2(c, {no, no, no, no});
    contract(c, "kmif,jf->ijkm", 1.0, Q, t1, 0.0, S2);
    contract(c, "ijkm,ma->ijka", 1.0, S2, t1, 1.0, G);
    if (c.have_tgrad) axpby(c, G.size(), 1.0, c.get("TGooov").p, 1.0, G.p);  // the (T) piece it starts from
    E[2] = dot_all(c, V(c, "ooov"), G);
  }
  {
    Tensor G = c.alloc("Gvvvo", {nv, nv, nv, no}, false);  // :237-259
    Temp taum(c, {no, no, nv, nv});  // 2 tau[m,i,a,b] - tau[i,m,a,b]
    transpose_add(c, "imab->miab", -1.0, tau, 0.0, taum);
    axpby(c, taum->size(), 2.0, tau.p, 1.0, taum->p);
    contract(c, "mc,miab->abci", 1.0, l1, taum, 0.0, G);
    contract(c, "ma,imbc->abci", 1.0, t1, l2, 1.0, G);
    Temp A1(c, {no, nv, nv, nv});  // A1[m,c,e,a] = l2[n,m,c,e] t1[n,a]
    contract(c, "nmce,na->mcea", 1.0, l2, t1, 0.0, A1);
    contract(c, "mcea,imbe->abci", 2.0, A1, t2, 1.0, G);
    Temp A2(c, {nv, nv});  // A2[c,a] = l2[n,m,c,e] t2[n,m,a,e]
    contract(c, "nmce,nmae->ca", 1.0, l2, t2, 0.0, A2);
    contract(c, "ca,ib->abci", 2.0, A2, t1, 1.0, G);
    contract(c, "mceb,imae->abci", -1.0, A1, t2, 1.0, G);
    contract(c, "cb,ia->abci", -1.0, A2, t1, 1.0, G);
    Temp A3(c, {no, nv, nv, nv});  // A3[n,c,e,b] = l2[n,m,c,e] t1[m,b]
    contract(c, "nmce,mb->nceb", 1.0, l2, t1, 0.0, A3);
    contract(c, "nceb,niae->abci", -1.0, A3, t2, 1.0, G);
    contract(c, "mcea,mibe->abci", -1.0, A1, t2, 1.0, G);
    Temp A4(c, {no, no, nv, no});  // A4[n,m,c,i] = l2[n,m,c,e] t1[i,e]
    contract(c, "nmce,ie->nmci", 1.0, l2, t1, 0.0, A4);
    contract(c, "nmci,nmab->abci", -1.0, A4, t2, 1.0, G);
    Temp A5(c, {no, nv, nv, no});
    contract(c, "nmci,mb->nbci", 1.0, A4, t1, 0.0, A5);
    contract(c, "nbci,na->abci", -1.0, A5, t1, 1.0, G);
    if (c.have_tgrad) axpby(c, G.size(), 1.0, c.get("TGvvvo").p, 1.0, G.p);
    E[3] = dot_all(c, V(c, "vvvo"), G);
  }
  {
    Tensor G = c.alloc("Govov", {no, nv, no, nv}, false);  // :268-276
    contract(c, "ia,jb->iajb", -1.0, t1, l1, 0.0, G);
    contract(c, "mibe,jmea->iajb", -1.0, tau, l2, 1.0, G);
    contract(c, "imbe,mjea->iajb", -1.0, t2, l2, 1.0, G);
    E[4] = dot_all(c, V(c, "ovov"), G);
  }
  {
    Tensor G = c.alloc("Goovv", {no, no, nv, nv}, false);  // :285-328
    Temp t2x(c, {no, no, nv, nv});
    transpose_add(c, "ijab->ijba", -1.0, t2, 0.0, t2x);
    axpby(c, t2x->size(), 2.0, t2.p, 1.0, t2x->p);
    contract(c, "ia,jb->ijab", 4.0, t1, l1, 0.0, G);
    axpby(c, G.size(), 4.0, tau.p, 1.0, G.p);
    transpose_add(c, "ijab->ijba", -2.0, tau, 1.0, G);
    axpby(c, G.size(), 1.0, l2.p, 1.0, G.p);
    Temp U(c, {no, nv});
    contract(c, "me,jmbe->jb", 1.0, l1, t2x, 0.0, U);
    contract(c, "ia,jb->ijab", 4.0, t1, U, 1.0, G);
    contract(c, "ib,ja->ijab", -2.0, t1, U, 1.0, G);
    Temp P1(c, {no, no});
    contract(c, "me,ie->mi", 1.0, l1, t1, 0.0, P1);
    contract(c, "mi,jmba->ijab", -2.0, P1, taux, 1.0, G);
    Temp P2(c, {nv, nv});
    contract(c, "me,ma->ea", 1.0, l1, t1, 0.0, P2);
    contract(c, "ea,ijeb->ijab", -2.0, P2, t2x, 1.0, G);
    contract(c, "imae,mjeb->ijab", 4.0, t2, l2, 1.0, G);
    contract(c, "mjbe,imae->ijab", -2.0, tau, l2, 1.0, G);
    // the doubly-quadratic bracket, weight 2 overall
    Temp Xa(c, {no, no, no, no});
    contract(c, "mnef,ijef->mnij", 1.0, l2, t2, 0.0, Xa);
    contract(c, "mnij,mnab->ijab", 1.0, Xa, t2, 1.0, G);
    Temp Xb(c, {no, nv, no, nv});
    contract(c, "mnef,njbf->mejb", 1.0, l2, t2, 0.0, Xb);
    contract(c, "mejb,miae->ijab", 1.0, Xb, t2, 1.0, G);
    Temp Xc(c, {no, nv, no, nv});
    contract(c, "mnef,imfb->neib", 1.0, l2, t2, 0.0, Xc);
    contract(c, "neib,njae->ijab", 1.0, Xc, t2, 1.0, G);
    Temp Xd(c, {nv, nv});
    contract(c, "mnef,mnbf->eb", 1.0, l2, t2, 0.0, Xd);
    Temp Xe(c, {no, no});
    contract(c, "mnef,jnef->mj", 1.0, l2, t2, 0.0, Xe);
    Temp Xf(c, {no, nv, no, nv});
    contract(c, "mnef,inaf->meia", 1.0, l2, t2, 0.0, Xf);
    contract(c, "ijae,eb->ijab", -4.0, tau, Xd, 1.0, G);
    contract(c, "imab,mj->ijab", -4.0, tau, Xe, 1.0, G);
    contract(c, "meia,mjbe->ijab", -4.0, Xf, tau, 1.0, G);
    contract(c, "mejb,imae->ijab", 4.0, Xf, t2, 1.0, G);
    contract(c, "ijbe,ea->ijab", 2.0, tau, Xd, 1.0, G);
    contract(c, "imba,mj->ijab", 2.0, tau, Xe, 1.0, G);
    contract(c, "meib,mjae->ijab", 2.0, Xf, tau, 1.0, G);
    contract(c, "meja,imbe->ijab", -2.0, Xf, t2, 1.0, G);
    // terms with two and four t1 factors
    Temp Y1(c, {no, no, no, nv});
    contract(c, "mnij,ma->nija", 1.0, Xa, t1, 0.0, Y1);
    contract(c, "nija,nb->ijab", 1.0, Y1, t1, 1.0, G);
    Temp W1(c, {no, no, no, nv});  // l2[m,n,e,f] t1[i,e]
    contract(c, "mnef,ie->mnif", 1.0, l2, t1, 0.0, W1);
    Temp W2(c, {no, no, no, no});
    contract(c, "mnif,jf->mnij", 1.0, W1, t1, 0.0, W2);
    contract(c, "mnij,mnab->ijab", 1.0, W2, t2, 1.0, G);
    Temp W4(c, {no, nv, no, nv});
    contract(c, "mnif,ma->nfia", 1.0, W1, t1, 0.0, W4);
    contract(c, "nfia,njbf->ijab", 1.0, W4, t2, 1.0, G);
    Temp W5(c, {no, no, nv, no});  // l2[m,n,e,f] t1[j,f]
    contract(c, "mnef,jf->mnej", 1.0, l2, t1, 0.0, W5);
    Temp W6(c, {no, nv, no, nv});
    contract(c, "mnej,nb->mejb", 1.0, W5, t1, 0.0, W6);
    contract(c, "mejb,miae->ijab", 1.0, W6, t2, 1.0, G);
    Temp W8(c, {no, nv, no, nv});
    contract(c, "mnjf,na->mfja", 1.0, W1, t1, 0.0, W8);
    contract(c, "mfja,imfb->ijab", 1.0, W8, t2, 1.0, G);
    Temp W9(c, {no, nv, no, nv});
    contract(c, "mnei,mb->neib", 1.0, W5, t1, 0.0, W9);
    contract(c, "neib,njae->ijab", 1.0, W9, t2, 1.0, G);
    Temp W10(c, {no, no, no, nv});
    contract(c, "mnij,ma->nija", 1.0, W2, t1, 0.0, W10);
    contract(c, "nija,nb->ijab", 1.0, W10, t1, 1.0, G);
    if (c.have_tgrad) axpby(c, G.size(), 1.0, c.get("TGoovv").p, 1.0, G.p);
    E[5] = 0.5 * dot_all(c, V(c, "oovv"), G);
  }
  for (int k = 0; k < 6; k++) c.e2_parts[k] = E[k];
  *e2 = E[0] + E[1] + E[2] + E[3] + E[4] + E[5];
  if (c.opt.print) {
    const char* nm[6] = {"OOOO", "VVVV", "OOOV", "VVVO", "OVOV", "OOVV"};
    for (int k = 0; k < 6; k++) std::printf("\t%s Energy = %20.14f\n", nm[k], E[k]);
  }
}

}  // namespace ucc
