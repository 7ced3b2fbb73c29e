// C++ class surface of the GB300 RHF-CC library, header-only over the C ABI.
//
// Same class names, constructor arguments and error behaviour as the reference plugin's
// classes (ugacc hamiltonian.h:12-34, ccwfn.h:12-106, hbar.h:11-36, cclambda.h:13-63,
// ccdensity.h:12-50, ccpert.h:15-80, ccresp.h:10-28): the objects share one device
// context the way the reference's objects share raw arrays through friend access, and
// non-convergence throws ConvergenceError("Computation has not converged.") like the
// reference's PSIEXCEPTION (ccwfn.cc:231).
#pragma once

#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "ugacc_gb300.h"

namespace ugacc_gb300 {

class Error : public std::runtime_error {
 public:
  Error(ucc_status s, const std::string& m) : std::runtime_error(m), status(s) {}
  ucc_status status;
};
class ConvergenceError : public Error {
 public:
  using Error::Error;
};

inline void check(ucc_ctx* ctx, ucc_status s) {
  if (s == UCC_OK) return;
  std::string msg = ctx ? ucc_last_error(ctx) : ucc_status_string(s);
  if (msg.empty()) msg = ucc_status_string(s);
  if (s == UCC_NOT_CONVERGED) throw ConvergenceError(s, msg);
  throw Error(s, msg);
}

// the reference's psi4 options (ugacc.cc:57-68) plus PRECISION / REFINE_SWEEPS
struct Options {
  std::string wfn = "CCSD", dertype = "NONE", myhand = "RIGHT", precision = "FP64";
  int maxiter = 100, refine_sweeps = 2, print = 0;
  double r_convergence = 1e-7, my_omega = 0.0, mixed_switch = 1e-5;
  bool diis = true, ooc = false;
};

class Hamiltonian {
 public:
  // ints: [nact]^4 with ints[p][q][r][s] = <pq|rs> (hamiltonian.cc:88 layout)
  Hamiltonian(int no, int nv, const double* fock, const double* ints, int device = 0) : no_(no), nv_(nv) {
    check(nullptr, ucc_ctx_create(&ctx_, device));
    check(ctx_, ucc_load_hamiltonian(ctx_, no, nv, fock, ints));
  }
  // B: [naux][nact][nact] density-fitting factors, (pq|rs) = sum_Q B[Q][p][q] B[Q][r][s]
  Hamiltonian(int no, int nv, int naux, const double* fock, const double* B, int device = 0) : no_(no), nv_(nv) {
    check(nullptr, ucc_ctx_create(&ctx_, device));
    check(ctx_, ucc_load_hamiltonian_df(ctx_, no, nv, naux, fock, B));
  }
  // hamiltonian.cc:21-102 from an MO-integral file in the FCIDUMP layout (ucc_fcidump_read):
  // nfzc frozen core and nfzv frozen virtual orbitals; enuc(), efzc() and escf() keep the
  // file's nuclear repulsion, the frozen-core energy and the SCF energy
  static std::shared_ptr<Hamiltonian> from_fcidump(const std::string& path, int nfzc = 0, int nfzv = 0,
                                                   int device = 0) {
    char err[512];
    int norb = 0, nelec = 0;
    ucc_status st = ucc_fcidump_dims(path.c_str(), &norb, &nelec, err, sizeof err);
    if (st != UCC_OK) throw Error(st, err);
    const int nact = norb - nfzc - nfzv, no = nelec / 2 - nfzc;
    if (nact <= 0 || no <= 0 || no >= nact) throw Error(UCC_BAD_ARGS, "fcidump: frozen orbitals leave no active space");
    std::vector<double> fock((size_t)nact * nact), ints((size_t)nact * nact * nact * nact);
    std::vector<int> order(nact);
    double en[3];
    st = ucc_fcidump_read(path.c_str(), nfzc, nfzv, fock.data(), ints.data(), en, order.data(), err, sizeof err);
    if (st != UCC_OK) throw Error(st, err);
    auto H = std::make_shared<Hamiltonian>(no, nact - no, fock.data(), ints.data(), device);
    H->enuc_ = en[0], H->efzc_ = en[1], H->escf_ = en[2];
    H->order_ = std::move(order);
    return H;
  }
  ~Hamiltonian() { ucc_ctx_destroy(ctx_); }
  Hamiltonian(const Hamiltonian&) = delete;
  Hamiltonian& operator=(const Hamiltonian&) = delete;
  ucc_ctx* ctx() const { return ctx_; }
  int no() const { return no_; }
  int nv() const { return nv_; }
  double enuc() const { return enuc_; }
  double efzc() const { return efzc_; }
  double escf() const { return escf_; }
  // from_fcidump: the file's orbital at each active QT position
  const std::vector<int>& orbital_order() const { return order_; }

 private:
  ucc_ctx* ctx_ = nullptr;
  int no_, nv_;
  double enuc_ = 0.0, efzc_ = 0.0, escf_ = 0.0;
  std::vector<int> order_;
};

class CCWfn {
 public:
  // ccwfn.h:14 takes the reference (SCF) wavefunction first; everything this class needs
  // from it is in the Hamiltonian, so it is only kept alive alongside, as the reference's
  // set_reference_wavefunction keeps it
  template <typename Ref>
  CCWfn(std::shared_ptr<Ref> reference, std::shared_ptr<Hamiltonian> H, const Options& o)
      : CCWfn(std::move(H), o) {
    ref_ = std::move(reference);
  }
  CCWfn(std::shared_ptr<Hamiltonian> H, const Options& o) : H_(std::move(H)), opt_(o) {
    ucc_options u;
    ucc_options_default(&u);
    u.maxiter = o.maxiter;
    u.r_convergence = o.r_convergence;
    u.diis = o.diis;
    u.precision = o.precision == "MIXED" ? UCC_MIXED : UCC_FP64;
    u.refine_sweeps = o.refine_sweeps;
    u.print = o.print;
    u.mixed_switch = o.mixed_switch;
    u.ooc = o.ooc ? 1 : 0;
    check(H_->ctx(), ucc_set_options(H_->ctx(), &u));
  }
  // ccwfn.cc:188-258: CCSD correlation energy, plus (T) for WFN == CCSD_T
  double compute_energy() {
    int it = 0;
    check(H_->ctx(), ucc_ccsd(H_->ctx(), &eccsd_, &it));
    double e = eccsd_;
    if (opt_.wfn == "CCSD_T") {
      check(H_->ctx(), ucc_triples(H_->ctx(), &et_));
      e += et_;
      // (T) gradient pieces for the derivative stages (ccwfn.cc:252-255)
      if (opt_.dertype == "FIRST") check(H_->ctx(), ucc_triples_gradient(H_->ctx()));
    }
    return e;
  }
  double eccsd() const { return eccsd_; }
  double et() const { return et_; }
  std::vector<double> tensor(const char* name, size_t n) const {
    std::vector<double> v(n);
    check(H_->ctx(), ucc_get_tensor(H_->ctx(), name, v.data(), n));
    return v;
  }
  std::vector<double> t1() const { return tensor("t1", (size_t)H_->no() * H_->nv()); }
  std::vector<double> t2() const {
    return tensor("t2", (size_t)H_->no() * H_->no() * H_->nv() * H_->nv());
  }
  const std::shared_ptr<Hamiltonian>& H() const { return H_; }

 private:
  std::shared_ptr<Hamiltonian> H_;
  std::shared_ptr<void> ref_;
  Options opt_;
  double eccsd_ = 0.0, et_ = 0.0;
};

class HBAR {
 public:
  HBAR(std::shared_ptr<Hamiltonian> H, std::shared_ptr<CCWfn> CC) : H_(std::move(H)), CC_(std::move(CC)) {
    check(H_->ctx(), ucc_hbar(H_->ctx()));
  }
  const std::shared_ptr<Hamiltonian>& H() const { return H_; }

 private:
  std::shared_ptr<Hamiltonian> H_;
  std::shared_ptr<CCWfn> CC_;
};

class CCLambda {
 public:
  CCLambda(std::shared_ptr<CCWfn> CC, std::shared_ptr<HBAR> hbar) : CC_(std::move(CC)), HBAR_(std::move(hbar)) {}
  void compute_lambda() {  // cclambda.cc:93-129
    int it = 0;
    check(CC_->H()->ctx(), ucc_lambda(CC_->H()->ctx(), &pseudo_, &it));
  }
  double pseudoenergy() const { return pseudo_; }
  const std::shared_ptr<CCWfn>& CC() const { return CC_; }

 private:
  std::shared_ptr<CCWfn> CC_;
  std::shared_ptr<HBAR> HBAR_;
  double pseudo_ = 0.0;
};

class CCDensity {
 public:
  CCDensity(std::shared_ptr<CCWfn> CC, std::shared_ptr<CCLambda> lam) : CC_(std::move(CC)), L_(std::move(lam)) {}
  double onepdm() {  // ccdensity.cc:89-151
    run();
    return e1_;
  }
  double twopdm() {  // ccdensity.cc:153-339
    run();
    return e2_;
  }

 private:
  void run() {
    if (!done_) check(CC_->H()->ctx(), ucc_density(CC_->H()->ctx(), &e1_, &e2_));
    done_ = true;
  }
  std::shared_ptr<CCWfn> CC_;
  std::shared_ptr<CCLambda> L_;
  double e1_ = 0.0, e2_ = 0.0;
  bool done_ = false;
};

enum hand { left, right };  // ccpert.h:15

class CCPert {
 public:
  // ccpert.h:19: the perturbation as the reference passes it, nact row pointers of nact
  // elements each (pert[p][q], QT order)
  CCPert(double** pert, double omega, std::shared_ptr<CCWfn> CC, std::shared_ptr<HBAR> hbar,
         std::shared_ptr<CCLambda> lam)
      : CCPert(rows_to_dense(pert, CC).data(), omega, CC, std::move(hbar), std::move(lam)) {}
  // the same matrix stored contiguously, [nact][nact]
  CCPert(const double* pert, double omega, std::shared_ptr<CCWfn> CC, std::shared_ptr<HBAR> hbar,
         std::shared_ptr<CCLambda> lam)
      : CC_(std::move(CC)), HBAR_(std::move(hbar)), L_(std::move(lam)), omega_(omega) {
    check(CC_->H()->ctx(), ucc_pert_create(CC_->H()->ctx(), pert, omega, &handle_));
  }
  // ccpert.h:21 / ccpert.cc:177-229: converge the right-hand (X) or left-hand (Y)
  // perturbed amplitudes; throws ConvergenceError like the reference
  void solve(hand h) {
    int it = 0;
    const int k = h == right ? 1 : 0;
    check(CC_->H()->ctx(), ucc_pert_solve(CC_->H()->ctx(), handle_, k, &pseudo_[k], &it));
  }
  // ccpert.cc:233-253: the pseudo-response of the last solve of that hand
  double pseudoresponse(hand h) const { return pseudo_[h == right ? 1 : 0]; }
  int handle() const { return handle_; }
  ucc_ctx* ctx() const { return CC_->H()->ctx(); }

 private:
  static std::vector<double> rows_to_dense(double** pert, const std::shared_ptr<CCWfn>& CC) {
    if (!pert || !CC) throw Error(UCC_BAD_ARGS, "CCPert: null perturbation or wavefunction");
    const size_t n = (size_t)CC->H()->no() + (size_t)CC->H()->nv();
    std::vector<double> d(n * n);
    for (size_t p = 0; p < n; p++) {
      if (!pert[p]) throw Error(UCC_BAD_ARGS, "CCPert: null perturbation row");
      for (size_t q = 0; q < n; q++) d[p * n + q] = pert[p][q];
    }
    return d;
  }
  std::shared_ptr<CCWfn> CC_;
  std::shared_ptr<HBAR> HBAR_;
  std::shared_ptr<CCLambda> L_;
  double omega_;
  int handle_ = -1;
  double pseudo_[2] = {0.0, 0.0};
};

class CCResp {
 public:
  CCResp(std::shared_ptr<CCPert> X, std::shared_ptr<CCPert> Y) : X_(std::move(X)), Y_(std::move(Y)) {}
  // ccresp.h:13: one perturbation on both sides
  explicit CCResp(std::shared_ptr<CCPert> X) : X_(X), Y_(std::move(X)) {}
  double linresp(const std::shared_ptr<CCPert>& X, const std::shared_ptr<CCPert>& Y) {  // ccresp.cc:28-124
    double v = 0.0;
    check(X->ctx(), ucc_linresp(X->ctx(), X->handle(), Y->handle(), &v));
    return v;
  }

 private:
  std::shared_ptr<CCPert> X_, Y_;
};

}  // namespace ugacc_gb300
