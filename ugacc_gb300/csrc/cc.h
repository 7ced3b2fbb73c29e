// Equation layer of the RHF-CC solver: integral blocks, DIIS and the solver stages.
#pragma once

#include <cmath>
#include <string>
#include <vector>

#include "engine.h"

namespace ucc {

// ---- integral blocks (physicist <pq|rs>, occupied indices first) ----------------------
void load_from_ints(Ctx& c, int no, int nv, const double* fock, const double* ints);
void load_from_df(Ctx& c, int no, int nv, int naux, const double* fock, const double* B);
// <pq|rs> block view, e.g. V(c,"ovvv")[m,a,e,f] = <ma|ef>; stored blocks are oooo ooov oovv
// ovov ovvv vvvv, the rest are permuted views of them
Tensor V(Ctx& c, const std::string& blk);
// L = 2<pq|rs> - <pq|sr> blocks: oovv ooov ovvv ovvo stored, oovo vovv as views
Tensor L(Ctx& c, const std::string& blk);
Tensor Fk(Ctx& c, const std::string& blk);  // Fock blocks oo ov vo vv
Tensor narrow(const Tensor& t, int axis, int64_t start, int64_t len);

// ---- DIIS over packed [x1 | x2] vectors ---------------------------------------------
// Circular 8-slot Pulay subspace, error = new - old, B scaled by max|B_pq|, -1 border,
// partial-pivot Gaussian elimination: the procedure of the reference's attic/diis.cc
// used through psi4's DIISManager at ccwfn.cc:206-221.
class Diis {
 public:
  Diis(Ctx& c, int64_t n, int nmax = 8);
  ~Diis();
  void add(const double* vnew, const double* vold);
  int size() const { return count_; }
  void extrapolate(double* out);
  void reset();

 private:
  Ctx& c_;
  int64_t n_;
  int nmax_, count_ = 0;
  long nadded_ = 0;
  DeviceBuffer err_, vec_;
  const double** d_errp_ = nullptr;
  const double** d_vecp_ = nullptr;
  std::vector<double> B_;
};

// Solve B x = rhs for the bordered DIIS system (same elimination as the oracle's shim).
std::vector<double> diis_coefficients(const std::vector<double>& Bfull, int n);

// ---- mixed-precision sweep policy (shared by the CCSD, Lambda and perturbed solves) ----
// split  - residual from BF16 hi+lo split GEMMs, until the residual norm reaches the
//          split-product noise floor (or stops falling);
// record - FP64 residual that also records every heavy GEMM as an anchor;
// delta  - FP64 residual whose heavy GEMMs are anchor + tensor-core corrections.
// The solve ends only on a record sweep with ||R|| < r_convergence (and at least
// refine_sweeps record sweeps); a delta sweep that gets there, or stalls, asks for one.
// A delta residual is accurate to about 3e-5 of the anchor's own residual (its error
// scales with the distance from the anchor), so an anchor taken above kReanchor *
// r_convergence is replaced once the delta residual falls below that level: the next
// anchor is close enough for the deltas to resolve r_convergence without stalling.
// With precision FP64 every sweep is plain FP64.
class MixedSweeps {
 public:
  enum Kind { kFp64, kSplit, kRecord, kDelta };
  explicit MixedSweeps(Ctx& c);
  ~MixedSweeps();
  Kind begin();  // kind of the coming sweep, anchors armed for it
  void end();    // anchors disarmed (call before the Jacobi update)
  // after the sweep's residual norm: true when the solve has converged; *restart_diis is
  // set when the DIIS history must start again (this sweep's vector is not added)
  bool after(double rms, bool* restart_diis);
  bool mixed() const { return mixed_; }
  Kind kind() const { return kind_; }
  int split = 0, record = 0, delta = 0;
  // digits (bf16 slices) of the coming record sweep's sliced products: enough to resolve the
  // residual level the delta sweeps after it must reach, 9 (the full 54 bits) for a sweep
  // that may end the solve or follows a stall
  int record_digits() const;

 private:
  Ctx& c_;
  bool mixed_, refine_, split_phase_, record_next_ = true;
  int stalls_ = 0, sweeps_ = 0, digits_ = 9, split_slow_ = 0;
  double rms_prev_ = INFINITY, anchor_rms_ = INFINITY;
  double record_target_ = 0.0;  // level the deltas after the coming record sweep resolve; 0: full digits
  Kind kind_ = kFp64, last_ = kFp64;
};

// ---- solver stages ---------------------------------------------------------------------
struct CCSDResult {
  double e_ccsd = 0.0, e_mp2 = 0.0;
  int iterations = 0;
  bool converged = false;
};
CCSDResult run_ccsd(Ctx& c);
void ccsd_alloc(Ctx& c);                                         // CCSD work arrays
void ccsd_residual(Ctx& c, const double* t_old, double* r);      // R(t_old), tau/ttau current
double ccsd_energy(Ctx& c, const double* t);                     // E from t and the stored tau
double run_triples(Ctx& c);
// R2 += alpha sum_ef W_abef amp_ijef on packed pairs (cc_ground.cpp), W from block src by
// mode (0: H_abef, 1: H_efab + H_feba, 2: H_abef + H_bafe)
void packed_ladder(Ctx& c, double alpha, const Tensor& amp, const char* src, int mode, const char* vp_name,
                   const char* vm_name, double* R2);
// the packed form needs pairs on both sides and runs eagerly (it is not part of a recorded sweep)
inline bool hbar_ladder_packed(Ctx& c) { return !recorder() && c.no > 1 && c.nv > 1; }
void run_triples_gradient(Ctx& c);  // tgrad.cu
void run_hbar(Ctx& c);
CCSDResult run_lambda(Ctx& c);
void run_density(Ctx& c, double* e1, double* e2);

// amplitude views into a packed [t1 | t2] buffer
inline Tensor amp1(Ctx& c, double* p) { return make_view(p, {c.no, c.nv}); }
inline Tensor amp2(Ctx& c, double* p) { return make_view(p + (int64_t)c.no * c.nv, {c.no, c.no, c.nv, c.nv}); }
inline int64_t npacked(const Ctx& c) {
  return (int64_t)c.no * c.nv + (int64_t)c.no * c.no * c.nv * c.nv;
}

// The six W3 terms of a (T) tuple (i,j,k): A operand of occupied index x, B operand of
// the ordered pair (y,z) (selectors into (i,j,k)), and the W3[a][b][c] strides of the GEMM
// output G[(u,v), w] (see triples.cpp).
struct TriplesTerm {
  int x, y, z;
  int64_t su, sv, sw;
};
inline void triples_terms(int64_t nv, TriplesTerm t[6]) {
  const int64_t nv2 = nv * nv;
  t[0] = {0, 2, 1, nv2, nv, 1};
  t[1] = {0, 1, 2, nv2, 1, nv};
  t[2] = {2, 1, 0, 1, nv2, nv};
  t[3] = {2, 0, 1, 1, nv, nv2};
  t[4] = {1, 0, 2, nv, 1, nv2};
  t[5] = {1, 2, 0, nv, nv2, 1};
}

// algorithmic FLOP counts (2 per multiply-add, no symmetry credit)
double flops_ccsd_iter(double no, double nv);
double flops_triples(double no, double nv);

}  // namespace ucc
