// Minimal stand-in for the parts of psi4 that ugacc's hot-path sources use.
//
// TEST INFRASTRUCTURE ONLY.  This header lets the reference's own
// array.cc ccwfn.cc hbar.cc cclambda.cc ccdensity.cc ccpert.cc ccresp.cc compile
// unchanged (they are read in place from the reference tree by oracle/Makefile) so
// that their outputs can pin the oracle and the golden fixtures.  Nothing here is
// linked into the GPU library.
//
// What is provided, and where the reference uses it:
//   outfile->Printf                       every .cc (iteration tables)
//   PSIEXCEPTION                          ccwfn.cc:231, cclambda.cc:128, ccpert.cc:228
//   block_matrix / free_block             contiguous zeroed 2-D arrays (libciomr)
//   Vector(name, n)->pointer()            DIIS buffers, ccwfn.cc:202-205
//   DIISManager                           Pulay DIIS, ccwfn.cc:206-221 (see psi4_shim.cc)
//   Options::get_{str,int,bool,double}    ccwfn.cc:15-20
//   Wavefunction / Molecule / Dimension   CCWfn base class data, ccwfn.cc:12-54
//   PSIO, MOSpace, IntegralTransform      only named in the Hamiltonian signature
#pragma once

#include <array>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#ifndef PSI_API
#define PSI_API
#endif

namespace psi {

class PsiOutStream {
 public:
  void Printf(const char* fmt, ...) __attribute__((format(printf, 2, 3)));
  void set_file(FILE* f) { f_ = f; }

 private:
  FILE* f_ = nullptr;
};
extern std::shared_ptr<PsiOutStream> outfile;

class PsiException : public std::runtime_error {
 public:
  PsiException(const std::string& msg, const char* file, int line)
      : std::runtime_error(msg), file_(file), line_(line) {}
  const char* file() const { return file_; }
  int line() const { return line_; }

 private:
  const char* file_;
  int line_;
};
#define PSIEXCEPTION(message) psi::PsiException(message, __FILE__, __LINE__)

double** block_matrix(size_t n, size_t m, bool memlock = false);
void free_block(double** A);

class Vector {
 public:
  Vector(const std::string& name, int n) : name_(name), data_(n > 0 ? n : 0, 0.0) {}
  double* pointer() { return data_.data(); }
  int dim() const { return (int)data_.size(); }
  const std::string& name() const { return name_; }

 private:
  std::string name_;
  std::vector<double> data_;
};

class Options {
 public:
  std::string get_str(const std::string& k) const;
  int get_int(const std::string& k) const;
  bool get_bool(const std::string& k) const;
  double get_double(const std::string& k) const;
  void set_str(const std::string& k, const std::string& v) { s_[k] = v; }
  void set_int(const std::string& k, int v) { i_[k] = v; }
  void set_bool(const std::string& k, bool v) { b_[k] = v; }
  void set_double(const std::string& k, double v) { d_[k] = v; }

 private:
  std::map<std::string, std::string> s_;
  std::map<std::string, int> i_;
  std::map<std::string, bool> b_;
  std::map<std::string, double> d_;
};

class Dimension {
 public:
  Dimension() = default;
  explicit Dimension(std::vector<int> v) : v_(std::move(v)) {}
  int operator[](int h) const { return v_.at(h); }
  int& operator[](int h) { return v_.at(h); }
  int n() const { return (int)v_.size(); }

 private:
  std::vector<int> v_;
};

class Molecule {
 public:
  std::vector<std::string> irrep_labels() const { return {"A"}; }
  double nuclear_repulsion_energy(const std::array<double, 3>&) const { return enuc_; }
  double enuc_ = 0.0;
};

class Wavefunction {
 public:
  explicit Wavefunction(Options& options) : options_(&options) {}
  Wavefunction() = default;
  virtual ~Wavefunction() = default;

  void set_reference_wavefunction(std::shared_ptr<Wavefunction> ref) { reference_wavefunction_ = ref; }
  void shallow_copy(std::shared_ptr<Wavefunction> other);
  const Dimension& doccpi() const { return doccpi_; }
  const Dimension& soccpi() const { return soccpi_; }
  double energy() const { return energy_; }
  std::array<double, 3> get_dipole_field_strength() const { return {0.0, 0.0, 0.0}; }
  int nirrep() const { return nirrep_; }

  // fields filled by the harness for a synthetic closed-shell reference
  int nirrep_ = 1;
  int nmo_ = 0;
  int nso_ = 0;
  int nfrzc_ = 0;
  Dimension doccpi_, soccpi_, frzcpi_, frzvpi_, nmopi_;
  double energy_ = 0.0;
  std::shared_ptr<Molecule> molecule_;
  std::shared_ptr<Wavefunction> reference_wavefunction_;
  Options* options_ = nullptr;
};
using SharedWavefunction = std::shared_ptr<Wavefunction>;

class PSIO {};
class MOSpace {
 public:
  static std::shared_ptr<MOSpace> all;
};
class IntegralTransform {};

// Pulay DIIS with the same call surface as psi4's pointer-based DIISManager.
// Circular 8-slot subspace, B matrix scaled by max|B_pq|, -1 border, partial-pivot
// Gaussian elimination: the procedure of the reference's own attic/diis.cc:13-161.
class DIISManager {
 public:
  DIISManager(int max_subspace, const std::string& label) : max_(max_subspace), label_(label) {}

  template <typename... V>
  void set_error_vector_size(V*... v) { err_sizes_ = {v->dim()...}; }
  template <typename... V>
  void set_vector_size(V*... v) { amp_sizes_ = {v->dim()...}; }

  template <typename... V>
  bool add_entry(V*... v) {
    std::vector<Vector*> all = {v...};
    const size_t ne = err_sizes_.size();
    std::vector<double> e, a;
    for (size_t k = 0; k < all.size(); k++) {
      auto& dst = k < ne ? e : a;
      dst.insert(dst.end(), all[k]->pointer(), all[k]->pointer() + all[k]->dim());
    }
    push(std::move(e), std::move(a));
    return true;
  }

  template <typename... V>
  bool extrapolate(V*... v) {
    std::vector<Vector*> outs = {v...};
    std::vector<double> res = solve_and_combine();
    size_t off = 0;
    for (Vector* o : outs) {
      std::memcpy(o->pointer(), res.data() + off, sizeof(double) * o->dim());
      off += o->dim();
    }
    return true;
  }

  int subspace_size() const { return (int)errs_.size(); }

 private:
  void push(std::vector<double> e, std::vector<double> a);
  std::vector<double> solve_and_combine();

  int max_;
  std::string label_;
  std::vector<int> err_sizes_, amp_sizes_;
  std::vector<std::vector<double>> errs_, amps_;
  long nadded_ = 0;
};

}  // namespace psi
