// Definitions for psi4_shim.h (test infrastructure; see the header).
#include "psi4_shim.h"

#include <algorithm>
#include <cstdlib>

namespace psi {

std::shared_ptr<PsiOutStream> outfile = std::make_shared<PsiOutStream>();
std::shared_ptr<MOSpace> MOSpace::all = std::make_shared<MOSpace>();

void PsiOutStream::Printf(const char* fmt, ...) {
  FILE* f = f_ ? f_ : stdout;
  va_list ap;
  va_start(ap, fmt);
  vfprintf(f, fmt, ap);
  va_end(ap);
  fflush(f);
}

double** block_matrix(size_t n, size_t m, bool) {
  if (n == 0 || m == 0) return nullptr;
  double** A = (double**)malloc(n * sizeof(double*));
  double* blk = (double*)calloc(n * m, sizeof(double));
  if (!A || !blk) throw PSIEXCEPTION("block_matrix: out of memory");
  for (size_t i = 0; i < n; i++) A[i] = blk + i * m;
  return A;
}

void free_block(double** A) {
  if (!A) return;
  free(A[0]);
  free(A);
}

std::string Options::get_str(const std::string& k) const {
  auto it = s_.find(k);
  if (it == s_.end()) throw PSIEXCEPTION("option not set: " + k);
  return it->second;
}
int Options::get_int(const std::string& k) const {
  auto it = i_.find(k);
  if (it == i_.end()) throw PSIEXCEPTION("option not set: " + k);
  return it->second;
}
bool Options::get_bool(const std::string& k) const {
  auto it = b_.find(k);
  if (it == b_.end()) throw PSIEXCEPTION("option not set: " + k);
  return it->second;
}
double Options::get_double(const std::string& k) const {
  auto it = d_.find(k);
  if (it == d_.end()) throw PSIEXCEPTION("option not set: " + k);
  return it->second;
}

void Wavefunction::shallow_copy(std::shared_ptr<Wavefunction> o) {
  nirrep_ = o->nirrep_;
  nmo_ = o->nmo_;
  nso_ = o->nso_;
  nfrzc_ = o->nfrzc_;
  doccpi_ = o->doccpi_;
  soccpi_ = o->soccpi_;
  frzcpi_ = o->frzcpi_;
  frzvpi_ = o->frzvpi_;
  nmopi_ = o->nmopi_;
  energy_ = o->energy_;
  molecule_ = o->molecule_;
}

void DIISManager::push(std::vector<double> e, std::vector<double> a) {
  if ((int)errs_.size() < max_) {
    errs_.push_back(std::move(e));
    amps_.push_back(std::move(a));
  } else {
    const size_t slot = (size_t)(nadded_ % max_);  // oldest entry is replaced
    errs_[slot] = std::move(e);
    amps_[slot] = std::move(a);
  }
  nadded_++;
}

std::vector<double> DIISManager::solve_and_combine() {
  const int n = (int)errs_.size();
  const int m = n + 1;
  std::vector<double> B((size_t)m * m, 0.0), c(m, 0.0);
  for (int p = 0; p < n; p++)
    for (int q = 0; q <= p; q++) {
      double s = 0.0;
      const double* x = errs_[p].data();
      const double* y = errs_[q].data();
      for (size_t k = 0; k < errs_[p].size(); k++) s += x[k] * y[k];
      B[p * m + q] = B[q * m + p] = s;
    }
  double mx = 0.0;
  for (int p = 0; p < n; p++)
    for (int q = 0; q < n; q++) mx = std::max(mx, std::fabs(B[p * m + q]));
  if (mx > 0.0)
    for (int p = 0; p < n; p++)
      for (int q = 0; q < n; q++) B[p * m + q] /= mx;
  for (int p = 0; p < n; p++) {
    B[p * m + n] = -1.0;
    B[n * m + p] = -1.0;
  }
  B[n * m + n] = 0.0;
  c[n] = -1.0;
  // Gaussian elimination with partial pivoting on the (n+1)x(n+1) bordered system.
  for (int col = 0; col < m; col++) {
    int piv = col;
    for (int r = col + 1; r < m; r++)
      if (std::fabs(B[r * m + col]) > std::fabs(B[piv * m + col])) piv = r;
    if (piv != col) {
      for (int k = 0; k < m; k++) std::swap(B[col * m + k], B[piv * m + k]);
      std::swap(c[col], c[piv]);
    }
    const double d = B[col * m + col];
    if (d == 0.0) throw PSIEXCEPTION("DIIS: singular B matrix");
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
  const size_t len = amps_[0].size();
  std::vector<double> out(len, 0.0);
  for (int p = 0; p < n; p++) {
    const double w = c[p];
    const double* x = amps_[p].data();
    for (size_t k = 0; k < len; k++) out[k] += w * x[k];
  }
  return out;
}

}  // namespace psi
