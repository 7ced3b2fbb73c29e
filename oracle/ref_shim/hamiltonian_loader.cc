// Replacement for the reference's Hamiltonian constructor (test infrastructure).
//
// The reference fills fock_, ints_ and L_ from psi4's integral transformation
// (hamiltonian.cc:19-104).  Here the same members are filled from the synthetic
// Hamiltonian file written by ugacc_gb300/generator.py, keeping the reference's
// layout contract:
//   fock_[p][q]          QT order, occupied first            (hamiltonian.cc:43-56)
//   ints_[p][q][r][s]    <pq|rs> = (pr|qs)                   (hamiltonian.cc:88)
//   L_[p][q][r][s]       2 <pq|rs> - <pq|sr>                 (hamiltonian.cc:96-102)
#include "hamiltonian_input.h"

#include "array.h"
#include "hamiltonian.h"

namespace psi {
namespace ugacc {

Hamiltonian::Hamiltonian(shared_ptr<PSIO>, shared_ptr<Wavefunction> ref, std::vector<shared_ptr<MOSpace> >) {
  const HamiltonianInput& in = current_input();
  nmo_ = ref->nmo_;
  nso_ = ref->nmo_;
  nfzc_ = 0;
  nfzv_ = 0;
  nact_ = in.nact;
  efzc_ = 0.0;
  const int n = nact_;

  fock_ = block_matrix(n, n);
  for (int p = 0; p < n; p++) fock_[p][p] = in.eps[p];

  ints_ = init_4d_array(n, n, n, n);
  const size_t n2 = (size_t)n * n, n3 = n2 * n;
  for (int p = 0; p < n; p++)
    for (int q = 0; q < n; q++)
      for (int r = 0; r < n; r++) {
        const double* src = in.ints.data() + p * n3 + q * n2 + (size_t)r * n;
        double* dst = ints_[p][q][r];
        for (int s = 0; s < n; s++) dst[s] = src[s];
      }

  L_ = init_4d_array(n, n, n, n);
  for (int p = 0; p < n; p++)
    for (int q = 0; q < n; q++)
      for (int r = 0; r < n; r++)
        for (int s = 0; s < n; s++) L_[p][q][r][s] = 2.0 * ints_[p][q][r][s] - ints_[p][q][s][r];
}

Hamiltonian::~Hamiltonian() {
  free_4d_array(ints_, nact_, nact_, nact_);
  free_4d_array(L_, nact_, nact_, nact_);
  free_block(fock_);
}

}  // namespace ugacc
}  // namespace psi
