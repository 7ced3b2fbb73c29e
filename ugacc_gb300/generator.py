"""Synthetic closed-shell RHF Hamiltonians (the one source of truth for every input).

The reference reads its Hamiltonian from psi4 (MO Fock matrix in QT order, occupied
orbitals first, and the MO two-electron integrals sorted so that
``ints[p][q][r][s] = <pq|rs> = (pr|qs)``; ugacc hamiltonian.cc:43-56 and :76-94).
psi4 is not available here, so every workload is built from a seeded density-fitted
model with the same layout contract:

* diagonal Fock matrix: occupied orbital energies ~ U[-1.5, -0.3] Eh, virtual orbital
  energies ~ U[0.2, 3.0] Eh, each block sorted ascending, f_ov = 0;
* three-index factors ``B[Q][p][q]`` symmetric in pq with N(0,1) * 0.08 / sqrt(naux)
  entries and ``naux = 3 * nmo``; ``(pq|rs) = sum_Q B[Q][p][q] B[Q][r][s]`` has the
  8-fold permutational symmetry of real orbitals and is positive semidefinite;
* one-electron perturbations: symmetric (dipole-like) or antisymmetric
  (angular-momentum-like) matrices with N(0, 0.1) entries.

Draw order is frozen (numpy PCG64 ``default_rng(seed)``): occupied energies, virtual
energies, then the upper triangle (p <= q, row-major) of every B^Q, Q = 0..naux-1.
Perturbations use an independent stream ``default_rng([seed, 17, k])``.
"""
from __future__ import annotations

import hashlib
import struct
from dataclasses import dataclass, field

import numpy as np

# Named workloads (no, nv, seed).  naux = 3 * (no + nv) throughout.
CONFIGS = {
    "c1_ccsd_h2o_shape": dict(no=5, nv=19, seed=0),
    "c2_ccsd_t": dict(no=16, nv=160, seed=1),
    "c3_mixed_ccsd_t": dict(no=32, nv=320, seed=2),
    "c4_lambda_response": dict(no=24, nv=240, seed=3),
}

# Frequencies (Eh) of the dynamic response workload.
RESPONSE_OMEGAS = (0.0, 0.0656)


@dataclass
class SyntheticHamiltonian:
    no: int
    nv: int
    naux: int
    seed: int
    eps: np.ndarray            # [nact] orbital energies, occupied first
    B: np.ndarray              # [naux][nact][nact], symmetric in the last two
    extra: dict = field(default_factory=dict)

    @property
    def nact(self) -> int:
        return self.no + self.nv

    @property
    def fock(self) -> np.ndarray:
        return np.diag(self.eps)

    def eri_chemist(self) -> np.ndarray:
        """(pq|rs) as a dense [nact]^4 array (small sizes only)."""
        n = self.nact
        Bm = self.B.reshape(self.naux, n * n)
        return (Bm.T @ Bm).reshape(n, n, n, n)

    def ints_physicist(self) -> np.ndarray:
        """<pq|rs> = (pr|qs), the reference's ints_ layout (hamiltonian.cc:88)."""
        return np.ascontiguousarray(self.eri_chemist().transpose(0, 2, 1, 3))

    def checksum(self) -> str:
        h = hashlib.sha256()
        h.update(np.ascontiguousarray(self.eps).tobytes())
        h.update(np.ascontiguousarray(self.B).tobytes())
        return h.hexdigest()[:16]


def make_hamiltonian(no: int, nv: int, seed: int, naux: int | None = None) -> SyntheticHamiltonian:
    if no < 1 or nv < 1:
        raise ValueError("need at least one occupied and one virtual orbital")
    nact = no + nv
    if naux is None:
        naux = 3 * nact
    rng = np.random.default_rng(seed)
    eps_o = np.sort(rng.uniform(-1.5, -0.3, size=no))
    eps_v = np.sort(rng.uniform(0.2, 3.0, size=nv))
    eps = np.concatenate([eps_o, eps_v])
    iu = np.triu_indices(nact)
    tri = rng.standard_normal(size=(naux, iu[0].size)) * (0.08 / np.sqrt(naux))
    B = np.zeros((naux, nact, nact))
    B[:, iu[0], iu[1]] = tri
    B[:, iu[1], iu[0]] = tri
    return SyntheticHamiltonian(no=no, nv=nv, naux=naux, seed=seed, eps=eps, B=B)


def make_config(name: str) -> SyntheticHamiltonian:
    c = CONFIGS[name]
    return make_hamiltonian(c["no"], c["nv"], c["seed"])


def make_perturbation(nact: int, seed: int, k: int, antisymmetric: bool = False) -> np.ndarray:
    """One-electron perturbation matrix [nact][nact] with N(0, 0.1) entries."""
    rng = np.random.default_rng([seed, 17, k])
    A = rng.normal(0.0, 0.1, size=(nact, nact))
    if antisymmetric:
        P = np.triu(A, 1)
        return P - P.T
    P = np.triu(A)
    return P + np.triu(A, 1).T


def make_perturbations(nact: int, seed: int, ndip: int = 3, nang: int = 3) -> list[np.ndarray]:
    """Three symmetric (dipole-like) then three antisymmetric (angular-momentum-like)."""
    out = [make_perturbation(nact, seed, k) for k in range(ndip)]
    out += [make_perturbation(nact, seed, 100 + k, antisymmetric=True) for k in range(nang)]
    return out


# ---------------------------------------------------------------------------------
# Binary Hamiltonian file shared by the compiled reference harness and the tests.
#   char[4] "UGAH"; int32 version=1; int32 no, nv, naux, npert, has_ints
#   double eps[nact]; double B[naux*nact*nact]; double pert[npert*nact*nact]
#   (has_ints=1) double ints[nact^4] in <pq|rs> order
# ---------------------------------------------------------------------------------
MAGIC = b"UGAH"


def write_input_file(path: str, ham: SyntheticHamiltonian, perts: list[np.ndarray] | None = None,
                     with_ints: bool = True) -> None:
    perts = perts or []
    with open(path, "wb") as f:
        f.write(MAGIC)
        f.write(struct.pack("<6i", 1, ham.no, ham.nv, ham.naux, len(perts), int(with_ints)))
        f.write(np.ascontiguousarray(ham.eps, dtype="<f8").tobytes())
        f.write(np.ascontiguousarray(ham.B, dtype="<f8").tobytes())
        for p in perts:
            f.write(np.ascontiguousarray(p, dtype="<f8").tobytes())
        if with_ints:
            n = ham.nact
            # write <pq|rs> p-slab by p-slab to bound host memory
            Bm = ham.B.reshape(ham.naux, n, n)
            for p in range(n):
                # <p q | r s> = (p r | q s) = sum_Q B[Q,p,r] B[Q,q,s]
                slab = np.einsum("Qr,Qqs->qrs", Bm[:, p, :], Bm, optimize=True)
                f.write(np.ascontiguousarray(slab, dtype="<f8").tobytes())


# ---------------------------------------------------------------------------------
# A smooth family of uneven-size Hamiltonians: B(s) = B0 + s * B1 at the largest size
# (no = 12, nv = 96, naux = 3 * 108), every member sliced to its own (no, nv): the no
# highest occupied and the nv lowest virtual orbitals of the largest model.
# ---------------------------------------------------------------------------------
FAMILY_MAX = (12, 96)


def make_family(count: int, seed: int, no_range=(4, 12), nv_range=(20, 96)):
    nomax, nvmax = FAMILY_MAX
    base = make_hamiltonian(nomax, nvmax, seed)
    pert = make_hamiltonian(nomax, nvmax, seed + 1)
    rng = np.random.default_rng([seed, 99])
    out = []
    for k in range(count):
        s = rng.uniform(0.0, 1.0)
        no = int(rng.integers(no_range[0], no_range[1] + 1))
        nv = int(rng.integers(nv_range[0], nv_range[1] + 1))
        idx = np.r_[np.arange(nomax - no, nomax), np.arange(nomax, nomax + nv)]
        B = (base.B + s * pert.B)[:, idx][:, :, idx]
        h = SyntheticHamiltonian(no=no, nv=nv, naux=base.naux, seed=seed, eps=base.eps[idx].copy(),
                                 B=np.ascontiguousarray(B), extra={"s": s, "member": k})
        out.append(h)
    return out
