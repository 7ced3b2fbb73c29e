"""numpy restatement of the reference Hamiltonian's integral side, and an FCIDUMP writer
(test infrastructure: only the tests use this file).

``hamiltonian`` follows hamiltonian.cc:21-102 from MO integrals over all orbitals: the
Fock matrix of the reference determinant restricted to the active orbitals in QT order
(:43-56, psi4's Fa in the MO basis), <pq|rs> = (pr|qs) over the active orbitals
(:76-91, ``ints_[p][r][q][s] = (pq|rs)``), with the first ``nfzc`` orbitals frozen core
and the last ``nfzv`` frozen virtuals (:24-27), and the frozen-core energy (:72, psi4
libtrans' ``get_frozen_core_energy``: sum over frozen i of h_ii + F^core_ii).
"""
from __future__ import annotations

import numpy as np


def fock_full(h: np.ndarray, eri: np.ndarray, nocc: int) -> np.ndarray:
    """F_pq = h_pq + sum_k [2 (pq|kk) - (pk|kq)] over the nocc doubly occupied orbitals."""
    k = slice(0, nocc)
    J = np.einsum("pqkk->pq", eri[:, :, k, k])
    K = np.einsum("pkkq->pq", eri[:, k, k, :])
    return h + 2.0 * J - K


def hamiltonian(h, eri, enuc, nocc, nfzc=0, nfzv=0, orbital_energies=None):
    """(fock_active, ints_active, enuc, efzc, escf) from full h [n][n], eri [n]^4 = (pq|rs).
    With ``orbital_energies`` the orbitals are first put in ascending-energy order (stable),
    which puts the nocc lowest (occupied) first, as the file reader does."""
    n = h.shape[0]
    if orbital_energies is not None:
        qt = np.argsort(np.asarray(orbital_energies), kind="stable")
        h = h[np.ix_(qt, qt)]
        eri = eri[np.ix_(qt, qt, qt, qt)]
    F = fock_full(h, eri, nocc)
    c = slice(0, nfzc)
    efzc = 2.0 * np.trace(h[c, c]) + 2.0 * np.einsum("iijj->", eri[c, c, c, c]) - np.einsum("ijji->", eri[c, c, c, c])
    escf = enuc + float(np.trace(h[:nocc, :nocc]) + np.trace(F[:nocc, :nocc]))
    a = slice(nfzc, n - nfzv)
    fock = F[a, a].copy()
    ints = np.ascontiguousarray(eri[a, a, a, a].transpose(0, 2, 1, 3))
    return fock, ints, float(enuc), float(efzc), escf


def core_hamiltonian_for(fock: np.ndarray, eri: np.ndarray, nocc: int) -> np.ndarray:
    """The h whose determinant Fock matrix (nocc orbitals occupied) is ``fock``."""
    return fock - (fock_full(np.zeros_like(fock), eri, nocc))


def write(path, h, eri, enuc, nelec, ms2=0, uhf=None, scramble=False, fortran_d=False, terminator="&END",
          orbital_energies=None, tol=0.0, seed=0):
    """Write an FCIDUMP text file: the unique (ij|kl) with i>=j, k>=l, (ij)>=(kl), h_ij with
    i>=j, optional orbital energies, then the nuclear repulsion.  ``scramble`` writes each
    two-electron entry under a random one of its 8 equivalent index orders."""
    n = h.shape[0]
    rng = np.random.default_rng(seed)

    def num(v):
        s = "%.17e" % v
        return s.replace("e", "D") if fortran_d else s

    lines = []
    head = " &FCI NORB=%d,NELEC=%d,MS2=%d,\n  ORBSYM=%s,\n  ISYM=1," % (n, nelec, ms2, ",".join(["1"] * n))
    if uhf is not None:
        head += "\n  UHF=%s," % (".TRUE." if uhf else ".FALSE.")
    lines.append(head)
    lines.append(" &END" if terminator == "&END" else " /")
    for i in range(n):
        for j in range(i + 1):
            ij = i * (i + 1) // 2 + j
            for k in range(n):
                for l in range(k + 1):
                    if k * (k + 1) // 2 + l > ij:
                        continue
                    v = eri[i, j, k, l]
                    if abs(v) <= tol:
                        continue
                    idx = (i, j, k, l)
                    if scramble:
                        forms = [(i, j, k, l), (j, i, k, l), (i, j, l, k), (j, i, l, k),
                                 (k, l, i, j), (l, k, i, j), (k, l, j, i), (l, k, j, i)]
                        idx = forms[rng.integers(8)]
                    lines.append("%s %d %d %d %d" % (num(v), idx[0] + 1, idx[1] + 1, idx[2] + 1, idx[3] + 1))
    for i in range(n):
        for j in range(i + 1):
            if h[i, j] != 0.0 or i == j:
                lines.append("%s %d %d 0 0" % (num(h[i, j]), i + 1, j + 1))
    if orbital_energies is not None:
        for i, e in enumerate(orbital_energies):
            lines.append("%s %d 0 0 0" % (num(e), i + 1))
    lines.append("%s 0 0 0 0" % num(enuc))
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
