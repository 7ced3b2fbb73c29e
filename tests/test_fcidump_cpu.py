"""The MO-integral-file front end (ucc_fcidump_*, host code) against the numpy restatement
of hamiltonian.cc:21-102 in oracle/fcidump.py.  No GPU needed."""
import numpy as np
import pytest

import ugacc_gb300 as U
from oracle import fcidump as FD
from ugacc_gb300.generator import make_hamiltonian


@pytest.fixture(scope="module", autouse=True)
def _lib():
    from ugacc_gb300.build import build

    build()
    U.load_library()


def _random_system(n, nocc, seed):
    """Random real-orbital integrals with the 8-fold symmetry, a symmetric h."""
    rng = np.random.default_rng(seed)
    B = rng.standard_normal((2 * n, n, n)) * 0.1
    B = B + B.transpose(0, 2, 1)
    eri = np.einsum("Qpq,Qrs->pqrs", B, B)
    h = rng.standard_normal((n, n))
    h = h + h.T
    return h, eri, float(rng.uniform(1, 10))


@pytest.mark.parametrize("nfzc,nfzv", [(0, 0), (1, 0), (0, 2), (2, 3)])
def test_active_hamiltonian_matches_oracle(tmp_path, nfzc, nfzv):
    n, nelec = 11, 10
    h, eri, enuc = _random_system(n, nelec // 2, 3 + nfzc + 7 * nfzv)
    path = str(tmp_path / "FCIDUMP")
    FD.write(path, h, eri, enuc, nelec, scramble=True, seed=nfzc)
    got = U.read_fcidump(path, nfzc, nfzv)
    fock, ints, en, efzc, escf = FD.hamiltonian(h, eri, enuc, nelec // 2, nfzc, nfzv)
    assert (got["no"], got["nv"]) == (nelec // 2 - nfzc, n - nelec // 2 - nfzv)
    np.testing.assert_allclose(got["fock"], fock, atol=1e-13, rtol=0)
    np.testing.assert_allclose(got["ints"], ints, atol=1e-14, rtol=0)
    assert got["enuc"] == enuc
    assert abs(got["efzc"] - efzc) < 1e-12 and abs(got["escf"] - escf) < 1e-12
    assert list(got["order"]) == list(range(nfzc, n - nfzv))  # no energies: the file order
    if nfzc == 0:
        assert got["efzc"] == 0.0


def test_header_and_number_variants(tmp_path):
    """'/' terminator, Fortran D exponents, UHF=.FALSE., orbital-energy lines."""
    n, nelec = 7, 6
    h, eri, enuc = _random_system(n, 3, 11)
    a, b = str(tmp_path / "a"), str(tmp_path / "b")
    FD.write(a, h, eri, enuc, nelec)
    FD.write(b, h, eri, enuc, nelec, fortran_d=True, terminator="/", uhf=False, orbital_energies=np.arange(n) * 0.1,
             scramble=True, seed=5)
    ra, rb = U.read_fcidump(a, 1, 1), U.read_fcidump(b, 1, 1)
    for k in ("fock", "ints"):
        np.testing.assert_array_equal(ra[k], rb[k])
    assert ra["escf"] == rb["escf"] and ra["efzc"] == rb["efzc"]


def test_synthetic_generator_round_trip(tmp_path):
    """The generator's Hamiltonian written as a file (h chosen so that its determinant's
    Fock matrix is diag(eps)) reads back as the generator's own fock and <pq|rs>; with
    frozen orbitals the active part is the generator's active block."""
    ham = make_hamiltonian(5, 14, seed=4)
    eri = ham.eri_chemist()
    h = FD.core_hamiltonian_for(ham.fock, eri, ham.no)
    path = str(tmp_path / "FCIDUMP")
    FD.write(path, h, eri, 0.5, 2 * ham.no)
    d = U.read_fcidump(path)
    np.testing.assert_allclose(d["fock"], ham.fock, atol=1e-13, rtol=0)
    np.testing.assert_allclose(d["ints"], ham.ints_physicist(), atol=1e-15, rtol=0)
    d = U.read_fcidump(path, 1, 2)
    a = slice(1, ham.nact - 2)
    np.testing.assert_allclose(d["fock"], ham.fock[a, a], atol=1e-13, rtol=0)
    np.testing.assert_allclose(d["ints"], ham.ints_physicist()[a, a, a, a], atol=1e-15, rtol=0)


def test_bad_files_raise(tmp_path):
    h, eri, enuc = _random_system(5, 2, 2)
    good = str(tmp_path / "good")
    FD.write(good, h, eri, enuc, 4)
    with pytest.raises(U.UccError, match="cannot open"):
        U.read_fcidump(str(tmp_path / "missing"))
    with pytest.raises(U.UccError, match="leave no active"):
        U.read_fcidump(good, 2, 0)
    with pytest.raises(U.UccError, match="leave no active"):
        U.read_fcidump(good, 0, 3)
    open_shell = str(tmp_path / "ms2")
    FD.write(open_shell, h, eri, enuc, 4, ms2=2)
    with pytest.raises(U.UccError, match="closed-shell") as e:
        U.read_fcidump(open_shell)
    assert e.value.status == 8
    text = open(good).read().splitlines()
    bad_idx = str(tmp_path / "idx")
    body = next(i for i, line in enumerate(text) if "&END" in line) + 1
    open(bad_idx, "w").write("\n".join(text[:body] + ["1.0 9 1 1 1"] + text[body:]) + "\n")
    with pytest.raises(U.UccError, match="out of range"):
        U.read_fcidump(bad_idx)
    no_hdr = str(tmp_path / "nohdr")
    open(no_hdr, "w").write("\n".join(text[body:]) + "\n")
    with pytest.raises(U.UccError, match="header"):
        U.read_fcidump(no_hdr)


def test_driver_rejects_frozen_orbitals_past_the_occupied_space(tmp_path):
    import subprocess

    from ugacc_gb300.build import DRIVER

    h, eri, enuc = _random_system(6, 3, 4)
    path = str(tmp_path / "FCIDUMP")
    FD.write(path, h, eri, enuc, 6)
    r = subprocess.run([DRIVER, path, "NFZC=3"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "no active" in r.stderr


def test_orbital_energies_put_irrep_grouped_files_in_qt_order(tmp_path):
    """A file whose orbitals are listed out of energy order (as symmetry-using programs
    group them by irrep), with an energy line for every orbital, reads as the same
    Hamiltonian as the energy-ordered file; without energy lines the file order is kept."""
    n, nelec = 10, 8
    h, eri, enuc = _random_system(n, 4, 21)
    eps = np.sort(np.random.default_rng(3).uniform(-2.0, 3.0, n))
    ordered = str(tmp_path / "ordered")
    FD.write(ordered, h, eri, enuc, nelec, orbital_energies=eps)
    perm = np.array([0, 4, 8, 1, 5, 9, 2, 6, 3, 7])  # "irreps" {0,4,8}, {1,5,9}, {2,6}, {3,7}
    hp, ep = h[np.ix_(perm, perm)], eps[perm]
    erip = eri[np.ix_(perm, perm, perm, perm)]
    grouped = str(tmp_path / "grouped")
    FD.write(grouped, hp, erip, enuc, nelec, orbital_energies=ep, scramble=True, seed=2)
    for nfzc, nfzv in [(0, 0), (1, 2)]:
        a, b = U.read_fcidump(ordered, nfzc, nfzv), U.read_fcidump(grouped, nfzc, nfzv)
        np.testing.assert_allclose(b["fock"], a["fock"], atol=1e-13, rtol=0)
        np.testing.assert_allclose(b["ints"], a["ints"], atol=1e-14, rtol=0)
        assert abs(a["escf"] - b["escf"]) < 1e-12 and abs(a["efzc"] - b["efzc"]) < 1e-12
        ref = FD.hamiltonian(hp, erip, enuc, 4, nfzc, nfzv, orbital_energies=ep)
        np.testing.assert_allclose(b["fock"], ref[0], atol=1e-13, rtol=0)
        # order maps each active QT orbital to the grouped file's orbital: a file-ordered
        # matrix cut with it equals the energy-ordered file's active block
        order = b["order"]
        assert np.array_equal(ep[order], eps[nfzc:n - nfzv])
        np.testing.assert_allclose(hp[np.ix_(order, order)], h[nfzc:n - nfzv, nfzc:n - nfzv], atol=0, rtol=0)
    no_e = str(tmp_path / "no_energies")
    FD.write(no_e, hp, erip, enuc, nelec)
    c = U.read_fcidump(no_e)
    np.testing.assert_allclose(c["fock"], FD.hamiltonian(hp, erip, enuc, 4)[0], atol=1e-13, rtol=0)
