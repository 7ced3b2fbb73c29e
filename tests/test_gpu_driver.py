"""The C++ class surface (include/ugacc_gb300.hpp) through the command-line driver."""
import json
import os
import subprocess

import pytest

from golden_util import load
from ugacc_gb300.build import DRIVER, build
from ugacc_gb300.generator import make_hamiltonian, make_perturbations, write_input_file

pytestmark = pytest.mark.gpu


def test_driver_pipeline_matches_reference(tmp_path):
    build()
    meta, _ = load("c1")
    run = meta["runs"]["right_w0"]
    h = make_hamiltonian(meta["no"], meta["nv"], meta["seed"])
    inp = str(tmp_path / "c1.bin")
    write_input_file(inp, h, make_perturbations(h.nact, meta["seed"]), with_ints=False)
    out = subprocess.run([DRIVER, inp, "WFN=CCSD_T", "DERTYPE=SECOND", "R_CONVERGENCE=1e-10"],
                         capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr
    r = json.loads(out.stdout)
    assert abs(r["e_ccsd"] - run["e_ccsd"]) < 1e-10
    assert abs(r["e_t"] - run["e_t_tjl"]) < 1e-10
    assert abs(r["pseudoenergy"] - run["pseudoenergy"]) < 1e-10
    assert abs(r["e_onepdm"] - run["e_onepdm"]) < 1e-10 and abs(r["e_twopdm"] - run["e_twopdm"]) < 1e-10
    for k in ["XX", "YX", "YY", "ZX", "ZY", "ZZ"]:
        assert abs(r["alpha_" + k] - run["alpha_" + k]) < 1e-9


def test_driver_reports_nonconvergence(tmp_path):
    build()
    h = make_hamiltonian(3, 7, 11)
    inp = str(tmp_path / "t.bin")
    write_input_file(inp, h, [], with_ints=False)
    out = subprocess.run([DRIVER, inp, "MAXITER=1", "R_CONVERGENCE=1e-12"], capture_output=True, text=True,
                         timeout=300)
    assert out.returncode == 3 and "not converged" in out.stderr


def test_driver_reads_fcidump_with_frozen_orbitals(tmp_path):
    """An MO-integral file (FCIDUMP layout) through Hamiltonian::from_fcidump: the driver's
    energies equal the Python API's on the same file; E_total = E_SCF + E_CC."""
    import numpy as np

    import ugacc_gb300 as U
    from oracle import fcidump as FD

    build()
    h = make_hamiltonian(6, 22, 9)
    eri = h.eri_chemist()
    path = str(tmp_path / "FCIDUMP")
    FD.write(path, FD.core_hamiltonian_for(h.fock, eri, h.no), eri, 2.5, 2 * h.no)
    out = subprocess.run([DRIVER, path, "WFN=CCSD_T", "NFZC=1", "NFZV=3", "R_CONVERGENCE=1e-10"],
                         capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr
    r = json.loads(out.stdout)
    H = U.Hamiltonian.from_fcidump(path, nfzc=1, nfzv=3)
    cc = U.CCWfn(H, {"R_CONVERGENCE": 1e-10, "WFN": "CCSD_T"})
    e = cc.compute_energy()
    assert abs(r["e_ccsd"] - cc.eccsd) < 1e-12 and abs(r["e_t"] - cc.et) < 1e-12
    assert abs(r["e_scf"] - H.escf) < 1e-12 and abs(r["e_frozen_core"] - H.efzc) < 1e-12
    assert abs(r["e_total"] - (H.escf + e)) < 1e-12
    assert np.isfinite(r["e_total"])
