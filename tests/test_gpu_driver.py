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
