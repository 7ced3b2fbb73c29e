"""The allocation-free (T) entry point against the regular one.

ucc_triples_noalloc is for callers that cannot let the library allocate device memory:
they hand in their own device buffers and the library works in a fixed static array.
This file runs last (pytest collects files alphabetically) and must pass both on its own
in a fresh process and after the rest of the suite.
"""
import ctypes

import numpy as np
import pytest

import ugacc_gb300 as U
from ugacc_gb300.generator import make_hamiltonian

pytestmark = pytest.mark.gpu


def _inputs(h, cc):
    import torch

    no = h.no
    V = h.ints_physicist()
    host = {
        "t1": cc.t1, "t2": cc.t2, "eps": h.eps,
        "ovvv": V[:no, no:, no:, no:], "ooov": V[:no, :no, :no, no:], "oovv": V[:no, :no, no:, no:],
    }
    dev = {k: torch.tensor(np.ascontiguousarray(v), dtype=torch.float64, device="cuda") for k, v in host.items()}
    torch.cuda.synchronize()
    return dev


def _call(lib, no, nv, d):
    e = ctypes.c_double(0.0)
    buf = ctypes.create_string_buffer(512)
    ptr = lambda k: ctypes.c_void_p(d[k].data_ptr())
    st = lib.ucc_triples_noalloc(no, nv, ptr("t1"), ptr("t2"), ptr("eps"), ptr("ovvv"), ptr("ooov"), ptr("oovv"),
                                 ctypes.byref(e), None, buf, len(buf))
    return st, e.value, buf.value.decode()


@pytest.mark.parametrize("no,nv,seed", [(5, 19, 0), (6, 40, 5)])
def test_noalloc_triples_matches_regular_entry_point(no, nv, seed):
    pytest.importorskip("torch")
    h = make_hamiltonian(no, nv, seed)
    H = U.Hamiltonian.from_synthetic(h, use_ints=True)
    cc = U.CCWfn(H, {"R_CONVERGENCE": 1e-10})
    cc.compute_energy()
    e_regular = cc.triples()
    d = _inputs(h, cc)
    lib = U.load_library()
    for _ in range(2):  # the static scratch keeps the previous call's contents
        st, e, msg = _call(lib, no, nv, d)
        assert st == 0, msg
        assert abs(e - e_regular) < 1e-10, (e, e_regular)


def test_noalloc_rejects_oversized_problems():
    torch = pytest.importorskip("torch")
    lib = U.load_library()
    no, nv = 2, 170  # nv^3 alone exceeds the 32 MiB static array
    one = torch.zeros(1, dtype=torch.float64, device="cuda")
    d = {k: one for k in ["t1", "t2", "eps", "ovvv", "ooov", "oovv"]}
    st, _, msg = _call(lib, no, nv, d)
    assert st == 4 and "static scratch" in msg
