"""GB300-native RHF coupled-cluster solver behind ugacc's class surface.

The classes mirror the reference's pipeline (ugacc.cc:108-241): ``Hamiltonian`` ->
``CCWfn.compute_energy`` -> ``HBAR`` -> ``CCLambda.compute_lambda`` ->
``CCDensity.onepdm/twopdm`` -> ``CCPert.solve`` -> ``CCResp.linresp``, with the same
option names (ugacc.cc:57-68) and the same error behaviour (non-convergence raises
``ConvergenceError("Computation has not converged.")`` like ccwfn.cc:231).  Every call
goes through the C ABI of ``lib/libugacc_gb300.so`` (include/ugacc_gb300.h); there is no
CPU fallback: without the library or a GPU the calls raise.
"""
from __future__ import annotations

import ctypes
import os
import re

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "lib", "libugacc_gb300.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "ugacc_gb300.h")

UCC_OK, UCC_NOT_CONVERGED = 0, 1
STATUS = {0: "ok", 1: "not converged", 2: "nan detected", 3: "out of memory", 4: "bad arguments",
          5: "bad state", 6: "cuda error", 7: "device timeout", 8: "unsupported"}
FP64, MIXED, MIXED_FINE, FP64_SLICED = 0, 1, 2, 3
LEFT, RIGHT = 0, 1


class UccError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class ConvergenceError(UccError):
    """The reference's PSIEXCEPTION("Computation has not converged.")."""


class _Options(ctypes.Structure):
    _fields_ = [("maxiter", ctypes.c_int), ("r_convergence", ctypes.c_double), ("diis", ctypes.c_int),
                ("precision", ctypes.c_int), ("refine_sweeps", ctypes.c_int), ("print", ctypes.c_int),
                ("mixed_switch", ctypes.c_double), ("ooc", ctypes.c_int)]


class Stats(ctypes.Structure):
    _fields_ = [("ccsd_ms", ctypes.c_double), ("triples_ms", ctypes.c_double), ("hbar_ms", ctypes.c_double),
                ("lambda_ms", ctypes.c_double), ("density_ms", ctypes.c_double), ("pert_ms", ctypes.c_double),
                ("ccsd_flops", ctypes.c_double), ("triples_flops", ctypes.c_double),
                ("ccsd_iterations", ctypes.c_int), ("lambda_iterations", ctypes.c_int),
                ("kernel_launches", ctypes.c_int64), ("ladder_ms", ctypes.c_double),
                ("ladder_bytes", ctypes.c_double), ("ladder_flops", ctypes.c_double),
                ("ladder_launches", ctypes.c_int64), ("fp64_iterations", ctypes.c_int),
                ("tc_gemm_launches", ctypes.c_int64), ("mixed_iterations", ctypes.c_int),
                ("tc_gemm_ms", ctypes.c_double), ("tc_gemm_flops", ctypes.c_double),
                ("anchored_iterations", ctypes.c_int), ("fp64_gemm_ms", ctypes.c_double),
                ("fp64_gemm_flops", ctypes.c_double), ("fp64_gemm_launches", ctypes.c_int64),
                ("sliced_gemm_ms", ctypes.c_double), ("sliced_gemm_flops", ctypes.c_double),
                ("sliced_gemm_launches", ctypes.c_int64), ("guess_ms", ctypes.c_double),
                ("sliced_gemm_product_flops", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class BatchInfo(ctypes.Structure):
    _fields_ = [("members", ctypes.c_int), ("sweeps", ctypes.c_int), ("grouped_ops", ctypes.c_int),
                ("graph_kernels", ctypes.c_int), ("shape_choice", ctypes.c_int * 4), ("solve_ms", ctypes.c_double),
                ("flops", ctypes.c_double), ("arena_bytes", ctypes.c_double), ("graph_launches", ctypes.c_int)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_}
        d["shape_choice"] = list(self.shape_choice)
        return d


_lib = None


def declared_functions() -> list[str]:
    """Names of the functions include/ugacc_gb300.h declares."""
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:[\w\s\*]+?)\b(ucc_\w+)\s*\(", text, flags=re.M)))


def load_library(path: str | None = None):
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIBPATH
    if not os.path.exists(path):
        raise UccError(6, f"GPU library not built: {path} (run python -m ugacc_gb300.build)")
    lib = ctypes.CDLL(path)
    P = ctypes.POINTER
    d, i, vp, cp = ctypes.c_double, ctypes.c_int, ctypes.c_void_p, ctypes.c_char_p
    dp = P(d)
    fp = P(ctypes.c_float)
    sig = {
        "ucc_options_default": (None, [P(_Options)]),
        "ucc_ctx_create": (i, [P(vp), i]),
        "ucc_ctx_destroy": (i, [vp]),
        "ucc_set_options": (i, [vp, P(_Options)]),
        "ucc_load_hamiltonian": (i, [vp, i, i, dp, dp]),
        "ucc_load_hamiltonian_df": (i, [vp, i, i, i, dp, dp]),
        "ucc_ccsd": (i, [vp, dp, P(i)]),
        "ucc_triples": (i, [vp, dp]),
        "ucc_triples_gradient": (i, [vp]),
        "ucc_hbar": (i, [vp]),
        "ucc_lambda": (i, [vp, dp, P(i)]),
        "ucc_density": (i, [vp, dp, dp]),
        "ucc_twopdm_energies": (i, [vp, dp]),
        "ucc_pert_create": (i, [vp, dp, d, P(i)]),
        "ucc_pert_solve": (i, [vp, i, i, dp, P(i)]),
        "ucc_linresp": (i, [vp, i, i, dp]),
        "ucc_get_tensor": (i, [vp, cp, dp, ctypes.c_size_t]),
        "ucc_set_tensor": (i, [vp, cp, dp, ctypes.c_size_t]),
        "ucc_get_stats": (i, [vp, P(Stats)]),
        "ucc_reset_stats": (i, [vp]),
        "ucc_last_error": (cp, [vp]),
        "ucc_status_string": (cp, [i]),
        "ucc_triples_noalloc": (i, [i, i, vp, vp, vp, vp, vp, vp, dp, vp, cp, ctypes.c_size_t]),
        "ucc_gemm": (i, [vp, i, i, i, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, d, dp, dp, d, dp]),
        "ucc_gemm_sliced": (i, [vp, i, i, i, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, d, dp, dp, d, dp]),
        "ucc_wait_selftest": (i, [vp, ctypes.c_uint64]),
        "ucc_mlp_create": (i, [P(vp), i, ctypes.c_uint64]),
        "ucc_mlp_destroy": (i, [vp]),
        "ucc_mlp_last_error": (cp, [vp]),
        "ucc_mlp_num_params": (i, []),
        "ucc_mlp_get_params": (i, [vp, fp, ctypes.c_size_t]),
        "ucc_mlp_set_params": (i, [vp, fp, ctypes.c_size_t]),
        "ucc_mlp_predict": (i, [vp, fp, ctypes.c_int64, fp]),
        "ucc_mlp_loss_grad": (i, [vp, fp, fp, ctypes.c_int64, fp, fp, ctypes.c_size_t]),
        "ucc_mlp_train": (i, [vp, fp, fp, ctypes.c_int64, i, i, ctypes.c_float, ctypes.c_uint64, fp]),
        "ucc_mlp_features": (i, [vp, fp, ctypes.c_size_t, i, fp]),
        "ucc_mlp_guess": (i, [vp, vp]),
        "ucc_batch_create": (i, [P(vp), i]),
        "ucc_batch_destroy": (i, [vp]),
        "ucc_batch_last_error": (cp, [vp]),
        "ucc_batch_add_df": (i, [vp, i, i, i, dp, dp, P(i)]),
        "ucc_batch_guess_mlp": (i, [vp, i, vp]),
        "ucc_batch_ccsd": (i, [vp, P(_Options), dp, P(i), P(i)]),
        "ucc_batch_set_time_limit": (i, [vp, d]),
        "ucc_batch_get_info": (i, [vp, P(BatchInfo)]),
        "ucc_batch_get_t2": (i, [vp, i, dp, ctypes.c_size_t]),
        "ucc_batch_features": (i, [vp, i, fp, ctypes.c_size_t, i, fp]),
        "ucc_fcidump_dims": (i, [cp, P(i), P(i), cp, ctypes.c_size_t]),
        "ucc_fcidump_read": (i, [cp, i, i, dp, dp, dp, P(i), cp, ctypes.c_size_t]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Context:
    """One device context (``ucc_ctx``) holding a Hamiltonian and every stage's arrays."""

    def __init__(self, device: int = 0):
        self.lib = load_library()
        h = ctypes.c_void_p()
        st = self.lib.ucc_ctx_create(ctypes.byref(h), device)
        if st != UCC_OK:
            raise UccError(st, "cannot create a context on CUDA device %d" % device)
        self.h = h

    def check(self, st: int):
        if st == UCC_OK:
            return
        msg = (self.lib.ucc_last_error(self.h) or b"").decode()
        if st == UCC_NOT_CONVERGED:
            raise ConvergenceError(st, msg or "Computation has not converged.")
        raise UccError(st, msg)

    def set_options(self, maxiter=100, r_convergence=1e-7, diis=True, precision=FP64, refine_sweeps=2, printing=0,
                    mixed_switch=1e-5, ooc=False):
        o = _Options(maxiter, r_convergence, int(diis), precision, refine_sweeps, printing, mixed_switch, int(bool(ooc)))
        self.check(self.lib.ucc_set_options(self.h, ctypes.byref(o)))

    def get(self, name: str, shape) -> np.ndarray:
        out = np.empty(shape, dtype=np.float64)
        self.check(self.lib.ucc_get_tensor(self.h, name.encode(), _ptr(out), out.size))
        return out

    def set(self, name: str, arr: np.ndarray):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        self.check(self.lib.ucc_set_tensor(self.h, name.encode(), _ptr(a), a.size))

    def gemm(self, A, B, C=None, alpha=1.0, beta=0.0, transa=False, transb=False, precision=FP64, digits=None):
        """C = alpha op(A) op(B) + beta C on the GPU (ucc_gemm); `digits` (2 to 9) selects the
        sliced FP64 product with that many base-2^6 digits per operand (ucc_gemm_sliced)."""
        A = np.ascontiguousarray(A, dtype=np.float64)
        B = np.ascontiguousarray(B, dtype=np.float64)
        M, K = (A.shape[1], A.shape[0]) if transa else A.shape
        N = B.shape[0] if transb else B.shape[1]
        C = np.zeros((M, N)) if C is None else np.array(C, dtype=np.float64, order="C")
        if digits is None:
            self.check(self.lib.ucc_gemm(self.h, precision, int(transa), int(transb), M, N, K, alpha, _ptr(A),
                                         _ptr(B), beta, _ptr(C)))
        else:
            self.check(self.lib.ucc_gemm_sliced(self.h, int(digits), int(transa), int(transb), M, N, K, alpha,
                                                _ptr(A), _ptr(B), beta, _ptr(C)))
        return C

    def wait_selftest(self, limit_s: float = 0.05):
        """Run a bounded device wait that nothing completes (ucc_wait_selftest); raises
        UccError with status 7 (device timeout) when the failure path works."""
        self.check(self.lib.ucc_wait_selftest(self.h, int(limit_s * 1e9)))

    def stats(self) -> dict:
        s = Stats()
        self.check(self.lib.ucc_get_stats(self.h, ctypes.byref(s)))
        return s.as_dict()

    def reset_stats(self):
        self.check(self.lib.ucc_reset_stats(self.h))

    def close(self):
        if getattr(self, "h", None):
            self.lib.ucc_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------------------------------------
# Mirror of the reference's classes
# ------------------------------------------------------------------------------------
DEFAULT_OPTIONS = {"WFN": "CCSD", "DERTYPE": "NONE", "MAXITER": 100, "R_CONVERGENCE": 1e-7, "DIIS": True,
                   "MYHAND": "RIGHT", "MY_OMEGA": 0.0, "PRECISION": "FP64", "REFINE_SWEEPS": 2, "PRINT": 0,
                   "MIXED_SWITCH": 1e-5, "OOC": False}


def read_fcidump(path: str, nfzc: int = 0, nfzv: int = 0) -> dict:
    """Active-space Hamiltonian from an MO-integral file in the FCIDUMP layout (host code,
    no GPU): the integral side of hamiltonian.cc:21-102 with ``nfzc`` frozen core and
    ``nfzv`` frozen virtual orbitals.  When the file gives an energy for every orbital,
    the NELEC/2 lowest are occupied and the orbitals go to QT order, occupied then
    virtual, each by ascending energy (stable, so an energy-ordered file keeps its
    order); otherwise the file's order is kept, the first NELEC/2 doubly occupied.
    Returns ``no``, ``nv``, ``fock`` [nact][nact], ``ints`` [nact]^4
    (``ints[p,q,r,s] = <pq|rs>``), ``enuc``, ``efzc`` (frozen-core energy), ``escf`` and
    ``order`` (the file's 0-based orbital at each active QT position: a file-ordered MO
    matrix ``P`` becomes ``P[np.ix_(order, order)]`` on the active space)."""
    lib = load_library()
    err = ctypes.create_string_buffer(512)
    norb, nelec = ctypes.c_int(), ctypes.c_int()
    bpath = os.fsencode(path)
    st = lib.ucc_fcidump_dims(bpath, ctypes.byref(norb), ctypes.byref(nelec), err, 512)
    if st:
        raise UccError(st, err.value.decode())
    nact = norb.value - nfzc - nfzv
    if nact <= 0:
        raise UccError(4, "fcidump: frozen orbitals leave no active orbital")
    fock = np.empty((nact, nact))
    ints = np.empty((nact,) * 4)
    en = np.empty(3)
    order = np.empty(nact, dtype=np.int32)
    st = lib.ucc_fcidump_read(bpath, nfzc, nfzv, _ptr(fock), _ptr(ints), _ptr(en),
                              order.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), err, 512)
    if st:
        raise UccError(st, err.value.decode())
    no = nelec.value // 2 - nfzc
    return {"no": no, "nv": nact - no, "fock": fock, "ints": ints, "enuc": float(en[0]), "efzc": float(en[1]),
            "escf": float(en[2]), "order": order}


class Hamiltonian:
    """hamiltonian.h:12-34: Fock matrix (QT order) and two-electron integrals.

    Either ``ints`` ([nact]^4, ``ints[p,q,r,s] = <pq|rs>``, the reference's layout) or the
    density-fitting factors ``B`` ([naux][nact][nact]) are accepted."""

    def __init__(self, no: int, nv: int, fock: np.ndarray, ints: np.ndarray | None = None,
                 B: np.ndarray | None = None, device: int = 0, context: Context | None = None,
                 precision: str | None = None):
        self.no, self.nv = no, nv
        self.ctx = context or Context(device)
        if precision is not None:  # "MIXED": the blocks are built by the sliced tensor-core GEMM
            self.ctx.set_options(precision=MIXED if precision.upper() == "MIXED" else FP64)
        f = np.ascontiguousarray(fock, dtype=np.float64)
        if ints is not None:
            x = np.ascontiguousarray(ints, dtype=np.float64)
            self.ctx.check(self.ctx.lib.ucc_load_hamiltonian(self.ctx.h, no, nv, _ptr(f), _ptr(x)))
        elif B is not None:
            b = np.ascontiguousarray(B, dtype=np.float64)
            self.ctx.check(self.ctx.lib.ucc_load_hamiltonian_df(self.ctx.h, no, nv, b.shape[0], _ptr(f), _ptr(b)))
        else:
            raise ValueError("need ints or B")

    @classmethod
    def from_fcidump(cls, path: str, nfzc: int = 0, nfzv: int = 0, **kw):
        """hamiltonian.cc:21-102 from an FCIDUMP file (``read_fcidump``); the file's
        energies are kept as ``enuc``, ``efzc`` and ``escf``."""
        d = read_fcidump(path, nfzc, nfzv)
        H = cls(d["no"], d["nv"], d["fock"], ints=d["ints"], **kw)
        H.enuc, H.efzc, H.escf, H.order = d["enuc"], d["efzc"], d["escf"], d["order"]
        return H

    @classmethod
    def from_synthetic(cls, ham, use_ints: bool = False, **kw):
        if use_ints:
            return cls(ham.no, ham.nv, ham.fock, ints=ham.ints_physicist(), **kw)
        return cls(ham.no, ham.nv, ham.fock, B=ham.B, **kw)


class CCWfn:
    """ccwfn.h:12-106: CCSD (and (T) for WFN=CCSD_T) ground state."""

    def __init__(self, H: Hamiltonian, options: dict | None = None):
        self.H, self.ctx = H, H.ctx
        self.options = dict(DEFAULT_OPTIONS, **(options or {}))
        o = self.options
        self.ctx.set_options(maxiter=int(o["MAXITER"]), r_convergence=float(o["R_CONVERGENCE"]), diis=bool(o["DIIS"]),
                             precision=MIXED if str(o["PRECISION"]).upper() == "MIXED" else FP64,
                             refine_sweeps=int(o["REFINE_SWEEPS"]), printing=int(o["PRINT"]),
                             mixed_switch=float(o["MIXED_SWITCH"]), ooc=bool(o["OOC"]))
        self.no, self.nv = H.no, H.nv
        self.eccsd = self.et = None
        self.iterations = 0

    def compute_energy(self) -> float:
        """ccwfn.cc:188-258: CCSD correlation energy, plus (T) when WFN == CCSD_T."""
        e = ctypes.c_double()
        it = ctypes.c_int()
        st = self.ctx.lib.ucc_ccsd(self.ctx.h, ctypes.byref(e), ctypes.byref(it))
        self.iterations = it.value
        self.ctx.check(st)
        self.eccsd = e.value
        total = self.eccsd
        if self.options["WFN"] == "CCSD_T":
            self.et = self.triples()
            total += self.et
            if self.options["DERTYPE"] == "FIRST":  # ccwfn.cc:252-255
                self.triples_gradient()
        return total

    def triples_gradient(self):
        """ccwfn.cc:854-1142 (tgrad, OOC false) or :1150-1316 (tgrad_ooc, OOC true): s1, s2 and
        the (T) density pieces, which the following CCLambda and CCDensity include."""
        self.ctx.check(self.ctx.lib.ucc_triples_gradient(self.ctx.h))

    def triples(self) -> float:
        """ccwfn.cc:795-852 (tcorr_ooc_TJL)."""
        e = ctypes.c_double()
        self.ctx.check(self.ctx.lib.ucc_triples(self.ctx.h, ctypes.byref(e)))
        return e.value

    @property
    def t1(self):
        return self.ctx.get("t1", (self.no, self.nv))

    @property
    def t2(self):
        return self.ctx.get("t2", (self.no, self.no, self.nv, self.nv))


class HBAR:
    """hbar.h:11-36: similarity-transformed Hamiltonian blocks."""

    SHAPES = {"Hov": "ov", "Hoo": "oo", "Hvv": "vv", "Hoooo": "oooo", "Hvvvv": "vvvv", "Hvovv": "vovv",
              "Hooov": "ooov", "Hovvo": "ovvo", "Hovov": "ovov", "Hvvvo": "vvvo", "Hovoo": "ovoo"}

    def __init__(self, H: Hamiltonian, cc: CCWfn):
        self.H, self.cc, self.ctx = H, cc, cc.ctx
        self.ctx.check(self.ctx.lib.ucc_hbar(self.ctx.h))

    def block(self, name: str) -> np.ndarray:
        shape = tuple(self.H.no if ch == "o" else self.H.nv for ch in self.SHAPES[name])
        return self.ctx.get(name, shape)


class CCLambda:
    """cclambda.h:13-63."""

    def __init__(self, cc: CCWfn, hbar: HBAR):
        self.cc, self.hbar, self.ctx = cc, hbar, cc.ctx
        self.pseudo = None
        self.iterations = 0

    def compute_lambda(self):
        e = ctypes.c_double()
        it = ctypes.c_int()
        st = self.ctx.lib.ucc_lambda(self.ctx.h, ctypes.byref(e), ctypes.byref(it))
        self.iterations = it.value
        self.ctx.check(st)
        self.pseudo = e.value

    def pseudoenergy(self):
        return self.pseudo

    @property
    def l1(self):
        return self.ctx.get("l1", (self.cc.no, self.cc.nv))

    @property
    def l2(self):
        return self.ctx.get("l2", (self.cc.no, self.cc.no, self.cc.nv, self.cc.nv))


class CCDensity:
    """ccdensity.h:12-50.  onepdm() and twopdm() return the energy contributions."""

    def __init__(self, cc: CCWfn, lam: CCLambda):
        self.cc, self.lam, self.ctx = cc, lam, cc.ctx
        self._e = None

    def _run(self):
        if self._e is None:
            a, b = ctypes.c_double(), ctypes.c_double()
            self.ctx.check(self.ctx.lib.ucc_density(self.ctx.h, ctypes.byref(a), ctypes.byref(b)))
            self._e = (a.value, b.value)
        return self._e

    def onepdm(self) -> float:
        return self._run()[0]

    def twopdm(self) -> float:
        return self._run()[1]

    PARTS = ("OOOO", "VVVV", "OOOV", "VVVO", "OVOV", "OOVV")

    def block(self, name: str) -> np.ndarray:
        """One- or two-particle density block: Doo Dvv Dov Dvo, Goooo Gvvvv Gooov Gvvvo
        Govov Goovv (ccdensity.h:32-44 layouts)."""
        shape = tuple(self.cc.no if ch == "o" else self.cc.nv for ch in name[1:])
        self._run()
        return self.ctx.get(name, shape)

    def twopdm_parts(self) -> dict:
        """The six two-particle energies the reference prints (ccdensity.cc:181-335)."""
        self._run()
        out = np.zeros(6)
        self.ctx.check(self.ctx.lib.ucc_twopdm_energies(self.ctx.h, _ptr(out)))
        return dict(zip(self.PARTS, out.tolist()))


class CCPert:
    """ccpert.h:17-80: perturbed wavefunction for one operator at frequency omega."""

    def __init__(self, pert: np.ndarray, omega: float, cc: CCWfn, hbar: HBAR, lam: CCLambda):
        self.cc, self.ctx, self.omega = cc, cc.ctx, omega
        p = np.ascontiguousarray(pert, dtype=np.float64)
        h = ctypes.c_int()
        self.ctx.check(self.ctx.lib.ucc_pert_create(self.ctx.h, _ptr(p), float(omega), ctypes.byref(h)))
        self.handle = h.value
        self.iterations = {}

    def solve(self, hand: str = "right") -> float:
        e = ctypes.c_double()
        it = ctypes.c_int()
        hd = RIGHT if hand in ("right", RIGHT) else LEFT
        st = self.ctx.lib.ucc_pert_solve(self.ctx.h, self.handle, hd, ctypes.byref(e), ctypes.byref(it))
        self.iterations["right" if hd == RIGHT else "left"] = it.value
        self.ctx.check(st)
        return e.value

    def amp(self, name: str) -> np.ndarray:
        no, nv = self.cc.no, self.cc.nv
        shape = (no, nv) if name.endswith("1") else (no, no, nv, nv)
        return self.ctx.get(f"{name}:{self.handle}", shape)


class CCResp:
    """ccresp.h:10-28."""

    def __init__(self, X: CCPert, Y: CCPert):
        self.X, self.Y, self.ctx = X, Y, X.ctx

    def linresp(self, X: CCPert, Y: CCPert) -> float:
        v = ctypes.c_double()
        self.ctx.check(self.ctx.lib.ucc_linresp(self.ctx.h, X.handle, Y.handle, ctypes.byref(v)))
        return v.value


def response(cc: CCWfn, hbar: HBAR, lam: CCLambda, perts, omega: float, hand: str = "right"):
    """The recipe of ugacc.cc:158-227 for 3 dipole and 3 angular-momentum operators:
    returns the symmetrised polarizability and the length-gauge rotation tensors."""
    axes = "XYZ"
    P = {}
    for x in range(3):
        P["Mu" + axes[x]] = CCPert(perts[x], omega, cc, hbar, lam)
        P["Mu" + axes[x]].solve("right")
        P["L" + axes[x]] = CCPert(perts[3 + x], omega, cc, hbar, lam)
        P["L" + axes[x]].solve("right")
        if hand == "left":
            P["Mu" + axes[x]].solve("left")
            P["L" + axes[x]].solve("left")
    alpha, rot = {}, {}
    for p in range(3):
        for q in range(p + 1):
            A, B = P["Mu" + axes[p]], P["Mu" + axes[q]]
            r = CCResp(A, B)
            alpha[axes[p] + axes[q]] = r.linresp(A, B) if p == q else 0.5 * r.linresp(A, B) + 0.5 * r.linresp(B, A)
    for p in range(3):
        for q in range(3):
            A, B = P["Mu" + axes[p]], P["L" + axes[q]]
            r = CCResp(A, B)
            rot[axes[p] + axes[q]] = -(0.5 * r.linresp(A, B) - 0.5 * r.linresp(B, A))
    return alpha, rot, P


# ------------------------------------------------------------------------------------
# Learned T2 starting amplitudes
# ------------------------------------------------------------------------------------
def _fptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


class MLP:
    """The guess network of mlp.cu: 15 pair features -> 256 -> 256 -> 1 (SiLU)."""

    NFEAT = 15

    def __init__(self, device: int = 0, seed: int = 0):
        self.lib = load_library()
        h = ctypes.c_void_p()
        st = self.lib.ucc_mlp_create(ctypes.byref(h), device, seed)
        if st != UCC_OK:
            raise UccError(st, "cannot create the network")
        self.h = h
        self.nparam = self.lib.ucc_mlp_num_params()

    def check(self, st):
        if st != UCC_OK:
            raise UccError(st, (self.lib.ucc_mlp_last_error(self.h) or b"").decode())

    @property
    def params(self) -> np.ndarray:
        out = np.empty(self.nparam, dtype=np.float32)
        self.check(self.lib.ucc_mlp_get_params(self.h, _fptr(out), out.size))
        return out

    @params.setter
    def params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        self.check(self.lib.ucc_mlp_set_params(self.h, _fptr(p), p.size))

    def predict(self, X) -> np.ndarray:
        X = np.ascontiguousarray(X, dtype=np.float32)
        y = np.empty(X.shape[0], dtype=np.float32)
        self.check(self.lib.ucc_mlp_predict(self.h, _fptr(X), X.shape[0], _fptr(y)))
        return y

    def loss_grad(self, X, t):
        X = np.ascontiguousarray(X, dtype=np.float32)
        t = np.ascontiguousarray(t, dtype=np.float32)
        loss = ctypes.c_float()
        g = np.empty(self.nparam, dtype=np.float32)
        self.check(self.lib.ucc_mlp_loss_grad(self.h, _fptr(X), _fptr(t), X.shape[0], ctypes.byref(loss), _fptr(g),
                                              g.size))
        return loss.value, g

    def train(self, X, t, epochs=5, batch=4096, lr=1e-3, seed=0) -> float:
        X = np.ascontiguousarray(X, dtype=np.float32)
        t = np.ascontiguousarray(t, dtype=np.float32)
        loss = ctypes.c_float()
        self.check(self.lib.ucc_mlp_train(self.h, _fptr(X), _fptr(t), X.shape[0], epochs, batch, lr, seed,
                                          ctypes.byref(loss)))
        return loss.value

    def guess(self, H: "Hamiltonian"):
        """The next CCWfn.compute_energy() on H starts from the network's T2."""
        H.ctx.check(self.lib.ucc_mlp_guess(H.ctx.h, self.h))

    def close(self):
        if getattr(self, "h", None):
            self.lib.ucc_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def mlp_features(H: "Hamiltonian", with_targets: bool = False):
    """Pair features (and targets after a converged CCSD) of every T2 element of H."""
    n = H.no * H.no * H.nv * H.nv
    X = np.empty((n, MLP.NFEAT), dtype=np.float32)
    t = np.empty(n, dtype=np.float32) if with_targets else None
    lib = H.ctx.lib
    H.ctx.check(lib.ucc_mlp_features(H.ctx.h, _fptr(X), n, int(with_targets),
                                     _fptr(t) if with_targets else None))
    return (X, t) if with_targets else X


# ------------------------------------------------------------------------------------
# Batched CCSD over many Hamiltonians
# ------------------------------------------------------------------------------------
class Batch:
    """Many small Hamiltonians solved together (ucc_batch_*): the whole solve is one graph
    launch whose sweep loop runs on the device."""

    def __init__(self, device: int = 0):
        self.lib = load_library()
        h = ctypes.c_void_p()
        st = self.lib.ucc_batch_create(ctypes.byref(h), device)
        if st != UCC_OK:
            raise UccError(st, "cannot create a batch on CUDA device %d" % device)
        self.h = h
        self.sizes = []

    def check(self, st):
        if st != UCC_OK:
            raise UccError(st, (self.lib.ucc_batch_last_error(self.h) or b"").decode())

    def add(self, ham) -> int:
        """Add a synthetic Hamiltonian (no, nv, naux, eps/fock, B)."""
        fock = np.ascontiguousarray(ham.fock, dtype=np.float64)
        B = np.ascontiguousarray(ham.B, dtype=np.float64)
        idx = ctypes.c_int()
        self.check(self.lib.ucc_batch_add_df(self.h, ham.no, ham.nv, ham.naux, _ptr(fock), _ptr(B), ctypes.byref(idx)))
        self.sizes.append((ham.no, ham.nv))
        return idx.value

    def guess(self, index: int, net: "MLP"):
        self.check(self.lib.ucc_batch_guess_mlp(self.h, index, net.h))

    def set_time_limit(self, seconds: float):
        """Device time limit of the next solves' sweep loop (UCC_DEVICE_TIMEOUT when it runs out)."""
        self.check(self.lib.ucc_batch_set_time_limit(self.h, float(seconds)))

    def ccsd(self, options: dict | None = None):
        """Energies, iteration counts and convergence flags of every member."""
        o = dict(DEFAULT_OPTIONS, **(options or {}))
        prec = MIXED if str(o["PRECISION"]).upper() == "MIXED" else FP64
        opts = _Options(int(o["MAXITER"]), float(o["R_CONVERGENCE"]), int(bool(o["DIIS"])), prec,
                        int(o["REFINE_SWEEPS"]), int(o["PRINT"]), float(o["MIXED_SWITCH"]))
        n = len(self.sizes)
        e = np.zeros(n)
        it = (ctypes.c_int * n)()
        cv = (ctypes.c_int * n)()
        self.check(self.lib.ucc_batch_ccsd(self.h, ctypes.byref(opts), _ptr(e), it, cv))
        return e, np.array(list(it)), np.array(list(cv), dtype=bool)

    def info(self) -> dict:
        out = BatchInfo()
        self.check(self.lib.ucc_batch_get_info(self.h, ctypes.byref(out)))
        return out.as_dict()

    def t2(self, index: int) -> np.ndarray:
        no, nv = self.sizes[index]
        out = np.empty((no, no, nv, nv))
        self.check(self.lib.ucc_batch_get_t2(self.h, index, _ptr(out), out.size))
        return out

    def features(self, index: int, with_targets: bool = False):
        """Pair features (and targets after a converged solve) of member `index`."""
        no, nv = self.sizes[index]
        n = no * no * nv * nv
        X = np.empty((n, MLP.NFEAT), dtype=np.float32)
        t = np.empty(n, dtype=np.float32) if with_targets else None
        self.check(self.lib.ucc_batch_features(self.h, index, _fptr(X), n, int(with_targets),
                                               _fptr(t) if with_targets else None))
        return (X, t) if with_targets else X

    def close(self):
        if getattr(self, "h", None):
            self.lib.ucc_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
