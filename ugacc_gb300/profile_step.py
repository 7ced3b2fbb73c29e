"""Run a bounded slice of the solver for profiling (ncu launch lists, kernel captures).

    python -m ugacc_gb300.profile_step --no 16 --nv 160 --seed 1 --iters 2 [--triples]
                                       [--precision fp64|mixed] [--gemm M N K]

--print shows the iteration tables; --iters n runs n CCSD iterations from the MP2 guess (MAXITER=n; the not-converged
status is expected and ignored); --triples then adds (T) on converged amplitudes;
--gemm runs one tensor-core GEMM of that shape through ucc_gemm instead.
Prints the library's per-stage CUDA-event timings.
"""
from __future__ import annotations

import argparse
import json
import sys

import numpy as np


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--no", type=int, default=16)
    ap.add_argument("--nv", type=int, default=160)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--iters", type=int, default=1)
    ap.add_argument("--triples", action="store_true")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed", "sliced"],
                    help="sliced: with --gemm only, the FP64-accurate sliced tensor-core GEMM")
    ap.add_argument("--gemm", type=int, nargs=3, metavar=("M", "N", "K"))
    ap.add_argument("--print", type=int, nargs="?", const=1, default=0,
                    help="print the iteration tables (2: also the residual error of every mixed sweep)")
    ap.add_argument("--switch", type=float, default=1e-5, help="MIXED hand-over residual norm")
    ap.add_argument("--diis", type=int, default=1, help="0 turns DIIS extrapolation off")
    ap.add_argument("--response", action="store_true",
                    help="CCSD, HBAR, Lambda, densities and the static + dynamic dipole polarizability "
                         "(3 symmetric perturbations, omega 0 and 0.0656, right-hand solves)")
    ap.add_argument("--tgrad", action="store_true", help="with --triples: also the (T) gradient pieces")
    ap.add_argument("--ccsd-fp64", action="store_true",
                    help="with --triples: converge CCSD in FP64, then run (T) at --precision")
    ap.add_argument("--guess", action="store_true",
                    help="with --triples: start CCSD from the learned-guess kernel (an untrained network of seed 1)")
    a = ap.parse_args(argv)

    import ugacc_gb300 as U
    from ugacc_gb300.generator import make_hamiltonian

    if a.gemm:
        M, N, K = a.gemm
        rng = np.random.default_rng(0)
        ctx = U.Context()
        A, B = rng.standard_normal((M, K)), rng.standard_normal((K, N))
        prec = {"mixed": U.MIXED, "sliced": U.FP64_SLICED}.get(a.precision, U.FP64)
        for rep in range(3):
            ctx.reset_stats()
            C = ctx.gemm(A, B, precision=prec)
            st = ctx.stats()
        ms = {U.MIXED: st["tc_gemm_ms"], U.FP64_SLICED: st["sliced_gemm_ms"]}.get(prec, st["fp64_gemm_ms"])
        err = None
        if M * N * K <= 2e10:
            ref = A @ B
            err = float(np.abs(C - ref).max() / np.abs(ref).max())
        print(json.dumps({"gemm": [M, N, K], "precision": a.precision, "ms": ms,
                          "tflops": 2.0 * M * N * K / (ms * 1e-3) / 1e12 if ms else None, "max_rel_err": err}))
        return 0
    h = make_hamiltonian(a.no, a.nv, a.seed)
    H = U.Hamiltonian.from_synthetic(h, precision=a.precision.upper() if a.precision != "sliced" else None)
    prec = a.precision.upper()
    if a.iters > 0:
        cc = U.CCWfn(H, {"MAXITER": a.iters, "R_CONVERGENCE": 1e-10, "PRECISION": prec, "PRINT": int(a.print),
                         "MIXED_SWITCH": a.switch, "DIIS": bool(a.diis)})
        try:
            cc.compute_energy()
        except U.ConvergenceError:
            pass
    if a.triples:
        cc = U.CCWfn(H, {"R_CONVERGENCE": 1e-10, "PRECISION": "FP64" if a.ccsd_fp64 else prec, "PRINT": int(a.print),
                         "MIXED_SWITCH": a.switch})
        if a.guess:
            U.MLP(seed=1).guess(H)
        e_cc = cc.compute_energy()
        st_cc = H.ctx.stats()
        if a.ccsd_fp64:
            cc = U.CCWfn(H, {"R_CONVERGENCE": 1e-10, "PRECISION": prec})
        H.ctx.reset_stats()
        e_t = cc.triples()
        if a.tgrad:
            st_t = H.ctx.stats()
            H.ctx.reset_stats()
            cc.triples_gradient()
            print(json.dumps({"tgrad_ms": H.ctx.stats()["triples_ms"], "triples_ms": st_t["triples_ms"]}))
        print(json.dumps({"e_ccsd": e_cc, "e_t": e_t, "ccsd_ms": st_cc["ccsd_ms"],
                          "ccsd_iterations": st_cc["ccsd_iterations"], "fp64_iterations": st_cc["fp64_iterations"],
                          "mixed_iterations": st_cc["mixed_iterations"],
                          "anchored_iterations": st_cc["anchored_iterations"]}))
    if a.response:
        from ugacc_gb300.generator import RESPONSE_OMEGAS, make_perturbations
        cc = U.CCWfn(H, {"R_CONVERGENCE": 1e-10, "PRECISION": prec, "PRINT": int(a.print), "MIXED_SWITCH": a.switch})
        e_cc = cc.compute_energy()
        hb = U.HBAR(H, cc)
        lam = U.CCLambda(cc, hb)
        lam.compute_lambda()
        dens = U.CCDensity(cc, lam)
        e1, e2 = dens.onepdm(), dens.twopdm()
        perts = make_perturbations(h.nact, a.seed)
        alphas = {}
        for w in RESPONSE_OMEGAS:
            mu = [U.CCPert(perts[x], w, cc, hb, lam) for x in range(3)]
            for m in mu:
                m.solve("right")
            tens = []
            for p in range(3):
                row = []
                for q in range(3):
                    r = U.CCResp(mu[p], mu[q])
                    row.append(r.linresp(mu[p], mu[q]) if p == q else
                               0.5 * r.linresp(mu[p], mu[q]) + 0.5 * r.linresp(mu[q], mu[p]))
                tens.append(row)
            alphas[str(w)] = tens
        print(json.dumps({"e_ccsd": e_cc, "pseudoenergy": lam.pseudoenergy(), "e_onepdm": e1, "e_twopdm": e2,
                          "alpha": alphas}))
    print(json.dumps(H.ctx.stats()))
    return 0


if __name__ == "__main__":
    sys.exit(main())
