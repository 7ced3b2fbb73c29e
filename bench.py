#!/usr/bin/env python
"""Benchmark: mixed-precision + learned-guess CCSD(T) against the plain FP64 GPU form.

Default workload: the synthetic RHF Hamiltonian no=32 / nv=320 (naux = 1056, seed 2;
<ab|ef> alone is 84 GB in FP64).  One step = the learned T2 guess (one fused tensor-core
pass) + a full CCSD solve to ||R|| < 1e-10 (BF16 hi+lo split sweeps, FP64-accurate
refinement sweeps on the sliced tensor-core GEMM) + the (T) correction, on Hamiltonian
blocks already resident in HBM.  Reported beside it, in the same run:

* the plain FP64 GPU form of the same CCSD(T) (DFMA kernels), timed once, and the energy
  and amplitude differences |dE_CCSD|, |dE_(T)|, max|dT2| of the mixed result against it;
* the same mixed solve from the MP2 guess, so that the sweeps the learned guess saves are
  measured on the workload itself;
* the guess network's training cost (outside the timed region): it is trained on the GPU
  by the library's own kernels on converged amplitudes of other Hamiltonians of the same
  generator and shape (no=32 / nv=320, seeds 11 and 12), never on the benchmark
  Hamiltonian.

value = algorithmic TFLOP/s of the whole job: (CCSD iterations of the FP64 form, i.e. the
reference's own iteration count) x 2(no^2 nv^4 + 2 no^4 nv^2 + 10 no^3 nv^3 + 8 no^2 nv^3)
+ (T) 2 no(no+1)(no+2) nv^3 (nv+no), over the device time (CUDA events on the library's
stream) of guess + CCSD + (T).  e2e repeats the step through the public API from pinned
host buffers: DF factors upload, block build, guess, CCSD(T), energies back.

--workload c2 keeps the no=16 / nv=160 case (seed 1) whose reference arm times the numpy
oracle's CCSD iteration.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload c3|c2] [--precision mixed|fp64] [--no-fp64-reference]
                    [--no-cpu-baseline] [--no-guess]
Multi-GPU: replicas only (each rank solves its own copy; weak scaling).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# workloads (no, nv, seed); naux = 3 (no + nv)
WORKLOADS = {"c2": (16, 160, 1), "c3": (32, 320, 2)}
NO, NV, SEED = WORKLOADS["c3"]
WORKLOAD = "ccsd_t_no32_nv320_seed2"
METRIC = "CCSD(T) wall-s & TFLOP/s vs plain FP64 GPU at |dE|<=1 uEh; iterations saved"
# training Hamiltonians of the guess network: the same generator and shape as the workload,
# other seeds (about 6.5e6 sampled rows).  Trained on no=16/nv=160 instead, the network's
# prediction error on the no=32/nv=320 amplitudes was 0.44 of their size (0.15 when trained
# at that shape) and it saved one sweep at most.
GUESS_TRAIN = {"no": 32, "nv": 320, "seeds": [11, 12], "row_fraction": 0.03, "epochs": 4, "batch": 8192,
               "lr": 1e-3, "r_convergence": 1e-8}


def select_workload(name):
    global NO, NV, SEED, WORKLOAD, METRIC
    NO, NV, SEED = WORKLOADS[name]
    WORKLOAD = "ccsd_t_no%d_nv%d_seed%d" % (NO, NV, SEED)
    if name == "c2":
        METRIC = "CCSD(T) TFLOP/s (algorithmic) at no=16/nv=160"
        GUESS_TRAIN.update({"no": 16, "nv": 160, "seeds": [11, 12, 13, 14], "row_fraction": 0.25})


# DRAM bytes (read + write) per launch of the roofline kernels at no=32/nv=320, from one
# ncu launch list of the same solve (the no=32/nv=320 launch-list summary under profiles/):
# split GEMM 1331 launches, sliced GEMM 91, DFMA GEMM 69
TRAFFIC_C3 = {"split": 4.68e9, "sliced": 84.2e9, "dfma": 0.28e9}
TRAFFIC_SOURCE = ("ncu launch list of the same workload, DRAM read + write per launch averaged over the "
                  "solve (the no=32/nv=320 launch-list summary under profiles/)")


def traffic_of(kind, workload):
    return TRAFFIC_C3[kind] if workload == "c3" else None


def flops_ccsd_iter(no, nv):
    return 2.0 * (no**2 * nv**4 + 2 * no**4 * nv**2 + 10 * no**3 * nv**3 + 8 * no**2 * nv**3)


def flops_triples(no, nv):
    return 2.0 * no * (no + 1) * (no + 2) * nv**3 * (nv + no)


def flops_triples_tuple(no, nv):
    """One i >= j >= k term of (T): six e-sums and six m-sums of nv^3 elements each."""
    return 12.0 * nv**3 * (nv + no)


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.f = None

    def start(self):
        try:
            self.f = tempfile.NamedTemporaryFile(mode="w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.flush()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
            except (ValueError, IndexError):
                continue
            for k, nm in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak(key):
    try:
        return float(json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))[key])
    except Exception:
        return None


def fp64_gemm_peak_tflops():
    """cuBLAS DGEMM 8192^3 (best of 5, CUDA events): the measured FP64 denominator."""
    try:
        import torch

        a = torch.randn(8192, 8192, dtype=torch.float64, device="cuda")
        b = torch.randn(8192, 8192, dtype=torch.float64, device="cuda")
        torch.matmul(a, b)
        best = 1e9
        for _ in range(5):
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record()
            torch.matmul(a, b)
            e.record()
            torch.cuda.synchronize()
            best = min(best, s.elapsed_time(e))
        del a, b
        torch.cuda.empty_cache()
        return 2 * 8192.0**3 / (best * 1e-3) / 1e12
    except Exception:
        return None


# ------------------------------------------------------------------------------------
# CPU legs: the numpy oracle (test infrastructure) on a bounded sample of the workload
# ------------------------------------------------------------------------------------
def cpu_oracle_sample(h, iters: int = 1):
    """The oracle's CCSD iteration (numpy, all host threads) at the same workload."""
    from oracle import cc as O

    H = O.Hamiltonian(h)
    for blk in ["oooo", "ooov", "oovo", "oovv", "ovov", "ovvo", "ovoo", "ovvv", "vvvo", "vvvv"]:
        H.V(blk)
    for blk in ["oovv", "ooov", "oovo", "ovvv", "vovv", "ovvo"]:
        H.L(blk)
    cc = O.CCWfn(H)
    times = []
    for _ in range(iters):
        t0 = time.perf_counter()
        cc.iterate_once()
        times.append(time.perf_counter() - t0)
    return times


def cpu_triples_sample(h, ntuples: int):
    """The oracle's (T) term (W3 e/m-sums and the energy algebra of ccwfn.cc:795-852 and
    :1388-1418, numpy on all host threads) for the first `ntuples` occupied triples
    i >= j >= k, on MP2 amplitudes: a bounded sample of the workload's (T).  Returns the
    setup seconds and the per-tuple seconds."""
    from oracle import cc as O

    t0 = time.perf_counter()
    H = O.Hamiltonian(h)
    for blk in ["oovv", "ovvv", "ooov"]:
        H.V(blk)
    cc = O.CCWfn(H)
    setup = cc.tuple_setup()
    setup_s = time.perf_counter() - t0
    tuples = [(i, j, k) for i in range(h.no) for j in range(i + 1) for k in range(j + 1)][:ntuples]
    times = []
    for (i, j, k) in tuples:
        t1 = time.perf_counter()
        cc.tcorr_tuple(i, j, k, setup)
        times.append(time.perf_counter() - t1)
    return setup_s, times


def recorded_reference_run() -> dict:
    """The reference's own compiled loops on the no=16/nv=160 workload, as recorded with
    the golden fixture (tests/golden/c2.json: one single-core x86 run); empty otherwise."""
    path = os.path.join(ROOT, "tests", "golden", "c2.json")
    if WORKLOAD != "ccsd_t_no16_nv160_seed1" or not os.path.exists(path):
        return {}
    run = json.load(open(path))["runs"]["ccsd_t"]
    it = len(run["tables"]["ccsd"])  # iterations 0 (MP2) ... n-1 printed; the converging one is not
    return {"reference_binary_recorded": {
        "ccsd_s": run["ccsd_s"], "triples_s": run["t_tjl_s"], "ccsd_iterations": it, "cores": 1,
        "e_ccsd": run["e_ccsd"], "e_t": run["e_t_tjl"],
        "source": "tests/golden/c2.json (the reference sources compiled by oracle/Makefile, one x86 core)"}}


def run_reference(args, rank):
    if rank != 0:
        return
    from ugacc_gb300.generator import make_hamiltonian

    h = make_hamiltonian(NO, NV, SEED)
    cores = os.cpu_count()
    if args.workload == "c2":
        times = cpu_oracle_sample(h, args.warmup + args.steps)[args.warmup:]
        step = "one CCSD iteration (residual + Jacobi update)"
        flops = flops_ccsd_iter(NO, NV)
        sample = "numpy oracle: one CCSD iteration at no=%d/nv=%d per step" % (NO, NV)
        extra = recorded_reference_run()
    else:
        # the CCSD iteration needs <ab|ef> (84 GB) and hours per sweep on the host; the (T)
        # tuples need 9 GB: one tuple term per step
        setup_s, times = cpu_triples_sample(h, args.warmup + args.steps)
        times = times[args.warmup:]
        step = "one (T) tuple term i >= j >= k (W3 e/m-sums + energy algebra) on MP2 amplitudes"
        flops = flops_triples_tuple(NO, NV)
        sample = ("numpy oracle: (T) tuple terms at no=%d/nv=%d, one per step (%.3g FLOP each), blocks built from "
                  "the DF factors in %.1f s" % (NO, NV, flops, setup_s))
        extra = {}
    ms = 1e3 * sum(times) / len(times)
    v = flops / (ms * 1e-3) / 1e12
    line = {"metric": METRIC, "value": v, "unit": "TFLOP/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": WORKLOAD, "step": step, "l2": "inputs larger than L2", **extra},
            "cpu_baseline": {"value": v, "unit": "TFLOP/s", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------------------------
# GPU arm
# ------------------------------------------------------------------------------------
def train_guess_network(U, make_hamiltonian, device):
    """Guess network trained on the GPU (the library's own forward/backward kernels) on
    converged amplitudes of the training Hamiltonians; returns the network and its cost."""
    import numpy as np

    g = GUESS_TRAIN
    rng = np.random.default_rng(0)
    t0 = time.perf_counter()
    Xs, ts = [], []
    for s in g["seeds"]:
        h = make_hamiltonian(g["no"], g["nv"], s)
        H = U.Hamiltonian.from_synthetic(h, device=device, precision="MIXED")
        U.CCWfn(H, {"R_CONVERGENCE": g["r_convergence"], "PRECISION": "MIXED"}).compute_energy()
        X, t = U.mlp_features(H, with_targets=True)
        keep = rng.random(X.shape[0]) < g["row_fraction"]
        Xs.append(X[keep])
        ts.append(t[keep])
        H.ctx.close()
    X = np.concatenate(Xs)
    t = np.concatenate(ts)
    data_s = time.perf_counter() - t0
    net = U.MLP(device=device, seed=1)
    t1 = time.perf_counter()
    loss0 = float(net.loss_grad(X[:200000], t[:200000])[0])
    loss = float(net.train(X, t, epochs=g["epochs"], batch=g["batch"], lr=g["lr"], seed=1))
    train_s = time.perf_counter() - t1
    info = {"hamiltonians": "no=%d/nv=%d, seeds %s, the same generator" % (g["no"], g["nv"], g["seeds"]),
            "rows": int(X.shape[0]), "epochs": g["epochs"], "loss_before": loss0, "loss_after": loss,
            "data_s": data_s, "train_s": train_s,
            "note": "outside the timed region; the benchmark Hamiltonian is not in the training set"}
    return net, info


def sweeps_of(st):
    return {"total": st["ccsd_iterations"], "split": st["mixed_iterations"], "record": st["fp64_iterations"],
            "delta": st["anchored_iterations"]}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64-reference", action="store_true")
    ap.add_argument("--no-guess", action="store_true", help="start every solve from the MP2 guess")
    ap.add_argument("--workload", default="c3", choices=sorted(WORKLOADS))
    args = ap.parse_args()
    select_workload(args.workload)
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank)
        return

    import numpy as np
    import torch
    import torch.distributed as dist

    import ugacc_gb300 as U
    from ugacc_gb300.generator import make_hamiltonian

    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()

    from ugacc_gb300.replicas import allmax as _allmax

    def allmax(x):
        return _allmax(x, dist if world > 1 else None, device="cuda")

    h = make_hamiltonian(NO, NV, SEED)
    mixed = args.precision == "mixed"
    use_guess = mixed and not args.no_guess
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        if args.workload == "c2":
            t = cpu_oracle_sample(h, 1)
            cpu = {"value": flops_ccsd_iter(NO, NV) / t[0] / 1e12, "unit": "TFLOP/s", "cores": os.cpu_count(),
                   "kind": "port", "sample": "numpy oracle (BLAS threads = host cores): one CCSD iteration at "
                                             "no=%d/nv=%d from the MP2 guess, %.1f s" % (NO, NV, t[0])}
        else:
            setup_s, t = cpu_triples_sample(h, 2)
            per = sum(t) / len(t)
            cpu = {"value": flops_triples_tuple(NO, NV) / per / 1e12, "unit": "TFLOP/s", "cores": os.cpu_count(),
                   "kind": "port", "sample": "numpy oracle (BLAS threads = host cores): 2 (T) tuple terms at "
                                             "no=%d/nv=%d on MP2 amplitudes, %.1f s each (+%.1f s block build)"
                                             % (NO, NV, per, setup_s)}
    fp64_peak = fp64_gemm_peak_tflops()
    net, guess_info = (train_guess_network(U, make_hamiltonian, local) if use_guess else (None, None))

    H = U.Hamiltonian.from_synthetic(h, device=local, precision="MIXED" if mixed else "FP64")
    opts = {"R_CONVERGENCE": 1e-10, "MAXITER": 100, "WFN": "CCSD_T", "PRECISION": args.precision.upper()}
    cc = U.CCWfn(H, opts)

    def step():
        if use_guess:
            net.guess(H)
        cc.compute_energy()

    for _ in range(args.warmup):
        step()
    # the same solve from the MP2 guess: the sweeps the learned guess saves
    mp2_start = None
    if use_guess:
        H.ctx.reset_stats()
        cc.compute_energy()
        st0 = H.ctx.stats()
        mp2_start = {"sweeps": sweeps_of(st0), "ccsd_ms": st0["ccsd_ms"]}

    barrier()
    H.ctx.reset_stats()
    clocks = ClockSampler(local)
    clocks.start()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    barrier()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    st = H.ctx.stats()
    e_ref = (cc.eccsd, cc.et)
    ms_dev = (st["ccsd_ms"] + st["triples_ms"] + st["guess_ms"]) / args.steps
    ms = allmax(ms_dev)
    sweeps = sweeps_of(st)  # the library keeps the sweep counts of the last solve
    t2_mixed = cc.t2 if not args.no_fp64_reference and mixed else None

    # the device-resident context is released before the end-to-end leg (the no=32/nv=320
    # blocks and their tensor-core copies would not fit twice)
    del cc
    H.ctx.close()
    Bp = torch.from_numpy(np.ascontiguousarray(h.B)).pin_memory()
    Fp = torch.from_numpy(np.ascontiguousarray(h.fock)).pin_memory()
    ctx2 = U.Context(local)
    e2e_steps = max(1, min(args.steps, 2))
    barrier()
    t1 = time.perf_counter()
    for _ in range(e2e_steps):
        H2 = U.Hamiltonian(NO, NV, Fp.numpy(), B=Bp.numpy(), context=ctx2, precision=args.precision.upper())
        if use_guess:
            net.guess(H2)
        c2 = U.CCWfn(H2, opts)
        c2.compute_energy()
    barrier()
    e2e_ms = allmax(1e3 * (time.perf_counter() - t1) / e2e_steps)
    del c2, H2
    ctx2.close()

    # the plain FP64 form of the same CCSD(T), once (the comparison the metric is quoted against)
    fp64 = None
    if mixed and not args.no_fp64_reference:
        ctx64 = U.Context(local)
        H64 = U.Hamiltonian.from_synthetic(h, context=ctx64, precision="FP64")
        c64 = U.CCWfn(H64, dict(opts, PRECISION="FP64"))
        ctx64.reset_stats()
        c64.compute_energy()
        s64 = ctx64.stats()
        t2_64 = c64.t2
        fp64 = {"ms_per_step": s64["ccsd_ms"] + s64["triples_ms"], "ccsd_ms": s64["ccsd_ms"],
                "triples_ms": s64["triples_ms"], "ccsd_iterations": s64["ccsd_iterations"],
                "e_ccsd": c64.eccsd, "e_t": c64.et, "runs": 1, "warmup": 0}
        dt2 = float(np.abs(t2_mixed - t2_64).max())
        del c64, H64, t2_64
        ctx64.close()
    # FLOPs per step on the FP64 form's (the reference's) iteration count
    it_flops = fp64["ccsd_iterations"] if fp64 else sweeps["total"]
    flops_step = flops_ccsd_iter(NO, NV) * it_flops + flops_triples(NO, NV)
    value = world * flops_step / (ms * 1e-3) / 1e12
    e2e_value = world * flops_step / (e2e_ms * 1e-3) / 1e12

    bf16 = measured_peak("bf16_tflops")
    bf16s = measured_peak("bf16_tflops_sustained")
    step_ms_total = ms_dev * args.steps
    tc = f64g = sl = None
    if st["tc_gemm_launches"]:
        ach = st["tc_gemm_flops"] / (st["tc_gemm_ms"] * 1e-3) / 1e12
        tc = {"bound": "tensor", "achieved": ach, "peak": bf16s, "unit": "TFLOP/s",
              "frac": (ach / bf16s) if bf16s else None, "traffic": traffic_of("split", args.workload),
              "traffic_unit": "bytes per launch", "traffic_source": TRAFFIC_SOURCE,
              "kernel": "tcgen05 BF16 hi+lo split GEMM (ucc::tc::gemm_kernel), all launches of the step",
              "flops": "algorithmic 2*M*N*K per launch over its CUDA-event time; the tensor pipe executes 3x "
                       "that (hi.hi + hi.lo + lo.hi)",
              "tensor_pipe_frac": (3 * ach / bf16s) if bf16s else None,
              "frac_of_burst": (ach / bf16) if bf16 else None,
              "peak_source": "MEASURED_PEAKS.json bf16_tflops_sustained (kernel timed inside a seconds-long step), "
                             "of measured",
              "share_of_step": st["tc_gemm_ms"] / step_ms_total,
              "launches": st["tc_gemm_launches"], "ms_per_launch": st["tc_gemm_ms"] / st["tc_gemm_launches"]}
    if st["fp64_gemm_launches"]:
        ach = st["fp64_gemm_flops"] / (st["fp64_gemm_ms"] * 1e-3) / 1e12
        f64g = {"bound": "tensor", "achieved": ach, "peak": fp64_peak, "unit": "TFLOP/s",
                "frac": (ach / fp64_peak) if fp64_peak else None, "traffic": traffic_of("dfma", args.workload),
                "traffic_unit": "bytes per launch", "traffic_source": TRAFFIC_SOURCE,
                "kernel": "FP64 DFMA GEMM (dgemm_kernel), all launches of the step (contractions below the tensor-"
                          "core thresholds)",
                "compute_unit": "FP64 pipe (compute bound, not the tensor cores)",
                "flops": "algorithmic 2*M*N*K per launch over its CUDA-event time",
                "peak_source": "cuBLAS DGEMM 8192^3 measured in this process on this GPU (FP64 has no entry in "
                               "MEASURED_PEAKS.json), of measured",
                "share_of_step": st["fp64_gemm_ms"] / step_ms_total,
                "launches": st["fp64_gemm_launches"],
                "ms_per_launch": st["fp64_gemm_ms"] / st["fp64_gemm_launches"]}
    if st["sliced_gemm_launches"]:
        fp64eq = st["sliced_gemm_flops"] / (st["sliced_gemm_ms"] * 1e-3) / 1e12
        ach = st["sliced_gemm_product_flops"] / (st["sliced_gemm_ms"] * 1e-3) / 1e12
        sl = {"bound": "tensor", "achieved": ach, "peak": bf16s, "unit": "TFLOP/s",
              "frac": (ach / bf16s) if bf16s else None, "traffic": traffic_of("sliced", args.workload),
              "traffic_unit": "bytes per launch", "traffic_source": TRAFFIC_SOURCE,
              "kernel": "tcgen05 sliced FP64 GEMM (ucc::tc::sliced_gemm_kernel): products of exact bf16 slices "
                        "per operand (9 for FP64 accuracy; fewer for anchors whose deltas resolve a residual well "
                        "above r_convergence), all launches of the step (record sweeps of the mixed solve)",
              "flops": "tensor-pipe rate: slice products (S(S+1)/2 for S digits: 45 at 9) x algorithmic 2*M*N*K "
                       "per launch over its CUDA-event time (slicing of non-cached operands included)",
              "slice_products_per_output": st["sliced_gemm_product_flops"] / st["sliced_gemm_flops"],
              "fp64_equivalent_tflops": fp64eq,
              "fp64_equivalent_vs_dgemm_peak": (fp64eq / fp64_peak) if fp64_peak else None,
              "frac_of_burst": (ach / bf16) if bf16 else None,
              "peak_source": "MEASURED_PEAKS.json bf16_tflops_sustained, of measured",
              "share_of_step": st["sliced_gemm_ms"] / step_ms_total,
              "launches": st["sliced_gemm_launches"],
              "ms_per_launch": st["sliced_gemm_ms"] / st["sliced_gemm_launches"]}
    cands = [r for r in (f64g, tc, sl) if r]
    cands.sort(key=lambda r: -r["share_of_step"])
    roof = cands[0] if cands else None
    roof_other = cands[1] if len(cands) > 1 else None
    if rank == 0:
        cfg = {"workload": WORKLOAD, "no": NO, "nv": NV, "naux": h.naux, "seed": SEED,
               "precision": args.precision, "learned_guess": use_guess, "sweeps_per_step": sweeps,
               "r_convergence": 1e-10, "e_ccsd": e_ref[0], "e_t": e_ref[1], "wall_s_per_step": wall / args.steps,
               "guess_ms_per_step": st["guess_ms"] / args.steps,
               "ccsd_ms_per_step": st["ccsd_ms"] / args.steps, "triples_ms_per_step": st["triples_ms"] / args.steps,
               "flop_iterations": it_flops,
               "flop_iterations_source": "the FP64 form's CCSD iteration count (the reference's)" if fp64
               else "this solve's sweeps (no FP64 run)",
               "l2": "inputs larger than L2 (vvvv block %.1f GB)" % (8.0 * NV**4 / 1e9),
               "parallelism": f"replicas x{world}"}
        if use_guess:
            cfg["guess_training"] = guess_info
            cfg["mp2_guess_solve"] = mp2_start
            cfg["iterations_saved"] = mp2_start["sweeps"]["total"] - sweeps["total"]
            cfg["ccsd_ms_saved_net_of_guess"] = mp2_start["ccsd_ms"] - (st["ccsd_ms"] + st["guess_ms"]) / args.steps
        if fp64:
            cfg["fp64_gpu"] = fp64
            cfg["speedup_vs_fp64_gpu"] = fp64["ms_per_step"] / ms_dev
            cfg["abs_dE_ccsd_vs_fp64"] = abs(e_ref[0] - fp64["e_ccsd"])
            cfg["abs_dE_t_vs_fp64"] = abs(e_ref[1] - fp64["e_t"])
            cfg["abs_dE_total_vs_fp64"] = abs(e_ref[0] + e_ref[1] - fp64["e_ccsd"] - fp64["e_t"])
            cfg["max_abs_dT2_vs_fp64"] = dt2
            cfg["within_1_uEh"] = cfg["abs_dE_total_vs_fp64"] <= 1e-6
        line = {"metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None,
                "dtype": "f64" if not mixed else "bf16x3-split + bf16-sliced-f64 (up to 45 products) + f16 guess net, f32-acc, f64 epilogue",
                "data": "synthetic", "config": cfg,
                "e2e": {"value": e2e_value, "unit": "TFLOP/s", "ms_per_step": e2e_ms,
                        "h2d_bytes_per_step": int(Bp.numel() * 8 + Fp.numel() * 8), "d2h_bytes_per_step": 16},
                "gpu_launches": int(st["kernel_launches"]),
                "roofline": roof, "roofline_secondary": roof_other, "roofline_others": cands[2:],
                "cpu_baseline": cpu, "clocks": clk}
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
