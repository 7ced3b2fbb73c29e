#!/usr/bin/env python
"""Benchmark: CCSD(T) on the no=16 / nv=160 synthetic RHF Hamiltonian (seed 1).

One step = one full CCSD(T) solve from the MP2 guess to ||R|| < 1e-10 followed by the
(T) correction, on Hamiltonian blocks already resident in HBM.  The default arm is the
mixed form (BF16 hi+lo split tensor-core contractions, FP64-accurate refinement sweeps,
tensor-core (T)); the plain FP64 form of the same step is timed alongside and the energy
differences between the two are reported.  value = algorithmic
TFLOP/s of the whole job (CCSD iterations x 2(no^2 nv^4 + 2 no^4 nv^2 + 10 no^3 nv^3 +
8 no^2 nv^3) + (T) 2 no(no+1)(no+2) nv^3 (nv+no)), device time from CUDA events on the
library's stream.  e2e repeats the step through the public API from pinned host
buffers: Hamiltonian upload (DF factors) + block build + CCSD(T) + energies back.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--precision mixed|fp64] [--no-fp64-reference] [--no-cpu-baseline]
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

# workloads: the default is the no=16 / nv=160 CCSD(T) case; "c3" (no=32 / nv=320, seed 2,
# Vvvvv 84 GB) is the large mixed-precision case, minutes per step, run on request
WORKLOADS = {"c2": (16, 160, 1), "c3": (32, 320, 2)}
NO, NV, SEED = WORKLOADS["c2"]
WORKLOAD = "ccsd_t_no16_nv160_seed1"
METRIC = "CCSD(T) TFLOP/s (algorithmic) at no=16/nv=160"


def select_workload(name):
    global NO, NV, SEED, WORKLOAD, METRIC
    NO, NV, SEED = WORKLOADS[name]
    WORKLOAD = "ccsd_t_no%d_nv%d_seed%d" % (NO, NV, SEED)
    METRIC = "CCSD(T) TFLOP/s (algorithmic) at no=%d/nv=%d" % (NO, NV)


# bf16 products per sliced FP64 GEMM (9 slices per operand, orders s + t < 9)
SLICE_PRODUCTS = 45


def flops_ccsd_iter(no, nv):
    return 2.0 * (no**2 * nv**4 + 2 * no**4 * nv**2 + 10 * no**3 * nv**3 + 8 * no**2 * nv**3)


def flops_triples(no, nv):
    return 2.0 * no * (no + 1) * (no + 2) * nv**3 * (nv + no)


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


def recorded_reference_run() -> dict:
    """The reference's own compiled loops on this workload, as recorded with the golden
    fixture (tests/golden/c2.json: one single-core x86 run); empty when absent."""
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tests", "golden", "c2.json")
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

    if args.workload != "c2":
        print(json.dumps({"impl": "reference", "unavailable": "the CPU path needs the full <pq|rs> array "
                          "(%.0f GB at no=%d/nv=%d), beyond host memory" % (8.0 * (NO + NV) ** 4 / 1e9, NO, NV)}))
        return
    h = make_hamiltonian(NO, NV, SEED)
    times = cpu_oracle_sample(h, args.warmup + args.steps)[args.warmup:]
    ms = 1e3 * sum(times) / len(times)
    v = flops_ccsd_iter(NO, NV) / (ms * 1e-3) / 1e12
    cores = os.cpu_count()
    line = {"metric": METRIC, "value": v, "unit": "TFLOP/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": WORKLOAD, "step": "one CCSD iteration (residual + Jacobi update)",
                       "l2": "inputs larger than L2", **recorded_reference_run()},
            "cpu_baseline": {"value": v, "unit": "TFLOP/s", "cores": cores, "kind": "port",
                             "sample": "numpy oracle: one CCSD iteration at no=%d/nv=%d per step" % (NO, NV)},
            "e2e": {"value": v, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64-reference", action="store_true")
    ap.add_argument("--workload", default="c2", choices=sorted(WORKLOADS))
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
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline and args.workload == "c2":
        t = cpu_oracle_sample(h, 1)
        cpu = {"value": flops_ccsd_iter(NO, NV) / t[0] / 1e12, "unit": "TFLOP/s", "cores": os.cpu_count(),
               "kind": "port", "sample": "numpy oracle (BLAS threads = host cores): one CCSD iteration at "
                                         "no=%d/nv=%d from the MP2 guess, %.1f s" % (NO, NV, t[0])}
    fp64_peak = fp64_gemm_peak_tflops()

    H = U.Hamiltonian.from_synthetic(h, device=local)
    # plain FP64 form of the same workload (the comparison the metric is quoted against)
    fp64 = None
    if args.precision == "mixed" and not args.no_fp64_reference:
        c64 = U.CCWfn(H, {"R_CONVERGENCE": 1e-10, "MAXITER": 100, "WFN": "CCSD_T", "PRECISION": "FP64"})
        c64.compute_energy()
        H.ctx.reset_stats()
        c64.compute_energy()
        s64 = H.ctx.stats()
        fp64 = {"ms_per_step": s64["ccsd_ms"] + s64["triples_ms"], "ccsd_ms": s64["ccsd_ms"],
                "triples_ms": s64["triples_ms"], "ccsd_iterations": s64["ccsd_iterations"],
                "e_ccsd": c64.eccsd, "e_t": c64.et}

    opts = {"R_CONVERGENCE": 1e-10, "MAXITER": 100, "WFN": "CCSD_T", "PRECISION": args.precision.upper()}
    cc = U.CCWfn(H, opts)
    for _ in range(args.warmup):
        cc.compute_energy()
    e_ref = (cc.eccsd, cc.et)

    barrier()
    H.ctx.reset_stats()
    clocks = ClockSampler(local)
    clocks.start()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        cc.compute_energy()
    barrier()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    st = H.ctx.stats()
    ms_dev = (st["ccsd_ms"] + st["triples_ms"]) / args.steps
    ms = allmax(ms_dev)
    iters = st["ccsd_iterations"]
    flops_step = flops_ccsd_iter(NO, NV) * iters + flops_triples(NO, NV)
    value = world * flops_step / (ms * 1e-3) / 1e12

    # the device-resident context is no longer needed: release its memory (the no=32/nv=320
    # blocks and their tensor-core copies would not fit twice)
    del cc
    H.ctx.close()
    # end to end through the public API from pinned host memory
    Bp = torch.from_numpy(np.ascontiguousarray(h.B)).pin_memory()
    Fp = torch.from_numpy(np.ascontiguousarray(h.fock)).pin_memory()
    ctx2 = U.Context(local)
    e2e_steps = max(1, min(args.steps, 2))
    barrier()
    t1 = time.perf_counter()
    for _ in range(e2e_steps):
        H2 = U.Hamiltonian(NO, NV, Fp.numpy(), B=Bp.numpy(), context=ctx2, precision=args.precision.upper())
        c2 = U.CCWfn(H2, opts)
        c2.compute_energy()
    barrier()
    e2e_ms = allmax(1e3 * (time.perf_counter() - t1) / e2e_steps)
    e2e_value = world * flops_step / (e2e_ms * 1e-3) / 1e12

    bf16 = measured_peak("bf16_tflops")
    step_ms_total = ms_dev * args.steps
    tc = f64g = None
    if st["tc_gemm_launches"]:
        ach = st["tc_gemm_flops"] / (st["tc_gemm_ms"] * 1e-3) / 1e12
        tc = {"bound": "tensor", "achieved": ach, "peak": bf16, "unit": "TFLOP/s",
              "frac": (ach / bf16) if bf16 else None, "traffic": None,
              "kernel": "tcgen05 BF16 hi+lo split GEMM (ucc::tc::gemm_kernel), all launches of the step",
              "flops": "algorithmic 2*M*N*K per launch over its CUDA-event time; the tensor pipe executes 3x "
                       "that (hi.hi + hi.lo + lo.hi)",
              "peak_source": "MEASURED_PEAKS.json bf16_tflops (burst), of measured",
              "share_of_step": st["tc_gemm_ms"] / step_ms_total,
              "launches": st["tc_gemm_launches"], "ms_per_launch": st["tc_gemm_ms"] / st["tc_gemm_launches"]}
    if st["fp64_gemm_launches"]:
        ach = st["fp64_gemm_flops"] / (st["fp64_gemm_ms"] * 1e-3) / 1e12
        f64g = {"bound": "tensor", "achieved": ach, "peak": fp64_peak, "unit": "TFLOP/s",
                "frac": (ach / fp64_peak) if fp64_peak else None, "traffic": None,
                "kernel": "FP64 DFMA GEMM (dgemm_kernel), all launches of the step (FP64 record sweeps of the "
                          "mixed solve, FP64 pieces)",
                "compute_unit": "FP64 pipe (compute bound, not the tensor cores)",
                "flops": "algorithmic 2*M*N*K per launch over its CUDA-event time",
                "peak_source": "cuBLAS DGEMM 8192^3 measured in this process on this GPU (FP64 has no entry in "
                               "MEASURED_PEAKS.json), of measured",
                "share_of_step": st["fp64_gemm_ms"] / step_ms_total,
                "launches": st["fp64_gemm_launches"],
                "ms_per_launch": st["fp64_gemm_ms"] / st["fp64_gemm_launches"]}
    sl = None
    if st["sliced_gemm_launches"]:
        fp64eq = st["sliced_gemm_flops"] / (st["sliced_gemm_ms"] * 1e-3) / 1e12
        ach = SLICE_PRODUCTS * fp64eq
        sl = {"bound": "tensor", "achieved": ach, "peak": bf16, "unit": "TFLOP/s",
              "frac": (ach / bf16) if bf16 else None, "traffic": None,
              "kernel": "tcgen05 sliced FP64 GEMM (ucc::tc::sliced_gemm_kernel): FP64-accurate products of 9 exact "
                        "bf16 slices per operand, all launches of the step (refinement sweeps of the mixed solve)",
              "flops": "tensor-pipe rate: 45 slice products x algorithmic 2*M*N*K per launch over its CUDA-event time "
                       "(slicing of non-cached operands included)",
              "fp64_equivalent_tflops": fp64eq,
              "fp64_equivalent_vs_dgemm_peak": (fp64eq / fp64_peak) if fp64_peak else None,
              "peak_source": "MEASURED_PEAKS.json bf16_tflops (burst), of measured",
              "share_of_step": st["sliced_gemm_ms"] / step_ms_total,
              "launches": st["sliced_gemm_launches"],
              "ms_per_launch": st["sliced_gemm_ms"] / st["sliced_gemm_launches"]}
    cands = [r for r in (f64g, tc, sl) if r]
    cands.sort(key=lambda r: -r["share_of_step"])
    roof = cands[0] if cands else None
    roof_other = cands[1] if len(cands) > 1 else None
    ladder = None
    if st["ladder_launches"]:
        ach = st["ladder_flops"] / (st["ladder_ms"] * 1e-3) / 1e12
        ladder = {"achieved": ach, "unit": "TFLOP/s", "ms_per_launch": st["ladder_ms"] / st["ladder_launches"],
                  "launches": st["ladder_launches"]}
    if rank == 0:
        cfg = {"workload": WORKLOAD, "no": NO, "nv": NV, "naux": h.naux, "seed": SEED,
               "precision": args.precision, "ccsd_iterations": iters,
               "mixed_iterations": st["mixed_iterations"] if args.precision == "mixed" else 0,
               "r_convergence": 1e-10, "e_ccsd": e_ref[0], "e_t": e_ref[1], "wall_s_per_step": wall / args.steps,
               "ccsd_ms_per_step": st["ccsd_ms"] / args.steps, "triples_ms_per_step": st["triples_ms"] / args.steps,
               "l2": "inputs larger than L2 (vvvv block %.1f GB)" % (8.0 * NV**4 / 1e9), "parallelism": f"replicas x{world}"}
        if fp64:
            cfg["fp64_gpu"] = fp64
            cfg["speedup_vs_fp64_gpu"] = fp64["ms_per_step"] / ms_dev
            cfg["abs_dE_ccsd_vs_fp64"] = abs(e_ref[0] - fp64["e_ccsd"])
            cfg["abs_dE_t_vs_fp64"] = abs(e_ref[1] - fp64["e_t"])
        if ladder:
            cfg["ladder"] = ladder
        line = {"metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None,
                "dtype": "f64" if args.precision == "fp64" else "bf16x3-split + bf16x45-sliced-f64, f32-acc, f64 epilogue",
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
