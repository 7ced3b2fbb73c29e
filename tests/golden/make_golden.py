"""Regenerates the golden fixtures in this directory from the reference's own code.

It writes each case's synthetic Hamiltonian (ugacc_gb300/generator.py), runs the
reference's hot-path sources compiled by ``make -C oracle`` (oracle/_ref/ugacc_ref),
and stores what that binary printed and dumped:

  <case>.json   energies, iteration counts, per-iteration CCSD/Lambda energies parsed
                from the reference's own iteration tables, timings, input checksum
  <case>.npz    selected tensors (float64), small cases only

Needs the reference tree (``--reference`` or the UGACC_REFERENCE environment variable)
and g++; not run by the tests.
    python tests/golden/make_golden.py --reference /path/to/ugacc [--big] [--only CASE ...]
"""
from __future__ import annotations

import argparse
import json
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from ugacc_gb300.generator import make_hamiltonian, make_perturbations, write_input_file  # noqa: E402

# name: (no, nv, seed, runs); each run = (tag, options, tensors-to-keep)
ALL_T = ["t1", "t2"]
HBAR_T = ["Hov", "Hoo", "Hvv", "Hoooo", "Hvvvv", "Hvovv", "Hooov", "Hovvo", "Hovov", "Hvvvo", "Hovoo"]
LAM_T = ["l1", "l2", "Doo", "Dvv", "Dov", "Dvo"]
G2_T = ["Goooo", "Gvvvv", "Gooov", "Gvvvo", "Govov", "Goovv"]  # the two-particle density blocks
CASES = {
    # H2O/cc-pVDZ shape (no=5, nv=19), seed 0: CCSD, all three (T) forms, Lambda,
    # densities, static right-hand and dynamic left-hand response
    "c1": (5, 19, 0, [
        ("right_w0", dict(DERTYPE="SECOND", TRIPLES="all", MYHAND="RIGHT", MY_OMEGA="0.0"), ALL_T + LAM_T + G2_T),
        ("left_w", dict(DERTYPE="SECOND", MYHAND="LEFT", MY_OMEGA="0.0656"), []),
        ("right_w", dict(DERTYPE="SECOND", MYHAND="RIGHT", MY_OMEGA="0.0656"), []),
    ]),
    # odd tiny sizes: every intermediate dumped (tile-edge coverage)
    "tiny": (3, 7, 11, [
        ("right_w0", dict(DERTYPE="SECOND", TRIPLES="all", MYHAND="RIGHT", MY_OMEGA="0.0"),
         ALL_T + HBAR_T + LAM_T + G2_T + ["X1_MuX", "X2_MuX", "Y1_MuX", "Y2_MuX", "X1_LZ", "X2_LZ"]),
        ("left_w", dict(DERTYPE="SECOND", MYHAND="LEFT", MY_OMEGA="0.0656"),
         ["X1_MuY", "X2_MuY", "Y1_MuY", "Y2_MuY", "Y1_LX", "Y2_LX"]),
    ]),
    # single occupied orbital (degenerate i=j=k triples weight)
    "one_occ": (1, 6, 4, [("ccsd_t", dict(DERTYPE="FIRST", TRIPLES="all"), ALL_T + ["l1", "l2"] + G2_T)]),
    # prime sizes
    "prime": (7, 13, 7, [("ccsd_t", dict(DERTYPE="FIRST", TRIPLES="all"), ALL_T)]),
    # more virtuals than a 32-wide tile
    "mid": (6, 40, 5, [("ccsd_t", dict(DERTYPE="NONE", TRIPLES="all"), ["t1"])]),
    # CCSD(T) first derivatives: the (T) gradient pieces (s1, s2, (T) densities), the
    # Lambda equations with s1/s2 and the densities that start from the (T) pieces
    # (OOC=1: tcorr_ooc + tgrad_ooc; OOC=0, the plugin's default: tcorr + tgrad over stored T3/L3)
    "tgrad": (4, 11, 9, [("ccsd_t_first", dict(WFN="CCSD_T", DERTYPE="FIRST"),
                          ["t1", "t2", "s1", "s2", "DooT", "DvvT", "DovT", "GoovvT", "GooovT", "GvvvoT",
                           "l1", "l2", "Doo", "Dvv", "Dov"] + G2_T),
                         ("ccsd_t_first_incore", dict(WFN="CCSD_T", DERTYPE="FIRST", OOC="0"),
                          ["s1", "s2", "DooT", "DvvT", "DovT", "GoovvT", "GooovT", "GvvvoT",
                           "l1", "l2", "Doo", "Dvv", "Dov"])]),
}
BIG = {
    # the plain FP64 CCSD(T) workload itself (no=16, nv=160, seed 1); hours on one core
    "c2": (16, 160, 1, [("ccsd_t", dict(DERTYPE="NONE", TRIPLES="tjl"), ["t1"])]),
}


def parse_twopdm(log: str):
    """The component energies of the two-particle density as the reference prints them
    (ccdensity.cc:181-335, %20.14f): OOOO, VVVV, OOOV, VVVO, OVOV, OOVV."""
    out = {}
    for m in re.finditer(r"^\t(OOOO|VVVV|OOOV|VVVO|OVOV|OOVV) Energy = \s*(-?\d+\.\d+)\s*$", log, flags=re.M):
        out[m.group(1)] = float(m.group(2))
    return out


def parse_tables(log: str):
    """Per-iteration energies from the reference's own tables (ccwfn.cc:224, cclambda.cc:125)."""
    out = {"ccsd": [], "lambda": [], "pert": []}
    section = None
    for line in log.splitlines():
        if "The Coupled-Cluster Iteration" in line:
            section = "ccsd"
        elif "Coupled-Cluster Lambda Iteration" in line:
            section = "lambda"
        elif "Perturbed Wfn Iteration" in line:
            section = "pert"
            out["pert"].append([])
        m = re.match(r"^\t\s+(\d+)\s+(-?\d+\.\d+)(\s+\S+)*\s*$", line)
        if m and section:
            it, val = int(m.group(1)), float(m.group(2))
            if section == "pert":
                out["pert"][-1].append([it, val])
            else:
                out[section].append([it, val])
    return out


def run_case(name, spec, binary, reference):
    no, nv, seed, runs = spec
    h = make_hamiltonian(no, nv, seed)
    perts = make_perturbations(h.nact, seed)
    with tempfile.TemporaryDirectory(dir=os.path.join(ROOT, "_work") if os.path.isdir(os.path.join(ROOT, "_work")) else None) as tmp:
        inp = os.path.join(tmp, "in.bin")
        write_input_file(inp, h, perts)
        meta = {"no": no, "nv": nv, "seed": seed, "naux": h.naux, "checksum": h.checksum(),
                "generator": "ugacc_gb300.generator.make_hamiltonian / make_perturbations",
                "binary": "oracle/_ref/ugacc_ref (reference sources compiled by oracle/Makefile)", "runs": {}}
        arrays = {}
        for tag, opts, keep in runs:
            outdir = os.path.join(tmp, tag)
            args = [binary, inp, outdir, "R_CONVERGENCE=1e-10", "MAXITER=100"] + [f"{k}={v}" for k, v in opts.items()]
            if keep:
                args.append("DUMP=1")
            subprocess.run(args, check=True)
            res = json.load(open(os.path.join(outdir, "result.json")))
            log = open(os.path.join(outdir, "log.txt")).read()
            tens = res.pop("tensors")
            res["options"] = dict(opts, R_CONVERGENCE="1e-10", MAXITER="100")
            res["tables"] = parse_tables(log)
            e2 = parse_twopdm(log)
            if e2:
                res["e_twopdm_parts"] = e2
            meta["runs"][tag] = res
            for k in keep:
                arrays[f"{tag}/{k}"] = np.fromfile(os.path.join(outdir, k + ".bin")).reshape(tens[k])
        with open(os.path.join(HERE, f"{name}.json"), "w") as f:
            json.dump(meta, f, indent=1, sort_keys=True)
        if arrays:
            np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **arrays)
    print(f"{name}: done", flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--big", action="store_true", help="also the no=16/nv=160 case (hours)")
    ap.add_argument("--only", nargs="*")
    ap.add_argument("--reference", default=os.environ.get("UGACC_REFERENCE"),
                    help="the reference tree (default: $UGACC_REFERENCE)")
    ap.add_argument("--build-dir", default="_ref", help="build directory under oracle/")
    a = ap.parse_args()
    if not a.reference:
        ap.error("the reference tree is needed: --reference PATH or UGACC_REFERENCE=PATH")
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), f"REFERENCE={a.reference}", f"OUT={a.build_dir}"],
                   check=True)
    binary = os.path.join(ROOT, "oracle", a.build_dir, "ugacc_ref")
    cases = dict(CASES)
    if a.big:
        cases.update(BIG)
    for name, spec in cases.items():
        if a.only and name not in a.only:
            continue
        run_case(name, spec, binary, a.reference)


if __name__ == "__main__":
    main()
