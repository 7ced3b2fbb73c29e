"""Loading helpers for the golden fixtures produced by tests/golden/make_golden.py."""
from __future__ import annotations

import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def cases():
    return sorted(f[:-5] for f in os.listdir(GOLDEN) if f.endswith(".json"))


def load(name: str):
    meta = json.load(open(os.path.join(GOLDEN, name + ".json")))
    npz = os.path.join(GOLDEN, name + ".npz")
    arrays = dict(np.load(npz)) if os.path.exists(npz) else {}
    return meta, arrays


def hamiltonian(meta):
    from ugacc_gb300.generator import make_hamiltonian, make_perturbations

    h = make_hamiltonian(meta["no"], meta["nv"], meta["seed"])
    assert h.checksum() == meta["checksum"], "generator stream changed: fixtures no longer apply"
    return h, make_perturbations(h.nact, meta["seed"])
