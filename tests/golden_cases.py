"""The golden fixtures under tests/golden (written by
tests/golden/make_golden.py from the reference's own CrsEquation): seeded
small meshes, fv::laplacian inputs, and the reference's slot arrays."""
from __future__ import annotations

import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = sorted(f[:-4] for f in os.listdir(GOLDEN) if f.endswith(".npz"))


def load(name):
    """(fixture arrays, gamma (float or per-face array), u or None)."""
    z = np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False)
    gamma = float(z["gamma"]) if bool(z["gamma_is_scalar"]) else z["gamma"]
    u = z["u"] if z["u"].size else None
    return z, gamma, u


def compact(z):
    """A fixture's reference slot arrays without the -1 placeholders."""
    rp, ci = z["row_ptr"], z["col_ind"]
    keep = ci >= 0
    counts = np.add.reduceat(keep.astype(np.int64), rp[:-1])
    rpc = np.concatenate([[0], np.cumsum(counts)]).astype(rp.dtype)
    return rpc, ci[keep], z["vals"][keep], z["rhs"]
