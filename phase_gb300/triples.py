"""On-disk form of solver triples (A_t, b_t, x_t) of a time sequence: the
training data of the learned initial guess, written by a solver loop and
read back by training, so dumps can be made once (or by another program)
and reused.

A dump is a directory:

    meta.json     {"format": "phase-gb300-triples", "version": 1, "n": N,
                   "nnz": NNZ, "steps": [t0, t1, ...], ...user fields}
    row_ptr.npy   int32[N + 1]   the CSR pattern, shared by every step
    col_ind.npy   int32[NNZ]     (columns in CrsEquation order; no -1 slots)
    step_<t>.npz  vals float64[NNZ], b float64[N], x float64[N]

b is the right-hand side the solver receives (-rhs_ of the CrsEquation)
and x its solution at step t, so A_t x_t ~= b_t.  Files are plain numpy
formats (little-endian, no pickles).
"""
from __future__ import annotations

import json
import os

import numpy as np

FORMAT = "phase-gb300-triples"
VERSION = 1


class TripleWriter:
    """Writes the pattern once, then one file per step."""

    def __init__(self, path: str, row_ptr, col_ind, **meta):
        self.path = path
        os.makedirs(path, exist_ok=True)
        self.row_ptr = np.ascontiguousarray(row_ptr, np.int32)
        self.col_ind = np.ascontiguousarray(col_ind, np.int32)
        if self.row_ptr.ndim != 1 or self.row_ptr[-1] != self.col_ind.size:
            raise ValueError("row_ptr and col_ind do not form a CSR pattern")
        if (self.col_ind < 0).any():
            raise ValueError("col_ind holds placeholder (-1) slots")
        self.n = self.row_ptr.size - 1
        self.meta = dict(meta)
        self.steps = []
        np.save(os.path.join(path, "row_ptr.npy"), self.row_ptr, allow_pickle=False)
        np.save(os.path.join(path, "col_ind.npy"), self.col_ind, allow_pickle=False)
        self._write_meta()

    def _write_meta(self):
        meta = dict(self.meta, format=FORMAT, version=VERSION, n=int(self.n),
                    nnz=int(self.col_ind.size), steps=list(self.steps))
        tmp = os.path.join(self.path, "meta.json.tmp")
        with open(tmp, "w") as f:
            json.dump(meta, f, indent=1)
        os.replace(tmp, os.path.join(self.path, "meta.json"))

    def write(self, t: int, vals, b, x):
        vals = np.ascontiguousarray(vals, np.float64)
        b = np.ascontiguousarray(b, np.float64)
        x = np.ascontiguousarray(x, np.float64)
        if vals.size != self.col_ind.size or b.size != self.n or x.size != self.n:
            raise ValueError("step arrays do not match the pattern")
        np.savez(os.path.join(self.path, f"step_{int(t)}.npz"), vals=vals, b=b, x=x)
        if int(t) not in self.steps:
            self.steps.append(int(t))
        self._write_meta()


class TripleReader:
    """Reads a dump written by TripleWriter."""

    def __init__(self, path: str):
        self.path = path
        with open(os.path.join(path, "meta.json")) as f:
            self.meta = json.load(f)
        if self.meta.get("format") != FORMAT or self.meta.get("version") != VERSION:
            raise ValueError(f"{path}: not a {FORMAT} v{VERSION} dump")
        self.row_ptr = np.load(os.path.join(path, "row_ptr.npy"), allow_pickle=False)
        self.col_ind = np.load(os.path.join(path, "col_ind.npy"), allow_pickle=False)
        self.n = int(self.meta["n"])
        self.steps = [int(t) for t in self.meta["steps"]]
        if self.row_ptr.size != self.n + 1 or self.col_ind.size != self.meta["nnz"]:
            raise ValueError(f"{path}: pattern does not match meta.json")

    def read(self, t: int):
        """(vals, b, x) of step t."""
        with np.load(os.path.join(self.path, f"step_{int(t)}.npz"),
                     allow_pickle=False) as z:
            return z["vals"], z["b"], z["x"]

    def __iter__(self):
        for t in self.steps:
            yield (t,) + self.read(t)
