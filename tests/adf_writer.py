"""A minimal ADF container writer for the CGNS reader's tests: builds node
trees with the layout phase_gb300.cgns reads (node headers, sub-node tables,
single data chunks, little-endian values).  Test infrastructure only."""
from __future__ import annotations

import numpy as np

BLOCK = 4096


def _addr(pos: int) -> bytes:
    return b"%08X%04X" % (pos // BLOCK, pos % BLOCK)


class Node:
    def __init__(self, name, label, dtype="MT", data=None, dims=None,
                 children=()):
        self.name, self.label, self.dtype = name, label, dtype
        self.data, self.dims, self.children = data, dims, list(children)


def _payload(n: Node):
    if n.dtype == "MT":
        return b"", []
    if n.dtype == "C1":
        b = n.data.encode("ascii")
        return b, [len(b)]
    a = np.asarray(n.data, {"I4": "<i4", "I8": "<i8", "R8": "<f8",
                            "R4": "<f4"}[n.dtype])
    dims = n.dims or (list(a.shape) if a.ndim else [1])
    return np.asfortranarray(a).T.tobytes(order="C") if a.ndim > 1 else \
        a.tobytes(), dims


def write(root_children) -> bytes:
    """An ADF file whose root node has the given children."""
    root = Node("ADF MotherNode", "Root Node of ADF File",
                children=root_children)
    out = bytearray()
    header = (b"\x00\x00\x00\x00ADF Database Version A02011>AdF0" +
              b" " * 28 + b"AdF1" + b" " * 28 + b"AdF2LBAdF4")
    root_at = 256
    out += header + _addr(root_at)
    out += b" " * (root_at - len(out))
    # lay every node out: header, then its data chunk, then its table
    pending = [root]
    pos_of = {}
    order = []
    while pending:
        n = pending.pop(0)
        order.append(n)
        pending.extend(n.children)
    # first pass: sizes
    sizes = {}
    for n in order:
        pay, _ = _payload(n)
        size = 246 + (16 + len(pay) + 4 if n.dtype != "MT" else 0) + \
            (16 + 44 * len(n.children) if n.children else 0)
        sizes[id(n)] = size
    p = root_at
    for n in order:
        pos_of[id(n)] = p
        p += sizes[id(n)]
    for n in order:
        at = pos_of[id(n)]
        pay, dims = _payload(n)
        data_at = at + 246
        table_at = data_at + (16 + len(pay) + 4 if n.dtype != "MT" else 0)
        h = bytearray(b"NoDe")
        h += n.name.encode().ljust(32) + n.label.encode().ljust(32)
        h += b"%08X%08X" % (len(n.children), len(n.children))
        h += _addr(table_at) if n.children else _addr(BLOCK)
        h += n.dtype.encode().ljust(32)
        h += b"%02X" % len(dims)
        h += b"".join(b"%08X" % d for d in dims).ljust(96, b"0")
        h += b"%04X" % (1 if n.dtype != "MT" else 0)
        h += _addr(data_at) if n.dtype != "MT" else _addr(BLOCK)
        h += b"TaiL"
        assert len(h) == 246
        body = bytes(h)
        if n.dtype != "MT":
            body += b"DaTa" + _addr(data_at + 16 + len(pay)) + pay + b"dEnD"
        if n.children:
            body += b"SNTb" + _addr(table_at + 16 + 44 * len(n.children))
            for c in n.children:
                body += c.name.encode().ljust(32) + _addr(pos_of[id(c)])
        assert len(body) == sizes[id(n)]
        out += body
    return bytes(out)
