"""Phase case files: the INFO format that Phase reads with
boost::property_tree::read_info (src/System/Input.cpp:8-15: case.info,
boundaries.info, initialConditions.info, postProcessing.info), and the two
parts of it that configure the pressure path here:

* ``LinearAlgebra.<equation>`` -> keyword arguments of SparseMatrixSolver
  (the keys of the ``lib gb300`` plugin, and the Trilinos keys of the
  reference's own backend mapped onto them);
* ``Boundaries.<field>`` -> boundary type and value per patch (``*`` is the
  default patch), as FiniteVolumeField reads them.

The INFO subset parsed: ``key value`` lines, ``key`` or ``key value``
followed by a ``{ ... }`` block (the brace on the same or the next line),
``;`` comments, double-quoted strings with backslash escapes, repeated keys
(kept in order).  ``#include`` is not supported (Phase's cases do not use
it).
"""
from __future__ import annotations

import re
from dataclasses import dataclass, field
from typing import Iterator


@dataclass
class Node:
    """A property-tree node: its value and its ordered children."""
    value: str = ""
    children: list = field(default_factory=list)  # [(key, Node)]

    def child(self, key: str) -> "Node | None":
        for k, n in self.children:
            if k == key:
                return n
        return None

    def get(self, path: str, default=None):
        """Value at a dotted path, or default."""
        node = self
        for part in path.split("."):
            node = node.child(part)
            if node is None:
                return default
        return node.value

    def keys(self):
        return [k for k, _ in self.children]


_TOKEN = re.compile(r'"((?:[^"\\]|\\.)*)"|([{}])|([^\s{};"]+)')


def _tokens(text: str) -> Iterator[tuple]:
    """(kind, text, line) tokens: 'str' (bare or quoted), '{', '}', 'nl'."""
    for ln, line in enumerate(text.splitlines(), 1):
        pos = 0
        while pos < len(line):
            c = line[pos]
            if c in " \t\r":
                pos += 1
                continue
            if c == ";":
                break
            m = _TOKEN.match(line, pos)
            if not m:
                raise ValueError(f"INFO line {ln}: cannot read {line[pos:]!r}")
            if m.group(1) is not None:
                yield ("str", bytes(m.group(1), "utf-8").decode("unicode_escape"), ln)
            elif m.group(2) is not None:
                yield (m.group(2), m.group(2), ln)
            else:
                yield ("str", m.group(3), ln)
            pos = m.end()
        yield ("nl", "", ln)


def parse_info(text: str) -> Node:
    """Parse INFO text into a Node tree."""
    root = Node()
    stack = [root]
    last: Node | None = None  # the node a following '{' opens
    line_toks: list = []

    def flush():
        nonlocal last
        if not line_toks:
            return
        key = line_toks[0]
        value = " ".join(line_toks[1:2]) if len(line_toks) > 1 else ""
        if len(line_toks) > 2:
            raise ValueError(f"INFO: more than one value for {key!r}")
        n = Node(value=value)
        stack[-1].children.append((key, n))
        last = n
        line_toks.clear()

    for kind, tok, ln in _tokens(text):
        if kind == "str":
            line_toks.append(tok)
        elif kind == "{":
            flush()
            if last is None:
                raise ValueError(f"INFO line {ln}: '{{' without a key")
            stack.append(last)
            last = None
        elif kind == "}":
            flush()
            if len(stack) == 1:
                raise ValueError(f"INFO line {ln}: unmatched '}}'")
            stack.pop()
            last = None
        else:  # end of line: a finished key/value pair, its block may follow
            flush()
    if len(stack) != 1:
        raise ValueError("INFO: unclosed '{'")
    return root


def read_info(path: str) -> Node:
    with open(path) as f:
        return parse_info(f.read())


# --------------------------------------------------------------- solver
_KRYLOV = {"BICGSTAB": 0, "TFQMR": 1, "GMRES": 2}


def solver_options(tree: Node, equation: str = "pEqn") -> dict:
    """Keyword arguments for SparseMatrixSolver from
    ``LinearAlgebra.<equation>``, read as the Belos backend reads them
    (src/Math/TrilinosBelosSparseMatrixSolver.cpp:44-86): tolerance,
    maxIters, solver (BICGSTAB | TFQMR | GMRES), innerPreconditioner
    (RILUK, or RELAXATION / DIAGONAL: point Jacobi), iluFill (the RILUK
    level of fill), schwarzIters (1), schwarzCombineMode (ADD),
    schwarzOverlap (0).  ``preconditioner`` is ignored as the reference
    ignores it without an ifpackParamFile (always Schwarz), except this
    library's own values none and jacobi.  Own keys: numBlocks (GMRES
    restart length), subdomainRows, coarseSpace, coarseWarmIters, precision
    (fp64 | mixed), mixedSweep.  Absent keys keep the solver's defaults; a
    value the library does not build raises ValueError (no silent
    substitution)."""
    sec = tree.child("LinearAlgebra")
    sec = sec.child(equation) if sec is not None else None
    if sec is None:
        raise KeyError(f"LinearAlgebra.{equation} not in the case")
    out = {}
    if sec.get("tolerance") is not None:
        out["tolerance"] = float(sec.get("tolerance"))
    if sec.get("maxIters") is not None:
        out["max_iters"] = int(sec.get("maxIters"))
    for key in ("belosParamFile", "ifpackParamFile"):
        if (sec.get(key) or "").strip():
            raise ValueError(f"{key}: Teuchos XML parameter lists are not "
                             "read; give the keys directly")
    solver = (sec.get("solver") or "BICGSTAB").strip().upper()
    if solver not in _KRYLOV:
        raise ValueError(f"solver {solver!r} is not built "
                         f"({', '.join(_KRYLOV)} are)")
    out["krylov"] = _KRYLOV[solver]
    if sec.get("numBlocks") is not None:
        out["krylov_dim"] = int(sec.get("numBlocks"))
    pre = (sec.get("preconditioner") or "schwarz").strip().lower()
    inner = (sec.get("innerPreconditioner") or "RILUK").strip().upper()
    if pre == "none":
        out["precond"] = 0
    elif pre == "jacobi" or inner in ("RELAXATION", "DIAGONAL"):
        out["precond"] = 1  # Schwarz over point-Jacobi blocks = point Jacobi
    elif inner == "RILUK":
        out["precond"] = 2
    else:
        raise ValueError(f"innerPreconditioner {inner!r} is not built "
                         "(RILUK with iluFill, RELAXATION, DIAGONAL are)")
    if sec.get("iluFill") is not None:
        fill = float(sec.get("iluFill"))
        if fill < 0 or fill != int(fill):
            raise ValueError("iluFill must be a non-negative whole level")
        out["ilu_fill"] = int(fill)
    if int(sec.get("schwarzIters") or 1) != 1:
        raise ValueError("schwarzIters other than 1 is not built")
    if (sec.get("schwarzCombineMode") or "ADD").strip().upper() != "ADD":
        raise ValueError("schwarzCombineMode other than ADD is not built")
    if int(sec.get("schwarzOverlap") or 0) != 0:
        raise ValueError("schwarzOverlap other than 0 is not built")
    if sec.get("subdomainRows") is not None:
        out["subdomain_rows"] = int(sec.get("subdomainRows"))
    if sec.get("coarseSpace") is not None:
        out["coarse"] = int(sec.get("coarseSpace"))
    if sec.get("coarseWarmIters") is not None:
        out["coarse_warm"] = int(sec.get("coarseWarmIters"))
    if sec.get("precision") is not None:
        p = sec.get("precision").strip().lower()
        if p not in ("fp64", "mixed"):
            raise ValueError(f"unknown precision {p!r}")
        out["precision"] = 1 if p == "mixed" else 0
    if sec.get("mixedSweep") is not None:
        out["mixed_sweep"] = int(sec.get("mixedSweep"))
    return out


# ----------------------------------------------------------- boundaries
BC_TYPES = {"fixed": 0, "normal_gradient": 1, "symmetry": 2}


def boundary_conditions(tree: Node, fld: str, patches) -> dict:
    """{patch: (type code, value string)} of field ``fld`` for the given patch
    names, from ``Boundaries.<fld>``: a patch's own block, else ``*``."""
    sec = tree.child("Boundaries")
    sec = sec.child(fld) if sec is not None else None
    if sec is None:
        raise KeyError(f"Boundaries.{fld} not in the case")
    out = {}
    for p in patches:
        node = sec.child(p) or sec.child("*")
        if node is None:
            raise KeyError(f"no boundary condition for {fld} on patch {p!r}")
        t = (node.get("type") or "").strip().lower()
        if t not in BC_TYPES:
            raise ValueError(f"unknown boundary type {t!r} for {fld} on {p!r}")
        out[p] = (BC_TYPES[t], node.get("value", ""))
    return out


# patch names of StructuredRectilinearGrid (meshes.rect_patch_of_faces ids)
RECT_PATCHES = ("x-", "x+", "y-", "y+")


def rect_face_bcs(tree: Node, fld: str, patch_of_face):
    """Per-face (bc_type, bc_value) arrays of a scalar field on a rectilinear
    box, patch ids as meshes.rect_patch_of_faces (-1 interior: type 1, 0)."""
    import numpy as np
    bcs = boundary_conditions(tree, fld, RECT_PATCHES)
    bc_type = np.ones(patch_of_face.shape, np.int32)
    bc_value = np.zeros(patch_of_face.shape)
    for pid, name in enumerate(RECT_PATCHES):
        t, v = bcs[name]
        sel = patch_of_face == pid
        bc_type[sel] = t
        bc_value[sel] = float(v) if v else 0.0
    return bc_type, bc_value


# -------------------------------------------------------------- backend
_DIRECT = ("eigen", "eigen3", "amesos", "amesos2")
_ITERATIVE = ("belos", "gb300")


def backend(tree: Node, equation: str = "pEqn") -> str:
    """Which library backend ``LinearAlgebra.<equation>.lib`` selects, read
    as FiniteVolumeEquation::configureSparseSolver does (lower-cased, no
    default; FiniteVolumeEquation.tpp:48-62) and mapped onto this library
    as SparseMatrixSolverFactory::create maps the names
    (SparseMatrixSolverFactory.cpp:26-40): "direct" for eigen / eigen3
    (SparseLU) and amesos / amesos2 (a direct Trilinos solver) -- the
    pg_lu backend --, "iterative" for belos and gb300 -- pg_solver.  muelu
    (algebraic multigrid) is not built and raises ValueError, as an unknown
    name raises in the factory."""
    sec = tree.child("LinearAlgebra")
    sec = sec.child(equation) if sec is not None else None
    if sec is None or sec.get("lib") is None:
        raise KeyError(f"LinearAlgebra.{equation}.lib not in the case")
    lib = sec.get("lib").strip().lower()
    if lib in _DIRECT:
        return "direct"
    if lib in _ITERATIVE:
        return "iterative"
    if lib == "muelu":
        raise ValueError("lib muelu (algebraic multigrid) is not built")
    raise ValueError(f'bad solver type "{lib}"')


# ----------------------------------------------------------------- grid
def _point(text: str):
    v = text.strip().strip("()").split(",")
    return float(v[0]), float(v[1])


def grid(tree: Node, case_root: str):
    """The grid of a case whose ``Grid.type`` is cgns
    (CgnsUnstructuredGrid(Input), CgnsUnstructuredGrid.cpp:7-11:
    ``Grid.filename`` relative to the directory the case runs in, optional
    ``Grid.origin``), read by phase_gb300.cgns.read_mesh."""
    from . import cgns
    import os
    sec = tree.child("Grid")
    if sec is None:
        raise KeyError("Grid not in the case")
    kind = (sec.get("type") or "").strip().lower()
    if kind != "cgns":
        raise ValueError(f"grid type {kind!r}: only cgns files are read here "
                         "(meshes.rectilinear builds rectilinear grids)")
    origin = _point(sec.get("origin", "(0,0)"))
    return cgns.read_mesh(os.path.join(case_root, sec.get("filename")),
                          origin=origin)


def face_bcs(tree: Node, fld: str, patch_of_face, names):
    """Per-face (bc_type, bc_value) arrays of a scalar field for patches
    ``names`` (patch_of_face: index into names, -1 interior: type 1, 0)."""
    import numpy as np
    bcs = boundary_conditions(tree, fld, names)
    bc_type = np.ones(np.shape(patch_of_face), np.int32)
    bc_value = np.zeros(np.shape(patch_of_face))
    for pid, name in enumerate(names):
        t, v = bcs[name]
        sel = np.asarray(patch_of_face) == pid
        bc_type[sel] = t
        bc_value[sel] = float(v) if v else 0.0
    return bc_type, bc_value
