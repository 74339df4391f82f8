"""phase_gb300 -- GB300 pressure assembly + BiCGStab/ILU(0) for Phase.

Python host binding over the C ABI of libphase_gb300.so
(include/phase_gb300.h).  Names mirror the reference interfaces the library
replaces: ``SparseMatrixSolver`` (src/Math/SparseMatrixSolver.h:11-62) with
setRank/set/setRhs/setGuess/solve/x/nIters/error, and the device
``FiniteVolumeEquation`` assembled by ``fv.laplacian(...) == src.div(u)``.

There is no CPU path: every call runs the CUDA library, and loading fails
loudly when the library has not been built or no GPU is present.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libphase_gb300.so")

PG_OK, PG_MAX_ITERS, PG_BREAKDOWN, PG_NON_FINITE, PG_BAD_ARG, PG_TIMEOUT, \
    PG_CUDA_ERROR = range(7)
PG_HOST, PG_DEVICE = 0, 1
FIXED, NORMAL_GRADIENT, SYMMETRY = 0, 1, 2
GAMMA_SCALAR, GAMMA_FACE = 0, 1
PREC_NONE, PREC_JACOBI, PREC_ILU0 = 0, 1, 2
FP64, MIXED = 0, 1
KRYLOV_BICGSTAB, KRYLOV_TFQMR, KRYLOV_GMRES = 0, 1, 2

STATUS_NAMES = {0: "converged", 1: "max_iters", 2: "breakdown",
                3: "non_finite", 4: "bad_arg", 5: "timeout", 6: "cuda_error"}


class PhaseError(RuntimeError):
    """A library call failed (bad argument or CUDA error)."""

    def __init__(self, status: int, message: str):
        super().__init__(f"[{STATUS_NAMES.get(status, status)}] {message}")
        self.status = status


class SolverCfg(ctypes.Structure):
    _fields_ = [("tolerance", ctypes.c_double), ("max_iters", ctypes.c_int),
                ("precond", ctypes.c_int), ("subdomain_rows", ctypes.c_int),
                ("precision", ctypes.c_int), ("mixed_sweep", ctypes.c_int),
                ("coarse", ctypes.c_int), ("coarse_warm", ctypes.c_int),
                ("krylov", ctypes.c_int), ("ilu_fill", ctypes.c_int),
                ("krylov_dim", ctypes.c_int), ("reserved_i", ctypes.c_int),
                ("reserved_d", ctypes.c_double)]


class LuStats(ctypes.Structure):
    _fields_ = [("n_fronts", ctypes.c_int), ("n_heights", ctypes.c_int),
                ("max_front", ctypes.c_int), ("replaced_pivots", ctypes.c_int),
                ("factor_entries", ctypes.c_int64), ("flops", ctypes.c_double),
                ("analyse_ms", ctypes.c_double), ("factor_ms", ctypes.c_double),
                ("solve_ms", ctypes.c_double),
                ("rel_residual", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class SolveStats(ctypes.Structure):
    _fields_ = [("iters", ctypes.c_int), ("outer_iters", ctypes.c_int),
                ("status", ctypes.c_int), ("fp64_iters", ctypes.c_int),
                ("rel_residual", ctypes.c_double),
                ("ms", ctypes.c_double), ("setup_ms", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_D = ctypes.c_double
_I = ctypes.c_int

# name -> (restype, argtypes); every entry point of include/phase_gb300.h
PROTOTYPES = {
    "pg_last_error": (ctypes.c_char_p, []),
    "pg_stream": (_P, []),
    "pg_synchronize": (_I, []),
    "pg_mesh_create": (_I, [_P, _I64, _P, _P, _I64, ctypes.POINTER(_P)]),
    "pg_mesh_destroy": (_I, [_P]),
    "pg_mesh_sizes": (_I, [_P, _P, _P, _P, _P]),
    "pg_mesh_faces": (_I, [_P, _P, _P, _P, _P, _P, _P]),
    "pg_mesh_cells": (_I, [_P, _P, _P, _P]),
    "pg_eqn_create": (_I, [_P, _I, _P, ctypes.POINTER(_P)]),
    "pg_correct_velocity": (_I, [_P, _D, _P, _P, _P, _P, _P, _P, _I]),
    "pg_set_boundary_faces": (_I, [_P, _P, _P, _P, _I]),
    "pg_eqn_create_gcib": (_I, [_P, _I, _P, _I, _P, _I, _D, ctypes.POINTER(_P)]),
    "pg_eqn_cell_class": (_I, [_P, _P]),
    "pg_eqn_update_gcib": (_I, [_P, _I, _P, _D, _P]),
    "pg_eqn_create_momentum": (_I, [_P, _P, ctypes.POINTER(_P)]),
    "pg_assemble_momentum": (_I, [_P, _D, _D, _D, _P, _P, _I]),
    "pg_interpolate_faces": (_I, [_P, _P, _P, _I]),
    "pg_eqn_destroy": (_I, [_P]),
    "pg_eqn_sizes": (_I, [_P, _P, _P]),
    "pg_assemble_laplacian": (_I, [_P, _P, _D, _P, _P, _I]),
    "pg_eqn_export": (_I, [_P, _P, _P, _P, _P]),
    "pg_eqn_device_values": (_I, [_P, ctypes.POINTER(_P), ctypes.POINTER(_P)]),
    "pg_face_dt_over_rho": (_I, [_P, _P, _D, _D, _D, _P, _I]),
    "pg_gradient": (_I, [_P, _P, _P, _P, _P, _I]),
    "pg_gradient_noalloc": (_I, [_P, _P, _P, _P]),
    "pg_solver_sweep_form": (_I, [_P]),
    "pg_solver_set_eqn_component": (_I, [_P, _P, _I]),
    "pg_eqn_diagonal": (_I, [_P, _P, _I]),
    "pg_solver_default_cfg": (None, [ctypes.POINTER(SolverCfg)]),
    "pg_solver_create": (_I, [ctypes.POINTER(SolverCfg), ctypes.POINTER(_P)]),
    "pg_solver_destroy": (_I, [_P]),
    "pg_solver_set_rank": (_I, [_P, _I64]),
    "pg_solver_set_csr": (_I, [_P, _P, _P, _P, _I]),
    "pg_solver_set_eqn": (_I, [_P, _P]),
    "pg_solver_set_rhs": (_I, [_P, _P, _I]),
    "pg_solver_set_guess": (_I, [_P, _P, _I]),
    "pg_solver_solve": (_I, [_P, ctypes.POINTER(SolveStats)]),
    "pg_solver_get_x": (_I, [_P, _P, _I]),
    "pg_solver_partition": (_I, [_P, _P, ctypes.POINTER(_I)]),
    "pg_solver_coarse_inverse": (_I, [_P, _P, ctypes.POINTER(_I)]),
    "pg_solver_set_row_coords": (_I, [_P, _P]),
    "pg_solver_profile": (_I, [_P, _I, _P]),
    "pg_solver_trace_kernels": (_I, [_P, _I]),
    "pg_solver_kernel_times": (_I, [_P, _P, _P, _P]),
    "pg_solver_apply_precond": (_I, [_P, _P, _P, _I]),
    "pg_batch_create": (_I, [_P, ctypes.POINTER(_P)]),
    "pg_batch_destroy": (_I, [_P]),
    "pg_batch_set_eqns": (_I, [_P, _I, _P]),
    "pg_batch_solve": (_I, [_P, _P, ctypes.POINTER(_D)]),
    "pg_batch_get_x": (_I, [_P, _I, _P, _I]),
    "pg_batch_tuning": (_I, [_P, ctypes.POINTER(_I), ctypes.POINTER(_I),
                             ctypes.POINTER(_I)]),
    "pg_mpnn_create": (_I, [ctypes.c_uint64, ctypes.POINTER(_P)]),
    "pg_mpnn_destroy": (_I, [_P]),
    "pg_mpnn_num_params": (_I, [_P]),
    "pg_mpnn_set_graph": (_I, [_P, _P, _P, _I64]),
    "pg_mpnn_predict": (_I, [_P, _P, _P, _P, _P, _P, _I]),
    "pg_mpnn_train_step": (_I, [_P, _P, _P, _P, _P, ctypes.c_float, _I, _P]),
    "pg_mpnn_gradient": (_I, [_P, _P, _P, _P, _P, _I, _P, _P]),
    "pg_mpnn_get_params": (_I, [_P, _P]),
    "pg_mpnn_set_params": (_I, [_P, _P]),
    "pg_mpnn_save": (_I, [_P, ctypes.c_char_p]),
    "pg_mpnn_load": (_I, [_P, ctypes.c_char_p]),
    "pg_lu_create": (_I, [ctypes.POINTER(_P)]),
    "pg_lu_destroy": (_I, [_P]),
    "pg_lu_set_rank": (_I, [_P, _I64]),
    "pg_lu_set_row_coords": (_I, [_P, _P]),
    "pg_lu_set_csr": (_I, [_P, _P, _P, _P, _I]),
    "pg_lu_set_eqn": (_I, [_P, _P]),
    "pg_lu_set_rhs": (_I, [_P, _P, _I]),
    "pg_lu_solve": (_I, [_P, ctypes.POINTER(LuStats)]),
    "pg_lu_get_x": (_I, [_P, _P, _I]),
    "pg_lu_analyse_pattern": (_I, [_I64, _P, _P, _P, _I, _P, _P, _P, _P]),
    "pg_kernel_launches": (ctypes.c_uint64, []),
}

_lib = None


def lib() -> ctypes.CDLL:
    """Load libphase_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with "
                "`python -c 'import __graft_entry__ as g; g.build()'`")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in PROTOTYPES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _check(rc: int, allow=(PG_OK,)):
    if rc not in allow:
        raise PhaseError(rc, lib().pg_last_error().decode())
    return rc


def _ptr(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


def _f64(a, n=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if n is not None and a.size != n:
        raise ValueError(f"expected {n} values, got {a.size}")
    return a


def _i32(a, n=None):
    a = np.ascontiguousarray(a, dtype=np.int32)
    if n is not None and a.size != n:
        raise ValueError(f"expected {n} values, got {a.size}")
    return a


def stream_handle() -> int:
    """cudaStream_t of the library (for torch.cuda.ExternalStream)."""
    return int(lib().pg_stream() or 0)


def kernel_launches() -> int:
    """Kernels launched by the library since it was loaded."""
    return int(lib().pg_kernel_launches())


def synchronize():
    _check(lib().pg_synchronize())


class Mesh:
    """FiniteVolumeGrid2D built on the device from (nodes, cptr, cind)."""

    def __init__(self, nodes_xy, cptr, cind):
        nodes_xy = _f64(nodes_xy)
        cptr = np.ascontiguousarray(cptr, dtype=np.int64)
        cind = np.ascontiguousarray(cind, dtype=np.int64)
        h = _P()
        _check(lib().pg_mesh_create(_ptr(nodes_xy), nodes_xy.size // 2,
                                    _ptr(cptr), _ptr(cind), cptr.size - 1,
                                    ctypes.byref(h)))
        self._h = h
        s = np.zeros(4, np.int64)
        _check(lib().pg_mesh_sizes(h, _ptr(s[0:1]), _ptr(s[1:2]), _ptr(s[2:3]),
                                   _ptr(s[3:4])))
        self.n_cells, self.n_faces, self.n_interior, self.n_boundary = map(int, s)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.pg_mesh_destroy(h)
            self._h = None

    def faces(self):
        nf = self.n_faces
        out = dict(lcell=np.empty(nf, np.int32), rcell=np.empty(nf, np.int32),
                   fx=np.empty(nf), fy=np.empty(nf), nx=np.empty(nf),
                   ny=np.empty(nf))
        _check(lib().pg_mesh_faces(self._h, *(_ptr(out[k]) for k in
                                              ("lcell", "rcell", "fx", "fy",
                                               "nx", "ny"))))
        return out

    def cells(self):
        n = self.n_cells
        out = dict(cx=np.empty(n), cy=np.empty(n), vol=np.empty(n))
        _check(lib().pg_mesh_cells(self._h, _ptr(out["cx"]), _ptr(out["cy"]),
                                   _ptr(out["vol"])))
        return out

    def interpolate_faces(self, cell_vals):
        c = _f64(cell_vals, self.n_cells)
        out = np.empty(self.n_faces)
        _check(lib().pg_interpolate_faces(self._h, _ptr(c), _ptr(out), PG_HOST))
        return out

    def interpolate_faces_device(self, cell_ptr: int, face_ptr: int):
        """interpolate_faces() from and to device memory."""
        _check(lib().pg_interpolate_faces(self._h, _P(cell_ptr), _P(face_ptr),
                                          PG_DEVICE))

    def dt_over_rho(self, gamma_cell, rho1, rho2, dt):
        g = _f64(gamma_cell, self.n_cells)
        out = np.empty(self.n_faces)
        _check(lib().pg_face_dt_over_rho(self._h, _ptr(g), rho1, rho2, dt,
                                         _ptr(out), PG_HOST))
        return out

    def dt_over_rho_device(self, gamma_cell_ptr: int, out_ptr: int, rho1,
                           rho2, dt):
        """dt_over_rho on device arrays (addresses as ints)."""
        _check(lib().pg_face_dt_over_rho(self._h, _P(gamma_cell_ptr), rho1,
                                         rho2, dt, _P(out_ptr), PG_DEVICE))

    def gradient(self, phi_cell, phi_face):
        pc = _f64(phi_cell, self.n_cells)
        pf = _f64(phi_face, self.n_faces)
        gf = np.empty(2 * self.n_faces)
        gc = np.empty(2 * self.n_cells)
        _check(lib().pg_gradient(self._h, _ptr(pc), _ptr(pf), _ptr(gf),
                                 _ptr(gc), PG_HOST))
        return gf.reshape(-1, 2), gc.reshape(-1, 2)

    def set_boundary_faces(self, bc_type, phi_cell, phi_face):
        """FiniteVolumeField::setBoundaryFaces: returns phi_face with the
        normal-gradient/symmetry boundary faces set to their cell values."""
        bc = _i32(bc_type, self.n_faces)
        pc = _f64(phi_cell, self.n_cells)
        pf = np.array(phi_face, np.float64).reshape(-1)
        _check(lib().pg_set_boundary_faces(self._h, _ptr(bc), _ptr(pc),
                                           _ptr(pf), PG_HOST))
        return pf

    def correct_velocity(self, dt, grad_cell, grad_face, u_cell, u_face,
                         rho_cell=None, rho_face=None):
        """FractionalStep::correctVelocity: returns (u_cell, u_face) after
        u -= dt / rho * grad p (rho = 1 when not given)."""
        uc = np.array(u_cell, np.float64).reshape(-1)
        uf = np.array(u_face, np.float64).reshape(-1)
        rc = None if rho_cell is None else _f64(rho_cell, self.n_cells)
        rf = None if rho_face is None else _f64(rho_face, self.n_faces)
        _check(lib().pg_correct_velocity(
            self._h, float(dt), _ptr(rc), _ptr(rf),
            _ptr(_f64(np.asarray(grad_cell).reshape(-1), 2 * self.n_cells)),
            _ptr(_f64(np.asarray(grad_face).reshape(-1), 2 * self.n_faces)),
            _ptr(uc), _ptr(uf), PG_HOST))
        return uc.reshape(-1, 2), uf.reshape(-1, 2)


class Equation:
    """Device FiniteVolumeEquation<Scalar> for one fv::laplacian overload."""

    def __init__(self, mesh: Mesh, gamma_kind: int, bc_type, ib_circles=None,
                 ib_bc=NORMAL_GRADIENT, ib_ref=0.0):
        """ib_circles [(cx, cy, r), ...] makes the ghost-cell immersed-boundary
        pressure equation (fv::laplacian + ib.bcs) of FractionalStepGCIB."""
        self.mesh = mesh
        bc = _i32(bc_type, mesh.n_faces)
        h = _P()
        if ib_circles is None:
            _check(lib().pg_eqn_create(mesh._h, gamma_kind, _ptr(bc),
                                       ctypes.byref(h)))
        else:
            c = np.ascontiguousarray(np.asarray(ib_circles, np.float64).reshape(-1, 3))
            _check(lib().pg_eqn_create_gcib(mesh._h, gamma_kind, _ptr(bc),
                                            len(c), _ptr(c), int(ib_bc),
                                            float(ib_ref), ctypes.byref(h)))
        self._h = h
        self.gamma_kind = gamma_kind
        s = np.zeros(2, np.int64)
        _check(lib().pg_eqn_sizes(h, _ptr(s[0:1]), _ptr(s[1:2])))
        self.n, self.nnz = int(s[0]), int(s[1])

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.pg_eqn_destroy(h)
            self._h = None

    def assemble(self, gamma_face=None, gamma_scalar=0.0, bc_value=None,
                 u_face=None):
        nf = self.mesh.n_faces
        g = None if gamma_face is None else _f64(gamma_face, nf)
        bv = None if bc_value is None else _f64(bc_value, nf)
        u = None if u_face is None else _f64(u_face, 2 * nf)
        _check(lib().pg_assemble_laplacian(self._h, _ptr(g), gamma_scalar,
                                           _ptr(bv), _ptr(u), PG_HOST))
        return self

    def assemble_device(self, gamma_face: int = 0, gamma_scalar=0.0,
                        bc_value: int = 0, u_face: int = 0):
        """assemble() with device pointers (0 = absent)."""
        _check(lib().pg_assemble_laplacian(
            self._h, _P(gamma_face or None), gamma_scalar,
            _P(bc_value or None), _P(u_face or None), PG_DEVICE))
        return self

    def move_ib(self, circles, ib_ref=0.0) -> bool:
        """GhostCellImmersedBoundary::updateCells after the bodies moved to
        ``circles`` [(cx, cy, r), ...]: classes and stencils rebuilt on the
        device.  Returns True when the pattern changed (the equation was
        rebuilt; a solver given it re-analyses), False when the new IB rows
        were written in place.  assemble() afterwards."""
        c = np.ascontiguousarray(np.asarray(circles, np.float64).reshape(-1, 3))
        flag = np.zeros(1, np.int32)
        _check(lib().pg_eqn_update_gcib(self._h, len(c), _ptr(c), float(ib_ref),
                                        _ptr(flag)))
        s = np.zeros(2, np.int64)
        _check(lib().pg_eqn_sizes(self._h, _ptr(s[0:1]), _ptr(s[1:2])))
        self.n, self.nnz = int(s[0]), int(s[1])
        return bool(flag[0])

    def cell_class(self):
        """0 fluid, 1 IB, 2 solid per cell (all 0 without an IB)."""
        out = np.empty(self.n, np.int32)
        _check(lib().pg_eqn_cell_class(self._h, _ptr(out)))
        return out

    def device_values(self):
        """(vals, rhs) device addresses of the assembled equation."""
        v, r = _P(), _P()
        _check(lib().pg_eqn_device_values(self._h, ctypes.byref(v),
                                          ctypes.byref(r)))
        return v.value, r.value

    def export(self):
        rp = np.empty(self.n + 1, np.int32)
        ci = np.empty(self.nnz, np.int32)
        v = np.empty(self.nnz)
        rhs = np.empty(self.n)
        _check(lib().pg_eqn_export(self._h, _ptr(rp), _ptr(ci), _ptr(v),
                                   _ptr(rhs)))
        # a ghost-cell IB equation leaves out exact zeros (row_ptr[n] entries)
        return rp, ci[:rp[-1]].copy(), v[:rp[-1]].copy(), rhs


def _eqn_diagonal(eqn, out_ptr=None):
    """a_P per row: a host array, or written to device memory at out_ptr."""
    if out_ptr is not None:
        _check(lib().pg_eqn_diagonal(eqn._h, _P(out_ptr), PG_DEVICE))
        return None
    d = np.empty(eqn.n)
    _check(lib().pg_eqn_diagonal(eqn._h, _ptr(d), PG_HOST))
    return d


Equation.diagonal = _eqn_diagonal


class MomentumEquation:
    """Device momentum operator ddt + div - laplacian(nu) of the vector
    equation: one N x N matrix shared by both components, rhs[2N]."""

    def __init__(self, mesh: Mesh, bc_type):
        self.mesh = mesh
        bc = _i32(bc_type, mesh.n_faces)
        h = _P()
        _check(lib().pg_eqn_create_momentum(mesh._h, _ptr(bc), ctypes.byref(h)))
        self._h = h
        s = np.zeros(2, np.int64)
        _check(lib().pg_eqn_sizes(h, _ptr(s[0:1]), _ptr(s[1:2])))
        self.n, self.nnz = int(s[0]), int(s[1])

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.pg_eqn_destroy(h)
            self._h = None

    def assemble(self, dt, nu, theta, u_old_cell, u_face):
        u0 = _f64(u_old_cell, 2 * self.mesh.n_cells)
        uf = _f64(u_face, 2 * self.mesh.n_faces)
        _check(lib().pg_assemble_momentum(self._h, dt, nu, theta, _ptr(u0),
                                          _ptr(uf), PG_HOST))
        return self

    def assemble_device(self, dt, nu, theta, u_old_ptr: int, u_face_ptr: int):
        """assemble() with device pointers (x, y interleaved per cell and
        per face)."""
        _check(lib().pg_assemble_momentum(self._h, dt, nu, theta,
                                          _P(u_old_ptr), _P(u_face_ptr),
                                          PG_DEVICE))
        return self

    def export(self):
        rp = np.empty(self.n + 1, np.int32)
        ci = np.empty(self.nnz, np.int32)
        v = np.empty(self.nnz)
        rhs = np.empty(2 * self.n)
        _check(lib().pg_eqn_export(self._h, _ptr(rp), _ptr(ci), _ptr(v),
                                   _ptr(rhs)))
        return rp, ci, v, rhs

    diagonal = _eqn_diagonal


def default_cfg(**kw) -> SolverCfg:
    c = SolverCfg()
    lib().pg_solver_default_cfg(ctypes.byref(c))
    for k, v in kw.items():
        if not hasattr(c, k):
            raise KeyError(k)
        setattr(c, k, v)
    return c


class SparseMatrixSolver:
    """The SparseMatrixSolver plugin backed by the GB300 library.

    Mirrors src/Math/SparseMatrixSolver.h:11-62: setRank, set(rowPtr,
    colInds, vals) (negative columns are CrsEquation placeholders and are
    skipped), setGuess, setRhs (already negated rhs), solve, x, nIters,
    error.  ``set_eqn`` takes a device equation without a host round trip.
    """

    def __init__(self, **cfg):
        c = default_cfg(**cfg)
        h = _P()
        _check(lib().pg_solver_create(ctypes.byref(c), ctypes.byref(h)))
        self._h = h
        self.cfg = c
        self.n = 0
        self.stats = SolveStats()

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.pg_solver_destroy(h)
            self._h = None

    # reference-named API
    def setRank(self, n: int):
        _check(lib().pg_solver_set_rank(self._h, int(n)))
        self.n = int(n)

    def set_row_coords(self, xy):
        """A point per row (cell centroids, [n, 2]) so set() cuts the
        Schwarz subdomains by coordinates; None clears it."""
        if xy is None:
            _check(lib().pg_solver_set_row_coords(self._h, None))
            return
        a = _f64(np.asarray(xy, np.float64).reshape(-1), 2 * self.n)
        _check(lib().pg_solver_set_row_coords(self._h, _ptr(a)))

    def set(self, row_ptr, col_ind, vals):
        rp = _i32(row_ptr, self.n + 1)
        ci = _i32(col_ind, int(rp[-1]))
        v = _f64(vals, int(rp[-1]))
        _check(lib().pg_solver_set_csr(self._h, _ptr(rp), _ptr(ci), _ptr(v),
                                       PG_HOST))

    def set_eqn(self, eqn, component: int | None = None):
        """Hand over a device equation; a MomentumEquation needs the
        component (0: x, 1: y) whose right-hand side is solved."""
        if component is None:
            _check(lib().pg_solver_set_eqn(self._h, eqn._h))
        else:
            _check(lib().pg_solver_set_eqn_component(self._h, eqn._h,
                                                     int(component)))
        self.n = eqn.n

    def setRhs(self, rhs):
        r = _f64(rhs, self.n)
        _check(lib().pg_solver_set_rhs(self._h, _ptr(r), PG_HOST))

    def setGuess(self, x0):
        """Initial guess for the next solve; None = zero guess."""
        if x0 is None:
            _check(lib().pg_solver_set_guess(self._h, None, PG_HOST))
            return
        x = _f64(x0, self.n)
        _check(lib().pg_solver_set_guess(self._h, _ptr(x), PG_HOST))

    def set_device(self, row_ptr: int, col_ind: int, vals: int):
        """set() with device pointers (e.g. torch.Tensor.data_ptr())."""
        _check(lib().pg_solver_set_csr(self._h, _P(row_ptr), _P(col_ind),
                                       _P(vals), PG_DEVICE))

    def setGuess_device(self, ptr: int):
        """Initial guess from device memory at ptr (0 = zero guess)."""
        if not ptr:
            _check(lib().pg_solver_set_guess(self._h, None, PG_HOST))
        else:
            _check(lib().pg_solver_set_guess(self._h, _P(ptr), PG_DEVICE))

    def x_device(self, out_ptr: int):
        """Copy the solution into device memory at out_ptr."""
        _check(lib().pg_solver_get_x(self._h, _P(out_ptr), PG_DEVICE))

    def solve(self) -> float:
        st = SolveStats()
        rc = lib().pg_solver_solve(self._h, ctypes.byref(st))
        _check(rc, allow=(PG_OK, PG_MAX_ITERS, PG_BREAKDOWN, PG_NON_FINITE))
        self.stats = st
        return st.rel_residual

    def x(self):
        out = np.empty(self.n)
        _check(lib().pg_solver_get_x(self._h, _ptr(out), PG_HOST))
        return out

    def nIters(self) -> int:
        return self.stats.iters

    def error(self) -> float:
        return self.stats.rel_residual

    def partition(self):
        part = np.empty(self.n, np.int32)
        k = ctypes.c_int()
        _check(lib().pg_solver_partition(self._h, _ptr(part), ctypes.byref(k)))
        return part, k.value

    def coarse_inverse(self):
        """The FP32 coarse inverse (K x K) of the two-level preconditioner."""
        k = ctypes.c_int()
        _check(lib().pg_solver_coarse_inverse(self._h, None, ctypes.byref(k)))
        out = np.empty((k.value, k.value), np.float32)
        _check(lib().pg_solver_coarse_inverse(self._h, _ptr(out), ctypes.byref(k)))
        return out

    def sweep_form(self) -> int:
        """1 line form, 0 stream form, -1 no ILU(0) sweep."""
        return int(lib().pg_solver_sweep_form(self._h))

    def apply_precond(self, r):
        """z = M^-1 r with the solver's preconditioner (float-float sweeps
        under MIXED), in the caller's row order."""
        r = np.ascontiguousarray(r, np.float64)
        assert r.shape == (self.n,)
        z = np.empty(self.n)
        _check(lib().pg_solver_apply_precond(self._h, _ptr(r), _ptr(z), PG_HOST))
        return z

    def profile(self, reps: int = 20):
        """Per-launch ms of the hot kernels on the current system: FP64 SpMV,
        preconditioner apply, x/r update, ILU(0) factorisation (with the
        coarse inverse), for the mixed precision solver the float-float
        ILU(0) apply, SpMV and update, the coarse correction, and the coarse
        matrix's assembly and inversion alone."""
        ms = np.zeros(9)
        _check(lib().pg_solver_profile(self._h, int(reps), _ptr(ms)))
        return dict(spmv=ms[0], precond=ms[1], update=ms[2], factor=ms[3],
                    precond_dd=ms[4], spmv_dd=ms[5], update_dd=ms[6],
                    coarse=ms[7], coarse_inverse=ms[8])

    KERNEL_KINDS = ("spmv", "sweep", "update", "coarse")

    def trace_kernels(self, on: bool = True):
        """Time the kernels inside the following solves (their iteration
        chunks launched directly, a CUDA event after every launch group)."""
        _check(lib().pg_solver_trace_kernels(self._h, 1 if on else 0))

    def kernel_times(self):
        """Device time inside the last traced solve, per launch-group kind:
        {kind: (total ms, groups)}, plus "dropped" (groups left untimed)."""
        ms = np.zeros(len(self.KERNEL_KINDS))
        cnt = np.zeros(len(self.KERNEL_KINDS), np.int64)
        dropped = np.zeros(1, np.int64)
        _check(lib().pg_solver_kernel_times(self._h, _ptr(ms), _ptr(cnt),
                                            _ptr(dropped)))
        out = {k: (float(ms[i]), int(cnt[i]))
               for i, k in enumerate(self.KERNEL_KINDS)}
        out["dropped"] = int(dropped[0])
        return out

    def printStatus(self, msg: str):
        print(f"{msg} iterations = {self.nIters()}, error = {self.error():f}.")


class SparseLU:
    """The direct backend (pg_lu_*), mirroring EigenSparseMatrixSolver
    (src/Math/EigenSparseMatrixSolver.cpp:5-64): setRank, set(rowPtr,
    colInds, vals) (negative columns skipped, repeated ones summed), setRhs,
    solve (factorise + solve; a new right-hand side alone reuses the
    factors), x, nIters() = 1 and error() = 0 as the reference reports.
    ``set_eqn`` hands over a device equation; ``stats`` holds the
    factorisation's figures and the FP64 true residual."""

    def __init__(self):
        h = _P()
        _check(lib().pg_lu_create(ctypes.byref(h)))
        self._h = h
        self.n = 0
        self.stats = LuStats()

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.pg_lu_destroy(h)
            self._h = None

    def setRank(self, n: int):
        _check(lib().pg_lu_set_rank(self._h, int(n)))
        self.n = int(n)

    def set_row_coords(self, xy):
        if xy is None:
            _check(lib().pg_lu_set_row_coords(self._h, None))
            return
        a = _f64(np.asarray(xy, np.float64).reshape(-1), 2 * self.n)
        _check(lib().pg_lu_set_row_coords(self._h, _ptr(a)))

    def set(self, row_ptr, col_ind, vals):
        rp = _i32(row_ptr, self.n + 1)
        ci = _i32(col_ind, int(rp[-1]))
        v = _f64(vals, int(rp[-1]))
        _check(lib().pg_lu_set_csr(self._h, _ptr(rp), _ptr(ci), _ptr(v),
                                   PG_HOST))

    def set_eqn(self, eqn):
        _check(lib().pg_lu_set_eqn(self._h, eqn._h))
        self.n = eqn.n

    def setRhs(self, rhs):
        r = _f64(rhs, self.n)
        _check(lib().pg_lu_set_rhs(self._h, _ptr(r), PG_HOST))

    def setGuess(self, x0):
        """Ignored, as EigenSparseMatrixSolver's solve ignores it."""

    def solve(self) -> float:
        st = LuStats()
        _check(lib().pg_lu_solve(self._h, ctypes.byref(st)))
        self.stats = st
        return 0.0

    def x(self):
        out = np.empty(self.n)
        _check(lib().pg_lu_get_x(self._h, _ptr(out), PG_HOST))
        return out

    def nIters(self) -> int:
        return 1

    def error(self) -> float:
        return 0.0


def lu_analyse_pattern(row_ptr, col_ind, xy=None, leaf=0):
    """The direct solver's nested-dissection ordering and fronts (host
    analysis only): (perm new->old, fronts [n_fronts, 4] = (s0, k, m,
    parent), list of index arrays per front, heights)."""
    rp = _i32(row_ptr)
    n = rp.size - 1
    ci = _i32(col_ind, int(rp[-1]))
    xa = None if xy is None else _f64(np.asarray(xy).reshape(-1), 2 * n)
    sizes = np.zeros(4, np.int64)
    _check(lib().pg_lu_analyse_pattern(n, _ptr(rp), _ptr(ci),
                                       None if xa is None else _ptr(xa),
                                       int(leaf), _ptr(sizes), None, None,
                                       None))
    perm = np.empty(n, np.int32)
    fr = np.empty((int(sizes[0]), 4), np.int32)
    fidx = np.empty(int(sizes[1]), np.int32)
    _check(lib().pg_lu_analyse_pattern(n, _ptr(rp), _ptr(ci),
                                       None if xa is None else _ptr(xa),
                                       int(leaf), _ptr(sizes), _ptr(perm),
                                       _ptr(fr), _ptr(fidx)))
    lists, o = [], 0
    for s0, k, m, parent in fr:
        lists.append(fidx[o:o + m])
        o += m
    return perm, fr, lists, int(sizes[2])


class BatchSolver:
    """Independent pressure systems solved together (pg_batch_*)."""

    def __init__(self, **cfg):
        c = default_cfg(**cfg)
        h = _P()
        _check(lib().pg_batch_create(ctypes.byref(c), ctypes.byref(h)))
        self._h = h
        self.eqns = []
        self.stats = []
        self.ms = 0.0

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.pg_batch_destroy(h)
            self._h = None

    def set_eqns(self, eqns):
        self.eqns = list(eqns)
        arr = (_P * len(self.eqns))(*[e._h for e in self.eqns])
        _check(lib().pg_batch_set_eqns(self._h, len(self.eqns), arr))

    def solve(self):
        st = (SolveStats * len(self.eqns))()
        ms = _D()
        _check(lib().pg_batch_solve(self._h, st, ctypes.byref(ms)),
               allow=(PG_OK, PG_MAX_ITERS, PG_BREAKDOWN, PG_NON_FINITE))
        self.stats = list(st)
        self.ms = ms.value
        return self.stats

    def x(self, i):
        out = np.empty(self.eqns[i].n)
        _check(lib().pg_batch_get_x(self._h, int(i), _ptr(out), PG_HOST))
        return out

    def tuning(self):
        a, b, c = _I(), _I(), _I()
        _check(lib().pg_batch_tuning(self._h, ctypes.byref(a), ctypes.byref(b),
                                     ctypes.byref(c)))
        return dict(block=a.value, rows_per_thread=b.value, n_tiles=c.value)


@dataclass
class _FvNamespace:
    """fv::laplacian as a function returning a device equation."""

    @staticmethod
    def laplacian(gamma, mesh: Mesh, bc_type, bc_value=None, div_u=None,
                  eqn: Equation | None = None) -> Equation:
        """fv::laplacian(gamma, phi) == src::div(u) on the device.

        gamma: float (Laplacian.h:49-83) or per-face array (:132-167).
        div_u: face velocities [n_faces, 2] for the src::div right-hand side.
        """
        face = not np.isscalar(gamma)
        kind = GAMMA_FACE if face else GAMMA_SCALAR
        if eqn is None or eqn.gamma_kind != kind:
            eqn = Equation(mesh, kind, bc_type)
        return eqn.assemble(gamma_face=gamma if face else None,
                            gamma_scalar=0.0 if face else float(gamma),
                            bc_value=bc_value, u_face=div_u)


fv = _FvNamespace()
