"""ctypes binding of the CPU oracle (oracle/liboracle.so) and of the
reference's own CrsEquation build (oracle/_ref/libref_crs.so).

Test infrastructure only: the oracle is the checker, never the product.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_SO = os.path.join(ORACLE_DIR, "liboracle.so")
REF_SO = os.path.join(ORACLE_DIR, "_ref", "libref_crs.so")

P = ctypes.c_void_p
I64 = ctypes.c_int64
D = ctypes.c_double

OR_PREC_NONE, OR_PREC_JACOBI, OR_PREC_ILU0, OR_PREC_ILUT = 0, 1, 2, 3


class OrCfg(ctypes.Structure):
    _fields_ = [("tol", D), ("max_iters", ctypes.c_int),
                ("precond", ctypes.c_int), ("ilut_drop", D),
                ("ilut_fill", ctypes.c_int), ("n_threads", ctypes.c_int),
                ("part", P), ("n_parts", ctypes.c_int),
                ("use_guess", ctypes.c_int), ("coarse", ctypes.c_int),
                ("krylov", ctypes.c_int), ("krylov_dim", ctypes.c_int),
                ("ilu_fill", ctypes.c_int)]


class OrStats(ctypes.Structure):
    _fields_ = [("iters", ctypes.c_int), ("status", ctypes.c_int),
                ("rel_residual", D), ("ms", D), ("setup_ms", D)]


def build_oracle():
    """Build liboracle.so (and oracle/_ref when the reference is present)."""
    subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True,
                   capture_output=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO) or (
                os.path.getmtime(ORACLE_SO) <
                os.path.getmtime(os.path.join(ORACLE_DIR, "oracle.cpp"))):
            build_oracle()
        L = ctypes.CDLL(ORACLE_SO)
        L.or_mesh_create.restype = P
        L.or_mesh_create.argtypes = [P, I64, P, P, I64]
        L.or_mesh_destroy.argtypes = [P]
        L.or_mesh_sizes.argtypes = [P, P, P, P, P]
        L.or_mesh_cells.argtypes = [P, P, P, P]
        L.or_mesh_faces.argtypes = [P] + [P] * 8
        L.or_mesh_nlinks.restype = I64
        L.or_mesh_nlinks.argtypes = [P]
        L.or_mesh_links.argtypes = [P, P, P, P]
        L.or_interpolate_faces.argtypes = [P, P, P]
        L.or_dt_over_rho_faces.argtypes = [P, P, D, D, D, P]
        L.or_laplacian.restype = P
        L.or_laplacian.argtypes = [P, P, D, P, P, P]
        L.or_eqn_destroy.argtypes = [P]
        L.or_eqn_sizes.argtypes = [P, P, P, P]
        L.or_eqn_export_slots.argtypes = [P, P, P, P, P]
        L.or_eqn_export_csr.argtypes = [P, P, P, P, P]
        L.or_gradient.argtypes = [P, P, P, P, P]
        L.or_bicgstab.restype = ctypes.c_int
        L.or_bicgstab.argtypes = [I64, P, P, P, P, P, ctypes.POINTER(OrCfg),
                                  ctypes.POINTER(OrStats)]
        L.or_bicgstab_history.restype = ctypes.c_int
        L.or_bicgstab_history.argtypes = [I64, P, P, P, P,
                                          ctypes.POINTER(OrCfg), P, P, P]
        L.or_bicgstab_history_x0.restype = ctypes.c_int
        L.or_bicgstab_history_x0.argtypes = [I64, P, P, P, P, P,
                                             ctypes.POINTER(OrCfg), P, P, P]
        L.or_ilu0.restype = ctypes.c_int
        L.or_ilu0.argtypes = [I64, P, P, P, P, P]
        L.or_ilu0_apply.argtypes = [I64, P, P, P, P, P, P]
        L.or_spmv.argtypes = [I64, P, P, P, P, P]
        L.or_iluk_apply.argtypes = [I64, P, P, P, P, ctypes.c_int, P, P]
        L.or_momentum.restype = P
        L.or_momentum.argtypes = [P, D, D, D, P, P, P]
        L.or_correct_velocity.argtypes = [P, D, P, P, P, P, P, P]
        L.or_set_boundary_faces.argtypes = [P, P, P, P]
        L.or_gcib_laplacian.restype = P
        L.or_gcib_laplacian.argtypes = [P, P, D, P, P, P, ctypes.c_int, P,
                                        ctypes.c_int, D, P]
        L.or_sparse_lu_solve.argtypes = [I64, P, P, P, P, P, P, P]
        _lib = L
    return _lib


def ptr(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


class OracleMesh:
    def __init__(self, nodes, cptr, cind):
        nodes = np.ascontiguousarray(nodes, np.float64)
        cptr = np.ascontiguousarray(cptr, np.int64)
        cind = np.ascontiguousarray(cind, np.int64)
        self.h = lib().or_mesh_create(ptr(nodes), nodes.size // 2, ptr(cptr),
                                      ptr(cind), cptr.size - 1)
        s = np.zeros(4, np.int64)
        lib().or_mesh_sizes(self.h, ptr(s[0:1]), ptr(s[1:2]), ptr(s[2:3]),
                            ptr(s[3:4]))
        self.n_cells, self.n_faces, self.n_interior, self.n_boundary = map(int, s)

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.or_mesh_destroy(self.h)
            self.h = None

    def faces(self):
        nf = self.n_faces
        o = dict(lcell=np.empty(nf, np.int32), rcell=np.empty(nf, np.int32),
                 lnode=np.empty(nf, np.int32), rnode=np.empty(nf, np.int32),
                 fx=np.empty(nf), fy=np.empty(nf), nx=np.empty(nf),
                 ny=np.empty(nf))
        lib().or_mesh_faces(self.h, *(ptr(o[k]) for k in (
            "lcell", "rcell", "lnode", "rnode", "fx", "fy", "nx", "ny")))
        return o

    def cells(self):
        n = self.n_cells
        o = dict(cx=np.empty(n), cy=np.empty(n), vol=np.empty(n))
        lib().or_mesh_cells(self.h, ptr(o["cx"]), ptr(o["cy"]), ptr(o["vol"]))
        return o

    def links(self):
        nl = lib().or_mesh_nlinks(self.h)
        lp = np.empty(self.n_cells + 1, np.int64)
        lf = np.empty(nl, np.int32)
        lc = np.empty(nl, np.int32)
        lib().or_mesh_links(self.h, ptr(lp), ptr(lf), ptr(lc))
        return lp, lf, lc

    def interpolate_faces(self, cell_vals):
        cv = np.ascontiguousarray(cell_vals, np.float64)
        out = np.empty(self.n_faces)
        lib().or_interpolate_faces(self.h, ptr(cv), ptr(out))
        return out

    def dt_over_rho(self, gamma_cell, rho1, rho2, dt):
        gf = self.interpolate_faces(gamma_cell)
        out = np.empty(self.n_faces)
        lib().or_dt_over_rho_faces(self.h, ptr(gf), rho1, rho2, dt, ptr(out))
        return out

    def laplacian(self, gamma, bc_type, bc_value, u_face=None, slots=False):
        """fv::laplacian(gamma, phi) == src::div(u): (row_ptr, col, vals, rhs)."""
        face = not np.isscalar(gamma)
        g = np.ascontiguousarray(gamma, np.float64) if face else None
        bc = np.ascontiguousarray(bc_type, np.int32)
        bv = np.ascontiguousarray(bc_value, np.float64)
        u = None if u_face is None else np.ascontiguousarray(u_face, np.float64)
        e = lib().or_laplacian(self.h, ptr(g), 0.0 if face else float(gamma),
                               ptr(bc), ptr(bv), ptr(u))
        s = np.zeros(3, np.int64)
        lib().or_eqn_sizes(e, ptr(s[0:1]), ptr(s[1:2]), ptr(s[2:3]))
        n, ns, nnz = map(int, s)
        m = ns if slots else nnz
        rp = np.empty(n + 1, np.int32)
        ci = np.empty(m, np.int32)
        v = np.empty(m)
        rhs = np.empty(n)
        (lib().or_eqn_export_slots if slots else lib().or_eqn_export_csr)(
            e, ptr(rp), ptr(ci), ptr(v), ptr(rhs))
        lib().or_eqn_destroy(e)
        return rp, ci, v, rhs

    def gcib_laplacian(self, gamma, bc_type, bc_value, u_face, circles,
                       ib_bc=1, ib_ref=0.0):
        """(fv::laplacian(gamma, p) + ib.bcs(p)) == src::div(u) with
        ghost-cell IB circles [(cx, cy, r), ...]: (row_ptr, col, vals, rhs,
        cell class 0 fluid / 1 IB / 2 solid)."""
        face = not np.isscalar(gamma)
        g = np.ascontiguousarray(gamma, np.float64) if face else None
        bc = np.ascontiguousarray(bc_type, np.int32)
        bv = np.ascontiguousarray(bc_value, np.float64)
        u = None if u_face is None else np.ascontiguousarray(u_face, np.float64)
        c = np.ascontiguousarray(np.asarray(circles, np.float64).reshape(-1, 3))
        cls = np.empty(self.n_cells, np.int32)
        e = lib().or_gcib_laplacian(self.h, ptr(g), 0.0 if face else float(gamma),
                                    ptr(bc), ptr(bv), ptr(u), len(c), ptr(c),
                                    int(ib_bc), float(ib_ref), ptr(cls))
        if not e:
            raise RuntimeError("or_gcib_laplacian: degenerate IB stencil")
        s = np.zeros(3, np.int64)
        lib().or_eqn_sizes(e, ptr(s[0:1]), ptr(s[1:2]), ptr(s[2:3]))
        n, ns, nnz = map(int, s)
        rp = np.empty(n + 1, np.int32)
        ci = np.empty(nnz, np.int32)
        v = np.empty(nnz)
        rhs = np.empty(n)
        lib().or_eqn_export_csr(e, ptr(rp), ptr(ci), ptr(v), ptr(rhs))
        lib().or_eqn_destroy(e)
        return rp, ci, v, rhs, cls

    def set_boundary_faces(self, bc_type, phi_cell, phi_face):
        out = np.array(phi_face, np.float64)
        lib().or_set_boundary_faces(self.h, ptr(np.ascontiguousarray(bc_type, np.int32)),
                                    ptr(np.ascontiguousarray(phi_cell, np.float64)),
                                    ptr(out))
        return out

    def correct_velocity(self, dt, grad_cell, grad_face, u_cell, u_face,
                         rho_cell=None, rho_face=None):
        uc = np.array(u_cell, np.float64).reshape(-1)
        uf = np.array(u_face, np.float64).reshape(-1)
        rc = None if rho_cell is None else np.ascontiguousarray(rho_cell, np.float64)
        rf = None if rho_face is None else np.ascontiguousarray(rho_face, np.float64)
        gc = np.ascontiguousarray(np.asarray(grad_cell, np.float64).reshape(-1))
        gf = np.ascontiguousarray(np.asarray(grad_face, np.float64).reshape(-1))
        lib().or_correct_velocity(self.h, float(dt), ptr(rc), ptr(rf), ptr(gc),
                                  ptr(gf), ptr(uc), ptr(uf))
        return uc.reshape(-1, 2), uf.reshape(-1, 2)

    def momentum(self, dt, nu, theta, u_old_cell, u_face, bc_type):
        """ddt + div - laplacian(nu) of the vector equation: compact CSR of
        2N rows (x then y) and rhs[2N]."""
        u0 = np.ascontiguousarray(u_old_cell, np.float64)
        uf = np.ascontiguousarray(u_face, np.float64)
        bc = np.ascontiguousarray(bc_type, np.int32)
        e = lib().or_momentum(self.h, dt, nu, theta, ptr(u0), ptr(uf), ptr(bc))
        s = np.zeros(3, np.int64)
        lib().or_eqn_sizes(e, ptr(s[0:1]), ptr(s[1:2]), ptr(s[2:3]))
        n, ns, nnz = map(int, s)
        rp = np.empty(n + 1, np.int32)
        ci = np.empty(nnz, np.int32)
        v = np.empty(nnz)
        rhs = np.empty(n)
        lib().or_eqn_export_csr(e, ptr(rp), ptr(ci), ptr(v), ptr(rhs))
        lib().or_eqn_destroy(e)
        return rp, ci, v, rhs

    def gradient(self, phi_cell, phi_face):
        pc = np.ascontiguousarray(phi_cell, np.float64)
        pf = np.ascontiguousarray(phi_face, np.float64)
        gf = np.empty(2 * self.n_faces)
        gc = np.empty(2 * self.n_cells)
        lib().or_gradient(self.h, ptr(pc), ptr(pf), ptr(gf), ptr(gc))
        return gf.reshape(-1, 2), gc.reshape(-1, 2)


def sparse_lu_solve(rp, ci, v, b):
    """Oracle direct solve (RCM band LU with partial pivoting); returns
    (x, dict(band=(kl, ku), replaced=count))."""
    rp = np.ascontiguousarray(rp, np.int32)
    ci = np.ascontiguousarray(ci, np.int32)
    v = np.ascontiguousarray(v, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    x = np.zeros(b.size)
    band = np.zeros(2, np.int64)
    rep = ctypes.c_int()
    lib().or_sparse_lu_solve(b.size, rp.ctypes.data, ci.ctypes.data,
                             v.ctypes.data, b.ctypes.data, x.ctypes.data,
                             band.ctypes.data, ctypes.byref(rep))
    return x, dict(band=(int(band[0]), int(band[1])), replaced=rep.value)


def bicgstab(rp, ci, v, b, tol=1e-8, max_iters=500, precond=OR_PREC_ILU0,
             part=None, x0=None, threads=0, ilut_drop=1e-4, ilut_fill=10,
             coarse=0, krylov=0, krylov_dim=0, ilu_fill=0):
    """Oracle BiCGStab solve; returns (x, stats dict)."""
    rp = np.ascontiguousarray(rp, np.int32)
    ci = np.ascontiguousarray(ci, np.int32)
    v = np.ascontiguousarray(v, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    n = b.size
    x = np.zeros(n) if x0 is None else np.array(x0, np.float64)
    pa = None if part is None else np.ascontiguousarray(part, np.int32)
    cfg = OrCfg(tol=tol, max_iters=max_iters, precond=precond,
                ilut_drop=ilut_drop, ilut_fill=ilut_fill, n_threads=threads,
                part=None if pa is None else pa.ctypes.data,
                n_parts=0 if pa is None else int(pa.max()) + 1,
                use_guess=0 if x0 is None else 1, coarse=coarse,
                krylov=krylov, krylov_dim=krylov_dim, ilu_fill=ilu_fill)
    st = OrStats()
    lib().or_bicgstab(n, ptr(rp), ptr(ci), ptr(v), ptr(b), ptr(x),
                      ctypes.byref(cfg), ctypes.byref(st))
    return x, {k: getattr(st, k) for k, _ in st._fields_}


def bicgstab_history(rp, ci, v, b, max_iters, precond=OR_PREC_ILU0, part=None,
                     threads=0, x0=None):
    """Run max_iters iterations from x0 (None: zero); return (residual
    history, ms, setup_ms)."""
    rp = np.ascontiguousarray(rp, np.int32)
    ci = np.ascontiguousarray(ci, np.int32)
    v = np.ascontiguousarray(v, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    pa = None if part is None else np.ascontiguousarray(part, np.int32)
    cfg = OrCfg(tol=0.0, max_iters=max_iters, precond=precond, ilut_drop=1e-4,
                ilut_fill=10, n_threads=threads,
                part=None if pa is None else pa.ctypes.data,
                n_parts=0 if pa is None else int(pa.max()) + 1, use_guess=0)
    hist = np.zeros(max_iters + 1)
    ms = np.zeros(1)
    sms = np.zeros(1)
    x = None if x0 is None else np.ascontiguousarray(x0, np.float64)
    it = lib().or_bicgstab_history_x0(b.size, ptr(rp), ptr(ci), ptr(v),
                                      ptr(b), ptr(x), ctypes.byref(cfg),
                                      ptr(hist), ptr(ms), ptr(sms))
    return hist[:it + 1], float(ms[0]), float(sms[0])


def ilu0(rp, ci, v, part=None):
    out = np.empty_like(np.asarray(v, np.float64))
    pa = None if part is None else np.ascontiguousarray(part, np.int32)
    rc = lib().or_ilu0(len(rp) - 1, ptr(np.ascontiguousarray(rp, np.int32)),
                       ptr(np.ascontiguousarray(ci, np.int32)),
                       ptr(np.ascontiguousarray(v, np.float64)), ptr(pa),
                       ptr(out))
    return out, rc


def ilu0_apply(rp, ci, lu, r, part=None):
    """z = (LU)^-1 r for the factors of ilu0() (per subdomain with part)."""
    z = np.empty(len(rp) - 1)
    pa = None if part is None else np.ascontiguousarray(part, np.int32)
    lib().or_ilu0_apply(len(rp) - 1, ptr(np.ascontiguousarray(rp, np.int32)),
                        ptr(np.ascontiguousarray(ci, np.int32)),
                        ptr(np.ascontiguousarray(lu, np.float64)), ptr(pa),
                        ptr(np.ascontiguousarray(r, np.float64)), ptr(z))
    return z


def iluk_apply(rp, ci, v, r, fill, part=None):
    """z = (LU)^-1 r with the level-of-fill ILU(k) factor of each subdomain
    (natural row order); returns (z, status)."""
    z = np.zeros(len(rp) - 1)
    pa = None if part is None else np.ascontiguousarray(part, np.int32)
    rc = lib().or_iluk_apply(len(rp) - 1, ptr(np.ascontiguousarray(rp, np.int32)),
                             ptr(np.ascontiguousarray(ci, np.int32)),
                             ptr(np.ascontiguousarray(v, np.float64)), ptr(pa),
                             int(fill), ptr(np.ascontiguousarray(r, np.float64)),
                             ptr(z))
    return z, rc


def spmv(rp, ci, v, x):
    y = np.empty(len(rp) - 1)
    lib().or_spmv(len(rp) - 1, ptr(np.ascontiguousarray(rp, np.int32)),
                  ptr(np.ascontiguousarray(ci, np.int32)),
                  ptr(np.ascontiguousarray(v, np.float64)),
                  ptr(np.ascontiguousarray(x, np.float64)), ptr(y))
    return y


# ---------------------------------------------------- reference CrsEquation
_ref = None


def ref_lib():
    """The reference's own CrsEquation (None when oracle/_ref is absent)."""
    global _ref
    if _ref is None:
        if not os.path.exists(REF_SO):
            try:
                build_oracle()
            except Exception:
                return None
        if not os.path.exists(REF_SO):
            return None
        L = ctypes.CDLL(REF_SO)
        L.ref_crs_create.restype = P
        L.ref_crs_create.argtypes = [I64, I64]
        L.ref_crs_destroy.argtypes = [P]
        L.ref_crs_apply.argtypes = [P, I64, P, P, P, P]
        L.ref_crs_eq_vector.argtypes = [P, I64, P]
        L.ref_crs_plus.argtypes = [P, P]
        L.ref_crs_sizes.argtypes = [P, P, P]
        L.ref_crs_export.argtypes = [P, P, P, P, P]
        _ref = L
    return _ref


class RefCrs:
    """Handle on a real reference CrsEquation(n_rows, nnz_per_row)."""

    def __init__(self, n, nnz=5):
        self.h = ref_lib().ref_crs_create(n, nnz)
        self.n = n

    def __del__(self):
        if getattr(self, "h", None) and _ref is not None:
            _ref.ref_crs_destroy(self.h)
            self.h = None

    def apply(self, ops, rows, cols, vals):
        ops = np.ascontiguousarray(ops, np.int32)
        rows = np.ascontiguousarray(rows, np.int32)
        cols = np.ascontiguousarray(cols, np.int32)
        vals = np.ascontiguousarray(vals, np.float64)
        ref_lib().ref_crs_apply(self.h, ops.size, ptr(ops), ptr(rows),
                                ptr(cols), ptr(vals))

    def eq_vector(self, v):
        v = np.ascontiguousarray(v, np.float64)
        ref_lib().ref_crs_eq_vector(self.h, v.size, ptr(v))

    def plus(self, other):
        ref_lib().ref_crs_plus(self.h, other.h)

    def export(self):
        s = np.zeros(2, np.int64)
        ref_lib().ref_crs_sizes(self.h, ptr(s[0:1]), ptr(s[1:2]))
        n, ns = map(int, s)
        rp = np.empty(n + 1, np.int32)
        ci = np.empty(ns, np.int32)
        v = np.empty(ns)
        rhs = np.empty(n)
        ref_lib().ref_crs_export(self.h, ptr(rp), ptr(ci), ptr(v), ptr(rhs))
        return rp, ci, v, rhs
