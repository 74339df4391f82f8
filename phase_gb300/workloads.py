"""Seeded synthetic pressure systems with the shapes of the benchmark cases.

Phase reads its cases from INFO files and CGNS meshes and obtains the
volume fraction by advection; none of that is on the pressure path, so the
inputs of the pressure equation are synthesised here with the sizes, value
ranges and boundary conditions of the cases they stand for.

Rising bubble (Examples/RisingBubble/case/boundaries.info): 1024x1024 quads on
[0,1]x[0,2]; gamma = smoothed Heaviside of a circle r=0.25 at (0.5,0.5) over
1.5 cells; rho1 = 1000 (liquid), rho2 = 1 (gas), so the face coefficient
dt/rho_f spans 1000x; p FIXED 0 on y+, NORMAL_GRADIENT elsewhere; the
right-hand side is src::div(u*) of a seeded divergent face velocity.
"""
from __future__ import annotations

import numpy as np

from . import meshes

RB_WIDTH, RB_HEIGHT = 1.0, 2.0
RB_RHO1, RB_RHO2 = 1000.0, 1.0
RB_DT = 1e-4
RB_RADIUS, RB_CENTRE = 0.25, (0.5, 0.5)


def smoothed_heaviside(phi, eps):
    """H_eps(phi): 0 below -eps, 1 above eps, sine-smoothed between."""
    h = 0.5 * (1.0 + phi / eps + np.sin(np.pi * phi / eps) / np.pi)
    return np.where(phi > eps, 1.0, np.where(phi < -eps, 0.0, h))


def bubble_gamma(cx, cy, nx, ny, centre=RB_CENTRE, radius=RB_RADIUS):
    hx, hy = RB_WIDTH / nx, RB_HEIGHT / ny
    eps = 1.5 * max(hx, hy)
    phi = radius - np.hypot(cx - centre[0], cy - centre[1])
    return smoothed_heaviside(phi, eps)


def rising_bubble_bcs(faces, nx, ny):
    """bc_type / bc_value per face for p: FIXED 0 on y+, NORMAL_GRADIENT else."""
    patch = meshes.rect_patch_of_faces(faces["fx"], faces["fy"], faces["rcell"],
                                       RB_WIDTH, RB_HEIGHT)
    bc_type = np.full(patch.shape, 1, np.int32)  # NORMAL_GRADIENT
    bc_type[patch == 3] = 0                       # FIXED on y+
    bc_value = np.zeros(patch.shape)
    return bc_type, bc_value, patch


def divergent_velocity(faces, patch, seed, amplitude=0.1, noise=0.01):
    """Seeded face velocity u* (n_faces x 2) with non-zero divergence.

    A smooth swirl plus seeded noise; zero on the walls x-, x+, y- (no slip)
    and free on y+.
    """
    rng = np.random.default_rng(seed)
    x, y = faces["fx"], faces["fy"]
    u = np.empty((x.size, 2))
    u[:, 0] = amplitude * np.sin(np.pi * x) * np.cos(0.5 * np.pi * y)
    u[:, 1] = amplitude * np.cos(np.pi * x) * np.sin(0.5 * np.pi * y) + 0.02
    u += noise * rng.standard_normal(u.shape)
    wall = (patch == 0) | (patch == 1) | (patch == 2)
    u[wall] = 0.0
    return u


def rising_bubble(nx=1024, ny=1024, seed=3, faces=None, cells=None):
    """Inputs of the rising-bubble pressure system.

    faces/cells: face and cell arrays of the mesh built from
    ``meshes.rectilinear(nx, ny, 1, 2)`` (from either the device mesh or any
    implementation with the reference's numbering).  Returns a dict with the
    mesh arrays, gamma per cell, bc_type/bc_value per face and u* per face.
    """
    nodes, cptr, cind = meshes.rectilinear(nx, ny, RB_WIDTH, RB_HEIGHT)
    out = dict(nodes=nodes, cptr=cptr, cind=cind, nx=nx, ny=ny,
               rho1=RB_RHO1, rho2=RB_RHO2, dt=RB_DT, seed=seed)
    if faces is not None and cells is not None:
        out["gamma"] = bubble_gamma(cells["cx"], cells["cy"], nx, ny)
        bc_type, bc_value, patch = rising_bubble_bcs(faces, nx, ny)
        out.update(bc_type=bc_type, bc_value=bc_value, patch=patch)
        out["u"] = divergent_velocity(faces, patch, seed)
    return out


# ---------------------------------------------------------------------------
# Ghost-cell immersed-boundary channels (batched solves): the pressure
# equation of FractionalStepGCIB, (fv::laplacian(dt/rho, p) + ib.bcs(p)) ==
# src::div(u), on a quad channel [0, 3H] x [0, H] with one cylinder.
GC_HEIGHT = 2.0
GC_LENGTH = 3.0 * GC_HEIGHT


def gcib_specs(n_systems=256, seed=5, min_cells=2_000, max_cells=200_000):
    """Seeded case list: cell counts log-uniform in [min_cells, max_cells]
    (ny rows, nx = 3 ny columns), cylinder radius uniform in [0.1, 0.5],
    centre uniform in the channel interior with a margin that keeps every
    image-point stencil inside the mesh."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_systems):
        n = float(np.exp(rng.uniform(np.log(min_cells), np.log(max_cells))))
        ny = max(8, int(round(np.sqrt(n / 3.0))))
        nx = 3 * ny
        h = GC_HEIGHT / ny
        r = float(rng.uniform(0.1, 0.5))
        m = r + 4.0 * h + 0.05
        cx = float(rng.uniform(1.0, GC_LENGTH - 2.0))
        cy = float(rng.uniform(m, GC_HEIGHT - m))
        out.append(dict(nx=nx, ny=ny, circle=(cx, cy, r),
                        seed=int(rng.integers(1 << 30))))
    return out


def gcib_case(spec, faces=None):
    """Mesh arrays and, given the mesh's faces, the inputs of one case:
    p FIXED 0 at the outlet (x+), NORMAL_GRADIENT elsewhere; scalar
    coefficient dt/rho = 1e-3; u* a seeded divergent field (inflow 1 at x-,
    no slip on the walls)."""
    nx, ny = spec["nx"], spec["ny"]
    nodes, cptr, cind = meshes.rectilinear(nx, ny, GC_LENGTH, GC_HEIGHT)
    out = dict(nodes=nodes, cptr=cptr, cind=cind, circle=spec["circle"],
               gamma=1e-3)
    if faces is not None:
        patch = meshes.rect_patch_of_faces(faces["fx"], faces["fy"],
                                           faces["rcell"], GC_LENGTH, GC_HEIGHT)
        bc = np.ones(patch.shape, np.int32)
        bc[patch == 1] = 0
        rng = np.random.default_rng(spec["seed"])
        x, y = faces["fx"], faces["fy"]
        u = np.zeros((x.size, 2))
        u[:, 0] = 4.0 * y * (GC_HEIGHT - y) / GC_HEIGHT ** 2
        u += 0.05 * rng.standard_normal(u.shape)
        u[(patch == 2) | (patch == 3)] = 0.0
        out.update(bc_type=bc, bc_value=np.zeros(patch.shape), u=u,
                   patch=patch)
    return out


def rising_bubble_step(faces, cells, patch, nx, t, seed=3, span=2000):
    """Host (numpy) fields of step t of the rising-bubble sequence: gamma per
    cell (the bubble centre rises from y = 0.5 to 1.5 over ``span`` steps)
    and the face velocity u* (a smooth swirl plus noise from a generator
    seeded by (seed, t), zero on the walls).  The bench's timed steps and
    the CPU reference arm build their systems from these, so both solve the
    same matrices."""
    cx0, cy0 = 0.5, 0.5 + min(t, span) / span
    hx, hy = RB_WIDTH / nx, RB_HEIGHT / nx
    eps = 1.5 * max(hx, hy)
    phi = RB_RADIUS - np.hypot(cells["cx"] - cx0, cells["cy"] - cy0)
    gamma = smoothed_heaviside(phi, eps)
    rng = np.random.default_rng([seed, t])
    x, y = faces["fx"], faces["fy"]
    u = np.empty((x.size, 2))
    u[:, 0] = 0.1 * np.sin(np.pi * x) * np.cos(0.5 * np.pi * y)
    u[:, 1] = 0.1 * np.cos(np.pi * x) * np.sin(0.5 * np.pi * y) + 0.02
    u += 0.01 * rng.standard_normal(u.shape)
    u[(patch == 0) | (patch == 1) | (patch == 2)] = 0.0
    return gamma, u
