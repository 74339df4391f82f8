"""The CGNS mesh reader (phase_gb300/cgns.py) against Phase's loader
semantics (CgnsUnstructuredGrid::load, CgnsUnstructuredGrid.cpp:13-96):
files written here by a minimal ADF writer (sections out of element order,
a MIXED section, PointList and PointRange patches), and the example meshes
of the reference's cases when its tree is present."""
import os

import numpy as np
import pytest

import adf_writer as W
from __graft_entry__ import REFERENCE_SRC
from phase_gb300 import cgns

REF_EXAMPLES = os.path.join(REFERENCE_SRC, "Examples")


def _tiny_file(mixed=False, point_range=False, zone_type="Unstructured",
               cell_dim=2):
    # 2 x 1 quads (nodes 1..6, row-major) + their 6 boundary edges
    x = [0., 1., 2., 0., 1., 2.]
    y = [0., 0., 0., 1., 1., 1.]
    quads = [1, 2, 5, 4, 2, 3, 6, 5]
    bars = [1, 2, 2, 3, 3, 6, 6, 5, 5, 4, 4, 1]
    if mixed:
        conn = [7, 1, 2, 5, 4, 7, 2, 3, 6, 5]  # QUAD_4 code before each
        cells = W.Node("Cells 5 - 6", "Elements_t", "I4", [20, 0], children=[
            W.Node("ElementRange", "IndexRange_t", "I4", [5, 6]),
            W.Node("ElementConnectivity", "DataArray_t", "I4", conn)])
    else:
        cells = W.Node("QUAD_4 5 - 6", "Elements_t", "I4", [7, 0], children=[
            W.Node("ElementRange", "IndexRange_t", "I4", [5, 6]),
            W.Node("ElementConnectivity", "DataArray_t", "I4", quads)])
    # edges 1..4 before the cells, 7..8 after (ids need not follow sections)
    bar_a = W.Node("BAR_2 1 - 4", "Elements_t", "I4", [3, 0], children=[
        W.Node("ElementRange", "IndexRange_t", "I4", [1, 4]),
        W.Node("ElementConnectivity", "DataArray_t", "I4", bars[:8])])
    bar_b = W.Node("BAR_2 7 - 8", "Elements_t", "I4", [3, 0], children=[
        W.Node("ElementRange", "IndexRange_t", "I4", [7, 8]),
        W.Node("ElementConnectivity", "DataArray_t", "I4", bars[8:])])
    if point_range:
        walls = W.Node("Walls", "BC_t", "C1", "BCWall", children=[
            W.Node("PointRange", "IndexRange_t", "I4", [[1, 4]], dims=[1, 2])])
    else:
        walls = W.Node("Walls", "BC_t", "C1", "BCWall", children=[
            W.Node("PointList", "IndexArray_t", "I4",
                   np.array([[1, 2, 3, 4]]), dims=[1, 4])])
    ends = W.Node("Ends", "BC_t", "C1", "BCInflow", children=[
        W.Node("PointList", "IndexArray_t", "I4", np.array([[7, 8]]),
               dims=[1, 2])])
    zone = W.Node("Zone", "Zone_t", "I4", np.array([[6, 2, 0]]), dims=[1, 3],
                  children=[
                      W.Node("ZoneType", "ZoneType_t", "C1", zone_type),
                      W.Node("GridCoordinates", "GridCoordinates_t", children=[
                          W.Node("CoordinateX", "DataArray_t", "R8", x),
                          W.Node("CoordinateY", "DataArray_t", "R8", y)]),
                      bar_a, cells, bar_b,
                      W.Node("ZoneBC", "ZoneBC_t", children=[walls, ends])])
    base = W.Node("Base", "CGNSBase_t", "I4", [cell_dim, 2], children=[zone])
    return W.write([W.Node("CGNSLibraryVersion", "CGNSLibraryVersion_t", "R4",
                           [3.13]), base])


@pytest.mark.parametrize("mixed", [False, True])
@pytest.mark.parametrize("point_range", [False, True])
def test_reader_on_a_written_file(mixed, point_range):
    m = cgns.read_mesh(_tiny_file(mixed, point_range), origin=(10.0, -1.0))
    assert m["n_elements"] == 8
    np.testing.assert_array_equal(m["cptr"], [0, 4, 8])
    np.testing.assert_array_equal(m["cind"], [0, 1, 4, 3, 1, 2, 5, 4])
    assert m["nodes"][0].tolist() == [10.0, -1.0]
    assert m["patches"]["Walls"] == [0, 1, 1, 2, 2, 5, 5, 4]
    assert m["patches"]["Ends"] == [4, 3, 3, 0]


def test_reader_rejects_what_phase_rejects():
    with pytest.raises(cgns.CgnsError, match="Unstructured"):
        cgns.read_mesh(_tiny_file(zone_type="Structured"))
    with pytest.raises(cgns.CgnsError, match="cell dimension"):
        cgns.read_mesh(_tiny_file(cell_dim=3))
    with pytest.raises(cgns.CgnsError, match="not an ADF file"):
        cgns.read_mesh(b"\x89HDF\r\n\x1a\n" + b"\0" * 600)


def _example(name):
    path = os.path.join(REF_EXAMPLES, name)
    if not os.path.exists(path):
        pytest.skip("the reference's example meshes are not present")
    return path


@pytest.mark.parametrize("name,n_cells,patch_faces", [
    ("UnstructuredFlowAroundCylinder/case/CylinderMesh.cgns", 15316,
     {"Cylinder": 100, "TopBottom": 82, "Inlet": 32, "Outlet": 32}),
    ("FlowAroundBox/case/BoxMesh.cgns", 10625,
     {"Inlet": 75, "BoxWalls": 100, "SymmetryPlanes": 300, "Outlet": 75}),
    ("SuddenExpansion/case/SuddenExpansionMesh.cgns", 2250,
     {"Inlet": 15, "Walls": 150, "Outlet": 45}),
])
def test_example_meshes_build_with_every_boundary_face_in_a_patch(
        oracle, name, n_cells, patch_faces):
    """The grid the reference builds from its example files: cell count,
    patches covering every boundary face exactly once, and a closed mesh
    (Euler characteristic 1 - holes)."""
    m = cgns.read_mesh(_example(name))
    assert len(m["cptr"]) - 1 == n_cells
    assert {k: len(v) // 2 for k, v in m["patches"].items()} == patch_faces
    om = oracle.OracleMesh(m["nodes"], m["cptr"], m["cind"])
    f = om.faces()
    nb = int(np.sum(f["rcell"] < 0))
    assert nb == sum(patch_faces.values())
    patch, names = cgns.patch_of_faces(m["nodes"], m["patches"], f["fx"],
                                       f["fy"], f["rcell"])
    assert np.all(patch[f["rcell"] < 0] >= 0)
    assert np.all(patch[f["rcell"] >= 0] == -1)
    counts = np.bincount(patch[patch >= 0], minlength=len(names))
    assert dict(zip(names, counts.tolist())) == patch_faces
    used = np.unique(m["cind"]).size
    holes = 1 if "Cylinder" in name or "Box" in name else 0
    assert used - om.n_faces + n_cells == 1 - holes


def test_cylinder_example_pressure_system_solves(oracle):
    """The pressure Laplacian of the cylinder case on its own mesh, with the
    boundary types of Examples/UnstructuredFlowAroundCylinder/case/
    boundaries.info for p (fixed at the outlet, normal gradient elsewhere),
    assembled and solved by the oracle: a nonsingular system whose direct
    solve has a small residual."""
    import scipy.sparse as sp
    m = cgns.read_mesh(_example(
        "UnstructuredFlowAroundCylinder/case/CylinderMesh.cgns"))
    om = oracle.OracleMesh(m["nodes"], m["cptr"], m["cind"])
    f = om.faces()
    patch, names = cgns.patch_of_faces(m["nodes"], m["patches"], f["fx"],
                                       f["fy"], f["rcell"])
    bc = np.ones(om.n_faces, np.int32)
    bc[patch == names.index("Outlet")] = 0
    rng = np.random.default_rng(2)
    rp, ci, v, rhs = om.laplacian(rng.uniform(0.5, 2.0, om.n_faces), bc,
                                  np.zeros(om.n_faces))
    b = rng.standard_normal(om.n_cells)
    x, info = oracle.sparse_lu_solve(rp, ci, v, b)
    A = sp.csr_matrix((v, ci, rp))
    assert info["replaced"] == 0
    assert np.linalg.norm(A @ x - b) / np.linalg.norm(b) < 1e-10


@pytest.mark.parametrize("case", ["UnstructuredFlowAroundCylinder",
                                  "SuddenExpansion", "FlowAroundBox"])
def test_example_case_loads_and_its_pressure_system_solves(oracle, case):
    """A whole example case as Phase reads it: case.info (the grid, the
    pressure equation's backend) and boundaries.info (p's boundary types per
    patch), then p's Laplacian on that grid solved by the oracle's direct
    solve."""
    import scipy.sparse as sp
    from phase_gb300 import caseinfo
    case_dir = os.path.join(REF_EXAMPLES, case)
    if not os.path.isdir(case_dir):
        pytest.skip("the reference's example cases are not present")
    tree = caseinfo.read_info(os.path.join(case_dir, "case", "case.info"))
    bnd = caseinfo.read_info(os.path.join(case_dir, "case", "boundaries.info"))
    assert caseinfo.backend(tree, "pEqn") in ("direct", "iterative")
    m = caseinfo.grid(tree, case_dir)
    om = oracle.OracleMesh(m["nodes"], m["cptr"], m["cind"])
    f = om.faces()
    patch, names = cgns.patch_of_faces(m["nodes"], m["patches"], f["fx"],
                                       f["fy"], f["rcell"])
    bc_type, bc_value = caseinfo.face_bcs(bnd, "p", patch, names)
    rp, ci, v, rhs = om.laplacian(np.ones(om.n_faces), bc_type, bc_value)
    A = sp.csr_matrix((v, ci, rp))
    b = np.random.default_rng(1).standard_normal(om.n_cells)
    if not np.any(bc_type[f["rcell"] < 0] == 0):
        b -= b.mean()  # all-Neumann: a consistent right-hand side
    x, info = oracle.sparse_lu_solve(rp, ci, v, b)
    assert np.linalg.norm(A @ x - b) / np.linalg.norm(b) < 1e-9
    if case == "SuddenExpansion":  # Grid.origin (0.25,0) shifts the nodes
        assert m["nodes"][:, 0].min() >= 0.25 - 1e-12
