"""Phase case files (INFO format) and the solver triple dumps: parsing,
the solver options and boundary conditions they carry, and the dump round
trip.  No GPU needed."""
import numpy as np
import pytest

from phase_gb300 import caseinfo, meshes, triples, workloads

CASE = """\
; a rising-bubble style case (comments start with a semicolon)
CaseName Bubble

Solver
{
  timeStep 2.5e-5 ; trailing comment
  surfaceTensionModel CELESTE
}

Properties
{
  rho1 998
  g (0,-9.8065)
  label "two words"
}

LinearAlgebra
{
  uEqn
  {
    lib trilinos
    preconditioner diagonal
    tolerance 1e-10
    maxIters 100
  }

  pEqn
  {
    lib gb300
    tolerance 1e-8
    maxIters 500
    preconditioner ilu0
    coarseSpace 1
    coarseWarmIters 0
    precision mixed
  }
  gammaEqn { lib trilinos }
}

Boundaries
{
  p
  {
    *
    {
      type normal_gradient
      value 0
    }
    y+
    {
      type fixed
      value 0
    }
  }
  u
  {
    *
    {
      type fixed
      value (0,0)
    }
  }
}

Repeated 1
Repeated 2
"""


def test_parse_info_tree():
    t = caseinfo.parse_info(CASE)
    assert t.get("CaseName") == "Bubble"
    assert t.get("Solver.timeStep") == "2.5e-5"
    assert t.get("Properties.g") == "(0,-9.8065)"
    assert t.get("Properties.label") == "two words"
    assert t.get("LinearAlgebra.gammaEqn.lib") == "trilinos"
    assert t.get("Missing.key", "dflt") == "dflt"
    assert [k for k in t.keys() if k == "Repeated"] == ["Repeated", "Repeated"]
    assert t.keys()[:2] == ["CaseName", "Solver"]


@pytest.mark.parametrize("bad", ["a {", "}", "{", "a b c"])
def test_parse_info_rejects_malformed(bad):
    with pytest.raises(ValueError):
        caseinfo.parse_info(bad)


def test_solver_options():
    t = caseinfo.parse_info(CASE)
    assert caseinfo.solver_options(t, "pEqn") == dict(
        tolerance=1e-8, max_iters=500, krylov=0, precond=2, coarse=1,
        coarse_warm=0, precision=1)
    # "preconditioner diagonal" is ignored as the Belos backend ignores it
    # without an ifpackParamFile (TrilinosBelosSparseMatrixSolver.cpp:63-67):
    # Schwarz over RILUK blocks
    assert caseinfo.solver_options(t, "uEqn") == dict(
        tolerance=1e-10, max_iters=100, krylov=0, precond=2)
    with pytest.raises(KeyError):
        caseinfo.solver_options(t, "nope")


def _opts(body):
    return caseinfo.solver_options(
        caseinfo.parse_info("LinearAlgebra\n{\n pEqn\n {\n" + body +
                            "\n }\n}\n"), "pEqn")


def test_solver_options_follow_the_belos_keys():
    assert _opts("solver TFQMR")["krylov"] == 1
    assert _opts("solver gmres\nnumBlocks 40") == dict(krylov=2, krylov_dim=40,
                                                       precond=2)
    assert _opts("innerPreconditioner RELAXATION")["precond"] == 1
    assert _opts("iluFill 1")["ilu_fill"] == 1
    assert _opts("preconditioner none")["precond"] == 0


@pytest.mark.parametrize("body", [
    "solver CG", "innerPreconditioner ILUT", "innerPreconditioner CHEBYSHEV",
    "iluFill 0.5", "schwarzOverlap 1", "schwarzCombineMode ZERO",
    "schwarzIters 2", "belosParamFile belos.xml", "ifpackParamFile p.xml",
    "precision fp16"])
def test_unbuilt_solver_options_raise(body):
    """A value the library does not build raises instead of being replaced
    by another method."""
    with pytest.raises(ValueError):
        _opts(body)


def test_boundaries_give_the_rising_bubble_bcs(oracle):
    t = caseinfo.parse_info(CASE)
    bcs = caseinfo.boundary_conditions(t, "p", caseinfo.RECT_PATCHES)
    assert bcs["y+"] == (0, "0") and bcs["x-"] == (1, "0")
    nx = 12
    nodes, cptr, cind = meshes.rectilinear(nx, nx, workloads.RB_WIDTH,
                                           workloads.RB_HEIGHT)
    om = oracle.OracleMesh(nodes, cptr, cind)
    f = om.faces()
    bt, bv, patch = workloads.rising_bubble_bcs(f, nx, nx)
    t2, v2 = caseinfo.rect_face_bcs(t, "p", patch)
    assert np.array_equal(t2, bt) and np.array_equal(v2, bv)


def test_triples_round_trip(tmp_path, oracle):
    nodes, cptr, cind = meshes.rectilinear(9, 7, 1.0, 1.0)
    om = oracle.OracleMesh(nodes, cptr, cind)
    f = om.faces()
    bc = np.where(f["rcell"] < 0, 0, 1).astype(np.int32)
    rng = np.random.default_rng(1)
    rp, ci, v, rhs = om.laplacian(rng.uniform(1, 2, om.n_faces), bc,
                                  np.zeros(om.n_faces),
                                  rng.standard_normal((om.n_faces, 2)))
    w = triples.TripleWriter(str(tmp_path / "d"), rp, ci, case="test")
    for t in (3, 4):
        w.write(t, v * t, -rhs, rng.standard_normal(om.n_cells))
    r = triples.TripleReader(str(tmp_path / "d"))
    assert r.steps == [3, 4] and r.meta["case"] == "test" and r.n == om.n_cells
    assert np.array_equal(r.row_ptr, rp) and np.array_equal(r.col_ind, ci)
    vals, b, x = r.read(4)
    assert np.array_equal(vals, v * 4) and np.array_equal(b, -rhs)
    assert len(list(r)) == 2
    with pytest.raises(ValueError):
        triples.TripleWriter(str(tmp_path / "e"), rp, np.where(ci == 0, -1, ci))


def test_backend_of_the_lib_key():
    """LinearAlgebra.<eqn>.lib selects the backend as Phase's factory
    names them (SparseMatrixSolverFactory.cpp:26-40)."""
    def case(lib):
        return caseinfo.parse_info(
            "LinearAlgebra\n{\n  pEqn\n  {\n    lib %s\n  }\n}\n" % lib)
    assert caseinfo.backend(case("eigen")) == "direct"
    assert caseinfo.backend(case("Eigen3")) == "direct"
    assert caseinfo.backend(case("amesos2")) == "direct"
    assert caseinfo.backend(case("belos")) == "iterative"
    assert caseinfo.backend(case("gb300")) == "iterative"
    with pytest.raises(ValueError, match="muelu"):
        caseinfo.backend(case("muelu"))
    with pytest.raises(ValueError, match="bad solver type"):
        caseinfo.backend(case("petsc"))
