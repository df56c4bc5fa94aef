"""The steady Navier-Stokes oracle (oracle/ns.c) against the golden fixtures
generated from the reference's own C (04_SS_NavierStokes_Equations driver:
Fill_LM, Build_K_F_SUPG_PSPG, BlockDiagDOF3_precond_EBE_setup, ebemvNDOF3,
Process), and against the reference build itself where it is present.
Everything is bit-exact, including the Picard loop's solution and GMRES
iteration count."""
import glob
import os

import numpy as np
import pytest

import oracle as O
from parallel_fem_codes_gb300 import meshgen as G

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "ns_*.npz")))


def _problem(g):
    m = G.Mesh(g["x"], g["y"], g["ien"], 3, g["type"], g["invp"], int(g["neq"]))
    return G.ns_problem(m, float(g["reynolds"]), g["coef"], bool(g["lid"]))


@pytest.fixture(scope="module", params=GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def case(request, oracle_lib):
    g = dict(np.load(request.param))
    return g, _problem(g)


def test_golden_present():
    assert len(GOLDEN) >= 2


def test_fill_lm(case):
    g, p = case
    assert np.array_equal(O.fill_lm(p.mesh).reshape(-1), g["lm"].reshape(-1))


def test_build_bit_exact(case):
    g, p = case
    A, F = O.build_ns(p, g["u"])
    assert np.array_equal(A, g["A"])
    assert np.array_equal(F, g["F"])


def test_blockdiag_dof3_bit_exact(case):
    g, p = case
    bd, ibd, Id, Fp = O.blockdiag_setup(p.mesh, g["A"], g["F"])
    assert np.array_equal(ibd, g["inv"])
    assert np.array_equal(Fp, g["Fp"])


def test_ebemv_ndof3_bit_exact(case):
    g, p = case
    Q = O.ebemv(O.fill_lm(p.mesh), g["A"], p.mesh.neq, g["P"])
    assert np.array_equal(Q, g["Q"])


def test_process_bit_exact(case):
    g, p = case
    if "U" not in g:
        pytest.skip("fixture without a Process run")
    u, nl, its, last = O.ns_process(p, 1e-10, 1e-6, 30, 1000, 30)
    assert its == int(g["process_its"])
    assert np.array_equal(u, g["U"])
    assert last <= 1e-6


def test_cavity_layout():
    """Cavity marks: velocity prescribed on the boundary, lid u = 1, one
    pressure pin at the centre, node-major numbering of the free dofs."""
    p = G.cavity_problem(9, jitter=0.2)
    m = p.mesh
    t = m.type.reshape(-1, 3)
    bnd = G.boundary_mask(m.x, m.y)
    assert np.all(t[bnd, :2] == 0) and np.all(t[~bnd, :2] == 1)
    assert int((t[:, 2] == 0).sum()) == 1
    up = p.upresc.reshape(-1, 3)
    assert np.all(up[np.abs(m.y - 1.0) <= 1e-15, 0] == 1.0)
    assert np.all(up[m.y < 1.0 - 1e-12, 0] == 0.0)
    assert m.neq == 3 * m.nnodes - 2 * int(bnd.sum()) - 1
    assert np.array_equal(m.invp[m.type != 0], np.arange(m.neq))


@pytest.mark.skipif(O.ref_ns() is None, reason="reference build absent (oracle/_ref)")
@pytest.mark.parametrize("n,jitter,re", [(17, 0.2, 1000.0), (11, 0.0, 10.0)])
def test_against_reference_build(n, jitter, re):
    p = G.cavity_problem(n, reynolds=re, jitter=jitter)
    u = np.random.default_rng(n).standard_normal(p.mesh.neq)
    A, F = O.build_ns(p, u)
    Ar, Fr = O.ref_ns_build(p, u)
    assert np.array_equal(A, Ar) and np.array_equal(F, Fr)
    inv, Fp = O.ref_ns_blockdiag(p.mesh, A, F)
    bd, ibd, Id, Fq = O.blockdiag_setup(p.mesh, A, F)
    assert np.array_equal(ibd, inv) and np.array_equal(Fq, Fp)


VMS = os.path.join(os.path.dirname(__file__), "golden", "vms_ns.npz")


@pytest.mark.parametrize("name", ["ns_9_cavity", "ns_9_affine"])
def test_vms_dcdd_bit_exact(name, oracle_lib):
    """Build_K_F_VMS_DCDD (StabilizationForm "VMS-DCDD") and, for the cavity,
    its Picard loop: the restatement against the reference's own build."""
    g = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", name + ".npz")))
    p = _problem(g)
    v = np.load(VMS)
    A, F = O.build_ns(p, v[name + "_u"], form=1)
    assert np.array_equal(A, v[name + "_A"])
    assert np.array_equal(F, v[name + "_F"])
    if name + "_U" in v:
        U, nl, its, last = O.ns_process(p, 1e-10, 1e-3, 30, 1000, 20, form=1)
        assert its == int(v[name + "_its"])
        assert np.array_equal(U, v[name + "_U"])


def test_vms_dcdd_against_reference_build(oracle_lib):
    if O.ref_ns() is None:
        pytest.skip("reference build (oracle/_ref) not present")
    p = G.cavity_problem(13, reynolds=1000.0, jitter=0.2, seed=5)
    u = np.random.default_rng(13).standard_normal(p.mesh.neq)
    A0, F0 = O.ref_ns_build(p, u, form=1)
    A1, F1 = O.build_ns(p, u, form=1)
    assert np.array_equal(A0, A1) and np.array_equal(F0, F1)
