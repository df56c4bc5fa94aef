"""The library's readers of the reference's mesh files (fg_mesh_read,
fg_mesh_read_rank; host only).  The global-format fixtures were written by
the reference's own structured mesh generator (tests/golden/
make_mesh_golden.py); they must read back as the node order, connectivity
and boundary marks that meshgen reproduces from meshGenerator.c."""
import os

import numpy as np
import pytest

from parallel_fem_codes_gb300 import meshgen as G

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def fg():
    from parallel_fem_codes_gb300 import femgpu
    femgpu.lib()
    return femgpu


def test_reads_generator_output_teste(fg):
    m = fg.read_mesh(os.path.join(HERE, "golden", "mesh_TESTE_8x8.dat"), ndof=1)
    ref = G.transport_problem(9, upmode=1).mesh            # every boundary node prescribed (TESTE)
    assert m.nnodes == 81 and m.nel == 128
    assert np.allclose(m.x, ref.x, atol=1e-13) and np.allclose(m.y, ref.y, atol=1e-13)
    assert np.array_equal(m.ien, ref.ien)
    assert np.array_equal(m.type, ref.type)
    assert m.neq == ref.neq == 49
    free = m.type == 1
    assert np.array_equal(m.invp[free], np.arange(m.neq)) and np.all(m.invp[~free] == -1)


def test_reads_generator_output_obliquo(fg):
    m = fg.read_mesh(os.path.join(HERE, "golden", "mesh_OBLIQUO_6x6.dat"), ndof=4)
    ref = G.obliquo_problem(7).mesh
    assert m.nnodes == 49 and m.nel == 72 and m.ndof == 4
    assert np.array_equal(m.ien, ref.ien)
    assert np.array_equal(m.type, ref.type)
    assert m.neq == ref.neq


def test_rank_file_round_trip(fg, tmp_path):
    ref = G.transport_problem(17, angle_deg=30.0).mesh
    # a numbering other than node order, as the partitioner's reordering gives
    perm = np.random.default_rng(0).permutation(ref.neq)
    invp = ref.invp.copy()
    invp[invp >= 0] = perm[invp[invp >= 0]]
    mesh = G.Mesh(x=ref.x, y=ref.y, ien=ref.ien, ndof=1, type=ref.type, invp=invp, neq=ref.neq)
    path = str(tmp_path / "RANK_00_SYNTH.dat")
    G.write_rank_file(mesh, path)
    m = fg.read_mesh(path, ndof=1, rank_file=True)
    assert np.array_equal(m.invp, invp) and np.array_equal(m.type, ref.type)
    assert np.array_equal(m.ien, ref.ien) and np.allclose(m.x, ref.x, atol=1e-13)


def test_rank_file_of_another_rank_is_refused(fg, tmp_path):
    path = str(tmp_path / "RANK_01.dat")
    with open(path, "w") as f:
        f.write("3\n0 0 1 1 0\n1 0 2 1 1\n0 1 0\n1\n0 1 2\n")
    with pytest.raises(fg.FemGpuError):
        fg.read_mesh(path, rank_file=True)
    with pytest.raises(fg.FemGpuError):
        fg.read_mesh(str(tmp_path / "missing.dat"))


def _vtu_arrays(path):
    import xml.etree.ElementTree as ET
    piece = ET.parse(path).getroot().find("UnstructuredGrid/Piece")
    pd = {d.get("Name"): np.array(d.text.split(), dtype=float) for d in piece.find("PointData")}
    pts = np.array(piece.find("Points/DataArray").text.split(), dtype=float).reshape(-1, 3)
    cells = {d.get("Name"): np.array(d.text.split(), dtype=int) for d in piece.find("Cells")}
    return piece, pd, pts, cells


def test_vtu_transport_output(fg, tmp_path):
    p = G.transport_problem(9)
    m = p.mesh
    u = np.linspace(0.1, 0.9, m.neq)
    path = str(tmp_path / "out.vtu")
    fg.write_transport_vtu(path, p, u)
    piece, pd, pts, cells = _vtu_arrays(path)
    assert int(piece.get("NumberOfPoints")) == m.nnodes and int(piece.get("NumberOfCells")) == m.nel
    # free nodes from u through invP_id, prescribed ones from upresc (Paraview_Output.c:30-35)
    want = np.array([u[m.invp[i]] if m.type[i] > 0 else p.upresc[i] for i in range(m.nnodes)])
    assert np.allclose(pd["solucao"], want, atol=1e-12)
    assert np.allclose(pts[:, 0], m.x) and np.allclose(pts[:, 1], m.y) and np.allclose(pts[:, 2], want)
    assert np.array_equal(cells["connectivity"].reshape(-1, 3), m.ien)
    assert np.array_equal(cells["offsets"], 3 * np.arange(1, m.nel + 1))
    assert np.all(cells["types"] == 5)
    # the reference's line layout: one value per line, %.12f
    lines = open(path).read().splitlines()
    assert lines[0] == '<VTKFile type="UnstructuredGrid" version="0.1" byte_order="BigEndian">'
    assert lines[5] == "\t\t\t\t   %.12f" % want[0]


def test_vtu_euler_ns_output(fg, tmp_path):
    ep = G.obliquo_problem(9)
    m = ep.mesh
    U = ep.initial_state()
    fg.write_euler_vtu(str(tmp_path / "e.vtu"), ep, U)
    _, pd, pts, _ = _vtu_arrays(str(tmp_path / "e.vtu"))
    assert list(pd) == ["Density", "Temperature", "Pressure"]
    V = fg.node_values(m, U, ep.upresc)
    aux = V[:, 3] - (V[:, 1] ** 2 + V[:, 2] ** 2) / (2 * V[:, 0])
    assert np.allclose(pd["Density"], V[:, 0], atol=1e-12)
    assert np.allclose(pd["Pressure"], (ep.gamma - 1) * aux, atol=1e-11)
    assert np.allclose(pd["Temperature"], aux / (V[:, 0] * 716.5), atol=1e-12)
    assert np.all(pts[:, 2] == 0)
    npb = G.cavity_problem(7)
    U = np.arange(npb.mesh.neq, dtype=float) * 1e-3
    fg.write_ns_vtu(str(tmp_path / "n.vtu"), npb, U)
    _, pd, _, _ = _vtu_arrays(str(tmp_path / "n.vtu"))
    V = fg.node_values(npb.mesh, U, npb.upresc)
    vel = pd["Velocity"].reshape(-1, 3)
    assert np.allclose(vel[:, :2], V[:, :2], atol=1e-12) and np.all(vel[:, 2] == 0)
    assert np.allclose(pd["Pressure"], V[:, 2], atol=1e-12)


def test_vtu_rejects_bad_input(fg, tmp_path):
    p = G.transport_problem(5)
    with pytest.raises(Exception):
        fg.write_vtu(str(tmp_path / "x.vtu"), p.mesh, {"a": np.zeros(3)})
    bad = G.Mesh(p.mesh.x, p.mesh.y, p.mesh.ien + 1000, 1, p.mesh.type, p.mesh.invp, p.mesh.neq)
    with pytest.raises(Exception):
        fg.write_vtu(str(tmp_path / "x.vtu"), bad, {"a": np.zeros(p.mesh.nnodes)})
