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
