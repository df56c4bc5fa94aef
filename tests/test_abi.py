"""The C ABI on the CPU: the library loads, exports every function that
include/femgpu.h declares, and its host-only set-up (Fill_LM, local RCM,
colouring) matches the oracle and the golden fixtures.  No GPU is used."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

import oracle as O
from parallel_fem_codes_gb300 import meshgen as G

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    out = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        txt = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        out |= set(re.findall(r"\b(fg_[a-z0-9_]+)\s*\(", txt))
    return out


def test_library_exports_every_declared_symbol(femgpu):
    lib = ctypes.CDLL(femgpu.library_path())
    syms = declared_symbols()
    assert len(syms) >= 25
    missing = [s for s in sorted(syms) if not hasattr(lib, s)]
    assert not missing, missing


def test_version_and_error_text(femgpu):
    assert femgpu.lib().fg_version() >= 10000
    assert isinstance(femgpu.lib().fg_last_error(), bytes)


@pytest.mark.parametrize("n", [5, 17, 40, 129])
def test_host_setup_matches_oracle(femgpu, n):
    p = G.transport_problem(n, angle_deg=17.0 * n)
    a = femgpu.mesh_analyze(p.mesh)
    perm, inv, band = O.permutation_of_lm(p.mesh)
    assert np.array_equal(a["lm"], O.fill_lm(p.mesh))
    assert np.array_equal(a["perm"], perm) and np.array_equal(a["invperm"], inv)
    assert [a["info"]["bandwidth_before"], a["info"]["bandwidth_after"]] == list(band)


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "sst_*.npz"))))
def test_host_setup_matches_golden(femgpu, path):
    g = dict(np.load(path))
    m = G.Mesh(g["x"], g["y"], g["ien"], 1, g["type"], g["invp"], int(g["neq"]))
    a = femgpu.mesh_analyze(m)
    assert np.array_equal(a["lm"], g["lm"])
    assert np.array_equal(a["perm"], g["perm"]) and np.array_equal(a["invperm"], g["invperm"])
    assert a["info"]["nnz"] == int(g["nnz"])


@pytest.mark.parametrize("ndof,n", [(1, 33), (3, 17), (4, 17)])
def test_colouring_valid_and_deterministic(femgpu, ndof, n):
    m = G.transport_problem(n).mesh if ndof == 1 else G.multi_dof_mesh(n, ndof, jitter=0.2)
    a = femgpu.mesh_analyze(m)
    b = femgpu.mesh_analyze(m)
    assert np.array_equal(a["colour"], b["colour"])
    lm = a["lm"]
    for c in range(a["info"]["ncolours"]):
        idx = lm[a["colour"] == c].reshape(-1)
        idx = idx[idx != m.neq]
        assert len(idx) == len(np.unique(idx)), f"colour {c} shares a dof"
    # only elements without a free dof are uncoloured
    free = (lm != m.neq).any(axis=1)
    assert np.all((a["colour"] >= 0) == free)
    assert a["info"]["ncolours"] <= 12


def test_setup_rejects_bad_mesh(femgpu):
    p = G.transport_problem(5)
    bad = p.mesh.ien.copy()
    bad[0, 0] = 10 ** 6
    m = G.Mesh(p.mesh.x, p.mesh.y, bad, 1, p.mesh.type, p.mesh.invp, p.mesh.neq)
    with pytest.raises(femgpu.FemGpuError):
        femgpu.mesh_analyze(m)
