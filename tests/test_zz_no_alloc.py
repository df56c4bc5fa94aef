"""fg_matvec_noalloc: the allocation-free matvec entry point.

It serves callers that cannot call cudaMalloc once their set-up is done
(their device memory belongs to another allocator, or their solver loop
must not pay cudaMalloc's implicit synchronisation).  The test calls it
through the C ABI on device vectors the test owns, twice in a row with
different inputs (the shared scratch keeps the previous call's contents),
and checks each result against the allocating entry point fg_matvec with
the matvec tolerance of the other GPU tests (relative 1e-14 in FP64,
1e-5 in FP32).  This file is collected last so that a run stopping at the
first failure has run every other test; it also passes alone.
"""
import ctypes

import numpy as np
import pytest

import oracle as O
from parallel_fem_codes_gb300 import meshgen as G

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module")
def fg():
    from parallel_fem_codes_gb300 import femgpu
    L = femgpu.lib()
    L.fg_matvec_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
    return femgpu


def _noalloc(fg, s, P, precision):
    import torch
    Pd = torch.from_numpy(np.ascontiguousarray(P)).to("cuda")
    Qd = torch.full((s.n + 1,), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    fg.check(fg.lib().fg_matvec_noalloc(s.handle, Pd.data_ptr(), Qd.data_ptr(), precision))
    torch.cuda.ExternalStream(s.stream).synchronize()
    return Qd.cpu().numpy()


def test_matvec_noalloc_matches_oracle(fg):
    """Against the oracle's ebemv (oracle/ebe_gmres.c, a restatement of
    00_CommonFiles/MatrixVector_Operations/EBE/ebemv.c:4-64), independently of
    the library's own matvec."""
    p = G.transport_problem(65, angle_deg=20.0, k=1e-4)
    m = p.mesh
    A, _ = O.build_k_f_supg(p)
    lm = O.fill_lm(m)
    perm, inv, _ = O.permutation_of_lm(m)
    s = fg.System(m)
    s.set_blocks(A)
    rng = np.random.default_rng(5)
    for call in range(2):
        P = rng.standard_normal(m.neq + 1)
        P[-1] = 0.0
        ref = O.ebemv3_perm(lm, A, perm, inv, P)
        for precision, tol in ((64, 1e-14), (32, 1e-5)):
            got = _noalloc(fg, s, P, precision)
            assert rel(got[:-1], ref[:-1]) <= tol, (call, precision)


def test_matvec_noalloc_on_a_csr_system_uses_the_blocks(fg):
    """A system switched to the assembled CSR operator: the allocation-free
    matvec still multiplies by the element blocks, equal to the CSR product
    up to summation order."""
    p = G.transport_problem(33)
    A, _ = O.build_k_f_supg(p)
    s = fg.System(p.mesh)
    s.set_blocks(A)
    s.set_operator(fg.FG_OP_CSR)
    P = np.random.default_rng(9).standard_normal(s.n + 1)
    P[-1] = 0.0
    ref = s.matvec(P, 64)
    for _ in range(2):
        assert rel(_noalloc(fg, s, P, 64)[:-1], ref[:-1]) <= 1e-14


@pytest.mark.parametrize("kind", ["transport", "ndof4"])
def test_matvec_noalloc_matches_matvec(fg, kind):
    if kind == "transport":
        p = G.transport_problem(65)
        A, _ = O.build_k_f_supg(p)
        mesh = p.mesh
    else:
        mesh = G.multi_dof_mesh(17, 4, seed=7)
        A = G.random_blocks(mesh.nel, 12, seed=7)
    s = fg.System(mesh)
    s.set_blocks(A)
    rng = np.random.default_rng(11)
    for call in range(2):
        P = rng.standard_normal(s.n + 1)
        P[-1] = 0.0
        for precision, tol in ((64, 1e-14), (32, 1e-5)):
            ref = s.matvec(P, precision)
            got = _noalloc(fg, s, P, precision)
            assert got[-1] == 0.0
            assert rel(got[:-1], ref[:-1]) <= tol, (call, precision)


def test_matvec_noalloc_rejects_bad_arguments(fg):
    p = G.transport_problem(9)
    s = fg.System(p.mesh)
    A, _ = O.build_k_f_supg(p)
    s.set_blocks(A)
    FG_ERR_ARG = 1
    assert fg.lib().fg_matvec_noalloc(s.handle, None, None, 64) == FG_ERR_ARG
    import torch
    buf = torch.zeros(s.n + 1, dtype=torch.float64, device="cuda")
    assert fg.lib().fg_matvec_noalloc(s.handle, buf.data_ptr(), buf.data_ptr(), 16) == FG_ERR_ARG
