"""Synthetic meshes and problems for the solve path (seeded, numpy only).

The reference reads meshes written by Mesh_Generator/Structured_Mesh/
meshGenerator.c (node order row by row, two triangles per quad, see
meshGenerator.c:113-177) and partitioned by Parallel_Preprocess.  The
single-GPU path needs no partitioning: a mesh here is one domain whose free
dofs are numbered in node order (node-major, dof-minor for NDOF > 1), which
is what Parallel_Preprocess produces for one rank before the local RCM of
Permutation_of_LM.c.

All problems are synthetic and seeded; no dataset is involved.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np


@dataclasses.dataclass
class Mesh:
    x: np.ndarray          # float64[nnodes]
    y: np.ndarray          # float64[nnodes]
    ien: np.ndarray        # int32[nel, 3]  (Element[e].Vertex)
    ndof: int
    type: np.ndarray       # int32[nnodes*ndof]  0 = Dirichlet, 1 = free (Node.Type)
    invp: np.ndarray       # int32[nnodes*ndof]  equation of a free dof, -1 otherwise (Node.invP_id)
    neq: int

    @property
    def nnodes(self) -> int:
        return int(self.x.shape[0])

    @property
    def nel(self) -> int:
        return int(self.ien.shape[0])


def structured_mesh(M: int, N: int, x0=0.0, y0=0.0, x1=1.0, y1=1.0, left=False):
    """Node coordinates and connectivity of an M x N structured rectangle
    (meshGenerator.c:113-177, "right" or "left" diagonal)."""
    nx = M + 1
    i = np.arange(M + 1, dtype=np.float64)
    j = np.arange(N + 1, dtype=np.float64)
    hx = (x1 - x0) / M
    hy = (y1 - y0) / N
    X = np.tile(x0 + i * hx, N + 1)
    Y = np.repeat(y0 + j * hy, M + 1)
    jj, ii = np.meshgrid(np.arange(N), np.arange(M), indexing="ij")
    a = (jj * nx + ii).reshape(-1).astype(np.int64)
    ien = np.empty((2 * M * N, 3), dtype=np.int32)
    if not left:
        ien[0::2] = np.stack([a, a + 1, a + nx + 1], axis=1)
        ien[1::2] = np.stack([a, a + nx + 1, a + nx], axis=1)
    else:
        ien[0::2] = np.stack([a, a + 1, a + nx], axis=1)
        ien[1::2] = np.stack([a + 1, a + nx + 1, a + nx], axis=1)
    return X, Y, ien


def number_dofs(type_: np.ndarray) -> tuple[np.ndarray, int]:
    """Sequential equation numbers for the free dofs (type != 0)."""
    free = type_ != 0
    invp = np.full(type_.shape, -1, dtype=np.int32)
    invp[free] = np.arange(int(free.sum()), dtype=np.int32)
    return invp, int(free.sum())


def boundary_mask(x, y, tol=1e-12):
    x0, x1, y0, y1 = x.min(), x.max(), y.min(), y.max()
    return (np.abs(x - x0) < tol) | (np.abs(x - x1) < tol) | (np.abs(y - y0) < tol) | (np.abs(y - y1) < tol)


@dataclasses.dataclass
class TransportProblem:
    """Steady SUPG/CAU convection-diffusion-reaction data (the FemFunctions
    callbacks Condutivity, Reaction, Velocity, Font, upresc of
    01_SS_Transport_Equation/2D/01_CommonFiles/SSTranspEquation.h:140-146),
    with a constant velocity field, conductivity, reaction and source."""
    mesh: Mesh
    k: float
    gamma: float
    beta: tuple[float, float]
    f: float
    upresc: np.ndarray     # float64[nnodes], Dirichlet value (read where type == 0)
    upmode: int = 0        # 0: 1 on inflow edges x=xmin, y=ymin, else 0;  1: constant
    upval: float = 0.0
    cau: int = 1           # ShockCapture: 0 none, 1 "CAU", 2 "CAUDD" (DD form only), 3 "YZBeta"
    form: int = 0          # StabilizationForm: 0 "SUPG", 1 "DD"
    h_shock: int = 0       # h_Shock: 0 "2sqrtArea", 1 "Option1", 2 "Option2"


def transport_problem(n_nodes_side: int, angle_deg=30.0, k=1e-6, gamma=0.0, f=0.0,
                      left=False, upmode=0, upval=1.0, cau=True) -> TransportProblem:
    """Unit square with n x n nodes, every boundary node Dirichlet.
    upmode 0: u = 1 on x = 0 and y = 0, u = 0 on the rest of the boundary
    (the steady transport workload: 129 x 129 nodes, beta = (cos 30, sin 30),
    k = 1e-6).  upmode 1: u = upval on the whole boundary (the TESTE problem of
    01_SS_Transport_Equation/2D/TESTE, exact solution u = upval when f = 0,
    gamma = 0)."""
    M = n_nodes_side - 1
    X, Y, ien = structured_mesh(M, M, left=left)
    bnd = boundary_mask(X, Y)
    type_ = np.where(bnd, 0, 1).astype(np.int32)
    invp, neq = number_dofs(type_)
    mesh = Mesh(X, Y, ien, 1, type_, invp, neq)
    if upmode == 0:
        up = np.where((X <= X.min() + 1e-12) | (Y <= Y.min() + 1e-12), 1.0, 0.0)
    else:
        up = np.full_like(X, upval)
    a = math.radians(angle_deg)
    return TransportProblem(mesh, float(k), float(gamma), (math.cos(a), math.sin(a)),
                            float(f), up.astype(np.float64), upmode, float(upval), cau)


def batch_transport_params(count=256, seed=4, nmin=33, nmax=513):
    """Per-instance parameters of the batched transport workload: lists of
    nodes per side N (uniform in [nmin, nmax]), velocity angle in degrees
    (uniform in [0, 360)) and conductivity (log-uniform in [1e-8, 1e-2]),
    drawn from numpy PCG64 with the given seed."""
    rng = np.random.Generator(np.random.PCG64(seed))
    ns = rng.integers(nmin, nmax + 1, size=count)
    angles = rng.uniform(0.0, 360.0, size=count)
    ks = 10.0 ** rng.uniform(-8.0, -2.0, size=count)
    return [int(n) for n in ns], [float(a) for a in angles], [float(k) for k in ks]


def batch_transport_sizes(count=256, seed=4, nmin=33, nmax=513):
    """(elements, free dofs) of every instance of the batched workload without
    building its meshes: 2 (N-1)^2 triangles, (N-2)^2 interior nodes."""
    ns, _, _ = batch_transport_params(count, seed, nmin, nmax)
    return [2 * (n - 1) ** 2 for n in ns], [(n - 2) ** 2 for n in ns]


def batch_transport_problem(i, count=256, seed=4, nmin=33, nmax=513, cau=True):
    """Instance i of the batched transport workload (only its own mesh is built)."""
    ns, angles, ks = batch_transport_params(count, seed, nmin, nmax)
    return transport_problem(ns[i], angles[i], ks[i], cau=cau)


def batch_transport_problems(count=256, seed=4, nmin=33, nmax=513, cau=True):
    """The batched transport workload: count independent steady SUPG problems,
    mesh N x N nodes with N uniform in [nmin, nmax], velocity angle uniform in
    [0, 360), conductivity log-uniform in [1e-8, 1e-2] (numpy PCG64, seeded)."""
    ns, angles, ks = batch_transport_params(count, seed, nmin, nmax)
    return [transport_problem(n, a, kk, cau=cau) for n, a, kk in zip(ns, angles, ks)]


def multi_dof_mesh(n_nodes_side: int, ndof: int, seed: int = 0, dirichlet=None, jitter: float = 0.0):
    """Structured unit-square mesh with ndof dofs per node (the Euler layout
    (rho, rho u, rho v, E) for ndof = 4 and the Navier-Stokes layout (u, v, p)
    for ndof = 3).  dirichlet(k) -> bool mask over nodes for dof k; default:
    every boundary dof Dirichlet except the last dof of each node."""
    M = n_nodes_side - 1
    X, Y, ien = structured_mesh(M, M)
    rng = np.random.Generator(np.random.PCG64(seed))
    bnd = boundary_mask(X, Y)
    if jitter:
        h = 1.0 / M
        X = X + np.where(bnd, 0.0, rng.uniform(-jitter * h, jitter * h, X.shape))
        Y = Y + np.where(bnd, 0.0, rng.uniform(-jitter * h, jitter * h, Y.shape))
    type_ = np.ones((X.shape[0], ndof), dtype=np.int32)
    for k in range(ndof):
        mask = dirichlet(k, X, Y, bnd) if dirichlet is not None else (bnd if k < ndof - 1 else np.zeros_like(bnd))
        type_[mask, k] = 0
    type_ = type_.reshape(-1)
    invp, neq = number_dofs(type_)
    return Mesh(X, Y, ien, ndof, type_, invp, neq)


def random_blocks(nel: int, S: int, seed: int = 0, dominance: float = 4.0):
    """Random nonsymmetric element blocks with a dominant diagonal (float64[nel, S*S])."""
    rng = np.random.Generator(np.random.PCG64(seed))
    A = rng.uniform(-1.0, 1.0, size=(nel, S, S))
    A[:, np.arange(S), np.arange(S)] += dominance
    return A.reshape(nel, S * S)


@dataclasses.dataclass
class NSProblem:
    """Steady incompressible Navier-Stokes data (the FemFunctions callbacks
    v1presc, v2presc, ppresc, f1ext, f2ext of
    04_SS_NavierStokes_Equations/2D/01_CommonFiles/SSNavierStokesEquations.h:153-157)
    evaluated at the nodes.  Each field is the affine function
    coef[k, 0] + coef[k, 1] x + coef[k, 2] y (k: v1, v2, p, f1, f2); with
    lid = True, v1 is the lid-driven-cavity rule of CAVITY_v1presc.c
    (1 where |y - 1| <= 1e-15, else 0)."""
    mesh: Mesh
    reynolds: float
    coef: np.ndarray       # float64[5, 3]
    lid: bool
    upresc: np.ndarray     # float64[nnodes*3]  prescribed u, v, p (read where type == 0)
    f1: np.ndarray         # float64[nnodes]
    f2: np.ndarray         # float64[nnodes]


def _ns_fields(mesh: Mesh, coef: np.ndarray, lid: bool):
    x, y = mesh.x, mesh.y
    val = [coef[k, 0] + coef[k, 1] * x + coef[k, 2] * y for k in range(5)]
    if lid:
        val[0] = np.where(np.abs(y - 1.0) <= 1e-15, 1.0, 0.0)
    up = np.stack(val[:3], axis=1).reshape(-1).astype(np.float64)
    return up, val[3].astype(np.float64), val[4].astype(np.float64)


def ns_problem(mesh: Mesh, reynolds: float, coef=None, lid=False) -> NSProblem:
    coef = np.zeros((5, 3)) if coef is None else np.asarray(coef, dtype=np.float64).reshape(5, 3)
    up, f1, f2 = _ns_fields(mesh, coef, lid)
    return NSProblem(mesh, float(reynolds), coef, bool(lid), up, f1, f2)


def cavity_problem(n_nodes_side: int, reynolds=1000.0, jitter=0.0, seed=3) -> NSProblem:
    """Lid-driven cavity on the unit square with n x n nodes (the CAVITY set-up:
    marks of Mesh_Generator/Structured_Mesh/meshGenerator.c:333-343, velocity
    prescribed on the whole boundary, u = 1 on the lid y = 1, pressure pinned at
    the centre node; n must be odd so that the centre is a node).  Interior
    nodes other than the centre are moved uniformly by up to jitter*h in x and
    y (numpy PCG64, seeded)."""
    if n_nodes_side % 2 == 0:
        raise ValueError("the cavity needs an odd number of nodes per side (pressure pin at the centre)")
    M = n_nodes_side - 1
    X, Y, ien = structured_mesh(M, M)
    bnd = boundary_mask(X, Y)
    centre = (np.abs(X - 0.5) <= 1e-15) & (np.abs(Y - 0.5) <= 1e-15)
    if jitter:
        rng = np.random.Generator(np.random.PCG64(seed))
        h = 1.0 / M
        keep = bnd | centre
        dx = rng.uniform(-jitter * h, jitter * h, X.shape)
        dy = rng.uniform(-jitter * h, jitter * h, Y.shape)
        X = X + np.where(keep, 0.0, dx)
        Y = Y + np.where(keep, 0.0, dy)
    type_ = np.ones((X.shape[0], 3), dtype=np.int32)
    type_[bnd, 0] = 0
    type_[bnd, 1] = 0
    type_[centre, 2] = 0
    type_ = type_.reshape(-1)
    invp, neq = number_dofs(type_)
    mesh = Mesh(X, Y, ien, 3, type_, invp, neq)
    return ns_problem(mesh, reynolds, lid=True)


@dataclasses.dataclass
class EulerProblem:
    """Compressible Euler data in conservative variables (rho, rho u, rho v,
    rho E): the FemFunctions callbacks gamma, rhopresc, v1presc, v2presc,
    epresc and InitialSolution of
    03_Euler_Equations/2D/01_CommonFiles/EulerEquations.h:171-177 and the
    Parameters the SUPG build reads.  Each prescribed field k is
    coef[k, 0] + coef[k, 1] x + coef[k, 2] y; wall = True adds the OBLIQUO
    wall rule for v2 (0 where |y| <= 1e-15 and x > 0,
    OBLIQUO/OBLIQUO_v2presc.c).  init[k] is the initial value of every free
    dof k (OBLIQUO_InitialSolution.c)."""
    mesh: Mesh
    gamma: float
    mach: float
    dimensionless: bool
    tolerance: float       # StabilizationTolerance
    alpha: float
    dt: float
    coef: np.ndarray       # float64[4, 3]
    wall: bool
    init: np.ndarray       # float64[4]
    upresc: np.ndarray     # float64[nnodes*4]

    def initial_state(self) -> np.ndarray:
        """Free-dof vector of the initial solution (length neq)."""
        m = self.mesh
        u = np.zeros(m.neq)
        t = m.type.reshape(-1, 4)
        ip = m.invp.reshape(-1, 4)
        for k in range(4):
            free = t[:, k] != 0
            u[ip[free, k]] = self.init[k]
        return u

    def params(self) -> np.ndarray:
        return np.array([self.gamma, self.mach, 1.0 if self.dimensionless else 0.0, self.tolerance,
                         self.alpha, self.dt], dtype=np.float64)


def _euler_presc(mesh: Mesh, coef: np.ndarray, wall: bool) -> np.ndarray:
    x, y = mesh.x, mesh.y
    val = [coef[k, 0] + coef[k, 1] * x + coef[k, 2] * y for k in range(4)]
    if wall:
        val[2] = np.where((np.abs(y) <= 1e-15) & (np.abs(x) > 0), 0.0, val[2])
    return np.stack(val, axis=1).reshape(-1).astype(np.float64)


def euler_problem(mesh: Mesh, gamma=1.4, mach=2.0, dimensionless=True, tolerance=1e-8, alpha=0.5, dt=1e-3,
                  coef=None, wall=False, init=(1.0, 0.0, 0.0, 1.0)) -> EulerProblem:
    coef = np.zeros((4, 3)) if coef is None else np.asarray(coef, dtype=np.float64).reshape(4, 3)
    return EulerProblem(mesh, float(gamma), float(mach), bool(dimensionless), float(tolerance), float(alpha),
                        float(dt), coef, bool(wall), np.asarray(init, dtype=np.float64),
                        _euler_presc(mesh, coef, wall))


def euler_dt(mesh: Mesh, gamma: float, state, cfl=0.5) -> float:
    """cfl * min_e h_e / (|v| + c) for the uniform state (rho, rho u, rho v,
    rho E), with h_e = sqrt(2 Area_e) and the sound speed
    c = sqrt(gamma (gamma - 1) (E - |v|^2 / 2)) as Build_M_K_F_SUPG.c:256-259
    computes them."""
    rho, mu, mv, E = state
    v1, v2 = mu / rho, mv / rho
    v = math.hypot(v1, v2)
    c = math.sqrt(gamma * (gamma - 1.0) * (E / rho - 0.5 * (v1 * v1 + v2 * v2)))
    x, y, ien = mesh.x, mesh.y, mesh.ien
    x1, x2, x3 = x[ien[:, 0]], x[ien[:, 1]], x[ien[:, 2]]
    y1, y2, y3 = y[ien[:, 0]], y[ien[:, 1]], y[ien[:, 2]]
    two_a = np.abs((x2 - x1) * (y3 - y1) - (x1 - x3) * (y1 - y2))
    return float(cfl * np.sqrt(two_a).min() / (v + c))


def obliquo_problem(n_nodes_side: int, mach=2.0, dimensionless=True, alpha=0.5, tolerance=1e-8, dt=None):
    """The oblique-shock set-up OBLIQUO on the unit square with n x n nodes:
    marks of Mesh_Generator/Structured_Mesh/meshGenerator.c:231-241 (bottom
    wall y = 0: rho v prescribed; inflow x = 0 and top y = 1: everything
    prescribed; elsewhere free), inflow (rho, rho u, rho v, rho E) =
    (1, 0.98481, -0.17365, 0.94643) at 10 degrees (OBLIQUO_*presc.c), the
    same initial state, gamma = 1.4.  dt defaults to 0.5 min h / (|v| + c)
    of the initial state."""
    M = n_nodes_side - 1
    X, Y, ien = structured_mesh(M, M)
    bottom = np.abs(Y) <= 1e-15
    inflow = (np.abs(X) <= 1e-15) | (np.abs(Y - 1.0) <= 1e-15)
    type_ = np.ones((X.shape[0], 4), dtype=np.int32)
    type_[bottom, 2] = 0
    type_[inflow & ~bottom, :] = 0
    type_ = type_.reshape(-1)
    invp, neq = number_dofs(type_)
    mesh = Mesh(X, Y, ien, 4, type_, invp, neq)
    state = (1.0, 0.98481, -0.17365, 0.94643)
    coef = np.zeros((4, 3))
    coef[:, 0] = state
    if dt is None:
        dt = euler_dt(mesh, 1.4, state, 0.5)
    return euler_problem(mesh, 1.4, mach, dimensionless, tolerance, alpha, dt, coef, True, state)


def write_rank_file(mesh: Mesh, path: str) -> None:
    """A one-rank partition file (the format SST/Preprocess.c:127-168 reads):
    per node x, y and per dof Type [Send invP_id] (Send = 1: nothing to
    exchange), then the elements."""
    with open(path, "w") as f:
        f.write(f"{mesh.nnodes}\n")
        for i in range(mesh.nnodes):
            f.write(f"{mesh.x[i]:.14f}\t{mesh.y[i]:.14f}\t")
            for k in range(mesh.ndof):
                q = i * mesh.ndof + k
                t = int(mesh.type[q])
                f.write(f"{t}\t" if t == 0 else f"{t}\t1\t{int(mesh.invp[q])}\t")
            f.write("\n")
        f.write(f"{mesh.nel}\n")
        for e in range(mesh.nel):
            f.write(" ".join(str(int(v)) for v in mesh.ien[e]) + "\n")

