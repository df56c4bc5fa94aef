"""Generate the golden fixtures from the reference's own C (checker build).

Run here, where the reference sources are present:
    make -C oracle ref && python tests/golden/make_golden.py
(the reference tree: PFC_REFERENCE_DIR, default `reference` beside this
repository)
It writes tests/golden/sst_*.npz: mesh, connectivity (lm, Perm, invPerm,
bandwidths), element blocks and right-hand side at u = 0, one Diag +
GMRES(30) solve, and the full CAU Process loop (solution and GMRES
iterations), all computed by the reference's Fill_LM, Permutation_of_LM,
Build_K_F_SUPG, Diag_precond_EBE_setup, pgmres and Process; and
tests/golden/ns_*.npz: the steady Navier-Stokes driver's Fill_LM,
Build_K_F_SUPG_PSPG at a state u, BlockDiagDOF3_precond_EBE_setup,
ebemvNDOF3 and (cavity) the Picard Process loop; and tests/golden/eu_*.npz:
the Euler driver's Fill_LM, Build_M_K_F_SUPG at a state (u, du),
BlockDiag_precond_EBE_setup, ebemvNDOF4 and the Predictor_Old time loop;
and tests/golden/time_schemes_euler.npz: the final states of Predictor_Old_BDF and
of Predictor_New_TRBDF2 (run with Build_M_K_F_SUPG, its bubble unknowns
zero) on the Euler cases; and tests/golden/vms_ns.npz: Build_K_F_VMS_DCDD
(blocks and residual at a state u) and its Picard Process loop on the NS
cases; and tests/golden/dd_sst.npz: the steady transport driver's
Build_K_F_DD with CAUDD and with CAU (blocks and F at a state u) and its
Process loop on the transport cases; and tests/golden/shock_sst.npz: the
YZBeta shock capture and the h_shock Option1 / Option2 lengths with both
forms (blocks and F at a state u, the Process loop); and
tests/golden/ilup_sst.npz: the reference's ILU(p) ("ILU1", "ILU2", "ILU3")
applied to a vector, with the CSR matrix it factorises; and
tests/golden/dd_euler.npz: the Euler driver's Build_M_K_F_DD_Transiente (with
Delta_DD) at a state (u, du) and its Predictor_Old loop, on the Euler cases
(the harness clears the stack before each DD build: the reference reads an
unassigned Jacobian entry there).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402
from parallel_fem_codes_gb300 import meshgen as G  # noqa: E402

CASES = {
    # name: (nodes per side, angle, conductivity, gamma, f, upmode, upval)
    "sst_17_adv": (17, 30.0, 1e-6, 0.0, 0.0, 0, 1.0),
    "sst_12_mixed": (12, 200.0, 1e-3, 0.5, 1.0, 0, 1.0),
    "sst_9_teste": (9, 0.0, 1.0, 0.0, 0.0, 1, 10.0),
}


def main():
    if not O.ref_available():
        raise SystemExit("build the reference first: make -C oracle ref")
    for name, (n, ang, k, gm, f, upm, upv) in CASES.items():
        p = G.transport_problem(n, angle_deg=ang, k=k, gamma=gm, f=f, upmode=upm, upval=upv)
        if name == "sst_9_teste":
            p.beta = (0.0, 0.0)
        m = p.mesh
        lm, perm, inv, band, nnz = O.ref_connectivity(m)
        A, F = O.ref_build(p)
        X, it, Diag, invDiag, Fp = O.ref_diag_pgmres(lm, A, perm, inv, F, kmax=30, lmax=1000, tol=1e-10)
        U, its = O.ref_process(p, 1e-10, 1e-3, 30, 1000)
        np.savez_compressed(
            os.path.join(HERE, name + ".npz"),
            x=m.x, y=m.y, ien=m.ien, type=m.type, invp=m.invp, neq=m.neq, upresc=p.upresc,
            k=p.k, gamma=p.gamma, beta=np.array(p.beta), f=p.f, upmode=p.upmode, upval=p.upval,
            lm=lm, perm=perm, invperm=inv, band=band, nnz=nnz, A=A, F=F[: m.neq],
            Fp=Fp[: m.neq], Diag=Diag[: m.neq], X=X[: m.neq], gmres_its=it,
            U=U, process_its=its)
        print(name, "neq", m.neq, "gmres", it, "process gmres", its)
    for name, (prob, seed, process) in ns_cases().items():
        m = prob.mesh
        rng = np.random.Generator(np.random.PCG64(seed))
        u = rng.standard_normal(m.neq) if seed else np.zeros(m.neq)
        lm = O.ref_ns_lm(m)
        A, F = O.ref_ns_build(prob, u)
        inv, Fp = O.ref_ns_blockdiag(m, A, F)
        P = rng.standard_normal(m.neq + 1)
        P[m.neq] = 0.0
        Q = O.ref_ns_ebemv(m, A, P)
        extra = {}
        if process:
            U, its = O.ref_ns_process(prob, 1e-10, 1e-6, 30, 1000, 30)
            extra = dict(U=U, process_its=its)
        np.savez_compressed(
            os.path.join(HERE, name + ".npz"),
            x=m.x, y=m.y, ien=m.ien, type=m.type, invp=m.invp, neq=m.neq, reynolds=prob.reynolds,
            coef=prob.coef, lid=int(prob.lid), u=u, lm=lm, A=A, F=F, inv=inv, Fp=Fp, P=P, Q=Q, **extra)
        print(name, "neq", m.neq, extra.get("process_its"))


def euler_cases():
    """name: (problem, seed of the perturbation of (u, du), time options)."""
    p9 = G.obliquo_problem(9)
    p7 = G.obliquo_problem(7, dimensionless=False)
    return {"eu_9_obliquo": (p9, 3, O.TimeOpts(0, 2, 1e-3, 0, 4 * p9.dt, 1e-6, 0)),
            "eu_7_dimensional": (p7, 4, O.TimeOpts(1, 4, 1e-2, 1, 20 * p7.dt, 1e-2, 0))}


def write_euler():
    for name, (prob, seed, to) in euler_cases().items():
        m = prob.mesh
        rng = np.random.Generator(np.random.PCG64(seed))
        u0 = prob.initial_state()
        u = u0 * (1.0 + 0.05 * rng.standard_normal(m.neq))
        du = 0.01 * rng.standard_normal(m.neq)
        lm = O.ref_euler_lm(m)
        A, R = O.ref_euler_build(prob, u, du)
        inv, Rp = O.ref_euler_blockdiag(m, A, R)
        P = rng.standard_normal(m.neq + 1)
        P[m.neq] = 0.0
        Q = O.ref_euler_ebemv(m, A, P)
        U, its, t = O.ref_euler_predictor(prob, to, 1e-10, 25, 1000)
        np.savez_compressed(
            os.path.join(HERE, name + ".npz"),
            x=m.x, y=m.y, ien=m.ien, type=m.type, invp=m.invp, neq=m.neq, params=prob.params(),
            coef=prob.coef, wall=int(prob.wall), init=prob.init, topts=to.as_array(), u=u, du=du, lm=lm,
            A=A, R=R, inv=inv, Rp=Rp, P=P, Q=Q, U=U, gmres_its=its, t=t)
        print(name, "neq", m.neq, "gmres", its, "t", t)


def ns_cases():
    """name: (problem, seed of the state u (0: u = 0), run the Process loop)."""
    cav = G.cavity_problem(9, reynolds=100.0)
    mesh = G.multi_dof_mesh(9, 3, seed=2, jitter=0.2)
    aff = G.ns_problem(mesh, 50.0, np.random.Generator(np.random.PCG64(5)).standard_normal((5, 3)))
    return {"ns_9_cavity": (cav, 0, True), "ns_9_affine": (aff, 6, False)}


def write_euler_schemes():
    out = {}
    for name, (prob, seed, to) in euler_cases().items():
        for scheme in (1, 2):
            to.scheme = scheme
            U, its, t = O.ref_euler_predictor(prob, to, 1e-10, 25, 1000)
            key = f"{name}_s{scheme}"
            out[key + "_U"], out[key + "_its"], out[key + "_t"] = U, its, t
            print(key, "gmres", its, "t", t)
    np.savez_compressed(os.path.join(HERE, "time_schemes_euler.npz"), **out)


def write_ns_vms():
    out = {}
    for name, (prob, seed, run) in ns_cases().items():
        m = prob.mesh
        u = np.random.Generator(np.random.PCG64(seed + 11)).standard_normal(m.neq)
        A, F = O.ref_ns_build(prob, u, form=1)
        out[name + "_u"], out[name + "_A"], out[name + "_F"] = u, A, F
        if run:
            U, its = O.ref_ns_process(prob, 1e-10, 1e-3, 30, 1000, 20, form=1)
            out[name + "_U"], out[name + "_its"] = U, its
            print(name, "VMS-DCDD gmres", its)
    np.savez_compressed(os.path.join(HERE, "vms_ns.npz"), **out)


def write_sst_dd():
    out = {}
    for name, (n, ang, k, gm, f, upm, upv) in CASES.items():
        if name == "sst_9_teste":
            continue
        for shock in (1, 2):
            p = G.transport_problem(n, angle_deg=ang, k=k, gamma=gm, f=f, upmode=upm, upval=upv, cau=shock)
            p.form = 1
            u = np.random.Generator(np.random.PCG64(n + shock)).random(p.mesh.neq)
            A, F = O.ref_build(p, u)
            U, its = O.ref_process(p, 1e-10, 1e-3, 30, 1000)
            key = f"{name}_c{shock}"
            out[key + "_u"], out[key + "_A"], out[key + "_F"] = u, A, F[: p.mesh.neq]
            out[key + "_U"], out[key + "_its"] = U, its
            print(key, "DD process gmres", its)
    np.savez_compressed(os.path.join(HERE, "dd_sst.npz"), **out)


SHOCK_CASES = [(0, 3, 0), (0, 3, 1), (0, 1, 2), (1, 3, 2), (1, 2, 1), (1, 3, 0)]   # (form, shock, h_shock)


def write_sst_shock():
    out = {}
    for form, shock, hs in SHOCK_CASES:
        p = G.transport_problem(13, angle_deg=110.0, k=1e-4, gamma=0.2, f=0.5, cau=shock)
        p.form, p.h_shock = form, hs
        u = np.random.Generator(np.random.PCG64(form * 100 + shock * 10 + hs)).random(p.mesh.neq)
        A, F = O.ref_build(p, u)
        U, its = O.ref_process(p, 1e-10, 1e-3, 30, 1000)
        key = f"f{form}_c{shock}_h{hs}"
        out[key + "_u"], out[key + "_A"], out[key + "_F"] = u, A, F[: p.mesh.neq]
        out[key + "_U"], out[key + "_its"] = U, its
        print(key, "process gmres", its)
    np.savez_compressed(os.path.join(HERE, "shock_sst.npz"), **out)


def write_ilup():
    out = {}
    for n, ang, k in [(13, 30.0, 1e-3), (17, 200.0, 1e-2)]:
        p = G.transport_problem(n, angle_deg=ang, k=k)
        A, F = O.build_k_f_supg(p)
        P = np.random.Generator(np.random.PCG64(n)).standard_normal(p.mesh.neq + 1)
        P[-1] = 0.0
        for lev in (1, 2, 3):
            IA, JA, AA, invp, Q, z = O.ref_csr(p, A, P, ilu_p=lev)
            key = f"n{n}_p{lev}"
            out[key + "_IA"], out[key + "_JA"], out[key + "_AA"] = IA, JA, AA
            out[key + "_P"], out[key + "_z"] = P, z[: p.mesh.neq]
            print(key, "nnz", len(JA))
    np.savez_compressed(os.path.join(HERE, "ilup_sst.npz"), **out)


def write_euler_dd():
    out = {}
    for name, (prob, seed, to) in euler_cases().items():
        prob.form = 1
        m = prob.mesh
        rng = np.random.Generator(np.random.PCG64(seed + 20))
        u = prob.initial_state() * (1.0 + 0.05 * rng.standard_normal(m.neq))
        du = 0.01 * rng.standard_normal(m.neq)
        A, R = O.ref_euler_build(prob, u, du)
        to.scheme = 0
        U, its, t = O.ref_euler_predictor(prob, to, 1e-10, 25, 1000)
        out[name + "_u"], out[name + "_du"], out[name + "_A"], out[name + "_R"] = u, du, A, R
        out[name + "_U"], out[name + "_its"], out[name + "_t"] = U, its, t
        print(name, "DD gmres", its, "t", t)
    np.savez_compressed(os.path.join(HERE, "dd_euler.npz"), **out)


TT_CASES = [(0, 1, 0), (0, 3, 1), (0, 1, 2), (1, 2, 0), (1, 3, 2)]   # (form, shock, h_shock)


def write_tt():
    """The transient transport driver's own builds (Build_M_K_R_SUPG /
    Build_M_K_R_DD, oracle/_ref/libref_tt.so) at random states (u, du)."""
    out = {}
    for form, cau, hs in TT_CASES:
        p = G.transport_problem(17, angle_deg=35.0, k=1e-3, gamma=0.2, f=0.5, cau=cau)
        p.form, p.h_shock = form, hs
        rng = np.random.default_rng(100 + 10 * form + cau + 3 * hs)
        u = rng.random(p.mesh.neq)
        du = rng.standard_normal(p.mesh.neq)
        A, R = O.ref_tt_build(p, 0.5, 0.01, u, du)
        key = f"tt_{form}_{cau}_{hs}"
        out[key + "_u"], out[key + "_du"], out[key + "_A"], out[key + "_R"] = u, du, A, R
        print(key)
    np.savez_compressed(os.path.join(HERE, "tt_ref.npz"), **out)


EU_P2_INVY = (1.0, 0.5, 2.0, 0.25)


def write_euler_yzbeta():
    """ShockCapture "YZBeta" (Delta_YZBeta.c) in the Euler SUPG and
    Predictor1 DD builds (oracle/_ref/libref_euler.so): one build at a
    random state per form, and Predictor_Old / Predictor_Old_BDF over 3
    steps of 2 corrections."""
    out = {}
    for form in (0, 1):
        p = G.obliquo_problem(9)
        p.form, p.shock, p.invY = form, 3, np.array(EU_P2_INVY)
        m = p.mesh
        rng = np.random.default_rng(40 + form)
        u = p.initial_state() * (1 + 0.05 * rng.standard_normal(m.neq))
        du = 0.05 * rng.standard_normal(m.neq)
        A, R = O.ref_euler_build(p, u, du)
        key = f"yz_{form}"
        out[key + "_u"], out[key + "_du"], out[key + "_A"], out[key + "_R"] = u, du, A, R
        for scheme in (0, 1):
            to = O.TimeOpts(0, 2, 1e-3, 0, 3 * p.dt + 1e-12, 1e-6, 0, scheme)
            U, its, t = O.ref_euler_predictor(p, to, 1e-10, 25, 1000)
            out[f"{key}_s{scheme}_U"], out[f"{key}_s{scheme}_its"] = U, np.array([its])
            print(key, scheme, "gmres", its)
    np.savez_compressed(os.path.join(HERE, "euler_yzbeta_ref.npz"), **out)


def write_euler_predictor2():
    """TimeIntegration "Predictor2" of the Euler driver with "DD" and
    "YZBeta" (oracle/_ref/libref_euler.so): one Build_M_F_DD_Transiente +
    calculate_DaB at a random state, and the reference's own Predictor_New
    loop (BlockDiag, pgmres) over 3 steps of 2 corrections."""
    p = G.obliquo_problem(9)
    p.invY = np.array(EU_P2_INVY)
    m = p.mesh
    rng = np.random.default_rng(31)
    u = p.initial_state() * (1 + 0.05 * rng.standard_normal(m.neq))
    du = 0.1 * rng.standard_normal(m.neq)
    uB = 0.01 * rng.standard_normal(4 * m.nel)
    duB = 0.01 * rng.standard_normal(4 * m.nel)
    Da = np.append(rng.standard_normal(m.neq), 3.0)
    A, F, cond, DaB = O.ref_euler_mfdd_build(p, u, du, uB, duB, Da)
    out = {"u": u, "du": du, "uB": uB, "duB": duB, "Da": Da, "A": A, "F": F, "cond": cond, "DaB": DaB}
    to = O.TimeOpts(0, 2, 1e-3, 0, 3 * p.dt + 1e-12, 1e-6, 0, 3)
    U, its, t = O.ref_euler_predictor(p, to, 1e-10, 25, 1000)
    out["U"], out["its"] = U, np.array([its])
    print("euler predictor2 gmres", its)
    # "Predictor2_BDF" (Predictor_New_BDF) and "Predictor2_TRBDF2"
    # (Predictor_New_TRBDF2 with the bubble build; the harness links a
    # uB_InitialSolution that reads prescribed values, see harness_euler.c)
    p.form = 2
    for scheme in (4, 2):
        to = O.TimeOpts(0, 2, 1e-3, 0, 3 * p.dt + 1e-12, 1e-6, 0, scheme)
        U, its, t = O.ref_euler_predictor(p, to, 1e-10, 25, 1000)
        out[f"U_s{scheme}"], out[f"its_s{scheme}"] = U, np.array([its])
        print("euler predictor2 scheme", scheme, "gmres", its)
    np.savez_compressed(os.path.join(HERE, "euler_predictor2_ref.npz"), **out)


def write_tt_predictor1():
    """The transient transport driver's own Predictor_Old loop (Diag,
    pgmres) with Build_M_K_R_SUPG (CAU) and Build_M_K_R_DD (CAUDD),
    4 steps of 2 corrections (oracle/_ref/libref_tt.so)."""
    out = {}
    for form, cau in ((0, 1), (1, 2)):
        p = G.transport_problem(17, angle_deg=30.0, k=1e-3, f=0.0, cau=cau)
        p.form = form
        to = O.TimeOpts(0, 2, 1e-3, 0, 4 * 0.02 + 1e-12, 1e-6, 0, 0)
        U, its = O.ref_tt_predictor1(p, 0.5, 0.02, to)
        out[f"p1_{form}_U"], out[f"p1_{form}_its"] = U, np.array([its])
        print("tt predictor1 form", form, "gmres", its)
    np.savez_compressed(os.path.join(HERE, "tt_predictor1_ref.npz"), **out)


TT_P2_CASES = [(2, 0), (3, 2)]   # (shock, h_shock) of the DD form


def write_tt_predictor2():
    """TimeIntegration "Predictor2" of the transient transport driver
    (oracle/_ref/libref_tt.so): one Build_M_F_DD + calculate_DaB at random
    states, and the reference's own Predictor_New loop (Diag, pgmres) over
    4 steps of 2 corrections."""
    out = {}
    for cau, hs in TT_P2_CASES:
        p = G.transport_problem(17, angle_deg=35.0, k=1e-3, gamma=0.2, f=0.5, cau=cau)
        p.form, p.h_shock = 1, hs
        m = p.mesh
        rng = np.random.default_rng(200 + 10 * cau + hs)
        u = rng.random(m.neq)
        du = rng.standard_normal(m.neq)
        uB = rng.random(m.nel)
        duB = rng.standard_normal(m.nel)
        Da = np.append(rng.standard_normal(m.neq), 5.0)
        A, F, cond, DaB = O.ref_tt_mfdd_build(p, 0.5, 0.01, u, du, uB, duB, Da)
        key = f"p2_{cau}_{hs}"
        for name, v in (("u", u), ("du", du), ("uB", uB), ("duB", duB), ("Da", Da), ("A", A), ("F", F),
                        ("cond", cond), ("DaB", DaB)):
            out[f"{key}_{name}"] = v
        to = O.TimeOpts(0, 2, 1e-3, 0, 0.04 + 1e-12, 1e-6, 0, 0)
        U, its = O.ref_tt_predictor2(p, 0.5, 0.01, to, tol=1e-10, kmax=30, lmax=1000)
        out[key + "_U"], out[key + "_its"] = U, np.array([its])
        print(key, "gmres", its)
    np.savez_compressed(os.path.join(HERE, "tt_predictor2_ref.npz"), **out)


def write_elem_prec():
    """The steady driver's element preconditioners (Preconditioner "LUe" and
    "SGSe": LU_precond_EBE*.c, SGS_precond_EBE*.c and pgmres with their
    precond / precondR pair, oracle/_ref/libref_sst.so) on the SUPG blocks
    of a 17x17 and a 33x33 transport problem: one application of each sweep
    to a random vector and the preconditioned right-hand side and solution
    of each solve."""
    out = {}
    for n in (17, 33):
        p = G.transport_problem(n, angle_deg=30.0, k=1e-3)
        m = p.mesh
        A, F = O.build_k_f_supg(p)
        lm = O.fill_lm(m)
        perm, inv, _ = O.permutation_of_lm(m)
        z = np.append(np.random.default_rng(n).standard_normal(m.neq), 0.0)
        key = f"ep_{n}"
        out[key + "_z"] = z
        for kind in (1, 2, 3):
            out[key + f"_apply{kind}"] = O.ref_elem_prec_apply(kind, lm, A, m.neq, z)
        for kind in (1, 2):
            X, it, Fp = O.ref_ebe_elem_solve(kind, lm, A, perm, inv, F, kmax=30, lmax=200, tol=1e-10)
            out[key + f"_X{kind}"], out[key + f"_F{kind}"], out[key + f"_it{kind}"] = X, Fp, np.array([it])
        print(key)
    np.savez_compressed(os.path.join(HERE, "elem_prec_sst.npz"), **out)


if __name__ == "__main__":
    main()
    write_euler()
    write_euler_schemes()
    write_ns_vms()
    write_sst_dd()
    write_sst_shock()
    write_ilup()
    write_euler_dd()
    write_tt()
    write_tt_predictor1()
    write_tt_predictor2()
    write_euler_predictor2()
    write_euler_yzbeta()
    write_elem_prec()
