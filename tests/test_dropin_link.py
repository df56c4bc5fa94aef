"""The reference's drivers link unchanged against the drop-in shims.

oracle/Makefile `dropin` compiles the reference's own driver files
(Process.c, Predictor_Old.c, the Build functions, set*.c, ...) unmodified
and links them, in place of the reference's solve-path files (pgmres.c,
the EBE and CSR matvecs, csr_assembly.c, the Diag / BlockDiag / NO /
ILU(p) / SPIKE preconditioners), against libfemgpu_sst.so,
libfemgpu_ns.so and libfemgpu_euler.so, with -Wl,--no-undefined.  This
test checks that the link succeeds and that the solve-path symbols the
drivers call come from the shims.  It needs the reference sources (it is
skipped where they are absent); the GPU runs of the linked drivers are in
test_gpu_dropin.py.
"""
import os
import shutil
import subprocess

import pytest

import oracle as O

LIBS = {"sst": ("libfemgpu_sst.so", ["pgmres", "ebemv", "csrmv", "Diag_precond", "Diag_precond_EBE_setup",
                                     "ILUp_precond_setup", "SPIKE_precond_setup", "csr_assembly", "LU_precond_EBE",
                                     "LU_precond_EBE_setup", "SGS_precond_EBE", "SGS_precondR_EBE",
                                     "SGS_precond_EBE_setup"]),
        "ns": ("libfemgpu_ns.so", ["pgmres", "ebemvNDOF3", "BlockDiagDOF3_precond",
                                   "BlockDiagDOF3_precond_EBE_setup", "csrmv", "ILUp_precond_setup"]),
        "euler": ("libfemgpu_euler.so", ["pgmres", "ebemvNDOF4", "BlockDiag_precond", "BlockDiag_precond_EBE_setup",
                                         "csrmv", "csr_assembly", "ILUp_precond_setup", "SPIKE_precond_setup"])}


def _symbols(path, undefined):
    args = ["nm", "-D", "--undefined-only" if undefined else "--defined-only", path]
    out = subprocess.run(args, check=True, capture_output=True, text=True).stdout
    return {line.split()[-1] for line in out.splitlines() if line.strip()}


@pytest.mark.skipif(not os.path.isdir(os.path.join(O.REF_SRC, "00_CommonFiles")), reason="reference sources absent")
@pytest.mark.skipif(shutil.which("nm") is None, reason="nm absent")
def test_reference_drivers_link_against_the_shims(femgpu):
    subprocess.run(["make", "-s", "-C", os.path.dirname(O.__file__), "dropin", f"REF={O.REF_SRC}"], check=True)
    lib_dir = os.path.dirname(femgpu.library_path())
    for kind, (shim, syms) in LIBS.items():
        so = O.DROPIN_SO[kind]
        assert os.path.exists(so)
        needed = subprocess.run(["readelf", "-d", so], check=True, capture_output=True, text=True).stdout
        assert shim in needed
        undef, defined = _symbols(so, True), _symbols(so, False)
        shim_defs = _symbols(os.path.join(lib_dir, shim), False)
        for sym in syms:
            assert sym in undef and sym not in defined, (kind, sym)   # called by the drivers, not compiled in
            assert sym in shim_defs, (kind, sym)                      # provided by the shim
        # the drivers themselves are the reference's
        assert ("Process" if kind != "euler" else "Predictor_Old") in defined


@pytest.mark.skipif(not os.path.isdir(os.path.join(O.REF_SRC, "02_Transport_Equation")),
                    reason="reference sources absent")
@pytest.mark.skipif(shutil.which("nm") is None, reason="nm absent")
def test_transient_driver_links_against_its_shim(femgpu):
    """The transient-transport driver (Predictor_Old.c, Predictor_New.c, its
    Build functions, from a private copy whose header points at the MPI
    stand-in) links against libfemgpu_tt.so in place of its solve path."""
    subprocess.run(["make", "-s", "-C", os.path.dirname(O.__file__), "dropin_tt", f"REF={O.REF_SRC}"], check=True)
    lib_dir = os.path.dirname(femgpu.library_path())
    so = O.DROPIN_TT_SO
    needed = subprocess.run(["readelf", "-d", so], check=True, capture_output=True, text=True).stdout
    assert "libfemgpu_tt.so" in needed
    undef, defined = _symbols(so, True), _symbols(so, False)
    shim_defs = _symbols(os.path.join(lib_dir, "libfemgpu_tt.so"), False)
    for sym in ("pgmres", "ebemv", "Diag_precond", "Diag_precond_EBE_setup", "NO_precond"):
        assert sym in undef and sym not in defined, sym
        assert sym in shim_defs, sym
    for sym in ("Predictor_Old", "Predictor_New", "Build_M_F_DD", "Build_M_K_R_SUPG", "calculate_DaB"):
        assert sym in defined, sym
