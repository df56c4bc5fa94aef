"""Mesh-file fixtures from the reference's own structured mesh generator.

Compiles Mesh_Generator/Structured_Mesh/meshGenerator.c (one file) into
oracle/_ref/, runs it there on two inputs, and copies its outputs here:

  mesh_TESTE_8x8.dat    TESTE, "right" diagonal, 8 x 8 cells (NDOF = 1)
  mesh_OBLIQUO_6x6.dat  OBLIQUO, "right" diagonal, 6 x 6 cells (NDOF = 4)

Needs the reference sources (PFC_REFERENCE_DIR, default: the directory
`reference` beside this repository) and gcc; the
fixtures are committed, the tests only read them.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("PFC_REFERENCE_DIR") or os.path.normpath(os.path.join(ROOT, "..", "reference"))
OUT = os.path.join(ROOT, "oracle", "_ref")


def main():
    src = os.path.join(REF, "Mesh_Generator", "Structured_Mesh", "meshGenerator.c")
    if not os.path.exists(src):
        sys.exit(f"reference generator not found: {src}")
    os.makedirs(OUT, exist_ok=True)
    exe = os.path.join(OUT, "meshGenerator")
    subprocess.run(["gcc", "-O2", "-w", "-o", exe, src, "-lm"], check=True)
    cases = [("TESTE", 8, 8, "mesh_TESTE_8x8.dat"), ("OBLIQUO", 6, 6, "mesh_OBLIQUO_6x6.dat")]
    for problem, M, N, name in cases:
        inp = os.path.join(OUT, f"{problem}_gen.txt")
        with open(inp, "w") as f:
            f.write("right\t:inclination\n")
            f.write(f"{M}\t:M\n{N}\t:N\n0\t:Xcria\n0\t:Ycria\n4\t:nodes\n")
            for x, y in ((0.0, 0.0), (1.0, 0.0), (1.0, 1.0), (0.0, 1.0)):
                f.write(f"{x}\t{y}\t:corner\n")
        subprocess.run([exe, inp, problem], check=True, cwd=OUT, stdout=subprocess.DEVNULL)
        nn, ne = (M + 1) * (N + 1), 2 * M * N
        shutil.copy(os.path.join(OUT, f"{problem}_{nn}_{ne}.dat"), os.path.join(HERE, name))
        print("wrote", name)


if __name__ == "__main__":
    main()
