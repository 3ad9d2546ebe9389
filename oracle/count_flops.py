"""Operation count of the reference algorithm (test infrastructure): runs one residual of the
oracle -- the CPU restatement of Flou's rhs! -- instantiated with a counting scalar on small
meshes of the benchmark configurations and prints the counts per node (DOF) as a Markdown table.

    python oracle/count_flops.py
"""
import math
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path[:0] = [ROOT, os.path.join(ROOT, "flou.jl_gb300"), os.path.join(ROOT, "tests")]

import numpy as np  # noqa: E402

import flou_cuda as F  # noqa: E402
from cases import oracle_for  # noqa: E402


def tgv(nel, n):
    import bench
    return bench.make_tgv(nel, n)


def vortex(nel, n):
    eq = F.EulerEquation(2, 1.4)
    mesh = F.CartesianMesh((-5.0, -5.0), (5.0, 5.0), (nel, nel))
    F.apply_periodicBCs(mesh, ("1", "2"), ("3", "4"))
    b = F.LagrangeBasis("GLL", n)
    disc = F.MultielementDisc(mesh, F.StdQuad(b, F.DGSEMrec(b), 4), eq, F.StrongDivOperator(F.LxF(F.StdAverage(), 1.0)))
    Q0 = np.asfortranarray(F.initial.isentropic_vortex(eq, disc.coords, (0.3, 0.1), beta=5.0, period=(10.0, 10.0)))
    return disc, Q0


def main():
    rows = []
    for name, (disc, Q) in (("3D TGV split Chandrashekar + HLLC, p=7 (4³ elements)", tgv(4, 8)),
                            ("3D TGV split Chandrashekar + HLLC, p=3 (8³ elements)", tgv(8, 4)),
                            ("2D vortex strong form + Rusanov, p=4 (8² elements)", vortex(8, 5))):
        c = oracle_for(disc).count(Q)
        nd = disc.ndofs
        flops = c["add"] + c["mul"]
        rows.append((name, c["add"] / nd, c["mul"] / nd, c["div"] / nd, c["sqrt"] / nd, c["log"] / nd, flops / nd))
    print("# Reference-algorithm operation count per node, one residual (oracle with a counting scalar)")
    print()
    print("Command: `python oracle/count_flops.py`. Each + - x is one flop (the reference has no fused")
    print("multiply-add); divisions, square roots and logarithms are counted apart. Per stage update add")
    print("the combination (2 to 4 flops per variable).")
    print()
    print("| configuration | add | mul | div | sqrt | log | flops (add+mul) |")
    print("|---|---|---|---|---|---|---|")
    for r in rows:
        print("| %s | %.1f | %.1f | %.1f | %.2f | %.2f | %.1f |" % r)


if __name__ == "__main__":
    main()
