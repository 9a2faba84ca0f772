"""Time the compiled reference's explicit step on this machine's cores, once per
Domain::computeInternalForces parallelisation strategy (Domain.C:155-735, chosen by the
``computeInternalForces`` environment variable, README.md:36-51), with all cores and, for the best
strategy, one core.  Test infrastructure: it runs ``oracle/_ref/ref_harness`` (``make -C oracle
ref``), which exists only where the reference's sources do.

    python oracle/time_reference.py [--quick]

Prints one markdown table row per workload and strategy: element-updates/s over K whole explicit
steps (ExplicitSolverCH's step: predictions, internal forces, corrections, internal matrices and
the time step) timed inside the harness with std::chrono.

3D workloads run on one thread only: Element3D::computeInternalMatrices inverts each Jacobian with
Matrix::inverse (linearAlgebra/Matrix.C:1653-1727), i.e. the f2c-translated dgetrf_/dgetri_ whose
Fortran locals are `static` (lapack/Lapack/dgetrf.c:71-81, dgetri.c:75-96), inside the OpenMP loop
over elements; with two or more threads they race (the workspace size lwkopt included) and the
process aborts with heap corruption under every strategy.
"""

from __future__ import annotations

import argparse
import dataclasses
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from oracle import dnl_io  # noqa: E402
from redynela_gb300 import meshes  # noqa: E402


def workloads(quick: bool):
    return [
        ("taylor_axi_5x50 (250 ElQua4nAx, Courant)", meshes.taylor_axi(5, 50), 200 if quick else 1000),
        ("taylor_axi_20x200 (4,000 ElQua4nAx, Courant)", meshes.taylor_axi(20, 200), 50 if quick else 200),
        ("taylor_hex_40x40x20 (25,280 ElHex8n3D, Pulse)", meshes.taylor_hex(40, 20), 5 if quick else 20),
    ]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--quick", action="store_true")
    args = ap.parse_args()
    if not dnl_io.reference_available():
        sys.exit("compiled reference missing: run `make -C oracle ref`")
    cores = os.cpu_count() or 1
    print(f"| workload | strategy | threads | steps | element-updates/s |")
    print("|---|---|---|---|---|")
    for name, m, k in workloads(args.quick):
        if m.dim == 3:  # the reference's 3D path is not thread-safe (see above)
            r = dnl_io.run_reference("bench", m, k, threads=1, strategy=0)
            rate1 = m.E * float(r["steps"][0]) / float(r["wall_s"][0])
            print(f"| {name} | 0 | 1 | {int(r['steps'][0])} | {rate1:.4g} |", flush=True)
            continue
        best = (0.0, 0)
        for strat in range(8):
            r = dnl_io.run_reference("bench", m, k, threads=cores, strategy=strat)
            rate = m.E * float(r["steps"][0]) / float(r["wall_s"][0])
            best = max(best, (rate, strat))
            print(f"| {name} | {strat} | {cores} | {int(r['steps'][0])} | {rate:.4g} |", flush=True)
        r = dnl_io.run_reference("bench", m, k, threads=1, strategy=best[1])
        rate1 = m.E * float(r["steps"][0]) / float(r["wall_s"][0])
        print(f"| {name} | {best[1]} (best) | 1 | {int(r['steps'][0])} | {rate1:.4g} |", flush=True)


if __name__ == "__main__":
    main()
