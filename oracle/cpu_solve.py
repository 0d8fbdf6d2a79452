"""Whole solves of the oracle's restatement of COCR_FP on the host cores: the
CPU baseline of bench.py (its `cpu_baseline` and its reference arm).

Test infrastructure: the oracle is the checker and the CPU baseline, never
part of the product path.  Each timed solve is the reference's
PCOCR_2x2_Folded (Code/COCR_FP/pcocr.cpp:40-126: folded-preconditioner
set-up, then the COCR iteration to the MRS stop rule) from x = 0, timed on
the wall clock like the reference's `kit` time (base_solver.cpp:181-200).

It runs in a process of its own so that nothing else shares its OpenMP
runtime or cores: `python -m oracle.cpu_solve WORKLOAD NU ALFA THREADS
[--slae FILE.npz] [--warmup W] [--steps K] [--sample-iterations N]`
prints one JSON line.  Warm-up solves stop after 20 iterations (they only
fault in the pages and caches); timed ones run to the stop rule.  With
--sample-iterations N it times set-up + N iterations instead (used for the
one-thread figure, which would take minutes per solve).
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def load_system(workload, nu, alfa, slae_file=None):
    from mtcalc_with_dfp_cocr_gb300 import normal1d, slae_io, workloads
    from oracle import pyoracle as O
    w = workloads.make(workload)
    mesh = slae_io.mesh_to_solve_mesh(w.mesh)
    if slae_file:
        g = np.load(slae_file)
        s = slae_io.BlockSLAE(int(len(g["ig"]) - 1), g["ig"], g["jg"], g["idi"], g["ijg"],
                              g["di"], g["gg"], g["pr"], float(g["eps"]), int(g["maxiter"]))
    else:
        tops, sig = [l.top for l in w.mesh.layers], [l.sigma for l in w.mesh.layers]
        s = O.assemble(w.mesh, nu, alfa, *normal1d.solve_1d(nu, tops, sig), eps=1e-8,
                       maxiter=20000)
    return s, mesh


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("workload")
    ap.add_argument("nu", type=float)
    ap.add_argument("alfa", type=int)
    ap.add_argument("threads", type=int)
    ap.add_argument("--slae", default=None)
    ap.add_argument("--warmup", type=int, default=0)
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--sample-iterations", type=int, default=0)
    a = ap.parse_args()
    from oracle import pyoracle as O
    s, mesh = load_system(a.workload, a.nu, a.alfa, a.slae)
    for _ in range(a.warmup):
        O.pcocr(s, mesh, nthreads=a.threads, iter_limit=20)
    seconds, iters, codes = [], [], []
    x = None
    for _ in range(a.steps):
        t0 = time.perf_counter()
        code, x, st = O.pcocr(s, mesh, nthreads=a.threads, iter_limit=a.sample_iterations)
        seconds.append(time.perf_counter() - t0)
        iters.append(int(st.iterations))
        codes.append(int(code))
    true_rel = float(np.linalg.norm(s.pr - O.spmv(s, x, nthreads=a.threads)) /
                     np.linalg.norm(s.pr))
    print(json.dumps({"seconds": seconds, "iterations": iters, "codes": codes,
                      "threads": a.threads, "true_rel": true_rel,
                      "sampled": a.sample_iterations > 0}), flush=True)


if __name__ == "__main__":
    main()
