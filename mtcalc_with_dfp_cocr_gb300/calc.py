"""Survey driver: a calculation directory in, the impedance table out.

    python -m mtcalc_with_dfp_cocr_gb300.calc CASE_DIR [--out FILE]

CASE_DIR holds the reference's five input files (frequencies, xyzVectorB,
z_sig_2d, objects, settings.cfg; the reference's readme.txt documents
them).  The driver does on one GPU what the reference's CalcStarter runs as
separate programs per frequency and polarisation (RegularMeshBuilder,
Harm1D, BuildMatrix, COCR_FP, OutputNu, then ImpedanceZToEdsAll and
calcimpedance over all of them): the mesh (meshbuilder.py), the 1-D normal
fields (normal1d.py), the device assembly, every frequency x polarisation
in one batched survey solve, the receiver fields
(by default through the reference's default output, subdomain smoothing;
--output direct evaluates the edge basis at the receivers) and the MT
responses.

With --results DIR (default CASE_DIR/Results) it also writes the files of
the reference's last step: calcimpedance's 4-byte result files (|Z|, phases,
rho_a, effective rho_a, the Wiese-Parkinson tipper and the complex values)
and ImpedanceZToEdsAll's edsall0_0_imp / ft0_0 (edsall.py).

Under torchrun (one process per GPU) the frequencies are split across the
ranks in contiguous blocks and rank 0 gathers the responses and writes the
files: the systems share no data, so no collective runs during the solves.

The table has the layout of the reference's published results
(CalculationResults/625_500_reg_R_Z.txt): per receiver and period,
northing, easting, period, |Zxx| |Zxy| |Zyx| |Zyy| (Ohm) and the apparent
resistivities Rxx Rxy Ryx Ryy (Ohm.m).  Northing is the model's x and
easting its -y, the convention of that table.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

from . import edsall, meshbuilder, normal1d
from .receivers import MT_RHO, MT_ZABS

def rank_frequencies(nf, rank, world):
    """The frequencies rank `rank` of `world` solves: contiguous, balanced
    blocks (frequencies share no data, so a survey splits across GPUs
    without any exchange until the responses are gathered)."""
    base, extra = divmod(nf, world)
    lo = rank * base + min(rank, extra)
    return list(range(lo, lo + base + (1 if rank < extra else 0)))


def gather_responses(local, idx, nf):
    """Every rank's responses [len(idx)][nrec][34] of frequencies idx into
    the survey's [nf][nrec][34] on rank 0 (None on the others), through
    torch.distributed (any backend; the data are a few KB per frequency)."""
    import torch.distributed as dist
    parts = [None] * dist.get_world_size()
    dist.all_gather_object(parts, (list(idx), np.asarray(local)))
    if dist.get_rank() != 0:
        return None
    out = None
    for ids, arr in parts:
        if out is None and len(ids):
            out = np.empty((nf,) + arr.shape[1:], arr.dtype)
        for k, i in enumerate(ids):
            out[i] = arr[k]
    return out


def run(case, eps=None, maxiter=None, device="cuda", log=None, output="smooth"):
    """Solve every frequency x polarisation of `case`; returns
    (responses [nf][nrec][34], stats dict).  output: "smooth", the
    reference's default receiver output (subdomain smoothing), or "direct"
    (receivers.py).  Under torch.distributed (one process per GPU) every
    rank solves its block of frequencies (rank_frequencies) and rank 0
    returns the whole survey's responses (the others None, None)."""
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        import dataclasses
        idx = rank_frequencies(len(case.freqs), dist.get_rank(), dist.get_world_size())
        sub = dataclasses.replace(case, freqs=np.asarray(case.freqs, np.float64)[idx])
        if idx:
            resp, stats = run_local(sub, eps, maxiter, device, log, output)
        else:
            resp, stats = np.zeros((0, len(case.receivers), 34)), {"systems": []}
        stats["frequencies"] = idx
        allstats = [None] * dist.get_world_size()
        dist.all_gather_object(allstats, stats)
        full = gather_responses(resp, idx, len(case.freqs))
        return full, ({"ranks": allstats} if dist.get_rank() == 0 else None)
    return run_local(case, eps, maxiter, device, log, output)


def run_local(case, eps=None, maxiter=None, device="cuda", log=None, output="smooth"):
    """run() on this process's GPU for all of case's frequencies."""
    import torch
    from .assembly import Assembly
    from .receivers import Receivers
    from .survey import Survey

    eps = case.eps if eps is None else eps
    maxiter = case.maxiter if maxiter is None else maxiter
    t0 = time.perf_counter()
    mesh = meshbuilder.build_mesh(case)
    A = Assembly(mesh)
    R = Receivers(A, case.receivers, output=output)
    miss, _ = R.info()
    tops = [l.top for l in case.layers]
    sig = [l.sigma for l in case.layers]
    freqs = np.asarray(case.freqs, np.float64)
    out = np.empty((len(freqs), len(case.receivers), 34))
    stats = {"nb": mesh.nb, "cells": mesh.kpar, "lines": [mesh.nx, mesh.ny, mesh.nz],
             "receivers_outside_mesh": miss, "eps": eps, "output": output, "systems": []}
    # every frequency x polarisation in one survey (CalcStarter's order: for
    # every frequency X then Y, Code/CalcStarter/main.cpp:311-325)
    nus = np.repeat(freqs, 2)
    alfas = np.tile(np.array([1, 0], np.int32), len(freqs))
    tabs = [normal1d.solve_1d(f, tops, sig) for f in freqs]
    us = np.repeat(np.stack([t[1] for t in tabs]), 2, axis=0)
    uc = np.repeat(np.stack([t[2] for t in tabs]), 2, axis=0)
    b = torch.empty(len(nus), 2 * mesh.nb, dtype=torch.float64, device=device)
    A.rhs(nus, alfas, tabs[0][0], us, uc, b)
    x = torch.zeros_like(b)
    sv = Survey(A, nus)
    code, st = sv.solve(b, x, eps=eps, maxiter=maxiter, verify=True)
    stats["batches"] = sv.batches
    sv.close()
    for k in range(len(nus)):
        stats["systems"].append({
            "nu": float(nus[k]), "polarisation": "XY"[1 - int(alfas[k])],
            "status": st["status"][k], "iterations": st["iterations"][k],
            "fp64_iterations": st["fp64_iterations"][k],
            "true_residual_rel": st["true_residual_rel"][k]})
    if log:
        log(f"{len(nus)} systems in {stats['batches']} batches: code {code}, "
            f"iterations {max(st['iterations'])}")
    E, H, _ = R.fields(x, nus, alfas, tabs[0][0], us, uc)
    out[:] = R.mt_response(freqs, np.arange(0, 2 * len(freqs), 2),
                           np.arange(1, 2 * len(freqs), 2), E, H).cpu().numpy()
    if output == "smooth":
        stats["smoothing"] = R.smoothing_info()
    stats["seconds"] = time.perf_counter() - t0
    return out, stats


def write_table(path, case, resp):
    """The published results' layout: one row per receiver and period
    (periods ascending), tab-separated."""
    freqs = np.asarray(case.freqs, np.float64)
    order = np.argsort(1.0 / freqs)
    with open(path, "w") as f:
        f.write("northing (m)\teasting (m)\tperiods (s)\t\t\tZxx (Ohm)\t\t\tZxy (Ohm)\t\t\t"
                "Zyx (Ohm)\t\t\tZyy (Ohm)\t\t\tRxx (Ohm)\t\t\tRxy (Ohm)\t\t\tRyx (Ohm)\t\t\t"
                "Ryy (Ohm)\t\n")
        for r, (x, y, _) in enumerate(case.receivers):
            for i in order:
                o = resp[i, r]
                vals = list(o[MT_ZABS:MT_ZABS + 4]) + list(o[MT_RHO:MT_RHO + 4])
                f.write(f"{x:g}\t\t\t{-y + 0.0:g}\t\t{1.0 / freqs[i]:e}\t\t" +
                        "\t\t".join(f"{v:e}" for v in vals) + "\n")


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("case", help="directory with frequencies, xyzVectorB, z_sig_2d, objects, "
                                 "settings.cfg")
    ap.add_argument("--out", default=None, help="results table (default CASE/results_R_Z.txt)")
    ap.add_argument("--eps", type=float, default=None,
                    help="relative residual of the solves (default: settings.cfg's)")
    ap.add_argument("--maxiter", type=int, default=None)
    ap.add_argument("--results", default=None,
                    help="directory of calcimpedance's result files and edsall0_0_imp "
                         "(default CASE/Results; '-' writes none)")
    ap.add_argument("--output", choices=["smooth", "direct"], default="smooth",
                    help="receiver output: the reference's default subdomain smoothing, or the "
                         "direct evaluation of the edge basis at the receiver")
    a = ap.parse_args(argv)
    case = meshbuilder.read_case(a.case)
    if int(os.environ.get("WORLD_SIZE", "1")) > 1:   # torchrun: one process per GPU
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    resp, stats = run(case, a.eps, a.maxiter, log=lambda s: print(s, file=sys.stderr),
                      output=a.output)
    if resp is None:   # ranks other than 0
        return
    out = a.out or os.path.join(a.case, "results_R_Z.txt")
    write_table(out, case, resp)
    if a.results != "-":
        edsall.write_results(a.results or os.path.join(a.case, "Results"), case.freqs,
                             case.receivers, resp)
    with open(os.path.splitext(out)[0] + "_stats.json", "w") as f:
        json.dump(stats, f, indent=1)
    print(f"{out}: {len(case.receivers)} receivers x {len(case.freqs)} periods, "
          f"{stats['seconds']:.1f} s", file=sys.stderr)


if __name__ == "__main__":
    main()
