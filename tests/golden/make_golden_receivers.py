"""Generate the receiver-evaluation fixture from the reference programs.

For the `small` workload at 0.1 Hz and both polarisations it runs the
reference Harm1D -> BuildMatrix -> COCR_FP (built by oracle/build_ref.sh into
oracle/_ref/) and then oracle/_ref/ref_receivers, a harness around the
reference's own OutputVect3d::OutputFieldAtReceivers
(Code/OutputNu/OutputArbitrary.cpp:202-293).  It stores, per polarisation:

  v3          the reference solution
  e2d, b2d    the reference Harm1D normal field at the receivers (R, 6)
  ref_a       A at the receivers, (R, 3) complex        (derive 0, 1, 2)
  ref_curl    curl A at the receivers, (R, 3) complex   (derive 4, 5, 3)
  z1d, usin, ucos   the 1-D tables that BuildMatrix read

The receivers are the workload's 3x3 surface grid plus points inside cells,
on faces, in the air and in the padding, to exercise the location rule.

Usage (needs the reference sources; not run by the tests):
    python tests/golden/make_golden_receivers.py [--ref REFERENCE_ROOT]
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from make_golden import REF_BIN, run_reference  # noqa: E402
from mtcalc_with_dfp_cocr_gb300 import workloads  # noqa: E402

EXTRA_RECEIVERS = np.array([
    [-50.0, 30.0, 0.0],       # surface, inside a cell's top face
    [120.0, -170.0, -40.0],   # inside an earth cell
    [35.0, 55.0, 60.0],       # in the air
    [-200.0, 200.0, 0.0],     # on a core corner line
    [333.0, -10.0, 0.0],      # in the padding
    [0.0, 0.0, -100.0],       # on a layer/block interface node
    [10.0, -100.0, -250.0],   # on a face inside the block
])


def read_rows(path, n):
    with open(path) as f:
        rows = [list(map(float, line.split())) for line in f if line.strip()]
    return np.array(rows[:n])


def run_receivers(m, rec, v3):
    nver = np.zeros((m.kpar, 14), np.int32)
    nver[:, :8] = m.cell_nodes()
    ed = np.zeros((m.kpar, 25), np.int32)
    ed[:, :12] = m.cell_edges()
    d = tempfile.mkdtemp(prefix="golden_rcv_")
    try:
        inp, out = os.path.join(d, "in.bin"), os.path.join(d, "out.bin")
        with open(inp, "wb") as f:
            np.array([m.kuzlov, m.kpar, m.nb, len(rec)], "<i4").tofile(f)
            m.xyz().astype("<f8").tofile(f)
            nver.astype("<i4").tofile(f)
            ed.astype("<i4").tofile(f)
            np.asarray(rec, "<f8").tofile(f)
            np.asarray(v3, "<f8").tofile(f)
        subprocess.check_call([os.path.join(REF_BIN, "ref_receivers"), inp, out])
        res = np.fromfile(out, "<f8").reshape(2, 6, len(rec))
    finally:
        shutil.rmtree(d, ignore_errors=True)
    c = res[0] + 1j * res[1]                      # (6, R): derive 0..5
    return np.stack([c[0], c[1], c[2]], 1), np.stack([c[4], c[5], c[3]], 1)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get(
        "MTCALC_REFERENCE_ROOT", os.path.join(os.path.dirname(ROOT), "reference")))
    a = ap.parse_args()
    subprocess.check_call([os.path.join(ROOT, "oracle", "build_ref.sh"), a.ref])
    w = workloads.make("small")
    rec = np.concatenate([w.receivers, EXTRA_RECEIVERS])
    w = workloads.Workload(w.name, w.mesh, w.freqs, rec)
    nu = 0.1
    out = {"nu": nu, "rec": rec}
    for alfa in (1, 0):
        d = tempfile.mkdtemp(prefix="golden_rcv_run_")
        try:
            s, (z1d, usin, ucos), v3, kit = run_reference(d, w, nu, alfa)
            e2d = read_rows(os.path.join(d, "e2d"), len(rec))
            b2d = read_rows(os.path.join(d, "b2d"), len(rec))
        finally:
            shutil.rmtree(d, ignore_errors=True)
        ref_a, ref_curl = run_receivers(w.mesh, rec, v3)
        p = "x" if alfa == 1 else "y"
        out.update({f"v3_{p}": v3, f"e2d_{p}": e2d, f"b2d_{p}": b2d, f"ref_a_{p}": ref_a,
                    f"ref_curl_{p}": ref_curl, f"z1d_{p}": z1d, f"usin_{p}": usin,
                    f"ucos_{p}": ucos})
        print("polarisation", p, "iterations", kit[2], "max|A|", np.abs(ref_a).max(),
              "max|curl A|", np.abs(ref_curl).max())
    np.savez_compressed(os.path.join(HERE, "receivers_small.npz"), **out)


if __name__ == "__main__":
    main()
