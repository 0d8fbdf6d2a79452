"""Generate the smoothing-output fixture from the reference's own code.

oracle/_ref/ref_smoothing (built by oracle/build_ref.sh) runs the
reference's default receiver output — the subdomain L2-projection smoothing
of Code/OutputNu (OutputResultant3d + Subdomain, PARDISO replaced by a
conjugate-gradient stand-in, oracle/ref_shim/pardiso_shim.cpp) — on:

  small   the `small` workload with the reference COCR_FP solutions stored in
          receivers_small.npz (both polarisations), at that fixture's
          receivers minus the one in the air (the reference stops when an
          E receiver lies in no earth cell);
  c1      the `c1` mesh (24^3 cells around the core, a layered earth and a
          conductive block) with seeded random edge values: the smoothing is
          linear in the solution, and on this mesh the five neighbour levels
          of the subdomains stop well inside the mesh.

It stores, per case, the receivers, ref_<case>[_<pol>] (12, R): the
smoothed Ax, Ay, Az, curl_x, curl_y, curl_z at the receivers, each as a
(real, imaginary) pair of rows, and sub_<case> (n, 2): the (nodes, bricks)
of every subdomain as the reference logs them (Subdomain.cpp:447-448), the
curl A subdomain first, then the A subdomains by material.

Usage (needs the reference sources; not run by the tests):
    python tests/golden/make_golden_smoothing.py [--ref REFERENCE_ROOT]
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

from mtcalc_with_dfp_cocr_gb300 import workloads  # noqa: E402

REF_BIN = os.path.join(ROOT, "oracle", "_ref")
C1_SEED = 20201217
C1_EXTRA = np.array([
    [-150.0, 50.0, 0.0],      # surface, inside a cell's top face
    [0.0, 0.0, -250.0],       # inside the block
    [220.0, -20.0, -60.0],    # earth, beside the block
    [-200.0, -200.0, -100.0], # on the block's corner
])


def c1_values(nb, seed=C1_SEED):
    """The seeded random edge values (nb, 2) of the c1 case."""
    return np.random.default_rng(seed).standard_normal((nb, 2))


def run_smoothing(m, rec, v3):
    nver = np.zeros((m.kpar, 14), np.int32)
    nver[:, :8] = m.cell_nodes()
    ed = np.zeros((m.kpar, 25), np.int32)
    ed[:, :12] = m.cell_edges()
    d = tempfile.mkdtemp(prefix="golden_smooth_")
    try:
        inp, out = os.path.join(d, "in.bin"), os.path.join(d, "out.bin")
        with open(inp, "wb") as f:
            np.array([m.nx - 1, m.ny - 1, m.nz - 1, m.kuzlov, m.kpar, m.nb, len(rec)],
                     "<i4").tofile(f)
            m.xyz().astype("<f8").tofile(f)
            nver.astype("<i4").tofile(f)
            ed.astype("<i4").tofile(f)
            m.nvkat.astype("<i4").tofile(f)
            np.asarray(rec, "<f8").tofile(f)
            np.asarray(v3, "<f8").tofile(f)
        log = subprocess.run([os.path.join(REF_BIN, "ref_smoothing"), inp, out], cwd=d,
                             check=True, capture_output=True, text=True).stdout
        subs = [(int(line.split()[2]), int(line.split()[4])) for line in log.splitlines()
                if line.startswith("Resultant mesh:")]
        return np.fromfile(out, "<f8").reshape(12, len(rec)), np.array(subs, np.int64)
    finally:
        shutil.rmtree(d, ignore_errors=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get(
        "MTCALC_REFERENCE_ROOT", os.path.join(os.path.dirname(ROOT), "reference")))
    a = ap.parse_args()
    subprocess.check_call([os.path.join(ROOT, "oracle", "build_ref.sh"), a.ref])
    out = {}
    g = np.load(os.path.join(HERE, "receivers_small.npz"))
    keep = g["rec"][:, 2] <= 0.0
    rec = g["rec"][keep]
    m = workloads.make("small").mesh
    out["rec_small"] = rec
    for p in ("x", "y"):
        out[f"ref_small_{p}"], out["sub_small"] = run_smoothing(m, rec, g[f"v3_{p}"])
    w = workloads.make("c1")
    rec = np.concatenate([w.receivers, C1_EXTRA])
    out["rec_c1"] = rec
    out["seed_c1"] = C1_SEED
    out["ref_c1"], out["sub_c1"] = run_smoothing(w.mesh, rec, c1_values(w.mesh.nb))
    for k, v in out.items():
        if k.startswith("ref_"):
            print(k, v.shape, "max |value|", np.abs(v).max())
        if k.startswith("sub_"):
            print(k, v.tolist())
    np.savez_compressed(os.path.join(HERE, "smoothing.npz"), **out)


if __name__ == "__main__":
    main()
