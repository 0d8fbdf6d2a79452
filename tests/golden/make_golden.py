"""Generate the golden fixtures from the reference programs themselves.

Runs the reference Harm1D -> BuildMatrix -> COCR_FP, built from the
reference sources by oracle/build_ref.sh into oracle/_ref/, on synthetic
meshes written by this package's generator, and stores what they produce:

  tiny.npz, small.npz   full fixtures: the 1-D normal field tables, the
                        assembled block SLAE, the solution v3.dat and kit
  c1_summary.json       the 24x24x24 benchmark case at 1 Hz, both
                        polarisations: SLAE sizes and checksums, iteration
                        counts, solution norms and seeded sample entries

Usage (needs the reference sources; not run by the tests):
    python tests/golden/make_golden.py [--ref REFERENCE_ROOT]
"""
from __future__ import annotations

import argparse
import json
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from mtcalc_with_dfp_cocr_gb300 import normal1d, slae_io, workloads  # noqa: E402

REF_BIN = os.path.join(ROOT, "oracle", "_ref")


def run_reference(workdir, w, nu, alfa, eps=1e-8, maxiter=10000):
    w.mesh.write(workdir, nu=nu, alfa=alfa, eps=eps, maxiter=maxiter, nthreads=1,
                 receivers=w.receivers)
    for prog in ("Harm1D", "BuildMatrix", "COCR_FP"):
        r = subprocess.run([os.path.join(REF_BIN, prog)], cwd=workdir, capture_output=True,
                           text=True)
        if r.returncode != 0:
            raise RuntimeError(f"{prog} failed: {r.stdout[-2000:]}\n{r.stderr[-2000:]}")
    s = slae_io.read_slae(workdir)
    z1d, usin, ucos = normal1d.read_tables(workdir)
    v3 = slae_io.read_v3(os.path.join(workdir, "v3.dat"), s.n)
    kit = slae_io.read_kit(os.path.join(workdir, "kit"))
    return s, (z1d, usin, ucos), v3, kit


def full_fixture(name, nu, alfa):
    w = workloads.make(name)
    d = tempfile.mkdtemp(prefix=f"golden_{name}_")
    try:
        s, (z1d, usin, ucos), v3, kit = run_reference(d, w, nu, alfa)
    finally:
        shutil.rmtree(d, ignore_errors=True)
    np.savez_compressed(
        os.path.join(HERE, f"{name}.npz"), nu=nu, alfa=alfa, eps=s.eps, maxiter=s.maxiter,
        ig=s.ig, jg=s.jg, idi=s.idi, ijg=s.ijg, di=s.di, gg=s.gg, pr=s.pr,
        z1d=z1d, usin=usin, ucos=ucos, v3=v3, kit_r=kit[0], kit_iter=kit[2])
    print(name, "nb", s.nb, "iterations", kit[2], "r", kit[0])


def c1_summary():
    w = workloads.make("c1")
    out = {"case": "c1", "systems": []}
    rng = np.random.default_rng(1234)
    for nu, alfa in w.systems:
        d = tempfile.mkdtemp(prefix="golden_c1_")
        try:
            s, (z1d, usin, ucos), v3, kit = run_reference(d, w, nu, alfa)
        finally:
            shutil.rmtree(d, ignore_errors=True)
        idx = np.sort(rng.choice(s.nb, 64, replace=False))
        xc = v3[0::2] + 1j * v3[1::2]
        A = None  # the dense matrix is too large here; the residual is checked by the tests
        out["systems"].append({
            "nu": float(nu), "alfa": int(alfa), "nb": int(s.nb), "nnz_lower": int(s.ig[-1]),
            "di_len": int(s.idi[-1]), "gg_len": int(s.ijg[-1]),
            "sum_di": float(s.di.sum()), "sum_abs_gg": float(np.abs(s.gg).sum()),
            "sum_abs_pr": float(np.abs(s.pr).sum()), "norm_pr": float(np.linalg.norm(s.pr)),
            "iterations": int(kit[2]), "kit_r": float(kit[0]),
            "norm_v3": float(np.linalg.norm(v3)),
            "sample_index": idx.tolist(),
            "sample_re": xc[idx].real.tolist(), "sample_im": xc[idx].imag.tolist(),
            "usin_top": float(usin[-1]), "ucos_top": float(ucos[-1]), "n1d": int(len(z1d)),
        })
        del A
        print("c1", nu, alfa, "iterations", kit[2])
    with open(os.path.join(HERE, "c1_summary.json"), "w") as f:
        json.dump(out, f, indent=1)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get(
        "MTCALC_REFERENCE_ROOT", os.path.join(os.path.dirname(ROOT), "reference")))
    a = ap.parse_args()
    subprocess.check_call([os.path.join(ROOT, "oracle", "build_ref.sh"), a.ref])
    full_fixture("tiny", 1.0, 1)
    full_fixture("small", 0.1, 0)
    c1_summary()


if __name__ == "__main__":
    main()
