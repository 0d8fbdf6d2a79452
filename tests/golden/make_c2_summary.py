"""Run the reference programs (built by oracle/build_ref.sh) on the 96x96x64
benchmark workload (c2, 0.1 Hz, both polarisations) with 7 OpenMP threads
(the reference cap omp_get_max_threads()-1 on this 8-core host) and record
what the CPU baseline needs: iteration counts, kit times and solution norms.

Usage: python tests/golden/make_c2_summary.py   (needs oracle/_ref built)
"""
import json
import os
import shutil
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from mtcalc_with_dfp_cocr_gb300 import slae_io, workloads  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref")


def main():
    w = workloads.make("c2")
    out = {"case": "c2", "threads": 7, "host": "8-core x86_64 (Xeon @ 2.7 GHz)", "systems": []}
    for nu, alfa in w.systems:
        d = tempfile.mkdtemp(prefix="c2ref_")
        try:
            w.mesh.write(d, nu=nu, alfa=alfa, eps=1e-8, maxiter=20000, nthreads=7,
                         receivers=w.receivers)
            times = {}
            for prog in ("Harm1D", "BuildMatrix", "COCR_FP"):
                t0 = time.time()
                r = subprocess.run([os.path.join(REF, prog)], cwd=d, capture_output=True, text=True)
                times[prog] = time.time() - t0
                if r.returncode != 0:
                    raise RuntimeError(prog + r.stdout[-1000:] + r.stderr[-1000:])
            kit = slae_io.read_kit(os.path.join(d, "kit"))
            s = slae_io.read_slae(d)
            v3 = slae_io.read_v3(os.path.join(d, "v3.dat"), s.n)
            out["systems"].append({"nu": nu, "alfa": alfa, "iterations": kit[2], "kit_r": kit[0],
                                   "kit_seconds": kit[3], "wall_seconds": times,
                                   "norm_v3": float(np.linalg.norm(v3)), "nb": s.nb,
                                   "nnz_lower": int(s.ig[-1])})
            print(out["systems"][-1], flush=True)
        finally:
            shutil.rmtree(d, ignore_errors=True)
    with open(os.path.join(HERE, "c2_summary.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
