"""Golden MT responses of the benchmark-size workloads, for the GPU parity
tests at the benchmark sizes (tests/test_gpu_bench_parity.py).

c2 (96x96x64 cells, 1,812,736 edges, 0.1 Hz, both polarisations) runs the
reference's own programs, built from its sources by oracle/build_ref.sh
(Harm1D -> BuildMatrix -> COCR_FP with 7 OpenMP threads), exactly as
tests/golden/make_c2_summary.py does; c3 (64x64x48 cells, 610,480 edges,
16 frequencies 1e-3..1e3 Hz x 2 polarisations = 32 systems) runs the
oracle's FP64 port of COCR_FP (pinned to the reference's iterates on the
small golden cases) on the oracle's assembly.  For every system the script
keeps the iteration count, the smoothed stop residual, the FP64 true
relative residual ||b - A x|| / ||b|| (the oracle's SpMV on the SLAE), and
the fields at the workload's surface receivers through the oracle's receiver
evaluation (pinned to OutputNu's direct evaluation); per frequency it keeps
the MT responses (calcimpedance's Z, |Z|, phase, rho_a) of every receiver.

Usage:
    python tests/golden/make_oracle_surveys.py c2     (needs oracle/_ref built)
    python tests/golden/make_oracle_surveys.py c3 [--threads 8]
"""
import argparse
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

from mtcalc_with_dfp_cocr_gb300 import normal1d, slae_io, workloads  # noqa: E402
from oracle import pyoracle as O  # noqa: E402

REF_BIN = os.path.join(ROOT, "oracle", "_ref")
TWO_PI = 2.0 * 3.1415926535897932384626433832795
# the record fields kept: Z (re, im) x 4, |Z| x 4, -arg Z [deg] x 4, rho_a x 4
KEEP = list(range(0, 8)) + list(range(12, 24))


def _reference_system(w, nu, alfa, threads):
    d = tempfile.mkdtemp(prefix=f"survey_{w.name}_")
    try:
        w.mesh.write(d, nu=nu, alfa=alfa, eps=1e-8, maxiter=20000, nthreads=threads,
                     receivers=w.receivers)
        for prog in ("Harm1D", "BuildMatrix", "COCR_FP"):
            r = subprocess.run([os.path.join(REF_BIN, prog)], cwd=d, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"{prog} failed: {r.stdout[-2000:]}\n{r.stderr[-2000:]}")
        s = slae_io.read_slae(d)
        tabs = normal1d.read_tables(d)
        x = slae_io.read_v3(os.path.join(d, "v3.dat"), s.n)
        kit = slae_io.read_kit(os.path.join(d, "kit"))
        return s, tabs, x, int(kit[2]), float(kit[0])
    finally:
        shutil.rmtree(d, ignore_errors=True)


def _oracle_system(w, nu, alfa, threads):
    tops, sig = [l.top for l in w.mesh.layers], [l.sigma for l in w.mesh.layers]
    tabs = normal1d.solve_1d(nu, tops, sig)
    s = O.assemble(w.mesh, nu, alfa, *tabs, eps=1e-8, maxiter=20000)
    code, x, st = O.pcocr(s, slae_io.mesh_to_solve_mesh(w.mesh), nthreads=threads)
    if code != 0:
        raise RuntimeError(f"oracle solve of {nu} Hz / {alfa} returned {code}")
    return s, tabs, x, int(st.iterations), float(st.residual_rel)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=["c2", "c3"])
    ap.add_argument("--threads", type=int, default=7)
    a = ap.parse_args()
    w = workloads.make(a.case)
    systems = w.systems
    R = len(w.receivers)
    fields, iters, kit_r, true_rel, secs = [], [], [], [], []
    for nu, alfa in systems:
        t0 = time.time()
        run = _reference_system if a.case == "c2" else _oracle_system
        s, (z1d, us, uc), x, it, rr = run(w, nu, alfa, a.threads)
        tr = np.linalg.norm(s.pr - O.spmv(s, x, nthreads=a.threads)) / np.linalg.norm(s.pr)
        av, curl = O.receiver_eval(w.mesh, w.receivers, x)
        e1, b1 = O.normal_field(w.receivers, z1d, us, uc, alfa, TWO_PI * nu)
        E, H, _ = O.receiver_fields(av, curl, TWO_PI * nu, e1, b1)
        fields.append((E, H))
        iters.append(it)
        kit_r.append(rr)
        true_rel.append(tr)
        secs.append(time.time() - t0)
        print(f"{a.case} {nu:.4g} Hz alfa {alfa}: {it} iterations, stop {rr:.3e}, "
              f"true {tr:.3e}, {secs[-1]:.1f} s", flush=True)
    freqs = np.asarray(w.freqs, np.float64)
    mt = np.zeros((len(freqs), R, len(KEEP)))
    for f, nu in enumerate(freqs):
        (e0, h0), (e1_, h1) = fields[2 * f], fields[2 * f + 1]
        for r in range(R):
            rec = O.mt_response(e0[r], h0[r], e1_[r], h1[r], TWO_PI * nu)
            mt[f, r] = rec[KEEP]
    np.savez_compressed(
        os.path.join(HERE, f"{a.case}_survey.npz"), freqs=freqs,
        nu=np.array([s[0] for s in systems]), alfa=np.array([s[1] for s in systems]),
        iterations=np.array(iters), stop_residual=np.array(kit_r), true_rel=np.array(true_rel),
        receivers=w.receivers, mt=mt, keep=np.array(KEEP),
        source=("reference COCR_FP (oracle/_ref), %d threads" % a.threads if a.case == "c2"
                else "oracle port of COCR_FP, %d threads" % a.threads))


if __name__ == "__main__":
    main()
