"""Benchmark: time per solve to true relative residual 1e-8 on the
96x96x64-cell survey mesh (1.8M edges, 0.1 Hz, both polarisations):
the batched double-float solver, with the plain FP64 GPU COCR beside it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference]

GPU arm (default).  A step solves every system of the workload together
from the device-resident assembly with the batched survey solver (set-up of
the batch included): the reference's COCR with the folded preconditioner and
MRS stop rule, in double-float arithmetic (FP32 pairs, 48-bit significand)
on the FP32 pipes, which GB300 runs at 64x its FP64 rate; each system also
continues until its true residual ||b - A x|| / ||b|| is below 1e-8.
(Plain FP32 iterations do not converge on these systems: the air layer
leaves the curl-curl null space regularised below FP32 resolution.)  `value` is seconds
per solve (lower is better) from CUDA events on the solver's stream; the
iteration's working set (twelve vectors of 58 MB plus the SpMV's matrix or
face arrays) is several times L2, so no flush is needed between
iterations.
`plain_fp64` times the reference's FP64 algorithm on the GPU on the same
systems.  `e2e` goes through the reference-facing C ABI
(mtgpu_pcocr_2x2_folded_ex, double-float) with the SLAE in host memory:
upload, set-up, solve and download of x every solve.  `roofline` is the
batched double-float SpMV, in the variant the set-up autotuning chose (on
this tensor mesh the matrix-free one), against the measured HBM copy
bandwidth.  The timed region is an NVTX range "timed" for ncu's
--nvtx-include.

Reference arm (--impl reference).  The reference's CPU algorithm (the
oracle restatement of COCR_FP with the reference's thread cap, nproc - 1)
on the headline system: every timed step is one whole solve (set-up and
iterations to the reference's stop rule), in a process of its own
(oracle/cpu_solve.py).  `cpu_baseline` of the GPU arm is one such solve.

Multi-GPU: systems are independent (replicas over the survey's systems);
every rank solves its own copy of the workload and `value` is the
whole-job seconds per solve (total time / total solves).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "time/solve to rel-res 1e-8: batched mixed vs plain FP64 GPU; SpMV HBM GB/s"
UNIT = "s/solve"
WORKLOAD = "c2"
# DRAM bytes of one matrix-free SpMV on c2 (two lanes, as the iteration
# launches it), per variant: the sum of its kernels' ncu dram__bytes_read.sum
# + dram__bytes_write.sum (profiles/bench_c2_launch_list.md,
# profiles/spmv_matfree_c2_s2.md: variant 32's k_mf_faces + k_mf_edges,
# variant 35's k_mf_gmarch + k_mf_edges_g)
SPMV_MF_TRAFFIC_C2 = {32: 300.6e6, 35: 314.3e6}
# what bounds the matrix-free SpMV instead of HBM (ncu on c2, two lanes)
SPMV_MF_BINDING = ("FP32 issue: k_mf_edges<2> 69 % issue-active, 51 % FMA pipe, 42 double-float "
                   "multiply-adds of 12 FP32 instructions per edge and system "
                   "(profiles/spmv_matfree_c2_s2.md)")


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ref_iterations():
    """The reference's own iteration counts for the workload's systems, or
    None when they have not been pinned."""
    p = os.path.join(ROOT, "tests", "golden", "c2_summary.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        d = json.load(f)
    return {(s["nu"], s["alfa"]): s["iterations"] for s in d["systems"]}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [t.strip() for t in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = max(smax, float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": smax or None, "reasons": sorted(reasons), "samples": len(sm)}


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(value, device):
    """The largest of every rank's value (the job's time is its slowest
    rank's); the value itself without a process group."""
    import torch
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return value
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_seconds_per_solve(ms, steps, systems_per_rank, world):
    """Replicas: every rank solves its own copy of the workload, so the job
    solves steps x systems x world systems in the slowest rank's time."""
    return (ms / 1e3) / (steps * systems_per_rank * world)


def cpu_model():
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    import platform
    return platform.processor() or platform.machine()


def make_inputs(w):
    from mtcalc_with_dfp_cocr_gb300 import normal1d
    tops = [l.top for l in w.mesh.layers]
    sig = [l.sigma for l in w.mesh.layers]
    tables = {}
    for nu in sorted(set(f for f, _ in w.systems)):
        tables[nu] = normal1d.solve_1d(nu, tops, sig)
    return tables


# ------------------------------------------------------------------- GPU arm
def gpu_arm(args):
    import torch
    world, rank, local = dist_init()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from mtcalc_with_dfp_cocr_gb300 import _lib, assembly, slae_io, solver, survey, workloads
    from mtcalc_with_dfp_cocr_gb300 import build as B
    B.build()

    w = workloads.make(WORKLOAD)
    systems = w.systems
    S = len(systems)
    tables = make_inputs(w)
    nb = w.mesh.nb
    nus = [f for f, _ in systems]
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    A = assembly.Assembly(w.mesh)
    z1d = tables[systems[0][0]][0]
    rhs = torch.empty(S, 2 * nb, dtype=torch.float64, device="cuda")
    A.rhs(nus, [a for _, a in systems], z1d, np.stack([tables[f][1] for f in nus]),
          np.stack([tables[f][2] for f in nus]), rhs)
    x = torch.zeros_like(rhs)
    eps, maxiter = 1e-8, 20000
    info = {}

    def step_batched():
        sv = survey.Survey(A, nus, stream)
        x.zero_()
        code, st = sv.solve(rhs, x, eps=eps, maxiter=maxiter, verify=True)
        if code != 0:
            raise RuntimeError(f"survey solve failed: {st}")
        info["batched"] = st
        sv.close()

    def step_plain():
        for nu in sorted(set(nus)):
            ctx = A.cocr(nu, stream)
            for k, (f, a) in enumerate(systems):
                if f != nu:
                    continue
                x[k].zero_()
                code, st = ctx.solve(rhs[k], x[k], eps=eps, maxiter=maxiter,
                                     stop_on_true_residual=True)
                if code != 0:
                    raise RuntimeError(f"solve failed with code {code}")
                info.setdefault("plain", {})[(f, a)] = (st.iterations, st.true_residual_rel)
            ctx.close()

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    def timed(fn, steps):
        barrier()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(steps):
            fn()
        ev1.record(stream)
        barrier()
        return max_over_ranks(ev0.elapsed_time(ev1), "cuda")

    # headline: the batched double-float solver
    for _ in range(args.warmup):
        step_batched()
    launches0 = _lib.kernel_launches()
    torch.cuda.nvtx.range_push("timed")   # lets ncu capture the timed region alone
    with ClockSampler(local) as clk:
        ms = timed(step_batched, args.steps)
    torch.cuda.nvtx.range_pop()
    launches = _lib.kernel_launches() - launches0
    ms_per_step = ms / args.steps
    value = whole_job_seconds_per_solve(ms, args.steps, S, world)
    batched = info["batched"]

    # per-result error of the headline solutions against the FP64 answers
    # of the reference's own COCR_FP (tests/golden/c2_survey.npz, made by
    # tests/golden/make_oracle_surveys.py) at the workload's receivers
    oracle_err = oracle_parity(w, systems, tables, A, x)

    # comparison: the plain FP64 COCR (the reference's algorithm) on the GPU
    step_plain()
    plain_steps = max(1, min(args.steps, 2))
    ms_plain = timed(step_plain, plain_steps)
    plain_value = (ms_plain / 1e3) / (plain_steps * S * world)

    # roofline of the dominant kernel: the batched double-float SpMV, in the
    # variant the set-up autotuning chose
    peak, peak_kind = load_peaks()
    sv = survey.Survey(A, nus, stream)
    variant = sv.tuning()[0]
    sv.spmv_timed(5)
    reps = 50
    spmv_ms = sv.spmv_timed(reps) / reps
    sv.close()
    inf = A.info()
    nc, nr = inf["nnz_complex"], inf["nnz_real"]
    nslices = (nb + 31) // 32
    meta = nslices * (8 + 8 + 4 + 4)
    SP = 1 << (S - 1).bit_length()
    m_ = w.mesh
    # as the iteration launches it: z = A s and (z, s) (the MRS smoothing
    # runs in k_update)
    tail = 0
    if variant in (32, 33, 35):
        # matrix-free, per launch as the iteration runs it.  Variants 32/33:
        # the faces kernel reads s and writes the face circulations f, the
        # edges kernel reads f, s, the six double-float weights of every cell
        # and the row positions and writes z.  Variant 35: k_mf_gmarch reads
        # s and the cells' face weights and writes g = F f per face, the
        # edges kernel reads g, s, the cells' mass weights and the row
        # positions and writes z.  Each value counted once: the same bytes.
        nx_, ny_, nz_ = m_.nx, m_.ny, m_.nz
        nf = nx_ * (ny_ - 1) * (nz_ - 1) + (nx_ - 1) * ny_ * (nz_ - 1) + (nx_ - 1) * (ny_ - 1) * nz_
        spmv_bytes = 16 * SP * (3 * nb + 2 * nf) + 48 * m_.kpar + 4 * nb + tail
        if variant == 35:
            spmv_kernel = ("k_mf_gmarch + k_mf_edges_g (matrix-free double-float SpMV, g = F f "
                           "formed per face from s, S systems)")
        else:
            edges = "k_mf_edges2" if variant == 33 else "k_mf_edges"
            spmv_kernel = f"k_mf_faces + {edges} (matrix-free double-float SpMV, S systems)"
        traffic = SPMV_MF_TRAFFIC_C2.get(variant) if WORKLOAD == "c2" else None
        traffic_src = (f"ncu dram__bytes_read.sum + dram__bytes_write.sum of the variant-{variant} "
                       f"kernels on c2 (profiles/bench_c2_launch_list.md)") if traffic else None
    else:
        spmv_bytes = nc * (4 + 8 + 8) + nr * (4 + 8) + meta + 2 * S * 16 * nb + tail
        spmv_kernel = f"k_spmv variant {variant} (batched double-float SELL-32 SpMV, S systems)"
        traffic = None
        traffic_src = None
    achieved = spmv_bytes / (spmv_ms * 1e-3) / 1e9
    # the whole iteration against HBM: the algorithmic bytes of its five
    # kernels (node: z, a gathered, D_S read, h written; edge: s, p, z, a,
    # D_A, x read, p, a, w, x written, h gathered, the compact G^T row;
    # update: a, w, s_m, r, s read, r, s, s_m written; the SpMV as above)
    # over the solve's time per iteration (its set-up and FP64 checks
    # included); m = the interior nodes, the rows of G on these meshes
    m_nodes = (m_.nx - 2) * (m_.ny - 2) * (m_.nz - 2)
    iter_bytes = 16 * SP * (20 * nb + 3 * m_nodes) + 8 * nb + spmv_bytes
    iter_ms = 1e3 * batched["seconds"] / max(batched["iterations"])
    # the FP64 SpMV of the plain path (bound by the FP64 pipe on GB300)
    ctx = A.cocr(nus[0], stream)
    xs = torch.randn(2 * nb, dtype=torch.float64, device="cuda")
    ys = torch.empty_like(xs)
    ctx.spmv_timed(xs, ys, 5)
    spmv64_ms = ctx.spmv_timed(xs, ys, reps) / reps
    ctx.close()
    spmv64_bytes = nc * (16 + 4) + nr * (8 + 4) + meta + 2 * 16 * nb
    achieved64 = spmv64_bytes / (spmv64_ms * 1e-3) / 1e9

    # e2e through the reference-facing C ABI with host buffers: every SLAE
    # array and x in pinned host memory (filled before the timed region)
    mesh_h = slae_io.mesh_to_solve_mesh(w.mesh)

    def pinned(v):
        t_ = torch.empty(v.shape, dtype=torch.from_numpy(np.ascontiguousarray(v)).dtype,
                         pin_memory=True).numpy()
        t_[...] = v
        return t_
    # the mesh tables the call uploads (cell nodes and materials, edges,
    # Dirichlet flags, node coordinates, material flags) pinned too, in the
    # types the call takes
    for fld, dt in (("xyz", np.float64), ("nvkat", np.int32), ("nver", np.int32),
                    ("sigma", np.float64), ("edges", np.int32), ("is_node_bound", np.int32)):
        setattr(mesh_h, fld, pinned(np.ascontiguousarray(getattr(mesh_h, fld), dtype=dt)))
    mesh_bytes = (mesh_h.xyz.nbytes + mesh_h.nvkat.nbytes + mesh_h.nver.nbytes +
                  mesh_h.sigma.nbytes + mesh_h.edges.nbytes + mesh_h.is_node_bound.nbytes)
    host, xpin = {}, {}
    for k, (f, a) in enumerate(systems):
        t = tables[f]
        s = A.block2x2(f, a, t[0], t[1], t[2], eps=eps, maxiter=maxiter)
        for fld in ("ig", "jg", "idi", "ijg", "di", "gg", "pr"):
            setattr(s, fld, pinned(getattr(s, fld)))
        host[k] = s
        xpin[k] = pinned(np.zeros(s.n))
    h2d = d2h = 0
    e2e_steps = max(1, min(args.steps, 3))
    e2e_setup = e2e_solve = 0.0
    e2e_calls = []
    # one untimed call first, as the batched arm has its warm-up steps: the
    # process's first one-system solve loads that width's kernels
    xpin[0][:] = 0.0
    solver.pcocr_2x2_folded(host[0], mesh_h, double_float=True, stop_on_true_residual=True,
                            x=xpin[0])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        for k in range(S):
            s = host[k]
            xpin[k][:] = 0.0
            code, xh, st = solver.pcocr_2x2_folded(s, mesh_h, double_float=True,
                                                   stop_on_true_residual=True, x=xpin[k])
            if code != 0:
                raise RuntimeError(f"e2e solve failed with code {code}")
            e2e_setup += st.setup_seconds
            e2e_solve += st.solve_seconds
            e2e_calls.append(round(st.setup_seconds * 1e3, 2))
            h2d += (s.ig.nbytes + s.jg.nbytes + s.idi.nbytes + s.ijg.nbytes + s.di.nbytes +
                    s.gg.nbytes + s.pr.nbytes + xh.nbytes + mesh_bytes)
            d2h += xh.nbytes
    e2e_s = (time.perf_counter() - t0) / (e2e_steps * S)
    A.close()

    lab = lambda f, a: f"{f}Hz/{'XY'[1 - a]}"
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "double-float (FP32 pairs, 48-bit significand) complex; FP64 scalars",
        "data": "synthetic (seeded layered earth + 20 random blocks, reference file formats)",
        "config": {"workload": "c2: 96x96x64 cells, 1,812,736 edges, 0.1 Hz x 2 polarisations; "
                               "batched double-float COCR + folded preconditioner + MRS stop "
                               "rule, every system also to true rel-res < 1e-8",
                   "systems_per_step": S, "nb": nb, "l2_flush": "none: the iteration's working set (12 double-float vectors of 58 MB, the SpMV's matrix or face arrays) exceeds L2 (129 MB)",
                   "iterations": {lab(f, a): it for (f, a), it in zip(systems, batched["iterations"])},
                   "true_rel_res": {lab(f, a): r for (f, a), r in zip(systems, batched["true_residual_rel"])},
                   "parallelism": f"replicas x{world}"},
        "plain_fp64": {"value": plain_value, "unit": UNIT,
                       "iterations": {lab(f, a): v[0] for (f, a), v in info["plain"].items()},
                       "true_rel_res": {lab(f, a): v[1] for (f, a), v in info["plain"].items()},
                       "speedup_of_batched_double_float": plain_value / value},
        "roofline": {"bound": "hbm", "kernel": spmv_kernel, "spmv_variant": variant,
                     "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": f"{peak_kind} hbm_gbs",
                     "bytes_per_launch": spmv_bytes, "ms_per_launch": spmv_ms,
                     "traffic": traffic, "traffic_source": traffic_src,
                     "binding": SPMV_MF_BINDING if variant in (32, 33, 35) else None},
        "roofline_iteration": {"bound": "hbm", "achieved": iter_bytes / (iter_ms * 1e-3) / 1e9,
                               "peak": peak, "unit": "GB/s",
                               "frac": iter_bytes / (iter_ms * 1e-3) / 1e9 / peak,
                               "bytes_per_iteration": iter_bytes, "ms_per_iteration": iter_ms},
        "roofline_fp64_spmv": {"bound": "fp64 pipe (GB300 FP64 = FP32/64)",
                               "achieved": achieved64, "peak": peak, "unit": "GB/s",
                               "frac": achieved64 / peak, "bytes_per_launch": spmv64_bytes,
                               "ms_per_launch": spmv64_ms},
        "e2e": {"value": e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d // e2e_steps,
                "d2h_bytes_per_step": d2h // e2e_steps,
                "setup_seconds_per_solve": e2e_setup / (e2e_steps * S),
                "solve_seconds_per_solve": e2e_solve / (e2e_steps * S),
                "setup_ms_per_call": e2e_calls,
                "path": "mtgpu_pcocr_2x2_folded_ex(double_float=1, stop_on_true_residual=1), pinned host SLAE, mesh and x buffers"},
        "oracle_parity": oracle_err,
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
    }
    if rank == 0 and world == 1 and not args.no_survey:
        # the benchmark spec's survey case: 16 frequencies x 2 polarisations on
        # the headline mesh in one batch, against the plain FP64 COCR
        out["survey_c2s"] = survey_compare("c2s", 1, 0, setup_device=False)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        import tempfile
        s0 = host[0]
        with tempfile.TemporaryDirectory() as td:
            f = os.path.join(td, "slae.npz")
            np.savez(f, ig=s0.ig, jg=s0.jg, idi=s0.idi, ijg=s0.ijg, di=s0.di, gg=s0.gg, pr=s0.pr,
                     eps=s0.eps, maxiter=s0.maxiter)
            pinned = ref_iterations()
            out["cpu_baseline"] = cpu_baseline(systems[0], f,
                                               pinned[systems[0]] if pinned else None)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def oracle_parity(w, systems, tables, A, x):
    """Errors of the batched solutions' MT responses against the reference's
    FP64 COCR_FP answers, per receiver result: Z of every component relative
    to the tensor's off-diagonal scale, |Z| and rho_a of Zxy, Zyx relative,
    their phases in degrees."""
    from mtcalc_with_dfp_cocr_gb300 import receivers
    p = os.path.join(ROOT, "tests", "golden", f"{WORKLOAD}_survey.npz")
    if not os.path.exists(p):
        return None
    g = np.load(p)
    nus = [f for f, _ in systems]
    alfas = [a for _, a in systems]
    z1d = tables[nus[0]][0]
    us = np.stack([tables[f][1] for f in nus])
    uc = np.stack([tables[f][2] for f in nus])
    R = receivers.Receivers(A, w.receivers)
    freqs = sorted(set(nus))
    if not np.allclose(freqs, g["freqs"], rtol=1e-14):
        return None
    sx = [systems.index((f, 1)) for f in freqs]
    sy = [systems.index((f, 0)) for f in freqs]
    E, H, _ = R.fields(x, nus, alfas, z1d, us, uc)
    mt = R.mt_response(freqs, sx, sy, E, H).cpu().numpy()[..., g["keep"]]
    R.close()
    ref = g["mt"]
    z = mt[..., 0:8:2] + 1j * mt[..., 1:8:2]
    zr = ref[..., 0:8:2] + 1j * ref[..., 1:8:2]
    off = [1, 2]
    scale = np.abs(zr[..., off]).max(axis=-1, keepdims=True)
    ph = np.abs(mt[..., 12:16][..., off] - ref[..., 12:16][..., off]) % 360.0
    return {"reference": str(g["source"]), "receivers": int(len(w.receivers)),
            "Z_rel_to_offdiag_max": float((np.abs(z - zr) / scale).max()),
            "Zabs_offdiag_rel_max": float((np.abs(mt[..., 8:12][..., off] - ref[..., 8:12][..., off])
                                           / ref[..., 8:12][..., off]).max()),
            "rho_a_offdiag_rel_max": float((np.abs(mt[..., 16:20][..., off] - ref[..., 16:20][..., off])
                                            / ref[..., 16:20][..., off]).max()),
            "phase_offdiag_deg_max": float(np.minimum(ph, 360.0 - ph).max()),
            "iterations_reference": [int(v) for v in g["iterations"]],
            "true_rel_reference": [float(v) for v in g["true_rel"]]}


# --------------------------------------------------------------- CPU baseline
def cpu_threads():
    """The reference's OpenMP cap, omp_get_max_threads() - 1
    (Code/COCR_FP/ControlOMP.cpp:46), on this host."""
    return max(1, (os.cpu_count() or 2) - 1)


def run_cpu_solves(key, threads, slae_file=None, warmup=0, steps=1, sample_iterations=0):
    """Whole solves of the oracle's COCR_FP restatement in a process of its
    own (oracle/cpu_solve.py): nothing else shares its cores or OpenMP
    runtime, in either arm."""
    cmd = [sys.executable, "-m", "oracle.cpu_solve", WORKLOAD, str(float(key[0])), str(int(key[1])),
           str(threads), "--warmup", str(warmup), "--steps", str(steps),
           "--sample-iterations", str(sample_iterations)]
    if slae_file:
        cmd += ["--slae", slae_file]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"CPU solve failed: {r.stdout[-2000:]}\n{r.stderr[-2000:]}")
    return json.loads(r.stdout.strip().splitlines()[-1])


def one_thread_estimate(key, slae_file, iterations):
    """The reference's default (nthreads.txt = 1): a whole one-thread solve
    takes minutes, so set-up + 5 and set-up + 45 iterations are timed and
    the solve is extrapolated to `iterations`."""
    a = run_cpu_solves(key, 1, slae_file, sample_iterations=5)["seconds"][0]
    b = run_cpu_solves(key, 1, slae_file, sample_iterations=45)["seconds"][0]
    per = (b - a) / 40.0
    return max(0.0, a - 5 * per) + per * iterations


def cpu_baseline(key, slae_file, ref_iters):
    """One whole solve of the headline system with the reference's thread
    cap, timed on the wall clock (set-up included, as the reference's kit
    time), plus the one-thread estimate."""
    threads = cpu_threads()
    r = run_cpu_solves(key, threads, slae_file, warmup=1, steps=1)
    t, it = r["seconds"][0], r["iterations"][0]
    return {"value": t, "unit": UNIT, "cores": threads, "kind": "port",
            "cpu_model": cpu_model(), "iterations": it,
            "iterations_reference": ref_iters, "true_rel": r["true_rel"],
            "value_1_thread_estimate": one_thread_estimate(key, slae_file, it),
            "sample": f"one whole solve of the {key[0]} Hz / {'XY'[1 - key[1]]} system (set-up + "
                      f"{it} iterations to the reference's stop rule) by the oracle's COCR_FP "
                      f"restatement with {threads} threads (the reference's cap, nproc - 1), "
                      f"in a process of its own; value_1_thread_estimate: set-up + 45 iterations "
                      f"on one thread, extrapolated to {it}"}


def reference_arm(args):
    world, rank, local = dist_init()
    if rank != 0:
        return
    from mtcalc_with_dfp_cocr_gb300 import workloads
    w = workloads.make(WORKLOAD)
    key = w.systems[0]
    threads = cpu_threads()
    t0 = time.perf_counter()
    r = run_cpu_solves(key, threads, warmup=args.warmup, steps=args.steps)
    wall = time.perf_counter() - t0
    secs = r["seconds"]
    v = statistics.median(secs)
    base = {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "cpu_model": cpu_model(),
            "iterations": r["iterations"][0], "true_rel": r["true_rel"],
            "seconds_per_step": secs, "process_wall_s": wall,
            "sample": f"{args.steps} whole solves of the {key[0]} Hz / {'XY'[1 - key[1]]} "
                      f"system (set-up + {r['iterations'][0]} iterations each, to the "
                      f"reference's stop rule) by the oracle's COCR_FP restatement with "
                      f"{threads} threads (the reference's cap, nproc - 1); {args.warmup} "
                      f"warm-up solves of 20 iterations; median reported"}
    out = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": statistics.mean(secs) * 1e3,
           "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
           "dtype": "f64 (complex128)",
           "data": "synthetic (seeded layered earth + 20 random blocks)",
           "config": {"workload": "c2: 96x96x64 cells, 1,812,736 edges, 0.1 Hz, COCR_FP "
                                  "algorithm on the host cores"},
           "impl": "reference", "cpu_baseline": base,
           "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def survey_compare(name, steps, warmup, setup_device=True):
    """A whole survey in one batch (--survey WORKLOAD, default c2s: the c2
    mesh under 16 frequencies x 2 polarisations = 32 systems): the batched
    double-float solver against the plain FP64 COCR on every system, and the
    impedance tensor, apparent resistivity and phase of both at the
    receivers, with the batched solver's error against FP64 per result."""
    import torch
    from mtcalc_with_dfp_cocr_gb300 import _lib, assembly, receivers, survey, workloads
    from mtcalc_with_dfp_cocr_gb300 import build as B
    if setup_device:
        B.build()
        torch.cuda.set_device(0)
    w = workloads.make(name)
    systems = w.systems
    S = len(systems)
    tables = make_inputs(w)
    nb = w.mesh.nb
    nus = [f for f, _ in systems]
    alfas = [a for _, a in systems]
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    A = assembly.Assembly(w.mesh)
    z1d = tables[nus[0]][0]
    us = np.stack([tables[f][1] for f in nus])
    uc = np.stack([tables[f][2] for f in nus])
    rhs = torch.empty(S, 2 * nb, dtype=torch.float64, device="cuda")
    A.rhs(nus, alfas, z1d, us, uc, rhs)
    eps, maxiter = 1e-8, 50000
    xb = torch.zeros_like(rhs)
    res = {}

    def step_batched():
        sv = survey.Survey(A, nus, stream)
        xb.zero_()
        code, st = sv.solve(rhs, xb, eps=eps, maxiter=maxiter, verify=True)
        if code != 0:
            raise RuntimeError(f"survey solve failed: {st}")
        res["batched"] = st
        sv.close()

    def timed(fn, steps):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    for _ in range(warmup):
        step_batched()
    l0 = _lib.kernel_launches()
    with ClockSampler(0) as clk:
        ms_b = timed(step_batched, steps)
    launches = _lib.kernel_launches() - l0
    t_b = ms_b / 1e3 / (steps * S)

    x64 = torch.zeros_like(rhs)
    plain = {}

    def step_plain():
        for k, (f, a) in enumerate(systems):
            ctx = A.cocr(f, stream)
            x64[k].zero_()
            code, st = ctx.solve(rhs[k], x64[k], eps=eps, maxiter=maxiter,
                                 stop_on_true_residual=True)
            ctx.close()
            if code != 0:
                raise RuntimeError(f"FP64 solve of system {k} failed with code {code}")
            plain[k] = (st.iterations, st.true_residual_rel)

    ms_p = timed(step_plain, 1)
    t_p = ms_p / 1e3 / S

    # impedances of both
    R = receivers.Receivers(A, w.receivers)
    freqs = sorted(set(nus))
    sx = [next(k for k, (f, a) in enumerate(systems) if f == nu and a == 1) for nu in freqs]
    sy = [next(k for k, (f, a) in enumerate(systems) if f == nu and a == 0) for nu in freqs]
    outs = []
    for x in (xb, x64):
        E, H, _ = R.fields(x, nus, alfas, z1d, us, uc)
        outs.append(R.mt_response(freqs, sx, sy, E, H).cpu().numpy())
    ob, o64 = outs
    zb = ob[..., 0:8].reshape(len(freqs), -1, 4, 2)
    z64 = o64[..., 0:8].reshape(len(freqs), -1, 4, 2)
    zb = zb[..., 0] + 1j * zb[..., 1]
    z64 = z64[..., 0] + 1j * z64[..., 1]
    off = [1, 2]   # Zxy, Zyx
    zerr = np.abs(zb - z64)[..., off] / np.abs(z64)[..., off]
    # the diagonal components, relative to the off-diagonal scale
    dscale = np.abs(z64)[..., off].max(axis=-1)
    derr = np.abs(zb - z64)[..., [0, 3]] / dscale[..., None]
    rho_err = np.abs(ob[..., 21:23] - o64[..., 21:23]) / np.abs(o64[..., 21:23])
    ph = np.abs(ob[..., 17:19] - o64[..., 17:19]) % 360.0
    ph_err = np.minimum(ph, 360.0 - ph)
    lab = lambda f, a: f"{f:.4g}Hz/{'XY'[1 - a]}"
    per_freq = {f"{nu:.4g}Hz": {"Z_offdiag_rel_max": float(zerr[i].max()),
                                "Z_diag_rel_to_offdiag_max": float(derr[i].max()),
                                "rho_a_rel_max": float(rho_err[i].max()),
                                "phase_deg_max": float(ph_err[i].max())}
                for i, nu in enumerate(freqs)}
    out = {
        "survey": name, "systems": S, "nb": nb, "receivers": len(w.receivers),
        "steps": steps, "warmup": warmup,
        "batched_s_per_solve": t_b, "batched_ms_per_survey": ms_b / steps,
        "plain_fp64_s_per_solve": t_p, "plain_fp64_ms_per_survey": ms_p,
        "speedup": t_p / t_b,
        "iterations_batched": {lab(f, a): it for (f, a), it in zip(systems, res["batched"]["iterations"])},
        "iterations_fp64": {lab(f, a): plain[k][0] for k, (f, a) in enumerate(systems)},
        "fp64_resolve_iterations_batched": {lab(f, a): it for (f, a), it in
                                            zip(systems, res["batched"]["fp64_iterations"]) if it},
        "true_rel_res_batched_max": max(res["batched"]["true_residual_rel"]),
        "true_rel_res_fp64_max": max(v[1] for v in plain.values()),
        "impedance_error_vs_fp64": {
            "Z_offdiag_rel_max": float(zerr.max()), "Z_diag_rel_to_offdiag_max": float(derr.max()),
            "rho_a_rel_max": float(rho_err.max()), "phase_deg_max": float(ph_err.max()),
            "per_frequency": per_freq},
        "gpu_launches": int(launches), "clocks": clk.summary(),
    }
    R.close()
    A.close()
    return out


def survey_run(args):
    print(json.dumps(survey_compare(args.survey, args.steps, args.warmup)), flush=True)


def adjoint_run(args):
    """The adjoint gradient on the c5 case (--adjoint): 48x48x32 cells,
    8 frequencies x 2 polarisations, 15x15 receivers.  Observed impedances
    come from the model with 5 seeded blocks perturbed by +-0.3 in
    log10(sigma).  Times the misfit + gradient with the batched solver and
    with the FP64 solver, compares the two gradients, and checks both
    against central differences (step 1e-4 in ln sigma) of the FP64 forward
    solve on 20 seed-chosen cells among those whose FP64 gradient is at
    least 1 % of the largest (cells with a negligible gradient have no
    meaningful relative error)."""
    import torch
    from mtcalc_with_dfp_cocr_gb300 import adjoint, workloads
    from mtcalc_with_dfp_cocr_gb300 import build as B
    B.build()
    torch.cuda.set_device(0)
    w = workloads.make("c5")
    m = w.mesh
    m0 = np.log(np.asarray(m.cell_sigma, np.float64))
    rng = np.random.default_rng(55)
    xyz = m.xyz()
    nodes = m.cell_nodes()
    c = 0.5 * (xyz[nodes[:, 0]] + xyz[nodes[:, 7]])
    m_true = m0.copy()
    for _ in range(5):
        lo = rng.uniform([-1500.0, -1500.0, -1500.0], [1000.0, 1000.0, -300.0])
        size = rng.uniform([200.0, 200.0, 200.0], [600.0, 600.0, 500.0])
        box = np.all((c >= lo) & (c <= lo + size), axis=1) & (c[:, 2] < 0)
        m_true[box] += 0.3 * np.log(10.0) * rng.choice([-1.0, 1.0])
    freqs = w.freqs
    p64 = adjoint.ImpedanceProblem(m, freqs, w.receivers, solver="fp64", eps=1e-10,
                                   maxiter=50000)
    resp, _ = p64.forward(m_true)
    z_obs = adjoint.impedances(resp).cpu().numpy()
    p64.set_observed(z_obs)
    pb = adjoint.ImpedanceProblem(m, freqs, w.receivers, z_obs=z_obs, solver="batched",
                                  eps=1e-8, maxiter=50000)

    def timed(problem):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        J, st = problem.misfit(m0)
        t1 = time.perf_counter()
        g = problem.gradient(st)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        return J, g.cpu().numpy(), t1 - t0, t2 - t1

    timed(pb)   # warm-up (library load, first-touch allocations)
    Jb, gb, tfb, tgb = timed(pb)
    J64, g64, tf64, tg64 = timed(p64)
    earth = np.asarray(m.cell_sigma0) > 1e-6
    err_b = float(np.linalg.norm((gb - g64)[earth]) / np.linalg.norm(g64[earth]))
    fd_problem = p64
    strong = np.nonzero(earth & (np.abs(g64) >= 0.01 * np.abs(g64[earth]).max()))[0]
    cells = rng.choice(strong, min(20, len(strong)), replace=False)
    h = 1e-4
    fd, e64, eb = [], [], []
    for cell in cells:
        mp, mm = m0.copy(), m0.copy()
        mp[cell] += h
        mm[cell] -= h
        d = (fd_problem.misfit(mp)[0] - fd_problem.misfit(mm)[0]) / (2 * h)
        fd.append(d)
        e64.append(abs(g64[cell] - d) / abs(d))
        eb.append(abs(gb[cell] - d) / abs(d))
    out = {"adjoint": "c5", "nb": m.nb, "cells": m.kpar, "systems": 2 * len(freqs),
           "receivers": len(w.receivers), "misfit_batched": Jb, "misfit_fp64": J64,
           "batched": {"forward_s": tfb, "gradient_s": tgb},
           "fp64": {"forward_s": tf64, "gradient_s": tg64},
           "speedup_forward_plus_gradient": (tf64 + tg64) / (tfb + tgb),
           "gradient_rel_err_batched_vs_fp64_earth": err_b,
           "fd": {"cells": [int(x) for x in cells], "step_ln_sigma": h,
                  "rel_err_fp64_max": float(max(e64)), "rel_err_fp64_median": float(np.median(e64)),
                  "rel_err_batched_max": float(max(eb)),
                  "rel_err_batched_median": float(np.median(eb)),
                  "cell_selection": "seeded among earth cells with |grad| >= 1% of max"}}
    print(json.dumps(out), flush=True)


def dtm_run(args):
    """The reference's published case (--dtm): the DTM model of
    CalculationExample on the reference RegularMeshBuilder's 625/500 m mesh
    (tests/golden/dtm_625_500.npz), 21 periods x 2 polarisations through the
    device assembly, the batched solver, the receiver fields and the MT
    responses, against CalculationResults/625_500_reg_R_Z.txt.  The table
    was produced with the reference's smoothing output path and FP32
    impedance post-processing.  The direct output is evaluated at the
    table's station coordinates taken both as (northing, easting) = (x, y)
    and as (x, -y) (the example's receiver file holds the mirrored set for
    part of the stations); the smoothing output at (x, -y)."""
    import torch
    from mtcalc_with_dfp_cocr_gb300 import assembly, mesh as M, normal1d, receivers, survey
    from mtcalc_with_dfp_cocr_gb300 import build as B
    B.build()
    torch.cuda.set_device(0)
    g = np.load(os.path.join(ROOT, "tests", "golden", "dtm_625_500.npz"))
    cm = g["cell_mat"].astype(np.int64)
    layers = [M.Layer(float(t), float(s)) for t, s in zip(g["layer_tops"], g["layer_sigma"])]
    m = M.RegularMesh(g["x"], g["y"], g["z"], layers, g["mat_sigma"][cm], g["mat_sigma0"][cm])
    freqs = 1.0 / g["periods"]
    st = g["stations"]
    pts = np.concatenate([np.c_[st[:, 0], st[:, 1], np.zeros(len(st))],
                          np.c_[st[:, 0], -st[:, 1], np.zeros(len(st))]])
    A = assembly.Assembly(m)
    R = receivers.Receivers(A, pts)
    # the reference's default output (subdomain smoothing) at the table's
    # receivers, (northing, -easting)
    Rs = receivers.Receivers(A, pts[len(st):], output="smooth")
    out_s = np.empty((len(freqs), len(st), 34))
    t_smooth = 0.0
    tops = [l.top for l in layers]
    sig = [l.sigma for l in layers]
    out = np.empty((len(freqs), len(pts), 34))
    t_solve = 0.0
    iters, fp64 = [], []
    for f0 in range(0, len(freqs), 16):
        fb = freqs[f0:f0 + 16]
        nus = np.repeat(fb, 2)
        alfas = np.tile([1, 0], len(fb))
        tabs = [normal1d.solve_1d(f, tops, sig) for f in fb]
        us = np.repeat(np.stack([t[1] for t in tabs]), 2, axis=0)
        uc = np.repeat(np.stack([t[2] for t in tabs]), 2, axis=0)
        b = torch.empty(len(nus), 2 * m.nb, dtype=torch.float64, device="cuda")
        A.rhs(nus, alfas, tabs[0][0], us, uc, b)
        x = torch.zeros_like(b)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sv = survey.Survey(A, nus)
        code, stt = sv.solve(b, x, eps=float(args.dtm_eps), maxiter=50000, verify=True)
        torch.cuda.synchronize()
        t_solve += time.perf_counter() - t0
        sv.close()
        if code != 0:
            raise RuntimeError(f"DTM solve failed: {stt}")
        iters += stt["iterations"]
        fp64 += stt["fp64_iterations"]
        E, H, _ = R.fields(x, nus, alfas, tabs[0][0], us, uc)
        out[f0:f0 + len(fb)] = R.mt_response(fb, np.arange(0, 2 * len(fb), 2),
                                             np.arange(1, 2 * len(fb), 2), E, H).cpu().numpy()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        E, H, _ = Rs.fields(x, nus, alfas, tabs[0][0], us, uc)
        torch.cuda.synchronize()
        t_smooth += time.perf_counter() - t0
        out_s[f0:f0 + len(fb)] = Rs.mt_response(fb, np.arange(0, 2 * len(fb), 2),
                                                np.arange(1, 2 * len(fb), 2), E, H).cpu().numpy()
    pub = g["published"]          # [station][period][8]
    n = len(st)
    res = {}
    for name, o in (("x=northing,y=easting", out[:, :n]), ("x=northing,y=-easting", out[:, n:]),
                    ("smoothing output, x=northing,y=-easting", out_s)):
        o = o.transpose(1, 0, 2)            # [station][period][34]
        zerr = np.abs(o[..., 13:15] - pub[..., 1:3]) / pub[..., 1:3]
        rerr = np.abs(o[..., 21:23] - pub[..., 5:7]) / pub[..., 5:7]
        res[name] = {"Zxy_Zyx_rel_median": float(np.median(zerr)), "Zxy_Zyx_rel_p95": float(np.percentile(zerr, 95)),
                     "Zxy_Zyx_rel_max": float(zerr.max()),
                     "rho_xy_yx_rel_median": float(np.median(rerr)), "rho_xy_yx_rel_max": float(rerr.max()),
                     "worst": {"station": st[int(np.argmax(zerr.max(axis=(1, 2))))].tolist()}}
    print(json.dumps({"dtm": "625_500", "nb": m.nb, "cells": m.kpar, "periods": len(freqs),
                      "systems": 2 * len(freqs), "stations": n, "solve_s": t_solve,
                      "eps": float(args.dtm_eps), "iterations_max": int(max(iters)),
                      "fp64_resolved_systems": int(sum(1 for v in fp64 if v > 0)),
                      "smoothing": dict(Rs.smoothing_info(), seconds_all_periods=t_smooth),
                      "vs_published": res}), flush=True)


def profile_run(args):
    """A short fixed run for ncu: the device assembly, one COCR context,
    10 SpMV launches and 30 COCR iterations, then the batched solver on
    --systems systems: 10 SpMV launches and 30 iterations (both end with the
    iteration-limit code, which is expected here)."""
    import torch
    from mtcalc_with_dfp_cocr_gb300 import assembly, workloads
    from mtcalc_with_dfp_cocr_gb300 import build as B
    B.build()
    torch.cuda.set_device(0)
    w = workloads.make(args.workload)
    tables = make_inputs(w)
    nu, alfa = w.systems[0]
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    A = assembly.Assembly(w.mesh)
    rhs = torch.empty(1, 2 * w.mesh.nb, dtype=torch.float64, device="cuda")
    t = tables[nu]
    A.rhs([nu], [alfa], t[0], t[1][None], t[2][None], rhs)
    ctx = A.cocr(nu, stream)
    xs = torch.randn(2 * w.mesh.nb, dtype=torch.float64, device="cuda")
    ys = torch.empty_like(xs)
    ms = ctx.spmv_timed(xs, ys, 10)
    x = torch.zeros_like(rhs[0])
    code, st = ctx.solve(rhs[0], x, eps=1e-8, maxiter=30)
    ctx.close()
    # the batched double-float solver on the workload's systems (all of them
    # with --systems 0, else the first S)
    from mtcalc_with_dfp_cocr_gb300 import survey
    systems = w.systems if args.systems <= 0 else w.systems[:args.systems]
    nus = [f for f, _ in systems]
    tabs = tables
    rhs2 = torch.empty(len(systems), 2 * w.mesh.nb, dtype=torch.float64, device="cuda")
    A.rhs(nus, [a for _, a in systems], t[0], np.stack([tabs[f][1] for f in nus]),
          np.stack([tabs[f][2] for f in nus]), rhs2)
    sv = survey.Survey(A, nus, stream)
    tuning = sv.tuning()
    ms2 = sv.spmv_timed(10)
    x2 = torch.zeros_like(rhs2)
    code2, st2 = sv.solve(rhs2, x2, eps=1e-8, maxiter=30, verify=False)
    sv.close()
    torch.cuda.synchronize()
    print(json.dumps({"profile": args.workload, "spmv_fp64_ms": ms / 10, "code": code,
                      "iterations": st.iterations, "systems": len(systems),
                      "spmv_batched_ms": ms2 / 10, "spmv_variant": tuning[0],
                      "spmv_variant_ms": tuning[1], "code_batched": code2}))
    A.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gpu", "reference"], default="gpu")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-survey", action="store_true",
                    help="skip the 32-system survey comparison (c2s) of the default run")
    ap.add_argument("--profile", action="store_true",
                    help="short fixed run for ncu captures (see profile_run)")
    ap.add_argument("--workload", default=None, help="workload of --profile (default c3)")
    ap.add_argument("--systems", type=int, default=2,
                    help="systems of the batched solve in --profile (0: all of the workload)")
    ap.add_argument("--survey", default=None, metavar="WORKLOAD",
                    help="time a whole survey in one batch (e.g. c2s, c3); see survey_run")
    ap.add_argument("--adjoint", action="store_true",
                    help="adjoint gradient on c5: timing and finite-difference check")
    ap.add_argument("--dtm", action="store_true",
                    help="the reference's published DTM case against its results table")
    ap.add_argument("--dtm-eps", default=1e-8, type=float,
                    help="relative residual of the DTM solves")
    args = ap.parse_args()
    if args.dtm:
        dtm_run(args)
        return
    if args.adjoint:
        adjoint_run(args)
        return
    if args.survey:
        args.steps = min(args.steps, 1) if args.steps else 1
        args.warmup = min(args.warmup, 1)
        survey_run(args)
        return
    if args.profile:
        args.workload = args.workload or "c3"
        profile_run(args)
        return
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        reference_arm(args)
    else:
        gpu_arm(args)


if __name__ == "__main__":
    main()
