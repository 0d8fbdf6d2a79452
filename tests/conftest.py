import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def load_golden(name):
    """(workload, BlockSLAE, SolveMesh, z1d, usin, ucos, v3, kit_iter, kit_r)"""
    from mtcalc_with_dfp_cocr_gb300 import slae_io, workloads
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    w = workloads.make(name)
    s = slae_io.BlockSLAE(int(len(g["ig"]) - 1), g["ig"].astype(np.int32), g["jg"].astype(np.int32),
                          g["idi"].astype(np.int32), g["ijg"].astype(np.int32), g["di"], g["gg"],
                          g["pr"], float(g["eps"]), int(g["maxiter"]))
    return (w, s, slae_io.mesh_to_solve_mesh(w.mesh), g["z1d"], g["usin"], g["ucos"], g["v3"],
            int(g["kit_iter"]), float(g["kit_r"]), float(g["nu"]), int(g["alfa"]))


@pytest.fixture(scope="session")
def gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from mtcalc_with_dfp_cocr_gb300 import build
    build.build()
    return torch
