"""The reference's published DTM results (CalculationResults/625_500_reg_R_Z.txt)
reproduced end to end on the GPU: the reference RegularMeshBuilder's mesh of
the example model (tests/golden/dtm_625_500.npz), device assembly, batched
solve, receiver fields and MT responses.  The table was computed with the
reference's smoothing output path and FP32 post-processing, so the check is
at the percent level.  The table's easting axis is the model's -y."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from mtcalc_with_dfp_cocr_gb300 import assembly, mesh as M, normal1d, receivers, survey

pytestmark = pytest.mark.gpu


def test_dtm_impedances_match_published_table(gpu):
    torch = gpu
    g = np.load(os.path.join(GOLDEN, "dtm_625_500.npz"))
    cm = g["cell_mat"].astype(np.int64)
    layers = [M.Layer(float(t), float(s)) for t, s in zip(g["layer_tops"], g["layer_sigma"])]
    m = M.RegularMesh(g["x"], g["y"], g["z"], layers, g["mat_sigma"][cm], g["mat_sigma0"][cm])
    periods = g["periods"]
    pick = [4, 8, 12, 16]                      # 1, 10, 100, 1000 s
    fb = 1.0 / periods[pick]
    st = g["stations"]
    pts = np.c_[st[:, 0], -st[:, 1], np.zeros(len(st))]
    A = assembly.Assembly(m)
    R = receivers.Receivers(A, pts)
    tops, sig = [l.top for l in layers], [l.sigma for l in layers]
    nus = np.repeat(fb, 2)
    alfas = np.tile([1, 0], len(fb))
    tabs = [normal1d.solve_1d(f, tops, sig) for f in fb]
    us = np.repeat(np.stack([t[1] for t in tabs]), 2, axis=0)
    uc = np.repeat(np.stack([t[2] for t in tabs]), 2, axis=0)
    b = torch.empty(len(nus), 2 * m.nb, dtype=torch.float64, device="cuda")
    A.rhs(nus, alfas, tabs[0][0], us, uc, b)
    x = torch.zeros_like(b)
    code, stt = survey.Survey(A, nus).solve(b, x, eps=1e-8, maxiter=50000, verify=True)
    assert code == 0 and max(stt["true_residual_rel"]) < 1e-8
    E, H, _ = R.fields(x, nus, alfas, tabs[0][0], us, uc)
    out = R.mt_response(fb, np.arange(0, 2 * len(fb), 2), np.arange(1, 2 * len(fb), 2),
                        E, H).cpu().numpy().transpose(1, 0, 2)
    pub = g["published"][:, pick]
    z_err = np.abs(out[..., 13:15] - pub[..., 1:3]) / pub[..., 1:3]
    r_err = np.abs(out[..., 21:23] - pub[..., 5:7]) / pub[..., 5:7]
    assert np.median(z_err) < 0.005
    assert z_err.max() < 0.03
    assert r_err.max() < 0.06
