"""The reference's impedance output files, written from the MT response
records of mtgpu_mt_response (receivers.py).

The reference's last step runs calcimpedance (Code/calcimpedance/
calcimpedance.for) in the Results directory and then reshapes its outputs in
ImpedanceZToEdsAll (Code/ImpedanceZToEdsAll/main.cpp:349-619).  This module
writes the same files from the GPU's FP64 records:

* calcimpedance's result files (openres, calcimpedance.for:430-465): one
  4-byte float record per receiver and frequency, receiver-major, the
  frequencies in the order of the survey's frequency list ("frec"; the
  record number KolOmega*m - j2 + 1 of :240-301 with the frequencies read
  backwards at :42-46):
    Zxx Zxy Zyx Zyy         |Z..|
    Fxx Fxy Fyx Fyy         -arg Z.. [deg]
    Rxx Rxy Ryx Ryy         |Z..|^2 / (omega mu0)
    Fixx Fixy Fiyx Fiyy     -2 arg Z.. [deg]
    Reff Fieff              |det Z| / (omega mu0), -arg det Z [deg]  (:256-276)
    Wzx WFzx Wzy WFzy       |Wz.|, -arg Wz. [deg] (Wiese-Parkinson, :279-323)
    ZxxRe ... ZyyIm, WzxRe ... WzyIm   the complex values;
* ImpedanceZToEdsAll's `edsall0_0_imp` (WriteToEdsAll, main.cpp:318-347):
  for |Z|, the phase, rho_a and the rho_a phase (types 1-4), for Zxx, Zxy,
  Zyx, Zyy, for every receiver a block of five header lines, the column
  legend and one line "nu 0 v v" per frequency, the frequencies in reverse
  list order; the phases folded into [-180, 180] as at :578-606; values
  read back from the 4-byte files, printed as C++ streams print doubles
  (6 significant digits), and `ft0_0` with the type of every block.

The values are FP64 here and FP32 in the reference (calcimpedance declares
`implicit real*4`), so they agree to FP32 rounding, which the 4-byte files
impose on both.
"""
from __future__ import annotations

import os

import numpy as np

from .receivers import MT_RHO, MT_RHOEFF, MT_RHOPHASE, MT_W, MT_WABS, MT_Z, MT_ZABS, MT_ZPHASE

COMP = ("xx", "xy", "yx", "yy")


def _fold(phase):
    """ImpedanceZToEdsAll's phase folding (main.cpp:578-606)."""
    p = phase.copy()
    p[p > 180.0] -= 180.0
    p[p < -180.0] += 180.0
    return p


def _fmt(v):
    """A double as an ofstream with default flags writes it (%g, 6 digits)."""
    return f"{v:g}"


def result_arrays(resp):
    """calcimpedance's result quantities: name -> (nrec, nfreq) float32, from
    records resp [nfreq][nrec][34] (frequencies in list order)."""
    r = np.transpose(np.asarray(resp, np.float64), (1, 0, 2))   # [nrec][nfreq][34]
    out = {}
    for i, c in enumerate(COMP):
        out["Z" + c] = r[..., MT_ZABS + i]
        out["F" + c] = r[..., MT_ZPHASE + i]
        out["R" + c] = r[..., MT_RHO + i]
        out["Fi" + c] = r[..., MT_RHOPHASE + i]
        out[f"Z{c}Re"] = r[..., MT_Z + 2 * i]
        out[f"Z{c}Im"] = r[..., MT_Z + 2 * i + 1]
    out["Reff"] = r[..., MT_RHOEFF]
    out["Fieff"] = r[..., MT_RHOEFF + 1]
    for i, c in enumerate(("zx", "zy")):
        out["W" + c] = r[..., MT_WABS + i]
        out["WF" + c] = r[..., MT_WABS + 2 + i]
        out[f"W{c}Re"] = r[..., MT_W + 2 * i]
        out[f"W{c}Im"] = r[..., MT_W + 2 * i + 1]
    return {k: v.astype(np.float32) for k, v in out.items()}


def write_results(path, freqs, receivers, resp):
    """Writes calcimpedance's 4-byte result files, ImpedanceZToEdsAll's
    edsall0_0_imp and ft0_0 into directory `path`."""
    os.makedirs(path, exist_ok=True)
    arrs = result_arrays(resp)
    for name, a in arrs.items():
        a.astype("<f4").tofile(os.path.join(path, name))
    freqs = np.asarray(freqs, np.float64)
    nf = len(freqs)
    rec = np.asarray(receivers, np.float64)
    blocks = (("Z", 1, False), ("F", 2, True), ("R", 3, False), ("Fi", 4, True))
    with open(os.path.join(path, "edsall0_0_imp"), "w") as fp, \
            open(os.path.join(path, "ft0_0"), "w") as fm:
        for prefix, typ, phase in blocks:
            for c in COMP:
                v = arrs[prefix + c].astype(np.float64)
                if phase:
                    v = _fold(v)
                for ir, (x, y, z) in enumerate(rec):
                    fm.write(f"{typ}\n")
                    fp.write(f"{int(x)} {int(y)}\n")
                    fp.write(f"{_fmt(x)} {_fmt(y)} {_fmt(z)}\n")
                    fp.write("1\n1 1 1 1\n1\n\tnu\tUn\tUa\tUs\n")
                    for j in range(nf - 1, -1, -1):
                        fp.write(f"{_fmt(freqs[j])} 0 {_fmt(v[ir, j])} {_fmt(v[ir, j])}\n")
    return sorted(arrs)


def read_result(path, name, nrec, nfreq):
    """One of calcimpedance's result files as (nrec, nfreq) float32."""
    return np.fromfile(os.path.join(path, name), "<f4").reshape(nrec, nfreq)
