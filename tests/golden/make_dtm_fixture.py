"""Fixture of the reference's published DTM case.

The reference ships one set of results, `CalculationResults/625_500_reg_R_Z.txt`
(|Z| and apparent resistivities of the DTM model at 53 receivers and 21
periods, computed with 625 m lateral and 500 m vertical mesh steps), and the
input files of that model in `CalculationExample/` (objects, z_sig_2d,
xyzVectorB, settings.cfg).  This script runs the reference RegularMeshBuilder
(built by oracle/build_ref.sh) on those inputs with 625/500 steps and keeps
what a solve needs, compactly:

  x, y, z             the mesh lines
  cell_mat            material of every cell (0-based, x fastest, z ascending)
  mat_sigma, mat_sigma0   conductivity and normal-field conductivity per material
  layer_tops, layer_sigma the 1-D background (bottom-up; tops, last 0)
  receivers           (53, 3), the example's xyzVectorB
  objects, settings   the example's objects (x1 x2 y1 y2 z1 z2 sigma) and the
                      first four rows of its settings.cfg
  stations            (53, 2): the table's (northing, easting), in table order
  periods             (21,) seconds
  published           (53, 21, 8) per station and period: |Zxx| |Zxy| |Zyx| |Zyy|
                      (Ohm), Rxx Rxy Ryx Ryy (Ohm.m)
  ex_*                the same mesh arrays for the example's own settings.cfg
                      (2500 m / 500 m steps)

Usage (needs the reference; not run by the tests):
    python tests/golden/make_dtm_fixture.py [--ref REFERENCE_ROOT]
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF_BIN = os.path.join(ROOT, "oracle", "_ref")


def read_settings(path):
    with open(path) as f:
        rows = [line.split() for line in f.readlines()[:6]]
    return rows


def run_builder(ex, s, steps):
    """The reference RegularMeshBuilder on the example's inputs with the given
    (lateral, vertical) steps, the other settings as in the example:
    (x, y, z lines, 0-based cell materials, material table [index, sigma, sigma0])."""
    d = tempfile.mkdtemp(prefix="dtm_")
    try:
        for n in ("objects", "z_sig_2d", "xyzVectorB"):
            shutil.copy(os.path.join(ex, n), d)
        with open(os.path.join(d, "RegularMeshBuilderSettings.cfg"), "w") as f:
            f.write(f"{steps[0]} {steps[1]}\n{s[1][0]} {s[1][1]}\n{s[2][0]} {s[2][1]}\n"
                    f"{s[3][0]} {s[3][1]}\nX\n1\n1\n{s[4][0]}\n{s[5][0]}\n")
        subprocess.check_call([os.path.join(REF_BIN, "RegularMeshBuilder")], cwd=d,
                              stdout=subprocess.DEVNULL)
        xyz = np.fromfile(os.path.join(d, "xyz.dat")).reshape(-1, 3)
        x, y, z = (np.unique(xyz[:, i]) for i in range(3))
        assert len(x) * len(y) * len(z) == len(xyz)
        nvkat = np.fromfile(os.path.join(d, "nvkat.dat"), "<i4") - 1
        sig = np.loadtxt(os.path.join(d, "Sig3d"))
    finally:
        shutil.rmtree(d, ignore_errors=True)
    return x, y, z, nvkat, sig[np.argsort(sig[:, 0])]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get(
        "MTCALC_REFERENCE_ROOT", os.path.join(os.path.dirname(ROOT), "reference")))
    a = ap.parse_args()
    subprocess.check_call([os.path.join(ROOT, "oracle", "build_ref.sh"), a.ref])
    ex = os.path.join(a.ref, "CalculationExample")
    s = read_settings(os.path.join(ex, "settings.cfg"))
    # the published run: 625 m lateral, 500 m vertical steps
    x, y, z, nvkat, mats = run_builder(ex, s, ("625", "500"))
    # the example's own settings
    x2, y2, z2, nvkat2, mats2 = run_builder(ex, s, (s[0][0], s[0][1]))
    with open(os.path.join(ex, "z_sig_2d")) as f:
        n = int(f.readline())
        lay = np.array([list(map(float, f.readline().split())) for _ in range(n)])
    with open(os.path.join(ex, "xyzVectorB")) as f:
        nr = int(f.readline())
        rec = np.array([list(map(float, f.readline().split())) for _ in range(nr)])
    with open(os.path.join(ex, "objects")) as f:
        no = int(f.readline())
        objects = np.array([list(map(float, f.readline().split())) for _ in range(no)])
    settings = np.array([[float(v) for v in row[:2]] for row in s[:4]])
    tab = np.loadtxt(os.path.join(a.ref, "CalculationResults", "625_500_reg_R_Z.txt"), skiprows=1)
    periods = np.unique(tab[:, 2])
    # the table's own stations (northing, easting), in first-appearance order;
    # they are not all in the example's xyzVectorB
    stations = []
    for row in tab:
        if (row[0], row[1]) not in stations:
            stations.append((row[0], row[1]))
    stations = np.array(stations)
    pub = np.full((len(stations), len(periods), 8), np.nan)
    for row in tab:
        r = np.nonzero((stations[:, 0] == row[0]) & (stations[:, 1] == row[1]))[0]
        p = np.nonzero(periods == row[2])[0]
        assert len(r) == 1 and len(p) == 1
        pub[r[0], p[0]] = row[3:11]
    assert not np.isnan(pub).any()
    assert nvkat.min() >= 0 and nvkat.max() < 256
    np.savez_compressed(
        os.path.join(HERE, "dtm_625_500.npz"), x=x, y=y, z=z, cell_mat=nvkat.astype(np.uint8),
        mat_sigma=mats[:, 1], mat_sigma0=mats[:, 2], layer_tops=lay[:, 0],
        layer_sigma=lay[:, 1], receivers=rec, stations=stations, periods=periods,
        published=pub, objects=objects, settings=settings, ex_x=x2, ex_y=y2, ex_z=z2, ex_cell_mat=nvkat2.astype(np.uint8),
        ex_mat_sigma=mats2[:, 1], ex_mat_sigma0=mats2[:, 2])
    print("mesh", len(x), len(y), len(z), "cells", len(nvkat), "materials", len(mats),
          "receivers", len(rec), "periods", len(periods))


if __name__ == "__main__":
    main()
