"""The smoothing-output restatement (oracle/smoothing.py) against the
reference's own smoothing classes (tests/golden/smoothing.npz, made by
tests/golden/make_golden_smoothing.py from oracle/_ref/ref_smoothing)."""
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN
from mtcalc_with_dfp_cocr_gb300 import workloads
from oracle import smoothing

sys.path.insert(0, GOLDEN)
from make_golden_smoothing import c1_values  # noqa: E402


def rows(a, c):
    """(12, R) in the fixture's row order."""
    out = []
    for f in (a, c):
        for d in range(3):
            out += [f[:, d].real, f[:, d].imag]
    return np.stack(out)


@pytest.fixture(scope="module")
def golden():
    return np.load(os.path.join(GOLDEN, "smoothing.npz"))


def _subdomain_sizes(m, rec):
    out = []
    eb = smoothing.locate(m, rec, skip_air=False)
    c, n = smoothing.subdomain(m, eb, -1)
    out.append((len(n), len(c)))
    ea = smoothing.locate(m, rec, skip_air=True)
    for mat in sorted({int(m.nvkat[e]) for e in ea if e >= 0}):
        c, n = smoothing.subdomain(m, ea, mat)
        out.append((len(n), len(c)))
    return np.array(out)


@pytest.mark.parametrize("pol", ["x", "y"])
def test_small_reference_solutions(golden, pol):
    r = np.load(os.path.join(GOLDEN, "receivers_small.npz"))
    m = workloads.make("small").mesh
    a, c = smoothing.smoothed_fields(m, golden["rec_small"], r[f"v3_{pol}"])
    ref = golden[f"ref_small_{pol}"]
    got = rows(a, c)
    assert np.abs(got - ref).max() < 1e-13 * np.abs(ref).max()
    # each value type to 1e-11 of its own scale
    scale = np.abs(ref).max(axis=1)
    assert (np.abs(got - ref).max(axis=1) <= 1e-11 * scale).all()


def test_c1_random_values(golden):
    w = workloads.make("c1")
    a, c = smoothing.smoothed_fields(w.mesh, golden["rec_c1"], c1_values(w.mesh.nb))
    ref = golden["ref_c1"]
    got = rows(a, c)
    scale = np.abs(ref).max(axis=1)
    assert (np.abs(got - ref).max(axis=1) <= 1e-12 * scale).all()


@pytest.mark.parametrize("case", ["small", "c1"])
def test_subdomains_match_reference_log(golden, case):
    m = workloads.make(case).mesh
    np.testing.assert_array_equal(_subdomain_sizes(m, golden[f"rec_{case}"]),
                                  golden[f"sub_{case}"])


def test_mass_matrix_rows():
    """Brick mass matrix: symmetric, entries V/27..V/216 by differing axes,
    row sums V/8 (Hex_Local_Matrix.cpp:120-198)."""
    b = smoothing.cell_mass(np.array([2.0]), np.array([3.0]), np.array([5.0]))[0]
    np.testing.assert_allclose(b, b.T)
    np.testing.assert_allclose(b.sum(axis=1), np.full(8, 30.0 / 8))
    assert b[0, 0] == 30.0 / 27.0 and b[0, 7] == 30.0 / 216.0
