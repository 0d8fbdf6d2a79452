"""Survey meshes from the reference's five input files (restating
Code/RegularMeshBuilder, main.cpp:241-1114).

    cfg = read_case(dir)        # frequencies, xyzVectorB, z_sig_2d, objects, settings.cfg
    mesh = build_mesh(cfg)      # a RegularMesh (mesh.py) with the reference's lines and
                                # cell conductivities

Lines per axis (x, y lateral; z vertical):
* the receivers' bounding box grown by the "regular domain" gap, its lower
  end rounded down to a multiple of the step and its length to whole steps
  (CalculateReceiversBounds, main.cpp:579-623);
* a uniform part over that box, geometric parts (step growing by the
  sparse factor) out to the receivers' box plus the far distance
  (Build1DUniformMesh / Build1DSparsedMesh / BuildBaseMesh1D, :268-377);
* the ends pinned to the far bounds, dropping a line closer than 0.3 of
  the neighbouring step (AlignMeshBounds, :441-463);
* object faces, then layer interfaces and z = 0, inserted or snapped onto
  the nearest line when closer than 0.1 of the local step
  (InsertCoordinateIntoSortedArray, :485-570).
Conductivities: air 1e-8 S/m above z = 0, each layer between its
interface and the next one up, objects over the cells between their
(snapped) faces; the normal-field conductivity of an object cell is the
layer's (SetMaterials, :686-902).

The reference reads its layer list in a way that leaves the lower bounds
of the deeper layers to whatever memory holds (ReadZSig2D, :1169-1217;
InsertLayersIntoMesh, :544-570).  With zeroed memory — what the reference
build here produces — that inserts every layer interface except the deepest
and gives every earth cell the topmost layer's conductivity before the
objects; for one earth conductivity (the reference's example) both agree
with the intended layering, which is what this module implements.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass

import numpy as np

from .mesh import AIR_SIGMA, Layer, RegularMesh

SNAP = 0.1   # Settings::eps (main.cpp:182)


@dataclass
class Case:
    freqs: np.ndarray          # Hz
    receivers: np.ndarray      # (R, 3)
    layers: list               # Layer(top, sigma), bottom-up, last top 0
    objects: np.ndarray        # (O, 7): x1 x2 y1 y2 z1 z2 sigma
    steps: tuple               # (lateral, vertical)
    sparse: tuple
    gap: tuple                 # regular domain distance from the receivers
    far: tuple                 # calculation domain distance from the regular domain
    eps: float                 # SLAE relative residual
    maxiter: int


def _numbers(path):
    with open(path) as f:
        return f.read().split()


def read_case(path: str) -> Case:
    """The reference's calculation inputs (readme.txt): frequencies,
    xyzVectorB, z_sig_2d, objects, settings.cfg."""
    p = lambda n: os.path.join(path, n)
    t = _numbers(p("frequencies"))
    freqs = np.array([float(v) for v in t[1:1 + int(t[0])]])
    t = _numbers(p("xyzVectorB"))
    rec = np.array([float(v) for v in t[1:1 + 3 * int(t[0])]]).reshape(-1, 3)
    t = _numbers(p("z_sig_2d"))
    lay = np.array([float(v) for v in t[1:1 + 2 * int(t[0])]]).reshape(-1, 2)
    layers = [Layer(float(z), float(s)) for z, s in lay]
    t = _numbers(p("objects"))
    obj = np.array([float(v) for v in t[1:1 + 7 * int(t[0])]]).reshape(-1, 7)
    with open(p("settings.cfg")) as f:
        rows = [line.split() for line in f.readlines()[:6]]
    return Case(freqs, rec, layers, obj, (float(rows[0][0]), float(rows[0][1])),
                (float(rows[1][0]), float(rows[1][1])), (float(rows[2][0]), float(rows[2][1])),
                (float(rows[3][0]), float(rows[3][1])), float(rows[4][0]), int(float(rows[5][0])))


def _round_down(v, step):
    """RoundDouble_ (main.cpp:572-576)."""
    n = int(abs(v / step))
    return -(n + 1) * step if v < 0 else n * step


def _uniform(step, a, b):
    """Build1DUniformMesh (main.cpp:268-294)."""
    n = int((b - a) / step + 0.5)
    if abs(step * n - (b - a)) > 1e-5:
        n += 1
    h = (b - a) / n
    return [a + i * h for i in range(n + 1)]


def _geometric(step, sparse, a, b, direction):
    """Build1DSparsedMesh (main.cpp:297-342): from the inner end outwards,
    the step growing by `sparse`, until the far end is passed."""
    if direction > 0:
        c = a
        out = [c]
        while True:
            c += step
            step *= sparse
            out.append(c)
            if not c < b:
                return out
    c = b
    out = [c]
    while True:
        c -= step
        step *= sparse
        out.append(c)
        if not c > a:
            return out[::-1]


def _nearest(lines, v):
    """BinarySearchInVectorSorted (main.cpp:241-265): index of the line
    nearest to v (the upper one of a tie), clamped to the ends."""
    n = len(lines)
    if v < lines[0]:
        return 0
    if v > lines[-1]:
        return n - 1
    lo, hi = 0, n - 1
    while hi - lo > 1:
        m = (lo + hi) // 2
        if v > lines[m]:
            lo = m
        else:
            hi = m
    if lo == hi:
        return lo
    return lo if abs(lines[lo] - v) < abs(lines[hi] - v) else hi


def _insert(lines, v, eps=SNAP):
    """InsertCoordinateIntoSortedArray (main.cpp:485-512)."""
    if v < lines[0] or v > lines[-1]:
        return
    i = _nearest(lines, v)
    j = i - 1 if (lines[i] > v and i != 0) else i + 1
    step = abs(lines[i] - lines[j])
    if abs(lines[i] - v) / step > eps:
        lines.insert(i if lines[i] > v else i + 1, v)
    else:
        lines[i] = v


def axis_lines(lo, hi, step, sparse, gap, far):
    """Lines of one axis for receivers spanning [lo, hi] (main.cpp:579-684,
    345-377, 441-463)."""
    a, b = lo - gap, hi + gap
    d = b - a
    n = int(d / step + 0.5)
    if abs(n * step - d) > 1e-7:
        n += 1
        a = _round_down(a, step)
        b = a + n * step
    b0, b3 = lo - far, hi + far
    left = _geometric(step, sparse, b0, a, -1)
    mid = _uniform(step, a, b)
    right = _geometric(step, sparse, b, b3, 1)
    lines = left[:-1] + mid[:-1] + right
    lines[0] = b0
    if lines[1] - lines[0] < (lines[2] - lines[1]) * 0.3:
        del lines[1]
    lines[-1] = b3
    if lines[-1] - lines[-2] < (lines[-2] - lines[-3]) * 0.3:
        del lines[-2]
    return lines


def build_mesh(case: Case) -> RegularMesh:
    rec = case.receivers
    steps = (case.steps[0], case.steps[0], case.steps[1])
    sparse = (case.sparse[0], case.sparse[0], case.sparse[1])
    gap = (case.gap[0], case.gap[0], case.gap[1])
    far = (case.far[0], case.far[0], case.far[1])
    lines = [axis_lines(rec[:, d].min(), rec[:, d].max(), steps[d], sparse[d], gap[d], far[d])
             for d in range(3)]
    for o in case.objects:
        for k in range(6):
            _insert(lines[k // 2], float(o[k]))
    # z = 0 and the interfaces (tops of all layers but the deepest), top down
    _insert(lines[2], 0.0)
    for l in reversed(case.layers[1:]):
        _insert(lines[2], l.top)
    x, y, z = (np.array(v) for v in lines)
    nx, ny, nz = len(x) - 1, len(y) - 1, len(z) - 1
    # layer conductivity of every z-cell; air above z = 0
    zc = np.empty(nz)
    iz0 = _nearest(list(z), 0.0)
    for k in range(nz):
        if k >= iz0:
            zc[k] = AIR_SIGMA
            continue
        zc[k] = case.layers[0].sigma
        for j, l in enumerate(case.layers):
            lo_line = _nearest(list(z), case.layers[j - 1].top) if j > 0 else 0
            if lo_line <= k < _nearest(list(z), l.top):
                zc[k] = l.sigma
    sigma0 = np.broadcast_to(zc[:, None, None], (nz, ny, nx)).copy()
    sigma = sigma0.copy()
    for o in case.objects:
        i = [_nearest(list(lines[k // 2]), float(o[k])) for k in range(6)]
        sigma[i[4]:i[5], i[2]:i[3], i[0]:i[1]] = o[6]
    return RegularMesh(x, y, z, list(case.layers), sigma.ravel(), sigma0.ravel())
