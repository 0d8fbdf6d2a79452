"""Synthetic survey workloads, seeded and deterministic.

The reference publishes no benchmark dataset; these models stand in for its
surveys with the shapes, sizes and conductivity distributions of the five
benchmark configurations of this project:

  c1  plain FP64: 24x24x24 cells, 100 m core, 6 padding cells per side
      (ratio 1.5), 6 air cells on top, half-space 0.01 S/m with one
      4x4x3-cell block of 1 S/m; 1 Hz; 5x5 receivers at 100 m
  c2  FP64 at scale: 96x96x64 cells, 50 m core, 10 padding cells per side
      (ratio 1.4), 3-layer earth (100, 10, 1000 Ohm.m; 500 m, 2 km, half-space)
      plus 20 random blocks with log10(rho) ~ U(0, 3); 0.1 Hz
  c2s the c2 mesh and model under a 16-frequency survey (1e-3..1e3 Hz, 32
      systems); 15x15 receivers at 200 m
  c3  batched survey: 64x64x48 cells, same layering plus 10 random blocks;
      16 frequencies log-spaced 1e-3..1e3 Hz; 25x25 receivers at 200 m
  c4  mixed precision: 128x128x80 cells, log-normal random conductivity
      (log10 sigma mean -2, std 0.7, Gaussian correlation length 5 cells);
      0.01, 1, 100 Hz
  c5  adjoint: 48x48x32 cells, 100 Ohm.m half-space plus 3 random blocks;
      8 frequencies log-spaced 1e-2..1e2 Hz; 15x15 receivers

Every case has both source polarisations (alfa = 1: x, alfa = 0: y).  Layer
interfaces and block faces are placed on mesh lines (the nearest line to the
nominal depth), so the 3-D background matches the 1-D normal-field model.
Small cases ("tiny", "small") serve the parity tests.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .mesh import Layer, RegularMesh, layered_model, padded_lines, z_lines


@dataclass
class Workload:
    name: str
    mesh: RegularMesh
    freqs: np.ndarray          # Hz
    receivers: np.ndarray      # (R, 3)

    @property
    def systems(self):
        """(frequency, alfa) of every system, in CalcStarter's order: for every
        frequency X then Y (Code/CalcStarter/main.cpp:311-325)."""
        return [(f, a) for f in self.freqs for a in (1, 0)]


def _snap(lines, v):
    lines = np.asarray(lines)
    return float(lines[np.argmin(np.abs(lines - v))])


def _snap_layers(z, layers):
    return [Layer(_snap(z, l.top) if l.top != 0.0 else 0.0, l.sigma) for l in layers]


def _grid_receivers(n, spacing):
    c = spacing * (np.arange(n) - (n - 1) / 2.0)
    X, Y = np.meshgrid(c, c, indexing="xy")
    return np.stack([X.ravel(), Y.ravel(), np.zeros(n * n)], axis=1)


def _random_blocks(rng, x, y, z, n, core_cells_xy, core_cells_z, logrho_range,
                   size_cells=(2, 8)):
    """Rectangular blocks on mesh lines inside the core region."""
    nx, nz = len(x) - 1, len(z) - 1
    pad_xy = (nx - core_cells_xy) // 2
    iz0 = int(np.argmin(np.abs(z - 0.0)))          # index of the z = 0 line
    blocks = []
    for _ in range(n):
        sx, sy = rng.integers(size_cells[0], size_cells[1] + 1, size=2)
        sz = int(rng.integers(size_cells[0], max(size_cells[0], size_cells[1] // 2) + 1))
        ix = int(rng.integers(pad_xy, pad_xy + core_cells_xy - sx + 1))
        iy = int(rng.integers(pad_xy, pad_xy + core_cells_xy - sy + 1))
        top = int(rng.integers(iz0 - core_cells_z + sz, iz0 + 1))
        lo = top - sz
        rho = 10.0 ** rng.uniform(*logrho_range)
        blocks.append((x[ix], x[ix + sx], y[iy], y[iy + sy], z[lo], z[top], 1.0 / rho))
    return blocks


def _lognormal_field(rng, shape, mean, std, corr_cells):
    """Gaussian random field with a Gaussian covariance of correlation length
    `corr_cells`, by FFT filtering of white noise; returns 10**field."""
    noise = rng.standard_normal(shape)
    k = [np.fft.fftfreq(n) for n in shape]
    K = np.meshgrid(*k, indexing="ij")
    k2 = sum(kk ** 2 for kk in K)
    filt = np.exp(-0.5 * (2.0 * np.pi) ** 2 * k2 * corr_cells ** 2 / 2.0)
    f = np.real(np.fft.ifftn(np.fft.fftn(noise) * filt))
    f = (f - f.mean()) / f.std()
    return 10.0 ** (mean + std * f)


def make(name: str) -> Workload:
    name = name.lower()
    if name == "tiny":
        x = padded_lines(100.0, 2, 1, 1.5)
        z = z_lines(100.0, 2, 1, 1.5, 1, 1.5)
        layers = [Layer(-100.0, 0.05), Layer(0.0, 0.01)]
        m = layered_model(x, x, z, layers, blocks=[(-100, 0, 0, 100, -200, -100, 1.0)])
        return Workload(name, m, np.array([1.0]), _grid_receivers(2, 100.0))
    if name == "small":
        x = padded_lines(100.0, 4, 1, 1.5)
        z = z_lines(100.0, 3, 1, 1.5, 2, 1.5)
        layers = [Layer(-200.0, 0.1), Layer(0.0, 0.01)]
        m = layered_model(x, x, z, layers, blocks=[(-100, 100, -200, 0, -300, -100, 0.5)])
        return Workload(name, m, np.array([0.1]), _grid_receivers(3, 100.0))
    if name == "c1":
        x = padded_lines(100.0, 12, 6, 1.5)
        z = z_lines(100.0, 12, 6, 1.5, 6, 1.5)
        layers = [Layer(0.0, 0.01)]
        m = layered_model(x, x, z, layers, blocks=[(-200, 200, -200, 200, -400, -100, 1.0)])
        return Workload(name, m, np.array([1.0]), _grid_receivers(5, 100.0))
    if name in ("c2", "c2s", "c3"):
        if name in ("c2", "c2s"):
            x = padded_lines(50.0, 76, 10, 1.4)
            z = z_lines(50.0, 44, 10, 1.4, 10, 1.4)
            nblocks, core_xy, core_z, seed = 20, 76, 44, 2
            freqs = np.array([0.1])
            rec = _grid_receivers(5, 100.0)
            if name == "c2s":   # the c2 mesh under a 16-frequency survey
                freqs = np.logspace(-3, 3, 16)
                rec = _grid_receivers(15, 200.0)
        else:
            x = padded_lines(100.0, 48, 8, 1.4)
            z = z_lines(100.0, 32, 8, 1.4, 8, 1.4)
            nblocks, core_xy, core_z, seed = 10, 48, 32, 3
            freqs = np.logspace(-3, 3, 16)
            rec = _grid_receivers(25, 200.0)
        layers = _snap_layers(z, [Layer(-2500.0, 1e-3), Layer(-500.0, 0.1), Layer(0.0, 0.01)])
        rng = np.random.default_rng(seed)
        blocks = _random_blocks(rng, x, x, z, nblocks, core_xy, core_z, (0.0, 3.0))
        m = layered_model(x, x, z, layers, blocks=blocks)
        return Workload(name, m, freqs, rec)
    if name == "c4":
        x = padded_lines(100.0, 108, 10, 1.4)
        z = z_lines(100.0, 60, 10, 1.4, 10, 1.4)
        layers = [Layer(0.0, 0.01)]
        rng = np.random.default_rng(4)
        shape = (len(z) - 1, len(x) - 1, len(x) - 1)
        sig = _lognormal_field(rng, shape, -2.0, 0.7, 5.0)
        m = layered_model(x, x, z, layers, cell_sigma=sig.ravel())
        return Workload(name, m, np.array([0.01, 1.0, 100.0]), _grid_receivers(5, 100.0))
    if name == "c5":
        x = padded_lines(100.0, 36, 6, 1.4)
        z = z_lines(100.0, 20, 6, 1.4, 6, 1.4)
        layers = [Layer(0.0, 0.01)]
        rng = np.random.default_rng(5)
        blocks = _random_blocks(rng, x, x, z, 3, 36, 20, (0.0, 3.0))
        m = layered_model(x, x, z, layers, blocks=blocks)
        return Workload(name, m, np.logspace(-2, 2, 8), _grid_receivers(15, 100.0))
    raise KeyError(f"unknown workload {name!r}")
