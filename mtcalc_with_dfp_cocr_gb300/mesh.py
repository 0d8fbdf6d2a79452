"""Regular hexahedral meshes in the reference's mesh file set.

This is the input generator for the solve stage: it produces exactly the
arrays and files that the reference's RegularMeshBuilder hands to BuildMatrix
and COCR_FP, for tensor-product meshes described directly by their node
lines (the reference derives those lines from receivers and settings; here
the synthetic workloads state them).

Conventions followed (reference paths are relative to the reference repo):

* nodes are numbered x-fastest, then y, then z, 1-based in files
  (Code/RegularMeshBuilder/main.cpp:1347-1387, WriteXyz);
* a cell lists its 8 nodes as (x-,y-,z-), (x+,y-,z-), (x-,y+,z-), (x+,y+,z-),
  then the same four at z+, followed by 6 zeros (main.cpp:1389-1448);
* edges are numbered in the lexicographic order of their (n1 < n2) node
  pairs, the order of the `std::set<pair<int,int>>` that BuildEdges fills
  (main.cpp:923-973).  On a tensor mesh that is: for every node in node order,
  its +x edge, then its +y edge, then its +z edge;
* a cell lists its 12 edges as 4 x-edges (y-z-, y+z-, y-z+, y+z+), 4 y-edges
  (x-z-, x-z+, x+z-, x+z+), 4 z-edges (x-y-, x+y-, x-y+, x+y+), then 12 zeros
  and a 1 (main.cpp:975-1032 and 1766-1798);
* boundary nodes (file L13d.dat) are all nodes on the 6 faces, in node order
  (main.cpp:1706-1736);
* materials: 1 is air, then the 1-D layers bottom-up, then every further
  (sigma, sigma_normal) pair in cell order (main.cpp:769-878).  Harm1D reads
  column 3 of the first n_layers+1 rows of sig3d as the layer conductivities
  (Code/Harm1D/mesh_1d_mtz.cpp:43-92).  Values are written with "%.7e" as
  WriteProperty3D does (main.cpp:1543-1572), and the arrays held in memory
  are rounded the same way, so files and memory agree bit for bit.
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field

import numpy as np

AIR_SIGMA = 1e-8  # Code/RegularMeshBuilder/main.cpp:1158-1167 (CreateAirMaterial)


def _q7(v):
    """Round to the "%.7e" text representation the reference writes."""
    v = np.asarray(v, dtype=np.float64)
    return np.array([float(f"{t:.7e}") for t in v.ravel()]).reshape(v.shape)


def padded_lines(core_h: float, n_core: int, n_pad: int, ratio: float,
                 center: float = 0.0) -> np.ndarray:
    """Node line: n_core uniform cells of size core_h centred on `center`,
    then n_pad cells growing geometrically by `ratio` on each side."""
    half = 0.5 * n_core * core_h
    core = center - half + core_h * np.arange(n_core + 1)
    steps = core_h * ratio ** np.arange(1, n_pad + 1)
    right = core[-1] + np.cumsum(steps)
    left = core[0] - np.cumsum(steps)
    return np.concatenate([left[::-1], core, right])


def z_lines(core_h: float, n_core: int, n_pad_bottom: int, ratio_bottom: float,
            n_air: int, ratio_air: float, air_h0: float | None = None) -> np.ndarray:
    """Vertical node line: air cells above z=0 growing upward, n_core uniform
    earth cells below z=0, then bottom padding growing downward."""
    air_h0 = core_h if air_h0 is None else air_h0
    air = np.cumsum(air_h0 * ratio_air ** np.arange(n_air))
    earth = -core_h * np.arange(n_core + 1)
    pad = earth[-1] - np.cumsum(core_h * ratio_bottom ** np.arange(1, n_pad_bottom + 1))
    return np.concatenate([pad[::-1], earth[::-1], air])


@dataclass
class Layer:
    """One horizontal layer of the 1-D background: conductivity below `top`."""
    top: float
    sigma: float


@dataclass
class RegularMesh:
    """A tensor-product hexahedral mesh with per-cell conductivities.

    x, y, z      node lines (ascending)
    layers       1-D background, bottom-up; the last layer's top is 0
    cell_sigma   conductivity of every cell (cell order = x-fastest)
    cell_sigma0  normal (background) conductivity of every cell
    """
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    layers: list
    cell_sigma: np.ndarray
    cell_sigma0: np.ndarray
    # derived
    nvkat: np.ndarray = field(init=False)           # 0-based material per cell
    mat_sigma: np.ndarray = field(init=False)       # sigma3d per material
    mat_sigma0: np.ndarray = field(init=False)      # sigma0 per material

    def __post_init__(self):
        self.x = np.asarray(self.x, np.float64)
        self.y = np.asarray(self.y, np.float64)
        self.z = np.asarray(self.z, np.float64)
        self.cell_sigma = _q7(self.cell_sigma)
        self.cell_sigma0 = _q7(self.cell_sigma0)
        self._materials()

    # ---------------------------------------------------------------- sizes
    @property
    def nx(self):
        return len(self.x)

    @property
    def ny(self):
        return len(self.y)

    @property
    def nz(self):
        return len(self.z)

    @property
    def kuzlov(self):
        return self.nx * self.ny * self.nz

    @property
    def kpar(self):
        return (self.nx - 1) * (self.ny - 1) * (self.nz - 1)

    @property
    def nb(self):
        nx, ny, nz = self.nx, self.ny, self.nz
        return (nx - 1) * ny * nz + nx * (ny - 1) * nz + nx * ny * (nz - 1)

    # ------------------------------------------------------------ materials
    def _materials(self):
        air = _q7([AIR_SIGMA])[0]
        lay = _q7([l.sigma for l in self.layers])
        keys = {}
        sig, sig0 = [air], [air]
        keys[(air, air)] = 0
        for s in lay:
            sig.append(s)
            sig0.append(s)
            keys.setdefault((s, s), len(sig) - 1)
        pairs = np.stack([self.cell_sigma, self.cell_sigma0], axis=1)
        uniq, inv = np.unique(pairs, axis=0, return_inverse=True)
        inv = inv.ravel()
        # keep first-appearance (cell) order for the extra materials
        first = np.full(len(uniq), np.iinfo(np.int64).max)
        np.minimum.at(first, inv, np.arange(len(inv)))
        mat_of_uniq = np.empty(len(uniq), np.int64)
        for u in np.argsort(first, kind="stable"):
            key = (uniq[u, 0], uniq[u, 1])
            if key not in keys:
                sig.append(key[0])
                sig0.append(key[1])
                keys[key] = len(sig) - 1
            mat_of_uniq[u] = keys[key]
        self.nvkat = mat_of_uniq[inv].astype(np.int32)
        self.mat_sigma = np.asarray(sig, np.float64)
        self.mat_sigma0 = np.asarray(sig0, np.float64)

    # ------------------------------------------------------------- topology
    def xyz(self) -> np.ndarray:
        Z, Y, X = np.meshgrid(self.z, self.y, self.x, indexing="ij")
        return np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)

    def _edge_ids(self):
        """0-based ids of the +x, +y, +z edge leaving every node (-1: none)."""
        nx, ny, nz = self.nx, self.ny, self.nz
        iz, iy, ix = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
        hx = (ix < nx - 1).ravel()
        hy = (iy < ny - 1).ravel()
        hz = (iz < nz - 1).ravel()
        cnt = hx.astype(np.int64) + hy + hz
        start = np.concatenate([[0], np.cumsum(cnt)[:-1]])
        ex = np.where(hx, start, -1)
        ey = np.where(hy, start + hx, -1)
        ez = np.where(hz, start + hx + hy, -1)
        return ex, ey, ez

    def edges(self) -> np.ndarray:
        """(nb, 2) 0-based node pairs, n1 < n2, in edge-number order."""
        nx, nxy = self.nx, self.nx * self.ny
        ex, ey, ez = self._edge_ids()
        out = np.empty((self.nb, 2), np.int32)
        nodes = np.arange(self.kuzlov)
        for ids, step in ((ex, 1), (ey, nx), (ez, nxy)):
            m = ids >= 0
            out[ids[m], 0] = nodes[m]
            out[ids[m], 1] = nodes[m] + step
        return out

    def cell_nodes(self) -> np.ndarray:
        """(kpar, 8) 0-based nodes of every cell in the reference order."""
        nx, ny, nz, nxy = self.nx, self.ny, self.nz, self.nx * self.ny
        iz, iy, ix = np.meshgrid(np.arange(nz - 1), np.arange(ny - 1), np.arange(nx - 1),
                                 indexing="ij")
        n0 = (iz * nxy + iy * nx + ix).ravel()
        return np.stack([n0, n0 + 1, n0 + nx, n0 + nx + 1,
                         n0 + nxy, n0 + nxy + 1, n0 + nxy + nx, n0 + nxy + nx + 1],
                        axis=1).astype(np.int32)

    def cell_edges(self) -> np.ndarray:
        """(kpar, 12) 0-based edges of every cell in the reference local order."""
        nx, nxy = self.nx, self.nx * self.ny
        ex, ey, ez = self._edge_ids()
        n0 = self.cell_nodes()[:, 0].astype(np.int64)
        return np.stack([
            ex[n0], ex[n0 + nx], ex[n0 + nxy], ex[n0 + nxy + nx],
            ey[n0], ey[n0 + nxy], ey[n0 + 1], ey[n0 + nxy + 1],
            ez[n0], ez[n0 + 1], ez[n0 + nx], ez[n0 + nx + 1],
        ], axis=1).astype(np.int32)

    def boundary_nodes(self) -> np.ndarray:
        nx, ny, nz = self.nx, self.ny, self.nz
        iz, iy, ix = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
        b = (ix == 0) | (ix == nx - 1) | (iy == 0) | (iy == ny - 1) | (iz == 0) | (iz == nz - 1)
        return np.nonzero(b.ravel())[0].astype(np.int32)

    def is_node_bound(self) -> np.ndarray:
        f = np.zeros(self.kuzlov, np.int32)
        f[self.boundary_nodes()] = 1
        return f

    # ----------------------------------------------------------------- files
    def write(self, path: str, nu: float, alfa: int, eps: float = 1e-8,
              maxiter: int = 10000, nthreads: int = 1, receivers=None) -> None:
        """Write the mesh file set COCR_FP / BuildMatrix / Harm1D read.

        `receivers` (R, 3) go to pointres, xyzVectorB and xyzVectorE, as
        RegularMeshBuilder writes them (main.cpp:1905-1951)."""
        os.makedirs(path, exist_ok=True)
        P = lambda f: os.path.join(path, f)
        nx, ny, nz = self.nx, self.ny, self.nz
        kt1 = len(self.boundary_nodes())
        with open(P("inftry.dat"), "w") as f:
            f.write(" ISLAU= 0 INDKU1= 0 INDFPO= 0\n"
                    f"KUZLOV= {self.kuzlov}   KPAR= {self.kpar}    KT1= {kt1}"
                    "   KTR2= 0   KTR3= 0\n   KT8= 0   KT9= 0\n"
                    "KISRS1= 0 KISRS2= 0 KISRS3= 0   KBRS= 0\n"
                    "   KT7= 0   KT10= 0  KTR4= 0  KTSIM= 0\n   KT6= 0")
        self.xyz().astype("<f8").tofile(P("xyz.dat"))
        nver = np.zeros((self.kpar, 14), np.int32)
        nver[:, :8] = self.cell_nodes() + 1
        nver.astype("<i4").tofile(P("nver.dat"))
        (self.nvkat + 1).astype("<i4").tofile(P("nvkat.dat"))
        (self.boundary_nodes() + 1).astype("<i4").tofile(P("l13d.dat"))
        (self.edges() + 1).astype("<i4").tofile(P("nodesforedges.dat"))
        ed = np.zeros((self.kpar, 25), np.int32)
        ed[:, :12] = self.cell_edges() + 1
        ed[:, 24] = 1
        ed.astype("<i4").tofile(P("edges.dat"))
        nmat = len(self.mat_sigma)
        with open(P("sig3d"), "w") as f:
            for i in range(nmat):
                f.write(f"{i + 1}\t{self.mat_sigma[i]:.7e}\t{self.mat_sigma0[i]:.7e}\n")
        for name in ("mu3d", "dpr3d"):
            val = 1.0 if name == "mu3d" else 0.0
            with open(P(name), "w") as f:
                for i in range(nmat):
                    f.write(f"{i + 1}\t{val:.7e}\t{val:.7e}\n")
        with open(P("tsize3d.dat"), "w") as f:
            f.write("0\n")
        with open(P("tsize3d_.dat"), "w") as f:
            f.write(f"0\n{self.nb}\n")
        with open(P("3dmeshregular"), "w") as f:
            for line in (self.x, self.y, self.z):
                f.write(f"{len(line)}\n")
                for i, v in enumerate(line):
                    f.write(f"{i + 1}\t{v:.14e}\n")
            f.write("0\n0\n")
        reg = np.concatenate([[self.kpar], np.arange(1, self.kpar + 1)]).astype("<i4")
        reg.tofile(P("regular"))
        with open(P("sreda1d.ay"), "w") as f:
            f.write(f"{len(self.layers)}\n")
            for l in self.layers:
                f.write(f"{l.top:.13e}\t{_q7([l.sigma])[0]:.13e}\t1\n")
        with open(P("alfa"), "w") as f:
            f.write(f"{int(alfa)}\n")
        with open(P("nu"), "w") as f:
            f.write(f"{nu:.13e}\n3")
        with open(P("issc.txt"), "w") as f:
            f.write(f"{maxiter}\n{eps:.13e}\n")
        with open(P("nthreads.txt"), "w") as f:
            f.write(f"{nthreads}\n")
        rec = np.zeros((1, 3)) if receivers is None else np.asarray(receivers, np.float64)
        for name in ("pointres", "xyzVectorB", "xyzVectorE"):
            with open(P(name), "w") as f:
                f.write(f"{len(rec)}\n")
                for r in rec:
                    f.write(f"{r[0]:.13e}\t{r[1]:.13e}\t{r[2]:.13e}\n")


def layered_model(x, y, z, layers, blocks=(), cell_sigma=None) -> RegularMesh:
    """Build a RegularMesh from node lines, a bottom-up layer list and
    rectangular blocks ((x1, x2, y1, y2, z1, z2, sigma), assigned by cell
    centre) or an explicit per-cell conductivity of the earth cells."""
    x, y, z = (np.asarray(a, np.float64) for a in (x, y, z))
    cz = 0.5 * (z[:-1] + z[1:])
    cy = 0.5 * (y[:-1] + y[1:])
    cx = 0.5 * (x[:-1] + x[1:])
    tops = np.array([l.top for l in layers])
    sig_l = np.array([l.sigma for l in layers])
    # layer index of every z-cell: the lowest layer whose top is above the centre
    col = np.empty(len(cz))
    for k, c in enumerate(cz):
        if c > 0.0:
            col[k] = AIR_SIGMA
        else:
            col[k] = sig_l[np.nonzero(tops > c)[0][0]]
    Z, Y, X = np.meshgrid(cz, cy, cx, indexing="ij")
    sigma0 = np.broadcast_to(col[:, None, None], Z.shape).copy()
    sigma = sigma0.copy()
    if cell_sigma is not None:
        cs = np.asarray(cell_sigma, np.float64).reshape(Z.shape)
        earth = Z < 0.0
        sigma[earth] = cs[earth]
    for (x1, x2, y1, y2, z1, z2, s) in blocks:
        m = (X > x1) & (X < x2) & (Y > y1) & (Y < y2) & (Z > z1) & (Z < z2)
        sigma[m] = s
    return RegularMesh(x, y, z, list(layers), sigma.ravel(), sigma0.ravel())
