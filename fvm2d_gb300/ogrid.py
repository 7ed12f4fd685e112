"""Seeded NACA 4-digit O-grid generator writing the amdba point/triangle layout.

The reference solver reads its grid from an amdba text file
(``src/read_grid.f:19-39``): ``np nt``, then one line per point
``i x y ptype`` and one line per triangle ``i n1 n2 n3 type``, all 1-based.
Point types are 0 (interior), 3 (solid wall), 4 (outflow) and 5 (farfield)
(``src/param.h:97-101``).  The reference ships no grid files, so the
workloads are generated here from fixed seeds:

* wall: NACA 4-digit thickness with the closed trailing edge (-0.1036 x^4
  coefficient) and the optional camber mean line; ``ni`` wall points spaced
  uniformly in the cosine parameter, one shared trailing-edge point;
* farfield: circle of radius ``radius`` chords centred at mid-chord;
* radial lines: straight from wall point ``i`` to the farfield point at the
  same parameter, with a geometric distribution whose first spacing is
  ``first_spacing`` chords and whose ratio is solved so the lines reach the
  farfield (the solved ratio is returned);
* triangles: each quad split in two with the diagonal alternating in a
  checkerboard pattern;
* jitter (optional): interior points moved by up to ``jitter`` of the local
  logical spacing in each grid direction, from a seeded RNG.

Vertex numbering is ``j*ni + i + 1`` (1-based), ``j`` the radial index.
"""
from __future__ import annotations

import dataclasses

import numpy as np

POINT_INTERIOR = 0
POINT_SOLID = 3
POINT_OUTFLOW = 4
POINT_FARFIELD = 5


@dataclasses.dataclass
class Grid:
    """A triangular grid in the reference's amdba layout (1-based indices)."""
    coord: np.ndarray   # [np, 2] float64
    elem: np.ndarray    # [nt, 3] int32, 1-based
    ptype: np.ndarray   # [np] int32
    ni: int = 0
    nr: int = 0
    ratio: float = 0.0  # solved geometric stretching ratio

    @property
    def np(self) -> int:
        return int(self.coord.shape[0])

    @property
    def nt(self) -> int:
        return int(self.elem.shape[0])


def naca4_surface(x: np.ndarray, thickness: float, camber: float = 0.0,
                  camber_pos: float = 0.4, upper: bool = True):
    """Surface point of a NACA 4-digit section at chord station ``x``."""
    t = thickness
    yt = 5.0 * t * (0.2969 * np.sqrt(x) - 0.1260 * x - 0.3516 * x**2
                    + 0.2843 * x**3 - 0.1036 * x**4)
    if camber == 0.0:
        return x.copy(), (yt if upper else -yt)
    m, p = camber, camber_pos
    yc = np.where(x < p, m / p**2 * (2 * p * x - x**2),
                  m / (1 - p)**2 * ((1 - 2 * p) + 2 * p * x - x**2))
    dyc = np.where(x < p, 2 * m / p**2 * (p - x), 2 * m / (1 - p)**2 * (p - x))
    th = np.arctan(dyc)
    if upper:
        return x - yt * np.sin(th), yc + yt * np.cos(th)
    return x + yt * np.sin(th), yc - yt * np.cos(th)


def solve_ratio(n_intervals: int, first: float, length: float) -> float:
    """Ratio r with first*(r^n - 1)/(r - 1) == length (bisection)."""
    if first * n_intervals >= length:
        raise ValueError("first spacing too large for the radial extent")
    lo, hi = 1.0 + 1e-12, 10.0
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        s = first * (mid**n_intervals - 1.0) / (mid - 1.0)
        if s > length:
            hi = mid
        else:
            lo = mid
    return 0.5 * (lo + hi)


def naca_ogrid(ni: int, nr: int, *, thickness: float = 0.12,
               camber: float = 0.0, camber_pos: float = 0.4,
               radius: float = 20.0, first_spacing: float = 2e-3,
               jitter: float = 0.0, seed: int = 0) -> Grid:
    """Build an O-grid of ``ni`` wall points by ``nr`` radial points."""
    if ni < 8 or ni % 2:
        raise ValueError("ni must be an even number >= 8")
    if nr < 3:
        raise ValueError("nr must be >= 3")
    theta = 2.0 * np.pi * np.arange(ni) / ni
    xs = 0.5 * (1.0 + np.cos(theta))
    lower = theta < np.pi
    wx = np.empty(ni)
    wy = np.empty(ni)
    xl, yl = naca4_surface(xs[lower], thickness, camber, camber_pos, upper=False)
    xu, yu = naca4_surface(xs[~lower], thickness, camber, camber_pos, upper=True)
    wx[lower], wy[lower] = xl, yl
    wx[~lower], wy[~lower] = xu, yu
    wx[0], wy[0] = 1.0, 0.0          # shared closed trailing edge
    ox = 0.5 + radius * np.cos(theta)
    oy = -radius * np.sin(theta)

    ratio = solve_ratio(nr - 1, first_spacing, radius)
    k = np.arange(nr, dtype=np.float64)
    s = first_spacing * (ratio**k - 1.0) / (ratio - 1.0) / radius
    s[-1] = 1.0
    s[0] = 0.0

    def evaluate(ifl: np.ndarray, jfl: np.ndarray):
        # bilinear in the logical (i periodic, j) space
        i0 = np.floor(ifl).astype(np.int64)
        fi = ifl - i0
        j0 = np.clip(np.floor(jfl).astype(np.int64), 0, nr - 2)
        fj = jfl - j0
        i0m = i0 % ni
        i1m = (i0 + 1) % ni

        def line(ii, jj):
            return (wx[ii] + s[jj] * (ox[ii] - wx[ii]),
                    wy[ii] + s[jj] * (oy[ii] - wy[ii]))
        x00, y00 = line(i0m, j0)
        x10, y10 = line(i1m, j0)
        x01, y01 = line(i0m, j0 + 1)
        x11, y11 = line(i1m, j0 + 1)
        x = (1 - fi) * (1 - fj) * x00 + fi * (1 - fj) * x10 + (1 - fi) * fj * x01 + fi * fj * x11
        y = (1 - fi) * (1 - fj) * y00 + fi * (1 - fj) * y10 + (1 - fi) * fj * y01 + fi * fj * y11
        return x, y

    jj, ii = np.meshgrid(np.arange(nr, dtype=np.float64),
                         np.arange(ni, dtype=np.float64), indexing="ij")
    ifl = ii.ravel().copy()
    jfl = jj.ravel().copy()
    if jitter > 0.0:
        rng = np.random.default_rng(seed)
        du = rng.uniform(-jitter, jitter, size=ifl.shape)
        dv = rng.uniform(-jitter, jitter, size=jfl.shape)
        interior = (jfl > 0) & (jfl < nr - 1)
        ifl[interior] += du[interior]
        jfl[interior] += dv[interior]
    x, y = evaluate(ifl, jfl)
    coord = np.stack([x, y], axis=1).astype(np.float64)

    ptype = np.zeros(ni * nr, dtype=np.int32)
    ptype[:ni] = POINT_SOLID
    ptype[(nr - 1) * ni:] = POINT_FARFIELD

    tris = []
    for j in range(nr - 1):
        i = np.arange(ni)
        ip = (i + 1) % ni
        a = j * ni + i + 1
        b = j * ni + ip + 1
        c = (j + 1) * ni + ip + 1
        d = (j + 1) * ni + i + 1
        even = ((i + j) % 2) == 0
        t1 = np.where(even[:, None], np.stack([a, b, c], 1), np.stack([a, b, d], 1))
        t2 = np.where(even[:, None], np.stack([a, c, d], 1), np.stack([b, c, d], 1))
        tt = np.empty((2 * ni, 3), dtype=np.int64)
        tt[0::2] = t1
        tt[1::2] = t2
        tris.append(tt)
    elem = np.concatenate(tris).astype(np.int32)
    return Grid(coord=coord, elem=elem, ptype=ptype, ni=ni, nr=nr, ratio=ratio)


def write_amdba(path: str, grid: Grid) -> None:
    """Write ``grid`` in the amdba text layout read by ``read_grid.f:19-39``."""
    with open(path, "w") as f:
        f.write(f"{grid.np} {grid.nt}\n")
        for i in range(grid.np):
            f.write(f"{i + 1} {float(grid.coord[i, 0])!r} {float(grid.coord[i, 1])!r} "
                    f"{int(grid.ptype[i])}\n")
        for i in range(grid.nt):
            n1, n2, n3 = (int(v) for v in grid.elem[i])
            f.write(f"{i + 1} {n1} {n2} {n3} 0\n")


def read_amdba(path: str) -> Grid:
    """Read an amdba grid file (the layout of ``read_grid.f:19-39``).

    Raises ``ValueError`` on an unrecognised point type, mirroring the stop
    at ``read_grid.f:91-94``.
    """
    with open(path) as f:
        tokens = f.read().split()
    npt, nt = int(tokens[0]), int(tokens[1])
    pos = 2
    pts = np.array(tokens[pos:pos + 4 * npt], dtype=object).reshape(npt, 4)
    pos += 4 * npt
    coord = np.stack([pts[:, 1].astype(np.float64), pts[:, 2].astype(np.float64)], 1)
    ptype = pts[:, 3].astype(np.int32)
    tri = np.array(tokens[pos:pos + 5 * nt], dtype=np.int64).reshape(nt, 5)
    elem = tri[:, 1:4].astype(np.int32)
    ok = np.isin(ptype, [POINT_INTERIOR, POINT_SOLID, POINT_OUTFLOW, POINT_FARFIELD])
    if not ok.all():
        raise ValueError("There seem to be some unrecognized point types")
    return Grid(coord=coord, elem=elem, ptype=ptype)


# Workloads (sizes and flow conditions of the five benchmark cases).
WORKLOADS = {
    "euler_160x48": dict(ni=160, nr=48, radius=20.0, first_spacing=2e-3),
    "euler_1024x384": dict(ni=1024, nr=384, radius=20.0, first_spacing=5e-4,
                           jitter=0.1, seed=2),
    "laminar_512x192": dict(ni=512, nr=192, radius=30.0, first_spacing=1e-4),
    "rans_768x256": dict(ni=768, nr=256, radius=50.0, first_spacing=1e-6),
}


def workload_grid(name: str, **overrides) -> Grid:
    kw = dict(WORKLOADS[name])
    kw.update(overrides)
    return naca_ogrid(**kw)


def cosine_area_check(grid: Grid) -> float:
    """Total signed area of all triangles (annulus area, a sanity figure)."""
    c = grid.coord
    e = grid.elem - 1
    a = 0.5 * ((c[e[:, 1], 0] - c[e[:, 0], 0]) * (c[e[:, 2], 1] - c[e[:, 0], 1])
               - (c[e[:, 2], 0] - c[e[:, 0], 0]) * (c[e[:, 1], 1] - c[e[:, 0], 1]))
    return float(np.abs(a).sum())


__all__ = ["Grid", "naca_ogrid", "naca4_surface", "solve_ratio", "write_amdba",
           "read_amdba", "workload_grid", "WORKLOADS", "POINT_INTERIOR",
           "POINT_SOLID", "POINT_OUTFLOW", "POINT_FARFIELD"]
