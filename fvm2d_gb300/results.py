"""Per-solve outputs the Fortran driver writes from the state: the wall
table of WALL.DAT (result.f:92-118) and the SOL restart file
(finalize.f:14-24 writes it, initialize.f:91-103 reads it back).

Host-side arithmetic on arrays returned by ``Solver.get_state`` /
``Batch.get_state`` (driver vertex order); nothing here runs on the GPU.
"""
from __future__ import annotations

import numpy as np


def wall_distance_first(mesh) -> np.ndarray:
    """wd1 of wall_dist.f:63-72: for each solid point (spts order) the
    smallest wall distance wd among its non-solid neighbours (the points
    sharing an edge with it)."""
    from .ogrid import POINT_SOLID
    spts = np.asarray(mesh.spts).ravel() - 1
    edge = np.asarray(mesh.edge).reshape(-1, 2) - 1
    ptype = np.asarray(mesh.ptype).ravel()
    wd = np.asarray(mesh.wd, dtype=np.float64).ravel()
    best = np.full(mesh.np, 1.0e10)
    a, b = edge[:, 0], edge[:, 1]
    for u, v in ((a, b), (b, a)):
        ok = ptype[v] != POINT_SOLID
        np.minimum.at(best, u[ok], wd[v[ok]])
    return best[spts]


def wall_table(mesh, state: dict, params, iflow: int) -> dict:
    """Columns of WALL.DAT (result.f:92-118) at the solid points: x and the
    pressure coefficient with the reference's sign, cp = -(p - p_inf) /
    (0.5 rho_inf q_inf^2); for viscous flows also the skin friction cf from
    the wall shear mu (du/dt . n), the first-point wall distance wd1 and
    y+ = rho u_tau wd1 / mu."""
    from ._lib import INVISCID
    spts = np.asarray(mesh.spts).ravel() - 1
    coord = np.asarray(mesh.coord).reshape(-1, 2)
    prim = np.asarray(state["prim"]).reshape(-1, 4)
    q = 0.5 * params.r_inf * params.q_inf ** 2
    out = {"x": coord[spts, 0], "cp": -(prim[spts, 3] - params.p_inf) / q}
    if iflow != INVISCID:
        qx = np.asarray(state["qx"]).reshape(-1, 4)[spts]
        qy = np.asarray(state["qy"]).reshape(-1, 4)[spts]
        mu = np.asarray(state["mu"]).ravel()[spts]
        dsb = np.asarray(mesh.dsb).reshape(-1, 2)[spts]
        ux, uy, vx, vy = qx[:, 1], qy[:, 1], qx[:, 2], qy[:, 2]
        nl = np.sqrt(dsb[:, 0] ** 2 + dsb[:, 1] ** 2)
        nx, ny = dsb[:, 0] / nl, dsb[:, 1] / nl
        tx, ty = ny, -nx
        tw = mu * ((ux * tx + vx * ty) * nx + (uy * tx + vy * ty) * ny)
        wd1 = wall_distance_first(mesh)
        us = np.sqrt(np.abs(tw) / prim[spts, 0])
        out.update(cf=tw / q, wd1=wd1, yplus=prim[spts, 0] * us * wd1 / mu)
    return out


def write_wall(path: str, table: dict) -> None:
    cols = ["x", "cp"] + (["cf", "wd1", "yplus"] if "cf" in table else [])
    np.savetxt(path, np.column_stack([table[c] for c in cols]), fmt="%.17E")


def write_sol(path: str, prim: np.ndarray, nut: np.ndarray, gamma1: float) -> None:
    """SOL (finalize.f:14-24): conserved variables and nu~ per vertex."""
    prim = np.asarray(prim).reshape(-1, 4)
    u1 = prim[:, 0]
    u2 = u1 * prim[:, 1]
    u3 = u1 * prim[:, 2]
    u4 = prim[:, 3] / gamma1 + 0.5 * prim[:, 0] * (prim[:, 1] ** 2 + prim[:, 2] ** 2)
    np.savetxt(path, np.column_stack([u1, u2, u3, u4, np.asarray(nut).ravel()]), fmt="%.17E")


def read_sol(path: str, gamma1: float) -> tuple[np.ndarray, np.ndarray]:
    """Restart state from SOL (initialize.f:91-103): primitive variables
    and nu~."""
    d = np.loadtxt(path, ndmin=2)
    u1, u2, u3, u4, u5 = (d[:, k] for k in range(5))
    prim = np.column_stack([u1, u2 / u1, u3 / u1, gamma1 * (u4 - 0.5 * (u2 ** 2 + u3 ** 2) / u1)])
    return prim, u5.copy()
