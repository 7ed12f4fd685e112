"""Writes the golden fixtures of this directory from the CPU oracle.

The reference ships no test vectors and cannot be run here (Fortran, no
compiler), so these fixtures come from the oracle itself: they pin the
oracle (and, through the FP64 parity tests, the GPU path) against later
change; they do not pin either against the reference.

    python tests/golden/make_golden.py

Cases:
  euler_160x48_roe.npz   the 160x48 Euler workload (M 0.8, AoA 1.25, Roe +
                         van Albada, CFL 1): RES.DAT columns of 100
                         iterations and the final state's checksums;
  laminar_64x24_roe.npz  a 64x24 laminar case (M 0.5, Re 5000, CFL 0.8):
                         the same for 40 iterations;
  fluxes.npz             Roe / KFVS / HLLC (rotated back) interface fluxes
                         for 64 seeded state pairs and face vectors.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from fvm2d_gb300.ogrid import naca_ogrid, workload_grid  # noqa: E402
from oracle import oracle  # noqa: E402

CASES = {
    "euler_160x48_roe": (lambda: workload_grid("euler_160x48"),
                         dict(mach=0.8, aoa_deg=1.25, cfl=1.0, iflux=1), 100),
    "laminar_64x24_roe": (lambda: naca_ogrid(64, 24, radius=20.0, first_spacing=2e-3),
                          dict(iflow=2, mach=0.5, aoa_deg=1.0, rey=5000.0, cfl=0.8, iflux=1), 40),
}


def run_case(name):
    grid, flow, n = CASES[name]
    g = grid()
    o = oracle.Oracle(g.coord, g.elem, g.ptype, **flow)
    st, h = o.iterate(n)
    prim = o.d("prim").copy()
    return dict(status=np.int32(st), fres=h["fres"], iresi=h["iresi"], fresi=h["fresi"],
                cl=h["cl"], cd=h["cd"], prim_sum=prim.sum(axis=0),
                prim_sq=(prim * prim).sum(axis=0), prim_first=prim[:8].copy())


def flux_cases():
    rng = np.random.default_rng(12345)
    n = 64
    ds = rng.uniform(-1.0, 1.0, size=(n, 2))
    pl = np.column_stack([rng.uniform(0.5, 2.0, n), rng.uniform(-1, 1, n), rng.uniform(-1, 1, n),
                          rng.uniform(0.3, 3.0, n)])
    pr = pl * rng.uniform(0.8, 1.25, size=(n, 4))
    return ds, pl, pr


def fluxes():
    g = naca_ogrid(20, 8)
    ds, pl, pr = flux_cases()
    out = dict(ds=ds, priml=pl, primr=pr)
    for iflux, bugcompat, key in ((1, 1, "roe"), (2, 1, "kfvs"), (3, 0, "hllc")):
        o = oracle.Oracle(g.coord, g.elem, g.ptype, iflux=iflux, bugcompat=bugcompat)
        f = np.zeros((len(ds), 4))
        st = np.zeros(len(ds), dtype=np.int32)
        for k in range(len(ds)):
            st[k], f[k] = o.flux(iflux, ds[k], pl[k], pr[k])
        out[key] = f
        out[key + "_status"] = st
    return out


def main():
    oracle.build()
    for name in CASES:
        np.savez(os.path.join(HERE, name + ".npz"), **run_case(name))
    np.savez(os.path.join(HERE, "fluxes.npz"), **fluxes())


if __name__ == "__main__":
    main()
