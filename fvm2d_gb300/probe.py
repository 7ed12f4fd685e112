"""Run a few iterations of a batch of NACA 0012 O-grid solves, for
profiling one flow type's kernels (the benchmark itself is Euler only).

    python -m fvm2d_gb300.probe --flow laminar --meshes 2 --iters 3

Prints one JSON line: the flow, the batch, the form of the iteration and
the wall time per iteration.  Each mesh is a jittered 1024 x 384 grid (or
--ni x --nr); laminar and turbulent flows use the parameters of the
512 x 192 laminar and 768 x 256 RANS-SA workloads.
"""
from __future__ import annotations

import argparse
import json
import time

FLOWS = {
    "euler": dict(mach=0.8, aoa_deg=1.25, cfl=1.0, iflux=1),
    "laminar": dict(iflow=2, mach=0.5, aoa_deg=0.0, rey=5000.0, cfl=0.8, iflux=1),
    "rans": dict(iflow=3, mach=0.7, aoa_deg=2.0, rey=6.5e6, cfl=0.5, iflux=3, nut_ratio=3.0),
}


def main(argv=None) -> dict:
    import fvm2d_gb300 as F
    from fvm2d_gb300.batch import Batch
    from fvm2d_gb300.ogrid import naca_ogrid

    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--flow", choices=sorted(FLOWS), default="euler")
    ap.add_argument("--meshes", type=int, default=2)
    ap.add_argument("--ni", type=int, default=1024)
    ap.add_argument("--nr", type=int, default=384)
    ap.add_argument("--iters", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--precision", choices=["fp32", "fp64"], default="fp32")
    ap.add_argument("--form", default="bulk", help="form of the iteration (Batch.set_form)")
    a = ap.parse_args(argv)
    prec = F.FP32 if a.precision == "fp32" else F.FP64
    flow = FLOWS[a.flow]
    meshes = []
    for k in range(a.meshes):
        g = naca_ogrid(a.ni, a.nr, radius=20.0, first_spacing=5e-4, jitter=0.1, seed=2 + k)
        meshes.append(F.build_geometry(g.coord, g.elem, g.ptype, wall_distance=a.flow == "rans",
                                       bugcompat=0))
    b = Batch(prec, vertices=sum(m.np for m in meshes), meshes=a.meshes,
              viscous=a.flow != "euler")
    par = F.make_params(precision=prec, bugcompat=0, **flow)
    slots = [b.add(par, m) for m in meshes]
    for s in slots:
        b.start(s, a.warmup + a.iters)
    b.set_form(a.form)
    b.step(a.warmup)
    b.sync()
    t0 = time.perf_counter()
    b.step(a.iters)
    b.sync()
    dt = (time.perf_counter() - t0) / max(a.iters, 1)
    polls = [b.poll(s) for s in slots]
    out = {"flow": a.flow, "precision": a.precision, "meshes": a.meshes,
           "vertices_per_mesh": meshes[0].np, "form": a.form, "iters": a.iters,
           "ms_per_iter": dt * 1e3, "status": [p["status"] for p in polls]}
    b.close()
    print(json.dumps(out), flush=True)
    return out


if __name__ == "__main__":
    main()
