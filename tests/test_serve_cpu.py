"""Serving workload generator (no GPU)."""
import math

import numpy as np

from fvm2d_gb300 import serve


def test_request_distribution():
    reqs = serve.generate_requests(n=512, rate=20.0, seed=0)
    arr = np.array([r.arrival for r in reqs])
    assert arr[0] == 0.0 and np.all(np.diff(arr) >= 0)
    assert 20.0 < arr[-1] < 32.0                      # 511 gaps of mean 1/20 s
    P = np.array([r.npts for r in reqs])
    assert P.min() >= 5000 and P.max() <= 400000
    # log-uniform: the median is near the geometric mean of the bounds
    assert abs(math.log(np.median(P)) - 0.5 * (math.log(5000) + math.log(400000))) < 0.4
    lam = np.array([r.laminar for r in reqs])
    assert 0.2 < lam.mean() < 0.4
    assert all(0.09 <= r.thickness <= 0.15 and 0.0 <= r.camber <= 0.04 for r in reqs)
    assert all(0.3 <= r.mach <= 0.85 and -3 <= r.aoa_deg <= 5 for r in reqs)
    assert all((1e3 <= r.rey <= 1e4) if r.laminar else r.rey == 0.0 for r in reqs)
    again = serve.generate_requests(n=512, rate=20.0, seed=0)
    assert [r.npts for r in again] == list(P)


def test_grid_sizes_follow_requests():
    for r in serve.generate_requests(n=20, seed=2):
        g = serve.grid_for(r)
        assert abs(g.np - r.npts) / r.npts < 0.15
        assert g.ni % 2 == 0
