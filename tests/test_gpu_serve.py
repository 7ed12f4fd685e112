"""Continuous batching: requests arriving while others run join them on the
device, and each result equals the same solve run alone (same kernels, so
bit for bit)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from fvm2d_gb300 import _lib as L  # noqa: E402


def test_serving_results_equal_alone(fvm_lib):
    from fvm2d_gb300 import serve
    from fvm2d_gb300.batch import Batch
    reqs = serve.generate_requests(n=8, rate=40.0, seed=3, pmin=1500, pmax=9000, laminar_frac=0.4)
    srv = serve.Server(vertices=30000, meshes=4, chunk=10, workers=4, max_iter=80, minres=1e-6)
    res, stats = srv.run(reqs)
    srv.close()
    assert stats["completed_ok"] == 8
    # the arena holds at most 4 meshes / 30k vertices: some requests waited
    # for others to retire, and some ran together
    assert any(r.admitted > r.arrival + 1e-3 for r in res) or stats["mean_resident_vertices"] > 0
    for req, r in zip(reqs, res):
        p = serve.prepare(req, L.FP32)
        b = Batch(L.FP32, vertices=p.np, meshes=1, viscous=True)
        s = b.add_prepared(p)
        b.start(s, 80, 1e-6)
        b.step(90)
        q = b.poll(s)
        b.close()
        assert (q["niter"], q["fres"], q["cl"], q["cd"]) == (r.niter, r.fres, r.cl, r.cd)


def test_prepared_refused_then_admitted(fvm_lib):
    from fvm2d_gb300 import serve
    from fvm2d_gb300.batch import Batch
    reqs = serve.generate_requests(n=2, seed=1, pmin=3000, pmax=3000)
    p0, p1 = (serve.prepare(r, L.FP32) for r in reqs)
    b = Batch(L.FP32, vertices=p0.np + 100, meshes=2, viscous=True)
    s0 = b.add_prepared(p0)
    assert b.add_prepared(p1) is None        # no room: p1 stays with the caller
    b.remove(s0)
    assert b.add_prepared(p1) is not None    # and is admitted once room frees


def test_request_larger_than_the_arena_is_refused_with_a_status(fvm_lib):
    from fvm2d_gb300 import serve
    reqs = serve.generate_requests(n=3, rate=100.0, seed=5, pmin=2000, pmax=2000)
    reqs[1].npts = 40000                        # cannot fit a 12k-vertex arena
    srv = serve.Server(vertices=12000, meshes=2, chunk=10, workers=2, max_iter=20, minres=1e-6)
    res, stats = srv.run(reqs)
    srv.close()
    assert [r.status for r in res] == [0, L.ERR_CAPACITY, 0]
    assert stats["completed_ok"] == 2 and len(stats["failures"]) == 1


def test_native_service_equals_alone(fvm_lib):
    """The native service (fvm_serve_*): the same results as each solve run
    alone in its own batch, an oversize request refused with a status, and
    the final state kept on request."""
    from fvm2d_gb300 import serve
    from fvm2d_gb300.batch import Batch
    reqs = serve.generate_requests(n=6, rate=100.0, seed=4, pmin=1500, pmax=6000, laminar_frac=0.4)
    srv = serve.NativeServer(vertices=20000, meshes=3, chunk=10, workers=3, max_iter=60,
                             minres=1e-6)
    grids = [serve.grid_for(r) for r in reqs]
    meshes = [fvm_lib.build_geometry(g.coord, g.elem, g.ptype) for g in grids]
    tickets = [srv.submit(serve.params_for(r, L.FP32), m, keep_state=(k == 0))
               for k, (r, m) in enumerate(zip(reqs, meshes))]
    big = serve.grid_for(serve.Request(rid=99, arrival=0.0, thickness=0.12, camber=0.0,
                                       camber_pos=0.4, npts=40000, laminar=False, mach=0.5,
                                       aoa_deg=1.0, rey=0.0, seed=1))
    tb = srv.submit(serve.params_for(reqs[0], L.FP32),
                    fvm_lib.build_geometry(big.coord, big.elem, big.ptype))
    for t in tickets + [tb]:
        assert srv.wait(t, 600.0)
    assert srv.result(tb)["status"] == L.ERR_CAPACITY
    for k, (r, m, t) in enumerate(zip(reqs, meshes, tickets)):
        q = srv.result(t)
        b = Batch(L.FP32, vertices=m.np, meshes=1, viscous=True)
        s = b.add(serve.params_for(r, L.FP32), m)
        b.start(s, 60, 1e-6)
        b.step(70)
        p = b.poll(s)
        assert (q["status"], q["niter"], q["fres"], q["cl"], q["cd"]) == \
            (p["status"], p["niter"], p["fres"], p["cl"], p["cd"])
        if k == 0:
            np.testing.assert_array_equal(srv.state(t, m.np)["prim"], b.get_state(s)["prim"])
        b.close()
    st = srv.stats()
    assert st["submitted"] == 7 and st["done"] == 7 and st["status"] == 0
    srv.close()


def test_native_service_destroy_wakes_waiters(fvm_lib):
    """Destroying the service while other threads wait on unfinished solves
    (one waiting 'forever') ends those solves with FVM_ERR_STATE: the waiters
    return, and destroy frees the server only after they have left."""
    import ctypes as C
    import threading

    from fvm2d_gb300 import serve
    reqs = serve.generate_requests(n=2, rate=100.0, seed=6, pmin=4000, pmax=4000, laminar_frac=0.0)
    srv = serve.NativeServer(vertices=20000, meshes=2, chunk=10, workers=1, max_iter=10 ** 6,
                             minres=0.0)
    tickets = []
    for r in reqs:
        g = serve.grid_for(r)
        tickets.append(srv.submit(serve.params_for(r, L.FP32),
                                  fvm_lib.build_geometry(g.coord, g.elem, g.ptype)))
    states = {}

    def waiter(t, timeout):
        st = C.c_int32(-1)
        rc = L.lib().fvm_serve_wait(srv.h, t, timeout, C.byref(st))
        states[t] = (rc, st.value)

    th = [threading.Thread(target=waiter, args=(tickets[0], float("inf"))),
          threading.Thread(target=waiter, args=(tickets[1], 1e12))]
    for t in th:
        t.start()
    assert not srv.wait(tickets[0], 0.5)      # still running (10^6 iterations allowed)
    st = C.c_int32(-1)
    assert L.lib().fvm_serve_wait(srv.h, tickets[0], float("nan"), C.byref(st)) == L.ERR_ARG
    srv.close()                               # returns only after both waiters left
    for t in th:
        t.join(timeout=30.0)
        assert not t.is_alive()
    assert states == {tickets[0]: (L.OK, 2), tickets[1]: (L.OK, 2)}


@pytest.mark.parametrize("laminar", [False, True])
def test_checkpointed_and_resumed_solve_equals_uninterrupted(fvm_lib, laminar):
    """A served solve stopped at a checkpoint and resumed from the kept
    state (its iteration count as iterlast) ends in the same state, bit for
    bit, as the same solve run uninterrupted for the same total number of
    iterations; the resumed run renormalises its residual at its first
    iteration, as the reference's restart does (conres.f:25-29)."""
    from fvm2d_gb300 import serve
    from fvm2d_gb300.batch import Batch
    req = serve.generate_requests(n=1, seed=8, pmin=3000, pmax=3000,
                                  laminar_frac=1.0 if laminar else 0.0)[0]
    g = serve.grid_for(req)
    mesh = fvm_lib.build_geometry(g.coord, g.elem, g.ptype)
    par = serve.params_for(req, L.FP32)
    srv = serve.NativeServer(vertices=20000, meshes=2, chunk=10, workers=1, max_iter=10 ** 6,
                             minres=0.0)
    t = srv.submit(par, mesh)
    import time
    t0 = time.time()
    while srv.stats()["steps"] < 3 and time.time() - t0 < 60:
        time.sleep(0.01)
    srv.checkpoint(t)
    assert srv.wait(t, 60.0)
    r = srv.result(t)
    assert r["status"] == L.CHECKPOINTED and r["niter"] >= 10
    ck = srv.checkpoint_read(t, mesh.np)
    assert ck["iter"] == r["niter"]
    extra = 25
    t2 = srv.resume(par, mesh, ck, nmax=extra, keep_state=True)
    assert srv.wait(t2, 60.0)
    r2 = srv.result(t2)
    assert r2["status"] == L.OK and r2["niter"] == extra
    got = srv.state(t2, mesh.np)["prim"]
    srv.close()
    total = ck["iter"] + extra
    b = Batch(L.FP32, vertices=mesh.np, meshes=1, viscous=True)
    s = b.add(par, mesh)
    b.start(s, total)
    b.step(total)
    q = b.poll(s)
    assert q["niter"] == total and q["status"] == L.OK
    np.testing.assert_array_equal(got, b.get_state(s)["prim"])
    b.close()
