"""Batched path: many meshes of uneven size in one arena and one launch per
kernel.  Each solve must give the same result alone and in any mix: the
per-vertex arithmetic never depends on other meshes, so "the same" is bit
for bit whenever the same compiled kernels run (always in FP64; in FP32
when the meshes share a Riemann solver) and within MIXED_FP32_RTOL for
FP32 mixes of solvers.  Meshes must be admissible and removable between
steps, and a full arena must refuse a mesh with a status, not fail."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from fvm2d_gb300 import _lib as L  # noqa: E402
from fvm2d_gb300.ogrid import naca_ogrid  # noqa: E402


def mesh(fvm_lib, ni, nr, seed=0, **kw):
    g = naca_ogrid(ni, nr, jitter=0.1 if seed else 0.0, seed=seed, **kw)
    return fvm_lib.build_geometry(g.coord, g.elem, g.ptype)


CASES = [dict(ni=64, nr=24, seed=0), dict(ni=96, nr=40, seed=3), dict(ni=48, nr=20, seed=5,
                                                                       thickness=0.15)]
FLOWS = [dict(mach=0.8, aoa_deg=1.25), dict(mach=0.5, aoa_deg=3.0, iflux=L.KFVS),
         dict(mach=0.7, aoa_deg=-1.0, iflux=L.HLLC, bugcompat=0)]


def alone(fvm_lib, prec, m, flow, n):
    from fvm2d_gb300.batch import Batch
    b = Batch(prec, vertices=m.np, meshes=1)
    s = b.add(fvm_lib.make_params(precision=prec, **flow), m)
    b.start(s, n)
    b.step(n)
    p = b.poll(s)
    h = b.history(s, 0, p["niter"])
    st = b.get_state(s)
    b.close()
    return h, st


SAME_FLUX = [dict(mach=0.8, aoa_deg=1.25), dict(mach=0.5, aoa_deg=3.0),
             dict(mach=0.7, aoa_deg=-1.0, ilimit=0)]
# FP32 solves that mix Riemann solvers run the generic flux kernel rather
# than the one compiled for a single solver; contraction may round those
# differently, so the mixed-solver FP32 comparison has a tolerance.
MIXED_FP32_RTOL = 1e-5


def run_mix(fvm_lib, prec, ms, flows, n):
    from fvm2d_gb300.batch import Batch
    b = Batch(prec, vertices=sum(m.np for m in ms) + 5000, meshes=5)
    slots = [b.add(fvm_lib.make_params(precision=prec, **f), m) for m, f in zip(ms, flows)]
    for s in slots:
        b.start(s, n)
    b.step(n + 5)      # extra steps: finished meshes must stay untouched
    out = []
    for s in slots:
        p = b.poll(s)
        assert p["status"] == 0 and p["niter"] == n and not p["active"]
        out.append((b.history(s, 0, n), b.get_state(s)))
    return out


@pytest.mark.parametrize("prec", [L.FP64, L.FP32])
def test_alone_equals_mix(fvm_lib, prec):
    """Uneven meshes and flow conditions, one Riemann solver: bit for bit."""
    ms = [mesh(fvm_lib, **c) for c in CASES]
    n = 40
    ref = [alone(fvm_lib, prec, m, f, n) for m, f in zip(ms, SAME_FLUX)]
    for (h, st), (h0, st0) in zip(run_mix(fvm_lib, prec, ms, SAME_FLUX, n), ref):
        for k in ("fres", "cl", "cd", "iresi"):
            np.testing.assert_array_equal(h[k], h0[k])
        np.testing.assert_array_equal(st["prim"], st0["prim"])


@pytest.mark.parametrize("prec", [L.FP64, L.FP32])
def test_alone_equals_mix_of_solvers(fvm_lib, prec):
    """Roe, KFVS and HLLC meshes in one batch: bit for bit in FP64 (no
    contraction), within MIXED_FP32_RTOL in FP32."""
    ms = [mesh(fvm_lib, **c) for c in CASES]
    n = 40
    ref = [alone(fvm_lib, prec, m, f, n) for m, f in zip(ms, FLOWS)]
    for (h, st), (h0, st0) in zip(run_mix(fvm_lib, prec, ms, FLOWS, n), ref):
        if prec == L.FP64:
            np.testing.assert_array_equal(h["fres"], h0["fres"])
            np.testing.assert_array_equal(st["prim"], st0["prim"])
        else:
            np.testing.assert_allclose(h["fres"], h0["fres"], rtol=MIXED_FP32_RTOL)
            np.testing.assert_allclose(h["cl"], h0["cl"], rtol=MIXED_FP32_RTOL, atol=1e-7)
            np.testing.assert_allclose(st["prim"], st0["prim"], rtol=MIXED_FP32_RTOL, atol=1e-6)


def test_fp64_batch_matches_handle(fvm_lib):
    """The batch path and the single-mesh C ABI run the same kernels."""
    from fvm2d_gb300.batch import Batch
    m = mesh(fvm_lib, 64, 24)
    s1 = fvm_lib.Solver(fvm_lib.make_params(), m)
    st, h1 = s1.iterate(30)
    b = Batch(L.FP64, vertices=m.np, meshes=1)
    s = b.add(fvm_lib.make_params(), m)
    b.start(s, 30)
    b.step(30)
    h = b.history(s, 0, 30)
    np.testing.assert_array_equal(h["fres"], h1["fres"])


def test_admit_and_retire_between_steps(fvm_lib):
    from fvm2d_gb300.batch import Batch
    prec = L.FP32
    a, c = mesh(fvm_lib, 64, 24), mesh(fvm_lib, 96, 40, seed=3)
    ref_a, _ = alone(fvm_lib, prec, a, FLOWS[0], 60)
    b = Batch(prec, vertices=a.np + c.np + 100, meshes=2)
    sa = b.add(fvm_lib.make_params(precision=prec, **FLOWS[0]), a)
    b.start(sa, 60)
    b.step(20)
    # admitted mid-solve, same Riemann solver (so the same compiled kernel
    # runs and the comparison is bit for bit)
    sc = b.add(fvm_lib.make_params(precision=prec, **SAME_FLUX[1]), c)
    b.start(sc, 100)
    b.step(20)
    b.remove(sc)                                                      # retired mid-solve
    b.step(25)
    p = b.poll(sa)
    assert p["niter"] == 60 and p["status"] == 0
    h = b.history(sa, 0, 60)
    np.testing.assert_array_equal(h["fres"], ref_a["fres"])
    # the freed range is reusable
    sd = b.add(fvm_lib.make_params(precision=prec, **FLOWS[2]), c)
    assert sd >= 0


def test_capacity_is_a_status(fvm_lib):
    from fvm2d_gb300.batch import Batch
    m = mesh(fvm_lib, 64, 24)
    b = Batch(L.FP32, vertices=m.np + 10, meshes=3)
    assert b.try_add(fvm_lib.make_params(precision=L.FP32), m) is not None
    assert b.try_add(fvm_lib.make_params(precision=L.FP32), m) is None
    b2 = Batch(L.FP32, vertices=10 * m.np, meshes=1)
    assert b2.try_add(fvm_lib.make_params(precision=L.FP32), m) is not None
    assert b2.try_add(fvm_lib.make_params(precision=L.FP32), m) is None


def test_mixed_euler_laminar(fvm_lib, oracle_lib):
    """A viscous-capable arena runs Euler and laminar meshes together; each
    matches its oracle run."""
    from fvm2d_gb300.batch import Batch
    g1 = naca_ogrid(64, 24)
    g2 = naca_ogrid(48, 20, thickness=0.1)
    flows = [dict(mach=0.8, aoa_deg=1.25), dict(iflow=L.LAMINAR, mach=0.5, aoa_deg=0.0,
                                                 rey=5000.0, cfl=0.8)]
    ors = [oracle_lib.Oracle(g.coord, g.elem, g.ptype, **f) for g, f in zip((g1, g2), flows)]
    b = Batch(L.FP64, vertices=g1.np + g2.np, meshes=2, viscous=True)
    slots = [b.add(fvm_lib.make_params(**f), o.mesh_arrays()) for f, o in zip(flows, ors)]
    for s in slots:
        b.start(s, 25)
    b.step(25)
    for s, o in zip(slots, ors):
        st, oh = o.iterate(25)
        h = b.history(s, 0, 25)
        assert np.max(np.abs(h["fres"] - oh["fres"]) / oh["fres"]) <= 1e-10


def run_variant(fvm_lib, prec, ms, flows, n, viscous=False, **caps):
    from fvm2d_gb300.batch import Batch
    b = Batch(prec, vertices=sum(m.np for m in ms), meshes=len(ms), viscous=viscous, **caps)
    slots = [b.add(fvm_lib.make_params(precision=prec, **f), m) for m, f in zip(ms, flows)]
    for s in slots:
        b.start(s, n)
    b.step(n)
    out = [(b.history(s, 0, n), b.get_state(s)) for s in slots]
    b.close()
    return out


@pytest.mark.parametrize("prec", [L.FP64, L.FP32])
def test_fused_pass_and_grid_give_identical_results(fvm_lib, prec):
    """The fused gradient+flux pass recomputes each halo gradient in the
    owner's triangle order; the three forms of the gradient pass (per-thread
    loads, per-vertex walks, bulk-copy staging) sum the same triangle terms
    in the same order; the grid only changes which CTA takes a block, and
    the two overlapped chains only when a mesh's blocks run: every variant
    must give the same bits, Euler and laminar.  In FP32 the Euler mesh
    takes the vertex-stencil gradient pass in every form; the variants
    cover the triangle forms of the laminar mesh, the pipelined one
    included."""
    g1, g2 = naca_ogrid(96, 40, jitter=0.1, seed=3), naca_ogrid(64, 24)
    ms = [fvm_lib.build_geometry(g.coord, g.elem, g.ptype) for g in (g1, g2)]
    flows = [dict(mach=0.8, aoa_deg=1.25),
             dict(iflow=L.LAMINAR, mach=0.5, aoa_deg=1.0, rey=5000.0, cfl=0.8)]
    n = 30
    ref = run_variant(fvm_lib, prec, ms, flows, n, viscous=True)
    variants = [dict(grid=3), dict(grad_mode=1), dict(grad_mode=2), dict(overlap=2),
                dict(overlap=4)]
    if prec == L.FP64:    # the fused pass exists in FP64 only
        variants += [dict(fused=1), dict(fused=1, grid=7), dict(overlap=2, fused=1)]
    if prec == L.FP32:
        # the pipelined gradient pass: one CTA (the stage ring wraps many
        # times), few CTAs, one consumer group with two stages, two chains
        variants += [dict(grad_mode=3, grid=5), dict(grad_mode=4, grid=1, pipe_stages=3),
                     dict(grad_mode=4, grid=5), dict(grad_mode=4, pipe_groups=1, pipe_stages=2),
                     dict(grad_mode=4, overlap=2)]
    for caps in variants:
        got = run_variant(fvm_lib, prec, ms, flows, n, viscous=True, **caps)
        for (h, st), (h0, st0) in zip(got, ref):
            np.testing.assert_array_equal(h["fres"], h0["fres"], err_msg=str(caps))
            np.testing.assert_array_equal(h["cl"], h0["cl"], err_msg=str(caps))
            np.testing.assert_array_equal(st["prim"], st0["prim"], err_msg=str(caps))


@pytest.mark.parametrize("prec", [L.FP64, L.FP32])
def test_autotuner_changes_no_result(fvm_lib, prec):
    """The tuner times each form of the iteration on the resident solves;
    its iterations are ordinary iterations, so a tuned solve equals an
    untuned one bit for bit."""
    from fvm2d_gb300.batch import Batch
    g1, g2 = naca_ogrid(96, 40, jitter=0.1, seed=3), naca_ogrid(64, 24)
    ms = [fvm_lib.build_geometry(g.coord, g.elem, g.ptype) for g in (g1, g2)]
    flows = [dict(mach=0.8, aoa_deg=1.25),
             dict(iflow=L.LAMINAR, mach=0.5, aoa_deg=1.0, rey=5000.0, cfl=0.8)]
    n = 40
    ref = run_variant(fvm_lib, prec, ms, flows, n, viscous=True)
    b = Batch(prec, vertices=sum(m.np for m in ms), meshes=2, viscous=True)
    slots = [b.add(fvm_lib.make_params(precision=prec, **f), m) for m, f in zip(ms, flows)]
    for s in slots:
        b.start(s, n)
    t = b.tune(iters=3)
    assert t["choice"] in Batch.TUNE_CANDIDATES
    timed = [k for k, v in t["ms_per_iter"].items() if v is not None]
    assert t["choice"] in timed and len(timed) >= 6
    assert ("bulk" in timed) == (prec == L.FP32)
    b.step(n)
    for s, (h0, st0) in zip(slots, ref):
        p = b.poll(s)
        assert p["niter"] == n and p["status"] == 0
        np.testing.assert_array_equal(b.history(s, 0, n)["fres"], h0["fres"])
        np.testing.assert_array_equal(b.get_state(s)["prim"], st0["prim"])
    b.close()


@pytest.mark.parametrize("prec", [L.FP64, L.FP32])
def test_state_round_trip_in_driver_order(fvm_lib, prec):
    """set_state/get_state permute and convert on the device: a state set in
    driver order reads back in driver order (exactly in FP64; rounded once
    to FP32 in FP32), and asking for some fields reads the same values."""
    from fvm2d_gb300.batch import Batch
    m = mesh(fvm_lib, 96, 40, seed=3)
    b = Batch(prec, vertices=m.np, meshes=1)
    s = b.add(fvm_lib.make_params(precision=prec, mach=0.8, aoa_deg=1.25), m)
    rng = np.random.default_rng(7)
    prim = 1.0 + 0.1 * rng.random((m.np, 4))
    nut = 1e-3 * rng.random(m.np)
    b.set_state(s, prim, nut=nut)
    full = b.get_state(s)
    want = prim if prec == L.FP64 else prim.astype(np.float32).astype(np.float64)
    np.testing.assert_array_equal(full["prim"], want)
    wnut = nut if prec == L.FP64 else nut.astype(np.float32).astype(np.float64)
    np.testing.assert_array_equal(full["nut"], wnut)
    only = b.get_state(s, fields=("prim",))
    assert set(only) == {"prim"}
    np.testing.assert_array_equal(only["prim"], full["prim"])
    b.close()


def test_bounded_wait_runs_out_with_a_status(fvm_lib):
    """The pipelined gradient pass's waits are bounded: a pass in which each
    CTA's first block is armed for copies that are never issued gives up
    after a short budget (nothing is in flight), the mesh reports
    FVM_ERR_TIMEOUT, and the context stays usable: a fresh batch then steps
    normally and reproduces a solve run before the failure."""
    from fvm2d_gb300.batch import Batch
    m = mesh(fvm_lib, 64, 24)
    flow = dict(mach=0.8, aoa_deg=1.25)
    h0, st0 = alone(fvm_lib, L.FP32, m, flow, 10)
    b = Batch(L.FP32, vertices=m.np, meshes=1)
    s = b.add(fvm_lib.make_params(precision=L.FP32, **flow), m)
    b.start(s, 10)
    b.step(2)
    assert b.poll(s)["status"] == L.OK
    L.check(L.lib().fvm_batch_test_wait_timeout(b.h, 1 << 22), "fvm_batch_test_wait_timeout")
    assert b.poll(s)["status"] == L.ERR_TIMEOUT
    b.close()
    h1, st1 = alone(fvm_lib, L.FP32, m, flow, 10)
    np.testing.assert_array_equal(h1["fres"], h0["fres"])
    np.testing.assert_array_equal(st1["prim"], st0["prim"])


def test_fp32_fused_pass_is_refused(fvm_lib):
    """The fused gradient+flux pass computes triangle-form gradients, which
    FP32 inviscid meshes no longer use: an FP32 batch asking for it is
    refused with FVM_ERR_ARG."""
    from fvm2d_gb300.batch import Batch
    with pytest.raises(L.FvmError) as e:
        Batch(L.FP32, vertices=1000, meshes=1, fused=1)
    assert e.value.status == L.ERR_ARG


def test_fp32_stencil_gradient_matches_triangle_sums(fvm_lib, oracle_lib):
    """The FP32 vertex-stencil Green-Gauss gradient (inviscid meshes) equals
    the oracle's triangle sums to FP32 rounding: both from the same state,
    after a few FP64 iterations."""
    from fvm2d_gb300.ogrid import naca_ogrid
    g = naca_ogrid(96, 40, jitter=0.1, seed=3)
    o = oracle_lib.Oracle(g.coord, g.elem, g.ptype, mach=0.8, aoa_deg=1.25)
    st, _ = o.iterate(5)
    assert st == 0
    s = fvm_lib.Solver(fvm_lib.make_params(precision=L.FP32, mach=0.8, aoa_deg=1.25),
                       o.mesh_arrays())
    sc = o.scalars()
    s.set_state(o.d("prim"), o.d("nut"), o.d("mul"), o.d("mu"), iterlast=sc["iter"])
    o.residu()
    s.residu()
    got = s.get_state()
    for k in ("qx", "qy"):
        ref = o.d(k)
        scale = np.abs(ref).max(axis=0)
        err = np.abs(got[k] - ref).max(axis=0) / scale
        assert np.all(err < 2e-5), f"{k}: {err}"


def test_fp32_runtime_constants_build(fvm_lib):
    """A mesh whose constants differ from math.f's (here the limiter's
    epsilon) sends the FP32 flux pass to its build with runtime constants,
    for every resident mesh.  A standard mesh in such a mix stays within
    FP32 rounding of its solve alone (the builds differ only in what the
    compiler rounds ahead), and the other mesh's solve (epsilon only keeps
    the limiter's quotient defined) within the same tolerance of it."""
    from fvm2d_gb300.batch import Batch
    m = mesh(fvm_lib, 96, 40, seed=3)
    flow = dict(mach=0.8, aoa_deg=1.25)
    n = 30
    h0, st0 = alone(fvm_lib, L.FP32, m, flow, n)
    b = Batch(L.FP32, vertices=2 * m.np + 5000, meshes=2)
    pa = fvm_lib.make_params(precision=L.FP32, **flow)
    pb = fvm_lib.make_params(precision=L.FP32, **flow)
    pb.epsilon = 2.0e-16
    slots = [b.add(pa, m), b.add(pb, m)]
    for s in slots:
        b.start(s, n)
    b.step(n)
    for s in slots:
        p = b.poll(s)
        assert p["status"] == 0 and p["niter"] == n
        np.testing.assert_allclose(b.get_state(s)["prim"], st0["prim"], rtol=1e-4, atol=1e-6)
        np.testing.assert_allclose(b.history(s, 0, n)["fres"], h0["fres"], rtol=1e-3)
    b.close()
