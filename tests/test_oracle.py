"""Pins for the CPU oracle (no GPU).

The reference ships no tests, golden vectors or grids, and cannot be
compiled here (no Fortran compiler), so the oracle is pinned by answers
derived from the equations, plus the committed golden fixtures of
tests/golden/ (which the oracle must keep reproducing):
  * Roe and KFVS return the exact Euler flux for equal states; so does
    HLLC once its momentum flux is rotated back (bugcompat=0);
  * every flux is rotationally invariant, and so is the whole unlimited
    Roe scheme (grid and freestream rotated together);
  * a uniform freestream gives a zero residual at interior points, with
    and without the viscous terms;
  * Green-Gauss reproduces linear fields exactly at every point;
  * the van Albada limiter is 0 on a sign change;
  * the residual history falls on the 160x48 workload.
"""
import numpy as np
import pytest

from fvm2d_gb300.ogrid import naca_ogrid, workload_grid


@pytest.fixture(scope="module")
def small_grid():
    return naca_ogrid(64, 24, radius=20.0, first_spacing=2e-3)


def euler_flux(prim, ds, gamma=1.4):
    r, u, v, p = prim
    length = np.hypot(*ds)
    nx, ny = ds[0] / length, ds[1] / length
    un = u * nx + v * ny
    E = p / (gamma - 1) + 0.5 * r * (u * u + v * v)
    return np.array([r * un, p * nx + r * u * un, p * ny + r * v * un, (E + p) * un]) * length


def random_state(rng):
    return np.array([rng.uniform(0.5, 2.0), rng.uniform(-1, 1), rng.uniform(-1, 1),
                     rng.uniform(0.3, 3.0)])


@pytest.mark.parametrize("iflux,bugcompat", [(1, 1), (2, 1), (3, 0)])
def test_flux_consistency(oracle_lib, small_grid, iflux, bugcompat):
    o = oracle_lib.Oracle(small_grid.coord, small_grid.elem, small_grid.ptype,
                          bugcompat=bugcompat)
    rng = np.random.default_rng(1)
    for _ in range(50):
        q = random_state(rng)
        ds = rng.normal(size=2)
        st, f = o.flux(iflux, ds, q, q)
        assert st == 0
        np.testing.assert_allclose(f, euler_flux(q, ds), rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("iflux,bugcompat", [(1, 1), (2, 1), (3, 0)])
def test_flux_rotational_invariance(oracle_lib, small_grid, iflux, bugcompat):
    o = oracle_lib.Oracle(small_grid.coord, small_grid.elem, small_grid.ptype,
                          bugcompat=bugcompat)
    rng = np.random.default_rng(2)
    for _ in range(50):
        ql, qr = random_state(rng), random_state(rng)
        ds = rng.normal(size=2)
        th = rng.uniform(0, 2 * np.pi)
        c, s = np.cos(th), np.sin(th)
        R = np.array([[c, -s], [s, c]])

        def rot(q):
            out = q.copy()
            out[1:3] = R @ q[1:3]
            return out
        _, f = o.flux(iflux, ds, ql, qr)
        _, fr = o.flux(iflux, R @ ds, rot(ql), rot(qr))
        np.testing.assert_allclose(fr, rot(f), rtol=1e-10, atol=1e-11)


def test_hllc_reference_form_differs(oracle_lib, small_grid):
    """hllc_flux.f:149-154 returns the normal/tangential momentum flux."""
    o = oracle_lib.Oracle(small_grid.coord, small_grid.elem, small_grid.ptype, bugcompat=1)
    q = np.array([1.0, 0.3, 0.4, 1.0])
    ds = np.array([0.0, 1.0])
    _, f = o.flux(3, ds, q, q)
    ex = euler_flux(q, ds)
    assert np.isclose(f[1], ex[2]) and np.isclose(f[2], -ex[1])


@pytest.mark.parametrize("iflux,bugcompat", [(1, 1), (2, 1), (3, 0)])
def test_freestream_preservation(oracle_lib, small_grid, iflux, bugcompat):
    o = oracle_lib.Oracle(small_grid.coord, small_grid.elem, small_grid.ptype, iflux=iflux,
                          bugcompat=bugcompat)
    o.residu()
    res = o.d("res")
    interior = small_grid.ptype == 0
    scale = np.abs(o.d("ds")).max() * 1.0
    assert np.abs(res[interior]).max() < 1e-12 * scale
    assert np.abs(o.d("qx")).max() < 1e-12 and np.abs(o.d("qy")).max() < 1e-12


def test_green_gauss_linear(oracle_lib, small_grid):
    o = oracle_lib.Oracle(small_grid.coord, small_grid.elem, small_grid.ptype)
    x, y = small_grid.coord[:, 0], small_grid.coord[:, 1]
    g = np.array([[0.01, -0.02], [0.3, 0.1], [-0.2, 0.05], [0.04, 0.02]])
    prim = o.d("prim")
    prim[:] = np.array([1.0, 0.5, 0.1, 0.8])[None, :] + x[:, None] * g[:, 0] + y[:, None] * g[:, 1]
    o.residu()
    np.testing.assert_allclose(o.d("qx"), np.broadcast_to(g[:, 0], prim.shape), rtol=1e-9, atol=1e-11)
    np.testing.assert_allclose(o.d("qy"), np.broadcast_to(g[:, 1], prim.shape), rtol=1e-9, atol=1e-11)


def test_limiter(oracle_lib):
    la = oracle_lib.limit_albada
    assert la(1.0, -2.0) == 0.0 and la(-1.0, 2.0) == 0.0 and la(0.0, 5.0) == 0.0
    assert np.isclose(la(1.0, 1.0), 1.0)
    assert np.isclose(la(2.0, 3.0), la(3.0, 2.0))
    assert 0 < la(1.0, 3.0) < 3.0


def test_residual_history_falls(oracle_lib):
    g = workload_grid("euler_160x48")
    o = oracle_lib.Oracle(g.coord, g.elem, g.ptype, mach=0.8, aoa_deg=1.25, cfl=1.0)
    st, h = o.iterate(150)
    assert st == 0 and h["fres"][0] == 1.0
    assert h["fres"][-1] < 0.05
    assert 0.0 < h["cl"][-1] < 0.6


def test_hllc_reference_form_blows_up(oracle_lib):
    """With the reference HLLC (no rotation back) the 160x48 run stops on a
    non-positive pressure in its first iteration; the corrected form runs."""
    g = workload_grid("euler_160x48")
    o = oracle_lib.Oracle(g.coord, g.elem, g.ptype, iflux=3, bugcompat=1)
    st, h = o.iterate(5)
    assert st == 3  # ORC_ERR_NONPOSITIVE
    o2 = oracle_lib.Oracle(g.coord, g.elem, g.ptype, iflux=3, bugcompat=0)
    st2, h2 = o2.iterate(5)
    assert st2 == 0 and len(h2["fres"]) == 5


def test_bugcompat_switches_change_results(oracle_lib, small_grid):
    kw = dict(iflow=3, mach=0.7, aoa_deg=2.0, rey=6.5e6, cfl=0.5, nut_ratio=3.0)
    a = oracle_lib.Oracle(small_grid.coord, small_grid.elem, small_grid.ptype, bugcompat=1, **kw)
    b = oracle_lib.Oracle(small_grid.coord, small_grid.elem, small_grid.ptype, bugcompat=0, **kw)
    assert not np.array_equal(a.d("wd"), b.d("wd"))
    a.iterate(3)
    b.iterate(3)
    assert not np.array_equal(a.d("nut"), b.d("nut"))


GOLDEN = __import__("os").path.join(__import__("os").path.dirname(__file__), "golden")


@pytest.mark.parametrize("name", ["euler_160x48_roe", "laminar_64x24_roe"])
def test_oracle_reproduces_golden_history(oracle_lib, name):
    """tests/golden/ fixtures (written by tests/golden/make_golden.py):
    RES.DAT columns and final-state checksums.  Exact up to libm (the
    laminar case calls pow)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", f"{GOLDEN}/make_golden.py")
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    ref = np.load(f"{GOLDEN}/{name}.npz")
    got = mg.run_case(name)
    tol = 0.0 if name.startswith("euler") else 1e-12
    assert int(got["status"]) == int(ref["status"]) == 0
    np.testing.assert_array_equal(got["iresi"], ref["iresi"])
    for k in ("fres", "fresi", "cl", "cd", "prim_sum", "prim_sq", "prim_first"):
        np.testing.assert_allclose(got[k], ref[k], rtol=tol, atol=0, err_msg=k)


def test_oracle_reproduces_golden_fluxes(oracle_lib):
    ref = np.load(f"{GOLDEN}/fluxes.npz")
    g = naca_ogrid(20, 8)
    for iflux, bugcompat, key, tol in ((1, 1, "roe", 0.0), (2, 1, "kfvs", 1e-13),
                                       (3, 0, "hllc", 1e-13)):
        o = oracle_lib.Oracle(g.coord, g.elem, g.ptype, iflux=iflux, bugcompat=bugcompat)
        for k in range(len(ref["ds"])):
            st, f = o.flux(iflux, ref["ds"][k], ref["priml"][k], ref["primr"][k])
            assert st == ref[key + "_status"][k]
            np.testing.assert_allclose(f, ref[key][k], rtol=tol, atol=1e-300, err_msg=key)


@pytest.mark.parametrize("iflow", [2, 3])
def test_freestream_preservation_viscous(oracle_lib, small_grid, iflow):
    """A uniform state has zero gradients, so the Green-Gauss viscous terms
    (stresses and heat flux from the triangle gradients, with the SA eddy
    viscosity in the turbulent case) vanish with the inviscid fluxes at
    interior points."""
    kw = dict(iflow=iflow, mach=0.5, aoa_deg=2.0, rey=5000.0 if iflow == 2 else 6.5e6, cfl=0.5,
              bugcompat=0)
    if iflow == 3:
        kw.update(iflux=3, nut_ratio=3.0)
    o = oracle_lib.Oracle(small_grid.coord, small_grid.elem, small_grid.ptype, **kw)
    o.residu()
    res = o.d("res")
    interior = small_grid.ptype == 0
    scale = np.abs(o.d("ds")).max()
    assert np.abs(res[interior]).max() < 1e-12 * scale
    assert np.abs(o.d("qx")).max() < 1e-12 and np.abs(o.d("qy")).max() < 1e-12


def test_whole_scheme_rotational_invariance(oracle_lib):
    """Rotating the grid and the freestream by the same angle rotates the
    solution: without the limiter (van Albada acts on u and v separately)
    every step of the Roe scheme is covariant, so after a few iterations
    rho and p agree, (u, v) rotate, and the residual history and the
    wind-axis cl, cd are unchanged."""
    g = naca_ogrid(48, 20, radius=15.0, first_spacing=3e-3)
    th = np.deg2rad(23.0)
    c, s = np.cos(th), np.sin(th)
    R = np.array([[c, -s], [s, c]])
    kw = dict(mach=0.6, iflux=1, ilimit=0, cfl=0.8)
    a = oracle_lib.Oracle(g.coord, g.elem, g.ptype, aoa_deg=2.0, **kw)
    b = oracle_lib.Oracle(g.coord @ R.T, g.elem, g.ptype, aoa_deg=2.0 + 23.0, **kw)
    sa, ha = a.iterate(6)
    sb, hb = b.iterate(6)
    assert sa == sb == 0
    pa, pb = a.d("prim"), b.d("prim")
    np.testing.assert_allclose(pb[:, 0], pa[:, 0], rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(pb[:, 3], pa[:, 3], rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(pb[:, 1:3], pa[:, 1:3] @ R.T, rtol=1e-9, atol=1e-11)
    np.testing.assert_allclose(hb["fres"], ha["fres"], rtol=1e-8)
    np.testing.assert_allclose(hb["cl"], ha["cl"], rtol=1e-8, atol=1e-12)
    np.testing.assert_allclose(hb["cd"], ha["cd"], rtol=1e-8, atol=1e-12)


def test_edge_gradient_linear(oracle_lib, small_grid):
    """gradient.f (edge-based Green-Gauss over the dual cells with the 5/6,
    1/6 boundary closure) is exact for linear fields at every vertex,
    boundary vertices included."""
    g = naca_ogrid(64, 24, jitter=0.1, seed=3)
    o = oracle_lib.Oracle(g.coord, g.elem, g.ptype)
    c = o.d("coord")
    prim = o.d("prim")
    a = np.array([0.3, -1.2, 0.7, 2.0])
    bx = np.array([1.5, 0.2, -0.4, 0.9])
    by = np.array([-0.6, 1.1, 0.3, -2.0])
    prim[:] = a + np.outer(c[:, 0], bx) + np.outer(c[:, 1], by)
    o.gradient()
    assert np.abs(o.d("qx") - bx).max() < 1e-9
    assert np.abs(o.d("qy") - by).max() < 1e-9


def test_shock_indicator(oracle_lib):
    """shockind.f: a uniform state gives an indicator at rounding level
    (the edge gradients of a constant are rounding noise) and keeps every
    gradient; a density step gives an indicator above 1 next to the step,
    where the gradients are then zero, and leaves them elsewhere."""
    g = naca_ogrid(64, 24, jitter=0.1, seed=3)
    o = oracle_lib.Oracle(g.coord, g.elem, g.ptype)
    o.gradient()
    qx0 = o.d("qx").copy()
    ind = o.shockind()
    assert np.all(ind < 1e-12)
    np.testing.assert_array_equal(o.d("qx"), qx0)
    prim = o.d("prim")
    c = o.d("coord")
    prim[:, 0] = np.where(c[:, 0] > 0.5, 1.5, 1.0)          # a density step at x = 0.5
    o.gradient()
    qx0 = o.d("qx").copy()
    ind = o.shockind()
    assert np.all(ind >= 0.0)
    hit = ind > 1.0
    near = np.abs(c[:, 0] - 0.5) < 0.2
    assert hit.any() and np.all(near[hit])
    np.testing.assert_array_equal(o.d("qx")[hit], 0.0)
    np.testing.assert_array_equal(o.d("qx")[~hit], qx0[~hit])
