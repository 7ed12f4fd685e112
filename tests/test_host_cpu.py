"""Host-side checks that need no GPU: the C-ABI library loads and exports
every function include/fvm_gpu.h declares; the driver-side geometry of the
library equals the oracle's bit for bit; the constants of fvm_params_init
equal math.f/initialize.f as restated by the oracle; the grid generator
and the amdba reader/writer."""
import ctypes
import os
import re

import numpy as np
import pytest

from fvm2d_gb300 import _lib as L
from fvm2d_gb300.ogrid import (POINT_FARFIELD, POINT_SOLID, naca_ogrid, read_amdba,
                               workload_grid, write_amdba)

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    txt = open(os.path.join(ROOT, "include", "fvm_gpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(fvm_\w+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(fvm_lib):
    names = header_functions()
    assert len(names) >= 23
    from fvm2d_gb300 import build
    for path in (build.LIB, build.LIB_FP64FMA):   # the main and the FP64-FMA library
        lib = ctypes.CDLL(path)
        missing = [n for n in names if not hasattr(lib, n)]
        assert not missing, (path, missing)
    assert set(names) == set(L.SIGNATURES), set(names) ^ set(L.SIGNATURES)


def test_oracle_exports_every_declared_symbol(oracle_lib):
    txt = open(os.path.join(ROOT, "oracle", "fvm_oracle.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    names = set(re.findall(r"\b(orc_\w+)\s*\(", txt))
    lib = ctypes.CDLL(oracle_lib.LIB_PATH)
    assert names and all(hasattr(lib, n) for n in names)


def test_strerror(fvm_lib):
    assert L.lib().fvm_gpu_strerror(L.ERR_NONPOSITIVE).decode().startswith("Density/pressure")
    assert L.lib().fvm_gpu_strerror(L.ERR_ROE_SONIC).decode() == "Sonic speed is negative"


def test_params_match_oracle(oracle_lib, fvm_lib):
    g = naca_ogrid(32, 12)
    for kw in (dict(iflow=1, mach=0.8, aoa_deg=1.25), dict(iflow=2, mach=0.5, aoa_deg=0.0, rey=5000.0),
               dict(iflow=3, mach=0.7, aoa_deg=2.0, rey=6.5e6, nut_ratio=3.0)):
        o = oracle_lib.Oracle(g.coord, g.elem, g.ptype, **kw)
        s = o.scalars()
        p = fvm_lib.make_params(**kw)
        for k in ["gamma", "gamma1", "pi", "prandtl", "prandtl_turb", "albada11", "albada12",
                  "albada21", "albada22", "cb1", "cb2", "sigma_sa", "kolm", "cw1", "cw2", "cw3",
                  "cv1", "cv2", "cv11", "cw31", "cw32", "kolm2", "cb2sig1", "cb2sig2",
                  "mach_inf", "aoa", "q_inf", "r_inf", "p_inf", "t_inf", "u_inf", "v_inf",
                  "a_inf", "sconst", "nut_inf"]:
            assert getattr(p, k) == s[k], k
        assert list(p.airk) == s["airk"] and list(p.birk) == s["birk"]


def test_params_reject_bad_input(fvm_lib):
    for bad in (dict(iflux=4), dict(iflow=0), dict(ilimit=2), dict(cell_type=3), dict(mach=0.0)):
        with pytest.raises(L.FvmError) as e:
            fvm_lib.make_params(**bad)
        assert e.value.status == L.ERR_ARG


@pytest.mark.parametrize("case", ["median", "barth", "jitter", "camber"])
def test_host_geometry_equals_oracle(oracle_lib, fvm_lib, case):
    g = {"median": lambda: workload_grid("euler_160x48"),
         "barth": lambda: naca_ogrid(96, 32),
         "jitter": lambda: naca_ogrid(96, 40, jitter=0.1, seed=7),
         "camber": lambda: naca_ogrid(80, 30, thickness=0.09, camber=0.04, camber_pos=0.3)}[case]()
    cell = L.BARTH if case == "barth" else L.MEDIAN
    m = fvm_lib.build_geometry(g.coord, g.elem, g.ptype, cell_type=cell, setup_on_gpu=False)
    o = oracle_lib.Oracle(g.coord, g.elem, g.ptype, cell_type=cell)
    om = o.mesh_arrays()
    for k in ["np", "nt", "ne", "netot", "nsp", "nbe", "nswe1", "nswe2", "nffe1", "nffe2"]:
        assert getattr(m, k) == om[k], k
    for k in ["elem", "edge", "edneigh", "iedge", "beindx", "spts"]:
        np.testing.assert_array_equal(np.asarray(getattr(m, k)).ravel(), om[k].ravel(), err_msg=k)
    for k in ["ds", "dsb", "elarea", "cvarea", "mcarea"]:
        np.testing.assert_array_equal(np.asarray(getattr(m, k)).ravel(), om[k].ravel(), err_msg=k)
    if case == "barth":
        assert m.ne < m.netot      # zero-length Barth faces dropped (flength.f:84-98)


@pytest.mark.parametrize("case", ["median", "barth", "jitter", "tiny"])
def test_block_layout_invariants(fvm_lib, case):
    """The fused pass reads halo gradients that it computes itself: every
    edge's local slots must decode to its ends, and every halo vertex must
    list the same triangles in the same order as its owner block (so both
    sum them in the same order).  Checked by the library on the host."""
    from fvm2d_gb300.batch import layout_stats
    g = {"median": lambda: workload_grid("euler_160x48"),
         "barth": lambda: naca_ogrid(96, 32),
         "jitter": lambda: naca_ogrid(96, 40, jitter=0.1, seed=3),
         "tiny": lambda: naca_ogrid(20, 8)}[case]()
    cell = L.BARTH if case == "barth" else L.MEDIAN
    m = fvm_lib.build_geometry(g.coord, g.elem, g.ptype, cell_type=cell, setup_on_gpu=False)
    st = layout_stats(m)
    assert st["layout_violations"] == 0
    assert st["max_loc"] <= 576 and st["max_tri2"] <= 1280       # default tiles
    assert st["max_tri2"] >= st["max_tri"]
    assert (st["halo_entries"] > 0) == (st["blocks"] > 1)


def test_geometry_rejects_degenerate(fvm_lib):
    coord = np.array([[0.0, 0.0], [1.0, 0.0], [2.0, 0.0], [0.0, 1.0]])
    elem = np.array([[1, 2, 3], [1, 2, 4]], dtype=np.int32)
    ptype = np.zeros(4, dtype=np.int32)
    with pytest.raises(L.FvmError) as e:
        fvm_lib.build_geometry(coord, elem, ptype, setup_on_gpu=False)
    assert e.value.status == L.ERR_GEOMETRY


@pytest.mark.parametrize("name", ["euler_160x48", "laminar_512x192"])
def test_ogrid_properties(name):
    g = workload_grid(name)
    ni, nr = g.ni, g.nr
    assert g.np == ni * nr and g.nt == 2 * ni * (nr - 1)
    assert (g.ptype == POINT_SOLID).sum() == ni and (g.ptype == POINT_FARFIELD).sum() == ni
    c, e = g.coord, g.elem - 1
    area = 0.5 * ((c[e[:, 1], 0] - c[e[:, 0], 0]) * (c[e[:, 2], 1] - c[e[:, 0], 1])
                  - (c[e[:, 2], 0] - c[e[:, 0], 0]) * (c[e[:, 1], 1] - c[e[:, 0], 1]))
    assert np.all(area != 0)
    # every vertex used, each edge shared by at most two triangles
    assert np.unique(e).size == g.np
    r = np.hypot(c[g.ptype == POINT_FARFIELD, 0] - 0.5, c[g.ptype == POINT_FARFIELD, 1])
    assert np.allclose(r, g.coord[g.ptype == POINT_FARFIELD][0, 0] - 0.5)


def test_ogrid_jitter_is_seeded():
    a = naca_ogrid(64, 20, jitter=0.1, seed=3)
    b = naca_ogrid(64, 20, jitter=0.1, seed=3)
    c = naca_ogrid(64, 20, jitter=0.1, seed=4)
    np.testing.assert_array_equal(a.coord, b.coord)
    assert not np.array_equal(a.coord, c.coord)
    # wall and farfield points are not moved
    d = naca_ogrid(64, 20)
    np.testing.assert_array_equal(a.coord[:64], d.coord[:64])


def test_amdba_roundtrip(tmp_path):
    g = naca_ogrid(40, 12, jitter=0.05, seed=1)
    p = tmp_path / "grid.amdba"
    write_amdba(str(p), g)
    h = read_amdba(str(p))
    np.testing.assert_array_equal(h.coord, g.coord)
    np.testing.assert_array_equal(h.elem, g.elem)
    np.testing.assert_array_equal(h.ptype, g.ptype)


def test_wall_table_and_sol_roundtrip(fvm_lib, oracle_lib, tmp_path):
    """WALL.DAT columns (result.f:92-118) and the SOL restart file
    (finalize.f:14-24 / initialize.f:91-103) from an oracle state."""
    from fvm2d_gb300 import results
    g = naca_ogrid(48, 16)
    o = oracle_lib.Oracle(g.coord, g.elem, g.ptype, iflow=L.LAMINAR, mach=0.5, rey=2000.0,
                          cfl=0.5)
    from fvm2d_gb300.solver import MeshArrays
    m = MeshArrays(o.mesh_arrays())
    m.wd = oracle_lib.wall_dist(m.coord, m.edge, m.ptype, bugcompat=0)
    par = fvm_lib.make_params(iflow=L.LAMINAR, mach=0.5, rey=2000.0, cfl=0.5)

    def state():
        return {k: o.d(k).copy() for k in ("prim", "qx", "qy", "mu", "nut")}
    st0 = state()
    t0 = results.wall_table(m, st0, par, L.LAMINAR)
    np.testing.assert_allclose(t0["cp"], 0.0, atol=1e-12)       # freestream start
    o.iterate(5)
    st = state()
    t = results.wall_table(m, st, par, L.LAMINAR)
    assert t["x"].shape == t["cp"].shape == t["cf"].shape == (m.nsp,)
    assert np.all(np.isfinite(t["cf"])) and np.all(t["wd1"] > 0) and np.all(t["yplus"] >= 0)
    p = tmp_path / "SOL"
    results.write_sol(str(p), st["prim"], st["nut"], par.gamma1)
    prim, nut = results.read_sol(str(p), par.gamma1)
    np.testing.assert_allclose(prim, st["prim"], rtol=1e-13, atol=1e-15)
    np.testing.assert_array_equal(nut, st["nut"])
    results.write_wall(str(tmp_path / "WALL.DAT"), t)
    assert np.loadtxt(str(tmp_path / "WALL.DAT")).shape == (m.nsp, 5)


def test_ctypes_mirrors_match_the_abi_structs(fvm_lib):
    """The Python mirrors of fvm_params, fvm_mesh, fvm_geom and
    fvm_batch_caps have the C structs' sizes (a drifted field would shift
    every later one)."""
    import ctypes as C
    out = (C.c_int64 * 4)()
    L.lib().fvm_abi_sizes(out)
    assert list(out) == [C.sizeof(L.FvmParams), C.sizeof(L.FvmMesh), C.sizeof(L.FvmGeom),
                         C.sizeof(L.FvmBatchCaps)]



def test_bench_cli_parses():
    """bench.py's options, including the probe mode used by the viscous-path
    profiles (the runs themselves need a GPU)."""
    import subprocess
    import sys
    r = subprocess.run([sys.executable, "bench.py", "--help"],
                       capture_output=True, text=True, cwd=ROOT, timeout=120)
    assert r.returncode == 0
    for opt in ("--mode", "probe", "--flow", "--meshes", "--steps", "--form", "--precision",
                "--ni", "--nr"):
        assert opt in r.stdout
