"""The driver geometry chain on the GPU (fvm_gpu_geom_build) against the host
restatement (fvm_geom_build, itself equal to the oracle's chain on CPU):
src/geometric.f:15-60 -- tri_orient, el_surr_point, pt_surr_pt,
create_edge, el_surr_edge, tri_coord, areas, flength, reorder_edges,
make_bdedges, geom_stat -- plus dtlength.f.

Integer arrays (edge numbering and orientation, neighbours, boundary lists)
must be identical, and every FP64 array bit for bit: the GPU unit is built
without FMA contraction and sums in the host's order.
"""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from fvm2d_gb300 import _lib as L  # noqa: E402
from fvm2d_gb300.ogrid import naca_ogrid, workload_grid  # noqa: E402

FIELDS_INT = ["elem", "edge", "edneigh", "iedge", "beindx", "spts"]
FIELDS_DBL = ["ds", "dsb", "elarea", "cvarea", "mcarea", "drmin"]


def both(fvm_lib, coord, elem, ptype, cell_type=L.MEDIAN):
    host = fvm_lib.build_geometry(coord, elem, ptype, cell_type=cell_type).as_dict()
    gpu = fvm_lib.build_geometry(coord, elem, ptype, cell_type=cell_type,
                                 chain_on_gpu=True).as_dict()
    return host, gpu


def assert_same(host, gpu):
    for k in ["np", "nt", "ne", "netot", "nsp", "nbe", "nswe1", "nswe2", "nffe1", "nffe2"]:
        assert host[k] == gpu[k], k
    for k in FIELDS_INT:
        np.testing.assert_array_equal(np.asarray(gpu[k]), np.asarray(host[k]), err_msg=k)
    for k in FIELDS_DBL:
        a, b = np.asarray(gpu[k]), np.asarray(host[k])
        assert a.shape == b.shape, k
        # bit for bit (also distinguishes -0.0 from 0.0)
        np.testing.assert_array_equal(a.view(np.int64), b.view(np.int64), err_msg=k)


@pytest.mark.parametrize("cell_type", [L.MEDIAN, L.BARTH])
def test_gpu_chain_equals_host_chain(fvm_lib, cell_type):
    """A jittered O-grid (irregular triangles, a mix of orientations after
    the jitter) for median and Barth cells."""
    g = naca_ogrid(96, 40, jitter=0.1, seed=11)
    host, gpu = both(fvm_lib, g.coord, g.elem, g.ptype, cell_type)
    assert_same(host, gpu)


def test_gpu_chain_reorients_like_the_host(fvm_lib):
    """Triangles given clockwise are turned (tri_orient.f:33-37) the same
    way, so the edge numbering and the neighbours that follow agree."""
    g = naca_ogrid(64, 24, jitter=0.05, seed=4)
    elem = g.elem.copy()
    elem[::3] = elem[::3, ::-1]          # every third triangle clockwise
    host, gpu = both(fvm_lib, g.coord, elem, g.ptype)
    assert_same(host, gpu)
    np.testing.assert_array_equal(np.asarray(gpu["elem"]), np.asarray(host["elem"]))


def test_gpu_chain_full_size_and_timing(fvm_lib):
    """The 1024 x 384 workload grid (393,216 points): equal arrays; the GPU
    chain's wall time is reported beside the host's."""
    g = workload_grid("euler_1024x384")
    t0 = time.perf_counter()
    host = fvm_lib.build_geometry(g.coord, g.elem, g.ptype).as_dict()
    t1 = time.perf_counter()
    gpu = fvm_lib.build_geometry(g.coord, g.elem, g.ptype, chain_on_gpu=True).as_dict()
    t2 = time.perf_counter()
    assert_same(host, gpu)
    print(f"geometry chain 1024x384: host {t1 - t0:.3f} s, gpu {t2 - t1:.3f} s")


def test_gpu_chain_refuses_a_degenerate_triangle(fvm_lib):
    """A zero-area triangle is FVM_ERR_GEOMETRY on both paths."""
    g = naca_ogrid(32, 12)
    elem = np.ascontiguousarray(g.elem.copy(), dtype=np.int32)
    elem[5] = [elem[5][0], elem[5][0], elem[5][1]]   # two equal corners
    for gpu in (False, True):
        with pytest.raises(L.FvmError) as ei:
            fvm_lib.build_geometry(g.coord, elem, g.ptype, chain_on_gpu=gpu)
        assert ei.value.status == L.ERR_GEOMETRY
