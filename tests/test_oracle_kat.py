"""Pin the CPU oracle against the reference's own known-answer tests.

The reference's unit tests (test/test_interpolation.f90:26-64,
test/test_search.f90:67-83, test/test_pcorvcor.f90:33-73) hold the only
golden values for this path; they are restated here against the oracle.
"""
import ctypes as C

import numpy as np

from oracle.bridge import Oracle, lib


def _prims():
    L = lib()
    L.orc_linear_interpolation.restype = C.c_double
    L.orc_linear_interpolation.argtypes = [C.c_double] * 5
    L.orc_bilinear_interpolation.restype = C.c_double
    L.orc_bilinear_interpolation.argtypes = [C.c_double] * 6 + [C.POINTER(C.c_double)]
    return L


def test_linear_interpolation_kat():
    # test/test_interpolation.f90:26-43
    L = _prims()
    assert L.orc_linear_interpolation(1.5, 2.0, 1.0, 2.0, 1.0) == 1.5
    assert L.orc_linear_interpolation(3.0, 2.0, 1.0, 2.0, 1.0) == 3.0      # extrapolation
    assert L.orc_linear_interpolation(50.0, 100.0, 1.0, 1.0, 1.0) == 1.0   # flat
    assert L.orc_linear_interpolation(0.5, 1.0, 0.0, 0.0, 10.0) == 5.0     # negative slope


def test_bilinear_interpolation_kat():
    # test/test_interpolation.f90:48-64
    L = _prims()
    f = (C.c_double * 4)(1.0, 1.0, 1.0, 1.0)
    assert L.orc_bilinear_interpolation(0.5, 0.5, 0.0, 1.0, 0.0, 1.0, f) == 1.0
    g = (C.c_double * 4)(1.0, 2.0, 3.0, 4.0)
    assert L.orc_bilinear_interpolation(2.0, 0.5, 0.0, 1.0, 0.0, 1.0, g) == 4.0


def test_cellcount_solid_coarse_kat():
    # test/test_search.f90:67-83: all-fluid 5^3 block -> fluid = 125 and
    # red + black = fluid
    o = Oracle()
    g = o.L.orc_block_new(5, 5, 5)
    o.arr(g, "cell")[...] = 0
    o.L.orc_cellcount_solid_coarse(g)
    assert o.geti(g, "fluidCellCount") == 125
    assert o.geti(g, "redCellCount") + o.geti(g, "blackCellCount") == 125
    # red cells are those with odd i+j+k (1-based, halo included)
    red = o.arr(g, "redCellIndexPtr")
    assert np.all(red.sum(axis=1) % 2 == 1)


def test_update_velocity_newv_kat():
    # test/test_pcorvcor.f90:33-73: with move_check = 1, ut/vt/wt <- u/v/w
    o = Oracle()
    g = o.L.orc_block_new(5, 5, 5)
    for nm, val in (("u", 1), ("v", 2), ("w", 3), ("ut", 4), ("vt", 5), ("wt", 6)):
        o.arr(g, nm)[...] = val
    assert not np.any(o.arr(g, "u") == o.arr(g, "ut"))
    o.seti(g, "move_check", 1)
    o.L.orc_update_velocity_newv(g)
    for a, b in (("u", "ut"), ("v", "vt"), ("w", "wt")):
        assert np.all(o.arr(g, a) == o.arr(g, b))


def test_update_velocity_newv_noop_without_move():
    o = Oracle()
    g = o.L.orc_block_new(5, 5, 5)
    o.arr(g, "u")[...] = 1
    o.arr(g, "ut")[...] = 4
    o.L.orc_update_velocity_newv(g)
    assert np.all(o.arr(g, "ut") == 4)


def test_find_dist_node_kat():
    # test/test_search.f90:47-54: six surface-51 nodes with x = y = z =
    # (0, -7, -4, 1, -10, 8) -> mk = 6 (the running value keeps the signed z)
    o = Oracle()
    g = o.L.orc_block_new(5, 5, 5)
    o.L.orc_alloc_surface(g, 1, 6)  # 1 element, 6 nodes
    vals = np.array([0.0, -7.0, -4.0, 1.0, -10.0, 8.0])
    for nm in ("xnode", "ynode", "znode"):
        o.arr(g, nm)[:] = vals
    o.arr(g, "ibNodeId")[:] = 51
    o.L.orc_find_dist_node(g)
    assert o.geti(g, "mk") == 6
    # the same rule for x: mkx1 follows |x| below the signed running value,
    # mkx2 above it
    assert o.geti(g, "mkx1") == 1 and o.geti(g, "mkx2") == 6
