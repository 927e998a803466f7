"""The device octree (include/lpm_octree.h, octree.cu) against the oracle's restatement of
src/LpmOctree.cpp: every array bit for bit -- box, level sizes and base addresses, keys, point
ranges, parents, kids, neighbours, sorted points, original ids and point-to-leaf map -- on the
reference's own test input (cubed-sphere level-6 sourceCoords, depth 4), on non-cubic point sets
(box2cube), at depths 1..10, for LayoutLeft strides, and on a level-8-sized point set."""
import numpy as np
import pytest
import torch

from lpmkokkos_gb300 import bve

pytestmark = pytest.mark.gpu


def _same(dev, ref):
    T = dev.arrays()
    assert np.array_equal(dev.box, ref["box"])
    assert np.array_equal(dev.nnodes_per_level, ref["nnodes_per_level"])
    assert np.array_equal(dev.base_address, ref["base_address"])
    assert np.array_equal(T["keys"], ref["keys"])
    for name in ("pt_inds", "parents", "kids", "sorted_pts", "orig_ids", "pt_in_leaf"):
        assert np.array_equal(T[name].cpu().numpy(), ref[name]), name
    if T["neighbors"] is not None:
        assert np.array_equal(T["neighbors"].cpu().numpy(), ref["neighbors"])


def _source_coords(seed, level):
    m = bve.build_mesh(seed, level)
    return np.concatenate([m["vx"], m["fx"][m["fmask"] == 0]])


def test_reference_test_input(oracle):
    x = _source_coords(1, 6)  # tests/LpmOctreeKernelTests.cpp:27-46
    t = bve.Octree(torch.from_numpy(x).cuda(), 4)
    _same(t, oracle.octree(x, 4))
    assert np.array_equal(t.box, [-1, 1, -1, 1, -1, 1])


@pytest.mark.parametrize("depth", [1, 2, 3, 6, 10])
def test_depths_on_non_cubic_box(oracle, depth):
    m = bve.build_mesh(0, 5)
    x = m["fx"][m["fmask"] == 0]
    t = bve.Octree(torch.from_numpy(x).cuda(), depth)
    _same(t, oracle.octree(x, depth))


def test_layout_left_and_clustered_points(oracle):
    rng = np.random.default_rng(3)
    x = np.concatenate([rng.normal(size=(20000, 3)) * 0.01 + [0.3, -0.2, 0.9], rng.uniform(-1, 1, size=(5000, 3))])
    xl = torch.from_numpy(x).t().contiguous().cuda().t()  # column-major, as Kokkos lays out on CUDA
    t = bve.Octree(xl, 7)
    _same(t, oracle.octree(x, 7))


def test_level8_sized_points_no_neighbours(oracle):
    x = _source_coords(0, 8)  # 1,966,082 points
    t = bve.Octree(torch.from_numpy(x).cuda(), 6, neighbors=False)
    ref = oracle.octree(x, 6)
    T = t.arrays()
    assert T["neighbors"] is None
    assert np.array_equal(T["keys"], ref["keys"])
    for name in ("pt_inds", "parents", "kids", "orig_ids", "pt_in_leaf"):
        assert np.array_equal(T[name].cpu().numpy(), ref[name]), name


def test_rebuild_reuses_the_tree_object(oracle):
    """Two builds of different sizes through the engine's buffers give independent results."""
    a = _source_coords(1, 5)
    b = _source_coords(0, 4)
    ta = bve.Octree(torch.from_numpy(a).cuda(), 5)
    tb = bve.Octree(torch.from_numpy(b).cuda(), 3)
    _same(tb, oracle.octree(b, 3))
    _same(ta, oracle.octree(a, 5))


def test_invalid_arguments():
    from lpmkokkos_gb300 import _lib as L
    import ctypes
    x = torch.zeros(4, 3, dtype=torch.float64, device="cuda")
    h = ctypes.c_void_p()
    for n, d in ((0, 3), (4, 0), (4, 11)):
        assert L.lib().lpm_octree_build(x.data_ptr(), 3, 1, n, d, 1, ctypes.byref(h), None) \
            == L.LPM_ERR_INVALID_ARGUMENT


@pytest.mark.skipif(torch.cuda.device_count() < 2, reason="needs a second GPU")
def test_neighbour_tables_on_a_second_device(oracle):
    """The neighbour tables live in __constant__ memory, which is per device: an octree built
    on device 1 after one on device 0 gets the same neighbour lists as the oracle."""
    x = _source_coords(1, 5)
    t0 = bve.Octree(torch.from_numpy(x).cuda(0), 3)
    t0.close()
    with torch.cuda.device(1):
        t1 = bve.Octree(torch.from_numpy(x).cuda(1), 3)
        _same(t1, oracle.octree(x, 3))
        t1.close()


@pytest.mark.parametrize("seed,level,depth", [(1, 6, 4), (0, 7, 5), (0, 5, 1), (1, 4, 6)])
def test_fixed_level_build_equals_concatenated(oracle, seed, level, depth):
    """The sync-free build (LPM_OCTREE_FIXED_LEVELS, used by the tree code): every level's first
    nnodes_per_level[l] nodes at its fixed base equal the oracle's level l (keys, point ranges,
    parents, kids), the rest have empty point ranges; per-point arrays equal the oracle's."""
    x = _source_coords(seed, level)
    ref = oracle.octree(x, depth)
    t = bve.Octree(torch.from_numpy(x).cuda(), depth, neighbors=False, fixed_levels=True)
    T = t.arrays()
    assert np.array_equal(t.nnodes_per_level, ref["nnodes_per_level"])
    assert np.array_equal(t.box, ref["box"])
    pt = T["pt_inds"].cpu().numpy()
    for lev in range(depth + 1):
        b, m, rb = t.base_address[lev], ref["nnodes_per_level"][lev], ref["base_address"][lev]
        cap = (t.base_address[lev + 1] if lev < depth else t.nnodes) - b
        assert cap >= m
        assert np.array_equal(T["keys"][b:b + m], ref["keys"][rb:rb + m]), lev
        for name in ("pt_inds", "parents", "kids"):
            assert np.array_equal(T[name].cpu().numpy()[b:b + m], ref[name][rb:rb + m]), (lev, name)
        assert (pt[b + m:b + cap, 1] == 0).all(), lev
    for name in ("sorted_pts", "orig_ids", "pt_in_leaf"):
        assert np.array_equal(T[name].cpu().numpy(), ref[name]), name
    t.close()
