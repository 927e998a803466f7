"""The oracle's Morton octree (oracle/lpm_oracle_octree.cpp) against the reference's own octree
tests and tables, on CPU:

  * key algebra -- tests/LpmOctreeKeyTests.cpp: depth-1 key boxes equal the bisected boxes,
    depth-2 cell centroids get their own index as key, parent/local/node keys compose;
  * tree build -- tests/LpmOctreeKernelTests.cpp / LpmNodeArrayDUnitTests.cpp /
    LpmNodeArrayInternalTests.cpp on the same input (cubed-sphere level-6 sourceCoords, octree
    depth 4): root box [-1, 1]^3, every point inside its key's box, codes sorted, counts adding
    up, points inside their leaf's box, full sibling sets, parents and kids consistent;
  * lookup tables -- tests/LpmOctreeLUTUnitTests.cpp identities, and the tables themselves
    against src/LpmOctreeLUT.hpp (tests/golden/octree_tables.json).  The generated ChildLUT
    differs from the reference's in row 0, columns 18-20 and 24-26: there the neighbour of child
    0 lies one cell in +x, so its local key has the x bit (4) set, which the reference's entries
    lack (columns 24-26 also miss the y bit).  Every neighbour is checked here against box
    adjacency instead.
"""
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
UNIT = np.array([-1.0, 1.0, -1.0, 1.0, -1.0, 1.0])


def _bisect(box):
    """bisectBoxAllDims (src/LpmBox3d.hpp): the 8 child boxes, index 4x + 2y + z."""
    cx, cy, cz = (box[0] + box[1]) / 2, (box[2] + box[3]) / 2, (box[4] + box[5]) / 2
    out = []
    for k in range(8):
        x = (box[0], cx) if not k & 4 else (cx, box[1])
        y = (box[2], cy) if not k & 2 else (cy, box[3])
        z = (box[4], cz) if not k & 1 else (cz, box[5])
        out.append(np.array([*x, *y, *z]))
    return out


def test_key_algebra(oracle):
    for k, kb in enumerate(_bisect(UNIT)):  # depth 1
        assert np.array_equal(oracle.octree_box(k, UNIT, 1, 1), kb)
    for k in range(64):  # depth 2: cell centroids
        c = np.zeros(3)
        h = 1.0
        for lev in (1, 2):
            h *= 0.5
            lk = oracle.octree_key(2, k=k, lev=lev, maxd=2)
            c += np.where([lk & 4, lk & 2, lk & 1], h, -h)
        assert oracle.octree_key(0, x=c, box=UNIT, lev=2) == k
        b = oracle.octree_box(k, UNIT, 2, 2)
        assert np.array_equal(((b[0] + b[1]) / 2, (b[2] + b[3]) / 2, (b[4] + b[5]) / 2), c)
        k4 = oracle.octree_key(0, x=c, box=UNIT, lev=4)
        pk, gpk = oracle.octree_key(1, k=k4, lev=4, maxd=4), oracle.octree_key(1, k=k4, lev=3, maxd=4)
        lk, plk = oracle.octree_key(2, k=k4, lev=4, maxd=4), oracle.octree_key(2, k=k4, lev=3, maxd=4)
        assert oracle.octree_key(3, k=pk, lk=lk, lev=4, maxd=4) == k4
        assert oracle.octree_key(3, k=gpk, lk=plk, lev=3, maxd=4) == pk


def test_tables_against_reference(oracle):
    with open(os.path.join(HERE, "golden", "octree_tables.json")) as f:
        ref = json.load(f)
    tp, tc = oracle.octree_tables()
    assert np.array_equal(tp, np.array(ref["ParentLUT"]))
    rc = np.array(ref["ChildLUT"])
    diff = {tuple(p) for p in np.argwhere(rc != tc)}
    assert diff == {(0, 18), (0, 19), (0, 20), (0, 24), (0, 25), (0, 26)}
    bad = [18, 19, 20, 24, 25, 26]  # neighbours one cell in +x of child 0: local x bit must be 1
    assert (tc[0, bad] & 4).all() and not (rc[0, bad] & 4).any()
    assert (tp[:, 13] == 13).all() and (tc[:, 13] == np.arange(8)).all()
    assert tp.min() >= 0 and tp.max() <= 26 and tc.min() >= 0 and tc.max() <= 7


def source_coords(native_bve, seed, level):
    """sourceCoords (src/LpmPolyMesh2d.hpp:236-256): vertices, then leaf face centres."""
    m = native_bve.build_mesh(seed, level)
    return np.concatenate([m["vx"], m["fx"][m["fmask"] == 0]])


@pytest.fixture(scope="module")
def cube6(oracle):
    from lpmkokkos_gb300 import bve
    x = source_coords(bve, 1, 6)
    return x, oracle.octree(x, 4)


def test_kernel_test_properties(oracle, cube6):
    x, T = cube6
    depth = 4
    assert np.array_equal(T["box"], UNIT)  # tests/LpmOctreeKernelTests.cpp:52-60
    n = len(x)
    assert np.array_equal(np.sort(T["orig_ids"]), np.arange(n))
    assert np.array_equal(T["sorted_pts"], x[T["orig_ids"]])
    b, nl = T["base_address"][depth], T["nnodes_per_level"][depth]
    leaf_keys = T["keys"][b + T["pt_in_leaf"]]
    assert (np.diff(leaf_keys.astype(np.int64)) >= 0).all()
    for i in range(0, n, 37):  # each point inside its key's box (encode test)
        box = oracle.octree_box(int(leaf_keys[i]), T["box"], depth, depth)
        p = T["sorted_pts"][i]
        assert box[0] <= p[0] <= box[1] and box[2] <= p[1] <= box[3] and box[4] <= p[2] <= box[5]
        assert oracle.octree_key(0, x=p, box=T["box"], lev=depth) == leaf_keys[i]
    cnt = T["pt_inds"][b:b + nl, 1]
    assert cnt.sum() == n
    st = T["pt_inds"][b:b + nl, 0]
    for t in np.nonzero(cnt)[0]:  # points inside their leaf's box, contiguous
        assert (T["pt_in_leaf"][st[t]:st[t] + cnt[t]] == t).all()
    assert (st[cnt == 0] == -1).all()


def _check_structure(T, depth, n):
    base, npl = T["base_address"], T["nnodes_per_level"]
    assert npl[0] == 1 and T["keys"][0] == 0 and T["parents"][0] == -1
    assert T["pt_inds"][0, 0] == 0 and T["pt_inds"][0, 1] == n
    for lev in range(1, depth + 1):
        b, m = base[lev], npl[lev]
        assert m % 8 == 0 and T["pt_inds"][b:b + m, 1].sum() == n
        keys = T["keys"][b:b + m].astype(np.int64)
        assert (np.diff(keys) > 0).all()  # unique, sorted
        par = T["parents"][b:b + m]
        assert (par >= 0).all() and (par < npl[lev - 1]).all()
        assert (par.reshape(-1, 8) == par[::8, None]).all()  # full sibling sets
        shift = 3 * (depth - lev + 1)
        pkeys = T["keys"][base[lev - 1] + par].astype(np.int64)
        assert np.array_equal(keys >> shift, pkeys >> shift)
    for lev in range(depth):
        b, m = base[lev], npl[lev]
        kids = T["kids"][b:b + m]
        cnt = T["pt_inds"][b:b + m, 1]
        for t in range(m):
            if cnt[t] == 0:
                assert (kids[t] == -1).all()
                continue
            k = kids[t]
            assert np.array_equal(k, k[0] + np.arange(8))
            assert (T["parents"][base[lev + 1] + k] == t).all()
            assert T["pt_inds"][base[lev + 1] + k, 1].sum() == cnt[t]
    assert (T["kids"][base[depth]:] == -1).all()


def _check_neighbors(oracle, T, depth):
    """Neighbour j of node t is the node whose box is t's box shifted by (a-1, b-1, c-1) edge
    lengths, j = 9a + 3b + c, when that node exists at t's level; -1 otherwise."""
    base, npl = T["base_address"], T["nnodes_per_level"]
    assert T["neighbors"][0, 13] == 0 and (np.delete(T["neighbors"][0], 13) == -1).all()
    for lev in range(1, depth + 1):
        b, m = base[lev], npl[lev]
        keys = T["keys"][b:b + m].astype(np.int64)
        index = {int(k): i for i, k in enumerate(keys)}
        shift = 3 * (depth - lev)
        cells = keys >> shift
        side = 1 << lev
        ijk = np.zeros((m, 3), dtype=np.int64)
        for bit in range(lev):  # de-interleave x y z from the cell key
            tri = (cells >> (3 * bit)) & 7
            ijk[:, 0] |= ((tri >> 2) & 1) << bit
            ijk[:, 1] |= ((tri >> 1) & 1) << bit
            ijk[:, 2] |= (tri & 1) << bit
        for j in range(27):
            off = np.array([j // 9 - 1, (j // 3) % 3 - 1, j % 3 - 1])
            q = ijk + off
            inside = ((q >= 0) & (q < side)).all(1)
            want = np.full(m, -1)
            for t in np.nonzero(inside)[0]:
                key = 0
                for bit in range(lev):
                    key |= (((q[t, 0] >> bit) & 1) << 2 | ((q[t, 1] >> bit) & 1) << 1 | ((q[t, 2] >> bit) & 1)) \
                        << (3 * bit)
                want[t] = index.get(int(key) << shift, -1)
            assert np.array_equal(T["neighbors"][b:b + m, j], want), (lev, j)


def test_tree_structure_and_neighbors(oracle, cube6):
    x, T = cube6
    _check_structure(T, 4, len(x))
    _check_neighbors(oracle, T, 4)


@pytest.mark.parametrize("depth", [1, 2, 5])
def test_other_depths_and_icosahedral_points(oracle, depth):
    """Depth 1 (root built from the leaves), a shallow and a deep tree, on the icosahedral leaf
    centres alone: their bounding box is not a cube, so box2cube applies to the keys."""
    from lpmkokkos_gb300 import bve
    m = bve.build_mesh(0, 4)
    x = m["fx"][m["fmask"] == 0]
    T = oracle.octree(x, depth)
    ext = T["box"][1::2] - T["box"][0::2]
    assert ext.max() / ext.min() - 1 > 1e-14
    _check_structure(T, depth, len(x))
    _check_neighbors(oracle, T, depth)


def test_invalid_depth(oracle):
    with pytest.raises(ValueError):
        oracle.octree(np.zeros((4, 3)), 0)
    with pytest.raises(ValueError):
        oracle.octree(np.zeros((4, 3)), 11)
