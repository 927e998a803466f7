"""Host-side parts of the product checked on CPU: mesh builder, initial conditions, and the
C ABI library's exported symbols (no compute call needs a GPU here)."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("seed", [0, 1])
@pytest.mark.parametrize("level", [0, 1, 2, 3, 4, 5])
def test_product_mesh_equals_oracle_bitwise(native, oracle, seed, level):
    from lpmkokkos_gb300 import bve
    a = bve.build_mesh(seed, level)
    b = oracle.mesh(seed, level)
    assert (a["nverts"], a["nfaces"], a["nleaves"]) == (b["nverts"], b["nfaces"], b["nleaves"])
    for k in ("vx", "fx", "farea", "fmask"):
        assert np.array_equal(a[k], b[k]), k


def test_mesh_counts(native):
    from lpmkokkos_gb300 import bve
    # per-seed counts (n*AtTreeLevel, src/LpmMeshSeed.cpp:369-391): icos L4/L7/L8, cube L4/L7
    assert bve.mesh_counts(0, 4) == (2562, 6820, 5120)
    assert bve.mesh_counts(0, 7) == (163842, 436900, 327680)
    assert bve.mesh_counts(0, 8) == (655362, 1747620, 1310720)
    assert bve.mesh_counts(1, 4) == (1538, 2046, 1536)
    assert bve.mesh_counts(1, 7) == (98306, 131070, 98304)


def test_initial_conditions_equal_oracle(native, oracle):
    from lpmkokkos_gb300 import bve
    m = oracle.mesh(0, 4)
    for x in (m["vx"], m["fx"]):
        assert np.array_equal(bve.ic_rh54(x), oracle.ic_rh54(x))
        assert np.array_equal(bve.rh54_velocity(x), oracle.rh54_velocity(x))
        assert np.array_equal(bve.ic_solid_body(x), oracle.ic_solid_body(x))
    c, a = bve.gaussian_params(20261204, 8)
    c2, a2 = oracle.gaussian_params(20261204, 8)
    assert np.array_equal(c, c2) and np.array_equal(a, a2)
    assert np.allclose(np.linalg.norm(c, axis=1), 1.0, atol=1e-15)
    assert np.all((a >= -2) & (a < 2))
    z = bve.ic_gaussians_add(m["fx"], bve.ic_rh54(m["fx"]), c, a, 0.1)
    assert np.array_equal(z, oracle.rh54_gaussians(m["fx"], 20261204, 8, 0.1))


def test_invalid_host_arguments(native):
    from lpmkokkos_gb300 import _lib as L
    lib = L.lib()
    assert lib.lpm_mesh_build(7, 2, None, None, None, None) == L.LPM_ERR_INVALID_ARGUMENT
    assert lib.lpm_mesh_build(0, -1, None, None, None, None) == L.LPM_ERR_INVALID_ARGUMENT
    assert lib.lpm_ic_gaussians_add(None, 4, None, None, 0, 0.1, None) == L.LPM_ERR_INVALID_ARGUMENT
    assert lib.lpm_bve_ctx_destroy(None) == L.LPM_ERR_INVALID_ARGUMENT
    assert lib.lpm_bve_velocity(None, None, None, None, 0, 0, None, 0, 0.0, None) == L.LPM_ERR_INVALID_ARGUMENT


def _declared_functions():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in sorted(os.listdir(inc)):
        if not f.endswith(".h"):
            continue
        text = open(os.path.join(inc, f)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_\s\*]*?\b(lpm_[a-z0-9_]+)\s*\(", text, re.M):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol(native):
    names = _declared_functions()
    assert {"lpm_bve_velocity", "lpm_bve_rk4_step", "lpm_bve_ctx_create", "lpm_bve_last_error",
            "lpm_bve_ensemble_create", "lpm_mesh_build"} <= names
    lib = ctypes.CDLL(native._name)
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_status_codes_match_header():
    """Every LPM_OK / LPM_ERR_* status of include/lpm_bve.h has the same value in the bindings."""
    from lpmkokkos_gb300 import _lib as L
    with open(os.path.join(ROOT, "include", "lpm_bve.h")) as f:
        codes = {m.group(1): int(m.group(2))
                 for m in re.finditer(r"#define\s+(LPM_(?:OK|ERR_\w+))\s+\(?(-?\d+)\)?", f.read())}
    assert "LPM_ERR_INTERNAL" in codes and len(codes) >= 9
    assert {k: getattr(L, k, None) for k in codes} == codes
    assert len(set(codes.values())) == len(codes)


def test_no_cpu_fallback_without_library(tmp_path, monkeypatch):
    """The product refuses to run if the native library is missing."""
    from lpmkokkos_gb300 import _build, _lib
    monkeypatch.setattr(_build, "LIB", str(tmp_path / "missing.so"))
    monkeypatch.setattr(_lib, "_lib", None)
    with pytest.raises(RuntimeError):
        _lib.lib()


def test_server_footprint_estimate(native):
    """The server's admission figure (host-only): grows ~4x per level, FP64 stores one packed
    source record instead of two, invalid requests are rejected."""
    from lpmkokkos_gb300 import _lib as L
    from lpmkokkos_gb300 import bve
    est = [bve.server_estimate(0, lv) for lv in range(4, 9)]
    ratios = [b / a for a, b in zip(est, est[1:])]
    assert all(3.5 < r < 4.5 for r in ratios), ratios
    nv, nf, nl = bve.mesh_counts(0, 7)
    state = 8 * (7 * nv + 8 * nf) + nf
    assert state < est[3] < 16 * state  # plan: chunk partials and RK4 increments per target slot
    assert bve.server_estimate(0, 7, flags=L.FP64) < est[3]
    with pytest.raises(L.LpmError):
        bve.server_estimate(0, 11)


def test_server_create_fails_cleanly_without_gpu(native):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from lpmkokkos_gb300 import _lib as L
    lib = L.lib()
    h = ctypes.c_void_p()
    opts = L.ServerOpts(0, 0, 0, L.FP32C, 0.0)
    assert lib.lpm_bve_server_create(ctypes.byref(opts), ctypes.byref(h)) != L.LPM_OK
    assert not h.value


def _lhuilier(a, b, c):
    def arc(p, q):
        return np.arctan2(np.linalg.norm(np.cross(p, q), axis=-1), np.sum(p * q, axis=-1))
    s1, s2, s3 = arc(a, b), arc(b, c), arc(c, a)
    h = 0.5 * (s1 + s2 + s3)
    t = np.tan(0.5 * h) * np.tan(0.5 * (h - s1)) * np.tan(0.5 * (h - s2)) * np.tan(0.5 * (h - s3))
    return 4 * np.arctan(np.sqrt(t))


@pytest.mark.parametrize("seed", [0, 1])
def test_face_connectivity_reproduces_areas(native, seed):
    """lpm_mesh_face_verts: every leaf face's area equals the spherical polygon area of its
    vertices fanned from the face centre (the reference's Faces area rule), to 1e-12 relative."""
    from lpmkokkos_gb300 import bve
    m = bve.build_mesh(seed, 3)
    fv = bve.mesh_face_verts(seed, 3)
    assert fv.shape == (m["nfaces"], 3 if seed == 0 else 4)
    assert fv.min() >= 0 and fv.max() < m["nverts"]
    v, c = m["vx"][fv], m["fx"]
    n = fv.shape[1]
    area = sum(_lhuilier(c, v[:, k], v[:, (k + 1) % n]) for k in range(n))
    leaf = m["fmask"] == 0  # a divided parent passes its area to its children (area 0)
    assert np.abs(area[leaf] - m["farea"][leaf]).max() <= 1e-12 * m["farea"].max()
    assert (m["farea"][~leaf] == 0).all()


def test_octree_and_tree_code_argument_checks(native):
    """The octree and tree-code entry points reject bad arguments before touching the device."""
    from lpmkokkos_gb300 import _lib as L
    lib = L.lib()
    h = ctypes.c_void_p()
    x = (ctypes.c_double * 12)()
    ptr = ctypes.cast(x, ctypes.c_void_p).value
    for args in ((None, 3, 1, 4, 3), (ptr, 3, 1, 0, 3), (ptr, 3, 1, 4, 0), (ptr, 3, 1, 4, 11), (ptr, -3, 1, 4, 3)):
        xp, si, sc, n, d = args
        assert lib.lpm_octree_build(xp, si, sc, n, d, 1, ctypes.byref(h), None) == L.LPM_ERR_INVALID_ARGUMENT
        assert not h.value
    assert lib.lpm_octree_build(ptr, 3, 1, 4, 3, 1, None, None) == L.LPM_ERR_INVALID_ARGUMENT
    assert lib.lpm_octree_info(None, None, None, None, None, None, None) == L.LPM_ERR_INVALID_ARGUMENT
    assert lib.lpm_octree_arrays(None, *([None] * 8)) == L.LPM_ERR_INVALID_ARGUMENT
    assert lib.lpm_octree_destroy(None) == L.LPM_ERR_INVALID_ARGUMENT
    assert lib.lpm_bve_ctx_set_treecode(None, 8, 0.6, 512, 0.0) == L.LPM_ERR_INVALID_ARGUMENT
    assert lib.lpm_bve_ctx_tree_stats(None, None, None, None, None, None, None, None) == L.LPM_ERR_INVALID_ARGUMENT
    assert lib.lpm_sphere_tangency(ptr, 3, 1, ptr, 3, 1, -1, ptr, None) == L.LPM_ERR_INVALID_ARGUMENT


@pytest.mark.parametrize("level", [2, 4, 7, 8])
def test_bench_work_units_match_the_mesh(native, level):
    """The benchmark's work units: its closed-form mesh sizes equal the library's counts, the
    algorithmic pairs per evaluation are (vertices + leaves) x leaves (3.933e7 at icosahedral
    level 4, 1.611e11 at 7, 2.577e12 at 8), and the computed pairs add the masked-parent targets."""
    import bench
    from lpmkokkos_gb300 import bve
    nv, nall, nl = bench.mesh_sizes(level)
    assert (nv, nall, nl) == bve.mesh_counts(0, level)
    alg = (nv + nl) * nl
    quoted = {4: 3.933e7, 7: 1.611e11, 8: 2.577e12}
    if level in quoted:
        assert alg == pytest.approx(quoted[level], rel=5e-4)
    assert bench.computed_pairs(0, level) == (nv + nall) * nl
    cnv, cnall, cnl = bve.mesh_counts(1, level)
    assert bench.computed_pairs(1, level) == (cnv + cnall) * cnl
