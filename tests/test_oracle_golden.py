"""The CPU oracle against the reference's own known answers (no GPU).

Pins the restatement before it is trusted as the oracle:
  * the recorded spherical-Poisson psi linf table, icosahedral and cubed sphere, levels 0-5
    (scripts/poissonOutput.py:6-30; the reference ran the same kernels on CPU and GPU and
    printed identical numbers) -- to the printed 6 significant digits;
  * geometry asserts of tests/LpmGeometryUnitTests.cpp:146-165;
  * mesh sizes (src/LpmMeshSeed.cpp:297-305, :369-391) and the 4 pi surface area
    (tests/LpmFacesUnitTests.cpp:95,132);
  * RH54 known answer psi = f/30 and u = RH54Velocity converge under refinement
    (src/LpmSpherePoisson.hpp:70-79);
  * solid-body rotation u = Omega (-y, x, 0) (tests/LpmBVETest.cpp:180-219);
  * exact small-integer reductions, the property tests/LpmKernelTest.cpp:85-103 asserts.
"""
import math

import numpy as np
import pytest

# scripts/poissonOutput.py:6-30 -- (mesh size deg, linf psi verts, linf psi faces)
POISSON_TABLE = {
    (0, 0): (45.4164, 2.42561, 1.49743), (1, 0): (82.9186, 0.2566, 0.0),
    (0, 1): (22.7082, 0.175552, 0.446258), (1, 1): (41.4593, 0.898719, 0.466355),
    (0, 2): (11.3541, 0.0327947, 0.18008), (1, 2): (20.7296, 0.105744, 0.330876),
    (0, 3): (5.67705, 0.0078577, 0.057519), (1, 3): (10.3648, 0.0242884, 0.153158),
    (0, 4): (2.83852, 0.00199034, 0.0170644), (1, 4): (5.18241, 0.00611779, 0.0500934),
    (0, 5): (1.41926, 0.000499979, 0.00492556), (1, 5): (2.59121, 0.00152096, 0.0148438),
}


def _six_digits(x, ref):
    return abs(x - ref) <= 5e-6 * abs(ref) + 1e-15


@pytest.mark.parametrize("kind,level", sorted(POISSON_TABLE))
def test_poisson_table(oracle, kind, level):
    deg, lv, lf = POISSON_TABLE[(kind, level)]
    got = oracle.poisson(kind, level)
    assert _six_digits(got[0], deg), got
    assert _six_digits(got[1], lv), got
    assert _six_digits(got[2], lf), got


def test_geometry_asserts(oracle):
    G = oracle.geometry()
    s = 0.57735026918962584
    p0 = [s, -s, s]; p1 = [s, -s, -s]; p2 = [s, s, -s]; p3 = [s, s, s]
    assert abs(G.tri_area(p0, p1, p2) - math.pi / 3) <= 1e-14
    mid = G.midpoint(p0, p1)
    assert abs(mid[0] - 0.5 * math.sqrt(2.0)) <= 1e-14
    c = G.cross(p0, p1)
    assert abs(c[0] - 2 / 3) <= 1e-14 and abs(c[1] - 2 / 3) <= 1e-14 and abs(c[2]) <= 1e-14
    bc = G.barycenter([p0, p1, p2, p3])
    assert bc[0] == 1 and bc[1] == 0 and bc[2] == 0
    assert abs(G.polygon_area(bc, [p0, p1, p2, p3]) - 2 * math.pi / 3) <= 1e-14


@pytest.mark.parametrize("kind", [0, 1])
def test_mesh_sizes_and_area(oracle, kind):
    for level in range(0, 6):
        m = oracle.mesh(kind, level)
        if kind == 0:
            nv, nl, nall = 2 + 10 * 4 ** level, 20 * 4 ** level, 20 * (4 ** (level + 1) - 1) // 3
        else:
            nv, nl, nall = 2 + 6 * 4 ** level, 6 * 4 ** level, 2 * (4 ** (level + 1) - 1)
        assert (m["nverts"], m["nleaves"], m["nfaces"]) == (nv, nl, nall)
        assert abs(m["farea"].sum() - 4 * math.pi) <= 1e-12
        assert np.all(m["farea"][m["fmask"] == 1] == 0.0)
        assert np.allclose(np.linalg.norm(m["vx"], axis=1), 1.0, atol=1e-15)
        assert np.allclose(np.linalg.norm(m["fx"], axis=1), 1.0, atol=1e-15)


def test_rh54_known_answer_converges(oracle):
    """Velocity error against RH54Velocity shrinks under refinement."""
    errs = []
    for level in (2, 3, 4):
        m = oracle.mesh(0, level)
        zf = oracle.ic_rh54(m["fx"])
        uv, uf = oracle.velocity(m["vx"], m["fx"], zf, m["farea"], m["fmask"])
        leaf = m["fmask"] == 0
        ex = oracle.rh54_velocity(m["fx"][leaf])
        errs.append(np.abs(uf[leaf] - ex).max() / np.abs(ex).max())
    assert errs[0] > errs[1] > errs[2]
    assert errs[1] / errs[2] > 1.5  # linf converges at ~first order (cf. the Poisson u errors)


def test_solid_body_rotation(oracle):
    omega = 2 * math.pi
    m = oracle.mesh(1, 3)
    zf = oracle.ic_solid_body(m["fx"])
    assert np.allclose(zf, 2 * omega * m["fx"][:, 2])
    uv, uf = oracle.velocity(m["vx"], m["fx"], zf, m["farea"], m["fmask"])
    leaf = m["fmask"] == 0
    x = m["fx"][leaf]
    ex = np.stack([-omega * x[:, 1], omega * x[:, 0], 0 * x[:, 0]], axis=1)
    n = oracle.errnorms_vec(uf[leaf], ex, m["farea"][leaf])
    assert n["l2"] < 0.05 and n["l1"] < 0.05


def test_integer_reduction_is_exact(oracle):
    """Sums of exactly representable terms are exact regardless of order (the property the
    reference's Tuple reduction test asserts)."""
    tx = np.array([[0.0, 0.0, 1.0]])
    sx = np.array([[1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [-1.0, 0.0, 0.0], [0.0, -1.0, 0.0]])
    zeta = np.array([1.0, 2.0, 4.0, 8.0])
    area = np.full(4, 4 * math.pi)       # strength = -zeta*A/(4 pi (1 - 0)) = -zeta, exactly
    u = oracle.velocity_distinct(tx, sx, zeta, area, np.zeros(4, np.uint8))
    # cross(z, x) = y, cross(z, y) = -x, cross(z, -x) = -y, cross(z, -y) = x
    want = np.array([[2.0 - 8.0, -1.0 + 4.0, 0.0]])
    assert np.array_equal(u, want)


def test_rk4_quirk_only_changes_face_vorticity(oracle):
    m = oracle.mesh(0, 2)
    zf = oracle.rh54_gaussians(m["fx"], 7, 2)
    zv = oracle.rh54_gaussians(m["vx"], 7, 2)
    uv, uf = oracle.velocity(m["vx"], m["fx"], zf, m["farea"], m["fmask"])
    a = oracle.rk4(m["vx"], zv, uv, m["fx"], zf, uf, m["farea"], m["fmask"], 0.01, 2 * math.pi, 1, quirk=True)
    b = oracle.rk4(m["vx"], zv, uv, m["fx"], zf, uf, m["farea"], m["fmask"], 0.01, 2 * math.pi, 1, quirk=False)
    same = lambda x, y: np.array_equal(x, y, equal_nan=True)  # noqa: E731 (masked parents may be inf/nan)
    assert same(a[0], b[0]) and same(a[1], b[1]) and same(a[3], b[3])
    assert not same(a[4], b[4])
    # one step later the changed face vorticity moves everything else too
    a2 = oracle.rk4(*a, m["farea"], m["fmask"], 0.01, 2 * math.pi, 1, quirk=True)
    b2 = oracle.rk4(*b, m["farea"], m["fmask"], 0.01, 2 * math.pi, 1, quirk=False)
    assert not same(a2[0], b2[0])


def test_rk4_conserves_absolute_vorticity_along_paths(oracle):
    """Dzeta/Dt = -2 Omega dz/dt: zeta + 2 Omega z is (nearly) conserved at vertices."""
    omega = 2 * math.pi
    m = oracle.mesh(0, 3)
    zf = oracle.rh54_gaussians(m["fx"], 9, 2)
    zv = oracle.rh54_gaussians(m["vx"], 9, 2)
    uv, uf = oracle.velocity(m["vx"], m["fx"], zf, m["farea"], m["fmask"])
    a0 = zv + 2 * omega * m["vx"][:, 2]
    out = oracle.rk4(m["vx"], zv, uv, m["fx"], zf, uf, m["farea"], m["fmask"], 0.01, omega, 3)
    a1 = out[1] + 2 * omega * out[0][:, 2]
    assert np.abs(a1 - a0).max() < 1e-6 * np.abs(a0).max()
