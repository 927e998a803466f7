"""ctypes wrapper of the CPU oracle (TEST INFRASTRUCTURE ONLY).

The oracle is a C++/OpenMP restatement of the reference's BVE path
(pbosler/lpmKokkos: src/LpmBVEKernels.hpp, src/LpmBVERK4_Impl.hpp, src/LpmFaces.cpp,
src/LpmSpherePoisson.hpp, ...).  Only tests/, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` may import this module; the product path never does.

Parity of the oracle itself is pinned against the reference's recorded spherical
Poisson psi-error table (scripts/poissonOutput.py:6-30) and the analytic known
answers its tests use.  All arrays are float64, row-major (n, 3) for vectors.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liblpm_oracle.so")
_lib = None

ICOS, CUBE = 0, 1


class _Mesh(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int), ("level", ctypes.c_int),
        ("nverts", ctypes.c_int), ("nfaces", ctypes.c_int), ("nleaves", ctypes.c_int),
        ("nedges", ctypes.c_int), ("nfv", ctypes.c_int),
        ("vx", ctypes.POINTER(ctypes.c_double)), ("fx", ctypes.POINTER(ctypes.c_double)),
        ("farea", ctypes.POINTER(ctypes.c_double)), ("fmask", ctypes.POINTER(ctypes.c_ubyte)),
        ("flevel", ctypes.POINTER(ctypes.c_int)), ("fverts", ctypes.POINTER(ctypes.c_int)),
    ]


def build(quiet: bool = True) -> str:
    """Compile the oracle with its Makefile (g++ -fopenmp); returns the library path."""
    cmd = ["make", "-C", _HERE]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + res.stdout + res.stderr)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        _lib = ctypes.CDLL(_LIB_PATH)
        _setup(_lib)
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) if a is not None else None


def _up(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte))


def _setup(L):
    D = ctypes.POINTER(ctypes.c_double)
    U = ctypes.POINTER(ctypes.c_ubyte)
    L.oracle_mesh_build.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(_Mesh)]
    L.oracle_mesh_build.restype = ctypes.c_int
    L.oracle_mesh_free.argtypes = [ctypes.POINTER(_Mesh)]
    L.oracle_bve_velocity.argtypes = [D, ctypes.c_long, D, D, D, U, ctypes.c_long, ctypes.c_double, D, D, D, D]
    L.oracle_velocity_distinct.argtypes = [D, ctypes.c_long, D, D, D, U, ctypes.c_long, ctypes.c_double, D, D]
    L.oracle_velocity_faces.argtypes = [ctypes.POINTER(ctypes.c_long), ctypes.c_long, D, D, D, U, ctypes.c_long,
                                         ctypes.c_double, D, D]
    L.oracle_bve_rk4.argtypes = [D, D, D, ctypes.c_long, D, D, D, D, U, ctypes.c_long,
                                 ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                 ctypes.c_double]
    for name in ("oracle_ic_rh54", "oracle_rh54_velocity", "oracle_ic_solid_body"):
        getattr(L, name).argtypes = [D, ctypes.c_long, D]
    L.oracle_ic_gaussians_add.argtypes = [D, ctypes.c_long, D, D, ctypes.c_int, ctypes.c_double, D]
    L.oracle_gaussian_params.argtypes = [ctypes.c_ulonglong, ctypes.c_int, ctypes.c_double, ctypes.c_double, D, D]
    L.oracle_errnorms_vec.argtypes = [D, D, D, ctypes.c_long, D]
    L.oracle_errnorms_scalar.argtypes = [D, D, D, ctypes.c_long, D]
    L.oracle_tangency.argtypes = [D, D, ctypes.c_long, D]
    IP = ctypes.POINTER(ctypes.c_int)
    L.oracle_octree_counts.argtypes = [D, ctypes.c_long, ctypes.c_int, IP]
    L.oracle_octree_counts.restype = ctypes.c_long
    L.oracle_octree_build.argtypes = [D, ctypes.c_long, ctypes.c_int, D, IP, IP, ctypes.c_void_p, IP, IP, IP, IP, D,
                                      IP, IP]
    L.oracle_octree_tables.argtypes = [IP, IP]
    L.oracle_octree_key.argtypes = [ctypes.c_int, D, D, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int, ctypes.c_int]
    L.oracle_octree_key.restype = ctypes.c_uint64
    L.oracle_octree_box.argtypes = [ctypes.c_uint64, D, ctypes.c_int, ctypes.c_int, D]
    L.oracle_poisson.argtypes = [ctypes.c_int, ctypes.c_int, D]
    L.oracle_poisson.restype = ctypes.c_int
    L.oracle_tri_area.argtypes = [D, D, D]
    L.oracle_tri_area.restype = ctypes.c_double
    L.oracle_midpoint.argtypes = [D, D, D]
    L.oracle_barycenter.argtypes = [D, ctypes.c_int, D]
    L.oracle_polygon_area.argtypes = [D, D, ctypes.c_int]
    L.oracle_polygon_area.restype = ctypes.c_double
    L.oracle_cross.argtypes = [D, D, D]


def mesh(kind: int, level: int) -> dict:
    """Uniformly refined mesh (PolyMesh2d::treeInit) as numpy arrays."""
    m = _Mesh()
    rc = lib().oracle_mesh_build(kind, level, ctypes.byref(m))
    if rc != 0:
        raise RuntimeError(f"oracle_mesh_build failed ({rc})")
    try:
        nv, nf = m.nverts, m.nfaces
        out = dict(
            kind=kind, level=level, nverts=nv, nfaces=nf, nleaves=m.nleaves, nedges=m.nedges, nfv=m.nfv,
            vx=np.ctypeslib.as_array(m.vx, shape=(nv, 3)).copy(),
            fx=np.ctypeslib.as_array(m.fx, shape=(nf, 3)).copy(),
            farea=np.ctypeslib.as_array(m.farea, shape=(nf,)).copy(),
            fmask=np.ctypeslib.as_array(m.fmask, shape=(nf,)).copy(),
            flevel=np.ctypeslib.as_array(m.flevel, shape=(nf,)).copy(),
            fverts=np.ctypeslib.as_array(m.fverts, shape=(nf, m.nfv)).copy(),
        )
    finally:
        lib().oracle_mesh_free(ctypes.byref(m))
    return out


def velocity(vx, fx, zeta, area, mask, eps=0.0, psi=False):
    """Velocity (and optionally stream function) at vertices and all faces."""
    vx = np.ascontiguousarray(vx, dtype=np.float64)
    fx = np.ascontiguousarray(fx, dtype=np.float64)
    zeta = np.ascontiguousarray(zeta, dtype=np.float64)
    area = np.ascontiguousarray(area, dtype=np.float64)
    mask = np.ascontiguousarray(mask, dtype=np.uint8)
    nv, nf = vx.shape[0], fx.shape[0]
    vu = np.zeros((nv, 3)); fu = np.zeros((nf, 3))
    vp = np.zeros(nv) if psi else None
    fp = np.zeros(nf) if psi else None
    lib().oracle_bve_velocity(_dp(vx), nv, _dp(fx), _dp(zeta), _dp(area), _up(mask), nf, float(eps),
                              _dp(vu), _dp(fu), _dp(vp), _dp(fp))
    return (vu, fu, vp, fp) if psi else (vu, fu)


def velocity_distinct(tx, sx, zeta, area, mask, eps=0.0, psi=False):
    tx = np.ascontiguousarray(tx, dtype=np.float64)
    sx = np.ascontiguousarray(sx, dtype=np.float64)
    zeta = np.ascontiguousarray(zeta, dtype=np.float64)
    area = np.ascontiguousarray(area, dtype=np.float64)
    mask = np.ascontiguousarray(mask, dtype=np.uint8)
    u = np.zeros((tx.shape[0], 3))
    p = np.zeros(tx.shape[0]) if psi else None
    lib().oracle_velocity_distinct(_dp(tx), tx.shape[0], _dp(sx), _dp(zeta), _dp(area), _up(mask), sx.shape[0],
                                   float(eps), _dp(u), _dp(p))
    return (u, p) if psi else u


def velocity_faces(idx, fx, zeta, area, mask, eps=0.0, psi=False):
    """Collocated velocity (and stream function) at the listed faces only: face k sums every
    unmasked face j != k (BVEFaceVelocity / BVEFaceStreamFn restricted to a target subset)."""
    idx = np.ascontiguousarray(idx, dtype=np.int64)
    fx = np.ascontiguousarray(fx, dtype=np.float64)
    zeta = np.ascontiguousarray(zeta, dtype=np.float64)
    area = np.ascontiguousarray(area, dtype=np.float64)
    mask = np.ascontiguousarray(mask, dtype=np.uint8)
    assert idx.size == 0 or (idx.min() >= 0 and idx.max() < fx.shape[0])
    u = np.zeros((idx.size, 3))
    p = np.zeros(idx.size) if psi else None
    lib().oracle_velocity_faces(idx.ctypes.data_as(ctypes.POINTER(ctypes.c_long)), idx.size, _dp(fx), _dp(zeta),
                                _dp(area), _up(mask), fx.shape[0], float(eps), _dp(u), _dp(p))
    return (u, p) if psi else u


def rk4(vx, vzeta, vvel, fx, fzeta, fvel, farea, fmask, dt, Omega, nsteps, quirk=True, renorm=False, eps=0.0):
    """Advance nsteps in place-free fashion; returns new (vx, vzeta, vvel, fx, fzeta, fvel)."""
    arrs = [np.array(a, dtype=np.float64, copy=True, order="C") for a in (vx, vzeta, vvel, fx, fzeta, fvel)]
    farea = np.ascontiguousarray(farea, dtype=np.float64)
    fmask = np.ascontiguousarray(fmask, dtype=np.uint8)
    vx_, vz_, vv_, fx_, fz_, fv_ = arrs
    lib().oracle_bve_rk4(_dp(vx_), _dp(vz_), _dp(vv_), vx_.shape[0], _dp(fx_), _dp(fz_), _dp(fv_),
                         _dp(farea), _up(fmask), fx_.shape[0], float(dt), float(Omega), int(nsteps),
                         int(bool(quirk)), int(bool(renorm)), float(eps))
    return vx_, vz_, vv_, fx_, fz_, fv_


def _map(fn, x, width):
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.zeros((x.shape[0], width)) if width > 1 else np.zeros(x.shape[0])
    fn(_dp(x), x.shape[0], _dp(out))
    return out


def ic_rh54(x):
    return _map(lib().oracle_ic_rh54, x, 1)


def rh54_velocity(x):
    return _map(lib().oracle_rh54_velocity, x, 3)


def ic_solid_body(x):
    return _map(lib().oracle_ic_solid_body, x, 1)


def ic_gaussians_add(x, zeta, centers, amps, width):
    x = np.ascontiguousarray(x, dtype=np.float64)
    z = np.array(zeta, dtype=np.float64, copy=True)
    c = np.ascontiguousarray(centers, dtype=np.float64)
    a = np.ascontiguousarray(amps, dtype=np.float64)
    lib().oracle_ic_gaussians_add(_dp(x), x.shape[0], _dp(c), _dp(a), a.shape[0], float(width), _dp(z))
    return z


def gaussian_params(seed, ng, lo=-2.0, hi=2.0):
    c = np.zeros((ng, 3)); a = np.zeros(ng)
    lib().oracle_gaussian_params(int(seed), int(ng), float(lo), float(hi), _dp(c), _dp(a))
    return c, a


def rh54_gaussians(x, seed, ng, width=0.1):
    """RH54 relative vorticity plus ng seeded Gaussian vortices (the benchmark's initial data)."""
    z = ic_rh54(x)
    if ng > 0:
        c, a = gaussian_params(seed, ng)
        z = ic_gaussians_add(x, z, c, a, width)
    return z


def errnorms_vec(appx, exact, wt):
    appx = np.ascontiguousarray(appx, dtype=np.float64)
    exact = np.ascontiguousarray(exact, dtype=np.float64)
    wt = np.ascontiguousarray(wt, dtype=np.float64)
    out = np.zeros(3)
    lib().oracle_errnorms_vec(_dp(appx), _dp(exact), _dp(wt), appx.shape[0], _dp(out))
    return dict(l1=out[0], l2=out[1], linf=out[2])


def errnorms_scalar(appx, exact, wt):
    appx = np.ascontiguousarray(appx, dtype=np.float64)
    exact = np.ascontiguousarray(exact, dtype=np.float64)
    wt = np.ascontiguousarray(wt, dtype=np.float64)
    out = np.zeros(3)
    lib().oracle_errnorms_scalar(_dp(appx), _dp(exact), _dp(wt), appx.shape[0], _dp(out))
    return dict(l1=out[0], l2=out[1], linf=out[2])


def tangency(x, u):
    """u . x per point of row-major (n, 3) arrays."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    u = np.ascontiguousarray(u, dtype=np.float64)
    out = np.zeros(x.shape[0])
    lib().oracle_tangency(_dp(x), _dp(u), x.shape[0], _dp(out))
    return out


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def octree(x, depth):
    """The Morton octree of src/LpmOctree.cpp over row-major (n, 3) points: box (6,),
    base_address / nnodes_per_level (depth + 1), keys (uint32), pt_inds (nn, 2), parents,
    kids (nn, 8), neighbors (nn, 27) -- level-local indices or -1 -- sorted_pts (n, 3), orig_ids,
    pt_in_leaf."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    n = x.shape[0]
    npl = np.zeros(depth + 1, dtype=np.int32)
    nn = lib().oracle_octree_counts(_dp(x), n, depth, _ip(npl))
    if nn < 0:
        raise ValueError("invalid octree depth or empty point set")
    out = dict(box=np.zeros(6), base_address=np.zeros(depth + 1, dtype=np.int32), nnodes_per_level=npl,
               keys=np.zeros(nn, dtype=np.uint32), pt_inds=np.zeros((nn, 2), dtype=np.int32),
               parents=np.zeros(nn, dtype=np.int32), kids=np.zeros((nn, 8), dtype=np.int32),
               neighbors=np.zeros((nn, 27), dtype=np.int32), sorted_pts=np.zeros((n, 3)),
               orig_ids=np.zeros(n, dtype=np.int32), pt_in_leaf=np.zeros(n, dtype=np.int32))
    rc = lib().oracle_octree_build(_dp(x), n, depth, _dp(out["box"]), _ip(out["base_address"]), _ip(npl),
                                   out["keys"].ctypes.data, _ip(out["pt_inds"]), _ip(out["parents"]),
                                   _ip(out["kids"]), _ip(out["neighbors"]), _dp(out["sorted_pts"]),
                                   _ip(out["orig_ids"]), _ip(out["pt_in_leaf"]))
    assert rc == 0
    return out


def octree_tables():
    """(ParentLUT, ChildLUT) as (8, 27) int arrays, generated from their geometric definition."""
    tp = np.zeros((8, 27), dtype=np.int32)
    tc = np.zeros((8, 27), dtype=np.int32)
    lib().oracle_octree_tables(_ip(tp), _ip(tc))
    return tp, tc


def octree_key(op, x=None, box=None, k=0, lk=0, lev=1, maxd=1):
    """Key algebra: op 0 compute_key_for_point(x, lev, box), 1 parent_key(k, lev, maxd),
    2 local_key(k, lev, maxd), 3 node_key(k, lk, lev, maxd)."""
    xx = np.ascontiguousarray(x if x is not None else np.zeros(3), dtype=np.float64)
    bb = np.ascontiguousarray(box if box is not None else np.zeros(6), dtype=np.float64)
    return int(lib().oracle_octree_key(op, _dp(xx), _dp(bb), k, lk, lev, maxd))


def octree_box(k, rbox, lev, maxd):
    """box_from_key: (xmin, xmax, ymin, ymax, zmin, zmax)."""
    rb = np.ascontiguousarray(rbox, dtype=np.float64)
    out = np.zeros(6)
    lib().oracle_octree_box(k, _dp(rb), lev, maxd, _dp(out))
    return out


def poisson(kind, level):
    """SpherePoisson solve with RH54 forcing: (mesh deg, linf psi verts, faces, |u| verts, faces)."""
    out = np.zeros(5)
    rc = lib().oracle_poisson(kind, level, _dp(out))
    if rc != 0:
        raise RuntimeError("oracle_poisson failed")
    return tuple(float(v) for v in out)


def geometry():
    """Namespace of the oracle's geometry helpers (for the reference's geometry asserts)."""
    L = lib()

    def v(a):
        return np.ascontiguousarray(a, dtype=np.float64)

    class G:
        @staticmethod
        def tri_area(a, b, c):
            return L.oracle_tri_area(_dp(v(a)), _dp(v(b)), _dp(v(c)))

        @staticmethod
        def midpoint(a, b):
            o = np.zeros(3); L.oracle_midpoint(_dp(v(a)), _dp(v(b)), _dp(o)); return o

        @staticmethod
        def barycenter(pts):
            p = v(pts); o = np.zeros(3); L.oracle_barycenter(_dp(p), p.shape[0], _dp(o)); return o

        @staticmethod
        def polygon_area(ctr, pts):
            p = v(pts); return L.oracle_polygon_area(_dp(v(ctr)), _dp(p), p.shape[0])

        @staticmethod
        def cross(a, b):
            o = np.zeros(3); L.oracle_cross(_dp(v(a)), _dp(v(b)), _dp(o)); return o

    return G
