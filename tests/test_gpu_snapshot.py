"""Snapshots and VTK output (include/lpm_bve_snapshot.h).

  * write -> read restores every evolving array bit for bit, across Kokkos layouts;
  * a run restarted from a snapshot continues as the uninterrupted run does, to the rounding of
    the summation order: stepping on builds a new plan whose target/source order comes from the
    restored (advected) positions (FP32C: 1e-6 relative L2, the FP32C bar; FP64: 1e-13);
  * a finished server request's snapshot, restored and stepped on, matches the same request run
    for more steps in the server (FP64, host initial condition, 1e-13);
  * a snapshot of another mesh is refused;
  * the VTK file's sections have the sizes its header announces, and its points are the
    vertex positions (big-endian float64, as legacy VTK binary requires).
"""
import math

import numpy as np
import pytest
import torch

import lpmkokkos_gb300 as P
from lpmkokkos_gb300 import _lib as L
from lpmkokkos_gb300 import bve
from vtk_reader import read_vtk_sections

pytestmark = pytest.mark.gpu

OMEGA = 2 * math.pi
FIELDS = ("physVerts", "relVortVerts", "velocityVerts", "physFaces", "relVortFaces", "velocityFaces")


def _sphere(ctx, seed, level, prec, layout="left", rseed=9):
    s = bve.BVESphere(seed, level, layout=layout)
    s.init_vorticity(bve.rh54_gaussians(rseed, 3), ctx, flags=prec)
    torch.cuda.synchronize()
    return s


def _same(a, b):
    return bool(torch.equal(torch.isnan(a), torch.isnan(b))) and bool(torch.equal(torch.nan_to_num(a),
                                                                                  torch.nan_to_num(b)))


def test_round_trip_across_layouts(ctx, tmp_path):
    a = _sphere(ctx, 0, 3, P.FP64, layout="left")
    ctx.rk4_step(a.state(), 0.01, OMEGA, 2, flags=P.FP64)
    path = str(tmp_path / "a.snap")
    bve.snapshot_write(path, a.state(), 0, 3, t=0.02, dt=0.01)
    info = bve.snapshot_info(path)
    assert info["nverts"] == a.physVerts.shape[0] and info["nfaces"] == a.physFaces.shape[0]
    assert info["t"] == 0.02 and info["seed"] == 0 and info["level"] == 3
    b = bve.BVESphere(0, 3, layout="right")
    assert bve.snapshot_read(path, b.state()) == 0.02
    torch.cuda.synchronize()
    for f in FIELDS:
        assert _same(getattr(a, f).contiguous(), getattr(b, f).contiguous()), f


def test_restart_continues_the_run(ctx, tmp_path):
    a = _sphere(ctx, 1, 4, P.FP32C)
    ctx.rk4_step(a.state(), 0.005, OMEGA, 2, flags=P.FP32C)
    path = str(tmp_path / "mid.snap")
    bve.snapshot_write(path, a.state(), 1, 4, t=0.01, dt=0.005)
    ctx.rk4_step(a.state(), 0.005, OMEGA, 2, flags=P.FP32C)
    b = bve.BVESphere(1, 4)
    bve.snapshot_read(path, b.state())
    ctx.rk4_step(b.state(), 0.005, OMEGA, 2, flags=P.FP32C)
    torch.cuda.synchronize()
    leaf = torch.from_numpy(a.mesh["fmask"] == 0).cuda()
    for f in FIELDS:
        x, y = getattr(a, f), getattr(b, f)
        if f.endswith("Faces"):
            x, y = x[leaf], y[leaf]
        assert (torch.linalg.norm(x - y) / torch.linalg.norm(x)).item() <= 1e-6, f


def test_server_snapshot_restart_matches_longer_request(ctx, tmp_path):
    spec = dict(seed=0, level=3, dt=0.01, ic_seed=4, n_gaussians=2, gauss_width=0.2)
    path = str(tmp_path / "srv.snap")
    with bve.Server(0, flags=P.FP64, host_ic=True) as srv:
        r4 = srv.submit(nsteps=4, **spec)
        r6 = srv.submit(nsteps=6, **spec)
        assert srv.wait(r4, 600) and srv.wait(r6, 600)
        srv.snapshot(r4, path)
        want = srv.result(r6)
    assert bve.snapshot_info(path)["t"] == pytest.approx(0.04)
    s = bve.BVESphere(0, 3, layout="right")
    bve.snapshot_read(path, s.state())
    ctx.rk4_step(s.state(), 0.01, OMEGA, 2, flags=P.FP64)
    torch.cuda.synchronize()
    got = dict(vx=s.physVerts, vzeta=s.relVortVerts, vvel=s.velocityVerts, fx=s.physFaces, fzeta=s.relVortFaces,
               fvel=s.velocityFaces)
    leaf = s.mesh["fmask"] == 0
    for k, v in got.items():
        g, w = v.cpu().numpy(), want[k]
        if k.startswith("f"):
            g, w = g[leaf], w[leaf]
        assert np.abs(g - w).max() <= 1e-13 * np.abs(w).max(), k


def test_snapshot_of_another_mesh_is_refused(ctx, tmp_path):
    a = _sphere(ctx, 0, 2, P.FP64)
    path = str(tmp_path / "a.snap")
    bve.snapshot_write(path, a.state(), 0, 2)
    with pytest.raises(L.LpmError):
        bve.snapshot_read(path, bve.BVESphere(0, 3).state())          # other sizes
    b = bve.BVESphere(0, 2)
    b.faces_area.mul_(1.0 + 1e-12)                                      # same sizes, other areas
    with pytest.raises(L.LpmError):
        bve.snapshot_read(path, b.state())
    bad = tmp_path / "bad.snap"
    bad.write_bytes(b"not a snapshot" * 20)
    with pytest.raises(L.LpmError):
        bve.snapshot_info(str(bad))


@pytest.mark.parametrize("seed", [0, 1])
def test_vtk_file_layout(ctx, tmp_path, seed):
    a = _sphere(ctx, seed, 3, P.FP64)
    path = tmp_path / "a.vtk"
    bve.vtk_write(str(path), a.state(), seed, 3)
    header, secs = read_vtk_sections(path.read_bytes())
    assert header[0].startswith("# vtk DataFile") and header[2] == "BINARY" and header[3] == "DATASET POLYDATA"
    kinds = [s[0].split()[0] for s in secs]
    assert kinds == ["POINTS", "POLYGONS", "POINT_DATA", "SCALARS", "VECTORS", "CELL_DATA", "SCALARS", "SCALARS",
                     "VECTORS"]
    pts = np.frombuffer(secs[0][1], dtype=">f8").reshape(-1, 3)
    assert np.array_equal(pts, a.physVerts.cpu().numpy())
    nleaf = int((a.mesh["fmask"] == 0).sum())
    vpf = 3 if seed == 0 else 4
    assert secs[1][0] == f"POLYGONS {nleaf} {nleaf * (vpf + 1)}"
    polys = np.frombuffer(secs[1][1], dtype=">i4").reshape(nleaf, vpf + 1)
    assert (polys[:, 0] == vpf).all()
    fv = bve.mesh_face_verts(seed, 3)[a.mesh["fmask"] == 0]
    assert np.array_equal(polys[:, 1:], fv)
    area = np.frombuffer(secs[7][1], dtype=">f8")
    assert np.array_equal(area, a.mesh["farea"][a.mesh["fmask"] == 0])
