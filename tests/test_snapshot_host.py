"""Snapshots and VTK output of a state held in HOST memory (include/lpm_bve_snapshot.h), on CPU.

Host arrays are copied with memcpy, so these calls need no CUDA device.  The device-array path
and restarts from a stepped run are in test_gpu_snapshot.py.

  * write -> read restores every array of the state bit for bit, across the two Kokkos layouts
    (LayoutRight: row-major n x 3; LayoutLeft: column-major) and both mesh seeds;
  * the header reports the mesh, sizes and time metadata written;
  * a snapshot of another mesh (other sizes, other areas or mask), a truncated file and a file
    that is not a snapshot are refused;
  * the VTK file's sections have the sizes its header announces and hold the state's fields.
"""
import numpy as np
import pytest
import torch

from lpmkokkos_gb300 import _lib as L
from lpmkokkos_gb300 import bve
from vtk_reader import read_vtk_sections

EVOLVING = ("vx", "vzeta", "vvel", "fx", "fzeta", "fvel")


def _tensor(a, layout):
    a = np.asfortranarray(a) if layout == "left" and a.ndim == 2 else np.ascontiguousarray(a)
    return torch.from_numpy(a)


def _state(seed, level, layout="right", rseed=3):
    """Mesh positions, areas and mask of (seed, level) with random vorticity and velocity."""
    m = bve.build_mesh(seed, level)
    rng = np.random.default_rng(rseed)
    nv, nf = m["nverts"], m["nfaces"]
    return bve.BVEState(_tensor(m["vx"], layout), _tensor(rng.normal(size=nv), layout),
                        _tensor(rng.normal(size=(nv, 3)), layout), _tensor(m["fx"], layout),
                        _tensor(rng.normal(size=nf), layout), _tensor(rng.normal(size=(nf, 3)), layout),
                        _tensor(m["farea"], layout), torch.from_numpy(m["fmask"].astype(np.uint8))), m


def _blank_like(st, layout):
    z = lambda t: _tensor(np.zeros(tuple(t.shape)), layout)  # noqa: E731
    return bve.BVEState(z(st.vx), z(st.vzeta), z(st.vvel), z(st.fx), z(st.fzeta), z(st.fvel), st.farea.clone(),
                        st.fmask.clone())


@pytest.mark.parametrize("seed", [0, 1])
@pytest.mark.parametrize("src_layout,dst_layout", [("right", "left"), ("left", "right"), ("left", "left")])
def test_host_round_trip_across_layouts(native, tmp_path, seed, src_layout, dst_layout):
    st, _ = _state(seed, 3, src_layout)
    assert st.vx.stride() == ((1, st.vx.shape[0]) if src_layout == "left" else (3, 1))
    path = str(tmp_path / "s.snap")
    bve.snapshot_write(path, st, seed, 3, t=1.25, dt=0.01, omega=2.5)
    out = _blank_like(st, dst_layout)
    assert bve.snapshot_read(path, out) == 1.25
    for k in EVOLVING:
        a, b = getattr(st, k), getattr(out, k)
        assert a.shape == b.shape and torch.equal(a, b), k


def test_host_snapshot_info(native, tmp_path):
    st, m = _state(0, 2)
    path = str(tmp_path / "s.snap")
    bve.snapshot_write(path, st, 0, 2, t=0.5, dt=0.02, omega=3.0)
    info = bve.snapshot_info(path)
    assert info == dict(seed=0, level=2, nverts=m["nverts"], nfaces=m["nfaces"], t=0.5, dt=0.02, omega=3.0)


def test_host_snapshot_of_another_mesh_is_refused(native, tmp_path):
    st, _ = _state(0, 2)
    path = tmp_path / "s.snap"
    bve.snapshot_write(str(path), st, 0, 2)
    with pytest.raises(L.LpmError):
        bve.snapshot_read(str(path), _state(0, 3)[0])                 # other sizes
    other = _blank_like(st, "right")
    other.farea.mul_(1.0 + 1e-12)                                     # same sizes, other areas
    with pytest.raises(L.LpmError):
        bve.snapshot_read(str(path), other)
    other = _blank_like(st, "right")
    other.fmask[0] ^= 1                                               # same sizes, other mask
    with pytest.raises(L.LpmError):
        bve.snapshot_read(str(path), other)
    raw = path.read_bytes()
    cut = tmp_path / "cut.snap"
    cut.write_bytes(raw[: len(raw) - 9])                              # truncated
    with pytest.raises(L.LpmError):
        bve.snapshot_read(str(cut), _blank_like(st, "right"))
    bad = tmp_path / "bad.snap"
    bad.write_bytes(b"not a snapshot" * 20)
    with pytest.raises(L.LpmError):
        bve.snapshot_info(str(bad))
    # a refused read writes nothing
    blank = _blank_like(st, "right")
    with pytest.raises(L.LpmError):
        bve.snapshot_read(str(cut), blank)
    assert all(not getattr(blank, k).any() for k in EVOLVING)


@pytest.mark.parametrize("seed", [0, 1])
def test_host_vtk_file_layout(native, tmp_path, seed):
    st, m = _state(seed, 3, "left")
    path = tmp_path / "a.vtk"
    bve.vtk_write(str(path), st, seed, 3)
    header, secs = read_vtk_sections(path.read_bytes())
    assert header[0].startswith("# vtk DataFile") and header[2] == "BINARY" and header[3] == "DATASET POLYDATA"
    assert [s[0].split()[0] for s in secs] == ["POINTS", "POLYGONS", "POINT_DATA", "SCALARS", "VECTORS",
                                                "CELL_DATA", "SCALARS", "SCALARS", "VECTORS"]
    leaf = m["fmask"] == 0
    nleaf, vpf = int(leaf.sum()), (3 if seed == 0 else 4)
    assert np.array_equal(np.frombuffer(secs[0][1], dtype=">f8").reshape(-1, 3), m["vx"])
    assert secs[1][0] == f"POLYGONS {nleaf} {nleaf * (vpf + 1)}"
    polys = np.frombuffer(secs[1][1], dtype=">i4").reshape(nleaf, vpf + 1)
    assert (polys[:, 0] == vpf).all()
    assert np.array_equal(polys[:, 1:], bve.mesh_face_verts(seed, 3)[leaf])
    assert secs[2][0] == f"POINT_DATA {m['nverts']}" and secs[5][0] == f"CELL_DATA {nleaf}"
    assert np.array_equal(np.frombuffer(secs[3][1], dtype=">f8"), st.vzeta.numpy())
    assert np.array_equal(np.frombuffer(secs[4][1], dtype=">f8").reshape(-1, 3), st.vvel.numpy())
    assert np.array_equal(np.frombuffer(secs[6][1], dtype=">f8"), st.fzeta.numpy()[leaf])
    assert np.array_equal(np.frombuffer(secs[7][1], dtype=">f8"), m["farea"][leaf])
    assert np.array_equal(np.frombuffer(secs[8][1], dtype=">f8").reshape(-1, 3), st.fvel.numpy()[leaf])
