"""The C++ drop-in (include/lpm_bve.hpp) running the reference's BVE driver unchanged in
shape (tests/LpmBVETest.cpp: solid-body rotation, cubed sphere depth 3, dt 0.01): it must
produce exactly the positions the Python interface produces through the same C ABI."""
import math
import os
import subprocess

import numpy as np
import pytest
import torch

import lpmkokkos_gb300 as P

pytestmark = pytest.mark.gpu

EXE = os.path.join(os.path.dirname(P._build.LIB), "bve_solid_body")


@pytest.mark.parametrize("prec,arg", [(P.FP64, []), (P.FP32C, ["-fp32c"])])
def test_cpp_driver_matches_python(ctx, tmp_path, prec, arg):
    from lpmkokkos_gb300 import bve
    out = tmp_path / "x.bin"
    res = subprocess.run([EXE, "-d", "3", "-dt", "0.01", "-tf", "0.1", "-o", str(out), *arg],
                         capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "tests pass" in res.stdout
    xc = np.fromfile(out, dtype=np.float64).reshape(-1, 3)

    omega = 2 * math.pi
    s = bve.BVESphere(P.SEED_CUBED, 3, omega=0.0)
    s.init_vorticity(lambda x: 2 * omega * x[:, 2], ctx, flags=prec)
    for _ in range(10):
        ctx.rk4_step(s.state(), 0.01, omega, 1, flags=prec)
    torch.cuda.synchronize()
    leaf = s.mesh["fmask"] == 0
    xp = s.physFaces.cpu().numpy()[leaf]
    assert np.array_equal(xc, xp)
    # and the rigid rotation is reproduced to discretisation accuracy
    pos_err = float(res.stdout.split("position error at t=tfinal ErrNorms: l2 =")[1].split()[0])
    assert pos_err < 1e-2
