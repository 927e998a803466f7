"""Device initial vorticity (lpm_ic_rh54_gaussians_device) against the host functions
(lpm_ic_rh54 + lpm_ic_gaussians_add) and the oracle's RH54: products and sums are rounded as on
the host, so only the math-library transcendentals differ (a few ulps): 1e-13 relative."""
import numpy as np
import pytest
import torch

from lpmkokkos_gb300 import _lib as L
from lpmkokkos_gb300 import bve

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed,level,ng,width", [(0, 5, 3, 0.1), (1, 5, 0, 0.1), (0, 3, 64, 0.3)])
def test_device_ic_matches_host(oracle, seed, level, ng, width):
    m = bve.build_mesh(seed, level)
    for pts, layout in ((m["vx"], "right"), (m["fx"], "left")):
        host = bve.rh54_gaussians(77, ng, width)(pts)
        t = torch.from_numpy(pts)
        x = (t.t().contiguous().cuda().t() if layout == "left" else t.cuda())
        dev = bve.ic_rh54_gaussians_device(x, 77, ng, width)
        torch.cuda.synchronize()
        d = dev.cpu().numpy()
        assert np.abs(d - host).max() <= 1e-13 * np.abs(host).max()
        if ng == 0:
            ref = oracle.ic_rh54(pts)
            assert np.abs(d - ref).max() <= 1e-13 * np.abs(ref).max()


def test_device_ic_rejects_too_many_gaussians():
    x = torch.zeros(4, 3, dtype=torch.float64, device="cuda")
    z = torch.zeros(4, dtype=torch.float64, device="cuda")
    c = np.zeros((65, 3)); a = np.zeros(65)
    rc = L.lib().lpm_ic_rh54_gaussians_device(x.data_ptr(), 4, 3, 1, c.ctypes.data, a.ctypes.data, 65, 0.1,
                                              z.data_ptr(), None)
    assert rc == L.LPM_ERR_INVALID_ARGUMENT
