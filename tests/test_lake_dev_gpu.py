"""The coupled run's DEM pre-pass on the device (a wavefront over the
raster's anti-diagonals) against the host sweep, which the CPU tests pin
bit for bit to the reference's own lake_catchment_smooth
(SW2D-EFDC.cu:2766-2827).  Tolerance: bit-identical."""
import numpy as np
import pytest

from sw2d_efdc_gb300 import api
from tests.test_efdc_cards import _smooth_case

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _device_smooth(mask, dem):
    m = torch.from_numpy(np.ascontiguousarray(mask, np.int32)).to("cuda")
    z = torch.from_numpy(np.ascontiguousarray(dem, np.float64)).to("cuda")
    torch.cuda.synchronize()
    api.lake_catchment_smooth_device(dem.shape[0], dem.shape[1], m.data_ptr(), z.data_ptr())
    return z.cpu().numpy()


def _staircase_case(R, C, seed):
    """A lake whose edge runs as a staircase from south-west to north-east,
    so that long chains of edge cells each read their neighbour's update."""
    rng = np.random.default_rng(seed)
    dem = rng.normal(20.0, 4.0, (R, C))
    dem[rng.random((R, C)) < 0.01] = -9999.0
    r = np.arange(R)[:, None]
    c = np.arange(C)[None, :]
    mask = ((R - 1 - r) + c > (R + C) // 2).astype(np.int32)
    mask[(r * 7 + c * 3) % 29 == 0] = 2
    return mask, dem


@pytest.mark.parametrize("seed,R,C", [(1, 30, 25), (2, 3, 40), (3, 64, 3), (4, 57, 61), (5, 2, 2), (6, 701, 556)])
def test_device_smoothing_matches_the_host_sweep(seed, R, C):
    mask, dem = _smooth_case(seed, R, C)
    assert _device_smooth(mask, dem).tobytes() == api.lake_catchment_smooth(mask, dem).tobytes()


@pytest.mark.parametrize("R,C", [(300, 420), (2048, 1536)])
def test_device_smoothing_keeps_the_sweep_order(R, C):
    mask, dem = _staircase_case(R, C, R + C)
    host = api.lake_catchment_smooth(mask, dem)
    assert _device_smooth(mask, dem).tobytes() == host.tobytes()
    # the case depends on the order: every edge cell evaluated from the
    # original neighbours gives another DEM
    z, m = dem, mask
    jac = dem.copy()
    inner = jac[1:-1, 1:-1]
    v = m[1:-1, 1:-1]
    guard = ((v != m[:-2, 1:-1]) & (z[2:, 1:-1] != -9999.0), (v != m[2:, 1:-1]) & (z[:-2, 1:-1] != -9999.0),
             (v != m[1:-1, :-2]) & (z[1:-1, 2:] != -9999.0), (v != m[1:-1, 2:]) & (z[1:-1, :-2] != -9999.0))
    means = ((z[:-2, 1:-1] + z[2:, 1:-1]) / 2.0, (z[:-2, 1:-1] + z[2:, 1:-1]) / 2.0,
             (z[1:-1, :-2] + z[1:-1, 2:]) / 2.0, (z[1:-1, :-2] + z[1:-1, 2:]) / 2.0)
    for g, mv in zip(guard, means):
        sel = g & (v != 1)
        inner[sel] = mv[sel]
    assert not np.array_equal(jac, host)
