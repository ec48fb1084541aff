"""The oracle's light evaluation against golden vectors from the reference's own
shader code (renderer/lights.hlsl dir_light_eval and point_light_eval, compiled
from the reference sources; tests/golden/make_golden.py).

* directional lights: radiance equal bit for bit, direction within 2.5e-7 (the
  pass renormalises it);
* point lights: the range falloff saturate(1 - (d^2 / range^2)^2) / max(d^2,
  0.001) and the direction to the light equal bit for bit, including points
  nearer than sqrt(0.001) and beyond the range;
* spot lights: the ramp clamp(cos, cos_outer, cos_inner) within 2e-4 of the
  unramped value (the pass renormalises the spot axis, which the reference
  takes as given; the ramp divides by cos_inner - cos_outer, down to 0.001),
  cases on the cone's inner and outer edges included.
The GPU evaluates the same function (pt_lights.cuh, used by both), and renders
with these lights match the oracle (tests/test_gpu_lights.py)."""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden", "lights_golden.npz")


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLD)


def point_rows(pin):
    rows = np.zeros((pin.shape[0], 16), np.float32)
    rows[:, 0] = 1.0                 # kind: point / spot
    rows[:, 1:13] = pin[:, :12]      # position, emission, range, direction to the light, cos_inner, cos_outer
    return rows


def test_point_and_spot_lights_match_reference_shader(oracle, golden):
    pin, pout = golden["point_in"], golden["point_out"]
    rows = point_rows(pin)
    got = np.stack([oracle.light_eval(rows[i], pin[i, 12:15][None])[0] for i in range(rows.shape[0])])
    assert np.array_equal(got[:, 3:6], pout[:, 3:6]), "direction to the light"
    spot = pin[:, 10] > pin[:, 11]
    assert spot.sum() > 1000 and (~spot).sum() > 1000
    assert np.array_equal(got[~spot, :3], pout[~spot, :3]), "point-light falloff"
    d2 = ((pin[:, 0:3] - pin[:, 12:15]) ** 2).sum(1)
    peak = np.abs(pin[:, 3:6]).max(1) / np.maximum(d2, 1e-3)
    err = np.abs(got[spot, :3] - pout[spot, :3]).max(1) / peak[spot]
    assert err.max() <= 2e-4, err.max()
    # the reached flag follows the radiance: nothing arrives outside the cone or beyond the range
    reached = got[:, 7] == 1.0
    assert np.array_equal(reached, np.abs(got[:, :3]).max(1) > 0.0)
    assert (~reached).sum() > 500 and (np.abs(pout[~reached, :3]).max(1) <= 2e-4 * peak[~reached]).all()


def test_directional_lights_match_reference_shader(oracle, golden):
    din, dout = golden["dir_in"], golden["dir_out"]
    for i in range(din.shape[0]):
        row = np.zeros(16, np.float32)
        row[1:7] = din[i, :6]
        got = oracle.light_eval(row, din[i, 6:9][None])[0]
        assert np.array_equal(got[:3], dout[i, :3])
        np.testing.assert_allclose(got[3:6], dout[i, 3:6], rtol=0, atol=2.5e-7)   # the pass normalises it
