"""Host-side helpers of bench.py: the equal-error frame time of the cache comparison."""
import importlib.util
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def pts(*rows):
    return [{"spp": s, "relmse": e, "ms": t} for s, e, t in rows]


def test_interpolates_log_log_between_bracketing_points(bench):
    curve = pts((2, 0.4, 10.0), (4, 0.1, 20.0))
    t = bench.equal_error_time(curve, "relmse", 0.2)
    u = (np.log(0.2) - np.log(0.4)) / (np.log(0.1) - np.log(0.4))
    assert t == pytest.approx(np.exp(np.log(10.0) + u * np.log(2.0)))
    assert bench.equal_error_time(curve, "relmse", 0.4) == pytest.approx(10.0)
    assert bench.equal_error_time(curve, "relmse", 0.1) == pytest.approx(20.0)


def test_outside_the_measured_range_is_none(bench):
    curve = pts((2, 0.4, 10.0), (4, 0.1, 20.0))
    assert bench.equal_error_time(curve, "relmse", 0.5) is None    # reached before the cheapest point
    assert bench.equal_error_time(curve, "relmse", 0.05) is None   # beyond the most accurate point


def test_a_noisy_point_above_a_cheaper_one_is_left_out(bench):
    """A slower point whose error is above a cheaper point's (a firefly in a noisy metric) does not count:
    the target between them is not interpolated against it."""
    curve = pts((2, 0.26, 6.8), (4, 0.39, 11.9), (8, 0.23, 21.6), (32, 0.038, 74.2))
    assert bench.equal_error_time(curve, "relmse", 0.30) is None
    t = bench.equal_error_time(curve, "relmse", 0.245)
    assert 6.8 < t < 21.6
    assert bench.equal_error_time(curve, "relmse", 0.1) > 21.6
