"""Batched multi-view rendering and the autotuner (GPU).

A batch of views of different sizes, sample counts and seeds rendered in one
wavefront equals each view rendered alone (same paths: within 1e-4 relative
per pixel) and equals the oracle; the autotuner returns valid parameters,
persists them and reads them back, and renders with tuned parameters still
match."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
RTOL = 1e-4


def rel_err(g, c):
    g = g[..., :3].astype(np.float64)
    c = c[..., :3].astype(np.float64)
    return np.abs(g - c) / np.maximum(np.abs(c), 1e-3)


def make_views(bsm, n, seed):
    rng = np.random.default_rng(seed)
    views = []
    for i in range(n):
        side = int(np.exp(rng.uniform(np.log(16), np.log(72))))
        w = side
        h = max(8, int(side * rng.uniform(0.6, 1.2)))
        pos = (rng.uniform(0.2, 0.8), rng.uniform(0.3, 0.6), rng.uniform(-0.2, 0.3))
        tgt = (rng.uniform(0.3, 0.7), 0.0, rng.uniform(0.4, 0.8))
        front = tuple(np.subtract(tgt, pos))
        cam = bsm.make_camera(pos, front, yfov_deg=float(rng.uniform(40, 70)), width=w, height=h)
        views.append((cam, int(rng.choice([1, 2, 4])), int(rng.choice([2, 4, 8])), int(rng.integers(1, 1000))))
    return views


@pytest.fixture(scope="module")
def scene(bsm, ctx, oracle):
    sc = bsm.generate_scene(bsm.BSM_SCENE_TERRAIN, seed=3, grid=64, spheres=120, sky_width=128, sky_height=64)
    return sc, ctx.load_scene(sc), oracle.OracleScene(sc)


def test_batch_equals_views_rendered_alone(bsm, ctx, scene):
    sc, sid, osc = scene
    views = make_views(bsm, 12, seed=1)
    s = bsm.settings(spp=1, max_segments=4, seed=1)
    imgs, st = ctx.render_batch(sid, views, s)
    assert st.paths == sum(v[0].width * v[0].height * v[1] for v in views)
    for (cam, spp, segs, seed), img in zip(views, imgs):
        alone, _ = ctx.render(sid, [cam], bsm.settings(spp=spp, max_segments=segs, seed=seed))
        assert rel_err(img, alone[0]).max() <= RTOL
    for (cam, spp, segs, seed), img in list(zip(views, imgs))[:3]:
        ref, _, _ = osc.render(cam.as_array(), spp=spp, max_segments=segs, seed=seed)
        assert rel_err(img, ref).max() <= RTOL


def test_autotune_persists_and_keeps_results(bsm, ctx, scene, tmp_path):
    sc, sid, osc = scene
    views = make_views(bsm, 6, seed=2)
    s = bsm.settings(spp=1, max_segments=4, seed=1)
    cache = str(tmp_path / "tune.txt")
    r = ctx.autotune(sid, views, s, cache)
    assert r.tried >= 5 and r.from_cache == 0
    assert r.best.block_size in (64, 128, 256) and r.best.postpone_depth <= 16 and 1 <= r.best.refill_lanes <= 32
    assert r.best_ms <= r.default_ms * 1.001
    assert os.path.getsize(cache) > 0
    r2 = ctx.autotune(sid, views, s, cache)
    assert r2.from_cache == 1 and r2.best.block_size == r.best.block_size
    # renders with the tuned parameters still match the oracle
    cam, spp, segs, seed = views[0]
    img, _ = ctx.render(sid, [cam], bsm.settings(spp=spp, max_segments=segs, seed=seed))
    ref, _, _ = osc.render(cam.as_array(), spp=spp, max_segments=segs, seed=seed)
    assert rel_err(img[0], ref).max() <= RTOL
    # every tunable corner gives the same image
    for p in [(64, 4096, 0, 1, 0), (256, 1 << 20, 16, 32, 1), (128, 1024, 4, 16, 1)]:
        ctx.set_tuning(sid, bsm.TuneParams(*p))
        im, _ = ctx.render(sid, [cam], bsm.settings(spp=spp, max_segments=segs, seed=seed))
        assert rel_err(im[0], ref).max() <= RTOL
    ctx.set_tuning(sid, None)


def test_set_tuning_rejects_bad_values(bsm, ctx, scene):
    sc, sid, osc = scene
    with pytest.raises(bsm.BsmError):
        ctx.set_tuning(sid, bsm.TuneParams(100, 0, 16, 8, 0))
    with pytest.raises(bsm.BsmError):
        ctx.set_tuning(sid, bsm.TuneParams(128, 0, 17, 8, 0))
    with pytest.raises(bsm.BsmError):
        ctx.set_tuning(sid, bsm.TuneParams(128, 0, 16, 8, 2))
