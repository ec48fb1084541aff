"""BSM_PT_DETERMINISTIC: bit-reproducible images.

By default contributions reach the per-pixel sums by FP32 atomics, so the last
bits of an image depend on the order in which the GPU adds them.  With the
flag, a call sums its contributions per pixel as 32.32 fixed-point integers
(exact, so independent of the order) and adds them to the view's history
once.  The images must then be identical bit for bit across repeats, launch
paths (graph or direct), wavefront chunking and batching, and equal the
oracle's images bit for bit when the oracle sums the same way (its F_FIXED
mode): every path's contributions agree exactly, only the float summation
order ever differed."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-4


def rel_err(g, c):
    g = g[..., :3].astype(np.float64)
    c = c[..., :3].astype(np.float64)
    return np.abs(g - c) / np.maximum(np.abs(c), 1e-3)


def bits(img):
    return np.ascontiguousarray(img).view(np.uint32)


@pytest.fixture(scope="module")
def room(bsm, ctx, oracle):
    sc = bsm.generate_scene(bsm.BSM_SCENE_ROOM, seed=1, width=64, height=64)
    return sc, ctx.load_scene(sc), oracle.OracleScene(sc)


@pytest.fixture(scope="module")
def terrain(bsm, ctx, oracle):
    sc = bsm.generate_scene(bsm.BSM_SCENE_TERRAIN, seed=2, grid=96, spheres=200, sky_width=256, sky_height=128,
                            width=96, height=54)
    return sc, ctx.load_scene(sc), oracle.OracleScene(sc)


def test_repeated_renders_are_bit_identical(bsm, terrain, ctx):
    sc, sid, _ = terrain
    s = bsm.settings(spp=16, max_segments=8, seed=4, flags=bsm.BSM_PT_DETERMINISTIC)
    first, _ = ctx.render(sid, [sc.camera], s)
    assert first[0][..., :3].mean() > 0.01
    for _ in range(3):
        again, _ = ctx.render(sid, [sc.camera], s)
        assert np.array_equal(bits(again[0]), bits(first[0]))


def test_deterministic_render_matches_oracle(bsm, terrain, ctx):
    sc, sid, osc = terrain
    imgs, st = ctx.render(sid, [sc.camera], bsm.settings(spp=4, max_segments=8, seed=4,
                                                         flags=bsm.BSM_PT_DETERMINISTIC))
    ref, ost, _ = osc.render(sc.camera.as_array(), spp=4, max_segments=8, seed=4)
    assert list(st.rays_per_segment[:8]) == [int(x) for x in ost[:8]]
    assert rel_err(imgs[0], ref).max() <= RTOL
    plain, _ = ctx.render(sid, [sc.camera], bsm.settings(spp=4, max_segments=8, seed=4))
    assert rel_err(imgs[0], plain[0]).max() <= 1e-5


@pytest.mark.parametrize("which, flags, spp, segs", [("room", 0, 4, 4), ("room", 1, 4, 4), ("room", 2, 4, 4),
                                                     ("room", 4, 4, 4), ("terrain", 0, 4, 8), ("terrain", 1, 8, 6)])
def test_images_equal_the_oracle_bit_for_bit(bsm, room, terrain, ctx, which, flags, spp, segs):
    """The oracle's F_FIXED mode sums the same contributions as the same fixed-point integers and converts them
    as the library does, so where every contribution agrees bit for bit the images do too."""
    sc, sid, osc = room if which == "room" else terrain
    imgs, st = ctx.render(sid, [sc.camera], bsm.settings(spp=spp, max_segments=segs, seed=3,
                                                         flags=flags | bsm.BSM_PT_DETERMINISTIC))
    ref, ost, _ = osc.render(sc.camera.as_array(), spp=spp, max_segments=segs, seed=3,
                             flags=flags | bsm.BSM_PT_DETERMINISTIC)
    assert list(st.rays_per_segment[:segs]) == [int(x) for x in ost[:segs]]
    g, o = bits(imgs[0]), bits(ref)
    bad = np.argwhere(g != o)
    assert bad.size == 0, (f"{len(bad)} values differ, first {bad[:4].tolist()}: gpu "
                           f"{imgs[0][tuple(bad[0])]!r} oracle {ref[tuple(bad[0])]!r}, largest ulp distance "
                           f"{int(np.abs(g.astype(np.int64) - o.astype(np.int64)).max())}")


def test_same_bits_with_chunks_and_without_graphs(bsm, terrain, ctx):
    """Exact sums do not depend on how the paths are cut into chunks or launched."""
    sc, sid, _ = terrain
    det = bsm.BSM_PT_DETERMINISTIC
    a, _ = ctx.render(sid, [sc.camera], bsm.settings(spp=8, max_segments=6, seed=7, flags=det))
    b, sb = ctx.render(sid, [sc.camera], bsm.settings(spp=8, max_segments=6, seed=7, flags=det,
                                                      wavefront_capacity=9000))
    c, _ = ctx.render(sid, [sc.camera], bsm.settings(spp=8, max_segments=6, seed=7,
                                                     flags=det | bsm.BSM_PT_NO_GRAPH))
    assert sb.chunks > 1
    assert np.array_equal(bits(a[0]), bits(b[0]))
    assert np.array_equal(bits(a[0]), bits(c[0]))


def test_progressive_accumulation_is_bit_reproducible(bsm, terrain, ctx):
    sc, sid, _ = terrain
    det = bsm.BSM_PT_DETERMINISTIC

    def two_calls():
        ctx.render(sid, [sc.camera], bsm.settings(spp=2, max_segments=4, seed=5, accumulate=0, flags=det))
        imgs, _ = ctx.render(sid, [sc.camera], bsm.settings(spp=2, max_segments=4, seed=5, accumulate=1, flags=det))
        return imgs[0]

    x = two_calls()
    y = two_calls()
    assert np.array_equal(bits(x), bits(y))


def test_batched_views_equal_separate_renders_bit_for_bit(bsm, terrain, ctx):
    sc, sid, _ = terrain
    det = bsm.BSM_PT_DETERMINISTIC
    cams = [bsm.make_camera((0.5, 0.35, -0.2), (0.0, -0.3, 1.0), width=40, height=24),
            bsm.make_camera((0.2, 0.3, 0.9), (0.6, -0.4, -0.7), width=32, height=32, yfov_deg=45.0)]
    views = [(cams[0], 4, 5, 11), (cams[1], 2, 6, 12)]
    batch, _ = ctx.render_batch(sid, views, bsm.settings(flags=det))
    for (cam, spp, segs, seed), img in zip(views, batch):
        one, _ = ctx.render(sid, [cam], bsm.settings(spp=spp, max_segments=segs, seed=seed, flags=det))
        assert np.array_equal(bits(img), bits(one[0]))


def test_cached_render_is_bit_reproducible(bsm, ctx):
    """The cache queries' network outputs add to the fixed-point sums too (fixed weights: no training)."""
    scene = bsm.generate_scene(bsm.BSM_SCENE_ROOM, seed=41, spheres=24)
    sid = ctx.load_scene(scene)
    cam = bsm.make_camera(tuple(scene.camera.position), tuple(scene.camera.front), width=64, height=48)
    c = bsm.RadianceCache(ctx, seed=5)
    try:
        cs = bsm.cache_settings(cache_segment=2, train_steps=0)
        s = bsm.settings(spp=8, seed=9, flags=bsm.BSM_PT_DETERMINISTIC)
        a, st, _ = c.render(sid, cam, s, cs)
        b, _, _ = c.render(sid, cam, s, cs)
        assert a[..., :3].mean() > 0.0
        assert np.array_equal(bits(a), bits(b))
        plain, _, _ = c.render(sid, cam, bsm.settings(spp=8, seed=9), cs)
        assert rel_err(a, plain).max() <= 1e-5
    finally:
        c.close()
        ctx.release(sid)
