"""Serving loop (GPU): resident scenes, admission by memory, continuous
batching.  A request's image is the same rendered alone and in a mix of
requests on several scenes, and equals bsm_render of the same view (within
the 1e-4 relative radiance tolerance; bit for bit when the server and the
render both sum in fixed point)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
RTOL = 1e-4


def rel_err(g, c):
    g = g[..., :3].astype(np.float64)
    c = c[..., :3].astype(np.float64)
    return np.abs(g - c) / np.maximum(np.abs(c), 1e-3)


@pytest.fixture(scope="module")
def served(bsm):
    ctx = bsm.Context(0)
    scenes = [bsm.generate_scene(bsm.BSM_SCENE_ROOM, seed=31, spheres=16),
              bsm.generate_scene(bsm.BSM_SCENE_TERRAIN, seed=32, grid=48, spheres=40, sky_width=64, sky_height=32),
              bsm.generate_scene(bsm.BSM_SCENE_TERRAIN, seed=33, grid=80, spheres=90, sky_width=128, sky_height=64)]
    ids = [ctx.load_scene(s) for s in scenes]
    yield ctx, scenes, ids
    ctx.close()


def request_mix(bsm, scenes, ids, n, seed):
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(n):
        k = int(rng.integers(0, len(ids)))
        base = scenes[k].camera
        w = int(rng.integers(24, 96))
        h = int(rng.integers(24, 80))
        cam = bsm.make_camera(tuple(base.position), tuple(base.front), width=w, height=h,
                              yfov_deg=float(rng.uniform(45, 70)))
        reqs.append((ids[k], cam, int(rng.choice([1, 2, 4])), int(rng.choice([2, 4, 8])), int(rng.integers(1, 99))))
    return reqs


def test_same_alone_and_in_the_mix(bsm, served):
    ctx, scenes, ids = served
    mix = request_mix(bsm, scenes, ids, 24, seed=1)
    target = mix[5]
    sid, cam, spp, segs, seed = target
    ref, _ = ctx.render(sid, [cam], bsm.settings(spp=spp, max_segments=segs, seed=seed))
    ctx.server_start(pool_bytes=64 << 20, chunk_paths=1 << 16, lanes=3)
    try:
        rid, alone = ctx.submit(sid, cam, spp, segs, seed)
        st = ctx.wait(rid, timeout_ms=60000)
        assert st.state == bsm.BSM_REQ_DONE and st.done_ms >= st.admit_ms >= st.submit_ms
        outs = [ctx.submit(*r) for r in mix]
        for rid_i, _ in outs:
            assert ctx.wait(rid_i, timeout_ms=60000).state == bsm.BSM_REQ_DONE
        stats = ctx.server_stats()
        assert stats.completed == len(mix) + 1 and stats.extend_rays > 0
    finally:
        ctx.server_stop()
    assert rel_err(alone, ref[0]).max() <= RTOL
    assert rel_err(outs[5][1], alone).max() <= RTOL
    for (sid_i, cam_i, spp_i, segs_i, seed_i), (_, img) in list(zip(mix, outs))[:8]:
        r, _ = ctx.render(sid_i, [cam_i], bsm.settings(spp=spp_i, max_segments=segs_i, seed=seed_i))
        assert rel_err(img, r[0]).max() <= RTOL


def test_same_bits_alone_in_the_mix_and_as_rendered(bsm, served):
    """BSM_SERVER_DETERMINISTIC: exact fixed-point sums make a request's image independent of the chunks and the
    company it ran in, bit for bit, and equal to bsm_render's with BSM_PT_DETERMINISTIC."""
    ctx, scenes, ids = served
    mix = request_mix(bsm, scenes, ids, 24, seed=3)
    sid, cam, spp, segs, seed = mix[7]
    ctx.server_start(pool_bytes=96 << 20, chunk_paths=1 << 16, lanes=3, deterministic=True)
    try:
        rid, alone = ctx.submit(sid, cam, spp, segs, seed)
        assert ctx.wait(rid, timeout_ms=60000).state == bsm.BSM_REQ_DONE
        outs = [ctx.submit(*r) for r in mix]
        for rid_i, _ in outs:
            assert ctx.wait(rid_i, timeout_ms=60000).state == bsm.BSM_REQ_DONE
    finally:
        ctx.server_stop()
    assert alone[..., :3].max() > 0.0
    assert np.array_equal(outs[7][1].view(np.uint32), alone.view(np.uint32))
    det = bsm.BSM_PT_DETERMINISTIC
    for (sid_i, cam_i, spp_i, segs_i, seed_i), (_, img) in list(zip(mix, outs))[:8]:
        r, _ = ctx.render(sid_i, [cam_i], bsm.settings(spp=spp_i, max_segments=segs_i, seed=seed_i, flags=det))
        assert np.array_equal(img.view(np.uint32), r[0].view(np.uint32))


def test_admission_waits_for_memory(bsm, served):
    ctx, scenes, ids = served
    cam = bsm.make_camera(tuple(scenes[0].camera.position), tuple(scenes[0].camera.front), width=64, height=64)
    # pool holds two such requests at a time
    ctx.server_start(pool_bytes=2 * 64 * 64 * 16, chunk_paths=1 << 14, lanes=2)
    try:
        with pytest.raises(bsm.BsmError) as e:
            big = bsm.make_camera((0.5, 0.5, -1), (0, 0, 1), width=200, height=200)
            ctx.submit(ids[0], big, 1)
        assert e.value.status == -10
        rids = [ctx.submit(ids[0], cam, 2, 4, s)[0] for s in range(6)]
        for r in rids:
            assert ctx.wait(r, timeout_ms=60000).state == bsm.BSM_REQ_DONE
        st = ctx.server_stats()
        assert st.admitted == 6 and st.completed == 6 and st.rejected == 1 and st.pool_used_bytes == 0
    finally:
        ctx.server_stop()


def test_server_rejects_unknown_flags(bsm, served):
    ctx, _, _ = served
    import ctypes as C
    opts = bsm.ServerOpts(1 << 20, 0, 0, 0, 2)   # bit 1 is not a server flag
    assert ctx._L.bsm_server_start(ctx.h, C.byref(opts)) == -1   # BSM_ERR_INVALID_ARG
    ctx.server_start(pool_bytes=1 << 20, deterministic=True)   # the one defined flag starts
    ctx.server_stop()


def test_scenes_locked_while_serving(bsm, served):
    ctx, scenes, ids = served
    ctx.server_start(pool_bytes=1 << 20)
    try:
        with pytest.raises(bsm.BsmError):
            ctx.upload(scenes[0])
    finally:
        ctx.server_stop()


def test_small_request_passes_a_large_one_of_the_same_scene(bsm, served):
    """Least work first within a scene: a small request submitted just after a large one of the same scene joins
    the next chunk and finishes long before the large one, whose image is still the same as rendered alone."""
    ctx, scenes, ids = served
    base = scenes[2].camera
    large = bsm.make_camera(tuple(base.position), tuple(base.front), width=640, height=480)
    small = bsm.make_camera(tuple(base.position), tuple(base.front), width=32, height=24)
    ctx.server_start(pool_bytes=64 << 20, chunk_paths=1 << 16, lanes=2)
    try:
        rid_l, img_l = ctx.submit(ids[2], large, 8, 8, 5)
        rid_s, img_s = ctx.submit(ids[2], small, 1, 4, 6)
        st_s = ctx.wait(rid_s, timeout_ms=60000)
        st_l = ctx.wait(rid_l, timeout_ms=60000)
        assert st_s.state == bsm.BSM_REQ_DONE and st_l.state == bsm.BSM_REQ_DONE
        assert st_s.done_ms < st_l.done_ms
    finally:
        ctx.server_stop()
    ref_l, _ = ctx.render(ids[2], [large], bsm.settings(spp=8, max_segments=8, seed=5))
    ref_s, _ = ctx.render(ids[2], [small], bsm.settings(spp=1, max_segments=4, seed=6))
    assert rel_err(img_l, ref_l[0]).max() <= RTOL
    assert rel_err(img_s, ref_s[0]).max() <= RTOL
