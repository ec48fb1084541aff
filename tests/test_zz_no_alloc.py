"""bsm_render_noalloc: the render entry point for callers that cannot allocate.

Callers such as an engine that owns all device memory through its own
allocator, or a frame loop that must not allocate while it renders, call this
entry point with a resident scene and their own device output buffer; its
working memory is a fixed array inside the library.  These tests check, through
the C ABI, that two calls in a row give the same image as the regular
bsm_render (within the 1e-4 relative tolerance used for radiance everywhere),
that the scratch layouts of non-opaque, two-level and multi-light scenes hold
at the largest chunk the array allows, and that a chunk larger than the fixed
array or a misaligned output buffer is refused.  The file sorts last so that a
run stopping at the first failure has run every other test first."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-4


def rel_err(g, c):
    g = g[..., :3].astype(np.float64)
    c = c[..., :3].astype(np.float64)
    return np.abs(g - c) / np.maximum(np.abs(c), 1e-3)


@pytest.fixture(scope="module")
def setup(bsm):
    ctx = bsm.Context(0)
    scene = bsm.generate_scene(bsm.BSM_SCENE_ROOM, seed=21, width=80, height=60)
    sid = ctx.load_scene(scene)
    yield ctx, scene, sid
    ctx.close()


def test_noalloc_matches_render_on_two_calls(bsm, setup):
    ctx, scene, sid = setup
    L = bsm.lib()
    cam = scene.camera
    s = bsm.settings(spp=4, max_segments=4, seed=13, accumulate=0)
    ref, _ = ctx.render(sid, [cam], s)
    nbytes = cam.width * cam.height * 16
    dev = C.c_void_p()
    ctx.check(L.bsm_device_alloc(ctx.h, nbytes, C.byref(dev)))
    try:
        for call in range(2):
            ctx.check(L.bsm_render_noalloc(ctx.h, sid, C.byref(cam), C.byref(s), dev))
            ctx.sync()
            host = np.zeros((cam.height, cam.width, 4), np.float32)
            ctx.check(L.bsm_memcpy(ctx.h, host.ctypes.data, dev, nbytes, 1))
            assert np.isfinite(host).all()
            err = rel_err(host, ref[0])
            assert err.max() <= RTOL, f"call {call}: max rel err {err.max():.3g}"
            assert np.all(host[..., 3] == 1.0)
    finally:
        L.bsm_device_free(ctx.h, dev)


def test_noalloc_small_chunks_match(bsm, setup):
    """Chunks smaller than the image (many passes over the fixed array) give the same image."""
    ctx, scene, sid = setup
    L = bsm.lib()
    cam = scene.camera
    s = bsm.settings(spp=2, max_segments=3, seed=5, accumulate=0, wavefront_capacity=2048)
    ref, _ = ctx.render(sid, [cam], bsm.settings(spp=2, max_segments=3, seed=5, accumulate=0))
    nbytes = cam.width * cam.height * 16
    dev = C.c_void_p()
    ctx.check(L.bsm_device_alloc(ctx.h, nbytes, C.byref(dev)))
    try:
        ctx.check(L.bsm_render_noalloc(ctx.h, sid, C.byref(cam), C.byref(s), dev))
        ctx.sync()
        host = np.zeros((cam.height, cam.width, 4), np.float32)
        ctx.check(L.bsm_memcpy(ctx.h, host.ctypes.data, dev, nbytes, 1))
        assert rel_err(host, ref[0]).max() <= RTOL
    finally:
        L.bsm_device_free(ctx.h, dev)


def test_noalloc_rejects_chunk_beyond_fixed_array(bsm, setup):
    ctx, scene, sid = setup
    L = bsm.lib()
    cam = scene.camera
    s = bsm.settings(spp=1, max_segments=2, wavefront_capacity=1 << 24)
    dev = C.c_void_p()
    ctx.check(L.bsm_device_alloc(ctx.h, cam.width * cam.height * 16, C.byref(dev)))
    try:
        st = L.bsm_render_noalloc(ctx.h, sid, C.byref(cam), C.byref(s), dev)
        assert st == -1
        assert b"scratch" in L.bsm_last_error(ctx.h)
    finally:
        L.bsm_device_free(ctx.h, dev)


def noalloc_image(bsm, ctx, sid, cam, s):
    """One bsm_render_noalloc call into a fresh device buffer, read back after bsm_sync."""
    L = bsm.lib()
    nbytes = cam.width * cam.height * 16
    dev = C.c_void_p()
    ctx.check(L.bsm_device_alloc(ctx.h, nbytes, C.byref(dev)))
    try:
        ctx.check(L.bsm_render_noalloc(ctx.h, sid, C.byref(cam), C.byref(s), dev))
        ctx.sync()     # reports a queue overflow of the call as BSM_ERR_DEVICE_CHECK
        host = np.zeros((cam.height, cam.width, 4), np.float32)
        ctx.check(L.bsm_memcpy(ctx.h, host.ctypes.data, dev, nbytes, 1))
        return host
    finally:
        L.bsm_device_free(ctx.h, dev)


def translucent_room(bsm):
    sc = bsm.generate_scene(bsm.BSM_SCENE_ROOM, seed=23, width=72, height=56)
    m = np.array(sc.materials, np.float32)
    m[1::3, 5] = 0.4
    m[1::3, 6] = bsm.BSM_BLEND_TRANSLUCENT
    m[2::5, 5] = 0.0
    m[2::5, 6] = bsm.BSM_BLEND_ALPHA_TEST
    sc.materials = m
    return sc


def lit_room(bsm):
    sc = bsm.generate_scene(bsm.BSM_SCENE_ROOM, seed=24, width=72, height=56)
    sc.point_lights = np.array([[0.3, 0.8, 0.4, 1.0, 0.9, 0.8, 2.0, 0.0, 1.0, 0.0, 0.0, 0.0],
                                [0.7, 0.8, 0.6, 0.6, 0.7, 1.2, 2.0, 0.0, 1.0, 0.0, np.cos(0.4), np.cos(0.9)]],
                               np.float32)
    sc.rect_lights = np.array([[0.5, 0.95, 0.5, 1, 0, 0, 0, 0, 1, 0.3, 0.2, 3.0, 3.0, 3.0, 0]], np.float32)
    return sc


@pytest.mark.parametrize("kind", ["non_opaque", "two_level", "multi_light"])
def test_noalloc_scratch_layouts_at_the_largest_chunk(bsm, setup, kind):
    """wavefront_capacity = 0 runs the largest chunk the fixed array holds for the scene's layout (the opacity
    seeds of non-opaque scenes, the two-level kernels, (lights + 1) shadow slots per path)."""
    ctx = setup[0]
    if kind == "non_opaque":
        sc = translucent_room(bsm)
        sid = ctx.load_scene(sc)
    elif kind == "two_level":
        sc = bsm.generate_instanced_scene(seed=6, instances=120, width=72, height=56, sphere_res=10, ground=24)
        sid = ctx.load_instanced(sc)
    else:
        sc = lit_room(bsm)
        sid = ctx.load_scene(sc)
    try:
        cam = sc.camera
        # enough paths for more than one full chunk: the largest chunk runs and is refilled
        s = bsm.settings(spp=96, max_segments=4, seed=31, accumulate=0, wavefront_capacity=0)
        ref, _ = ctx.render(sid, [cam], s)
        for call in range(2):
            host = noalloc_image(bsm, ctx, sid, cam, s)
            err = rel_err(host, ref[0])
            assert err.max() <= RTOL, f"{kind}, call {call}: max rel err {err.max():.3g}"
    finally:
        ctx.release(sid)


def test_noalloc_rejects_a_misaligned_output(bsm, setup):
    ctx, scene, sid = setup
    L = bsm.lib()
    cam = scene.camera
    s = bsm.settings(spp=1, max_segments=2)
    dev = C.c_void_p()
    ctx.check(L.bsm_device_alloc(ctx.h, cam.width * cam.height * 16 + 64, C.byref(dev)))
    try:
        st = L.bsm_render_noalloc(ctx.h, sid, C.byref(cam), C.byref(s), C.c_void_p(dev.value + 4))
        assert st == -1
        assert b"aligned" in L.bsm_last_error(ctx.h)
        bad = bsm.settings(spp=1, max_segments=2, block_size=96)
        assert L.bsm_render_noalloc(ctx.h, sid, C.byref(cam), C.byref(bad), dev) == -1
    finally:
        L.bsm_device_free(ctx.h, dev)
