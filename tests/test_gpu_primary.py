"""Primary-hit outputs on the GPU (bsm_render_primary) and the pass mirror's OutputData.

Depth, the packed G-buffer and hit positions equal the oracle's bit for bit
(same camera ray, same closest hit, same float operations), on host and on
device buffers; the miss mask is where a one-segment render sees the sky; and
PathTracingPass.render returns colour + depth + G-buffer with the reference's
history rules (accumulate over consecutive frames, reset after a gap)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def same_bits(a, b):
    a = np.ascontiguousarray(a, np.float32).view(np.uint32)
    b = np.ascontiguousarray(b, np.float32).view(np.uint32)
    return np.array_equal(a, b)


@pytest.fixture(scope="module", params=["room", "terrain"])
def scene(request, bsm, ctx, oracle):
    if request.param == "room":
        sc = bsm.generate_scene(bsm.BSM_SCENE_ROOM, seed=6, spheres=16, width=80, height=60)
    else:
        sc = bsm.generate_scene(bsm.BSM_SCENE_TERRAIN, seed=3, grid=64, spheres=120, sky_width=128,
                                sky_height=64, width=96, height=54)
    return sc, ctx.load_scene(sc), oracle.OracleScene(sc)


def test_primary_outputs_equal_oracle(bsm, ctx, scene):
    sc, sid, osc = scene
    cam = sc.camera
    for near, far in [(0.01, 10000.0), (0.05, 3.0)]:
        d, g, h = ctx.render_primary(sid, cam, None, near, far)
        do, go, ho = osc.primary(cam.as_array(), near_z=near, far_z=far)
        assert same_bits(h, ho)
        assert same_bits(d, do)
        assert same_bits(g, go)
    assert (h[..., 3] > 0).any()


def test_primary_with_settings_and_device_buffers(bsm, ctx, scene):
    sc, sid, osc = scene
    cam = sc.camera
    s = bsm.settings(ray_length=0.6, t_min=0.05)
    d, g, h = ctx.render_primary(sid, cam, s)
    do, go, ho = osc.primary(cam.as_array(), ray_length=0.6, t_min=0.05)
    assert same_bits(h, ho) and same_bits(d, do) and same_bits(g, go)
    # device outputs: same values
    L = ctx._L
    npix = cam.width * cam.height
    ptrs = []
    for nbytes in [npix * 4] + [npix * 16] * 5:
        p = C.c_void_p()
        ctx.check(L.bsm_device_alloc(ctx.h, nbytes, C.byref(p)))
        ptrs.append(p.value)
    try:
        out = bsm.PrimaryOutput()
        out.depth = ptrs[0]
        for k in range(4):
            out.gbuffer[k] = ptrs[1 + k]
        out.hit_positions = ptrs[5]
        out.location = bsm.BSM_DEVICE
        ctx.check(L.bsm_render_primary(ctx.h, sid, C.byref(cam), C.byref(s), 0.0, 0.0, C.byref(out)))
        dd = np.zeros_like(d)
        hh = np.zeros_like(h)
        g1 = np.zeros_like(g[1])
        ctx.check(L.bsm_memcpy(ctx.h, dd.ctypes.data, ptrs[0], dd.nbytes, 1))
        ctx.check(L.bsm_memcpy(ctx.h, g1.ctypes.data, ptrs[2], g1.nbytes, 1))
        ctx.check(L.bsm_memcpy(ctx.h, hh.ctypes.data, ptrs[5], hh.nbytes, 1))
        assert same_bits(dd, d) and same_bits(g1, g[1]) and same_bits(hh, h)
    finally:
        for p in ptrs:
            L.bsm_device_free(ctx.h, p)


def test_primary_rejects_bad_arguments(bsm, ctx, scene):
    sc, sid, _ = scene
    cam = sc.camera
    with pytest.raises(bsm.BsmError):
        ctx.render_primary(sid, cam, None, 1.0, 0.5)          # near >= far
    bad = bsm.make_camera((0.5, 0.5, -1.0), (0.0, 0.0, 1.0), width=0, height=4)
    with pytest.raises(bsm.BsmError):
        ctx.render_primary(sid, bad)
    with pytest.raises(bsm.BsmError):
        ctx.render_primary(12345, cam)


def test_primary_misses_are_where_the_first_segment_sees_the_sky(bsm, ctx, scene):
    sc, sid, _ = scene
    _, _, h = ctx.render_primary(sid, sc.camera)
    imgs, _ = ctx.render(sid, [sc.camera], bsm.settings(spp=1, max_segments=1, flags=6))
    lit = imgs[0][..., :3].max(-1) > 0.0
    assert np.array_equal(lit, h[..., 3] < 0.0)


def test_path_tracing_pass_output_data_and_history(bsm, ctx):
    sc = bsm.generate_scene(bsm.BSM_SCENE_ROOM, seed=8, spheres=10, width=48, height=40)
    pt = bsm.PathTracingPass(ctx, sc)
    ps = bsm.PathTracingSettings(max_bounces=4, spp=1, seed=3, accumulate=True)
    f1 = pt.render(sc.camera, ps)
    assert f1.color.shape == (40, 48, 4) and f1.depth.shape == (40, 48) and f1.velocity is None
    assert f1.gbuffer.base_color.shape == (40, 48, 4) and f1.gbuffer.material_0.shape == (40, 48, 4)
    f2 = pt.render(sc.camera, ps)                 # consecutive frame: running mean of two samples
    two, _ = ctx.render(pt.scene_id, [sc.camera], bsm.settings(spp=2, max_bounces=4, seed=3))
    assert np.abs(f2.color - two[0]).max() <= 1e-4 * max(1.0, float(np.abs(two[0]).max()))
    # a gap resets the history: the same samples as the first frame (sums of a pixel's
    # contributions may be added in another order)
    f5 = pt.render(sc.camera, ps, frame_index=pt.frame + 3)
    assert np.abs(f5.color - f1.color).max() <= 1e-5 * max(1.0, float(np.abs(f1.color).max()))
    assert np.array_equal(f5.depth, f1.depth)
    off = bsm.PathTracingSettings(max_bounces=4, spp=1, seed=3, accumulate=False)
    f6 = pt.render(sc.camera, off)                # accumulate off: this frame only
    assert np.abs(f6.color - f1.color).max() <= 1e-5 * max(1.0, float(np.abs(f1.color).max()))
