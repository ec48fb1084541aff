"""The render boundary is asynchronous on a caller's stream.

The reference's PathTracingPass::render only records passes; they run later,
when the render graph executes on the engine's command encoder
(bisemutum/src/graphics/graphics_manager.cpp:418-419).  The C ABI mirrors that:
after bsm_set_stream(ctx, stream) a render whose outputs stay on the device
queues its kernels on that stream and returns before the GPU has finished; the
caller synchronises (bsm_sync) when it needs the result.  These tests check
that two renders issued back to back on a caller stream return while the
stream is still busy, that both images equal a synchronous render's after
bsm_sync, that statistics come back through bsm_render_stats_read, and that
work queued before a stream switch stays ordered before work queued after it."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

RTOL = 1e-4


def rel_err(g, c):
    g = g[..., :3].astype(np.float64)
    c = c[..., :3].astype(np.float64)
    return np.abs(g - c) / np.maximum(np.abs(c), 1e-3)


@pytest.fixture(scope="module")
def env(bsm):
    ctx = bsm.Context(0)
    sc = bsm.generate_scene(bsm.BSM_SCENE_TERRAIN, seed=3, grid=256, spheres=300, sky_width=256, sky_height=128,
                            width=960, height=540)
    sid = ctx.load_scene(sc)
    yield ctx, sc, sid
    ctx.set_stream(None)
    ctx.close()


def device_buffer(bsm, ctx, nbytes):
    p = C.c_void_p()
    ctx.check(bsm.lib().bsm_device_alloc(ctx.h, nbytes, C.byref(p)))
    return p


def test_two_renders_on_caller_stream_return_before_the_gpu_finishes(bsm, env):
    ctx, sc, sid = env
    L = bsm.lib()
    cam = sc.camera
    s = bsm.settings(spp=16, max_segments=8, seed=21, accumulate=0)
    ref, _ = ctx.render(sid, [cam], s)          # synchronous render on the context's own stream
    stream = torch.cuda.Stream(device=0)
    ctx.set_stream(stream.cuda_stream)
    assert L.bsm_get_stream(ctx.h) == stream.cuda_stream
    nbytes = cam.width * cam.height * 16
    bufs = [device_buffer(bsm, ctx, nbytes) for _ in range(2)]
    try:
        outs = []
        for b in bufs:
            o = (bsm.ViewOutput * 1)()
            o[0].rgba = b.value
            o[0].location = bsm.BSM_DEVICE
            outs.append(o)
        cams = (bsm.Camera * 1)(cam)
        ctx.check(L.bsm_render(ctx.h, sid, cams, 1, C.byref(s), outs[0], None))   # first: graph capture
        ctx.sync()
        ctx.check(L.bsm_render(ctx.h, sid, cams, 1, C.byref(s), outs[0], None))
        ctx.check(L.bsm_render(ctx.h, sid, cams, 1, C.byref(s), outs[1], None))
        busy = not stream.query()
        ctx.sync()
        assert stream.query()
        assert busy, "bsm_render returned after its work had finished: it did not run asynchronously"
        for b in bufs:
            host = np.zeros((cam.height, cam.width, 4), np.float32)
            ctx.check(L.bsm_memcpy(ctx.h, host.ctypes.data, b, nbytes, 1))
            assert rel_err(host, ref[0]).max() <= RTOL
        st = ctx.last_stats()
        assert st.paths == cam.width * cam.height * 16
        assert st.extend_rays > st.paths
    finally:
        ctx.set_stream(None)
        for b in bufs:
            L.bsm_device_free(ctx.h, b)


def test_stats_read_waits_for_an_async_render(bsm, env):
    ctx, sc, sid = env
    cam = sc.camera
    s = bsm.settings(spp=4, max_segments=8, seed=5, accumulate=0)
    _, st_sync = ctx.render(sid, [cam], s, outputs=False, stats=True)
    ctx.render(sid, [cam], s, outputs=False, stats=False)    # returns at once
    st = ctx.last_stats()
    assert list(st.rays_per_segment) == list(st_sync.rays_per_segment)
    assert st.shadow_rays == st_sync.shadow_rays
    assert st.ms_total > 0.0


def test_work_keeps_its_order_across_a_stream_switch(bsm, env):
    """A render queued on the context's stream, then the switch to a caller stream and a history read on
    it: the read sees the finished render."""
    ctx, sc, sid = env
    cam = sc.camera
    s = bsm.settings(spp=4, max_segments=4, seed=8, accumulate=0)
    ref, _ = ctx.render(sid, [cam], s)
    ctx.render(sid, [cam], s, outputs=False, stats=False)
    stream = torch.cuda.Stream(device=0)
    ctx.set_stream(stream.cuda_stream)
    try:
        img = np.zeros((cam.height, cam.width, 4), np.float32)
        o = bsm.ViewOutput()
        o.rgba = img.ctypes.data
        o.location = bsm.BSM_HOST
        ctx.check(bsm.lib().bsm_read_view(ctx.h, 0, C.byref(o)))
        assert rel_err(img, ref[0]).max() <= RTOL
    finally:
        ctx.set_stream(None)
