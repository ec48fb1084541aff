"""Failure handling on the host side, with no fault on the GPU.

* bsm_sync returns BSM_ERR_TIMEOUT when its limit runs out before the work
  ends (the work keeps running; a later sync without a limit succeeds and the
  image is right).
* bsm_server_wait returns BSM_ERR_TIMEOUT for a request still running.
* bsm_server_cancel: a queued request is dropped without running; a running
  one stops issuing paths, gives its accumulator back to the pool and its
  output is never written; other requests are unaffected.
* An allocation refused by the context's allocator (a memory budget smaller
  than the wavefront a render asks for) fails the call with
  BSM_ERR_OUT_OF_MEMORY and leaves the context usable."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

BSM_ERR_TIMEOUT, BSM_ERR_OUT_OF_MEMORY, BSM_ERR_CANCELLED = -4, -2, -11


@pytest.fixture(scope="module")
def terrain(bsm):
    ctx = bsm.Context(0)
    sc = bsm.generate_scene(bsm.BSM_SCENE_TERRAIN, seed=5, grid=256, spheres=300, sky_width=256, sky_height=128,
                            width=1920, height=1080)
    sid = ctx.load_scene(sc)
    yield ctx, sc, sid
    ctx.close()


def test_sync_times_out_then_completes(bsm, terrain):
    ctx, sc, sid = terrain
    L = bsm.lib()
    s = bsm.settings(spp=32, max_segments=8, seed=2, accumulate=0)
    ref, _ = ctx.render(sid, [sc.camera], s)
    ctx.render(sid, [sc.camera], s, outputs=False, stats=False)   # queued: about 0.1 s of GPU work
    assert L.bsm_sync(ctx.h, 1) == BSM_ERR_TIMEOUT
    assert b"timed out" in L.bsm_last_error(ctx.h)
    ctx.sync()
    img = np.zeros((sc.camera.height, sc.camera.width, 4), np.float32)
    o = bsm.ViewOutput()
    o.rgba = img.ctypes.data
    o.location = bsm.BSM_HOST
    ctx.check(L.bsm_read_view(ctx.h, 0, C.byref(o)))
    err = np.abs(img[..., :3] - ref[0][..., :3]) / np.maximum(np.abs(ref[0][..., :3]), 1e-3)
    assert err.max() <= 1e-4


def test_server_wait_times_out_and_cancel(bsm, terrain):
    ctx, sc, sid = terrain
    L = bsm.lib()
    cam = sc.camera
    px = cam.width * cam.height
    # one lane and a pool that holds one full-frame accumulator: the second request queues
    ctx.server_start(pool_bytes=px * 16, chunk_paths=1 << 20, lanes=1)
    try:
        big, big_out = ctx.submit(sid, cam, 64, 8, 1)          # ~130 M paths in 1 M-path chunks
        queued, q_out = ctx.submit(sid, cam, 1, 2, 2)          # waits for the pool
        big_out[...] = -7.0
        q_out[...] = -7.0
        st = bsm.RequestStatus()
        assert L.bsm_server_wait(ctx.h, big, 1, C.byref(st)) == BSM_ERR_TIMEOUT
        assert st.state in (bsm.BSM_REQ_RUNNING, bsm.BSM_REQ_QUEUED)
        # the queued request is dropped at once
        ctx.cancel(queued)
        assert ctx.poll(queued).state == bsm.BSM_REQ_CANCELLED
        assert L.bsm_server_wait(ctx.h, queued, 0, C.byref(st)) == BSM_ERR_CANCELLED
        # the running one stops issuing chunks
        ctx.cancel(big)
        assert L.bsm_server_wait(ctx.h, big, 60000, C.byref(st)) == BSM_ERR_CANCELLED
        assert st.cancelled == 1 and st.state == bsm.BSM_REQ_CANCELLED
        assert (big_out == -7.0).all() and (q_out == -7.0).all(), "a cancelled request's output was written"
        stats = ctx.server_stats()
        assert stats.cancelled == 2
        assert stats.pool_used_bytes == 0
        # the server keeps serving: a new request fits the freed pool and completes
        rid, out = ctx.submit(sid, bsm.make_camera(tuple(cam.position), tuple(cam.front), width=320, height=180),
                              4, 4, 3)
        st2 = ctx.wait(rid, timeout_ms=60000)
        assert st2.state == bsm.BSM_REQ_DONE
        assert np.isfinite(out).all() and out[..., :3].mean() > 0.0
        assert ctx.server_stats().extend_rays < 64 * px, "the cancelled request ran to the end"
    finally:
        ctx.server_stop()


def test_allocation_refused_by_the_budget(bsm):
    """A context whose budget cannot hold the requested wavefront: the render fails cleanly and the
    context renders again with a wavefront that fits."""
    sc = bsm.generate_scene(bsm.BSM_SCENE_ROOM, seed=3, width=64, height=64)
    with bsm.Context(0, budget_bytes=256 << 20) as ctx:
        sid = ctx.load_scene(sc)
        L = bsm.lib()
        s_big = bsm.settings(spp=8, max_segments=4, seed=1, wavefront_capacity=1 << 24)   # ~5 GB of queues
        cams = (bsm.Camera * 1)(sc.camera)
        st = L.bsm_render(ctx.h, sid, cams, 1, C.byref(s_big), None, None)
        assert st == BSM_ERR_OUT_OF_MEMORY
        assert b"budget" in L.bsm_last_error(ctx.h)
        p = C.c_void_p()
        assert L.bsm_device_alloc(ctx.h, 1 << 30, C.byref(p)) == BSM_ERR_OUT_OF_MEMORY
        imgs, rs = ctx.render(sid, [sc.camera], bsm.settings(spp=8, max_segments=4, seed=1, wavefront_capacity=4096))
        ref, _ = ctx.render(sid, [sc.camera], bsm.settings(spp=8, max_segments=4, seed=1))
        assert rs.chunks > 1
        err = np.abs(imgs[0][..., :3] - ref[0][..., :3]) / np.maximum(np.abs(ref[0][..., :3]), 1e-3)
        assert err.max() <= 1e-4
