"""Radiance cache on the GPU.

* the fused BF16 tensor-core forward and the training kernel's gradients against
  the CPU oracle of the same network (same bf16 rounding points; sums in another
  order), one Adam step against the oracle's Adam;
* training on tracer-style samples lowers the loss; weights save and load;
* the gain of the trained cache: with paths ending at their third vertex,
  finishing them with the trained network is closer to a high-spp reference
  (relMSE) than ending them without it."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def random_samples(n, seed):
    rng = np.random.default_rng(seed)
    s = np.zeros((n, 16), np.float32)
    s[:, :12] = rng.uniform(0.0, 1.0, (n, 12))
    s[:, 12:15] = rng.uniform(0.0, 2.0, (n, 3))
    return s


@pytest.fixture(scope="module")
def cache(bsm, ctx):
    c = bsm.RadianceCache(ctx, seed=7)
    yield c
    c.close()


def test_forward_matches_oracle(cache, oracle):
    S = random_samples(1000, 1)
    W = cache.weights()
    g = cache.predict(S)
    o = oracle.mlp_forward(W, S, bf16=True)
    scale = float(np.abs(o).max())
    assert np.abs(g - o).max() <= 1e-2 * scale + 1e-5
    assert np.median(np.abs(g - o)) <= 1e-3 * scale


@pytest.mark.parametrize("n", [1, 127, 128, 129, 4097, 100_000])
def test_forward_sizes_match_oracle(cache, oracle, n):
    """Partial and multiple 128-query tiles of the tensor-core forward (several tiles per CTA at 100,000)."""
    S = random_samples(n, 10 + n % 97)
    W = cache.weights()
    g = cache.predict(S)
    o = oracle.mlp_forward(W, S, bf16=True)
    scale = float(np.abs(o).max())
    assert g.shape == o.shape
    assert np.abs(g - o).max() <= 1e-2 * scale + 1e-5


@pytest.mark.parametrize("n", [1, 64, 129, 20_000])
def test_gradient_sizes_match_oracle(cache, oracle, n):
    """One sample, part of one 128-sample tile, a full tile and one row of a second, and more tiles than SMs
    (so that CTAs of the training kernel take several tiles and reduce their gradients on the last)."""
    S = random_samples(n, 20 + n % 89)
    W = cache.weights()
    dg, lg = cache.gradient(S)
    do, lo = oracle.mlp_gradient(W, S, bf16=True)
    assert abs(lg - lo) <= 1e-3 * abs(lo)
    x, y = dg.astype(np.float64), do.astype(np.float64)
    assert float(x @ y / (np.linalg.norm(x) * np.linalg.norm(y))) > 0.999
    assert np.abs(x - y).max() <= 2e-2 * np.abs(y).max()


def test_gradient_matches_oracle(cache, oracle):
    S = random_samples(777, 2)     # not a multiple of the 16-row tile
    W = cache.weights()
    dg, lg = cache.gradient(S)
    do, lo = oracle.mlp_gradient(W, S, bf16=True)
    assert abs(lg - lo) <= 1e-3 * abs(lo)
    blocks = [(0, 4096), (4096, 8192), (8192, 12288), (12288, 16384), (16384, 16384 + 192)]
    for a, b in blocks:
        x, y = dg[a:b].astype(np.float64), do[a:b].astype(np.float64)
        assert np.abs(x - y).max() <= 2e-2 * np.abs(y).max(), (a, np.abs(x - y).max(), np.abs(y).max())
        cos = float(x @ y / (np.linalg.norm(x) * np.linalg.norm(y)))
        assert cos > 0.999, (a, cos)
    assert np.all(dg[16384 + 192:] == 0.0)


def test_adam_step_matches_oracle(cache, oracle):
    W0 = cache.weights()
    cache.weights(W0)              # resets the Adam state
    S = random_samples(512, 3)
    dg, _ = cache.gradient(S)
    cache.train(S, batch=512, lr=1e-2)
    W1 = cache.weights()
    W1o, _, _ = oracle.mlp_adam(W0, dg, np.zeros_like(W0), np.zeros_like(W0), 1e-2, 1)
    ok = np.abs(dg) > 1e-6         # the first Adam step is lr * sign(g): skip gradients at the noise floor
    assert np.abs(W1[ok] - W1o[ok]).max() <= 1e-5
    assert np.all(W1[16384 + 192:] == 0.0)


def test_training_lowers_loss(bsm, ctx):
    c = bsm.RadianceCache(ctx, seed=11)
    try:
        S = random_samples(8192, 4)
        # smooth target: radiance depending on position and normal
        S[:, 12] = 0.5 + 0.4 * np.sin(3.0 * S[:, 0]) * S[:, 6]
        S[:, 13] = 0.3 + 0.3 * S[:, 1] * S[:, 8]
        S[:, 14] = 0.2 + 0.5 * S[:, 2] ** 2
        first = c.train(S, batch=8192, lr=1e-2)
        for _ in range(60):
            last = c.train(S, batch=8192, lr=1e-2)
        assert last < 0.25 * first, (first, last)
    finally:
        c.close()


def test_save_load_roundtrip(bsm, ctx, cache, tmp_path):
    path = str(tmp_path / "cache.bin")
    W = cache.weights()
    cache.save(path)
    other = bsm.RadianceCache(ctx, seed=99)
    try:
        other.load(path)
        assert np.array_equal(other.weights(), W)
        S = random_samples(100, 5)
        assert np.array_equal(other.predict(S), cache.predict(S))
    finally:
        other.close()


def test_trained_cache_beats_the_plain_tracer_at_equal_device_time(bsm, ctx):
    """The gain the learned part brings over the method without it: the plain full-length tracer.  In the
    room scene (light reaches most points over several bounces) the cache, trained online for 60 frames,
    renders frames whose device time (training step included) is at most the plain pass's, with a lower relMSE
    against a 1024-spp plain render: untrimmed, averaged over three seeds."""
    scene = bsm.generate_scene(bsm.BSM_SCENE_ROOM, seed=41, spheres=24)
    sid = ctx.load_scene(scene)
    cam = bsm.make_camera(tuple(scene.camera.position), tuple(scene.camera.front), width=256, height=256)
    ctx.render(sid, [cam], bsm.settings(spp=256, max_segments=8, seed=1000, accumulate=0), outputs=False)
    for k in range(3):
        refs, _ = ctx.render(sid, [cam], bsm.settings(spp=256, max_segments=8, seed=1000, accumulate=1),
                             outputs=k == 2)
    ref = refs[0]
    c = bsm.RadianceCache(ctx, seed=5)
    try:
        cs = bsm.cache_settings(cache_segment=2)
        for f in range(60):
            c.render(sid, cam, bsm.settings(spp=1, seed=f + 1), cs, outputs=False)
        seeds = (77, 177, 277)

        def plain(spp):
            out = [ctx.render(sid, [cam], bsm.settings(spp=spp, max_segments=8, seed=sd)) for sd in seeds]
            return np.mean([bsm.rel_mse(im[0], ref) for im, _ in out]), np.mean([st.ms_total for _, st in out])

        def cached(spp):
            out = [c.render(sid, cam, bsm.settings(spp=spp, seed=sd), cs) for sd in seeds]   # trains, then renders
            return np.mean([bsm.rel_mse(im, ref) for im, _, _ in out]), np.mean([st.ms_total for _, st, _ in out])

        plain(16)
        e_plain, t_plain = plain(16)
        spp_c, e_c, t_c = None, None, None
        for spp in (4, 8, 16, 32):
            cached(spp)
            e, t = cached(spp)
            if t <= t_plain:
                spp_c, e_c, t_c = spp, e, t
        assert spp_c is not None, ("no cached frame as fast as the plain one", t_plain)
        assert e_c < e_plain, (spp_c, e_c, t_c, e_plain, t_plain)
    finally:
        c.close()
    ctx.release(sid)


def test_smooth_hits_continue_past_the_cache_segment(bsm, ctx):
    """min_roughness / extra_segments: hits of the cache segment smoother than the threshold shade and
    continue; the last allowed segment queries the cache whatever its roughness, so no path goes further."""
    scene = bsm.generate_scene(bsm.BSM_SCENE_ROOM, seed=41, spheres=24)
    sid = ctx.load_scene(scene)
    cam = bsm.make_camera(tuple(scene.camera.position), tuple(scene.camera.front), width=64, height=64)
    c = bsm.RadianceCache(ctx, seed=6)
    try:
        base = bsm.cache_settings(cache_segment=2, train_steps=0)
        _, st0, _ = c.render(sid, cam, bsm.settings(spp=4, seed=3), base)
        assert st0.rays_per_segment[3] == 0
        gated = bsm.cache_settings(cache_segment=2, train_steps=0, min_roughness=0.5, extra_segments=2)
        img, st1, _ = c.render(sid, cam, bsm.settings(spp=4, seed=3), gated)
        assert list(st1.rays_per_segment[:3]) == list(st0.rays_per_segment[:3])   # same prefix
        assert st1.rays_per_segment[3] > 0 and st1.rays_per_segment[5] == 0
        assert np.isfinite(img).all()
    finally:
        c.close()
    ctx.release(sid)


def test_renders_read_the_corrected_moving_average(bsm, ctx):
    """With ema_decay d the weights renders read are e_k / (1 - d^k), e_k = d e_(k-1) + (1 - d) w_k over the
    master weights w_k after each Adam step (e_0 = 0); before any averaged step they are the master weights."""
    scene = bsm.generate_scene(bsm.BSM_SCENE_ROOM, seed=41, spheres=8)
    sid = ctx.load_scene(scene)
    cam = bsm.make_camera(tuple(scene.camera.position), tuple(scene.camera.front), width=32, height=32)
    c = bsm.RadianceCache(ctx, seed=9)
    try:
        d = 0.9
        cs = bsm.cache_settings(train_paths=4096, train_batch=8192, train_steps=1, cache_segment=2, ema_decay=d)
        assert np.array_equal(c.render_weights(), c.weights())
        e = np.zeros(c.nparams, np.float64)
        for k in range(1, 7):
            c.render(sid, cam, bsm.settings(spp=1, seed=k), cs, outputs=False)
            e = d * e + (1.0 - d) * c.weights().astype(np.float64)
            np.testing.assert_allclose(c.render_weights(), e / (1.0 - d ** k), rtol=2e-5, atol=2e-7)
        # a cache whose weights are set again renders with them until it trains
        w = c.weights()
        c.weights(w)
        assert np.array_equal(c.render_weights(), w)
    finally:
        c.close()
    ctx.release(sid)


def test_cached_render_as_the_first_call_of_a_context(bsm):
    """bsm_render_cached on a context that has rendered nothing before: its training paths' shadow pass launches
    with the configuration the render sets up, and the frame agrees with the same frame on a context that
    rendered a plain frame first (same seeds, fresh caches with the same start weights; the training step's
    gradient sums run in another order, so the two trained networks differ in the last bits)."""
    scene = bsm.generate_scene(bsm.BSM_SCENE_ROOM, seed=41, spheres=24)
    cam = bsm.make_camera(tuple(scene.camera.position), tuple(scene.camera.front), width=64, height=48)
    cs = bsm.cache_settings(cache_segment=2, train_paths=2048, train_batch=4096, train_steps=1)
    images = []
    for warm in (False, True):
        c2 = bsm.Context(0)
        try:
            sid = c2.load_scene(scene)
            if warm:
                c2.render(sid, [cam], bsm.settings(spp=1, max_segments=4, seed=3), outputs=False)
            cache = bsm.RadianceCache(c2, seed=5)
            try:
                img, st, loss = cache.render(sid, cam, bsm.settings(spp=2, seed=9), cs)
                assert st.extend_rays > 0 and np.isfinite(loss)
                images.append(img)
            finally:
                cache.close()
        finally:
            c2.close()
    a, b = images[0][..., :3].astype(np.float64), images[1][..., :3].astype(np.float64)
    assert np.isfinite(a).all() and np.isfinite(b).all()
    assert np.abs(a - b).mean() <= 1e-2 * np.abs(b).mean()


def test_online_training_is_bit_reproducible(bsm, ctx):
    """Two caches from the same seed, trained online by the same cached frames, end with the same weights and
    render the same images bit for bit: the training paths' shadow pass sums each vertex's radiance exactly,
    the samples sit at offsets from a scan of the per-path counts, and Adam sums the training kernel's per-CTA
    gradient slots in a fixed order (the frames sum in fixed point too: BSM_PT_DETERMINISTIC)."""
    scene = bsm.generate_scene(bsm.BSM_SCENE_ROOM, seed=41, spheres=24)
    sid = ctx.load_scene(scene)
    cam = bsm.make_camera(tuple(scene.camera.position), tuple(scene.camera.front), width=64, height=48)
    cs = bsm.cache_settings(cache_segment=2, train_paths=20000, train_steps=2, train_batch=8192)
    s = bsm.settings(spp=2, seed=9, flags=bsm.BSM_PT_DETERMINISTIC)
    runs = []
    try:
        for _ in range(2):
            c = bsm.RadianceCache(ctx, seed=5)
            try:
                w0 = c.weights().copy()
                frames = [c.render(sid, cam, s, cs)[0] for _ in range(3)]
                runs.append((w0, c.weights().copy(), frames))
            finally:
                c.close()
    finally:
        ctx.release(sid)
    (w0, wa, fa), (_, wb, fb) = runs
    assert not np.array_equal(w0, wa), "no training happened"
    assert np.array_equal(wa.view(np.uint32), wb.view(np.uint32))
    for x, y in zip(fa, fb):
        assert x[..., :3].mean() > 0.0
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32))


@pytest.mark.parametrize("extra, min_rough", [(0, 0.0), (2, 0.5)])
def test_cached_render_matches_oracle(bsm, ctx, oracle, extra, min_rough):
    """The cached pass without its training step (bsm_render_cached, train_steps = 0) against the oracle's
    cached pass with the same network weights: the paths agree up to their cache vertex (equal rays per
    segment), and the radiance agrees within the network's tolerance.  The cache-vertex terms differ only by
    the two networks' arithmetic (BF16 products with sums in another order; the encoding's base sine and
    cosine from the special-function unit on the GPU, which can move a BF16 feature by one step).  With
    extra segments, hits smoother than min_roughness shade and continue, and the last segment queries."""
    scene = bsm.generate_scene(bsm.BSM_SCENE_ROOM, seed=41, spheres=24)
    sid = ctx.load_scene(scene)
    cam = bsm.make_camera(tuple(scene.camera.position), tuple(scene.camera.front), width=64, height=48)
    c = bsm.RadianceCache(ctx, seed=5)
    try:
        W = c.weights()
        cs = bsm.cache_settings(cache_segment=2, train_steps=0, extra_segments=extra, min_roughness=min_rough)
        img, st, _ = c.render(sid, cam, bsm.settings(spp=4, seed=9), cs)
        ref, ost = oracle.OracleScene(scene).render_cached(cam.as_array(), spp=4, weights=W, cache_segment=2,
                                                            extra_segments=extra, min_roughness=min_rough, seed=9)
        segs = 3 + extra
        assert [int(x) for x in st.rays_per_segment[:segs]] == [int(x) for x in ost[:segs]]
        g, o = img[..., :3].astype(np.float64), ref[..., :3].astype(np.float64)
        assert o.mean() > 0.0
        err = np.abs(g - o)
        assert err.max() <= 2e-2 * max(float(np.abs(o).max()), 1e-3)
        assert np.median(err / np.maximum(np.abs(o), 1e-3 * o.mean())) <= 1e-3
    finally:
        c.close()
        ctx.release(sid)
