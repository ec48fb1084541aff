"""Non-opaque materials on the GPU: the any-hit rule of rt_gbuffer_hit.hlsl:20-35.

* renders with translucent and alpha-tested materials take the same paths as
  the oracle (per-segment ray counts equal, radiance within 1e-4);
* alpha-tested surfaces below the threshold are invisible to closest- and
  any-hit rays, above it they are opaque;
* a translucent quad of opacity a in front of an opaque one stops a fraction a
  of the rays (the per-ray uniform is uniform), in the oracle and on the GPU
  with the same decisions ray by ray."""
import numpy as np
import pytest

from conftest import assert_bits_equal

pytestmark = pytest.mark.gpu


def quads_scene(bsm, front_opacity, front_blend):
    # front quad z = 0.5 (material 0), back quad z = 1.0 (material 1), both over [0, 1]^2
    pos = np.array([[0, 0, .5], [1, 0, .5], [1, 1, .5], [0, 1, .5],
                    [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], np.float32)
    idx = np.array([[0, 1, 2], [0, 2, 3], [4, 5, 6], [4, 6, 7]], np.uint32)
    mats = np.array([[0.8, 0.8, 0.8, 0.5, 0.0, front_opacity, front_blend],
                     [0.5, 0.5, 0.5, 0.5, 0.0, 1.0, 0]], np.float32)
    lights = np.array([[0.3, 0.4, -1.0, 2.0, 2.0, 2.0]], np.float32)
    cam = bsm.make_camera((0.5, 0.5, -1.0), (0.0, 0.0, 1.0), yfov_deg=40.0, width=64, height=64)
    return bsm.SceneData(pos, idx, np.array([0, 0, 1, 1], np.uint32), mats, lights, bsm.BSM_SKY_CONSTANT,
                         (0.3, 0.3, 0.3), None, cam)


def rays_through(n, seed):
    rng = np.random.default_rng(seed)
    r = np.zeros((n, 8), np.float32)
    r[:, 0:2] = rng.uniform(0.2, 0.8, (n, 2))
    r[:, 2] = 0.0
    d = np.c_[rng.normal(0, 0.05, (n, 2)), np.ones(n)]
    r[:, 4:7] = d / np.linalg.norm(d, axis=1, keepdims=True)
    r[:, 7] = 10.0
    return r


@pytest.mark.parametrize("opacity", [0.3, 0.75])
def test_translucent_quad_stops_its_opacity(bsm, ctx, oracle, opacity):
    sc = quads_scene(bsm, opacity, bsm.BSM_BLEND_TRANSLUCENT)
    sid = ctx.load_scene(sc)
    rays = rays_through(40000, 1)
    h = ctx.trace_closest(sid, rays)
    ho = oracle.OracleScene(sc).trace(rays)
    assert np.array_equal(h[:, 1], ho[:, 1]) and np.array_equal(h[:, 0], ho[:, 0])
    front = np.mean(h[:, 1] < 2)
    assert abs(front - opacity) < 0.015, front
    occ = ctx.trace_any(sid, rays)
    assert occ.all()                               # the back quad is opaque
    ctx.release(sid)


def test_alpha_test_threshold(bsm, ctx, oracle):
    rays = rays_through(5000, 2)
    for opacity, visible in [(0.005, False), (0.5, True)]:
        sc = quads_scene(bsm, opacity, bsm.BSM_BLEND_ALPHA_TEST)
        sid = ctx.load_scene(sc)
        h = ctx.trace_closest(sid, rays)
        assert np.all((h[:, 1] < 2) == visible)
        assert np.array_equal(h, oracle.OracleScene(sc).trace(rays))
        ctx.release(sid)


def test_render_with_non_opaque_materials_equals_oracle(bsm, ctx, oracle):
    sc = bsm.generate_scene(bsm.BSM_SCENE_ROOM, seed=12, spheres=24, width=48, height=40)
    m = np.concatenate([sc.materials, np.ones((len(sc.materials), 1)), np.zeros((len(sc.materials), 1))], 1)
    rng = np.random.default_rng(3)
    pick = rng.permutation(len(m))
    m[pick[: len(m) // 3], 5] = rng.uniform(0.2, 0.8, len(m) // 3)
    m[pick[: len(m) // 3], 6] = bsm.BSM_BLEND_TRANSLUCENT
    m[pick[len(m) // 3: len(m) // 2], 5] = 0.0
    m[pick[len(m) // 3: len(m) // 2], 6] = bsm.BSM_BLEND_ALPHA_TEST
    sc.materials = m.astype(np.float32)
    sid = ctx.load_scene(sc)
    osc = oracle.OracleScene(sc)
    for flags in (0, 1):
        imgs, st = ctx.render(sid, [sc.camera], bsm.settings(spp=3, max_segments=5, seed=4, flags=flags))
        ref, ost, _ = osc.render(sc.camera.as_array(), spp=3, max_segments=5, seed=4, flags=flags)
        assert [int(x) for x in st.rays_per_segment[:5]] == [int(x) for x in ost[:5]]
        assert int(st.shadow_rays) == int(ost[16:32].sum())
        g = imgs[0][..., :3].astype(np.float64)
        o = ref[..., :3].astype(np.float64)
        assert (np.abs(g - o) / np.maximum(np.abs(o), 1e-3)).max() <= 1e-4
        det = flags | bsm.BSM_PT_DETERMINISTIC   # fixed-point sums on both sides: equal bit for bit
        imgs, _ = ctx.render(sid, [sc.camera], bsm.settings(spp=3, max_segments=5, seed=4, flags=det))
        ref, _, _ = osc.render(sc.camera.as_array(), spp=3, max_segments=5, seed=4, flags=det)
        assert_bits_equal(imgs[0], ref)
    d, gb, hp = ctx.render_primary(sid, sc.camera, bsm.settings(seed=4))
    do, go, ho = osc.primary(sc.camera.as_array(), seed=4)
    assert np.array_equal(hp.view(np.uint32), ho.view(np.uint32))
    assert np.array_equal(gb.view(np.uint32), go.view(np.uint32))
    ctx.release(sid)
