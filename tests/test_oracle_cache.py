"""The oracle's cached pass (the reference for bsm_render_cached without training): its paths are the plain
pass's up to the cache vertex, a zero network adds nothing there, and a network's terms are non-negative."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def room(bsm, oracle):
    scene = bsm.generate_scene(bsm.BSM_SCENE_ROOM, seed=41, spheres=24)
    cam = bsm.make_camera(tuple(scene.camera.position), tuple(scene.camera.front), width=40, height=30)
    return oracle.OracleScene(scene), cam.as_array()


def test_paths_agree_with_the_plain_pass_up_to_the_cache_vertex(room):
    osc, cam = room
    W = np.zeros(16896, np.float32)
    cached, cst = osc.render_cached(cam, spp=2, weights=W, cache_segment=2, seed=3)
    plain, pst, _ = osc.render(cam, spp=2, max_segments=3, seed=3)
    assert [int(x) for x in cst[:3]] == [int(x) for x in pst[:3]]
    # a zero network ends paths at their segment-2 hits with nothing; the plain pass adds those hits' direct light
    assert (cached[..., :3] <= plain[..., :3] + 1e-6).all()
    assert cached[..., :3].sum() < plain[..., :3].sum()
    # a shadow-ray count of zero at segment 2: cache vertices shoot none
    assert int(cst[16 + 2]) == 0 and int(pst[16 + 2]) > 0


def test_network_terms_are_non_negative(room):
    osc, cam = room
    rng = np.random.default_rng(4)
    W = rng.normal(0.0, 0.15, 16896).astype(np.float32)
    W[4 * 4096 + 3 * 64:] = 0.0
    zero, _ = osc.render_cached(cam, spp=2, weights=np.zeros_like(W), cache_segment=2, seed=3)
    with_net, _ = osc.render_cached(cam, spp=2, weights=W, cache_segment=2, seed=3)
    assert (with_net[..., :3] >= zero[..., :3] - 1e-6).all()
    assert with_net[..., :3].sum() > zero[..., :3].sum()


def test_smooth_hits_continue_with_extra_segments(room):
    osc, cam = room
    W = np.zeros(16896, np.float32)
    _, st0 = osc.render_cached(cam, spp=2, weights=W, cache_segment=2, seed=3)
    _, st1 = osc.render_cached(cam, spp=2, weights=W, cache_segment=2, extra_segments=2, min_roughness=0.5, seed=3)
    assert int(st0[3]) == 0 and int(st1[3]) > 0       # smooth segment-2 hits continued
    assert int(st1[5]) == 0                            # nothing goes past the last allowed segment
