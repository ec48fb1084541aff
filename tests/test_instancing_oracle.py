"""Two-level scenes in the oracle (no GPU).

The oracle traces every instance with the ray moved into its object space; its
closest hits must name the same global primitives as the same scene flattened
into one world-space mesh (t agrees to float rounding of the two spaces), and a
render of both takes the same path decisions."""
import numpy as np


def random_world_rays(n, seed):
    rng = np.random.default_rng(seed)
    r = np.zeros((n, 8), np.float32)
    r[:, 0:3] = rng.uniform(-3.0, 3.0, (n, 3))
    r[:, 1] = rng.uniform(0.2, 2.0, n)
    d = rng.normal(size=(n, 3))
    r[:, 4:7] = d / np.linalg.norm(d, axis=1, keepdims=True)
    r[:, 7] = 50.0
    return r


def test_instanced_hits_equal_flattened_scene(bsm, oracle):
    sc = bsm.generate_instanced_scene(seed=2, instances=60, width=32, height=24, sphere_res=8, ground=16)
    osc = oracle.OracleScene(sc)
    ofl = oracle.OracleScene(sc.flattened())
    rays = random_world_rays(20000, 1)
    h, hf = osc.trace(rays), ofl.trace(rays)
    assert np.mean(h[:, 1] != 0xFFFFFFFF) > 0.2
    agree = np.mean(h[:, 1] == hf[:, 1])
    assert agree > 0.999, agree                     # edge-grazing rays may differ across the two spaces
    hit = (h[:, 1] != 0xFFFFFFFF) & (h[:, 1] == hf[:, 1])
    t, tf = h[hit, 0].view(np.float32), hf[hit, 0].view(np.float32)
    assert np.median(np.abs(t - tf) / tf) < 1e-6
    # any-hit agrees with closest-hit
    a = osc.trace(rays, any_hit=True)
    assert np.array_equal(a[:, 1] != 0xFFFFFFFF, h[:, 1] != 0xFFFFFFFF)


def test_instanced_render_matches_flattened_render(bsm, oracle):
    sc = bsm.generate_instanced_scene(seed=3, instances=30, width=40, height=30, sphere_res=8, ground=16)
    img, st, _ = oracle.OracleScene(sc).render(sc.camera.as_array(), spp=2, max_segments=3, seed=5)
    imgf, stf, _ = oracle.OracleScene(sc.flattened()).render(sc.camera.as_array(), spp=2, max_segments=3, seed=5)
    assert np.isfinite(img).all()
    assert st[0] == stf[0] == 40 * 30 * 2
    # primary rays hit the same triangles in both spaces; later segments may diverge on a few paths
    assert abs(int(st[1]) - int(stf[1])) <= 0.01 * st[1]
    assert abs(float(img.mean()) - float(imgf.mean())) <= 0.02 * float(imgf.mean())
