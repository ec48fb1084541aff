"""Procedural scenes: sizes and value ranges of the seeded inputs (no GPU)."""
import numpy as np


def test_room_scene(bsm):
    sc = bsm.generate_scene(bsm.BSM_SCENE_ROOM, seed=1)
    assert sc.num_triangles == 12 * 2 + 64 * 320 == 20504
    m = sc.materials
    assert ((m[:, :3] >= 0.1) & (m[:, :3] <= 0.9)).all()
    assert ((m[:, 3] >= 0.05) & (m[:, 3] <= 1.0)).all()
    assert set(np.unique(m[:, 4])) <= {0.0, 1.0}
    assert sc.lights.shape == (1, 6) and sc.lights[0, 1] > 0 and np.allclose(sc.lights[0, 3:], 3.0)
    assert np.isclose(np.linalg.norm(sc.lights[0, :3]), 1.0, atol=1e-6)
    assert sc.sky_kind == bsm.BSM_SKY_CONSTANT and np.allclose(sc.sky_color, 0.5)
    assert sc.camera.yfov_deg == 60.0


def test_terrain_scene_full_size(bsm):
    sc = bsm.generate_scene(bsm.BSM_SCENE_TERRAIN, seed=1, grid=512, spheres=2000)
    assert sc.num_triangles == 511 * 511 * 2 + 2000 * 480 == 1482242
    terrain = sc.positions[: 512 * 512]
    assert np.isclose(terrain[:, 1].min(), 0.0) and np.isclose(terrain[:, 1].max(), 0.15, atol=1e-6)
    assert sc.sky_texels.shape == (512, 1024, 4)
    tex = sc.sky_texels.view(np.float16).astype(np.float32)
    assert np.isfinite(tex).all() and (tex[..., :3] > 0).all()
    assert len(sc.materials) == 2001


def test_generation_is_deterministic(bsm):
    a = bsm.generate_scene(bsm.BSM_SCENE_TERRAIN, seed=5, grid=64, spheres=20)
    b = bsm.generate_scene(bsm.BSM_SCENE_TERRAIN, seed=5, grid=64, spheres=20)
    c = bsm.generate_scene(bsm.BSM_SCENE_TERRAIN, seed=6, grid=64, spheres=20)
    assert np.array_equal(a.positions, b.positions) and np.array_equal(a.sky_texels, b.sky_texels)
    assert not np.array_equal(a.positions, c.positions)


def test_serving_scene_sizes(bsm):
    # the 250k scene: terrain grid 256 + 250 spheres
    sc = bsm.generate_scene(bsm.BSM_SCENE_TERRAIN, seed=1, grid=256, spheres=250, sky_width=64, sky_height=32)
    assert sc.num_triangles == 255 * 255 * 2 + 250 * 480 == 250050
