"""Point / spot / rect lights and the cubemap sky in the oracle (no GPU).

* a spot light lights the floor inside its outer cone only; a point light's
  falloff follows point_light_eval (lights.hlsl:15-25) for a pixel straight below;
* a one-sided rect light lights only the side its corners run counter-clockwise
  towards (local -z), a two-sided one both;
* a cubemap sky shows each face's colour along that face's axis."""
import numpy as np

HALF_ONE = 0x3C00


def floor_scene(bsm, point_lights=None, rect_lights=None, width=64, height=64, base=0.8, rough=1.0):
    pos = np.array([[-5, 0, -5], [5, 0, -5], [5, 0, 5], [-5, 0, 5]], np.float32)
    idx = np.array([[0, 2, 1], [0, 3, 2]], np.uint32)
    mats = np.array([[base, base, base, rough, 0.0]], np.float32)
    cam = bsm.make_camera((0.0, 4.0, 0.001), (0.0, -1.0, 0.0), up=(0.0, 0.0, -1.0), yfov_deg=90.0, width=width,
                          height=height)
    return bsm.SceneData(pos, idx, np.zeros(2, np.uint32), mats, np.zeros((0, 6), np.float32), bsm.BSM_SKY_CONSTANT,
                         (0.0, 0.0, 0.0), None, cam, point_lights=point_lights, rect_lights=rect_lights)


def render(oracle, sc, spp=1, segs=1, seed=1):
    img, st, _ = oracle.OracleScene(sc).render(sc.camera.as_array(), spp=spp, max_segments=segs, seed=seed)
    return img[..., :3].mean(-1)


def test_spot_cone_and_point_falloff(bsm, oracle):
    # spot 2 above the floor pointing down (direction to the light = +y), outer half angle 30 deg
    spot = np.array([[0, 2, 0, 5, 5, 5, 100, 0, 1, 0, np.cos(np.radians(20)), np.cos(np.radians(30))]], np.float32)
    img = render(oracle, floor_scene(bsm, point_lights=spot))
    # floor radius of the outer cone: 2 tan 30 = 1.155; the view spans +-4 over 64 px
    yy, xx = np.mgrid[0:64, 0:64]
    r = np.hypot((xx + 0.5) / 64 * 8 - 4, (yy + 0.5) / 64 * 8 - 4)
    assert img[r > 1.3].max() == 0.0
    assert img[r < 0.6].min() > 0.0
    # point light: the pixel below it is lit by emission * saturate(1 - (d^2/range^2)^2) / d^2 * BSDF
    for rng_ in (3.0, 100.0):
        pt = np.array([[0, 2, 0, 5, 5, 5, rng_, 0, 0, 1, 0, 0]], np.float32)
        c = render(oracle, floor_scene(bsm, point_lights=pt))[31:33, 31:33].mean()
        assert c > 0.0
        if rng_ == 3.0:
            ratio = c
        else:
            far = c
    assert abs(ratio / far - (1 - (4.0 / 9.0) ** 2)) < 0.02


def test_rect_light_sides(bsm, oracle):
    # a 1x1 rect 1 above the floor; axes x, z: local +z = cross(x, z) = -y, so it emits towards +y (away)
    away = np.array([[0, 1, 0, 1, 0, 0, 0, 0, 1, 1, 1, 4, 4, 4, 0]], np.float32)
    toward = away.copy()
    toward[0, 6:9] = [0, 0, -1]                      # cross(x, -z) = +y: emits towards -y (the floor)
    both = away.copy()
    both[0, 14] = 1
    i_away = render(oracle, floor_scene(bsm, rect_lights=away), spp=4)
    i_toward = render(oracle, floor_scene(bsm, rect_lights=toward), spp=4)
    i_both = render(oracle, floor_scene(bsm, rect_lights=both), spp=4)
    assert i_away.max() == 0.0
    assert i_toward[24:40, 24:40].min() > 0.0
    assert abs(float(i_both.mean()) - float(i_toward.mean())) < 0.05 * float(i_toward.mean())


def test_cubemap_faces(bsm, oracle):
    S = 8
    colors = np.array([[1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 1, 0], [0, 1, 1], [1, 0, 1]], np.float32)
    faces = np.zeros((6, S, S, 4), np.float16)
    faces[..., :3] = colors[:, None, None, :]
    faces[..., 3] = 1
    sc = floor_scene(bsm, width=3, height=3)
    sc.positions = np.array([[100, 100, 100], [100.1, 100, 100], [100, 100.1, 100]], np.float32)  # out of view
    sc.indices = np.array([[0, 1, 2]], np.uint32)
    sc.material_ids = np.zeros(1, np.uint32)
    sc.sky_kind, sc.sky_color, sc.sky_texels = bsm.BSM_SKY_CUBEMAP, (1.0, 1.0, 1.0), faces.view(np.uint16)
    axes = [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)]
    for f, a in enumerate(axes):
        up = (0.0, 0.0, 1.0) if abs(a[1]) == 1 else (0.0, 1.0, 0.0)
        sc.camera = bsm.make_camera((0.0, 0.0, 0.0), a, up=up, yfov_deg=10.0, width=3, height=3)
        img, _, _ = oracle.OracleScene(sc).render(sc.camera.as_array(), spp=1, max_segments=1)
        assert np.allclose(img[1, 1, :3], colors[f], atol=1e-3), (f, img[1, 1])
    # a rotation of the lookup: 90 deg about y maps the +x view onto the -z face (x -> -z)
    sc.sky_transform = np.array([0, 0, 1, 0, 1, 0, -1, 0, 0], np.float32)
    sc.camera = bsm.make_camera((0.0, 0.0, 0.0), (1, 0, 0), yfov_deg=10.0, width=3, height=3)
    img, _, _ = oracle.OracleScene(sc).render(sc.camera.as_array(), spp=1, max_segments=1)
    assert np.allclose(img[1, 1, :3], colors[5], atol=1e-3)
