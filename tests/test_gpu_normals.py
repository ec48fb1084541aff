"""Interpolated vertex normals at the hit (the reference's fetch_vertex_attributes,
bisemutum/shaders/core/raytracing/hit.hlsl:55-71, 158), on the GPU against the oracle.

* A scene of UV spheres carrying their analytic vertex normals: closest hits are
  unchanged by the normals; renders take the oracle's paths (equal ray counts
  per segment, radiance within 1e-4); the primary G-buffer's packed normal
  equals the oracle's bit for bit and differs from the faceted render's.
* A project in the reference's format whose mesh carries normals, loaded from
  its files: the GPU render matches the oracle and differs from the same scene
  shaded with geometric normals."""
import numpy as np
import pytest

from conftest import assert_bits_equal

pytestmark = pytest.mark.gpu


def rel_err(g, c):
    g = g[..., :3].astype(np.float64)
    c = c[..., :3].astype(np.float64)
    return np.abs(g - c) / np.maximum(np.abs(c), 1e-3)


def spheres_scene(bsm, n_lat=10, n_lon=14):
    """Three coarse UV spheres on a floor; each sphere vertex carries its analytic normal."""
    pos, nrm, idx, mids = [], [], [], []
    centres = [(0.3, 0.25, 0.5, 0.22), (0.72, 0.18, 0.35, 0.16), (0.6, 0.2, 0.78, 0.18)]
    for si, (cx, cy, cz, r) in enumerate(centres):
        base = len(pos)
        for i in range(n_lat + 1):
            th = np.pi * i / n_lat
            for j in range(n_lon):
                ph = 2 * np.pi * j / n_lon
                n = np.array([np.sin(th) * np.cos(ph), np.cos(th), np.sin(th) * np.sin(ph)])
                pos.append([cx + r * n[0], cy + r * n[1], cz + r * n[2]])
                nrm.append(n)
        for i in range(n_lat):
            for j in range(n_lon):
                a = base + i * n_lon + j
                b = base + i * n_lon + (j + 1) % n_lon
                c = a + n_lon
                d = b + n_lon
                if i > 0:
                    idx.append([a, b, c])
                    mids.append(si + 1)
                if i < n_lat - 1:
                    idx.append([b, d, c])
                    mids.append(si + 1)
    base = len(pos)
    for p in [(-1, 0, -1), (2, 0, -1), (2, 0, 2), (-1, 0, 2)]:
        pos.append(p)
        nrm.append((0.0, 1.0, 0.0))
    idx += [[base, base + 2, base + 1], [base, base + 3, base + 2]]
    mids += [0, 0]
    mats = np.array([[0.6, 0.6, 0.6, 0.8, 0.0], [0.8, 0.3, 0.2, 0.4, 0.0], [0.9, 0.9, 0.9, 0.15, 1.0],
                     [0.2, 0.5, 0.8, 0.6, 0.0]], np.float32)
    lights = np.array([[0.4, 0.8, -0.3, 3.0, 2.9, 2.7]], np.float32)
    cam = bsm.make_camera((0.5, 0.55, -0.6), (0.0, -0.3, 1.0), yfov_deg=55.0, width=96, height=72)
    sc = bsm.SceneData(np.array(pos, np.float32), np.array(idx, np.uint32), np.array(mids, np.uint32), mats, lights,
                       bsm.BSM_SKY_CONSTANT, (0.4, 0.5, 0.6), None, cam, normals=np.array(nrm, np.float32))
    return sc, centres


def test_smooth_spheres_match_oracle(bsm, ctx, oracle):
    sc, centres = spheres_scene(bsm)
    flat = bsm.SceneData(sc.positions, sc.indices, sc.material_ids, sc.materials, sc.lights, sc.sky_kind,
                         sc.sky_color, None, sc.camera)
    sid = ctx.load_scene(sc)
    fid = ctx.load_scene(flat)
    osc = oracle.OracleScene(sc)
    try:
        from conftest import random_rays
        rays = random_rays(20000, -0.2, 1.2, seed=3)
        assert np.array_equal(ctx.trace_closest(sid, rays), ctx.trace_closest(fid, rays))
        s = bsm.settings(spp=4, max_segments=6, seed=5)
        imgs, st = ctx.render(sid, [sc.camera], s)
        ref, ost, _ = osc.render(sc.camera.as_array(), spp=4, max_segments=6, seed=5)
        assert [int(x) for x in st.rays_per_segment[:6]] == [int(x) for x in ost[:6]]
        assert rel_err(imgs[0], ref).max() <= 1e-4
        det = bsm.BSM_PT_DETERMINISTIC
        dimg, _ = ctx.render(sid, [sc.camera], bsm.settings(spp=4, max_segments=6, seed=5, flags=det))
        dref, _, _ = osc.render(sc.camera.as_array(), spp=4, max_segments=6, seed=5, flags=det)
        assert_bits_equal(dimg[0], dref)
        flat_img, _ = ctx.render(fid, [sc.camera], s)
        assert rel_err(imgs[0], flat_img[0]).max() > 0.05, "vertex normals did not change the shading"
        # primary G-buffer: packed shading normal bit-exact with the oracle
        depth, gb, hp = ctx.render_primary(sid, sc.camera)
        od, ogb, ohp = osc.primary(sc.camera.as_array())
        assert np.array_equal(gb, ogb) and np.array_equal(depth, od)
        _, fgb, _ = ctx.render_primary(fid, sc.camera)
        assert not np.array_equal(gb[1], fgb[1])
        # the camera sees the spheres: many primary hits lie on them
        P = hp[..., :3][hp[..., 3] > 0]
        on_sphere = np.zeros(P.shape[0], bool)
        for cx, cy, cz, r in centres:
            on_sphere |= np.abs(np.linalg.norm(P - [cx, cy, cz], axis=1) - r) < 0.05 * r
        assert on_sphere.sum() > 500
    finally:
        ctx.release(sid)
        ctx.release(fid)


def test_loaded_project_with_normals_matches_oracle(bsm, ctx, oracle, tmp_path):
    """A project in the reference's format whose mesh carries vertex normals (written to a temporary directory):
    the loader turns them to world space, the GPU render matches the oracle and differs from the same scene
    shaded with geometric normals."""
    from test_assets import write_project
    root = str(tmp_path / "proj")
    write_project(root, bsm, normals=True)
    scene, info = bsm.load_project(root)
    assert scene.normals is not None and np.abs(scene.normals).sum() > 0
    cam = scene.camera
    sid = ctx.load_scene(scene)
    flat = bsm.SceneData(scene.positions, scene.indices, scene.material_ids, scene.materials, scene.lights,
                         scene.sky_kind, scene.sky_color, scene.sky_texels, cam, point_lights=scene.point_lights,
                         rect_lights=scene.rect_lights)
    fid = ctx.load_scene(flat)
    try:
        s = bsm.settings(spp=8, max_segments=4, seed=2, ray_length=info.settings.ray_length)
        imgs, st = ctx.render(sid, [cam], s)
        ref, ost, _ = oracle.OracleScene(scene).render(cam.as_array(), spp=8, max_segments=4, seed=2,
                                                       ray_length=info.settings.ray_length)
        assert [int(x) for x in st.rays_per_segment[:4]] == [int(x) for x in ost[:4]]
        assert rel_err(imgs[0], ref).max() <= 1e-4
        assert ref[..., :3].max() > 0.0
        det = bsm.BSM_PT_DETERMINISTIC
        dimg, _ = ctx.render(sid, [cam], bsm.settings(spp=8, max_segments=4, seed=2, ray_length=info.settings.ray_length,
                                                      flags=det))
        dref, _, _ = oracle.OracleScene(scene).render(cam.as_array(), spp=8, max_segments=4, seed=2,
                                                      ray_length=info.settings.ray_length, flags=det)
        assert_bits_equal(dimg[0], dref)
        flat_img, _ = ctx.render(fid, [cam], s)
        assert not np.allclose(imgs[0], flat_img[0]), "the project's normals did not reach the shading"
    finally:
        ctx.release(sid)
        ctx.release(fid)
