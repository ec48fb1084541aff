"""Edge cases of the GPU path against the oracle.

* coincident triangles: the lower primitive id wins the tie at equal t;
  zero-area triangles are never hit;
* shared edges and vertices of a triangle grid do not leak (watertight test);
* rays with a non-finite origin or direction, a zero direction, or an empty
  or NaN interval are misses (no traversal);
* tiny and odd image sizes render like the oracle;
* cameras that cannot be rendered are rejected with an error, on every
  render entry point."""
import numpy as np
import pytest

from conftest import assert_bits_equal
from edge_scenes import MISS, coincident_scene, edge_rays, grid_scene, invalid_rays, rays_along_z

pytestmark = pytest.mark.gpu


def test_ties_degenerates_and_invalid_rays(bsm, ctx, oracle):
    sc = coincident_scene(bsm)
    sid = ctx.load_scene(sc)
    osc = oracle.OracleScene(sc)
    rays = np.concatenate([rays_along_z(4000, seed=3), invalid_rays()])
    g = ctx.trace_closest(sid, rays)
    c = osc.trace(rays)
    assert np.array_equal(g[:, :2], c[:, :2])
    assert not np.isin(g[:, 1], [2, 3, 4]).any()
    n = 4000
    assert (g[n:, 1] == MISS).all()
    occ = ctx.trace_any(sid, rays)
    assert occ[:n].all() and not occ[n:].any()
    ctx.release(sid)


def test_shared_edges_do_not_leak(bsm, ctx, oracle):
    sc = grid_scene(bsm)
    sid = ctx.load_scene(sc)
    rays = edge_rays()
    g = ctx.trace_closest(sid, rays)
    c = oracle.OracleScene(sc).trace(rays)
    assert (g[:, 1] != MISS).all()
    assert np.array_equal(g[:, :2], c[:, :2])
    ctx.release(sid)


@pytest.mark.parametrize("w,h", [(1, 1), (3, 5), (257, 1), (1, 67)])
def test_tiny_and_odd_images(bsm, ctx, oracle, w, h):
    sc = bsm.generate_scene(bsm.BSM_SCENE_ROOM, seed=5, width=w, height=h)
    sid = ctx.load_scene(sc)
    s = bsm.settings(spp=3, max_segments=4, seed=2)
    imgs, st = ctx.render(sid, [sc.camera], s)
    ref, ost, _ = oracle.OracleScene(sc).render(sc.camera.as_array(), spp=3, max_segments=4, seed=2)
    assert imgs[0].shape == (h, w, 4)
    assert list(st.rays_per_segment[:4]) == [int(x) for x in ost[:4]]
    gi, ci = imgs[0][..., :3].astype(np.float64), ref[..., :3].astype(np.float64)
    assert (np.abs(gi - ci) / np.maximum(np.abs(ci), 1e-3)).max() <= 1e-4
    det = bsm.BSM_PT_DETERMINISTIC   # fixed-point sums on both sides: equal bit for bit
    dimg, _ = ctx.render(sid, [sc.camera], bsm.settings(spp=3, max_segments=4, seed=2, flags=det))
    dref, _, _ = oracle.OracleScene(sc).render(sc.camera.as_array(), spp=3, max_segments=4, seed=2, flags=det)
    assert_bits_equal(dimg[0], dref)
    ctx.release(sid)


def test_unrenderable_cameras_are_rejected(bsm, ctx):
    sc = bsm.generate_scene(bsm.BSM_SCENE_ROOM, seed=5, width=8, height=8)
    sid = ctx.load_scene(sc)
    s = bsm.settings(spp=1, max_segments=2)
    good = sc.camera
    bad = []
    for field, value in [("position", (np.nan, 0.5, 0.5)), ("front", (0.0, 0.0, 0.0)), ("front", (0.0, 1.0, 0.0)),
                         ("up", (np.inf, 1.0, 0.0)), ("yfov_deg", 0.0), ("yfov_deg", 180.0)]:
        cam = bsm.make_camera(tuple(good.position), tuple(good.front), tuple(good.up), good.yfov_deg, 8, 8)
        if field == "yfov_deg":
            cam.yfov_deg = value
        else:
            getattr(cam, field)[:] = list(value)
        bad.append(cam)
    for cam in bad:
        with pytest.raises(bsm.BsmError):
            ctx.render(sid, [cam], s)
        with pytest.raises(bsm.BsmError):
            ctx.render_primary(sid, cam, s)
    # the context stays usable
    imgs, _ = ctx.render(sid, [good], s)
    assert np.isfinite(imgs[0]).all()
    ctx.release(sid)
