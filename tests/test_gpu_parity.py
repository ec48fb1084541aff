"""GPU parity: the CUDA pass (through the C ABI) against the CPU oracle.

Bar: closest-hit primitive ids and t bit-exact; any-hit decisions exact;
per-pixel radiance within 1e-4 relative (absolute floor 1e-3 * 1e-4); ray
counts per segment equal (they only agree if every path took the same
decisions on both sides)."""
import numpy as np
import pytest

from conftest import random_rays


def assert_same_hits(g, c):
    bad = np.nonzero((g[:, 0] != c[:, 0]) | (g[:, 1] != c[:, 1]))[0]
    assert bad.size == 0, f"{bad.size} rays differ, first {bad[:5].tolist()}: gpu {g[bad[:5], :2].tolist()} " \
                          f"oracle {c[bad[:5], :2].tolist()}"

pytestmark = pytest.mark.gpu

RTOL = 1e-4


def rel_err(g, c):
    g = g[..., :3].astype(np.float64)
    c = c[..., :3].astype(np.float64)
    return np.abs(g - c) / np.maximum(np.abs(c), 1e-3)


@pytest.fixture(scope="module")
def room(bsm, ctx, oracle):
    sc = bsm.generate_scene(bsm.BSM_SCENE_ROOM, seed=1, width=64, height=64)
    return sc, ctx.load_scene(sc), oracle.OracleScene(sc)


@pytest.fixture(scope="module")
def terrain(bsm, ctx, oracle):
    sc = bsm.generate_scene(bsm.BSM_SCENE_TERRAIN, seed=2, grid=96, spheres=200, sky_width=256, sky_height=128,
                            width=96, height=54)
    return sc, ctx.load_scene(sc), oracle.OracleScene(sc)


@pytest.mark.parametrize("which", ["room", "terrain"])
def test_closest_hit_random_rays_bit_exact(which, room, terrain, ctx):
    sc, sid, osc = room if which == "room" else terrain
    rays = random_rays(200_000, -0.3, 1.3, seed=5)
    g = ctx.trace_closest(sid, rays)
    c = osc.trace(rays)
    assert_same_hits(g, c)
    hit = c[:, 1] != 0xFFFFFFFF
    assert hit.mean() > (0.3 if which == "room" else 0.05)
    assert np.array_equal(g[hit, 2:], c[hit, 2:])


def test_any_hit_matches_oracle(room, ctx):
    sc, sid, osc = room
    rays = random_rays(100_000, -0.3, 1.3, seed=6, tmax=0.3)
    g = ctx.trace_any(sid, rays)
    c = osc.trace(rays, any_hit=True)
    assert np.array_equal(g.astype(bool), c[:, 1] != 0xFFFFFFFF)


def test_axis_aligned_and_grazing_rays(terrain, ctx):
    sc, sid, osc = terrain
    rng = np.random.default_rng(9)
    n = 50_000
    o = rng.uniform(0.0, 1.0, (n, 3)).astype(np.float32)
    o[:, 1] = 0.4
    d = np.zeros((n, 3), np.float32)
    d[:, 1] = -1.0                        # straight down: two zero components
    rays = np.concatenate([o, np.zeros((n, 1), np.float32), d, np.full((n, 1), 10.0, np.float32)], 1)
    # rays through grid vertices exactly (shared by up to six triangles: ties)
    g = 96
    ij = rng.integers(0, g, (n, 2))
    rays[: n // 2, 0] = ij[: n // 2, 0] / np.float32(g - 1)
    rays[: n // 2, 2] = ij[: n // 2, 1] / np.float32(g - 1)
    gh = ctx.trace_closest(sid, rays)
    ch = osc.trace(rays)
    assert_same_hits(gh, ch)
    # grazing rays along the x axis at terrain height
    rays2 = random_rays(n, 0.0, 1.0, seed=10)
    rays2[:, 1] = rng.uniform(0.0, 0.15, n)
    rays2[:, 4:7] = [1.0, 0.0, 0.0]
    gh = ctx.trace_closest(sid, rays2)
    ch = osc.trace(rays2)
    assert_same_hits(gh, ch)


def test_empty_and_tiny_tmax(room, ctx):
    sc, sid, osc = room
    assert ctx.trace_closest(sid, np.zeros((0, 8), np.float32)).shape == (0, 4)
    rays = random_rays(1000, 0.2, 0.8, seed=1, tmax=1e-7)
    g = ctx.trace_closest(sid, rays)
    c = osc.trace(rays)
    assert np.array_equal(g[:, :2], c[:, :2])


@pytest.mark.parametrize("flags", [0, 1, 2, 4])
def test_render_room_matches_oracle(bsm, room, ctx, flags):
    sc, sid, osc = room
    s = bsm.settings(spp=4, max_segments=4, seed=3, flags=flags)
    imgs, st = ctx.render(sid, [sc.camera], s)
    ref, ost, _ = osc.render(sc.camera.as_array(), spp=4, max_segments=4, seed=3, flags=flags)
    assert list(st.rays_per_segment[:4]) == [int(x) for x in ost[:4]]
    assert st.shadow_rays == int(ost[16:].sum())
    assert rel_err(imgs[0], ref).max() <= RTOL


def test_render_terrain_matches_oracle(bsm, terrain, ctx):
    sc, sid, osc = terrain
    s = bsm.settings(spp=4, max_segments=8, seed=4)
    imgs, st = ctx.render(sid, [sc.camera], s)
    ref, ost, _ = osc.render(sc.camera.as_array(), spp=4, max_segments=8, seed=4)
    assert list(st.rays_per_segment[:8]) == [int(x) for x in ost[:8]]
    assert rel_err(imgs[0], ref).max() <= RTOL
    assert imgs[0][..., :3].mean() > 0.01


def test_small_wavefront_chunks_same_image(bsm, room, ctx):
    """Chunked wavefronts (capacity below the path count) give the same image."""
    sc, sid, osc = room
    a, sa = ctx.render(sid, [sc.camera], bsm.settings(spp=4, max_segments=4, seed=8))
    b, sb = ctx.render(sid, [sc.camera], bsm.settings(spp=4, max_segments=4, seed=8, wavefront_capacity=5000))
    assert sb.chunks > 1
    assert list(sa.rays_per_segment) == list(sb.rays_per_segment)
    assert rel_err(a[0], b[0]).max() <= RTOL


def test_progressive_accumulation_equals_one_call(bsm, room, ctx):
    """Two accumulated calls of 2 spp equal one oracle render of 4 spp (the running mean)."""
    sc, sid, osc = room
    ctx.render(sid, [sc.camera], bsm.settings(spp=2, max_segments=4, seed=5, accumulate=0))
    imgs, _ = ctx.render(sid, [sc.camera], bsm.settings(spp=2, max_segments=4, seed=5, accumulate=1))
    ref, _, _ = osc.render(sc.camera.as_array(), spp=4, max_segments=4, seed=5)
    assert rel_err(imgs[0], ref).max() <= RTOL


def test_multi_view_equals_separate_renders(bsm, room, ctx):
    sc, sid, osc = room
    cams = [bsm.make_camera((0.5, 0.55, -1.1), (0.0, -0.09, 1.0), width=48, height=32),
            bsm.make_camera((1.5, 0.8, 0.5), (-1.0, -0.3, 0.0), width=40, height=40, yfov_deg=45.0)]
    s = bsm.settings(spp=2, max_segments=3, seed=9)
    imgs, _ = ctx.render(sid, cams, s)
    for i, cam in enumerate(cams):
        ref, _, _ = osc.render(cam.as_array(), spp=2, max_segments=3, seed=9)
        assert rel_err(imgs[i], ref).max() <= RTOL


def test_bvh_download_invariants(bsm, room, ctx):
    sc, sid, osc = room
    st = ctx.build_bvh(sid)
    nodes, tris = ctx.download_bvh(sid, st)
    prims = tris.view(np.uint32).reshape(-1, 12)[:, 3]
    assert np.array_equal(np.sort(prims), np.arange(sc.num_triangles, dtype=np.uint32))
