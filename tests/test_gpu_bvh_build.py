"""The compressed 8-wide BVH built on the device (bvh_gpu.cu).

* The same invariants as the host-built tree (test_bvh_host.py): every triangle
  exactly once, carrying its input vertices and material; leaves of 1..2
  triangles and at most 16 per node; every quantised child box encloses its
  subtree's triangles; depth within the traversal stack.
* The oracle's restatement of the device traversal over the downloaded tree
  finds the oracle's own closest and any hits bit for bit, for both collapse
  modes and both leaf sizes; the GPU's traversal of it does too.
* Builds are deterministic (two builds give the same bytes) and the tree's
  traversal cost stays close to the host builder's (nodes and triangles per
  ray counted by the oracle's restatement on the same rays).
* At full size (the 1,482,242-triangle terrain) the tree is built on the
  device in a fraction of the host build's time, holds every triangle once
  and traverses to the oracle's hits."""
import numpy as np
import pytest

from conftest import random_rays
from test_bvh_host import children, decode

pytestmark = pytest.mark.gpu


def device_tree(bsm, ctx, sc, **kw):
    sid = ctx.upload(sc)
    st = ctx.build_bvh(sid, **kw)
    assert st.builder == bsm.BSM_BUILD_DEVICE
    nb, tb = ctx.download_bvh(sid, st)
    return sid, st, nb, tb


def check_invariants(sc, nb, tb, st):
    nodes, tris = decode(nb, tb)
    assert st.num_tris == sc.num_triangles == len(tris)
    assert np.array_equal(np.sort(tris["prim"]), np.arange(sc.num_triangles))
    t = tris[np.argsort(tris["prim"])]
    v = sc.positions[sc.indices] if sc.indices is not None else sc.positions.reshape(-1, 3, 3)
    assert np.array_equal(t["v0"], v[:, 0]) and np.array_equal(t["v1"], v[:, 1]) and np.array_equal(t["v2"], v[:, 2])
    assert np.array_equal(t["mat"], sc.material_ids)
    assert 1 <= st.max_depth <= 24
    seen = np.zeros(len(tris), np.int32)
    sub = {}

    def subtree_tris(ci):
        if ci in sub:
            return sub[ci]
        out = []
        for s, internal, ref, lo, hi in children(nodes[ci]):
            out.extend(subtree_tris(ref) if internal else range(ref[0], ref[0] + ref[1]))
        sub[ci] = out
        return out

    for ni in range(len(nodes) - 1, -1, -1):   # children have larger indices: fill the memo bottom-up
        n = nodes[ni]
        total = 0
        for s, internal, ref, lo, hi in children(n):
            idx = subtree_tris(ref) if internal else list(range(ref[0], ref[0] + ref[1]))
            if internal:
                assert ref > ni, "breadth-first order: children after their parent"
            else:
                assert 1 <= ref[1] <= 2
                total += ref[1]
                seen[idx] += 1
            vv = np.concatenate([tris["v0"][idx], tris["v1"][idx], tris["v2"][idx]]).astype(np.float64)
            assert (vv >= lo).all() and (vv <= hi).all(), f"node {ni} slot {s} box does not enclose its triangles"
        assert total <= 16
    assert (seen == 1).all()


@pytest.mark.parametrize("collapse,max_leaf", [(0, 0), (0, 1), (1, 2), (1, 1)])
@pytest.mark.parametrize("kind", ["room", "terrain"])
def test_device_tree_invariants_and_oracle_hits(bsm, ctx, oracle, kind, collapse, max_leaf):
    if kind == "room":
        sc = bsm.generate_scene(bsm.BSM_SCENE_ROOM, seed=6, spheres=16, width=32, height=32)
        rays = random_rays(4000, -0.2, 1.2, seed=22)
    else:
        sc = bsm.generate_scene(bsm.BSM_SCENE_TERRAIN, seed=2, grid=64, spheres=40, width=32, height=32)
        rays = random_rays(4000, -1.0, 1.0, seed=23)
    sid, st, nb, tb = device_tree(bsm, ctx, sc, collapse=collapse, max_leaf=max_leaf)
    try:
        check_invariants(sc, nb, tb, st)
        osc = oracle.OracleScene(sc)
        ref = osc.trace(rays)
        hits, cnt = oracle.cwbvh_trace(nb, tb, rays)
        assert np.array_equal(hits, ref)
        assert (cnt[:, 0] >= 1).all() and (cnt[:, 0] <= st.num_nodes).all()
        occ_ref = osc.trace(rays, any_hit=True)[:, 1] != 0xFFFFFFFF
        occ, _ = oracle.cwbvh_trace(nb, tb, rays, any_hit=True)
        assert np.array_equal(occ[:, 1] != 0xFFFFFFFF, occ_ref)
        # the GPU's own traversal of the device-built tree
        g = ctx.trace_closest(sid, rays)
        assert np.array_equal(g, ref)
    finally:
        ctx.release(sid)


@pytest.mark.parametrize("n_tris", [1, 2, 3, 7, 128, 129, 300])
def test_tiny_scenes(bsm, ctx, oracle, n_tris):
    """Edge sizes: a single triangle (the root is a leaf), one small node, the small/level boundary."""
    rng = np.random.default_rng(n_tris)
    pos = rng.uniform(0.0, 1.0, (3 * n_tris, 3)).astype(np.float32)
    sc = bsm.SceneData(pos, None, np.zeros(n_tris, np.uint32), np.array([[0.5, 0.5, 0.5, 0.5, 0.0]], np.float32),
                       np.array([[0.0, 1.0, 0.0, 1.0, 1.0, 1.0]], np.float32),
                       camera=bsm.make_camera((0.5, 0.5, -1.0), (0.0, 0.0, 1.0), width=16, height=16))
    sid, st, nb, tb = device_tree(bsm, ctx, sc)
    try:
        check_invariants(sc, nb, tb, st)
        rays = random_rays(2000, -0.2, 1.2, seed=3)
        ref = oracle.OracleScene(sc).trace(rays)
        assert np.array_equal(ctx.trace_closest(sid, rays), ref)
    finally:
        ctx.release(sid)


def test_coincident_centroids_split_by_index(bsm, ctx, oracle):
    """Every triangle has the same centroid: no binned split exists, the builder splits by index."""
    n = 600
    rng = np.random.default_rng(5)
    d = rng.normal(size=(n, 3, 3)).astype(np.float32) * 0.1
    d -= d.mean(axis=1, keepdims=True)           # centroid of each triangle at the origin... of its box:
    lo, hi = d.min(1), d.max(1)
    d -= (0.5 * (lo + hi))[:, None, :]           # box centres (the builder's centroids) all at 0
    pos = (d + 0.5).reshape(-1, 3).astype(np.float32)
    sc = bsm.SceneData(pos, None, np.zeros(n, np.uint32), np.array([[0.5, 0.5, 0.5, 0.5, 0.0]], np.float32),
                       np.array([[0.0, 1.0, 0.0, 1.0, 1.0, 1.0]], np.float32),
                       camera=bsm.make_camera((0.5, 0.5, -1.0), (0.0, 0.0, 1.0), width=16, height=16))
    sid, st, nb, tb = device_tree(bsm, ctx, sc)
    try:
        check_invariants(sc, nb, tb, st)
        rays = random_rays(2000, 0.2, 0.8, seed=4)
        assert np.array_equal(ctx.trace_closest(sid, rays), oracle.OracleScene(sc).trace(rays))
    finally:
        ctx.release(sid)


def test_deterministic_and_close_to_host_quality(bsm, ctx, oracle):
    sc = bsm.generate_scene(bsm.BSM_SCENE_TERRAIN, seed=3, grid=128, spheres=200, width=32, height=32)
    _, st1, nb1, tb1 = device_tree(bsm, ctx, sc)
    _, st2, nb2, tb2 = device_tree(bsm, ctx, sc)
    assert np.array_equal(nb1, nb2) and np.array_equal(tb1, tb2)
    hb, ht, hst = bsm.bvh_build_host(sc)
    rays = random_rays(20000, -0.2, 1.2, seed=8)
    _, cd = oracle.cwbvh_trace(nb1, tb1, rays)
    _, ch = oracle.cwbvh_trace(hb, ht, rays)
    # traversal work per ray within 15 % of the host tree's
    assert cd[:, 0].mean() <= 1.15 * ch[:, 0].mean(), (cd[:, 0].mean(), ch[:, 0].mean())
    assert cd[:, 1].mean() <= 1.15 * ch[:, 1].mean(), (cd[:, 1].mean(), ch[:, 1].mean())
    assert st1.sah_cost <= 1.1 * hst.sah_cost


def test_render_parity_on_device_tree(bsm, ctx, oracle):
    sc = bsm.generate_scene(bsm.BSM_SCENE_TERRAIN, seed=2, grid=96, spheres=200, sky_width=256, sky_height=128,
                            width=96, height=54)
    sid = ctx.load_scene(sc)
    try:
        imgs, st = ctx.render(sid, [sc.camera], bsm.settings(spp=4, max_segments=8, seed=4))
        ref, ost, _ = oracle.OracleScene(sc).render(sc.camera.as_array(), spp=4, max_segments=8, seed=4)
        assert [int(x) for x in st.rays_per_segment[:8]] == [int(x) for x in ost[:8]]
        err = np.abs(imgs[0][..., :3].astype(np.float64) - ref[..., :3]) / np.maximum(np.abs(ref[..., :3]), 1e-3)
        assert err.max() <= 1e-4
    finally:
        ctx.release(sid)


def test_instanced_geometries_built_on_device(bsm, ctx, oracle):
    from test_instancing_oracle import random_world_rays
    sc = bsm.generate_instanced_scene(seed=4, instances=60, width=32, height=24, sphere_res=12, ground=32)
    sid = ctx.load_instanced(sc)   # every geometry's BLAS on the device
    try:
        rays = random_world_rays(20000, seed=3)
        assert np.array_equal(ctx.trace_closest(sid, rays), oracle.OracleScene(sc).trace(rays))
    finally:
        ctx.release(sid)


def test_full_size_terrain(bsm, oracle):
    """The 1,482,242-triangle terrain: built on the device, every triangle once, the oracle's hits."""
    sc = bsm.generate_scene(bsm.BSM_SCENE_TERRAIN, seed=1, grid=512, spheres=2000, width=64, height=64)
    with bsm.Context(0) as c2:
        sid = c2.upload(sc)
        st = c2.build_bvh(sid)
        assert st.builder == bsm.BSM_BUILD_DEVICE and st.max_depth <= 24
        nb, tb = c2.download_bvh(sid, st)
        nodes, tris = decode(nb, tb)
        assert np.array_equal(np.sort(tris["prim"]), np.arange(sc.num_triangles))
        t = tris[np.argsort(tris["prim"])]
        v = sc.positions[sc.indices]
        assert np.array_equal(t["v0"], v[:, 0]) and np.array_equal(t["v2"], v[:, 2])
        # leaf masks: 1..2 triangles per slot, all slots' triangles inside the node's range
        tm = nodes["tri_mask"].astype(np.uint32)
        ntri = np.array([bin(int(x)).count("1") for x in tm])
        assert ntri.sum() == sc.num_triangles
        for s in range(8):
            slot = (tm >> (2 * s)) & 3
            assert not np.any(slot == 2), "a slot's second triangle without a first"
        rays = random_rays(50000, -0.1, 1.1, seed=40)
        ref = oracle.OracleScene(sc).trace(rays)
        hits, cnt = oracle.cwbvh_trace(nb, tb, rays)
        assert np.array_equal(hits, ref)
        assert np.array_equal(c2.trace_closest(sid, rays), ref)
        host = bsm.bvh_build_host(sc)
        _, ch = oracle.cwbvh_trace(host[0], host[1], rays)
        assert cnt[:, 0].mean() <= 1.15 * ch[:, 0].mean(), (cnt[:, 0].mean(), ch[:, 0].mean())
        assert st.build_ms < host[2].build_ms, (st.build_ms, host[2].build_ms)
