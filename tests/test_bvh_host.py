"""The compressed 8-wide BVH built by the product (host build, no GPU).

Invariants: every triangle referenced exactly once; leaves hold 1..2
triangles and at most 16 per node; every quantised child box, decoded in
double precision, encloses all triangles of its subtree; depth within the
traversal stack.  A numpy restatement of the octant-ordered traversal over
the decoded boxes finds the same closest hits as the oracle."""
import numpy as np
import pytest

from conftest import random_rays

NODE_DT = np.dtype([("p", "<f4", 3), ("e", "u1", 3), ("imask", "u1"), ("child_base", "<u4"), ("tri_base", "<u4"),
                    ("tri_mask", "<u2"), ("pad", "u1", 6), ("qlo", "u1", (3, 8)), ("qhi", "u1", (3, 8))])
TRI_DT = np.dtype([("v0", "<f4", 3), ("prim", "<u4"), ("v1", "<f4", 3), ("mat", "<u4"), ("v2", "<f4", 3),
                   ("pad", "<u4")])


def decode(nodes_b, tris_b):
    assert NODE_DT.itemsize == 80 and TRI_DT.itemsize == 48
    return nodes_b.view(NODE_DT), tris_b.view(TRI_DT)


def children(node):
    """Yields (slot, is_internal, child index or (first tri, count), lo(3), hi(3)) in double precision."""
    scale = np.ldexp(1.0, node["e"].astype(np.int64) - 127)
    p = node["p"].astype(np.float64)
    tmask = int(node["tri_mask"])
    for s in range(8):
        inner = (int(node["imask"]) >> s) & 1
        tm = (tmask >> (2 * s)) & 3
        if not inner and tm == 0:
            continue
        lo = p + node["qlo"][:, s] * scale
        hi = p + node["qhi"][:, s] * scale
        if inner:
            rel = bin(int(node["imask"]) & ((1 << s) - 1)).count("1")
            yield s, True, int(node["child_base"]) + rel, lo, hi
        else:
            assert tm in (1, 3), "a slot's second triangle without a first"
            first = int(node["tri_base"]) + bin(tmask & ((1 << (2 * s)) - 1)).count("1")
            yield s, False, (first, bin(tm).count("1")), lo, hi


@pytest.fixture(scope="module")
def built(bsm):
    sc = bsm.generate_scene(bsm.BSM_SCENE_ROOM, seed=4, spheres=12, width=32, height=32)
    nb, tb, st = bsm.bvh_build_host(sc)
    nodes, tris = decode(nb, tb)
    return sc, nodes, tris, st


def test_every_triangle_once(built):
    sc, nodes, tris, st = built
    assert st.num_tris == sc.num_triangles == len(tris)
    assert np.array_equal(np.sort(tris["prim"]), np.arange(sc.num_triangles))
    # leaf triangles carry their input vertices and material
    t = tris[np.argsort(tris["prim"])]
    v = sc.positions[sc.indices]
    assert np.array_equal(t["v0"], v[:, 0]) and np.array_equal(t["v1"], v[:, 1]) and np.array_equal(t["v2"], v[:, 2])
    assert np.array_equal(t["mat"], sc.material_ids)


def test_boxes_enclose_subtrees_and_leaf_sizes(built):
    sc, nodes, tris, st = built
    assert st.max_depth <= 24
    seen = np.zeros(len(tris), np.int32)

    def subtree_tris(ci):
        out = []
        stack = [ci]
        while stack:
            n = nodes[stack.pop()]
            for s, internal, ref, lo, hi in children(n):
                if internal:
                    stack.append(ref)
                else:
                    out.extend(range(ref[0], ref[0] + ref[1]))
        return out

    for ni in range(len(nodes)):
        n = nodes[ni]
        total = 0
        for s, internal, ref, lo, hi in children(n):
            idx = subtree_tris(ref) if internal else list(range(ref[0], ref[0] + ref[1]))
            if not internal:
                assert 1 <= ref[1] <= 2
                total += ref[1]
                seen[idx] += 1
            v = np.concatenate([tris["v0"][idx], tris["v1"][idx], tris["v2"][idx]]).astype(np.float64)
            assert (v >= lo).all() and (v <= hi).all(), f"node {ni} slot {s} box does not enclose its triangles"
        assert total <= 16
    assert (seen == 1).all()


def test_octant_traversal_finds_oracle_hits(bsm, oracle, built):
    sc, nodes, tris, st = built
    rays = random_rays(400, -0.2, 1.2, seed=21)
    osc = oracle.OracleScene(sc)
    ref = osc.trace(rays)
    tv = np.stack([tris["v0"], tris["v1"], tris["v2"]], 1)
    from test_oracle import watertight_brute
    for i in range(rays.shape[0]):
        o = rays[i, :3].astype(np.float64)
        d = rays[i, 4:7].astype(np.float64)
        with np.errstate(divide="ignore"):
            inv = 1.0 / d
        oct_key = 7 ^ ((d[0] < 0) | ((d[1] < 0) << 1) | ((d[2] < 0) << 2))
        best_t, best_p = float(rays[i, 7]), 0xFFFFFFFF
        stack = [0]
        while stack:
            n = nodes[stack.pop()]
            hits = []
            for s, internal, ref_, lo, hi in children(n):
                with np.errstate(invalid="ignore"):
                    t0 = (lo - o) * inv
                    t1 = (hi - o) * inv
                tn = np.nanmax(np.minimum(t0, t1).tolist() + [0.0])
                tf = np.nanmin(np.maximum(t0, t1).tolist() + [best_t])
                if tn <= tf * (1 + 1e-6):
                    hits.append((s ^ oct_key, internal, ref_))
            # visit children near to far: highest key first (push in reverse)
            for key, internal, ref_ in sorted(hits, key=lambda h: h[0]):
                if internal:
                    stack.append(ref_)
                else:
                    idx = np.arange(ref_[0], ref_[0] + ref_[1])
                    r = rays[i:i + 1].copy()
                    r[0, 7] = best_t
                    t, p = watertight_brute(tv[idx], r)
                    if p[0] != 0xFFFFFFFF:
                        prim = int(tris["prim"][idx[p[0]]])
                        if t[0] < best_t or (t[0] == best_t and prim < best_p):
                            best_t, best_p = float(t[0]), prim
        assert best_p == ref[i, 1], f"ray {i}"


@pytest.mark.parametrize("collapse", [0, 1])
@pytest.mark.parametrize("kind", ["room", "terrain"])
def test_kernel_arithmetic_traversal_finds_oracle_hits(bsm, oracle, kind, collapse):
    """The oracle's restatement of the device traversal (quantised slab
    arithmetic in float, octant order) over the host-built tree finds the
    closest and any hits of the oracle's own binary BVH, bit for bit, for
    both collapse modes; the per-ray counts are positive and bounded."""
    if kind == "room":
        sc = bsm.generate_scene(bsm.BSM_SCENE_ROOM, seed=6, spheres=16, width=32, height=32)
        rays = random_rays(3000, -0.2, 1.2, seed=22)
    else:
        sc = bsm.generate_scene(bsm.BSM_SCENE_TERRAIN, seed=2, grid=64, spheres=40, width=32, height=32)
        rays = random_rays(3000, -1.0, 1.0, seed=23)
    nb, tb, st = bsm.bvh_build_host(sc, collapse=collapse)
    osc = oracle.OracleScene(sc)
    ref = osc.trace(rays)
    hits, cnt = oracle.cwbvh_trace(nb, tb, rays)
    assert np.array_equal(hits[:, 1], ref[:, 1])
    hit = ref[:, 1] != 0xFFFFFFFF
    assert hit.sum() > 100
    assert np.array_equal(hits[hit, 0], ref[hit, 0]) and np.array_equal(hits[hit, 2:], ref[hit, 2:])
    assert (cnt[:, 0] >= 1).all() and (cnt[:, 0] <= st.num_nodes).all()
    assert (cnt[hit, 1] >= 1).all()
    occ_ref = osc.trace(rays, any_hit=True)[:, 1] != 0xFFFFFFFF
    occ, _ = oracle.cwbvh_trace(nb, tb, rays, any_hit=True)
    assert np.array_equal(occ[:, 1] != 0xFFFFFFFF, occ_ref)


def test_axis_parallel_rays_stay_cheap(bsm, oracle):
    """A direction component of exactly zero (a sky sample at the zenith, a
    ray along an axis) must still let that axis's slabs cull: the traversal
    of axis-parallel rays visits about as many nodes as that of slightly
    tilted ones, and finds the same hits as the oracle's binary BVH."""
    sc = bsm.generate_scene(bsm.BSM_SCENE_TERRAIN, seed=2, grid=128, spheres=200, width=32, height=32)
    nb, tb, _ = bsm.bvh_build_host(sc)
    osc = oracle.OracleScene(sc)
    lo, hi = sc.positions.min(0), sc.positions.max(0)
    rng = np.random.default_rng(1)
    n = 3000

    def rays(d, axis_origin):
        r = np.zeros((n, 8), np.float32)
        r[:, 0] = rng.uniform(lo[0], hi[0], n)
        r[:, 1] = rng.uniform(lo[1], hi[1], n)
        r[:, 2] = rng.uniform(lo[2], hi[2], n)
        k, v = axis_origin
        r[:, k] = v
        d = np.array(d, np.float32)
        r[:, 4:7] = d / np.linalg.norm(d)
        r[:, 7] = 100.0
        return r

    cases = [((0, -1, 0), (1, hi[1] + 0.1)), ((1, 0, 0), (0, lo[0] - 0.1)), ((0, 0, -1), (2, hi[2] + 0.1)),
             ((0, -1e-30, 1), (2, lo[2] - 0.1))]
    tilted = rays((1e-3, -1, 2e-3), (1, hi[1] + 0.1))
    _, ct = oracle.cwbvh_trace(nb, tb, tilted)
    for d, o in cases:
        r = rays(d, o)
        h, c = oracle.cwbvh_trace(nb, tb, r)
        assert np.array_equal(h[:, 1], osc.trace(r)[:, 1])
        assert c[:, 0].mean() <= 3.0 * ct[:, 0].mean() + 8, (d, c[:, 0].mean(), ct[:, 0].mean())
        assert c[:, 0].max() <= 400, (d, c[:, 0].max())
