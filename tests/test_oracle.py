"""The CPU oracle against known answers (no GPU).

* PCG32: the published output of the pcg32 demo (O'Neill, pcg-c-basic,
  pcg32_srandom_r(42, 54)).
* BSDF, frame, anisotropic roughness: golden vectors produced from the
  reference's own shader sources (tests/golden/make_golden.py).
* Closest hit: the oracle's BVH traversal against a brute-force numpy float32
  restatement of the same watertight test over every triangle (bit-exact).
"""
import numpy as np
import pytest

from conftest import random_rays

GOLD = None


def golden():
    global GOLD
    if GOLD is None:
        import os
        GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "bsdf_golden.npz"))
    return GOLD


def test_pcg32_published_vector(oracle):
    assert [int(x) for x in oracle.pcg32(42, 54, 6)] == [0xa15c02b7, 0x7b47f409, 0xba1d3330, 0x83d2f293,
                                                        0xbfa4784b, 0xcbed606e]


def test_sincos_and_atan2_accuracy(oracle):
    t = np.linspace(-2.0, 2.0, 200001, dtype=np.float32)
    s, c = oracle.sincos_turns(t)
    ang = 2 * np.pi * t.astype(np.float64)
    assert np.abs(s - np.sin(ang)).max() < 4e-7
    assert np.abs(c - np.cos(ang)).max() < 4e-7
    rng = np.random.default_rng(1)
    y = rng.normal(size=100000).astype(np.float32)
    x = rng.normal(size=100000).astype(np.float32)
    x[:10] = 0.0
    y[10:20] = 0.0
    a = oracle.atan2(y, x)
    assert np.abs(a - np.arctan2(y.astype(np.float64), x.astype(np.float64))).max() < 1e-6


def test_bsdf_matches_reference_shader_golden(oracle):
    g = golden()
    out = oracle.eval_lit(g["lit_in"])
    ref = g["lit_out"]
    err = np.abs(out - ref) / np.maximum(np.abs(ref), 1e-6)
    assert err.max() < 2e-5, err.max()
    assert float(g["inv_pi"]) == np.float32(0.318309873)


def test_vndf_matches_reference_shader_golden(oracle):
    g = golden()
    out = oracle.vndf(g["vndf_in"])
    ref = g["vndf_out"]
    assert np.abs(out[:, :3] - ref[:, :3]).max() < 3e-5   # sin/cos of the azimuth differ in the last bits
    assert (np.abs(out[:, 3] - ref[:, 3]) / np.abs(ref[:, 3])).max() < 1e-4


def test_frame_matches_reference_shader_golden(oracle):
    g = golden()
    assert np.array_equal(oracle.frame(g["frame_in"]), g["frame_out"])


# ---- brute-force watertight closest hit in numpy float32 (same op order) ----
def watertight_brute(tris, rays):
    """tris (T,3,3) float32; rays (N,8).  Returns (t, prim) per ray; ties -> lower prim."""
    f = np.float32
    out_t = rays[:, 7].copy()
    out_p = np.full(rays.shape[0], 0xFFFFFFFF, np.uint32)
    for i in range(rays.shape[0]):
        o = rays[i, 0:3]
        d = rays[i, 4:7]
        tmin = rays[i, 3]
        ad = np.abs(d)
        kz = 0
        if ad[1] > ad[kz]:
            kz = 1
        if ad[2] > ad[kz]:
            kz = 2
        kx = (kz + 1) % 3
        ky = (kx + 1) % 3
        if d[kz] < 0:
            kx, ky = ky, kx
        Sx = f(d[kx] / d[kz])
        Sy = f(d[ky] / d[kz])
        Sz = f(f(1.0) / d[kz])
        A = tris[:, 0, :] - o
        B = tris[:, 1, :] - o
        C = tris[:, 2, :] - o
        Ax = A[:, kx] - Sx * A[:, kz]
        Ay = A[:, ky] - Sy * A[:, kz]
        Bx = B[:, kx] - Sx * B[:, kz]
        By = B[:, ky] - Sy * B[:, kz]
        Cx = C[:, kx] - Sx * C[:, kz]
        Cy = C[:, ky] - Sy * C[:, kz]
        U = Cx * By - Cy * Bx
        V = Ax * Cy - Ay * Cx
        W = Bx * Ay - By * Ax
        z = (U == 0) | (V == 0) | (W == 0)
        if z.any():
            U[z] = (Cx[z].astype(np.float64) * By[z] - Cy[z].astype(np.float64) * Bx[z]).astype(f)
            V[z] = (Ax[z].astype(np.float64) * Cy[z] - Ay[z].astype(np.float64) * Cx[z]).astype(f)
            W[z] = (Bx[z].astype(np.float64) * Ay[z] - By[z].astype(np.float64) * Ax[z]).astype(f)
        inside = ~(((U < 0) | (V < 0) | (W < 0)) & ((U > 0) | (V > 0) | (W > 0)))
        det = (U + V) + W
        ok = inside & (det != 0)
        T = (U * (Sz * A[:, kz]) + V * (Sz * B[:, kz])) + W * (Sz * C[:, kz])
        with np.errstate(divide="ignore", invalid="ignore"):
            t = T * (f(1.0) / det)
        ok &= (t > tmin) & (t <= rays[i, 7])
        if ok.any():
            cand = np.nonzero(ok)[0]
            tt = t[cand]
            best = tt.min()
            prim = cand[tt == best].min()
            out_t[i] = best
            out_p[i] = prim
    return out_t, out_p


def small_scene(bsm, spheres=6, seed=3):
    return bsm.generate_scene(bsm.BSM_SCENE_ROOM, seed=seed, spheres=spheres, width=32, height=32)


def test_oracle_closest_hit_equals_brute_force(bsm, oracle):
    sc = small_scene(bsm)
    tris = sc.positions[sc.indices].astype(np.float32)
    rays = random_rays(3000, -0.2, 1.2, seed=11)
    # axis-aligned rays through box corners and edges
    rays[:300, 4:7] = [0.0, -1.0, 0.0]
    rays[300:600, 4:7] = [1.0, 0.0, 0.0]
    osc = oracle.OracleScene(sc)
    h = osc.trace(rays)
    t, p = watertight_brute(tris, rays)
    assert np.array_equal(h[:, 1], p)
    assert np.array_equal(h[:, 0].view(np.float32), t)


def test_oracle_any_hit_consistent_with_closest(bsm, oracle):
    sc = small_scene(bsm, seed=5)
    osc = oracle.OracleScene(sc)
    rays = random_rays(20000, -0.2, 1.2, seed=12, tmax=0.25)
    c = osc.trace(rays)
    a = osc.trace(rays, any_hit=True)
    assert np.array_equal(c[:, 1] != 0xFFFFFFFF, a[:, 1] != 0xFFFFFFFF)


def test_zero_direction_ray_is_a_miss(bsm, oracle):
    osc = oracle.OracleScene(small_scene(bsm))
    rays = np.array([[0.5, 0.5, 0.5, 0.0, 0.0, 0.0, 0.0, 100.0]], np.float32)
    assert osc.trace(rays)[0, 1] == 0xFFFFFFFF


def test_oracle_render_is_deterministic_and_finite(bsm, oracle):
    sc = small_scene(bsm, spheres=10)
    osc = oracle.OracleScene(sc)
    cam = sc.camera.as_array()
    a, sa, _ = osc.render(cam, spp=2, max_segments=4, seed=9, threads=3)
    b, sb, _ = osc.render(cam, spp=2, max_segments=4, seed=9, threads=1)
    assert np.isfinite(a).all()
    assert np.array_equal(sa, sb)
    assert np.abs(a - b).max() <= 1e-5 * max(1.0, float(np.abs(a).max()))
    assert sa[0] == 32 * 32 * 2


def test_oracle_fixed_point_sums(bsm, oracle):
    """F_FIXED (64, the library's BSM_PT_DETERMINISTIC): exact 32.32 fixed-point pixel sums; the image equals
    the FP32-sum image within the quantisation and does not depend on threads or on a split into row bands."""
    sc = small_scene(bsm, spheres=10)
    osc = oracle.OracleScene(sc)
    cam = sc.camera.as_array()
    f, sf, _ = osc.render(cam, spp=3, max_segments=4, seed=9, flags=64, threads=3)
    g, _, _ = osc.render(cam, spp=3, max_segments=4, seed=9, flags=64, threads=1)
    top, _, _ = osc.render(cam, spp=3, max_segments=4, seed=9, flags=64, rows=(0, 13))
    bottom, _, _ = osc.render(cam, spp=3, max_segments=4, seed=9, flags=64, rows=(13, 32))
    a, sa, _ = osc.render(cam, spp=3, max_segments=4, seed=9)
    assert np.array_equal(f.view(np.uint32), g.view(np.uint32))
    assert np.array_equal(f.view(np.uint32), np.concatenate([top, bottom]).view(np.uint32))
    assert np.array_equal(sf, sa)
    err = np.abs(f[..., :3].astype(np.float64) - a[..., :3]) / np.maximum(np.abs(a[..., :3]), 1e-3)
    assert err.max() <= 1e-6 and f[..., :3].mean() > 0.0


@pytest.mark.parametrize("flags", [0, 1, 2, 4, 6])
def test_oracle_render_flags(bsm, oracle, flags):
    sc = small_scene(bsm, spheres=4, seed=2)
    osc = oracle.OracleScene(sc)
    img, st, _ = osc.render(sc.camera.as_array(), spp=1, max_segments=3, seed=1, flags=flags)
    assert np.isfinite(img).all() and (img[..., :3] >= 0).all()
    if flags & 6 == 6:
        assert st[16:].sum() == 0    # no shadow rays without sun and sky NEE


def test_oracle_ties_at_shared_vertices_equal_brute_force(bsm, oracle):
    """Vertical rays through terrain grid vertices hit up to six triangles at
    (nearly) the same t; the BVH must keep every candidate box."""
    g = 24
    sc = bsm.generate_scene(bsm.BSM_SCENE_TERRAIN, seed=2, grid=g, spheres=5, sky_width=64, sky_height=32)
    rng = np.random.default_rng(9)
    n = 3000
    ij = rng.integers(0, g, (n, 2))
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0] = ij[:, 0] / np.float32(g - 1)
    rays[:, 2] = ij[:, 1] / np.float32(g - 1)
    rays[:, 1] = 0.4
    rays[:, 5] = -1.0
    rays[:, 7] = 10.0
    h = oracle.OracleScene(sc).trace(rays)
    t, p = watertight_brute(sc.positions[sc.indices].astype(np.float32), rays)
    assert np.array_equal(h[:, 1], p)


def test_sky_alias_sampling_matches_its_pdf(bsm, oracle):
    """Texels are chosen with the probabilities the sky's weights give (chi-square over texels), and the
    returned pdf equals sky_pdf of the sampled direction."""
    sc = bsm.generate_scene(bsm.BSM_SCENE_TERRAIN, seed=5, grid=16, spheres=4, sky_width=32, sky_height=16)
    osc = oracle.OracleScene(sc)
    n = 400000
    u = np.random.default_rng(1).uniform(0.0, 1.0, (n, 3)).astype(np.float32)
    s = osc.sky_sample(u)
    d, pdf, pdf2 = s[:, :3].astype(np.float64), s[:, 3], s[:, 4]
    ok = pdf > 0
    assert ok.mean() > 0.999
    # a direction rounded onto a texel boundary may be looked up in the neighbouring texel
    assert np.mean(np.abs(pdf[ok] - pdf2[ok]) > 1e-5 * pdf2[ok]) < 1e-4
    # texel of each direction (row from theta about +y, column from phi = atan2(z, x))
    H, W = 16, 32
    th = np.arccos(np.clip(d[:, 1], -1, 1))
    ph = np.arctan2(d[:, 2], d[:, 0])
    i = np.clip((th / np.pi * H).astype(int), 0, H - 1)
    j = np.clip(((ph / (2 * np.pi) + 0.5) * W).astype(int), 0, W - 1)
    counts = np.bincount(i * W + j, minlength=H * W).astype(np.float64)
    # texel probabilities from the sky's own weights (r + g + b) * sin(theta at the row centre)
    tex = sc.sky_texels.view(np.float16).astype(np.float64)
    w = tex[..., :3].sum(-1) * np.sin(np.pi * (np.arange(H) + 0.5) / H)[:, None]
    p = (w / w.sum()).ravel()
    expect = p * n
    m = expect > 20
    chi2 = float(((counts[m] - expect[m]) ** 2 / expect[m]).sum())
    assert chi2 < 1.3 * m.sum(), (chi2, m.sum())


def test_edge_cases_of_the_traversal(bsm, oracle):
    """Coincident triangles resolve to the lower primitive id, zero-area
    triangles are never hit, shared edges and vertices do not leak, and rays
    with a non-finite component or an empty interval are misses — in the
    oracle's binary BVH and in its restatement of the device traversal over
    the product's compressed BVH alike."""
    from edge_scenes import MISS, coincident_scene, edge_rays, grid_scene, invalid_rays, rays_along_z
    sc = coincident_scene(bsm)
    osc = oracle.OracleScene(sc)
    nb, tb, _ = bsm.bvh_build_host(sc)
    rays = rays_along_z(4000, seed=3)
    h = osc.trace(rays)
    hc, _ = oracle.cwbvh_trace(nb, tb, rays)
    assert np.array_equal(h[:, :2], hc[:, :2])
    in_front = rays[:, 0] + rays[:, 1] < 1.0           # inside the front triangle
    assert (h[in_front, 1] == 1).all()
    assert set(np.unique(h[~in_front, 1]).tolist()) <= {0, 5, 1}
    assert not np.isin(h[:, 1], [2, 3, 4]).any()
    occ = osc.trace(rays, any_hit=True)[:, 1] != MISS
    assert occ.all()
    g = grid_scene(bsm)
    er = edge_rays()
    og = oracle.OracleScene(g)
    gh = og.trace(er)
    assert (gh[:, 1] != MISS).all(), "a ray through a shared edge or vertex leaked"
    gnb, gtb, _ = bsm.bvh_build_host(g)
    assert np.array_equal(oracle.cwbvh_trace(gnb, gtb, er)[0][:, :2], gh[:, :2])
    bad = invalid_rays()
    assert (osc.trace(bad)[:, 1] == MISS).all()
    assert (osc.trace(bad, any_hit=True)[:, 1] == MISS).all()
    assert (oracle.cwbvh_trace(nb, tb, bad)[0][:, 1] == MISS).all()
    # an infinite tmax is a valid interval
    inf_tmax = rays_along_z(100, seed=4)
    inf_tmax[:, 7] = np.inf
    assert np.array_equal(osc.trace(inf_tmax)[:, 1], osc.trace(rays_along_z(100, seed=4))[:, 1])
