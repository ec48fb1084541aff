"""Primary-hit outputs (depth, G-buffer, hit positions) on the CPU.

* G-buffer packing: the oracle's restatement against golden vectors made by the
  reference's own pack_surface_to_gbuffer (renderer/gbuffer.hlsl:18-31 with
  core/utils/pack.hlsl), bit for bit, including the octahedral fold's edge cases;
* the reference's own decoder (unpack_gbuffer_to_surface), run on that packing
  after the stores into its G-buffer texture formats, recovers the surface;
* the oracle's primary outputs are self-consistent: hit position = eye + t dir,
  reverse-Z depth of pt_depth.hlsl, misses where the first segment sees the sky.
"""
import os

import numpy as np

GOLD = os.path.join(os.path.dirname(__file__), "golden", "gbuffer_golden.npz")


def test_gbuffer_pack_matches_reference_golden(oracle):
    g = np.load(GOLD)
    out = oracle.gbuffer_pack(g["gbuffer_in"])
    assert np.array_equal(out, g["gbuffer_out"])


def test_reference_decoder_recovers_the_surface(oracle):
    g = np.load(GOLD)
    gi, u = g["gbuffer_in"], g["unpacked"]
    N, T = gi[:, 3:6], gi[:, 6:9]
    assert np.abs(u[:, 0:3] - N).max() < 2e-3                      # normal through fp16 + octahedral map
    inplane = np.abs(np.sum(T * N, 1)) < 1e-5
    assert np.abs(u[inplane, 3:6] - T[inplane]).max() < 3e-3         # tangent in the normal's plane
    assert np.abs(u[:, 6:9] - gi[:, 9:12]).max() < 1e-3              # base colour (fp16)
    assert np.abs(u[:, 15] - gi[:, 15]).max() < 1e-3                 # roughness (fp16)
    assert np.all(u[:, 16] == 0.0) and np.allclose(u[:, 17], 1.5, atol=1e-3)
    assert np.all(u[:, 18] == 1.0)                                   # MATERIAL_SURFACE_MODEL_LIT
    # f0 / f90 through rg11b10 in two unorm16 halves: the reference packs x / 65536 and unpacks
    # trunc(x * 65535.5), which for a large high half can move bit 16 (g's bit 5); all other
    # cases are within the 11/10-bit steps
    e = np.abs(u[:, 9:12] - gi[:, 12:15]).max(1)
    assert np.mean(e < 0.02) > 0.99
    assert np.abs(u[:, 12:15] - 1.0).max() < 0.02


def room(bsm, w=64, h=48):
    sc = bsm.generate_scene(bsm.BSM_SCENE_ROOM, seed=4, spheres=12, width=w, height=h)
    return sc


def test_oracle_primary_outputs_are_consistent(bsm, oracle):
    sc = room(bsm)
    osc = oracle.OracleScene(sc)
    cam = sc.camera.as_array()
    near, far = 0.01, 10000.0
    depth, gb, hp = osc.primary(cam, near_z=near, far_z=far, threads=2)
    hit = hp[..., 3] > 0.0
    miss = ~hit
    assert hit.any() and np.all(hp[miss, 3] == -1.0)
    # misses: unit direction, zero depth and G-buffer
    assert np.allclose(np.linalg.norm(hp[miss, :3], axis=-1), 1.0, atol=1e-6)
    assert np.all(depth[miss] == 0.0) and np.all(gb[:, miss] == 0.0)
    # hits: reverse-Z depth of the hit position's view distance, in (0, 1]
    eye = cam[0:3].astype(np.float64)
    f = cam[3:6].astype(np.float64)
    f /= np.linalg.norm(f)
    P = hp[hit, :3].astype(np.float64)
    d = (P - eye) @ f
    expect = near * (far - d) / ((far - near) * d)
    assert np.allclose(depth[hit], expect, rtol=1e-5)
    assert np.all((depth[hit] > 0.0) & (depth[hit] <= 1.0))
    # |P - eye| = t (unit directions)
    assert np.allclose(np.linalg.norm(P - eye, axis=-1), hp[hit, 3], rtol=1e-5)
    # G-buffer: base colour alpha 1, lit model, ior 1.5, normal faces the camera
    assert np.all(gb[0][hit][:, 3] == 1.0)
    assert np.all(gb[3][hit][:, 3] == np.float32(1.0 / 256.0))
    assert np.all(gb[3][hit][:, 1] == np.float32(1.0 / 1.5))
    o = gb[1][hit][:, :2].astype(np.float64)
    n = np.stack([o[:, 0], o[:, 1], 1.0 - np.abs(o[:, 0]) - np.abs(o[:, 1])], -1)
    t = np.clip(-n[:, 2], 0.0, 1.0)
    n[:, 0] += np.where(n[:, 0] >= 0.0, -t, t)
    n[:, 1] += np.where(n[:, 1] >= 0.0, -t, t)
    n /= np.linalg.norm(n, axis=-1, keepdims=True)
    assert np.all(np.sum(n * (P - eye), -1) <= 1e-6)


def test_oracle_primary_misses_are_where_the_first_segment_sees_the_sky(bsm, oracle):
    sc = bsm.generate_scene(bsm.BSM_SCENE_TERRAIN, seed=2, grid=32, spheres=20, sky_width=64, sky_height=32,
                            width=48, height=32)
    osc = oracle.OracleScene(sc)
    cam = sc.camera.as_array()
    _, _, hp = osc.primary(cam)
    # one segment, no next-event estimation: a pixel is lit only when its primary ray escapes
    img, _, _ = osc.render(cam, spp=1, max_segments=1, flags=6)
    lit = img[..., :3].max(-1) > 0.0
    assert np.array_equal(lit, hp[..., 3] < 0.0)
