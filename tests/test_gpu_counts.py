"""Traversal counters on the GPU against the oracle.

The bench's traversal-bytes figure (80 B per node visited + 48 B per
triangle tested) rests on the device's per-ray counters.  The oracle's
restatement of the device traversal, run over the BVH bytes downloaded from
the device, must visit the same nodes and test the same triangles for every
ray (exact counts), and find the same hits."""
import numpy as np
import pytest

from conftest import random_rays

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("collapse", [0, 1])
def test_counts_and_hits_match_oracle_traversal(bsm, ctx, oracle, collapse):
    sc = bsm.generate_scene(bsm.BSM_SCENE_TERRAIN, seed=3, grid=128, spheres=300, sky_width=64, sky_height=32,
                            width=64, height=36)
    sid = ctx.upload(sc)
    st = ctx.build_bvh(sid, collapse=collapse)
    nb, tb = ctx.download_bvh(sid, st)
    short = random_rays(20000, -1.0, 1.0, seed=32, tmax=0.5)
    short[:, 3] = 1e-3
    # rays along the axes (exactly zero direction components)
    axis = random_rays(3000, -1.0, 1.0, seed=33)
    axis[:, 4:7] = np.eye(3, dtype=np.float32)[np.arange(3000) % 3] * np.where(np.arange(3000) % 2, 1, -1)[:, None]
    rays = np.concatenate([random_rays(20000, -1.0, 1.0, seed=31), short, axis])
    g_cnt = ctx.trace_counts(sid, rays)
    g_hit = ctx.trace_closest(sid, rays)
    o_hit, o_cnt = oracle.cwbvh_trace(nb, tb, rays)
    assert np.array_equal(g_cnt, o_cnt), f"{int((g_cnt != o_cnt).any(1).sum())} rays count differently"
    assert np.array_equal(g_hit[:, :2], o_hit[:, :2])
    # and the oracle's own binary BVH agrees on the hits
    ref = oracle.OracleScene(sc).trace(rays)
    assert np.array_equal(o_hit[:, 1], ref[:, 1])
    ctx.release(sid)
