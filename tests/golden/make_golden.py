"""Generates tests/golden/bsdf_golden.npz, gbuffer_golden.npz and
lights_golden.npz from the reference's own shader math.

The reference's material / frame / sampling HLSL files (bisemutum/shaders/core/
material/utils.hlsl, lit.hlsl, core/utils/frame.hlsl, sampling.hlsl, math.hlsl)
its G-buffer packing (renderer/gbuffer.hlsl pack_surface_to_gbuffer with the
helpers of core/utils/pack.hlsl) and its light evaluation (renderer/lights.hlsl
dir_light_eval and point_light_eval) are compiled from their sources by
oracle/build.py (through a C++ HLSL shim) and evaluated here on seeded inputs.
Needs the reference tree; the committed .npz files are what the tests read.

    python tests/golden/make_golden.py            # all three files
    python tests/golden/make_golden.py lights     # one of them
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402


def unit(v):
    return v / np.linalg.norm(v, axis=-1, keepdims=True)


def store_gbuffer_formats(g):
    """What the reference's G-buffer textures hold after a store of the packed floats: base colour and
    normal/roughness rgba16_sfloat, fresnel rgba16_unorm, material_0 rgba8_unorm (round to nearest)."""
    q = np.array(g, np.float32).reshape(-1, 16).copy()
    q[:, 0:8] = q[:, 0:8].astype(np.float16).astype(np.float32)
    q[:, 8:12] = (np.round(np.clip(q[:, 8:12], 0, 1) * 65535.0) / 65535.0).astype(np.float32)
    q[:, 12:16] = (np.round(np.clip(q[:, 12:16], 0, 1) * 255.0) / 255.0).astype(np.float32)
    return np.ascontiguousarray(q)


def gbuffer(R):
    """pack_surface_to_gbuffer on random surfaces plus the octahedral fold's edge cases."""
    rng = np.random.default_rng(20240602)
    n = 2048
    N = unit(rng.normal(size=(n, 3)))
    # edge cases: axes (both signs), the equator (z = 0), the fold's diagonals
    special = np.array([[0, 0, 1], [0, 0, -1], [1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0],
                        [1, 1, 0], [-1, 1, 0], [1, -1, 0], [-1, -1, 0], [1, 1, -1], [-1, -1, -1],
                        [0.6, 0, -0.8], [0, -0.6, -0.8]], np.float64)
    N[:len(special)] = unit(special)
    V = unit(rng.normal(size=(n, 3)))
    # tangents: in the plane of N (as a triangle edge is), some arbitrary, one per frame axis
    R3 = unit(rng.normal(size=(n, 3)))
    T = unit(R3 - np.sum(R3 * N, 1, keepdims=True) * N)
    T[n // 2:n // 2 + 128] = R3[n // 2:n // 2 + 128]
    base = rng.uniform(0.0, 1.0, (n, 3))
    base[:8] = [[0, 0, 0], [1, 1, 1], [0.5, 0.5, 0.5], [1, 0, 0], [0, 1, 0], [0, 0, 1], [0.04, 0.04, 0.04],
                [0.999, 0.001, 0.5]]
    metal = (rng.uniform(size=(n, 1)) < 0.4).astype(np.float64)
    f0 = 0.04 + (base - 0.04) * metal
    rough = rng.uniform(0.0, 1.0, (n, 1))
    g_in = np.concatenate([V, N, T, base, f0, rough], 1).astype(np.float32)
    g_out = np.zeros((n, 16), np.float32)
    R.ref_gbuffer(g_in.ctypes.data, n, g_out.ctypes.data)
    # the reference's own decoder on its packing after the texture stores of its G-buffer formats
    # (renderer/context/gbuffer.hpp:14-17): N T base f0 f90 roughness anisotropy ior model
    q = store_gbuffer_formats(g_out)
    unpacked = np.zeros((n, 20), np.float32)
    R.ref_gbuffer_unpack(q.ctypes.data, n, unpacked.ctypes.data)
    out = os.path.join(HERE, "gbuffer_golden.npz")
    np.savez_compressed(out, gbuffer_in=g_in, gbuffer_out=g_out, unpacked=unpacked[:, :19])
    print("wrote", out, os.path.getsize(out), "bytes")


def lights(R):
    """point_light_eval on random point and spot lights (range falloff, spot ramp inside, on the edges of and
    outside the cone, points beyond the range and nearer than sqrt(0.001)) and dir_light_eval."""
    rng = np.random.default_rng(20240603)
    n = 4096
    pos = rng.uniform(-2.0, 2.0, (n, 3))
    emis = rng.uniform(0.1, 5.0, (n, 3))
    rng_ = rng.uniform(0.2, 4.0, (n, 1))
    axis = unit(rng.normal(size=(n, 3)))
    outer = rng.uniform(0.1, 1.4, (n, 1))
    inner = outer * rng.uniform(0.0, 1.0, (n, 1))
    spot = rng.uniform(size=(n, 1)) < 0.6
    ci = np.where(spot, np.cos(inner), 0.0)
    co = np.where(spot, np.cos(outer), 0.0)
    P = pos + unit(rng.normal(size=(n, 3))) * rng.uniform(0.0, 1.0, (n, 1)) * rng_ * 1.3
    P[:64] = pos[:64] + unit(rng.normal(size=(64, 3))) * 0.01          # closer than sqrt(0.001)
    # points on the cone's edges: the direction from the light to P at the inner / outer angle
    k = slice(64, 192)
    t = unit(np.cross(axis[k], rng.normal(size=(128, 3))))
    ang = np.where(np.arange(128)[:, None] % 2 == 0, inner[k], outer[k])
    d_from_light = -(axis[k] * np.cos(ang) + t * np.sin(ang))          # axis points to the light
    P[k] = pos[k] + d_from_light * rng.uniform(0.1, 1.0, (128, 1)) * rng_[k]
    spot[k] = True
    ci[k], co[k] = np.cos(inner[k]), np.cos(outer[k])
    pin = np.concatenate([pos, emis, rng_, axis, ci, co, P, np.zeros((n, 1))], 1).astype(np.float32)
    pout = np.zeros((n, 6), np.float32)
    R.ref_point_light(pin.ctypes.data, n, pout.ctypes.data)
    din = np.concatenate([unit(rng.normal(size=(256, 3))), rng.uniform(0.0, 4.0, (256, 3)),
                          rng.uniform(-1, 1, (256, 3))], 1).astype(np.float32)
    dout = np.zeros((256, 6), np.float32)
    R.ref_dir_light(din.ctypes.data, 256, dout.ctypes.data)
    out = os.path.join(HERE, "lights_golden.npz")
    np.savez_compressed(out, point_in=pin, point_out=pout, dir_in=din, dir_out=dout)
    print("wrote", out, os.path.getsize(out), "bytes")


def main(which=("bsdf", "gbuffer", "lights")):
    R = oracle.ref_lib()
    if R is None:
        raise SystemExit("reference tree not present: cannot regenerate the golden vectors")
    if "gbuffer" in which:
        gbuffer(R)
    if "lights" in which:
        lights(R)
    if "bsdf" not in which:
        return
    rng = np.random.default_rng(20240601)
    n = 4096
    # surface_eval_lit inputs: N, V, L on the upper side of N, base, f0, roughness
    N = unit(rng.normal(size=(n, 3)))
    V = unit(rng.normal(size=(n, 3)))
    L = unit(rng.normal(size=(n, 3)))
    V = np.where((np.sum(V * N, 1) < 0)[:, None], -V, V)
    L = np.where((np.sum(L * N, 1) < 0)[:, None], -L, L)
    base = rng.uniform(0.1, 0.9, (n, 3))
    metal = (rng.uniform(size=(n, 1)) < 0.3).astype(np.float64)
    f0 = 0.04 + (base - 0.04) * metal
    rough = rng.uniform(0.05, 1.0, (n, 1))
    lit_in = np.concatenate([N, V, L, base, f0, rough], 1).astype(np.float32)
    lit_out = np.zeros((n, 3), np.float32)
    R.ref_eval_lit(lit_in.ctypes.data, n, lit_out.ctypes.data)
    # VNDF sample + pdf: local view on the upper hemisphere
    v = unit(rng.normal(size=(n, 3)))
    v[:, 2] = np.abs(v[:, 2]) + 1e-3
    v = unit(v)
    r = rng.uniform(0.05, 1.0, n) ** 2
    r = np.maximum(r, 0.001)
    u = rng.uniform(0.0, 1.0, (n, 2))
    vndf_in = np.concatenate([v, r[:, None], r[:, None], u], 1).astype(np.float32)
    vndf_out = np.zeros((n, 4), np.float32)
    R.ref_vndf(vndf_in.ctypes.data, n, vndf_out.ctypes.data)
    # frames
    fr_in = unit(rng.normal(size=(n, 3))).astype(np.float32)
    fr_out = np.zeros((n, 6), np.float32)
    R.ref_frame(fr_in.ctypes.data, n, fr_out.ctypes.data)
    # anisotropic roughness (anisotropy 0) and samplers
    an_in = rng.uniform(0.0, 1.0, n).astype(np.float32)
    an_out = np.zeros((n, 2), np.float32)
    R.ref_aniso(an_in.ctypes.data, n, an_out.ctypes.data)
    sm_in = rng.uniform(0.0, 1.0, (n, 2)).astype(np.float32)
    sm_out = np.zeros((n, 6), np.float32)
    R.ref_samplers(sm_in.ctypes.data, n, sm_out.ctypes.data)
    inv_pi = np.float32(R.ref_inv_pi())
    out = os.path.join(HERE, "bsdf_golden.npz")
    np.savez_compressed(out, lit_in=lit_in, lit_out=lit_out, vndf_in=vndf_in, vndf_out=vndf_out, frame_in=fr_in,
                        frame_out=fr_out, aniso_in=an_in, aniso_out=an_out, samplers_in=sm_in,
                        samplers_out=sm_out, inv_pi=inv_pi)
    print("wrote", out, os.path.getsize(out), "bytes")


if __name__ == "__main__":
    R_ = C  # keep ctypes imported for the loaded library's argtypes
    main(tuple(sys.argv[1:]) or ("bsdf", "gbuffer", "lights"))
