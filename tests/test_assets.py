"""The reference's on-disk formats (no GPU): .static_mesh.biasset, TOML, projects.

* meshes round-trip through the library's writer and reader (versions 1 and 2);
* version-2 files compressed by Python's zlib (fixed and dynamic Huffman
  blocks, levels 0-9) read back exactly, and the library's zlib stream
  decompresses with Python's zlib: the DEFLATE decoder and the container agree
  with an independent implementation of the format written here with struct;
* truncated, corrupt and foreign files are rejected;
* the TOML reader accepts the constructs the reference's files use and rejects
  malformed text;
* a synthetic project (parents, shared meshes, submeshes, materials, lights,
  camera, renderer override) loads into the expected world-space scene;
* where the reference tree is present, its example project's meshes equal the
  independent reader's arrays and the project loads.
"""
import os
import struct
import zlib

import numpy as np
import pytest

REF_EXAMPLE = os.path.join(os.environ.get("BSM_REFERENCE_ROOT", "/root/reference"), "examples/scene_basic")
MAGIC = 0x0B1A55E7


# ---- an independent writer / reader of the format (struct + zlib) ----
def body_bytes(m):
    out = b""
    for name, comps, fmt in [("positions", 3, "f"), ("normals", 3, "f"), ("tangents", 4, "f"), ("colors", 3, "f"),
                             ("texcoords", 2, "f"), ("texcoords2", 2, "f"), ("indices", 1, "I")]:
        a = np.asarray(m.get(name, np.zeros((0, comps))), np.float32 if fmt == "f" else np.uint32)
        a = a.reshape(-1, comps) if comps > 1 else a.ravel()
        out += struct.pack("<Q", a.shape[0]) + a.tobytes()
    sub = np.asarray(m.get("submeshes", np.zeros((0, 4))), np.uint32).reshape(-1, 4)
    out += struct.pack("<Q", sub.shape[0])
    for s in sub:
        out += struct.pack("<IIIB3x", int(s[0]), int(s[1]), int(s[2]), int(s[3]))
    return out


def file_bytes(m, version=2, level=6, type_name=b"StaticMesh"):
    head = struct.pack("<I", MAGIC) + struct.pack("<Q", len(type_name)) + type_name + struct.pack("<I", version)
    body = body_bytes(m)
    if version == 1:
        return head + body
    z = zlib.compress(body, level)
    return head + struct.pack("<QQ", len(body), len(z)) + z


def parse_independent(data):
    magic, = struct.unpack_from("<I", data, 0)
    n, = struct.unpack_from("<Q", data, 4)
    name = data[12:12 + n]
    version, = struct.unpack_from("<I", data, 12 + n)
    off = 16 + n
    assert magic == MAGIC and name == b"StaticMesh"
    if version == 2:
        ln, cl = struct.unpack_from("<QQ", data, off)
        body = zlib.decompress(data[off + 16:off + 16 + cl])
        assert len(body) == ln
    else:
        body = data[off:]
    out, p = {}, 0
    for name, comps, dt in [("positions", 3, np.float32), ("normals", 3, np.float32), ("tangents", 4, np.float32),
                            ("colors", 3, np.float32), ("texcoords", 2, np.float32), ("texcoords2", 2, np.float32),
                            ("indices", 1, np.uint32)]:
        k, = struct.unpack_from("<Q", body, p)
        p += 8
        a = np.frombuffer(body, dt, k * comps, p)
        p += 4 * k * comps
        out[name] = a.reshape(-1, comps) if comps > 1 else a.copy()
    k, = struct.unpack_from("<Q", body, p)
    p += 8
    sub = [struct.unpack_from("<IIIB3x", body, p + 16 * i) for i in range(k)]
    out["submeshes"] = np.array(sub, np.uint32).reshape(-1, 4)
    return out


def random_mesh(seed, nv=300, ntri=500, nsub=3):
    rng = np.random.default_rng(seed)
    m = {"positions": rng.normal(size=(nv, 3)).astype(np.float32),
         "normals": rng.normal(size=(nv, 3)).astype(np.float32),
         "tangents": rng.normal(size=(nv, 4)).astype(np.float32),
         "texcoords": rng.uniform(size=(nv, 2)).astype(np.float32),
         "indices": rng.integers(0, nv, 3 * ntri).astype(np.uint32)}
    cuts = np.sort(rng.choice(np.arange(1, ntri), nsub - 1, replace=False)) * 3
    starts = np.concatenate([[0], cuts])
    ends = np.concatenate([cuts, [3 * ntri]])
    m["submeshes"] = np.array([[0, s, e - s, 3] for s, e in zip(starts, ends)], np.uint32)
    return m


def same_mesh(a, b):
    for k in ["positions", "normals", "tangents", "colors", "texcoords", "texcoords2", "indices", "submeshes"]:
        x = np.asarray(a.get(k, []))
        y = np.asarray(b.get(k, []))
        if x.size == 0 and y.size == 0:
            continue
        if x.shape != y.shape or not np.array_equal(x.view(np.uint32) if x.dtype == np.float32 else x,
                                                     y.view(np.uint32) if y.dtype == np.float32 else y):
            return False
    return True


def test_mesh_round_trip_through_the_library(bsm):
    m = random_mesh(1)
    for version in (1, 2):
        data = bsm.write_static_mesh(m, version)
        assert same_mesh(bsm.read_static_mesh(data), m)
        assert same_mesh(parse_independent(data), m)    # the library's file reads with zlib + struct


@pytest.mark.parametrize("level", [0, 1, 6, 9])
def test_python_zlib_streams_read_exactly(bsm, level):
    for seed, nv in [(2, 5), (3, 300), (4, 5000)]:
        m = random_mesh(seed, nv=nv, ntri=2 * nv, nsub=2)
        m["positions"][: nv // 2] = 0.25            # repeated bytes: long back-references
        assert same_mesh(bsm.read_static_mesh(file_bytes(m, 2, level)), m)
    assert same_mesh(bsm.read_static_mesh(file_bytes(m, 1)), m)


def test_empty_mesh_and_non_indexed_submesh(bsm):
    m = {"positions": np.zeros((0, 3), np.float32), "submeshes": np.zeros((0, 4), np.uint32)}
    out = bsm.read_static_mesh(file_bytes(m, 2))
    assert out["positions"].shape == (0, 3) and out["submeshes"].shape == (0, 4)
    m = {"positions": np.arange(18, dtype=np.float32).reshape(6, 3),
         "submeshes": np.array([[0, 0, 0xFFFFFFFF, 3]], np.uint32)}
    out = bsm.read_static_mesh(bsm.write_static_mesh(m, 2))
    assert out["indices"].shape == (0,) and out["submeshes"][0, 2] == 0xFFFFFFFF


def test_corrupt_files_are_rejected(bsm):
    m = random_mesh(5, nv=64, ntri=40)
    good = file_bytes(m, 2, 9)
    bad = [good[:10], good[:len(good) // 2], good[:-3],
           struct.pack("<I", 0x12345678) + good[4:],                 # magic
           file_bytes(m, 2, 9, type_name=b"TextureAsset"),            # another asset type
           good[:16 + 10] + struct.pack("<I", 7) + good[16 + 14:]]    # version 7
    z = bytearray(good)
    z[-1] ^= 0xFF                                                     # Adler-32
    bad.append(bytes(z))
    z = bytearray(good)
    z[60] ^= 0x55                                                     # deflate data
    bad.append(bytes(z))
    v1 = bytearray(file_bytes(m, 1))
    v1[16 + 10:16 + 18] = struct.pack("<Q", 1 << 40)                  # absurd array length
    bad.append(bytes(v1))
    for b in bad:
        with pytest.raises(bsm.BsmError):
            bsm.read_static_mesh(b)


def test_toml_reader(bsm):
    ok = ["a = 1\nb = 'x'\nc = \"y\\n\\u00e9\"\n",
          "[t]\nx = [ 1.0, -2.5e-3, +3 ]\n[[arr]]\nk = true\n[[arr]]\nk = false\n",
          "[[objects]]\nname = 'A'\n    [[objects.components]]\n    type = 'T'\n"
          "        [objects.components.value]\n        v = [ 1, 2, 3 ]\n"
          "            [[objects.components.value.materials]]\n            asset_id = 4\n",
          "f = '''line one\nline two\n'''\ng = { a = 1, b = { c = [1, 2] } }\n# comment\n",
          "x.y.z = 1_000\nw = [\n  1,\n  2, # two\n]\n"]
    for t in ok:
        bsm.toml_check(t)
    for t, frag in [("a = \n", "line 1"), ("a = 1\na = 2\n", "line 2"), ("[t\n", "line 1"), ("a = [1, 2\n", ""),
                    ("a = 'unterminated\n", "line 1"), ("= 3\n", "line 1"), ("a = 1 2\n", "line 1")]:
        with pytest.raises(bsm.BsmError) as e:
            bsm.toml_check(t)
        assert frag in str(e.value)


# ---- projects ----
def euler_zxy(deg):
    x, y, z = np.radians(deg)
    Rz = np.array([[np.cos(z), -np.sin(z), 0], [np.sin(z), np.cos(z), 0], [0, 0, 1]])
    Rx = np.array([[1, 0, 0], [0, np.cos(x), -np.sin(x)], [0, np.sin(x), np.cos(x)]])
    Ry = np.array([[np.cos(y), 0, np.sin(y)], [0, 1, 0], [-np.sin(y), 0, np.cos(y)]])
    return Rz @ Rx @ Ry


def affine(t, r, s):
    M = np.eye(4)
    M[:3, :3] = euler_zxy(r) * np.asarray(s)[None, :]
    M[:3, 3] = t
    return M


def quad_mesh(normals=False):
    # two submeshes: a unit quad in y = 0 and a triangle above it; optionally with bent vertex normals
    pos = np.array([[-1, 0, -1], [1, 0, -1], [1, 0, 1], [-1, 0, 1], [0, 1, 0], [1, 1, 0], [0, 1, 1]], np.float32)
    idx = np.array([0, 2, 1, 0, 3, 2, 0, 1, 2], np.uint32)
    m = {"positions": pos, "indices": idx, "submeshes": np.array([[0, 0, 6, 3], [4, 6, 3, 3]], np.uint32)}
    if normals:
        n = pos * np.array([0.4, 0.0, 0.4], np.float32) + np.array([0.0, 1.0, 0.0], np.float32)
        n[4:] = [[0.2, 0.3, 1.0], [-0.3, 0.1, 1.0], [0.1, -0.2, 1.0]]
        m["normals"] = (n / np.linalg.norm(n, axis=1, keepdims=True)).astype(np.float32)
    return m


def write_project(root, bsm, normals=False):
    os.makedirs(os.path.join(root, "meshes"))
    os.makedirs(os.path.join(root, "materials"))
    with open(os.path.join(root, "meshes", "q.static_mesh.biasset"), "wb") as f:
        f.write(bsm.write_static_mesh(quad_mesh(normals), 2))
    with open(os.path.join(root, "project.toml"), "w") as f:
        f.write('name = "T"\nasset_metadata_file = "/project/meta.toml"\nscene_file = "/project/scene.toml"\n'
                'renderer = "BasicRenderer"\n')
    with open(os.path.join(root, "meta.toml"), "w") as f:
        f.write("[[assets]]\nid = 0\npath = '/project/meshes/q.static_mesh.biasset'\ntype = 'StaticMesh'\n"
                "[[assets]]\nid = 1\npath = '/project/materials/red.toml'\ntype = 'Material'\n"
                "[[assets]]\nid = 2\npath = '/project/materials/gold.toml'\ntype = 'Material'\n"
                "[[assets]]\nid = 3\npath = '/project/materials/fancy.toml'\ntype = 'Material'\n")
    with open(os.path.join(root, "materials", "red.toml"), "w") as f:
        f.write("blend_mode = 'opaque'\nmaterial_function = '''surface.base_color = PARAM_base_color;\n"
                "surface.roughness = 0.25;\n'''\nsurface_model = 'lit'\n\n[[params]]\nname = 'base_color'\n"
                "value = [ 0.9, 0.1, 0.1 ]\n")
    with open(os.path.join(root, "materials", "gold.toml"), "w") as f:
        f.write("material_function = '''surface.base_color = float3(1.0, 0.8, 0.3);\n"
                "surface.roughness = PARAM_roughness;\n'''\n[[params]]\nname = 'roughness'\nvalue = 0.4\n"
                "[[params]]\nname = 'metallic'\nvalue = 1.0\n")
    with open(os.path.join(root, "materials", "fancy.toml"), "w") as f:
        f.write("blend_mode = 'translucent'\nmaterial_function = '''int g = int(vertex.position_world.x);\n"
                "surface.base_color = (g & 1) == 1 ? PARAM_a : PARAM_a;\nsurface.opacity = 0.35;\n'''\n"
                "[[params]]\nname = 'a'\nvalue = [ 0.2, 0.2, 0.2 ]\n")
    scene = """
[[objects]]
name = 'Camera'
    [[objects.components]]
    type = 'Transform'
        [objects.components.value]
        rotation = [ -10.0, 20.0, 0.0 ]
        scaling = [ 1.0, 1.0, 1.0 ]
        translation = [ 0.5, 2.0, 6.0 ]
    [[objects.components]]
    type = 'CameraComponent'
        [objects.components.value]
        far_z = 500.0
        near_z = 0.05
        projection_type = 'perspective'
        render_target_size = [ 64, 48 ]
        yfov = 45.0
[[objects]]
name = 'Sun'
    [[objects.components]]
    type = 'Transform'
        [objects.components.value]
        rotation = [ 10.0, 0.0, -30.0 ]
    [[objects.components]]
    type = 'DirectionalLightComponent'
        [objects.components.value]
        color = [ 1.0, 0.9, 0.8 ]
        strength = 4.0
[[objects]]
name = 'Dark'
    [[objects.components]]
    type = 'DirectionalLightComponent'
        [objects.components.value]
        color = [ 1.0, 1.0, 1.0 ]
        strength = 0.0
[[objects]]
name = 'Parent'
    [[objects.components]]
    type = 'Transform'
        [objects.components.value]
        rotation = [ 0.0, 90.0, 0.0 ]
        scaling = [ 2.0, 1.0, 2.0 ]
        translation = [ 1.0, 0.0, 0.0 ]
    [[objects.components]]
    type = 'StaticMeshComponent'
        [objects.components.value.static_mesh]
        asset_id = 0
    [[objects.components]]
    type = 'MeshRendererComponent'
        [objects.components.value]
        submesh_start_index = 0
            [[objects.components.value.materials]]
            asset_id = 1
            [[objects.components.value.materials]]
            asset_id = 2
[[objects]]
name = 'Child'
parent = 3
    [[objects.components]]
    type = 'Transform'
        [objects.components.value]
        rotation = [ 0.0, 0.0, 45.0 ]
        translation = [ 0.0, 3.0, 0.0 ]
    [[objects.components]]
    type = 'StaticMeshComponent'
        [objects.components.value.static_mesh]
        asset_id = 0
    [[objects.components]]
    type = 'MeshRendererComponent'
        [objects.components.value]
        submesh_start_index = 1
            [[objects.components.value.materials]]
            asset_id = 3
            [[objects.components.value.materials]]
            asset_id = 1
[[objects]]
name = 'Spot'
    [[objects.components]]
    type = 'Transform'
        [objects.components.value]
        rotation = [ 0.0, 0.0, 180.0 ]
        translation = [ 0.0, 4.0, 0.0 ]
    [[objects.components]]
    type = 'PointLightComponent'
        [objects.components.value]
        color = [ 1.0, 1.0, 1.0 ]
        strength = 10.0
        range = 12.0
        spot = true
        spot_inner_angle = 20.0
        spot_outer_angle = 40.0
[[objects]]
name = 'Panel'
    [[objects.components]]
    type = 'Transform'
        [objects.components.value]
        rotation = [ 90.0, 0.0, 0.0 ]
        translation = [ 1.0, 3.0, 1.0 ]
    [[objects.components]]
    type = 'RectLightComponent'
        [objects.components.value]
        color = [ 0.5, 0.5, 1.0 ]
        strength = 2.0
        width = 2.0
        height = 0.5
        two_sided = true
[[objects]]
name = 'Override'
    [[objects.components]]
    type = 'BasicRendererOverrideVolume'
        [objects.components.value]
        priority = 0.0
            [objects.components.value.settings]
            pipeline_mode = 'deferred'
                [objects.components.value.settings.path_tracing]
                accumulate = false
                denoise = true
                max_bounces = 5
                ray_length = 40.0
"""
    with open(os.path.join(root, "scene.toml"), "w") as f:
        f.write(scene)


def test_project_loads_into_world_space(bsm, tmp_path):
    root = str(tmp_path / "proj")
    write_project(root, bsm)
    sc, info = bsm.load_project(root)
    q = quad_mesh()
    P = affine([1, 0, 0], [0, 90, 0], [2, 1, 2])
    Cw = P @ affine([0, 3, 0], [0, 0, 45], [1, 1, 1])
    # parent: submesh 0 (red) and 1 (gold); child: submesh 1 only (materials beyond the submeshes dropped)
    assert info.num_objects == 8 and info.num_drawables == 3
    assert sc.num_triangles == 2 + 1 + 1
    hom = np.c_[q["positions"], np.ones(7)]
    expect_parent = (hom @ P.T)[:, :3]
    expect_child = (hom @ Cw.T)[:, :3]
    tri = sc.positions[sc.indices]
    assert np.allclose(tri[0], expect_parent[[0, 2, 1]], atol=1e-5)
    assert np.allclose(tri[2], expect_parent[[4, 5, 6]], atol=1e-5)
    assert np.allclose(tri[3], expect_child[[4, 5, 6]], atol=1e-5)
    mats = sc.materials
    red, gold, fancy = mats[sc.material_ids[0]], mats[sc.material_ids[2]], mats[sc.material_ids[3]]
    # base rgb, roughness, metallic, opacity, blend mode
    assert np.allclose(red, [0.9, 0.1, 0.1, 0.25, 0.0, 1.0, 0])
    assert np.allclose(gold, [1.0, 0.8, 0.3, 0.4, 1.0, 1.0, 0])
    assert np.allclose(fancy, [0.5, 0.5, 0.5, 0.5, 0.0, 0.35, 2])  # base approximated: surface defaults
    assert info.num_materials_approximated == 1 and info.num_non_opaque_materials == 1
    # lights: zero emission skipped; direction = R (0, 1, 0)
    assert sc.lights.shape == (1, 6)
    assert np.allclose(sc.lights[0, :3], euler_zxy([10, 0, -30]) @ [0, 1, 0], atol=1e-6)
    assert np.allclose(sc.lights[0, 3:], [4.0, 3.6, 3.2])
    # spot: position = translation, direction = R (0, 1, 0), cone cosines; rect: centre, axes R x / R y
    assert sc.point_lights.shape == (1, 12)
    p = sc.point_lights[0]
    assert np.allclose(p[0:3], [0, 4, 0]) and np.allclose(p[3:6], 10.0) and p[6] == 12.0
    assert np.allclose(p[7:10], euler_zxy([0, 0, 180]) @ [0, 1, 0], atol=1e-6)
    assert np.allclose(p[10:12], np.cos(np.radians([20.0, 40.0])))
    r = sc.rect_lights[0]
    Rr = euler_zxy([90, 0, 0])
    assert np.allclose(r[0:3], [1, 3, 1]) and np.allclose(r[3:6], Rr @ [1, 0, 0], atol=1e-6)
    assert np.allclose(r[6:9], Rr @ [0, 1, 0], atol=1e-6) and tuple(r[9:11]) == (2.0, 0.5)
    assert np.allclose(r[11:14], [1.0, 1.0, 2.0]) and r[14] == 1
    # camera
    R = euler_zxy([-10, 20, 0])
    assert info.has_camera == 1
    assert np.allclose(list(info.camera.position), [0.5, 2.0, 6.0])
    assert np.allclose(list(info.camera.front), R @ [0, 0, -1], atol=1e-6)
    assert np.allclose(list(info.camera.up), R @ [0, 1, 0], atol=1e-6)
    assert (info.camera.width, info.camera.height) == (64, 48) and info.camera.yfov_deg == 45.0
    assert np.isclose(info.near_z, 0.05) and info.far_z == 500.0
    s = info.settings
    assert (s.max_bounces, s.accumulate, s.ray_length) == (5, 0, 40.0)


def test_project_normals_go_to_world_space(bsm, tmp_path):
    """Vertex normals leave the loader as the inverse transpose of each object's linear transform times the
    mesh normal (hit.hlsl:158 applies WorldToObject to normals); scale does not matter, direction does."""
    root = str(tmp_path / "proj")
    write_project(root, bsm, normals=True)
    sc, info = bsm.load_project(root)
    assert sc.normals is not None and sc.normals.shape == sc.positions.shape
    n = quad_mesh(True)["normals"].astype(np.float64)
    P = affine([1, 0, 0], [0, 90, 0], [2, 1, 2])
    Cw = P @ affine([0, 3, 0], [0, 0, 45], [1, 1, 1])
    unit = lambda v: v / np.linalg.norm(v, axis=-1, keepdims=True)
    expect_parent = unit(n @ np.linalg.inv(P[:3, :3]))          # (L^-T n)^T = n^T L^-1
    expect_child = unit(n @ np.linalg.inv(Cw[:3, :3]))
    got = unit(sc.normals.astype(np.float64))
    assert np.allclose(got[:7], expect_parent, atol=1e-6)
    assert np.allclose(got[7:14], expect_child, atol=1e-6)
    # a project whose meshes have no normals gives none
    root2 = str(tmp_path / "proj2")
    write_project(root2, bsm)
    sc2, _ = bsm.load_project(root2)
    assert sc2.normals is None


def test_project_errors(bsm, tmp_path):
    root = str(tmp_path / "p")
    write_project(root, bsm)
    os.remove(os.path.join(root, "materials", "gold.toml"))
    with pytest.raises(bsm.BsmError) as e:
        bsm.load_project(root)
    assert "gold.toml" in str(e.value)
    with pytest.raises(bsm.BsmError):
        bsm.load_project(str(tmp_path / "missing"))
    root2 = str(tmp_path / "p2")
    write_project(root2, bsm)
    with open(os.path.join(root2, "scene.toml"), "a") as f:
        f.write("[[objects]]\nname = 'Loop'\nparent = 8\n")   # its own parent (the ninth object)
    with pytest.raises(bsm.BsmError) as e:
        bsm.load_project(root2)
    assert "cycle" in str(e.value)


@pytest.mark.skipif(not os.path.isdir(REF_EXAMPLE), reason="reference tree not present")
def test_reference_example_meshes_and_project(bsm):
    for name in ["plane", "cube", "sphere"]:
        data = open(os.path.join(REF_EXAMPLE, "meshes", f"{name}.static_mesh.biasset"), "rb").read()
        assert same_mesh(bsm.read_static_mesh(data), parse_independent(data))
    sc, info = bsm.load_project(REF_EXAMPLE)
    assert info.num_drawables == 5 and info.has_camera == 1
    assert sc.num_triangles == 2 + 960 + 12 * 3                      # plane, sphere, three cubes
    assert np.allclose(sc.lights[0, :3], euler_zxy([10, 0, -30]) @ [0, 1, 0], atol=1e-6)
    assert (info.camera.width, info.camera.height) == (1298, 635)
    assert info.settings.max_bounces == 3 and info.settings.accumulate == 1
