"""Small hand-built scenes and ray sets for the edge cases of the traversal
(shared by the oracle and GPU tests)."""
import numpy as np

MISS = 0xFFFFFFFF


def coincident_scene(bsm):
    """Prims 0..5 over the unit square in planes z = const:
    0: a quad half at z = 1 (back); 1 and 3: the same triangle at z = 0.5
    (a tie at equal t, which the lower primitive id wins); 2: a collinear
    (zero-area) triangle at z = 0.25; 4: all three vertices equal, at z = 0.2;
    5: the other quad half at z = 1."""
    P = np.array([[0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1],          # 0-3 back quad
                  [0, 0, .5], [1, 0, .5], [0, 1, .5],                   # 4-6 front triangle
                  [0, 0, .25], [.5, .5, .25], [1, 1, .25],              # 7-9 collinear
                  [.5, .5, .2]], np.float32)                            # 10 a point
    idx = np.array([[0, 1, 2], [4, 5, 6], [7, 8, 9], [4, 5, 6], [10, 10, 10], [0, 2, 3]], np.uint32)
    mats = np.array([[0.5, 0.5, 0.5, 0.5, 0.0], [0.8, 0.2, 0.2, 0.5, 0.0]], np.float32)
    mids = np.array([0, 1, 0, 0, 0, 0], np.uint32)
    lights = np.array([[0.3, 0.4, -1.0, 2.0, 2.0, 2.0]], np.float32)
    cam = bsm.make_camera((0.5, 0.5, -1.0), (0.0, 0.0, 1.0), yfov_deg=40.0, width=16, height=16)
    return bsm.SceneData(P, idx, mids, mats, lights, bsm.BSM_SKY_CONSTANT, (0.3, 0.3, 0.3), None, cam)


def rays_along_z(n, seed, z0=-1.0):
    rng = np.random.default_rng(seed)
    r = np.zeros((n, 8), np.float32)
    r[:, 0:2] = rng.uniform(0.02, 0.98, (n, 2))
    r[:, 2] = z0
    r[:, 6] = 1.0
    r[:, 7] = 10.0
    return r


def grid_scene(bsm, n=8):
    """An n x n grid of unit squares in z = 0, two triangles each, sharing
    every edge and vertex."""
    xs = np.arange(n + 1, dtype=np.float32)
    X, Y = np.meshgrid(xs, xs, indexing="xy")
    P = np.stack([X.ravel(), Y.ravel(), np.zeros(X.size, np.float32)], 1).astype(np.float32)
    tris = []
    for j in range(n):
        for i in range(n):
            a, b, c, d = j * (n + 1) + i, j * (n + 1) + i + 1, (j + 1) * (n + 1) + i + 1, (j + 1) * (n + 1) + i
            tris += [[a, b, c], [a, c, d]]
    idx = np.array(tris, np.uint32)
    mats = np.array([[0.5, 0.5, 0.5, 0.5, 0.0]], np.float32)
    lights = np.array([[0.0, 0.0, -1.0, 1.0, 1.0, 1.0]], np.float32)
    cam = bsm.make_camera((n / 2, n / 2, -5.0), (0.0, 0.0, 1.0), yfov_deg=60.0, width=16, height=16)
    return bsm.SceneData(P, idx, np.zeros(len(tris), np.uint32), mats, lights, bsm.BSM_SKY_CONSTANT,
                         (0.3, 0.3, 0.3), None, cam)


def edge_rays(n=8, seed=5):
    """Rays through the grid's shared edges and vertices: from z = -1 along a
    tilted direction, aimed exactly at points on the edges, the diagonals and
    the vertices (every one of them must hit a triangle)."""
    rng = np.random.default_rng(seed)
    pts = []
    for j in range(1, n):
        for i in range(1, n):
            pts += [(i, j), (i + 0.5, j), (i, j + 0.5), (i + 0.25, j + 0.25), (i + 0.5, j + 0.5)]
    pts = np.array(pts, np.float32)
    m = pts.shape[0]
    d = np.c_[rng.normal(0, 0.3, (m, 2)), np.ones(m)].astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = np.zeros((m, 8), np.float32)
    # origin = target - d * (1 / d.z): the ray reaches z = 0 at (about) the target
    s = (1.0 / d[:, 2]).astype(np.float32)
    r[:, 0] = pts[:, 0] - d[:, 0] * s
    r[:, 1] = pts[:, 1] - d[:, 1] * s
    r[:, 2] = -1.0
    r[:, 4:7] = d
    r[:, 7] = 10.0
    # and exactly axis-aligned rays through the vertices and edges
    a = np.zeros((m, 8), np.float32)
    a[:, 0:2] = pts
    a[:, 2] = -1.0
    a[:, 6] = 1.0
    a[:, 7] = 10.0
    return np.concatenate([r, a])


def invalid_rays():
    """Rays that are misses without traversal: non-finite origin or direction,
    zero direction, tmin > tmax, NaN tmax."""
    nan, inf = np.float32(np.nan), np.float32(np.inf)
    good = [0.5, 0.5, -1.0, 0.0, 0.0, 0.0, 1.0, 10.0]
    rows = []
    for k in (0, 1, 2, 4, 5, 6):
        for v in (nan, inf, -inf):
            r = list(good)
            r[k] = v
            rows.append(r)
    rows.append([0.5, 0.5, -1.0, 0.0, 0.0, 0.0, 0.0, 10.0])   # zero direction
    rows.append([0.5, 0.5, -1.0, 5.0, 0.0, 0.0, 1.0, 2.0])    # tmin > tmax
    rows.append([0.5, 0.5, -1.0, 0.0, 0.0, 0.0, 1.0, nan])    # NaN tmax
    rows.append([0.5, 0.5, -1.0, nan, 0.0, 0.0, 1.0, 10.0])   # NaN tmin
    return np.array(rows, np.float32)
