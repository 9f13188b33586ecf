"""Seeded procedural workloads for the batch renderer.

No public dataset is used: every scene is generated here from one integer
seed (numpy PCG64).  A ``Workload`` lists meshes, textures, materials,
hierarchy templates, per-scene instances and per-env cameras; ``build_*``
feeds it to any object with the renderer's procedural call surface
(``addMesh``, ``addTexture``, ``addMaterial``, ``addNodeHierarchyTemplate``,
``addNodeHierarchy``, ``setSemanticId``, ``updateCameras``).

Workloads (sizes as named by the benchmark configurations):
  * ``config0``  16 envs share one room: an 8 x 8 x 3 m box whose six faces
    are each a 64 x 64 quad grid (49,152 triangles) plus 20 axis-aligned
    boxes with sides U(0.3, 1.5) m resting on the floor; random RGB per
    vertex, one object id per object (per-vertex ids); 128 x 128 pinhole
    cameras, hfov 90 deg, 1.25 m high, uniform position and yaw; near 0.01,
    far 10.
  * ``config1``  1024 envs over 4 scenes; each scene is a ~20k-triangle
    room shell plus 200 instances of 16 prototypes (geodesic spheres and
    subdivided boxes of 500-5k triangles, planar UVs) textured from a
    512 x 512 x 16 RGBA8 uniform-noise array, bilinear; random yaw, floor
    position and scale U(0.5, 1.5); per-instance semantic ids.
  * ``config2``  4096 envs over 64 scenes with triangle counts log-uniform
    in 20k-2M (shell subdivision and instance count raised together),
    resolution drawn from {64, 128, 256}^2 with p = {0.3, 0.5, 0.2}, hfov
    U(60, 110) deg.
  * ``config3``  256 envs over 8 scan-like scenes: a 12 x 12 x 3 m room
    (floor, walls, ceiling) tessellated into a quad grid, about 5M
    triangles per scene (1.31 cm edges; 1 cm edges would give 8.6M),
    vertex positions perturbed by Gaussian noise with sigma 1 cm, per-vertex
    RGB from a smooth value-noise field (trilinear over a 0.5 m lattice),
    per-vertex semantic ids from 64 Voronoi regions; triangles emitted in
    16 x 16-quad tiles; 256 x 256 cameras at 1.25 m doing a random walk of
    0.25 m and 10 deg per step.
"""
import dataclasses
import math

import numpy as np

NEAR = 0.01
FAR = 10.0
ROOM = (8.0, 3.0, 8.0)


@dataclasses.dataclass
class Workload:
    name: str
    envs: int
    viewports: list            # (w, h) per env
    hfov: np.ndarray           # degrees per env
    scene_of_env: np.ndarray   # scene index per env
    meshes: list = dataclasses.field(default_factory=list)
    textures: list = dataclasses.field(default_factory=list)
    materials: list = dataclasses.field(default_factory=list)  # (color, texture idx|-1, layer)
    templates: list = dataclasses.field(default_factory=list)  # (name, [(mesh, off, cnt, mat)])
    instances: list = dataclasses.field(default_factory=list)  # per scene [(tmpl, bake, id)]
    seed: int = 0
    uniform: bool = True       # all envs share one resolution -> tile grid layout
    room: tuple = ROOM         # extent (x, y, z) of the room the cameras move in
    walk: bool = False         # cameras random-walk from step to step (else fresh poses)

    def triangles_per_env(self):
        tri = {name: sum(c // 3 for (_, _, c, _) in views) for name, views in self.templates}
        per_scene = [sum(tri[t] for (t, _, _) in inst) for inst in self.instances]
        return np.array([per_scene[s] for s in self.scene_of_env], np.int64)

    def geometry_bytes(self):
        """Bytes of unique geometry and textures as stored on the device:
        16 B position + 16 B colour + 8 B uv per vertex, 4 B per index,
        4 B per texel."""
        v = sum(len(m["positions"]) for m in self.meshes)
        i = sum(len(m["indices"]) for m in self.meshes)
        t = sum(p["pixels"].size for p in self.textures)
        return v * 40 + i * 4 + t


# ----------------------------------------------------------------- geometry
def _face_grid(origin, a, b, n):
    """(n+1)^2 vertices and 2n^2 triangles of the parallelogram origin + s*a + t*b,
    counter-clockwise seen from the side a x b points to."""
    s = np.linspace(0.0, 1.0, n + 1)
    ss, tt = np.meshgrid(s, s, indexing="xy")
    pos = (np.asarray(origin)[None, None, :] + ss[..., None] * np.asarray(a)[None, None, :] +
           tt[..., None] * np.asarray(b)[None, None, :]).reshape(-1, 3)
    idx = np.arange((n + 1) * (n + 1)).reshape(n + 1, n + 1)  # [t][s]
    v00 = idx[:-1, :-1].reshape(-1)
    v10 = idx[:-1, 1:].reshape(-1)
    v11 = idx[1:, 1:].reshape(-1)
    v01 = idx[1:, :-1].reshape(-1)
    tris = np.stack([np.stack([v00, v10, v11], 1), np.stack([v00, v11, v01], 1)], 1).reshape(-1, 3)
    return pos, tris


def box_faces(lo, hi, n, inward):
    """Six subdivided faces of the box [lo, hi]; normals inward or outward."""
    lo = np.asarray(lo, np.float64)
    hi = np.asarray(hi, np.float64)
    d = hi - lo
    X, Y, Z = np.array([d[0], 0, 0]), np.array([0, d[1], 0]), np.array([0, 0, d[2]])
    # (origin, a, b) with a x b pointing into the box.
    faces_in = [
        (lo, Z, X),                         # floor y=lo, +y
        (lo + Y, X, Z),                     # ceiling y=hi, -y
        (lo, Y, Z),                         # x=lo, +x
        (lo + X, Z, Y),                     # x=hi, -x
        (lo, X, Y),                         # z=lo, +z
        (lo + Z, Y, X),                     # z=hi, -z
    ]
    pos_all, tri_all = [], []
    base = 0
    for (o, a, b) in faces_in:
        if not inward:
            a, b = b, a
        p, t = _face_grid(o, a, b, n)
        pos_all.append(p)
        tri_all.append(t + base)
        base += len(p)
    return np.concatenate(pos_all), np.concatenate(tri_all)


def geodesic_sphere(freq, radius):
    """Icosahedron with each face split into freq^2 triangles, projected to a sphere
    (outward, counter-clockwise)."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t],
                  [0, -1, -t], [0, 1, -t], [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]],
                 np.float64)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9],
                  [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2],
                  [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10],
                  [8, 6, 7], [9, 8, 1]])
    pos, tris = [], []
    base = 0
    for (i0, i1, i2) in f:
        a, b, c = v[i0], v[i1], v[i2]
        lut = {}
        for r in range(freq + 1):
            for q in range(freq + 1 - r):
                p = a + (b - a) * (q / freq) + (c - a) * (r / freq)
                lut[(q, r)] = base + len(lut)
                pos.append(p)
        for r in range(freq):
            for q in range(freq - r):
                tris.append([lut[(q, r)], lut[(q + 1, r)], lut[(q, r + 1)]])
                if q + r + 1 < freq:
                    tris.append([lut[(q + 1, r)], lut[(q + 1, r + 1)], lut[(q, r + 1)]])
        base += len(lut)
    pos = np.array(pos)
    pos = pos / np.linalg.norm(pos, axis=1, keepdims=True) * radius
    return pos, np.array(tris, np.int64)


def _mesh(pos, tris, colors=None, uv=None, ids=None):
    return dict(positions=np.ascontiguousarray(pos, np.float32),
                colors=None if colors is None else np.ascontiguousarray(colors, np.float32),
                texcoords=None if uv is None else np.ascontiguousarray(uv, np.float32),
                object_ids=None if ids is None else np.ascontiguousarray(ids, np.uint32),
                indices=np.ascontiguousarray(tris, np.uint32).reshape(-1))


def _rgb(rng, n):
    c = np.empty((n, 4), np.float32)
    c[:, :3] = rng.integers(0, 256, size=(n, 3)).astype(np.float32) / np.float32(255.0)
    c[:, 3] = 1.0
    return c


def _concat(parts):
    """Concatenate meshes into one (for batch-friendly composite meshes); returns
    the mesh and each part's (index offset, index count)."""
    pos, col, uv, idx, ranges = [], [], [], [], []
    vb = ib = 0
    for p in parts:
        pos.append(p["positions"])
        col.append(p["colors"])
        uv.append(p["texcoords"])
        idx.append(p["indices"].astype(np.int64) + vb)
        ranges.append((ib, len(p["indices"])))
        vb += len(p["positions"])
        ib += len(p["indices"])
    m = _mesh(np.concatenate(pos), np.concatenate(idx),
              None if col[0] is None else np.concatenate(col),
              None if uv[0] is None else np.concatenate(uv))
    return m, ranges


def _prototypes(rng, count, radius=0.5):
    protos = []
    for k in range(count):
        target = math.exp(rng.uniform(math.log(500), math.log(5000)))
        if k % 2 == 0:
            freq = int(np.clip(round(math.sqrt(target / 20.0)), 5, 15))
            pos, tris = geodesic_sphere(freq, radius)
        else:
            n = int(np.clip(round(math.sqrt(target / 12.0)), 7, 20))
            pos, tris = box_faces([-radius] * 3, [radius] * 3, n, inward=False)
        uv = np.stack([pos[:, 0] / (2 * radius) + 0.5, pos[:, 2] / (2 * radius) + 0.5], 1)
        protos.append(_mesh(pos, tris, None, uv))
    return protos


def _bake(x, y, z, yaw, scale):
    c, s = math.cos(yaw), math.sin(yaw)
    m = np.zeros((4, 4), np.float64)     # [col][row]
    m[0, :3] = [c * scale, 0, -s * scale]
    m[1, :3] = [0, scale, 0]
    m[2, :3] = [s * scale, 0, c * scale]
    m[3, :3] = [x, y, z]
    m[3, 3] = 1.0
    return m.astype(np.float32)


# ---------------------------------------------------------------- workloads
def config0(seed=0, envs=16, resolution=128, room_subdiv=64, boxes=20):
    rng = np.random.default_rng(seed)
    lo = np.array([-ROOM[0] / 2, 0.0, -ROOM[2] / 2])
    hi = np.array([ROOM[0] / 2, ROOM[1], ROOM[2] / 2])
    wl = Workload("config0", envs, [(resolution, resolution)] * envs, np.full(envs, 90.0),
                  np.zeros(envs, np.int64), seed=seed)
    pos, tris = box_faces(lo, hi, room_subdiv, inward=True)
    wl.meshes.append(_mesh(pos, tris, _rgb(rng, len(pos)), None, np.full(len(pos), 1, np.uint32)))
    views = [(0, 0, len(wl.meshes[0]["indices"]), 0)]
    for b in range(boxes):
        size = rng.uniform(0.3, 1.5, size=3)
        cx = rng.uniform(lo[0] + size[0] / 2, hi[0] - size[0] / 2)
        cz = rng.uniform(lo[2] + size[2] / 2, hi[2] - size[2] / 2)
        blo = np.array([cx - size[0] / 2, 0.0, cz - size[2] / 2])
        p, t = box_faces(blo, blo + size, 1, inward=False)
        wl.meshes.append(_mesh(p, t, _rgb(rng, len(p)), None, np.full(len(p), 2 + b, np.uint32)))
        views.append((1 + b, 0, len(wl.meshes[-1]["indices"]), 0))
    wl.materials.append(((1, 1, 1, 1), -1, 0))
    wl.templates.append(("config0/room", views))
    wl.instances.append([("config0/room", None, 0)])
    return wl


def config1(seed=1, envs=1024, scenes=4, resolution=128, shell_subdiv=41, instances=200,
            prototypes=16, texture_size=512):
    rng = np.random.default_rng(seed)
    wl = Workload("config1", envs, [(resolution, resolution)] * envs, np.full(envs, 90.0),
                  np.arange(envs) % scenes, seed=seed)
    lo = np.array([-ROOM[0] / 2, 0.0, -ROOM[2] / 2])
    hi = np.array([ROOM[0] / 2, ROOM[1], ROOM[2] / 2])
    for s in range(scenes):
        _add_textured_scene(wl, rng, s, lo, hi, shell_subdiv, instances, prototypes, texture_size)
    return wl


def _add_textured_scene(wl, rng, s, lo, hi, shell_subdiv, instances, prototypes, texture_size):
    pos, tris = box_faces(lo, hi, shell_subdiv, inward=True)
    shell = len(wl.meshes)
    wl.meshes.append(_mesh(pos, tris, _rgb(rng, len(pos))))
    protos = _prototypes(rng, prototypes)
    comp, ranges = _concat(protos)
    proto_mesh = len(wl.meshes)
    wl.meshes.append(comp)
    tex = len(wl.textures)
    wl.textures.append(dict(pixels=rng.integers(0, 256, size=(prototypes, texture_size,
                                                              texture_size, 4), dtype=np.uint8),
                            filter=1, wrap_s=0, wrap_t=0))
    mat_shell = len(wl.materials)
    wl.materials.append(((1, 1, 1, 1), -1, 0))
    mats = []
    for k in range(prototypes):
        mats.append(len(wl.materials))
        wl.materials.append(((1, 1, 1, 1), tex, k))
    tname = f"{wl.name}/s{s}/shell"
    wl.templates.append((tname, [(shell, 0, len(wl.meshes[shell]["indices"]), mat_shell)]))
    pnames = []
    for k in range(prototypes):
        nm = f"{wl.name}/s{s}/proto{k}"
        wl.templates.append((nm, [(proto_mesh, ranges[k][0], ranges[k][1], mats[k])]))
        pnames.append(nm)
    inst = [(tname, None, 1)]
    for i in range(instances):
        k = int(rng.integers(0, prototypes))
        scale = rng.uniform(0.5, 1.5)
        x = rng.uniform(lo[0] + 0.5, hi[0] - 0.5)
        z = rng.uniform(lo[2] + 0.5, hi[2] - 0.5)
        inst.append((pnames[k], _bake(x, 0.5 * scale, z, rng.uniform(0, 2 * math.pi), scale),
                     1000 + i))
    wl.instances.append(inst)


def _tiled_grid(origin, a, b, nu, nv, tile=16):
    """nu x nv quads of the parallelogram origin + s*a + t*b, counter-clockwise
    seen from the side a x b points to; triangles emitted tile x tile quads
    at a time so that consecutive triangles lie close together."""
    s = np.linspace(0.0, 1.0, nu + 1)
    t = np.linspace(0.0, 1.0, nv + 1)
    ss, tt = np.meshgrid(s, t, indexing="xy")
    pos = (np.asarray(origin)[None, None, :] + ss[..., None] * np.asarray(a)[None, None, :] +
           tt[..., None] * np.asarray(b)[None, None, :]).reshape(-1, 3)
    idx = np.arange((nu + 1) * (nv + 1)).reshape(nv + 1, nu + 1)
    qi, qj = np.meshgrid(np.arange(nu), np.arange(nv), indexing="xy")
    tiles_u = (nu + tile - 1) // tile
    key = (((qj // tile) * tiles_u + qi // tile) * tile + qj % tile) * tile + qi % tile
    order = np.argsort(key.reshape(-1), kind="stable")
    qi, qj = qi.reshape(-1)[order], qj.reshape(-1)[order]
    v00, v10, v11, v01 = idx[qj, qi], idx[qj, qi + 1], idx[qj + 1, qi + 1], idx[qj + 1, qi]
    tris = np.stack([np.stack([v00, v10, v11], 1), np.stack([v00, v11, v01], 1)], 1).reshape(-1, 3)
    return pos, tris


def _value_noise(rng, pts, lo, hi, spacing):
    """Smooth RGB field: trilinear interpolation of uniform random values on a
    lattice with the given spacing covering [lo, hi]."""
    n = np.ceil((np.asarray(hi) - np.asarray(lo)) / spacing).astype(int) + 2
    lattice = rng.uniform(0.0, 1.0, size=(n[0], n[1], n[2], 3))
    f = (pts - np.asarray(lo)) / spacing
    i = np.clip(np.floor(f).astype(int), 0, n - 2)
    w = np.clip(f - i, 0.0, 1.0)
    out = np.zeros((len(pts), 3))
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                wt = ((w[:, 0] if dx else 1 - w[:, 0]) * (w[:, 1] if dy else 1 - w[:, 1]) *
                      (w[:, 2] if dz else 1 - w[:, 2]))
                out += wt[:, None] * lattice[i[:, 0] + dx, i[:, 1] + dy, i[:, 2] + dz]
    return out


def scan_scene(rng, lo, hi, edge, noise=0.01, regions=64):
    """One scan-like room mesh (see config3)."""
    lo = np.asarray(lo, np.float64)
    hi = np.asarray(hi, np.float64)
    d = hi - lo
    X, Y, Z = np.array([d[0], 0, 0]), np.array([0, d[1], 0]), np.array([0, 0, d[2]])
    faces = [(lo, Z, X), (lo + Y, X, Z), (lo, Y, Z), (lo + X, Z, Y), (lo, X, Y), (lo + Z, Y, X)]
    pos_all, tri_all, base = [], [], 0
    for (o, a, b) in faces:
        nu = max(1, int(round(np.linalg.norm(a) / edge)))
        nv = max(1, int(round(np.linalg.norm(b) / edge)))
        p, t = _tiled_grid(o, a, b, nu, nv)
        pos_all.append(p)
        tri_all.append(t + base)
        base += len(p)
    pos = np.concatenate(pos_all)
    pos += rng.normal(0.0, noise, size=pos.shape)
    col = np.ones((len(pos), 4), np.float32)
    rgb = _value_noise(rng, pos, lo - 0.5, hi + 0.5, 0.5)
    col[:, :3] = np.round(np.clip(rgb, 0, 1) * 255.0).astype(np.float32) / np.float32(255.0)
    seeds = rng.uniform(lo, hi, size=(regions, 3))
    from scipy.spatial import cKDTree
    ids = (1 + cKDTree(seeds).query(pos)[1]).astype(np.uint32)
    return _mesh(pos, np.concatenate(tri_all), col, None, ids)


def config3(seed=3, envs=256, scenes=8, resolution=256, edge=0.0131, room=(12.0, 3.0, 12.0)):
    rng = np.random.default_rng(seed)
    wl = Workload("config3", envs, [(resolution, resolution)] * envs, np.full(envs, 90.0),
                  np.arange(envs) % scenes, seed=seed, room=tuple(room), walk=True)
    lo = np.array([-room[0] / 2, 0.0, -room[2] / 2])
    hi = np.array([room[0] / 2, room[1], room[2] / 2])
    for s in range(scenes):
        wl.meshes.append(scan_scene(rng, lo, hi, edge))
        wl.templates.append((f"config3/s{s}", [(s, 0, len(wl.meshes[-1]["indices"]), 0)]))
        wl.instances.append([(f"config3/s{s}", None, 0)])
    wl.materials.append(((1, 1, 1, 1), -1, 0))
    return wl


def config2(seed=2, envs=4096, scenes=64, tri_range=(2e4, 2e6), prototypes=16, texture_size=512):
    rng = np.random.default_rng(seed)
    res = rng.choice([64, 128, 256], size=envs, p=[0.3, 0.5, 0.2])
    wl = Workload("config2", envs, [(int(r), int(r)) for r in res], rng.uniform(60, 110, envs),
                  np.arange(envs) % scenes, seed=seed, uniform=False)
    lo = np.array([-ROOM[0] / 2, 0.0, -ROOM[2] / 2])
    hi = np.array([ROOM[0] / 2, ROOM[1], ROOM[2] / 2])
    for s in range(scenes):
        target = math.exp(rng.uniform(math.log(tri_range[0]), math.log(tri_range[1])))
        n = max(8, int(round(math.sqrt(0.3 * target / 12.0))))
        inst = max(1, int(round(0.7 * target / 2750.0)))
        _add_textured_scene(wl, rng, s, lo, hi, n, inst, prototypes, texture_size)
    return wl


# ------------------------------------------------------------------ cameras
def projection(hfov_deg, width, height, near=NEAR, far=FAR):
    """Pinhole projection of habitat-sim's CameraSensor
    (src/esp/sensor/CameraSensor.cpp:46-56): near-plane size
    {1, H/W} * 2 near tan(hfov/2), Magnum perspectiveProjection(size, n, f)."""
    f32 = np.float32
    n, fa = f32(near), f32(far)
    sx = f32(2.0) * n * f32(math.tan(math.radians(hfov_deg) / 2.0))
    sy = sx * (f32(height) / f32(width))
    m = np.zeros((4, 4), f32)
    m[0, 0] = f32(2.0) * n / sx
    m[1, 1] = f32(2.0) * n / sy
    zs = f32(1.0) / (n - fa)
    m[2, 2] = (fa + n) * zs
    m[2, 3] = -1.0
    m[3, 2] = f32(2.0) * fa * n * zs
    return m


def _walk(wl, step):
    """Random walk of every env's camera: uniform start 0.5 m inside the
    walls, then per step 0.25 m along a uniform direction (reflected at the
    walls) and a yaw change of +-10 deg."""
    rx, rz = wl.room[0] / 2 - 0.5, wl.room[2] / 2 - 0.5
    rng = np.random.default_rng([wl.seed, 104723])
    E = wl.envs
    x, z = rng.uniform(-rx, rx, E), rng.uniform(-rz, rz, E)
    yaw = rng.uniform(0, 2 * math.pi, E)
    for k in range(step):
        r = np.random.default_rng([wl.seed, 104729, k])
        a = r.uniform(0, 2 * math.pi, E)
        x, z = x + 0.25 * np.cos(a), z + 0.25 * np.sin(a)
        x = np.where(x > rx, 2 * rx - x, np.where(x < -rx, -2 * rx - x, x))
        z = np.where(z > rz, 2 * rz - z, np.where(z < -rz, -2 * rz - z, z))
        yaw = yaw + np.radians(10.0) * r.choice([-1.0, 1.0], E)
    return x, z, yaw


def camera_poses(wl, step=0):
    """(projections [E,4,4], views [E,4,4]) for one step: at 1.25 m, position
    uniform in the room and yaw uniform (fresh every step), or the random
    walk of ``_walk`` for walking workloads."""
    rng = np.random.default_rng([wl.seed, 7919, step])
    E = wl.envs
    x = rng.uniform(-wl.room[0] / 2 + 0.05, wl.room[0] / 2 - 0.05, E)
    z = rng.uniform(-wl.room[2] / 2 + 0.05, wl.room[2] / 2 - 0.05, E)
    yaw = rng.uniform(0, 2 * math.pi, E)
    if wl.walk:
        x, z, yaw = _walk(wl, step)
    views = np.zeros((E, 4, 4), np.float64)
    c, s = np.cos(yaw), np.sin(yaw)
    # camera-to-world = T(x, 1.25, z) * Ry(yaw); view = its inverse
    views[:, 0, 0] = c
    views[:, 0, 2] = s
    views[:, 1, 1] = 1.0
    views[:, 2, 0] = -s
    views[:, 2, 2] = c
    views[:, 3, 0] = -(c * x - s * z)
    views[:, 3, 1] = -1.25
    views[:, 3, 2] = -(s * x + c * z)
    views[:, 3, 3] = 1.0
    projs = np.stack([projection(wl.hfov[e], *wl.viewports[e]) for e in range(E)]) \
        if not wl.uniform else np.repeat(projection(wl.hfov[0], *wl.viewports[0])[None], E, 0)
    return projs.astype(np.float32), views.astype(np.float32)


# ----------------------------------------------------------------- builders
def add_resources(r, wl):
    """Add the workload's textures, meshes, materials and named hierarchy
    templates to renderer r (no scene content)."""
    tex = [r.addTexture(t["pixels"], t["filter"], t["wrap_s"], t["wrap_t"]) for t in wl.textures]
    meshes = [r.addMesh(m["positions"], m["colors"], m["texcoords"], m["object_ids"], m["indices"])
              for m in wl.meshes]
    mats = [r.addMaterial(c, 0 if t < 0 else tex[t], layer) for (c, t, layer) in wl.materials]
    for name, views in wl.templates:
        r.addNodeHierarchyTemplate(name, [(meshes[m], off, cnt, mats[mt], None)
                                          for (m, off, cnt, mt) in views])


def populate(r, wl, envs=None):
    """Add the workload's resources and per-env hierarchies to renderer r."""
    add_resources(r, wl)
    env_list = range(wl.envs) if envs is None else envs
    for slot, e in enumerate(env_list):
        for (tmpl, bake, sid) in wl.instances[wl.scene_of_env[e]]:
            node = r.addNodeHierarchy(slot, tmpl, bake)
            if sid:
                r.setSemanticId(slot, node, sid)


def scene_keyframe(pkg, wl, scene):
    """The gfx-replay keyframe that creates one scene's instances: a load
    and a creation per instance (hierarchy template name, uniform scale), a
    state update with the instance's translation and yaw, and its semantic
    id as metadata."""
    k = pkg.Keyframe()
    for name, _ in wl.templates:
        k.load(name)
    for key, (tmpl, bake, sid) in enumerate(wl.instances[scene]):
        b = np.eye(4) if bake is None else np.asarray(bake, np.float64)
        scale = float(np.linalg.norm(b[1, :3]))
        yaw = math.atan2(float(b[2, 0]), float(b[0, 0]))
        k.create(key, tmpl, scale=(scale, scale, scale))
        k.update(key, tuple(float(v) for v in b[3, :3]), (0.0, math.sin(yaw / 2), 0.0, math.cos(yaw / 2)))
        if sid:
            k.set_metadata(key, sid, sid)
    return k


def camera_keyframe(pkg, view, name="sensor_rgba_camera"):
    """A keyframe carrying only the camera pose (the inverse of `view`) as
    the user transform `name`."""
    m = np.linalg.inv(np.asarray(view, np.float64).T)     # row-major camera-to-world
    r = m[:3, :3]
    w = math.sqrt(max(0.0, 1.0 + r[0, 0] + r[1, 1] + r[2, 2])) / 2
    if w > 1e-6:
        q = ((r[2, 1] - r[1, 2]) / (4 * w), (r[0, 2] - r[2, 0]) / (4 * w), (r[1, 0] - r[0, 1]) / (4 * w), w)
    else:   # 180-degree turn: largest diagonal element
        i = int(np.argmax(np.diag(r)))
        j, k_ = (i + 1) % 3, (i + 2) % 3
        s = math.sqrt(max(0.0, 1.0 + r[i, i] - r[j, j] - r[k_, k_])) * 2
        qv = [0.0, 0.0, 0.0]
        qv[i] = s / 4
        qv[j] = (r[j, i] + r[i, j]) / s
        qv[k_] = (r[k_, i] + r[i, k_]) / s
        q = (qv[0], qv[1], qv[2], (r[k_, j] - r[j, k_]) / s)
    return pkg.Keyframe().user_transform(name, tuple(m[:3, 3]), q)


def grid_for(n):
    """Tile grid of the reference's environmentGridSize: {ceil(sqrt n), ceil(n/x)}
    (src/esp/sim/AbstractReplayRenderer.cpp:26-31)."""
    x = int(math.ceil(math.sqrt(n)))
    return x, int(math.ceil(n / x))


def build_renderer(pkg, wl, mode=None, envs=None, planes=None, double_buffer=False):
    env_list = list(range(wl.envs)) if envs is None else list(envs)
    cfg = pkg.RendererConfiguration()
    if wl.uniform:
        w, h = wl.viewports[0]
        cfg.setTileSizeCount((w, h), grid_for(len(env_list)))
    else:
        cfg.setViewports([wl.viewports[e] for e in env_list])
    if mode is not None:
        cfg.setDrawMode(mode)
    if planes is not None:
        cfg.setPlanes(planes)
    flags = pkg.RendererStandaloneFlags.QuietLog
    if double_buffer:
        flags |= pkg.RendererStandaloneFlags.DoubleBuffer
    r = pkg.RendererStandalone(cfg, pkg.RendererStandaloneConfiguration().setFlags(flags))
    populate(r, wl, env_list)
    return r


def build_oracle(cls, wl, envs=None):
    env_list = list(range(wl.envs)) if envs is None else list(envs)
    if wl.uniform:
        w, h = wl.viewports[0]
        r = cls((w, h), grid_for(len(env_list)))
    else:
        r = cls(viewports=[wl.viewports[e] for e in env_list])
    populate(r, wl, env_list)
    return r


def set_cameras(r, wl, poses, envs=None):
    projs, views = poses
    if envs is not None:
        projs, views = projs[list(envs)], views[list(envs)]
    r.updateCameras(projs, views)
