"""Oracle restatement of the batch replay renderer (test infrastructure).

Used only by ``tests/``.  It applies gfx-replay keyframes to an
``OracleRenderer`` the way habitat-sim's replay stack does:

* keyframe JSON fields (``src/esp/io/JsonEspTypes.cpp:102-201``,
  quaternions stored [w, x, y, z] by ``io/JsonMagnumTypes.cpp:133-162``);
* ``Player``: asset-info registry, creations with material overrides
  stripped after '?', metadata, the batch deletion path that clears the
  scene and re-creates the remaining instances with their latest transforms,
  state updates, light setups, ``setKeyframeIndex`` / ``setSingleKeyframe``
  (``src/esp/gfx/replay/Player.cpp:103-370``);
* ``BatchPlayerImplementation``: unsupported primitive names, files loaded
  whole when no hierarchy has the name, bake = scaling * frame rotation,
  node handle = root node + 1, transforms written to the root node, lights as
  empty nodes (``src/esp/sim/BatchPlayerImplementation.cpp:14-170``);
* ``BatchReplayRenderer``: tile grid of ``environmentGridSize``, camera view
  = inverse of the sensor transform, sensor projection
  (``src/esp/sim/BatchReplayRenderer.cpp:22-151``,
  ``AbstractReplayRenderer.cpp:26-31``, ``src/esp/sensor/CameraSensor.cpp:44-60``).

The small linear algebra is written out in float32, one rounding per
operation in the order the native driver uses, so both produce the same
matrices bit for bit; deviations from Magnum's own rounding are within the
float32 rounding of each formula (Magnum is not vendored in the reference).
"""
import json
import math

import numpy as np

from .model import FILE_GENERATE_MIPMAP, FILE_WHOLE, LIGHT_DIRECTIONAL, LIGHT_POINT, \
    OracleRenderer

F = np.float32
EPS = F(1.1920929e-07)

UNSUPPORTED_PREFIXES = (
    "capsule3DSolid", "capsule3DWireframe", "coneSolid", "coneWireframe", "cubeSolid",
    "cubeWireframe", "cylinderSolid", "cylinderWireframe", "icosphereSolid",
    "icosphereWireframe", "uvSphereSolid", "uvSphereWireframe")


# ------------------------------------------------------------------- math
def _dot3(a, b):
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]


def _cross3(a, b):
    return [a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]]


def _normalize3(v):
    ln = np.sqrt(_dot3(v, v))
    return [v[0] / ln, v[1] / ln, v[2] / ln]


def quat_to_matrix(q):
    """Column-major 3x3 list of a unit quaternion (x, y, z, w)."""
    x, y, z, w = q
    xx, yy, zz = x * x, y * y, z * z
    xy, xz, yz = x * y, x * z, y * z
    wx, wy, wz = w * x, w * y, w * z
    one, two = F(1), F(2)
    return [one - two * (yy + zz), two * (xy + wz), two * (xz - wy),
            two * (xy - wz), one - two * (xx + zz), two * (yz + wx),
            two * (xz + wy), two * (yz - wx), one - two * (xx + yy)]


def quat_between(a, b):
    c = _dot3(a, b)
    if c < F(-1) + EPS:
        axis = _cross3([F(1), F(0), F(0)], a)
        if _dot3(axis, axis) < EPS:
            axis = _cross3([F(0), F(1), F(0)], a)
        axis = _normalize3(axis)
        return (axis[0], axis[1], axis[2], F(0))
    axis = _cross3(a, b)
    s = np.sqrt((F(1) + c) * F(2))
    inv = F(1) / s
    return (axis[0] * inv, axis[1] * inv, axis[2] * inv, s * F(0.5))


def quat_mul(a, b):
    av, bv = a[:3], b[:3]
    c = _cross3(av, bv)
    return (a[3] * b[0] + b[3] * a[0] + c[0], a[3] * b[1] + b[3] * a[1] + c[1],
            a[3] * b[2] + b[3] * a[2] + c[2], a[3] * b[3] - _dot3(av, bv))


def quat_normalized(q):
    ln = np.sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3])
    return (q[0] / ln, q[1] / ln, q[2] / ln, q[3] / ln)


def quat_rotate(q, v):
    qv = q[:3]
    t = _cross3(qv, v)
    t = [F(2) * t[0], F(2) * t[1], F(2) * t[2]]
    c = _cross3(qv, t)
    return [v[i] + q[3] * t[i] + c[i] for i in range(3)]


def frame_to_world(up, front):
    """geo/CoordinateFrame.cpp:31-43 (inverse of the world-to-frame rotation)."""
    r_up = quat_between([F(0), F(1), F(0)], up)
    f = quat_rotate(r_up, [F(0), F(0), F(-1)])
    w2f = quat_normalized(quat_mul(quat_between(f, front), r_up))
    return (-w2f[0], -w2f[1], -w2f[2], w2f[3])


def rigid_matrix(q, t):
    """[R(q) | t] as a 4x4 array indexed [col][row]."""
    r = quat_to_matrix(q)
    m = np.zeros((4, 4), np.float32)
    for c in range(3):
        for i in range(3):
            m[c, i] = r[c * 3 + i]
    m[3, :3] = t
    m[3, 3] = 1
    return m


def invert4(m):
    """Inverse by Laplace expansion in 2x2 minors (D. Eberly, Geometric Tools)."""
    m = np.asarray(m, np.float32)

    def a(r, c):
        return m[c, r]
    s0 = a(0, 0) * a(1, 1) - a(1, 0) * a(0, 1)
    s1 = a(0, 0) * a(1, 2) - a(1, 0) * a(0, 2)
    s2 = a(0, 0) * a(1, 3) - a(1, 0) * a(0, 3)
    s3 = a(0, 1) * a(1, 2) - a(1, 1) * a(0, 2)
    s4 = a(0, 1) * a(1, 3) - a(1, 1) * a(0, 3)
    s5 = a(0, 2) * a(1, 3) - a(1, 2) * a(0, 3)
    c5 = a(2, 2) * a(3, 3) - a(3, 2) * a(2, 3)
    c4 = a(2, 1) * a(3, 3) - a(3, 1) * a(2, 3)
    c3 = a(2, 1) * a(3, 2) - a(3, 1) * a(2, 2)
    c2 = a(2, 0) * a(3, 3) - a(3, 0) * a(2, 3)
    c1 = a(2, 0) * a(3, 2) - a(3, 0) * a(2, 2)
    c0 = a(2, 0) * a(3, 1) - a(3, 0) * a(2, 1)
    det = s0 * c5 - s1 * c4 + s2 * c3 + s3 * c2 - s4 * c1 + s5 * c0
    if det == 0 or not np.isfinite(det):
        raise ValueError("singular transform")
    inv = F(1) / det
    b = np.zeros((4, 4), np.float32)  # b[row][col]
    b[0, 0] = (a(1, 1) * c5 - a(1, 2) * c4 + a(1, 3) * c3) * inv
    b[0, 1] = (-a(0, 1) * c5 + a(0, 2) * c4 - a(0, 3) * c3) * inv
    b[0, 2] = (a(3, 1) * s5 - a(3, 2) * s4 + a(3, 3) * s3) * inv
    b[0, 3] = (-a(2, 1) * s5 + a(2, 2) * s4 - a(2, 3) * s3) * inv
    b[1, 0] = (-a(1, 0) * c5 + a(1, 2) * c2 - a(1, 3) * c1) * inv
    b[1, 1] = (a(0, 0) * c5 - a(0, 2) * c2 + a(0, 3) * c1) * inv
    b[1, 2] = (-a(3, 0) * s5 + a(3, 2) * s2 - a(3, 3) * s1) * inv
    b[1, 3] = (a(2, 0) * s5 - a(2, 2) * s2 + a(2, 3) * s1) * inv
    b[2, 0] = (a(1, 0) * c4 - a(1, 1) * c2 + a(1, 3) * c0) * inv
    b[2, 1] = (-a(0, 0) * c4 + a(0, 1) * c2 - a(0, 3) * c0) * inv
    b[2, 2] = (a(3, 0) * s4 - a(3, 1) * s2 + a(3, 3) * s0) * inv
    b[2, 3] = (-a(2, 0) * s4 + a(2, 1) * s2 - a(2, 3) * s0) * inv
    b[3, 0] = (-a(1, 0) * c3 + a(1, 1) * c1 - a(1, 2) * c0) * inv
    b[3, 1] = (a(0, 0) * c3 - a(0, 1) * c1 + a(0, 2) * c0) * inv
    b[3, 2] = (-a(3, 0) * s3 + a(3, 1) * s1 - a(3, 2) * s0) * inv
    b[3, 3] = (a(2, 0) * s3 - a(2, 1) * s1 + a(2, 2) * s0) * inv
    return np.ascontiguousarray(b.T)  # [col][row]


def sensor_projection(resolution, hfov=90.0, near=0.01, far=1000.0, orthographic=False,
                      ortho_scale=0.1):
    """CameraSensorSpec::projectionMatrix (sensor/CameraSensor.cpp:44-60):
    near-plane size {1, height/width} scaled to the field of view."""
    aspect = F(resolution[0]) / F(resolution[1])
    n, f = F(near), F(far)
    p = np.zeros((4, 4), np.float32)
    if orthographic:
        sx, sy = F(1) / F(ortho_scale), aspect / F(ortho_scale)
        zs = F(2) / (n - f)
        p[0, 0] = F(2) / sx
        p[1, 1] = F(2) / sy
        p[2, 2] = zs
        p[3, 2] = (n + f) / (n - f)
        p[3, 3] = 1
        return p
    rad = F(hfov) * F(3.14159265358979323846) / F(180)
    t = F(math.tan(float(F(0.5) * rad)))
    scale = F(1) / (F(2) * n * t)
    sx, sy = F(1) / scale, aspect / scale
    zs = F(1) / (n - f)
    p[0, 0] = F(2) * n / sx
    p[1, 1] = F(2) * n / sy
    p[2, 2] = (f + n) * zs
    p[2, 3] = -1
    p[3, 2] = F(2) * f * n * zs
    return p


def environment_grid_size(n):
    x = int(math.ceil(math.sqrt(float(np.float32(n)))))
    return (x, (n + x - 1) // x)


# ---------------------------------------------------------------- keyframe
def _vec(v, n):
    if not isinstance(v, list) or len(v) != n:
        raise ValueError("bad vector")
    return [F(x) for x in v]


def _quat(v):
    w, x, y, z = _vec(v, 4)
    return (x, y, z, w)


def _transform(t):
    return (_vec(t["translation"], 3), _quat(t["rotation"]))


def parse_keyframe(obj):
    k = dict(loads=[], creations=[], deletions=[], metadata=[], state_updates=[],
             user_transforms={}, lights=[], lights_changed=False)
    for ld in obj.get("loads") or []:
        fr = ld.get("frame")
        k["loads"].append(dict(filepath=ld["filepath"],
                               up=_vec(fr["up"], 3) if fr else [F(0), F(1), F(0)],
                               front=_vec(fr["front"], 3) if fr else [F(0), F(0), F(-1)]))
    for c in obj.get("creations") or []:
        cr = c["creation"]
        scale = cr.get("scale")
        k["creations"].append((int(c["instanceKey"]),
                               dict(filepath=cr["filepath"],
                                    scale=None if scale is None else _vec(scale, 3))))
    k["deletions"] = [int(d) for d in obj.get("deletions") or []]
    for u in obj.get("stateUpdates") or []:
        k["state_updates"].append((int(u["instanceKey"]), _transform(u["state"]["absTransform"])))
    for m in obj.get("metadata") or []:
        k["metadata"].append((int(m["instanceKey"]), dict(object_id=int(m["metadata"]["objectId"]),
                                                          semantic_id=int(m["metadata"]["semanticId"]))))
    for u in obj.get("userTransforms") or []:
        k["user_transforms"][u["name"]] = _transform(u["transform"])
    k["lights_changed"] = bool(obj.get("lightsChanged", False))
    if k["lights_changed"]:
        for li in obj.get("lights") or []:
            k["lights"].append(dict(vector=_vec(li["vector"], 4), color=_vec(li["color"], 3),
                                    model=str(li.get("model", "global")).lower()))
    return k


# ------------------------------------------------------------------ player
class OracleBatchPlayer:
    def __init__(self, renderer, scene):
        self.r = renderer
        self.scene = scene

    def load_and_create(self, info, creation):
        path = creation["filepath"]
        if path.startswith(UNSUPPORTED_PREFIXES):
            return 0
        if not self.r.hasNodeHierarchy(path):
            self.r.addFile(path, FILE_WHOLE | FILE_GENERATE_MIPMAP)
        r = quat_to_matrix(frame_to_world(info["up"], info["front"]))
        s = creation["scale"] or [F(1), F(1), F(1)]
        bake = np.zeros((4, 4), np.float32)
        for c in range(3):
            for i in range(3):
                bake[c, i] = s[i] * r[c * 3 + i]
        bake[3, 3] = 1
        return self.r.addNodeHierarchy(self.scene, path, bake) + 1

    def delete_all(self):
        self.r.clear(self.scene)

    def set_matrix(self, node, m):
        self.r.transformations(self.scene)[node - 1] = np.array(m, np.float32)

    def get_matrix(self, node):
        return np.array(self.r.transformations(self.scene)[node - 1], np.float32)

    def set_metadata(self, node, md):
        if node and md["semantic_id"] >= 0:
            self.r.set_semantic_id(self.scene, node - 1, md["semantic_id"])

    def change_lights(self, lights):
        if not self.r.max_light_count:
            return
        self.r.clearLights(self.scene)
        for li in lights:
            if li["model"] != "global":
                raise ValueError("only global lights")
            node = self.r.addEmptyNode(self.scene)
            m = np.eye(4, dtype=np.float32)
            v = li["vector"]
            if v[3] != 0:
                m[3, :3] = v[:3]
                kind = LIGHT_POINT
            else:
                back = _normalize3([F(0) - v[0], F(0) - v[1], F(0) - v[2]])
                right = _normalize3(_cross3([F(0), F(1), F(0)], back))
                up = _cross3(back, right)
                m[0, :3], m[1, :3], m[2, :3] = right, up, back
                kind = LIGHT_DIRECTIONAL
            self.r.transformations(self.scene)[node] = m
            lid = self.r.addLight(self.scene, node, kind)
            self.r.lightColors(self.scene)[lid] = li["color"]


class OraclePlayer:
    def __init__(self, impl):
        self.impl = impl
        self.keyframes = []
        self.index = -1
        self.asset_infos = {}
        self.failed = set()
        self.created = {}
        self.records = {}

    def set_single_keyframe(self, k):
        self.keyframes = [k]
        self.index = -1
        self.set_keyframe_index(0)

    def set_keyframes(self, ks):
        self.close()
        self.keyframes = list(ks)

    def set_keyframe_index(self, index):
        if not -1 <= index < len(self.keyframes):
            raise IndexError("keyframe index out of range")
        if index < self.index:
            self.clear_frame()
        while self.index < index:
            self.index += 1
            self.apply(self.keyframes[self.index])

    def user_transform(self, name):
        if not 0 <= self.index < len(self.keyframes):
            return None
        return self.keyframes[self.index]["user_transforms"].get(name)

    def close(self):
        self.clear_frame()
        self.keyframes = []

    def clear_frame(self):
        self.impl.delete_all()
        self.created = {}
        self.asset_infos = {}
        self.records = {}
        self.index = -1

    def apply(self, k):
        for info in k["loads"]:
            if info["filepath"] not in self.failed:
                self.asset_infos[info["filepath"]] = info
        for key, c in k["creations"]:
            c = dict(c, filepath=c["filepath"].split("?", 1)[0])
            info = self.asset_infos.get(c["filepath"])
            if info is None:
                self.failed.add(c["filepath"])
                continue
            node = self.impl.load_and_create(info, c)
            if not node:
                self.failed.add(c["filepath"])
                continue
            assert key not in self.created
            self.created[key] = node
            self.records[key] = dict(creation=c, metadata=dict(object_id=-1, semantic_id=-1))
        for key, md in k["metadata"]:
            if key in self.created:
                self.impl.set_metadata(self.created[key], md)
                self.records[key]["metadata"] = md
        if k["deletions"]:
            latest = {key: self.impl.get_matrix(node) for key, node in self.created.items()}
            self.impl.delete_all()
            for key in k["deletions"]:
                if key in self.created:
                    del self.created[key]
                    del self.records[key]
            for key in sorted(self.created):
                rec = self.records[key]
                node = self.impl.load_and_create(self.asset_infos[rec["creation"]["filepath"]],
                                                 rec["creation"])
                self.impl.set_metadata(node, rec["metadata"])
                self.created[key] = node
                self.impl.set_matrix(node, latest[key])
        for key, (t, q) in k["state_updates"]:
            if key in self.created:
                self.impl.set_matrix(self.created[key], rigid_matrix(q, t))
        if k["lights_changed"]:
            self.impl.change_lights(k["lights"])


class OracleReplayRenderer:
    """The batch replay renderer on the CPU oracle (one scene per environment)."""

    def __init__(self, num_environments, resolution=(128, 128), sensor_uuid="rgba_camera",
                 hfov=90.0, near=0.01, far=1000.0, orthographic=False, ortho_scale=0.1,
                 max_light_count=0, ambient_factor=0.1):
        self.n = num_environments
        self.res = tuple(resolution)
        self.grid = environment_grid_size(num_environments)
        self.uuid = sensor_uuid
        self.projection = sensor_projection(resolution, hfov, near, far, orthographic, ortho_scale)
        self.r = OracleRenderer((resolution[1], resolution[0]), self.grid,
                                max_light_count=max_light_count, ambient_factor=ambient_factor)
        self.players = [OraclePlayer(OracleBatchPlayer(self.r, i)) for i in range(num_environments)]

    def preload_file(self, path):
        self.r.addFile(path)

    def set_environment_keyframe(self, env, keyframe):
        self.players[env].set_single_keyframe(parse_keyframe(json.loads(keyframe)["keyframe"]))

    def set_environment_keyframes(self, env, doc):
        self.players[env].set_keyframes([parse_keyframe(k) for k in json.loads(doc)["keyframes"]])

    def set_environment_keyframe_index(self, env, index):
        self.players[env].set_keyframe_index(index)

    def set_sensor_transform(self, env, sensor_name, m):
        self.r.updateCamera(env, self.projection, invert4(m))

    def set_sensor_transforms_from_keyframe(self, env, prefix):
        t, q = self.players[env].user_transform(prefix + self.uuid)
        self.set_sensor_transform(env, self.uuid, rigid_matrix(q, t))

    def render(self, threads=1):
        """Per environment: (RGBA8 [h, w, 4], depth in metres [h, w])."""
        self.r.draw(threads=threads)
        out = []
        for e in range(self.n):
            c = self.r.scene_image(self.r.color, e).view(np.uint8).reshape(self.res + (4,))
            d = self.r.scene_image(self.r.linear_depth, e)
            out.append((c, d))
        return out
