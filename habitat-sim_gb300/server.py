"""Request serving over the batch renderer: continuous batching, a device
memory budget with least-recently-used eviction, latency percentiles.

A serving process keeps a catalog of scenes in host memory (as if read from
disk), a bounded set of them resident on the GPU, and answers requests --
(scene, 6-DoF camera pose, resolution) -- with RGBA8 colour, linear depth in
metres and uint32 semantic ids.  Each step packs pending requests into
render slots: fixed square viewports of each resolution class, laid out at
the start of one ragged framebuffer.  Every used slot is pointed at its
request's resident scene (``setSceneSources``), unused slots are disabled,
all slots are drawn by one batched launch (a CUDA graph), and the used slot
rectangles are copied to pinned host memory on a second stream while the
host prepares the next step and the GPU draws it (two plane sets, alternated
by the draws).  Scenes are loaded on first use into "content" scenes (1 x 1 viewports
that are never drawn themselves) and evicted least-recently-used when the
device budget or the number of content scenes would be exceeded; eviction
returns their device ranges to the renderer's free lists.

habitat-sim's batch renderer draws a fixed set of environments per call
(src/esp/gfx_batch/Renderer.cpp:1292-1353) and its callers own the request
loop (src/esp/sim/BatchReplayRenderer.cpp:117-151); this module is that loop
for a request-driven caller of the same draw path.
"""
import collections
import concurrent.futures
import dataclasses
import gc
import math
import os
import time

import numpy as np

from . import procedural

CLASSES = (64, 128, 256)
CLASS_P = (0.3, 0.5, 0.2)
ROOM_LO = np.array([-6.0, 0.0, -6.0])
ROOM_HI = np.array([6.0, 3.0, 6.0])


# ------------------------------------------------------------------ catalog
@dataclasses.dataclass
class SceneAsset:
    positions: np.ndarray   # [V, 3] float32
    colors: np.ndarray      # [V, 4] float32
    texcoords: np.ndarray   # [V, 2] float32
    object_ids: np.ndarray  # [V] uint32
    indices: np.ndarray     # [3T] uint32
    texture: np.ndarray     # [layers, h, w, 4] uint8
    parts: list             # per object: (first index, index count, texture layer)

    @property
    def triangles(self):
        return len(self.indices) // 3

    def device_bytes(self):
        """Bytes the renderer keeps on the device for this scene: 40 per
        vertex (position, colour, texcoord), 4 per index, 4 per texel, and
        per object (one mesh view) 32 per box: one per 32-triangle chunk and
        one per 32 chunks."""
        boxes = 0
        for (_, count, _) in self.parts:
            chunks = (count // 3 + 31) // 32
            boxes += chunks + (chunks + 31) // 32
        return len(self.positions) * 40 + len(self.indices) * 4 + self.texture.size + boxes * 32


class TexelPool:
    """Uniform-noise RGBA8 texels (alpha 255) in host memory.  Every catalog
    scene's texture layers are a window of the pool at an offset drawn from
    the scene's seed: the host holds one pool, the device a distinct copy of
    every resident scene's layers."""

    def __init__(self, nbytes, seed):
        rng = np.random.default_rng([seed, 2718])
        self.data = np.frombuffer(rng.bytes(nbytes), np.uint8).copy()
        self.data.reshape(-1, 4)[:, 3] = 255

    def window(self, key, layers, side):
        n = layers * side * side * 4
        if n > len(self.data):
            raise ValueError(f"{layers} layers of {side}^2 texels exceed the texel pool")
        rng = np.random.default_rng([key, 161803])
        off = int(rng.integers(0, (len(self.data) - n) // 4 + 1)) * 4
        return self.data[off:off + n].reshape(layers, side, side, 4)


def serving_scene(seed, triangles, texture=None):
    """One catalog scene of about ``triangles`` triangles: a 12 x 3 x 12 m
    room shell (80 % of the budget) and 20 boxes (20 %), random RGB per
    vertex, object id 1 for the shell and 2..21 for the boxes, planar
    texcoords.  ``texture`` is the scene's [layers, h, w, 4] texel array
    (default: one 64 x 64 noise layer); object k samples layer k % layers."""
    rng = np.random.default_rng([seed, 104729])
    n = max(2, int(round(math.sqrt(0.8 * triangles / 12.0))))
    m = max(1, int(round(math.sqrt(0.2 * triangles / (20 * 12.0)))))
    parts = [procedural.box_faces(ROOM_LO, ROOM_HI, n, inward=True)]
    ids = [np.full(len(parts[0][0]), 1, np.uint32)]
    for b in range(20):
        size = rng.uniform(0.3, 1.5, size=3)
        c = rng.uniform(ROOM_LO[[0, 2]] + 1.0, ROOM_HI[[0, 2]] - 1.0)
        lo = np.array([c[0] - size[0] / 2, 0.0, c[1] - size[2] / 2])
        parts.append(procedural.box_faces(lo, lo + size, m, inward=False))
        ids.append(np.full(len(parts[-1][0]), 2 + b, np.uint32))
    if texture is None:
        texture = rng.integers(0, 256, size=(1, 64, 64, 4), dtype=np.uint8)
        texture[..., 3] = 255
    layers = texture.shape[0]
    pos, idx, views, base, first = [], [], [], 0, 0
    for k, (p, t) in enumerate(parts):
        pos.append(p)
        idx.append(t + base)
        views.append((first, t.size, k % layers))
        base += len(p)
        first += t.size
    pos = np.concatenate(pos).astype(np.float32)
    col = np.ones((len(pos), 4), np.float32)
    col[:, :3] = rng.integers(0, 256, size=(len(pos), 3)).astype(np.float32) / np.float32(255.0)
    uv = np.stack([pos[:, 0] + pos[:, 1], pos[:, 2] + pos[:, 1]], 1).astype(np.float32) / 2.0
    return SceneAsset(pos, col, uv, np.concatenate(ids),
                      np.concatenate(idx).astype(np.uint32).reshape(-1), texture, views)


def add_asset(r, asset, name, texture_filter=1):
    """Add one catalog scene's resources to renderer ``r`` (the GPU renderer
    or the oracle): its texture array, its mesh, one material per texture
    layer it uses, and a hierarchy template ``name`` with one mesh view per
    object.  Returns (mesh, texture)."""
    tex = r.addTexture(asset.texture, filter=texture_filter)
    mesh = r.addMesh(asset.positions, asset.colors, asset.texcoords, asset.object_ids, asset.indices)
    mats, views = {}, []
    for (first, count, layer) in asset.parts:
        if layer not in mats:
            mats[layer] = r.addMaterial((1, 1, 1, 1), tex, layer)
        views.append((mesh, first, count, mats[layer], None))
    r.addNodeHierarchyTemplate(name, views)
    return mesh, tex


class SceneCatalog:
    """``count`` scenes with triangle counts log-uniform in ``tri_range``,
    generated on first use from (seed, scene) and kept in host memory.
    With ``texture_side``, scene s gets max(1, round(triangles /
    tris_per_layer)) texture layers of texture_side^2 RGBA8 noise, windows
    of one shared host pool of ``pool_bytes`` (the default sizes make a
    256-scene catalog of 10k-1M triangles about 40 GB on the device);
    otherwise one 64 x 64 layer per scene."""

    def __init__(self, count, seed=0, tri_range=(1e4, 1e6), texture_side=None,
                 tris_per_layer=24000, pool_bytes=1 << 30):
        rng = np.random.default_rng([seed, 31337])
        self.seed = seed
        self.targets = np.exp(rng.uniform(math.log(tri_range[0]), math.log(tri_range[1]), count))
        self.texture_side = texture_side
        self.tris_per_layer = tris_per_layer
        self.pool_bytes = pool_bytes
        self._pool = None
        self._assets = {}

    def __len__(self):
        return len(self.targets)

    def layers(self, scene):
        return max(1, int(round(self.targets[scene] / self.tris_per_layer))) if self.texture_side else 1

    def asset(self, scene):
        a = self._assets.get(scene)
        if a is None:
            key = self.seed * 100003 + scene
            tex = None
            if self.texture_side:
                if self._pool is None:
                    self._pool = TexelPool(self.pool_bytes, self.seed)
                tex = self._pool.window(key, self.layers(scene), self.texture_side)
            a = self._assets[scene] = serving_scene(key, int(self.targets[scene]), tex)
        return a


# ----------------------------------------------------------------- requests
@dataclasses.dataclass
class Request:
    scene: int
    resolution: int
    view: np.ndarray          # world -> camera, [col][row] float32
    hfov: float = 90.0
    arrival: float = 0.0      # seconds after the start of serving
    rid: int = -1
    done: float = math.nan    # seconds after the start of serving
    color: np.ndarray = None     # [res, res, 4] uint8, row 0 = bottom
    depth: np.ndarray = None     # [res, res] float32 metres, 0 = nothing drawn
    semantic: np.ndarray = None  # [res, res] uint32

    @property
    def latency(self):
        return self.done - self.arrival


def _rot(axis, a):
    """Rotation matrices [..., 3, 3] by angles ``a`` about x (0), y (1), z (2)."""
    c, s = np.cos(a), np.sin(a)
    m = np.zeros(np.shape(a) + (3, 3))
    i, j = [(1, 2), (2, 0), (0, 1)][axis]
    k = 3 - i - j
    m[..., k, k] = 1.0
    m[..., i, i] = c
    m[..., i, j] = -s
    m[..., j, i] = s
    m[..., j, j] = c
    return m


def pose_views(x, y, z, yaw, pitch, roll):
    """World -> camera matrices ([n][col][row] float32) of cameras at
    (x, y, z) rotated by yaw (about +y), then pitch (about +x), then roll
    (about -z); arguments are arrays of n values."""
    r = _rot(1, np.asarray(yaw, np.float64)) @ _rot(0, np.asarray(pitch, np.float64)) @ \
        _rot(2, np.asarray(roll, np.float64))
    t = np.stack([x, y, z], -1).astype(np.float64)
    inv = np.zeros(r.shape[:-2] + (4, 4))
    rt = np.swapaxes(r, -1, -2)
    inv[..., :3, :3] = rt
    inv[..., :3, 3] = -(rt @ t[..., None])[..., 0]
    inv[..., 3, 3] = 1.0
    return np.swapaxes(inv, -1, -2).astype(np.float32)


def pose_view(x, y, z, yaw, pitch, roll):
    """pose_views for one camera."""
    return pose_views(np.array([x]), np.array([y]), np.array([z]), np.array([yaw]),
                      np.array([pitch]), np.array([roll]))[0]


def random_requests(catalog, count, rate, seed=0, classes=CLASSES, p=CLASS_P, zipf=None):
    """Poisson arrivals at ``rate`` per second; scene uniform over the
    catalog (or Zipf with exponent ``zipf``); resolution from ``classes``
    with probabilities ``p``; 6-DoF pose inside the room: position uniform
    (0.5 m from the walls, 0.5-2.5 m high), yaw uniform, pitch U(-30, 30)
    deg, roll U(-10, 10) deg; hfov 90 deg."""
    rng = np.random.default_rng([seed, 7])
    arrivals = np.cumsum(rng.exponential(1.0 / rate, count)) if rate else np.zeros(count)
    if zipf:
        w = 1.0 / np.arange(1, len(catalog) + 1) ** zipf
        scenes = rng.choice(len(catalog), size=count, p=w / w.sum())
    else:
        scenes = rng.integers(0, len(catalog), count)
    res = rng.choice(classes, size=count, p=p)
    xz = rng.uniform(ROOM_LO[[0, 2]] + 0.5, ROOM_HI[[0, 2]] - 0.5, size=(count, 2))
    y = rng.uniform(0.5, 2.5, count)
    yaw = rng.uniform(0, 2 * math.pi, count)
    pitch = np.radians(rng.uniform(-30, 30, count))
    roll = np.radians(rng.uniform(-10, 10, count))
    views = pose_views(xz[:, 0], y, xz[:, 1], yaw, pitch, roll)
    return [Request(int(scenes[i]), int(res[i]), views[i], 90.0, float(arrivals[i]), i)
            for i in range(count)]


# ------------------------------------------------------------ host policies
class Residency:
    """Which catalog scenes are resident, in least-recently-used order, under
    a byte budget and a count limit (pure bookkeeping; no device calls)."""

    def __init__(self, budget_bytes, capacity):
        self.budget = budget_bytes
        self.capacity = capacity
        self.lru = collections.OrderedDict()  # scene -> (slot, bytes)
        self.free_slots = list(range(capacity - 1, -1, -1))
        self.bytes = 0

    def touch(self, scene):
        """The scene's content slot if resident (now most recently used), else None."""
        e = self.lru.get(scene)
        if e is None:
            return None
        self.lru.move_to_end(scene)
        return e[0]

    def plan(self, need, pinned):
        """Scenes to evict, oldest first, so that ``need`` more bytes and one
        more slot fit; scenes in ``pinned`` stay.  Raises if impossible."""
        if need > self.budget:
            raise MemoryError(f"a scene of {need} bytes exceeds the budget of {self.budget}")
        out, freed, slots = [], 0, len(self.free_slots)
        for scene, (_, b) in self.lru.items():
            if self.bytes - freed + need <= self.budget and slots > 0:
                break
            if scene in pinned:
                continue
            out.append(scene)
            freed += b
            slots += 1
        if self.bytes - freed + need > self.budget or slots == 0:
            raise MemoryError("budget too small for the scenes one step needs")
        return out

    def remove(self, scene):
        slot, b = self.lru.pop(scene)
        self.bytes -= b
        self.free_slots.append(slot)
        return slot

    def add(self, scene, nbytes):
        slot = self.free_slots.pop()
        self.lru[scene] = (slot, nbytes)
        self.bytes += nbytes
        return slot


def take_batch(queues, slots, max_batch=None):
    """Continuous batching: up to ``slots[c]`` oldest requests of each
    resolution class ``c`` (FIFO per class); with ``max_batch``, at most that
    many requests in all, the earliest arrivals first."""
    batch = {}
    if max_batch is not None:
        for _ in range(max_batch):
            heads = [(q[0].arrival, c) for c, q in queues.items()
                     if q and len(batch.get(c, ())) < slots.get(c, 0)]
            if not heads:
                break
            c = min(heads)[1]
            batch.setdefault(c, []).append(queues[c].popleft())
        return batch
    for c, q in queues.items():
        k = min(len(q), slots.get(c, 0))
        if k:
            batch[c] = [q.popleft() for _ in range(k)]
    return batch


def percentiles(latencies_s):
    lat = np.sort(np.asarray(latencies_s, np.float64)) * 1e3
    if not len(lat):
        return dict(p50_ms=None, p99_ms=None, mean_ms=None)
    return dict(p50_ms=float(np.percentile(lat, 50)), p99_ms=float(np.percentile(lat, 99)),
                mean_ms=float(lat.mean()))


# ------------------------------------------------------------------ server
class RenderServer:
    """Serves requests for the scenes of ``catalog`` on one GPU.

    ``slots`` maps each square resolution to its number of render slots (the
    largest batch of that class one step takes; the default, 96 + 160 + 64,
    is 320 requests of the 0.3 / 0.5 / 0.2 mix of 64, 128 and 256 px, so that
    no class saturates before the others); ``max_resident`` bounds the
    resident scenes; ``budget_bytes`` bounds their device bytes (geometry,
    textures, chunk boxes; default: no limit); ``max_loads_per_step`` bounds
    the scene loads one step may wait for (requests beyond it wait for a
    later step, so that requests for resident scenes are not held up: loads
    are serial either way, and with one per step a request for a resident
    scene waits for at most one)."""

    def __init__(self, pkg, catalog, slots=None, max_resident=64, budget_bytes=None, graph=True,
                 device=0, max_loads_per_step=1):
        import torch

        self.torch = torch
        self.pkg = pkg
        self.catalog = catalog
        self.slots = dict(slots or {64: 96, 128: 160, 256: 64})
        self.graph = graph
        viewports, self.slot_base, self.class_offset = [], {}, {}
        px = 0
        for c in sorted(self.slots):
            self.slot_base[c] = len(viewports)
            self.class_offset[c] = px
            viewports += [(c, c)] * self.slots[c]
            px += c * c * self.slots[c]
        self.slot_px = px
        self.n_slots = len(viewports)
        self.content_base = len(viewports)
        viewports += [(1, 1)] * max_resident
        cfg = pkg.RendererConfiguration().setViewports(viewports).setDrawMode(pkg.DrawMode.Batched)
        # Two plane sets, alternated by the draws: the copy-back of step k
        # reads one set while step k + 1 draws into the other.
        self.r = pkg.RendererStandalone(cfg, pkg.RendererStandaloneConfiguration().setCudaDevice(
            device).setFlags(pkg.RendererStandaloneFlags.QuietLog | pkg.RendererStandaloneFlags.DoubleBuffer))
        # The launch shape that served the serving workload best (1024-thread
        # CTAs on 128 x 64 regions, 4 px small-triangle threshold: 238 k
        # requests/s against 185 k for the library's default 128 x 128
        # regions); tune() picks one for the caller's own catalog.
        self.r.setTuning(threads=1024, region_width=128, region_height=64, small_area=4, ctas_per_sm=1)
        for s in range(len(viewports)):
            self.r.setSceneEnabled(s, False)
        self.enabled = np.zeros(self.n_slots, bool)
        self.sources = np.arange(len(viewports), dtype=np.uint32)
        self.residency = Residency(budget_bytes if budget_bytes is not None else 1 << 62,
                                   max_resident)
        self.handles = {}  # scene -> (mesh, texture, template name)
        self.loads = self.evictions = 0
        self.max_loads_per_step = max_loads_per_step
        self.device = torch.device("cuda", device)
        self.stream = torch.cuda.Stream(device=self.device)
        self.copy_stream = torch.cuda.Stream(device=self.device)
        self._planes = (pkg.Plane.Color, pkg.Plane.LinearDepth, pkg.Plane.Semantic)
        self._views = {}  # device address of a plane set's colour plane -> views of its planes
        first = self._set_views()
        self.host = [[torch.empty((self.slot_px,) + tuple(t.shape[1:]), dtype=t.dtype,
                                  pin_memory=True) for t in first] for _ in range(2)]
        self._copies = collections.deque()  # copy-back events of the last two steps
        self._proj = {}
        self._step = 0
        self._copier = concurrent.futures.ThreadPoolExecutor(
            max_workers=max(1, min(8, (os.cpu_count() or 2) - 1)))

    def _set_views(self):
        """Device views of the plane set the last draw wrote (made once per set)."""
        key = self.r.planeDevicePointer(self.pkg.Plane.Color)[0]
        views = self._views.get(key)
        if views is None:
            views = self._views[key] = [self.r.deviceTensor(p) for p in self._planes]
        return views

    def close(self):
        self._copier.shutdown()
        self.torch.cuda.synchronize(self.device)
        self._views = {}
        self.r.close()

    # -- residency
    def _load(self, scene, pinned):
        a = self.catalog.asset(scene)
        need = a.device_bytes()
        for victim in self.residency.plan(need, pinned):
            self._evict(victim)
        r = self.r
        live0 = r.memoryUsage()[0]
        name = f"serving/{scene}"
        mesh, tex = add_asset(r, a, name)
        nbytes = r.memoryUsage()[0] - live0
        slot = self.residency.add(scene, nbytes)
        r.addNodeHierarchy(self.content_base + slot, name)
        self.handles[scene] = (mesh, tex, name)
        self.loads += 1
        return slot

    def _evict(self, scene):
        slot = self.residency.remove(scene)
        mesh, tex, name = self.handles.pop(scene)
        self.r.clear(self.content_base + slot)
        self.r.removeNodeHierarchyTemplate(name)
        self.r.removeMesh(mesh)
        self.r.removeTexture(tex)
        self.evictions += 1

    def _projection(self, hfov, c):
        key = (hfov, c)
        p = self._proj.get(key)
        if p is None:
            p = self._proj[key] = procedural.projection(hfov, c, c)
        return p

    # -- one step
    def _admit(self, batch):
        """Make the batch's scenes resident, oldest request first; a request
        whose scene cannot be loaded next to the scenes already taken (budget
        or resident-scene limit), or would exceed this step's loads, is
        deferred to a later step."""
        taken, deferred, pinned = {}, [], set()
        loads = 0
        for c in sorted(batch):
            for req in batch[c]:
                if self.residency.touch(req.scene) is None:
                    if self.catalog.asset(req.scene).device_bytes() > self.residency.budget:
                        raise MemoryError(f"scene {req.scene} exceeds the device budget")
                    if loads >= self.max_loads_per_step:
                        deferred.append(req)
                        continue
                    try:
                        self._load(req.scene, pinned)
                    except MemoryError:
                        deferred.append(req)
                        continue
                    loads += 1
                pinned.add(req.scene)
                taken.setdefault(c, []).append(req)
        return taken, deferred

    def launch(self, batch):
        """Bind, draw and start the copy-back of one step.  Returns a handle
        for ``finish`` and the requests deferred to a later step."""
        torch = self.torch
        batch, deferred = self._admit(batch)
        want = np.zeros(self.n_slots, bool)
        for c, reqs in batch.items():
            base = self.slot_base[c]
            projs = np.empty((len(reqs), 4, 4), np.float32)
            views = np.empty((len(reqs), 4, 4), np.float32)
            for i, req in enumerate(reqs):
                slot = self.residency.touch(req.scene)
                self.sources[base + i] = self.content_base + slot
                want[base + i] = True
                projs[i] = self._projection(req.hfov, c)
                views[i] = req.view
            self.r.updateCameras(projs, views, first=base)
        for s in np.nonzero(want != self.enabled)[0]:
            self.r.setSceneEnabled(int(s), bool(want[s]))
        self.enabled = want
        self.r.setSceneSources(self.sources[:self.n_slots])
        # This draw writes the plane set of the step before last: its
        # copy-back must be done first.
        if len(self._copies) == 2:
            self.stream.wait_event(self._copies.popleft())
        self.r.draw(self.stream, graph=self.graph)
        planes = self._set_views()
        buf = self.host[self._step % 2]
        self._step += 1
        self.copy_stream.wait_stream(self.stream)
        with torch.cuda.stream(self.copy_stream):
            for c, reqs in batch.items():
                o, n = self.class_offset[c], len(reqs) * c * c
                for dst, src in zip(buf, planes):
                    dst[o:o + n].copy_(src[o:o + n], non_blocking=True)
        ev = torch.cuda.Event()
        ev.record(self.copy_stream)
        self._copies.append(ev)
        return (batch, buf, ev), deferred

    def finish(self, handle, clock=None, keep_images=True):
        """Wait for a launched step and hand each request its images (with
        ``keep_images`` false, only its completion time: the images reached
        pinned host memory, where they stay until the step after next)."""
        batch, buf, ev = handle
        ev.synchronize()
        now = clock() if clock else math.nan
        if not keep_images:
            for reqs in batch.values():
                for req in reqs:
                    req.done = now
            return batch
        planes = [t.numpy() for t in buf]
        # One new array per resolution class and plane, copied out of the
        # double-buffered pinned staging on worker threads (the copies are
        # memory-bound); each request keeps views of its class's arrays.
        jobs = [(c, reqs, k, planes[k][self.class_offset[c]:self.class_offset[c] + len(reqs) * c * c])
                for c, reqs in batch.items() for k in range(3)]
        blocks = list(self._copier.map(np.copy, [j[3] for j in jobs]))
        for (c, reqs, k, _), blk in zip(jobs, blocks):
            for i, req in enumerate(reqs):
                img = blk[i * c * c:(i + 1) * c * c]
                if k == 0:
                    req.color = img.reshape(c, c, 4)
                elif k == 1:
                    req.depth = img.reshape(c, c)
                else:
                    req.semantic = img.reshape(c, c).view(np.uint32)
                    req.done = now
        return batch

    # -- launch shape
    def tune(self, make_requests, reps=2):
        """Choose the raster kernel's launch shape for serving: every shape of
        the autotuner's search space (threads per CTA, region, small-triangle
        threshold), then the bin capacity on the best, each timed as the
        closed-loop throughput of serving ``make_requests()`` (a fresh list
        per run, for scenes that are already resident; the best of ``reps``
        runs after an untimed one).  Applies the best and returns (tuning,
        trials)."""
        from . import autotune

        def rate(**cand):
            self.r.setTuning(**cand)
            self.serve(make_requests(), realtime=False, keep_images=False)
            return max(self.serve(make_requests(), realtime=False, keep_images=False)["requests_per_s"]
                       for _ in range(reps))

        trials = []
        for cand in autotune.BATCHED_SPACE:
            try:
                trials.append(dict(cand, queue_fill_percent=75, requests_per_s=rate(queue_fill_percent=75,
                                                                                   **cand)))
            except Exception as e:  # does not fit this GPU's shared memory
                trials.append(dict(cand, error=str(e)))
        best = max((t for t in trials if "requests_per_s" in t), key=lambda t: t["requests_per_s"])
        shape = {k: best[k] for k in ("threads", "region_width", "region_height", "small_area", "ctas_per_sm")}
        for fill in autotune.QUEUE_FILL:
            if fill != 75:
                t = dict(shape, queue_fill_percent=fill, requests_per_s=rate(queue_fill_percent=fill, **shape))
                trials.append(t)
                if t["requests_per_s"] > best["requests_per_s"]:
                    best = t
        self.r.setTuning(**shape, queue_fill_percent=best["queue_fill_percent"])
        return self.r.tuning(), trials

    # -- the request loop
    def serve(self, requests, realtime=True, keep_images=True, max_batch=None):
        """Serve ``requests`` (sorted by arrival).  With ``realtime`` a request
        is admitted once the wall clock passes its arrival time; otherwise
        all are pending from the start (a closed-loop saturation run).
        ``max_batch`` caps the requests of one step (1: the plain path, one
        request per draw).  Returns statistics; each request gets ``done``
        and, with ``keep_images``, its images."""
        queues = {c: collections.deque() for c in self.slots}
        pending = collections.deque(sorted(requests, key=lambda q: q.arrival))
        for req in pending:
            if req.resolution not in self.slots:
                raise ValueError(f"no render slots for resolution {req.resolution}")
        # The cyclic garbage collector is paused while serving: a full
        # collection walks every live request (images included) and stalls the
        # loop for tens of milliseconds, which would show in the tail latency.
        gc_was_enabled = gc.isenabled()
        gc.disable()
        try:
            return self._serve(queues, pending, requests, realtime, keep_images, max_batch)
        finally:
            if gc_was_enabled:
                gc.enable()

    def _serve(self, queues, pending, requests, realtime, keep_images, max_batch):
        t0 = time.perf_counter()
        clock = lambda: time.perf_counter() - t0
        if not realtime:
            for req in pending:
                req.arrival = 0.0
        inflight = collections.deque()
        steps = batched = 0
        loads0, ev0 = self.loads, self.evictions
        while pending or inflight or any(queues.values()):
            now = clock()
            while pending and pending[0].arrival <= now:
                req = pending.popleft()
                queues[req.resolution].append(req)
            batch = take_batch(queues, self.slots, max_batch)
            if batch:
                handle, deferred = self.launch(batch)
                for req in reversed(deferred):
                    queues[req.resolution].appendleft(req)
                inflight.append(handle)
                steps += 1
                batched += sum(len(v) for v in handle[0].values())
            if inflight and (len(inflight) >= 2 or not batch):
                self.finish(inflight.popleft(), clock, keep_images)
            elif not batch and pending:
                time.sleep(max(0.0, min(pending[0].arrival - clock(), 0.002)))
        elapsed = clock()
        lat = [q.latency for q in requests]
        stats = dict(requests=len(requests), steps=steps, elapsed_s=elapsed,
                     requests_per_s=len(requests) / elapsed if elapsed > 0 else None,
                     mean_batch=batched / steps if steps else 0.0,
                     loads=self.loads - loads0, evictions=self.evictions - ev0)
        stats.update(percentiles(lat))
        return stats
