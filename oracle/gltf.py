"""Oracle-side importer for batch-friendly glTF files (test infrastructure).

This module is part of the CPU oracle: it is used only by ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU baseline, never by the
product path.  It restates, in plain Python/numpy, what habitat-sim's batch
renderer gets out of its importer stack for a file passed to
``Renderer::addFile`` (``src/esp/gfx_batch/Renderer.cpp:354-867``):

* textures, one per imported texture, as RGBA8 2D arrays whose row 0 is the
  *bottom* row (the importer flips images to a Y-up origin);
* meshes made indexed, with texture coordinates flipped to a Y-up origin
  (``v' = 1 - v``), triangle fans/strips expanded to triangle lists;
* flat materials (base colour, texture, array layer, texture matrix);
* mesh views (mesh, index byte offset, index count, material, transform),
  taken from the ``MAGNUMX_mesh_views`` extras when present
  (``Renderer.cpp:700-738``), else one per mesh assignment;
* named node-hierarchy templates: named root nodes whose immediate children
  are the mesh views (``Renderer.cpp:750-790``), or the whole file flattened
  with absolute transforms under one name (``Renderer.cpp:795-820``), or a
  scene-less single-mesh file (``Renderer.cpp:663-690``).

The glTF 2.0 reader itself (JSON, accessors, KHR_texture_transform,
KHR_texture_ktx, KHR_materials_unlit) follows the published glTF/KTX2
specifications; the conventions above are those of the third-party Magnum
importer the reference links (not vendored in the reference checkout) and
are pinned by the reference's golden screenshots.
"""
import json
import os
import struct
import zlib

import numpy as np

GL_NEAREST = 9728
GL_LINEAR = 9729
GL_REPEAT = 10497
GL_CLAMP_TO_EDGE = 33071
GL_MIRRORED_REPEAT = 33648

FILTER_NEAREST, FILTER_LINEAR = 0, 1
WRAP_REPEAT, WRAP_CLAMP, WRAP_MIRROR = 0, 1, 2

_WRAP = {GL_REPEAT: WRAP_REPEAT, GL_CLAMP_TO_EDGE: WRAP_CLAMP,
         GL_MIRRORED_REPEAT: WRAP_MIRROR}

_COMPONENT = {5120: np.int8, 5121: np.uint8, 5122: np.int16, 5123: np.uint16,
              5125: np.uint32, 5126: np.float32}
_NCOMP = {"SCALAR": 1, "VEC2": 2, "VEC3": 3, "VEC4": 4, "MAT4": 16}


class ImportError_(Exception):
    pass


# --------------------------------------------------------------------------
# Images

def decode_png(data):
    """Decode an 8-bit non-interlaced PNG into uint8 [h, w, 4], row 0 = bottom."""
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ImportError_("not a PNG")
    pos = 8
    idat = b""
    palette = None
    trns = None
    w = h = depth = ctype = None
    while pos < len(data):
        (length,) = struct.unpack(">I", data[pos:pos + 4])
        tag = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + length]
        pos += 12 + length
        if tag == b"IHDR":
            w, h, depth, ctype, _, _, interlace = struct.unpack(">IIBBBBB", body)
            if depth != 8 or interlace != 0:
                raise ImportError_("only 8-bit non-interlaced PNG is supported")
        elif tag == b"PLTE":
            palette = np.frombuffer(body, np.uint8).reshape(-1, 3)
        elif tag == b"tRNS":
            trns = np.frombuffer(body, np.uint8)
        elif tag == b"IDAT":
            idat += body
        elif tag == b"IEND":
            break
    channels = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    raw = zlib.decompress(idat)
    stride = w * channels
    out = np.zeros((h, stride), np.int32)
    prev = np.zeros(stride, np.int32)
    bpp = channels
    p = 0
    for y in range(h):
        ftype = raw[p]
        line = np.frombuffer(raw[p + 1:p + 1 + stride], np.uint8).astype(np.int32)
        p += 1 + stride
        cur = np.zeros(stride, np.int32)
        if ftype == 0:
            cur = line.copy()
        elif ftype == 2:
            cur = (line + prev) & 255
        else:
            for i in range(stride):
                a = cur[i - bpp] if i >= bpp else 0
                b = prev[i]
                c = prev[i - bpp] if i >= bpp else 0
                if ftype == 1:
                    pred = a
                elif ftype == 3:
                    pred = (a + b) >> 1
                elif ftype == 4:
                    pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
                    pred = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
                else:
                    raise ImportError_(f"bad PNG filter {ftype}")
                cur[i] = (line[i] + pred) & 255
        out[y] = cur
        prev = cur
    px = out.astype(np.uint8).reshape(h, w, channels)
    rgba = np.empty((h, w, 4), np.uint8)
    if ctype == 0:
        rgba[..., :3] = px[..., :1]
        rgba[..., 3] = 255
    elif ctype == 2:
        rgba[..., :3] = px
        rgba[..., 3] = 255
    elif ctype == 3:
        rgba[..., :3] = palette[px[..., 0]]
        alpha = np.full(256, 255, np.uint8)
        if trns is not None:
            alpha[:len(trns)] = trns
        rgba[..., 3] = alpha[px[..., 0]]
    elif ctype == 4:
        rgba[..., :3] = px[..., :1]
        rgba[..., 3] = px[..., 1]
    else:
        rgba[:] = px
    return rgba[::-1].copy()  # Y-up: row 0 is the bottom row


def _bc1_block(block, rgba_out):
    c0, c1, bits = struct.unpack("<HHI", block)

    def expand(c):
        r, g, b = (c >> 11) & 31, (c >> 5) & 63, c & 31
        return np.array([(r << 3) | (r >> 2), (g << 2) | (g >> 4), (b << 3) | (b >> 2), 255],
                        np.int32)

    p0, p1 = expand(c0), expand(c1)
    if c0 > c1:
        p2 = (2 * p0 + p1) // 3
        p3 = (p0 + 2 * p1) // 3
        p2[3] = p3[3] = 255
    else:
        p2 = (p0 + p1) // 2
        p2[3] = 255
        p3 = np.array([0, 0, 0, 255], np.int32)
    pal = [p0, p1, p2, p3]
    for i in range(16):
        rgba_out[i // 4, i % 4] = pal[(bits >> (2 * i)) & 3]


def decode_ktx2(data):
    """Decode a KTX2 file (RGB8/RGBA8 or BC1) into uint8 [layers, h, w, 4], row 0 = bottom.

    Returns (pixels, is_array).  Only the base mip level is decoded."""
    if data[:12] != b"\xabKTX 20\xbb\r\n\x1a\n":
        raise ImportError_("not a KTX2 file")
    vk, _ts, w, h, d, layers, faces, levels, sc = struct.unpack("<9I", data[12:48])
    if sc != 0 or faces != 1 or d > 1:
        raise ImportError_("unsupported KTX2 layout")
    _dfo, _dfl, kvo, kvl = struct.unpack("<4I", data[48:64])
    off, length, _ = struct.unpack("<3Q", data[80:104])
    orient = "rd"
    kv = data[kvo:kvo + kvl]
    p = 0
    while p + 4 <= len(kv):
        (n,) = struct.unpack("<I", kv[p:p + 4])
        entry = kv[p + 4:p + 4 + n]
        key, _, val = entry.partition(b"\x00")
        if key == b"KTXorientation":
            orient = val.rstrip(b"\x00").decode()
        p += 4 + ((n + 3) & ~3)
    nl = max(layers, 1)
    h = max(h, 1)
    level = data[off:off + length]
    if vk in (23, 29):  # R8G8B8 UNORM / SRGB
        px = np.frombuffer(level, np.uint8).reshape(nl, h, w, 3)
        out = np.empty((nl, h, w, 4), np.uint8)
        out[..., :3] = px
        out[..., 3] = 255
    elif vk in (37, 43):  # R8G8B8A8 UNORM / SRGB
        out = np.frombuffer(level, np.uint8).reshape(nl, h, w, 4).copy()
    elif vk in (131, 132, 133, 134):  # BC1
        bw, bh = (w + 3) // 4, (h + 3) // 4
        out = np.empty((nl, bh * 4, bw * 4, 4), np.uint8)
        q = 0
        for layer in range(nl):
            for by in range(bh):
                for bx in range(bw):
                    blk = np.empty((4, 4, 4), np.int32)
                    _bc1_block(level[q:q + 8], blk)
                    q += 8
                    out[layer, by * 4:by * 4 + 4, bx * 4:bx * 4 + 4] = blk
        out = out[:, :h, :w].copy()
    else:
        raise ImportError_(f"unsupported KTX2 vkFormat {vk}")
    if len(orient) > 1 and orient[1] == "d":
        out = out[:, ::-1].copy()
    return out, layers > 0


# --------------------------------------------------------------------------
# glTF

def _mat_from_node(node):
    if "matrix" in node:
        return np.array(node["matrix"], np.float32).reshape(4, 4)  # [col][row]
    t = np.array(node.get("translation", [0, 0, 0]), np.float64)
    q = np.array(node.get("rotation", [0, 0, 0, 1]), np.float64)
    s = np.array(node.get("scale", [1, 1, 1]), np.float64)
    x, y, z, w = q
    r = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y + z * w), 2 * (x * z - y * w)],
                  [2 * (x * y - z * w), 1 - 2 * (x * x + z * z), 2 * (y * z + x * w)],
                  [2 * (x * z + y * w), 2 * (y * z - x * w), 1 - 2 * (x * x + y * y)]])
    m = np.eye(4)
    m[:3, :3] = r * s[:, None]  # column c = R[:, c] * s[c], stored as [col][row]
    m[3, :3] = t
    return m.astype(np.float32)


def _matmul(a, b):
    """Column-major 4x4 product a*b (storage [col][row]) in float32, each
    entry summed left to right without fused multiply-adds:
    ``((a0*b0 + a1*b1) + a2*b2) + a3*b3``."""
    f = np.float32
    out = np.empty((4, 4), np.float32)
    for c in range(4):
        for r in range(4):
            s = f(a[0, r]) * f(b[c, 0])
            for k in range(1, 4):
                s = f(s + f(f(a[k, r]) * f(b[c, k])))
            out[c, r] = s
    return out


class GltfFile:
    """Everything ``addFile`` needs out of one file, before renderer offsets."""

    def __init__(self):
        self.textures = []   # dict(pixels [L,h,w,4] u8, mag, wrap_s, wrap_t)
        self.meshes = []     # dict(positions, colors|None, texcoords|None, object_ids|None, indices)
        self.materials = []  # dict(color[4], texture|None, layer, matrix 3x3 [col][row])
        self.mesh_views = []  # dict(mesh, index_offset_bytes, index_count, material, transform)
        self.templates = []  # (name, begin, end) over mesh_views
        self.scene_count = 0


def load_gltf(path, whole=False, name=None, no_textures=False):
    with open(path, "rb") as f:
        raw = f.read()
    base = os.path.dirname(path)
    bin_chunk = None
    if raw[:4] == b"glTF":
        _, _, total = struct.unpack("<III", raw[:12])
        p = 12
        doc = None
        while p < total:
            clen, ctype = struct.unpack("<II", raw[p:p + 8])
            chunk = raw[p + 8:p + 8 + clen]
            if ctype == 0x4E4F534A:
                doc = json.loads(chunk)
            elif ctype == 0x004E4942:
                bin_chunk = chunk
            p += 8 + clen
    else:
        doc = json.loads(raw)

    buffers = []
    for b in doc.get("buffers", []):
        if "uri" in b:
            with open(os.path.join(base, b["uri"]), "rb") as f:
                buffers.append(f.read())
        else:
            buffers.append(bin_chunk)

    def view_bytes(i):
        bv = doc["bufferViews"][i]
        o = bv.get("byteOffset", 0)
        return buffers[bv["buffer"]][o:o + bv["byteLength"]], bv.get("byteStride")

    def accessor(i):
        acc = doc["accessors"][i]
        dt = np.dtype(_COMPONENT[acc["componentType"]])
        nc = _NCOMP[acc["type"]]
        count = acc["count"]
        data, stride = view_bytes(acc["bufferView"])
        off = acc.get("byteOffset", 0)
        elem = dt.itemsize * nc
        stride = stride or elem
        buf = np.frombuffer(data, np.uint8)
        rows = np.empty((count, elem), np.uint8)
        for k in range(count):
            rows[k] = buf[off + k * stride: off + k * stride + elem]
        out = rows.view(dt).reshape(count, nc)
        if acc.get("normalized"):
            out = out.astype(np.float32) / np.float32(np.iinfo(dt).max)
        return out

    out = GltfFile()

    # Textures: KHR_texture_ktx textures sharing one image and sampler become
    # one 2D array texture, the layer goes to the material.
    texture_map = {}     # glTF texture index -> (file texture id, layer)
    if not no_textures:
        dedup = {}
        for ti, tex in enumerate(doc.get("textures", [])):
            ext = tex.get("extensions", {}).get("KHR_texture_ktx")
            src = ext["source"] if ext else tex["source"]
            layer = ext.get("layer", 0) if ext else 0
            key = (src, tex.get("sampler")) if ext else ("tex", ti)
            if key not in dedup:
                img = doc["images"][src]
                if "bufferView" in img:
                    blob, _ = view_bytes(img["bufferView"])
                    mime = img.get("mimeType", "")
                else:
                    with open(os.path.join(base, img["uri"]), "rb") as f:
                        blob = f.read()
                    mime = "image/ktx2" if img["uri"].endswith(".ktx2") else "image/png"
                compressed = False
                if mime == "image/ktx2" or blob[:4] == b"\xabKTX":
                    pixels, _ = decode_ktx2(blob)
                    compressed = struct.unpack("<I", blob[12:16])[0] in (131, 132, 133, 134)
                else:
                    pixels = decode_png(blob)[None]
                smp = doc["samplers"][tex["sampler"]] if "sampler" in tex else {}
                dedup[key] = len(out.textures)
                minf = smp.get("minFilter", 9987)    # absent: linear, linear between levels
                out.textures.append(dict(
                    pixels=pixels,
                    mag=FILTER_NEAREST if smp.get("magFilter", GL_LINEAR) == GL_NEAREST
                    else FILTER_LINEAR,
                    min=FILTER_NEAREST if minf in (9728, 9984, 9986) else FILTER_LINEAR,
                    mip=1 if minf in (9984, 9985) else (2 if minf in (9986, 9987) else 0),
                    compressed=bool(compressed),
                    wrap_s=_WRAP[smp.get("wrapS", GL_REPEAT)],
                    wrap_t=_WRAP[smp.get("wrapT", GL_REPEAT)]))
            texture_map[ti] = (dedup[key], layer)
    else:
        # Texture ids are still assigned so draw batching sees the same ids.
        dedup = {}
        for ti, tex in enumerate(doc.get("textures", [])):
            ext = tex.get("extensions", {}).get("KHR_texture_ktx")
            src = ext["source"] if ext else tex["source"]
            key = (src, tex.get("sampler")) if ext else ("tex", ti)
            if key not in dedup:
                dedup[key] = len(dedup)
            texture_map[ti] = (dedup[key], ext.get("layer", 0) if ext else 0)
    out.texture_id_count = len(set(v[0] for v in texture_map.values()))

    # Meshes: one per primitive.
    prim_ids = []
    for m in doc.get("meshes", []):
        ids = []
        for prim in m["primitives"]:
            attrs = prim["attributes"]
            pos = accessor(attrs["POSITION"]).astype(np.float32)
            n = len(pos)
            colors = None
            if "COLOR_0" in attrs:
                c = accessor(attrs["COLOR_0"]).astype(np.float32)
                colors = np.ones((n, 4), np.float32)
                colors[:, :c.shape[1]] = c
            tc = None
            if "TEXCOORD_0" in attrs:
                tc = accessor(attrs["TEXCOORD_0"]).astype(np.float32).copy()
                tc[:, 1] = np.float32(1.0) - tc[:, 1]
            normals = None
            if "NORMAL" in attrs:
                normals = accessor(attrs["NORMAL"]).astype(np.float32).reshape(-1, 3)
            oid = None
            if "_OBJECT_ID" in attrs:
                oid = accessor(attrs["_OBJECT_ID"]).reshape(-1).astype(np.uint32)
            if "indices" in prim:
                idx = accessor(prim["indices"]).reshape(-1).astype(np.uint32)
            else:
                idx = np.arange(n, dtype=np.uint32)
            mode = prim.get("mode", 4)
            if mode == 6:    # triangle fan
                idx = np.array([[idx[0], idx[i], idx[i + 1]] for i in range(1, len(idx) - 1)],
                               np.uint32).reshape(-1)
            elif mode == 5:  # triangle strip
                tris = []
                for i in range(len(idx) - 2):
                    if i % 2 == 0:
                        tris.append([idx[i], idx[i + 1], idx[i + 2]])
                    else:
                        tris.append([idx[i + 1], idx[i], idx[i + 2]])
                idx = np.array(tris, np.uint32).reshape(-1)
            elif mode != 4:
                raise ImportError_(f"unsupported primitive mode {mode}")
            ids.append(len(out.meshes))
            out.meshes.append(dict(positions=pos, colors=colors, texcoords=tc,
                                   object_ids=oid, indices=idx, normals=normals))
            prim_ids.append(prim.get("material", -1))
        m["_ids"] = ids

    # Materials.
    for mat in doc.get("materials", []):
        pbr = mat.get("pbrMetallicRoughness", {})
        color = np.array(pbr.get("baseColorFactor", [1, 1, 1, 1]), np.float32)
        texture = None
        layer = 0
        matrix = np.eye(3, dtype=np.float32)
        bct = pbr.get("baseColorTexture")
        if bct is not None:
            texture, layer = texture_map[bct["index"]]
            tt = bct.get("extensions", {}).get("KHR_texture_transform")
            if tt:
                matrix = _texture_transform(tt)
        out.materials.append(dict(color=color, texture=texture, layer=layer, matrix=matrix,
                                  flat="KHR_materials_unlit" in mat.get("extensions", {})))

    nodes = doc.get("nodes", [])
    scenes = doc.get("scenes", [])
    out.scene_count = len(scenes)
    if not scenes:
        if len(out.meshes) != 1 or out.materials:
            raise ImportError_("expected exactly one mesh and no material for a scene-less file")
        if not whole:
            raise ImportError_("scene-less file has to be added with the Whole flag")
        out.mesh_views.append(dict(mesh=0, index_offset_bytes=0,
                                   index_count=len(out.meshes[0]["indices"]),
                                   material=-1, transform=np.eye(4, dtype=np.float32)))
        out.templates.append((name or path, 0, 1))
        return out
    if len(scenes) != 1:
        raise ImportError_("expected exactly one scene")

    parent = {}
    for i, nd in enumerate(nodes):
        for c in nd.get("children", []):
            parent[c] = i
    has_views = any("meshViewIndexOffset" in nd.get("extras", {}) for nd in nodes)

    local = [_mat_from_node(nd) for nd in nodes]

    def absolute(i):
        chain = []
        while i is not None:
            chain.append(i)
            i = parent.get(i)
        m = np.eye(4, dtype=np.float32)
        for j in reversed(chain):
            m = _matmul(m, local[j])
        return m

    node_views = {}
    for i, nd in enumerate(nodes):
        if "mesh" not in nd:
            continue
        mesh = doc["meshes"][nd["mesh"]]
        for k, mid in enumerate(mesh["_ids"]):
            ex = nd.get("extras", {})
            if has_views:
                off = int(ex["meshViewIndexOffset"])
                cnt = int(ex["meshViewIndexCount"])
                mat = int(ex["meshViewMaterial"])
            else:
                off = 0
                cnt = len(out.meshes[mid]["indices"])
                mat = mesh["primitives"][k].get("material", -1)
            node_views.setdefault(i, []).append(len(out.mesh_views))
            out.mesh_views.append(dict(mesh=mid, index_offset_bytes=off, index_count=cnt,
                                       material=mat,
                                       transform=absolute(i) if whole else local[i]))

    if whole:
        out.templates.append((name or path, 0, len(out.mesh_views)))
    else:
        offset = 0
        for root in scenes[0]["nodes"]:
            children = nodes[root].get("children", [])
            nm = nodes[root].get("name")
            if not nm:
                raise ImportError_(f"node {root} has no name")
            out.templates.append((nm, offset, offset + len(children)))
            offset += len(children)
        if offset != len(out.mesh_views):
            raise ImportError_("mesh views are not immediate children of named roots")
    return out


def _texture_transform(tt):
    """KHR_texture_transform (Y-down texture space) as a Y-up 3x3 matrix [col][row]."""
    off = tt.get("offset", [0.0, 0.0])
    rot = tt.get("rotation", 0.0)
    sc = tt.get("scale", [1.0, 1.0])
    c, s = np.cos(rot), np.sin(rot)
    t = np.array([[1, 0, off[0]], [0, 1, off[1]], [0, 0, 1]], np.float64)
    r = np.array([[c, s, 0], [-s, c, 0], [0, 0, 1]], np.float64)
    scl = np.diag([sc[0], sc[1], 1.0])
    m_gltf = t @ r @ scl                    # row-major, acts on column vectors
    flip = np.array([[1, 0, 0], [0, -1, 1], [0, 0, 1]], np.float64)
    m = flip @ m_gltf @ flip
    return m.T.astype(np.float32)           # storage [col][row]
