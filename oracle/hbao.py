"""Oracle restatement of horizon-based ambient occlusion (test infrastructure).

Used only by ``tests/``.  It restates habitat-sim's HBAO
(``src/esp/gfx_batch/Hbao.cpp:595-1038``; shaders
``src/shaders/gfx_batch/hbao/hbao.frag``, ``bilateralblur.frag``,
``hbao_blur.frag``, ``viewnormal.frag``, ``hbao_deinterleave.frag``,
``hbao_reinterleave.frag``) -- the classic and the cache-aware algorithms,
each with the bilateral or the special blur -- as numpy float32 arithmetic
in the operation order the GB300 kernels use.  Classic:
view positions from linear depth (background = far plane), normals from the
nearer of the forward/backward neighbour differences, 8 jittered directions
x 4 steps, 8-bit AO, depth-aware 7-tap blurs along x then y (8-bit between
them) and the colour multiply.  The jitter table is rebuilt from the
Mersenne twister (numpy's legacy generator with seed 5489 is
``std::mt19937``'s default stream), and pow / exp2 use the same polynomial
definitions (Taylor series of 2^f, atanh series of log2) as the kernels, so
results are bit-identical.  The GL effect itself is unavailable on this
machine, so parity with the reference's pixels is unpinned.

Cache-aware (``drawCacheAwareInternal``, Hbao.cpp:943-1038): the linear
depth deinterleaved into 16 quarter-resolution layers (layer oy * 4 + ox
holds full-resolution pixels (4 qx + ox, 4 qy + oy); quarter size
ceil(w / 4) x ceil(h / 4), texels beyond the image read as the far plane),
view normals reconstructed at full resolution and stored as RGBA8
(n * 0.5 + 0.5), each layer's AO computed with the layer's unquantized jitter
``random[layer]`` at quarter-resolution steps (radius / 4, samples in the
same layer), stored as 8-bit AO (or RG16F) and reinterleaved to full
resolution.  Special blur (``HbaoFlag::UseAoSpecialBlur``): the AO pass
stores (AO, view depth) as two IEEE halves (round to nearest even) and both
blur passes take the depth from there (``hbao_blur.frag``); the first pass
stores (blurred AO, centre depth) as halves again.
"""
import math

import numpy as np

F = np.float32
EXP2_C = [1.0178086284895471e-07, 1.3215486660556053e-06, 1.5252733646775596e-05,
          0.0001540352968731895, 0.0013333557872101665, 0.009618128649890423,
          0.05550410971045494, 0.24022650718688965, 0.6931471824645996, 1.0]
LOG2_C = [0.1111111119389534, 0.1428571492433548, 0.20000000298023224, 0.3333333432674408, 1.0]


def config(intensity=0.732, bias=0.05, radius=1.84, blur_sharpness=10.0, no_blur=False,
           special_blur=False, cache_aware=False):
    """HbaoConfiguration defaults (Hbao.h:135-138) and the algorithm
    (HbaoType::Classic or CacheAware)."""
    assert not (no_blur and special_blur), "NoBlur and UseAoSpecialBlur exclude each other"
    return dict(intensity=F(intensity), bias=F(bias), radius=F(radius),
                blur_sharpness=F(blur_sharpness), no_blur=bool(no_blur),
                special_blur=bool(special_blur), cache_aware=bool(cache_aware))


def poly_exp2(x):
    x = np.asarray(x, F)
    n = np.floor(x)
    f = (x - n).astype(F)
    p = np.full_like(x, F(EXP2_C[0]))
    for c in EXP2_C[1:]:
        p = (p * f + F(c)).astype(F)
    with np.errstate(over="ignore", invalid="ignore"):
        out = np.ldexp(p, np.clip(n, -1000, 1000).astype(np.int32)).astype(F)
    return np.where(x < F(-149), F(0), out).astype(F)


def poly_log2(x):
    m, e = np.frexp(np.asarray(x, F))
    sel = m < F(0.7071067690849304)
    m = np.where(sel, m * F(2), m).astype(F)
    e = np.where(sel, e - 1, e)
    t = ((m - F(1)) / (m + F(1))).astype(F)
    t2 = (t * t).astype(F)
    q = np.full_like(t, F(LOG2_C[0]))
    for c in LOG2_C[1:]:
        q = (q * t2 + F(c)).astype(F)
    return (e.astype(F) + (t * q) * F(2.885390043258667)).astype(F)


def poly_pow(a, e):
    a = np.asarray(a, F)
    with np.errstate(divide="ignore", invalid="ignore"):
        r = poly_exp2(F(e) * poly_log2(np.where(a > 0, a, F(1))))
    return np.where(a > 0, r, F(1) if e == 0 else F(0)).astype(F)


def jitter_table(quantized=True):
    """4 x 4 x (cos, sin, start offset, 0), Hbao.cpp:603-617: 16-bit snorm as
    the classic algorithm reads it from its texture, or the float values the
    cache-aware algorithm passes as a uniform (Hbao.cpp:1000)."""
    raw = np.random.RandomState(5489)._bit_generator.random_raw(32).astype(np.uint64)
    out = np.zeros((16, 4), np.float32)
    for i in range(16):
        r1 = F(float(raw[2 * i])) / F(4294967296.0)
        r2 = F(float(raw[2 * i + 1])) / F(4294967296.0)
        angle = F(6.28318530718) * r1 / F(8)
        v = [F(math.cos(float(angle))), F(math.sin(float(angle))), r2]
        for k in range(3):
            if not quantized:
                out[i, k] = v[k]
                continue
            s = float(v[k] * F(32767))
            out[i, k] = F(math.floor(s + 0.5) if s >= 0 else -math.floor(-s + 0.5)) / F(32767)
    return out


def directions():
    out = np.zeros((8, 2), np.float32)
    for d in range(8):
        a = F(2) * F(3.14159265) / F(8) * F(d)
        out[d] = (F(math.cos(float(a))), F(math.sin(float(a))))
    return out


def scene_info(projection, w, h, radius):
    """Per-image constants (Hbao.cpp:761-786, 874-895)."""
    m = np.asarray(projection, np.float32).reshape(4, 4)   # [col][row]
    p00, p11, p20, p21, p22 = m[0, 0], m[1, 1], m[2, 0], m[2, 1], m[2, 2]
    p30, p31, p32 = m[3, 0], m[3, 1], m[3, 2]
    ortho = m[3, 3] != 0
    pi = np.zeros(4, np.float32)
    pi[0] = F(2) / p00
    pi[1] = F(2) / p11
    if ortho:
        pi[2] = -(F(1) + p30) / p00
        pi[3] = -(F(1) - p31) / p11
        far = (p32 - F(1)) / p22
        rts = F(radius) * F(0.5) * (F(h) / pi[1])
    else:
        pi[2] = -(F(1) - p20) / p00
        pi[3] = -(F(1) + p21) / p11
        far = p32 / (p22 + F(1))
        rts = F(radius) * F(0.5) * (F(0.5) * F(h) * p00)
    return dict(pi=pi, far=F(far), rts=F(rts), ortho=bool(ortho))


def _clamp01(v):
    return np.fmin(np.fmax(v, F(0)), F(1)).astype(F)


def _unorm8(v):
    return (_clamp01(v) * F(255) + F(0.5)).astype(np.uint8)


def _half(v):
    """IEEE half, round to nearest even, back to float32."""
    return np.asarray(v, F).astype(np.float16).astype(F)


def hbao(color, depth, projection, cfg):
    """Apply the effect to one image: color uint8 [h, w, 4], depth float32
    [h, w] (metres, 0 = background); returns the new colour."""
    depth = np.asarray(depth, np.float32)
    h, w = depth.shape
    s = scene_info(projection, w, h, cfg["radius"])
    L = np.where(depth == 0, s["far"], depth).astype(F)
    pi = s["pi"]
    r2 = cfg["radius"] * cfg["radius"]
    neg_inv_r2 = F(-1) / F(r2)
    pow_exp = max(cfg["intensity"], F(0))
    bias = min(max(cfg["bias"], F(0)), F(1))
    ao_mult = F(1) / (F(1) - bias)
    cache = cfg.get("cache_aware", False)
    special = cfg.get("special_blur", False)
    jit = jitter_table(quantized=not cache)
    dirs = directions()
    y, x = np.meshgrid(np.arange(h), np.arange(w), indexing="ij")
    inv_w, inv_h = F(1) / F(w), F(1) / F(h)
    u = ((x.astype(F) + F(0.5)) / F(w)).astype(F)
    v = ((y.astype(F) + F(0.5)) / F(h)).astype(F)

    def fetch(tx, ty):
        return L[np.clip(ty, 0, h - 1), np.clip(tx, 0, w - 1)]

    def view(uu, vv, z):
        k = F(1) if s["ortho"] else z
        return [((uu * pi[0] + pi[2]) * k).astype(F), ((vv * pi[1] + pi[3]) * k).astype(F), z]

    def sub(a, b):
        return [(a[i] - b[i]).astype(F) for i in range(3)]

    def dot(a, b):
        return ((a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]).astype(F)

    def min_diff(p, pr, pl):
        v1, v2 = sub(pr, p), sub(p, pl)
        sel = dot(v1, v1) < dot(v2, v2)
        return [np.where(sel, v1[i], v2[i]).astype(F) for i in range(3)]

    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        # Normal reconstruction at full resolution (both algorithms).
        Pf = view(u, v, fetch(x, y))
        pr = view((u + inv_w).astype(F), v, fetch(x + 1, y))
        pl = view((u + (-inv_w)).astype(F), v, fetch(x - 1, y))
        pt = view(u, (v + inv_h).astype(F), fetch(x, y + 1))
        pb = view(u, (v + (-inv_h)).astype(F), fetch(x, y - 1))
        a, b = min_diff(Pf, pr, pl), min_diff(Pf, pt, pb)
        c = [(a[1] * b[2] - a[2] * b[1]).astype(F), (a[2] * b[0] - a[0] * b[2]).astype(F),
             (a[0] * b[1] - a[1] * b[0]).astype(F)]
        inv_len = (F(1) / np.sqrt(dot(c, c))).astype(F)
        if not cache:
            P = Pf
            N = [(-(c[i] * inv_len)).astype(F) for i in range(3)]
            radius = (s["rts"] / (F(1) if s["ortho"] else P[2])).astype(F)
            j = jit[(y & 3) * 4 + (x & 3)]
        else:
            # The normal through its RGBA8 texture; the pixel's own layer and
            # quarter-resolution texel; uv from the layer's texel centre.
            qw, qh = (w + 3) // 4, (h + 3) // 4
            inv_q4x, inv_q4y = (F(1) / F(qw)) / F(4), (F(1) / F(qh)) / F(4)
            ox, oy, qx, qy = x & 3, y & 3, x >> 2, y >> 2
            enc = [_unorm8((c[i] * inv_len) * F(0.5) + F(0.5)) for i in range(3)]
            N = [(-((enc[i].astype(F) / F(255)) * F(2) - F(1))).astype(F) for i in range(3)]
            u = ((qx.astype(F) * F(4) + (ox.astype(F) + F(0.5))) * inv_q4x).astype(F)
            v = ((qy.astype(F) * F(4) + (oy.astype(F) + F(0.5))) * inv_q4y).astype(F)
            P = view(u, v, L)
            radius = ((s["rts"] / (F(1) if s["ortho"] else P[2])) / F(4)).astype(F)
            j = jit[oy * 4 + ox]
            inv_w, inv_h = (F(1) / F(qw)), (F(1) / F(qh))
        step = (radius / F(5)).astype(F)
        ao = np.zeros((h, w), np.float32)
        for d in range(8):
            dc, ds = dirs[d]
            dx = (dc * j[..., 0] - ds * j[..., 1]).astype(F)
            dy = (dc * j[..., 1] + ds * j[..., 0]).astype(F)
            ray = (j[..., 2] * step + F(1)).astype(F)
            for _ in range(4):
                kx = np.rint((ray * dx).astype(F))
                ky = np.rint((ray * dy).astype(F))
                su = (kx * inv_w + u).astype(F)
                sv = (ky * inv_h + v).astype(F)
                ox_ = np.fmin(np.fmax(kx, F(-65536)), F(65536)).astype(np.int64)
                oy_ = np.fmin(np.fmax(ky, F(-65536)), F(65536)).astype(np.int64)
                if not cache:
                    zs = fetch(x + ox_, y + oy_)
                else:
                    tx = np.clip(qx + ox_, 0, qw - 1) * 4 + ox
                    ty = np.clip(qy + oy_, 0, qh - 1) * 4 + oy
                    inside = (tx < w) & (ty < h)
                    zs = np.where(inside, L[np.minimum(ty, h - 1), np.minimum(tx, w - 1)], s["far"]).astype(F)
                S = view(su, sv, zs)
                ray = (ray + step).astype(F)
                V = sub(S, P)
                vv = dot(V, V)
                ndotv = (dot(N, V) / np.sqrt(vv)).astype(F)
                ao = (ao + _clamp01(ndotv - bias) * _clamp01(vv * neg_inv_r2 + F(1))).astype(F)
        ao = (ao * (ao_mult / F(32))).astype(F)
        occl = poly_pow(_clamp01(F(1) - ao * F(2)), pow_exp)

    color = np.array(color, np.uint8, copy=True)

    def modulate(f):
        for ch in range(3):
            color[..., ch] = _unorm8((color[..., ch].astype(F) / F(255)) * f)
        return color

    if cfg["no_blur"]:
        # The cache-aware result reaches the colour through its 8-bit layers.
        return modulate((_unorm8(occl).astype(F) / F(255)).astype(F) if cache else occl)
    falloff = F(1) / (F(2) * F(1.5) * F(1.5))
    sharp = F(cfg["blur_sharpness"]) / F(1)
    if special:
        aoq, dq = _half(occl), _half(P[2])
    else:
        q = _unorm8(occl)
    for axis in (0, 1):
        if special:
            ct = aoq.copy()
        else:
            ct = (q.astype(F) / F(255)).astype(F)
        cd = dq if special else L
        wt = np.ones((h, w), np.float32)
        for sign in (1, -1):
            for r in (1, 2, 3):
                tx = np.clip(x + sign * r, 0, w - 1) if axis == 0 else x
                ty = np.clip(y + sign * r, 0, h - 1) if axis == 1 else y
                cc = aoq[ty, tx] if special else (q[ty, tx].astype(F) / F(255)).astype(F)
                dd = ((cd[ty, tx] - cd) * sharp).astype(F)
                wgt = poly_exp2(((F(-r) * F(r)) * falloff - dd * dd).astype(F))
                wt = (wt + wgt).astype(F)
                ct = (ct + cc * wgt).astype(F)
        out = (ct / wt).astype(F)
        if axis == 0:
            if special:
                aoq = _half(out)
            else:
                q = _unorm8(out)
        else:
            return modulate(out)
