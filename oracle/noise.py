"""Oracle restatements of the Redwood depth-noise model (test infrastructure).

Used only by ``tests/``.  Two restatements:

* ``redwood_f32`` -- the float32 arithmetic of habitat-sim's CUDA kernel
  (``src/esp/sensor/RedwoodNoiseModel.cu:20-101``) driven by the same
  random numbers the GB300 kernel uses: Philox4x32-10 (Salmon et al.,
  SC'11; pinned by the Random123 known-answer vectors in the tests) of the
  counter (pixel, image, call) under the seed, mapped through a 4097-knot
  normal quantile table computed here with ``scipy.special.ndtri``.  Same
  inputs and state give bit-identical output.
* ``redwood_reference_cpu`` -- habitat-sim's own CPU algorithm
  (``src_python/habitat_sim/sensors/noise_models/redwood_depth_noise_model.py``:
  float64 index remapping and quantisation, numpy normals), for the
  statistical GPU-versus-CPU comparison the reference's test makes
  (``tests/test_noise_models.py:24-51``).
"""
import numpy as np

F = np.float32
KNOTS = 4097
M32 = 0xFFFFFFFF


def philox4x32_10(c0, c1, c2, c3, k0, k1):
    """Vectorised Philox4x32-10 of uint32 counters under a 2 x 32-bit key."""
    c = [np.asarray(x, np.uint32) for x in np.broadcast_arrays(c0, c1, c2, c3)]
    k0, k1 = int(k0) & M32, int(k1) & M32
    m0, m1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
    for _ in range(10):
        p0 = c[0].astype(np.uint64) * m0
        p1 = c[2].astype(np.uint64) * m1
        n0 = (p1 >> np.uint64(32)).astype(np.uint32) ^ c[1] ^ np.uint32(k0)
        n2 = (p0 >> np.uint64(32)).astype(np.uint32) ^ c[3] ^ np.uint32(k1)
        c = [n0, (p1 & np.uint64(M32)).astype(np.uint32), n2, (p0 & np.uint64(M32)).astype(np.uint32)]
        k0 = (k0 + 0x9E3779B9) & M32
        k1 = (k1 + 0xBB67AE85) & M32
    return c


def normal_table():
    """Knot k = Phi^-1((k + 0.5) / 4097) in float32, mirrored to be odd."""
    from scipy.special import ndtri
    t = np.zeros(KNOTS, np.float32)
    k = np.arange(KNOTS // 2 + 1)
    v = ndtri((k + 0.5) / KNOTS).astype(np.float32)
    t[k] = v
    t[KNOTS - 1 - k] = -v
    t[KNOTS // 2] = 0
    return t


def normals(bits, table):
    u = bits >> np.uint32(8)
    k = (u >> np.uint32(12)).astype(np.int64)
    f = (u & np.uint32(4095)).astype(F) * F(1.0 / 4096.0)
    t0, t1 = table[k], table[k + 1]
    return t0 + f * (t1 - t0)


def _c_round(q):
    """C round(): halves away from zero."""
    r = np.trunc(q)
    frac = q - r
    return r + np.where(frac >= 0.5, 1.0, 0.0) - np.where(frac <= -0.5, 1.0, 0.0)


def redwood_f32(depth, model, mult, seed, call, image=0, table=None):
    """Noisy depth of one H x W image, as the GB300 kernel computes it."""
    depth = np.ascontiguousarray(depth, np.float32)
    H, W = depth.shape
    table = normal_table() if table is None else table
    cells = np.ascontiguousarray(model, np.float32).reshape(-1, 5)
    idx = np.arange(H * W, dtype=np.uint32)
    b = philox4x32_10(idx, np.uint32(image), np.uint32(call & M32), np.uint32((call >> 32) & M32),
                      seed & M32, (seed >> 32) & M32)
    n0, n1, n2 = normals(b[0], table), normals(b[1], table), normals(b[2], table)
    r = (idx // W).astype(np.int64)
    col = (idx % W).astype(np.int64)
    ymax, xmax, m = F(H - 1), F(W - 1), F(mult)
    y = (np.minimum(np.maximum(r.astype(F) + (n0 * F(0.25)) * m, F(0)), ymax) + F(0.5)).astype(np.int64)
    x = (np.minimum(np.maximum(col.astype(F) + (n1 * F(0.25)) * m, F(0)), xmax) + F(0.5)).astype(np.int64)
    d = depth[y - y % 2, x - x % 2]
    with np.errstate(divide="ignore", invalid="ignore"):
        ux = ((x.astype(F) / xmax) * F(639) + F(0.5)).astype(np.int64) if xmax > 0 else np.zeros_like(x)
        uy = ((y.astype(F) / ymax) * F(479) + F(0.5)).astype(np.int64) if ymax > 0 else np.zeros_like(y)
        i2 = ((d + F(1)) / F(2)).astype(np.int64)
        i1 = i2 - 1
        w = (d - (i1.astype(F) * F(2) + F(1))) / F(2)
        cell = (uy // 6) * 80 + ux // 8
        f = (F(1) - w) * cells[cell, np.clip(i1, 0, 4)] + w * cells[cell, np.clip(i2, 0, 4)]
        ud = np.where(f < F(1e-5), F(0), d / f).astype(F)
        q = (np.float64(F(35.13)) / ud.astype(np.float64) +
             ((n2 * F(0.027778)) * m).astype(np.float64)) * 8.0
        denom = _c_round(q).astype(F)
        out = np.where(denom > F(1e-5), (F(35.13) * F(8)) / denom, F(0)).astype(F)
    out = np.where((d >= F(10)) | (ud == 0), F(0), out)
    return out.reshape(H, W)


def redwood_reference_cpu(depth, model, mult, rng):
    """habitat-sim's CPU implementation of the model (float64 remapping and
    quantisation; normals from `rng`), vectorised."""
    depth = np.asarray(depth, np.float32)
    H, W = depth.shape
    cells = np.asarray(model, np.float32).reshape(80, 80, 5)
    rn = rng.standard_normal((H, W, 3)).astype(np.float32)
    j, i = np.meshgrid(np.arange(H), np.arange(W), indexing="ij")
    ymax, xmax = H - 1.0, W - 1.0
    y = (np.minimum(np.maximum(j + rn[..., 0] * 0.25 * mult, 0.0), ymax) + 0.5).astype(np.int64)
    x = (np.minimum(np.maximum(i + rn[..., 1] * 0.25 * mult, 0.0), xmax) + 0.5).astype(np.int64)
    d = depth[y - y % 2, x - x % 2].astype(np.float64)
    ux = (x / xmax * 639.0 + 0.5).astype(np.int64) // 8
    uy = (y / ymax * 479.0 + 0.5).astype(np.int64) // 6
    i2 = ((d + 1) / 2).astype(np.int64)
    i1 = i2 - 1
    a = (d - (i1 * 2.0 + 1.0)) / 2.0
    f = (1.0 - a) * cells[uy, ux, np.clip(i1, 0, 4)] + a * cells[uy, ux, np.minimum(i2, 4)]
    with np.errstate(divide="ignore", invalid="ignore"):
        ud = np.where(f < 1e-5, 0.0, d / f)
        denom = np.round((35.130 / ud + rn[..., 2] * 0.027778 * mult) * 8.0)
        out = np.where(denom <= 1e-5, 0.0, 35.130 * 8.0 / denom)
    out = np.where((d >= 10.0) | (ud == 0.0), 0.0, out)
    return out.astype(np.float32)
