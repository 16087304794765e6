"""Seeded synthetic workloads for the encoder hot path.

The reference publishes no dataset or benchmark inputs, so every workload is a
deterministic function of a 64-bit seed (splitmix64 counter streams), shared
byte-for-byte by the CPU oracle, the CUDA path, the tests and the benchmark:

* ``smooth_texture``   uniform noise low-pass filtered by a 5x5 box (integer mean);
* ``pan_sequence``     frames cut from one texture at a random-walk global pan with
                       quarter-pel resolution (H.264 6-tap / bilinear sampling),
                       plus Gaussian noise sigma=2, clipped to 0..255;
* ``shift_sequence``   integer global shift plus per-16x16-block local offsets and
                       noise (the QCIF integer-pel workload);
* ``residual_blocks``  int16 residuals, Laplacian(scale 6) clipped to +-255;
* ``rgb_frame``        packed BGR24 uniform bytes.
"""
from __future__ import annotations

import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def splitmix64(seed: int, n: int, stream: int = 0) -> np.ndarray:
    """n outputs of the splitmix64 generator for (seed, stream)."""
    with np.errstate(over="ignore"):
        base = np.uint64((seed * 0x2545F4914F6CDD1D + stream * 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF)
        i = np.arange(1, n + 1, dtype=np.uint64)
        z = base + i * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def uniform_u8(seed: int, shape, stream: int = 0) -> np.ndarray:
    n = int(np.prod(shape))
    return (splitmix64(seed, n, stream) >> np.uint64(56)).astype(np.uint8).reshape(shape)


def _unit(seed: int, n: int, stream: int) -> np.ndarray:
    """Uniform doubles in (0, 1]."""
    return ((splitmix64(seed, n, stream) >> np.uint64(11)).astype(np.float64) + 1.0) / 9007199254740992.0


def gaussian(seed: int, shape, sigma: float, stream: int = 0) -> np.ndarray:
    """Box-Muller normals, rounded half away from zero to int32."""
    n = int(np.prod(shape))
    u1 = _unit(seed, n, 2 * stream + 1)
    u2 = _unit(seed, n, 2 * stream + 2)
    x = np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2) * sigma
    return (np.sign(x) * np.floor(np.abs(x) + 0.5)).astype(np.int32).reshape(shape)


def box5(img: np.ndarray) -> np.ndarray:
    """5x5 box filter with edge replication and truncating integer mean."""
    p = np.pad(img.astype(np.int32), 2, mode="edge")
    c = np.cumsum(np.cumsum(p, 0), 1)
    c = np.pad(c, ((1, 0), (1, 0)))
    h, w = img.shape
    s = c[5:5 + h, 5:5 + w] - c[0:h, 5:5 + w] - c[5:5 + h, 0:w] + c[0:h, 0:w]
    return s // 25


def smooth_texture(seed: int, h: int, w: int) -> np.ndarray:
    return box5(uniform_u8(seed, (h, w), stream=7)).astype(np.int16)


def _tap6(a, axis):
    """Unscaled (1,-5,20,20,-5,1) filter; output index i covers input i..i+5."""
    n = a.shape[axis] - 5
    s = [np.take(a, np.arange(k, k + n), axis=axis).astype(np.int64) for k in range(6)]
    return s[0] - 5 * s[1] + 20 * s[2] + 20 * s[3] - 5 * s[4] + s[5]


def qpel_crop(base: np.ndarray, oy_q: int, ox_q: int, h: int, w: int) -> np.ndarray:
    """h x w block of `base` starting at quarter-pel offset (oy_q, ox_q) >= 0,
    sampled with the H.264 luma interpolation (6-tap half-pel, bilinear
    quarter-pel), edges replicated."""
    fy, ry = oy_q >> 2, oy_q & 3
    fx, rx = ox_q >> 2, ox_q & 3
    pad = 4
    reg = np.pad(base.astype(np.int64), pad, mode="edge")
    y0, x0 = fy + pad, fx + pad
    # sample planes over rows y0-3..y0+h+3 and cols x0-3..x0+w+3
    R = reg[y0 - 3:y0 + h + 4, x0 - 3:x0 + w + 4]

    def G(dy, dx):
        return R[3 + dy:3 + dy + h, 3 + dx:3 + dx + w]

    def clip(v):
        return np.clip(v, 0, 255)

    def B(dy, dx):  # half-pel right of (dy,dx)
        t = _tap6(R[3 + dy:3 + dy + h, 3 + dx - 2:3 + dx + w + 3], 1)
        return clip((t + 16) >> 5)

    def H(dy, dx):  # half-pel below (dy,dx)
        t = _tap6(R[3 + dy - 2:3 + dy + h + 3, 3 + dx:3 + dx + w], 0)
        return clip((t + 16) >> 5)

    def J(dy, dx):
        v = _tap6(R[3 + dy - 2:3 + dy + h + 3, 3 + dx - 2:3 + dx + w + 3], 0)
        t = _tap6(v, 1)
        return clip((t + 512) >> 10)

    sel = rx | (ry << 2)
    avg = lambda a, b: (a + b + 1) >> 1
    table = {
        0: lambda: G(0, 0), 2: lambda: B(0, 0), 8: lambda: H(0, 0), 10: lambda: J(0, 0),
        1: lambda: avg(G(0, 0), B(0, 0)), 3: lambda: avg(G(0, 1), B(0, 0)),
        4: lambda: avg(G(0, 0), H(0, 0)), 12: lambda: avg(G(1, 0), H(0, 0)),
        6: lambda: avg(J(0, 0), B(0, 0)), 14: lambda: avg(J(0, 0), B(1, 0)),
        9: lambda: avg(J(0, 0), H(0, 0)), 11: lambda: avg(J(0, 0), H(0, 1)),
        5: lambda: avg(B(0, 0), H(0, 0)), 7: lambda: avg(B(0, 0), H(0, 1)),
        13: lambda: avg(H(0, 0), B(1, 0)), 15: lambda: avg(H(0, 1), B(1, 0)),
    }
    return table[sel]().astype(np.int16)


def pan_sequence(seed: int, w: int, h: int, nframes: int, max_pan_px: int = 16,
                 sigma: float = 2.0) -> list[np.ndarray]:
    """Frames of one smooth texture under a global pan random walk; each step
    is uniform in [-max_pan_px, max_pan_px]^2 at quarter-pel resolution."""
    margin = 4 * max_pan_px + 8
    base = smooth_texture(seed, h + 2 * margin, w + 2 * margin)
    steps = (splitmix64(seed, 2 * nframes, stream=11) % np.uint64(8 * max_pan_px + 1)).astype(np.int64)
    steps = steps - 4 * max_pan_px
    py, px = 4 * margin, 4 * margin
    lo, hi = 4 * 4, 4 * (2 * margin - 4)
    frames = []
    for t in range(nframes):
        f = qpel_crop(base, py, px, h, w).astype(np.int32)
        f += gaussian(seed + 1000 + t, (h, w), sigma)
        frames.append(np.clip(f, 0, 255).astype(np.int16))
        ny, nx = py + int(steps[2 * t]), px + int(steps[2 * t + 1])
        py = ny if lo <= ny <= hi else py - int(steps[2 * t])
        px = nx if lo <= nx <= hi else px - int(steps[2 * t + 1])
    return frames


def shift_sequence(seed: int, w: int, h: int, nframes: int, max_global: int = 8,
                   max_local: int = 4, sigma: float = 2.0) -> list[np.ndarray]:
    """Integer global shift per frame plus per-16x16-block local offsets and
    Gaussian noise, clipped to 0..255."""
    cur = smooth_texture(seed, h, w).astype(np.int32)
    frames = [cur.astype(np.int16)]
    rows, cols = h // 16, w // 16
    for t in range(1, nframes):
        g = (splitmix64(seed + t, 2, stream=21) % np.uint64(2 * max_global + 1)).astype(np.int64) - max_global
        loc = (splitmix64(seed + t, 2 * rows * cols, stream=22) % np.uint64(2 * max_local + 1)).astype(np.int64)
        loc = loc.reshape(rows, cols, 2) - max_local
        nxt = np.empty_like(cur)
        yy, xx = np.mgrid[0:16, 0:16]
        for r in range(rows):
            for c in range(cols):
                sy = np.clip(r * 16 + yy + g[0] + loc[r, c, 0], 0, h - 1)
                sx = np.clip(c * 16 + xx + g[1] + loc[r, c, 1], 0, w - 1)
                nxt[r * 16:(r + 1) * 16, c * 16:(c + 1) * 16] = cur[sy, sx]
        nxt = np.clip(nxt + gaussian(seed + 2000 + t, (h, w), sigma), 0, 255)
        frames.append(nxt.astype(np.int16))
        cur = nxt
    return frames


def tile_sequence(seed: int, w: int, h: int, nframes: int, period: int = 4, max_global: int = 8) -> list[np.ndarray]:
    """A random period x period tile repeated over the frame, each next frame
    the previous one rolled by a seeded integer shift: every candidate a whole
    number of periods from the match has the same distortion, so the scans
    meet exact ties everywhere and the prediction decides them."""
    tile = (splitmix64(seed, period * period, stream=23) % np.uint64(256)).astype(np.int16).reshape(period, period)
    cur = np.tile(tile, ((h + period - 1) // period, (w + period - 1) // period))[:h, :w]
    frames = [cur.copy()]
    for t in range(1, nframes):
        g = (splitmix64(seed + t, 2, stream=24) % np.uint64(2 * max_global + 1)).astype(np.int64) - max_global
        cur = np.roll(cur, (int(g[0]), int(g[1])), axis=(0, 1))
        frames.append(cur.copy())
    return frames


def residual_blocks(seed: int, n: int, scale: float = 6.0) -> np.ndarray:
    """n int16 values, Laplacian(0, scale) rounded half away from zero, clipped to +-255."""
    u = _unit(seed, n, 31) - 0.5
    x = -scale * np.sign(u) * np.log(np.maximum(1.0 - 2.0 * np.abs(u), 1e-300))
    x = np.sign(x) * np.floor(np.abs(x) + 0.5)
    return np.clip(x, -255, 255).astype(np.int16)


def residual_frame_420(seed: int, w: int = 1920, h: int = 1080):
    """Y (h x w), U, V (h/2 x w/2) residual planes of a 4:2:0 frame."""
    y = residual_blocks(seed, w * h).reshape(h, w)
    u = residual_blocks(seed + 1, (w // 2) * (h // 2)).reshape(h // 2, w // 2)
    v = residual_blocks(seed + 2, (w // 2) * (h // 2)).reshape(h // 2, w // 2)
    return y, u, v


def rgb_frame(seed: int, w: int, h: int) -> np.ndarray:
    """Packed BGR24 (h x w x 3) uniform bytes."""
    return uniform_u8(seed, (h, w, 3), stream=41)
