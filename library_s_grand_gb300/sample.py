"""Host restatement of the on-device shot sampler (grand_engine_sample).

The device kernel (csrc/grand_sample.cu) draws every error position of a shot
with Philox4x32-10 (Salmon et al., SC 2011): key = the 64-bit seed, counter =
{group * 32 + lane, shot low word, shot high word, 0x47524E44}; word u of that
block decides position 128 * group + 32 * u + lane, which flips when the word
is below floor(p * 2^32) (2^32 - 1 for p >= 1).  This module reproduces the
same draws on the host, vectorised with numpy, so tests and users can check a
device-sampled batch bit for bit.
"""
from __future__ import annotations

import numpy as np

_M32 = np.uint64(0xFFFFFFFF)


def philox4x32_10(c0, c1, c2, c3, k0, k1):
    """Philox4x32-10 on arrays of 32-bit counters (any broadcastable shapes) and
    a 32-bit key pair; returns the four output words as uint64 arrays."""
    c = [np.asarray(x, dtype=np.uint64) & _M32 for x in (c0, c1, c2, c3)]
    k0, k1 = np.uint64(k0) & _M32, np.uint64(k1) & _M32
    for _ in range(10):
        p0 = np.uint64(0xD2511F53) * c[0]
        p1 = np.uint64(0xCD9E8D57) * c[2]
        c = [((p1 >> np.uint64(32)) ^ c[1] ^ k0) & _M32, p1 & _M32,
             ((p0 >> np.uint64(32)) ^ c[3] ^ k1) & _M32, p0 & _M32]
        k0 = (k0 + np.uint64(0x9E3779B9)) & _M32
        k1 = (k1 + np.uint64(0xBB67AE85)) & _M32
    return c


def thresholds(p) -> np.ndarray:
    """floor(p * 2^32) per position, clamped to [0, 2^32 - 1] (FP32 p, as on the device)."""
    s = np.asarray(p, dtype=np.float32).astype(np.float64) * 4294967296.0
    return np.clip(np.floor(s), 0, 4294967295).astype(np.uint64)


def flips(p, seed: int, first_shot: int, num_shots: int) -> np.ndarray:
    """(num_shots, m) uint8 flips exactly as the device sampler draws them."""
    thr = thresholds(p)
    m = thr.shape[0]
    groups = (m + 127) // 128
    shot = np.arange(first_shot, first_shot + num_shots, dtype=np.uint64)[:, None, None]
    g = np.arange(groups, dtype=np.uint64)[None, :, None]
    lane = np.arange(32, dtype=np.uint64)[None, None, :]
    words = philox4x32_10(g * np.uint64(32) + lane, shot & _M32, shot >> np.uint64(32),
                          np.uint64(0x47524E44), seed & 0xFFFFFFFF, seed >> 32)
    # (shot, group, word u, lane) flattens to position 128 * group + 32 * u + lane
    w = np.stack([np.broadcast_to(words[u], (num_shots, groups, 32)) for u in range(4)], axis=2)
    w = w.reshape(num_shots, groups * 128)
    t = np.zeros(groups * 128, dtype=np.uint64)
    t[:m] = thr
    out = (w < t[None, :]).astype(np.uint8)
    return out[:, :m]


def css_records(h, p, seed: int, first_shot: int, num_shots: int, errors: bool) -> np.ndarray:
    """Records of a CSS code registered with `errors` (m entries) or syndromes
    (n entries of h . e mod 2), as grand_engine_sample writes them."""
    f = flips(p, seed, first_shot, num_shots).astype(np.int64)
    if errors:
        return f.astype(np.int32)
    return (f @ np.asarray(h, dtype=np.int64).T % 2).astype(np.int32)


def dem_records(h, l, p, seed: int, first_shot: int, num_shots: int) -> np.ndarray:
    """DEM records: detectors (h . f mod 2) then true logical flips (f . l mod 2)."""
    f = flips(p, seed, first_shot, num_shots).astype(np.int64)
    det = f @ np.asarray(h, dtype=np.int64).T % 2
    log = f @ np.asarray(l, dtype=np.int64) % 2
    return np.concatenate([det, log], axis=1).astype(np.int32)
