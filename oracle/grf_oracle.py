"""CPU restatement of the random-field generator (csrc/ep_grf.cu).

TEST INFRASTRUCTURE ONLY: imported by tests/ as the checker of the GPU field.
The product never imports it.

Randomization (spectral) method (Shinozuka & Deodatis 1991; Kramer,
Kurbanmuradov & Sabelfeld 2007) with the library's draws restated: one
splitmix64 stream of the seed, 8 uniforms ((z >> 11) + 0.5) 2^-53 per harmonic,
u0..u3 for the wave vector (exponential: radial CDF inversion + uniform
direction; Gaussian: Box-Muller normals times sqrt 2), u4, u5 for the Box-Muller
amplitudes; components divided by the correlation lengths.  Field in FP64.
"""
from __future__ import annotations

import math

import numpy as np

M64 = (1 << 64) - 1


def _splitmix(seed, n):
    s = seed & M64
    out = np.empty(n, dtype=np.float64)
    for i in range(n):
        s = (s + 0x9E3779B97F4A7C15) & M64
        z = s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
        z = z ^ (z >> 31)
        out[i] = ((z >> 11) + 0.5) * (1.0 / 9007199254740992.0)
    return out


def _inv_exp3(u):
    F = lambda k: (2.0 / math.pi) * (math.atan(k) - k / (1.0 + k * k))
    lo, hi = 0.0, 1.0
    while F(hi) < u and hi < 1e300:
        hi *= 2.0
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        if F(mid) < u:
            lo = mid
        else:
            hi = mid
        if hi - lo <= 1e-15 * hi:
            break
    return 0.5 * (lo + hi)


def spectrum(dim, covariance, ell, nh, seed):
    u = _splitmix(seed, 8 * nh).reshape(nh, 8)
    kap = np.zeros((nh, dim))
    if covariance == "exponential":
        if dim == 2:
            q = 1.0 / (1.0 - u[:, 0])
            kr = np.sqrt(q * q - 1.0)
            th = 2.0 * math.pi * u[:, 1]
            kap[:, 0], kap[:, 1] = kr * np.cos(th), kr * np.sin(th)
        else:
            kr = np.array([_inv_exp3(v) for v in u[:, 0]])
            ct = 1.0 - 2.0 * u[:, 1]
            st = np.sqrt(np.maximum(0.0, 1.0 - ct * ct))
            ph = 2.0 * math.pi * u[:, 2]
            kap[:, 0], kap[:, 1], kap[:, 2] = kr * st * np.cos(ph), kr * st * np.sin(ph), kr * ct
    else:
        r1, r2 = np.sqrt(-2.0 * np.log(u[:, 0])), np.sqrt(-2.0 * np.log(u[:, 2]))
        comps = [math.sqrt(2.0) * r1 * np.cos(2 * math.pi * u[:, 1]), math.sqrt(2.0) * r1 * np.sin(2 * math.pi * u[:, 1]),
                 math.sqrt(2.0) * r2 * np.cos(2 * math.pi * u[:, 3])]
        for i in range(dim):
            kap[:, i] = comps[i]
    kap /= np.asarray(ell[:dim], dtype=np.float64)
    ra = np.sqrt(-2.0 * np.log(u[:, 4]))
    ab = np.stack([ra * np.cos(2 * math.pi * u[:, 5]), ra * np.sin(2 * math.pi * u[:, 5])], axis=1)
    return kap, ab


def field(X, dim, covariance, ell, mean, std, vmin, nh, seed, amplitudes_f32=True):
    """max(mean + f(X), vmin) in FP64 (amplitudes rounded to FP32 as the GPU stores them)."""
    kap, ab = spectrum(dim, covariance, ell, nh, seed)
    if amplitudes_f32:
        ab = ab.astype(np.float32).astype(np.float64)
    X = np.asarray(X, dtype=np.float64)
    f = np.zeros(X.shape[0])
    for c in range(0, nh, 256):
        ph = X @ kap[c:c + 256].T
        f += np.cos(ph) @ ab[c:c + 256, 0] + np.sin(ph) @ ab[c:c + 256, 1]
    return np.maximum(mean + std / math.sqrt(nh) * f, vmin)
