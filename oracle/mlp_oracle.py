"""CPU restatement of the learned return map: labels, features and the MLP.

TEST INFRASTRUCTURE ONLY: imported by tests/ (and by bench.py, which states
the error of the learned step) as the checker of the tensor-core network
kernels and of the exact labels.  The product never imports it.

Three parts:

* ``label`` -- the reference's finite-strain Drucker-Prager return
  (src/constitutive/plast/DP.jl:33-62, psi = 0 at :37; stress invariants as
  DP.jl:1-12, material parameters of the 2d branch as DP.jl:13-18) applied in
  the principal frame of the trial log strain, everything scaled by the
  cohesion c (strains by s = c / (2G), stresses by c, so c = 1 below).  The
  plane-strain stiffness is setup_cmpr.jl:21-48 with lambda / (2G) = l2g.  Rows
  with x[7] = 1 use the 3d branch instead (outer cone, DP.jl:19-21 and 69-98, on
  the three principal stresses; sin and cos of phi from tan phi), their target
  expressed in the trial's frame (frame3).
  Output: the plastic correction per unit overstress phi_n = f_s / c,
  y = (returned strains / s - trial strains / s) / phi_n.
* ``features`` -- the feature rows the step builds from a trial log strain.
* ``forward`` / ``backward`` -- the 6 -> 128 x 4 (SiLU) -> 3 network with the
  BF16 roundings of the GPU kernels emulated (inputs, weights, hidden
  activations and back-propagated errors are rounded to BF16 before each
  product; sums are carried in FP64 here and in FP32 on the GPU), or in plain
  FP64 (``bf16=False``) for finite-difference checks.
"""
from __future__ import annotations

import numpy as np

NX, NY, NIN, NOUT, WIDTH = 8, 4, 6, 3, 128
CREF = 2.0e4
PHI_MIN = 1.0e-6
LAYOUT = [("W1", (WIDTH, NIN)), ("b1", (WIDTH,)), ("W2", (WIDTH, WIDTH)), ("b2", (WIDTH,)),
          ("W3", (WIDTH, WIDTH)), ("b3", (WIDTH,)), ("W4", (WIDTH, WIDTH)), ("b4", (WIDTH,)),
          ("W5", (NOUT, WIDTH)), ("b5", (NOUT,))]
NPARAM = sum(int(np.prod(s)) for _, s in LAYOUT)


# ---------------------------------------------------------------------------
# labels and features
def _dp_params(tphi):
    den = np.sqrt(9.0 + 12.0 * tphi * tphi)
    return 3.0 * tphi / den, 3.0 / den          # eta, xi with c = 1 (DP.jl:14-17)


def trial_stress(e1, e2, l2g):
    """Scaled plane-strain stress (xx, yy) / c of scaled principal strains."""
    tr = e1 + e2
    return l2g * tr + e1, l2g * tr + e2


def overstress(t1, t2, tphi):
    """f_s / c of a scaled principal stress (DP.jl:40-46)."""
    P = 0.5 * (t1 + t2)
    tII = np.sqrt(0.5 * ((t1 - P) ** 2 + (t2 - P) ** 2))
    eta, xi = _dp_params(tphi)
    return tII + eta * P - xi


def dp_return_scaled(t1, t2, tphi):
    """Returned scaled principal stress and a yield flag (DP.jl:47-62, c = 1, psi = 0)."""
    t1 = np.asarray(t1, dtype=np.float64)
    t2 = np.asarray(t2, dtype=np.float64)
    P = 0.5 * (t1 + t2)
    d1, d2 = t1 - P, t2 - P
    tII = np.sqrt(0.5 * (d1 * d1 + d2 * d2))
    eta, xi = _dp_params(tphi)
    sm = xi / eta
    tP = xi - eta * sm
    fs = tII + eta * P - xi
    hh = tII - tP - np.sqrt(1.0 + eta * eta) * (P - sm)
    shear = ((fs > 0) & (P < sm)) | ((hh > 0) & (P >= sm))
    apex = (hh <= 0) & (P >= sm)
    with np.errstate(divide="ignore", invalid="ignore"):
        r = np.where(shear, (xi - eta * P) / tII, 1.0)
    o1 = np.where(shear, d1 * r + P, t1)
    o2 = np.where(shear, d2 * r + P, t2)
    # the tension-apex branch sets the mean stress to sm - P and the deviator to 0 (DP.jl:53-58)
    o1 = np.where(apex, sm - P, o1)
    o2 = np.where(apex, sm - P, o2)
    dl = np.where(apex, P - sm, np.where(shear, fs, 0.0))
    return o1, o2, (shear | apex) & (dl != 0)


def strain_of_stress(t1, t2, l2g):
    tr = (t1 + t2) / (1.0 + 2.0 * l2g)
    return t1 - l2g * tr, t2 - l2g * tr


# 3d (outer cone, DP.jl:19-21): rows with x[:, 7] = 1
SQ3 = np.sqrt(3.0)


def _dp_params3(tphi):
    r = 1.0 / np.sqrt(1.0 + tphi * tphi)
    sphi, cphi = tphi * r, r
    return 6.0 * sphi / (SQ3 * (3.0 + sphi)), 6.0 * cphi / (SQ3 * (3.0 + sphi))   # eta, xi with c = 1


def trial_stress3(e, l2g):
    """Scaled principal stress (n x 3) of scaled principal strains (n x 3)."""
    e = np.asarray(e, dtype=np.float64)
    return l2g * e.sum(axis=1, keepdims=True) + e


def strain_of_stress3(t, l2g):
    t = np.asarray(t, dtype=np.float64)
    tr = t.sum(axis=1, keepdims=True) / (1.0 + 3.0 * l2g)
    return t - l2g * tr


def _inv3(t):
    P = t.mean(axis=1)
    d = t - P[:, None]
    return P, d, np.sqrt(0.5 * (d * d).sum(axis=1))


def overstress3(t, tphi):
    P, _, tII = _inv3(np.asarray(t, dtype=np.float64))
    eta, xi = _dp_params3(tphi)
    return tII + eta * P - xi


def dp_return_scaled3(t, tphi):
    """Returned scaled principal stress (n x 3) and a yield flag (DP.jl:69-98, c = 1, psi = 0)."""
    t = np.asarray(t, dtype=np.float64)
    P, d, tII = _inv3(t)
    eta, xi = _dp_params3(tphi)
    sm = xi / eta
    tP = xi - eta * sm
    fs = tII + eta * P - xi
    hh = tII - tP - np.sqrt(1.0 + eta * eta) * (P - sm)
    shear = ((fs > 0) & (P < sm)) | ((hh > 0) & (P >= sm))
    apex = (hh <= 0) & (P >= sm)
    with np.errstate(divide="ignore", invalid="ignore"):
        r = np.where(shear, (xi - eta * P) / tII, 1.0)
    o = np.where(shear[:, None], d * r[:, None] + P[:, None], t)
    o = np.where(apex[:, None], (sm - P)[:, None] * np.ones((1, 3)), o)
    dl = np.where(apex, P - sm, np.where(shear, fs, 0.0))
    return o, (shear | apex) & (dl != 0)


def frame3(e):
    """The 3d output frame of trial rows (ep_rmap.h rm_frame3): e_m, the unit trial deviator q
    ((1,-1,0)/sqrt2 when hydrostatic) and r = e_m x q, each n x 3."""
    e = np.asarray(e, dtype=np.float64)
    d = e - e.mean(axis=1, keepdims=True)
    n = np.sqrt((d * d).sum(axis=1, keepdims=True))
    with np.errstate(divide="ignore", invalid="ignore"):
        q = np.where(n > 0, d / n, np.array([[np.sqrt(0.5), -np.sqrt(0.5), 0.0]]))
    em = np.full_like(q, np.sqrt(1.0 / 3.0))
    return em, q, np.cross(em, q)


def _label3(x, l2g):
    e = x[:, 0:3].astype(np.float64)
    tphi = x[:, 4].astype(np.float64)
    t = trial_stress3(e, l2g)
    phin = overstress3(t, tphi)
    o, yl = dp_return_scaled3(t, tphi)
    r = strain_of_stress3(o, l2g)
    ok = yl & (phin > PHI_MIN)
    y = np.zeros((x.shape[0], NY), dtype=np.float32)
    with np.errstate(divide="ignore", invalid="ignore"):
        c = np.where(ok[:, None], (r - e) / phin[:, None], 0.0)
    em, q, rr = frame3(e)
    y[:, 0] = (c * em).sum(axis=1)
    y[:, 1] = (c * q).sum(axis=1)
    y[:, 2] = (c * rr).sum(axis=1)
    return y, ok


def label(x, l2g):
    """Exact labels of feature rows (n x 8, float32) -> (n x 4 float32, plastic mask)."""
    x = np.asarray(x)
    d3 = x[:, 7] > 0.5
    if d3.any():
        y = np.zeros((x.shape[0], NY), dtype=np.float32)
        ok = np.zeros(x.shape[0], dtype=bool)
        y[d3], ok[d3] = _label3(x[d3], l2g)
        if (~d3).any():
            y[~d3], ok[~d3] = label(x[~d3], l2g)
        return y, ok
    e1 = x[:, 0].astype(np.float64)
    e2 = x[:, 1].astype(np.float64)
    tphi = x[:, 4].astype(np.float64)
    t1, t2 = trial_stress(e1, e2, l2g)
    phin = overstress(t1, t2, tphi)
    o1, o2, yl = dp_return_scaled(t1, t2, tphi)
    r1, r2 = strain_of_stress(o1, o2, l2g)
    ok = yl & (phin > PHI_MIN)
    y = np.zeros((x.shape[0], NY), dtype=np.float32)
    with np.errstate(divide="ignore", invalid="ignore"):
        y[:, 0] = np.where(ok, (r1 - e1) / phin, 0.0)
        y[:, 1] = np.where(ok, (r2 - e2) / phin, 0.0)
    return y, ok


def accept3(x, y, l2g, tol=1e-3):
    """accept() for 3d rows: returns the mask and the returned scaled principal stresses (n x 3)."""
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)[:, 0:3].copy()
    e, tphi, phin = x[:, 0:3], x[:, 4], x[:, 6]
    dev = (x[:, 5] == 0.0)[:, None]
    # the correction from the trial's frame; psi = 0 keeps the component along q (radial return)
    em, q, rr = frame3(e)
    y = np.where(dev, 0.0, y[:, 0:1]) * em + y[:, 1:2] * q + np.where(dev, 0.0, y[:, 2:3]) * rr
    r = e + phin[:, None] * y
    t = trial_stress3(r, l2g)
    P, _, tII = _inv3(t)
    eta, xi = _dp_params3(tphi)
    fs = tII + eta * P - xi
    Ptr = (l2g + 1.0 / 3.0) * e.sum(axis=1)
    _, _, tIItr = _inv3(e)
    dl = tIItr - tII
    with np.errstate(divide="ignore"):
        below = np.where(tphi > 0, Ptr < 1.0 / np.where(tphi > 0, tphi, 1.0), True)
    ok = ((phin >= PHI_MIN) & (np.abs(fs) <= tol) & (np.abs(P - Ptr) <= tol) & (dl >= 0)
          & (r[:, 0] >= r[:, 1]) & (r[:, 1] >= r[:, 2]) & below & np.isfinite(fs))
    return ok, t


def accept(x, y, l2g, tol=1e-3):
    """The step's acceptance of network outputs, restated (km_rmap_finish): returns the mask
    of accepted rows and their returned scaled principal stresses."""
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    e1, e2, tphi, phin = x[:, 0], x[:, 1], x[:, 4], x[:, 6]
    y0, y1 = y[:, 0].copy(), y[:, 1].copy()
    dev = x[:, 5] == 0.0
    yd = 0.5 * (y0 - y1)
    y0 = np.where(dev, yd, y0)
    y1 = np.where(dev, -yd, y1)
    r1, r2 = e1 + phin * y0, e2 + phin * y1
    t1, t2 = trial_stress(r1, r2, l2g)
    P = 0.5 * (t1 + t2)
    tII = 0.5 * np.abs(t1 - t2)
    eta, xi = _dp_params(tphi)
    fs = tII + eta * P - xi
    Ptr = (l2g + 0.5) * (e1 + e2)
    dl = 0.5 * (e1 - e2) - tII
    with np.errstate(divide="ignore"):
        below = np.where(tphi > 0, Ptr < 1.0 / np.where(tphi > 0, tphi, 1.0), True)
    ok = ((phin >= PHI_MIN) & (np.abs(fs) <= tol) & (np.abs(P - Ptr) <= tol) & (dl >= 0) & (r1 >= r2)
          & below & np.isfinite(fs))
    return ok, t1, t2


def features(e11, e22, e12, coh, tphi, G, l2g):
    """Feature rows of trial log strains (tensor components), FP64."""
    em, ed = 0.5 * (e11 + e22), 0.5 * (e11 - e22)
    r = np.sqrt(ed * ed + e12 * e12)
    s = coh / (2.0 * G)
    x = np.zeros((np.size(e11), NX), dtype=np.float64)
    x[:, 0] = (em + r) / s
    x[:, 1] = (em - r) / s
    x[:, 3] = coh / CREF
    x[:, 4] = tphi
    t1, t2 = trial_stress(x[:, 0], x[:, 1], l2g)
    x[:, 6] = np.maximum(overstress(t1, t2, tphi), 0.0)
    return x


def features3(eps, coh, tphi, G, l2g):
    """3d feature rows of trial log strains (n x 3 x 3 tensors), FP64; principal strains descending."""
    lam = np.linalg.eigvalsh(np.asarray(eps, dtype=np.float64))[:, ::-1]
    s = np.asarray(coh, dtype=np.float64) / (2.0 * G)
    x = np.zeros((lam.shape[0], NX), dtype=np.float64)
    x[:, 0:3] = lam / np.reshape(s, (-1, 1))
    x[:, 3] = coh / CREF
    x[:, 4] = tphi
    x[:, 6] = np.maximum(overstress3(trial_stress3(x[:, 0:3], l2g), tphi), 0.0)
    x[:, 7] = 1.0
    return x


def sample_trials3(n, l2g, seed=0, tphi=(np.tan(np.radians(15.0)), np.tan(np.radians(35.0))), spread=0.5):
    """3d synthetic plastic trial rows: a random overstress beyond the outer cone at a random
    Lode angle (deviator d_k = 2 tII / sqrt(3) cos(theta - 2 pi k / 3), J2 = tII^2)."""
    rng = np.random.default_rng(seed)
    tp = rng.uniform(tphi[0], tphi[1], n)
    eta, xi = _dp_params3(tp)
    P = -rng.uniform(0.0, 20.0, n) * xi
    fs = rng.uniform(0.0, spread, n)
    tII = np.maximum(xi - eta * P + fs, 1e-3)
    th = rng.uniform(0.0, 2.0 * np.pi, n)
    k = np.arange(3)[None, :]
    t = P[:, None] + (2.0 / SQ3) * tII[:, None] * np.cos(th[:, None] - 2.0 * np.pi * k / 3.0)
    t = -np.sort(-t, axis=1)
    x = np.zeros((n, NX), dtype=np.float32)
    x[:, 0:3] = strain_of_stress3(t, l2g)
    x[:, 3] = rng.uniform(0.05, 2.0, n)
    x[:, 4] = tp
    x[:, 6] = np.maximum(overstress3(trial_stress3(x[:, 0:3].astype(np.float64), l2g), tp), 0.0)
    x[:, 7] = 1.0
    return x


def sample_trials(n, l2g, seed=0, tphi=(np.tan(np.radians(15.0)), np.tan(np.radians(35.0))), spread=0.5, dim=2):
    """Synthetic plastic trial rows: trial stresses a random overstress beyond the DP surface."""
    if dim == 3:
        return sample_trials3(n, l2g, seed, tphi, spread)
    rng = np.random.default_rng(seed)
    tp = rng.uniform(tphi[0], tphi[1], n)
    eta, xi = _dp_params(tp)
    P = -rng.uniform(0.0, 20.0, n) * xi                      # compressive mean stress (scaled)
    fs = rng.uniform(0.0, spread, n)                         # overstress f_s / c
    tII = np.maximum(xi - eta * P + fs, 1e-3)
    t1, t2 = P + tII, P - tII
    tr = (t1 + t2) / (1.0 + 2.0 * l2g)
    x = np.zeros((n, NX), dtype=np.float32)
    x[:, 0] = t1 - l2g * tr
    x[:, 1] = t2 - l2g * tr
    x[:, 3] = rng.uniform(0.05, 2.0, n)
    x[:, 4] = tp
    t1r, t2r = trial_stress(x[:, 0].astype(np.float64), x[:, 1].astype(np.float64), l2g)
    x[:, 6] = np.maximum(overstress(t1r, t2r, x[:, 4].astype(np.float64)), 0.0)
    return x


# ---------------------------------------------------------------------------
# the network
def bf16(a):
    """Round float32 values to bfloat16 (round to nearest even), returned as float32."""
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32)


def unpack(p):
    p = np.asarray(p).reshape(-1)
    if p.dtype != np.float64:
        p = p.astype(np.float32)
    out, o = {}, 0
    for name, shape in LAYOUT:
        n = int(np.prod(shape))
        out[name] = p[o:o + n].reshape(shape)
        o += n
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], dtype=np.float32).reshape(-1) for name, _ in LAYOUT])


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(p, x, bf=True):
    """y (n x 3) and the cache for backward; bf emulates the kernels' BF16 operands."""
    P = unpack(p)
    q = bf16 if bf else (lambda a: np.asarray(a, dtype=np.float64))
    f = (lambda a: np.asarray(a, dtype=np.float32)) if bf else (lambda a: a)
    H = [q(np.asarray(x, dtype=np.float32)[:, :NIN])]
    Z = []
    for l in range(1, 5):
        z = f(H[-1].astype(np.float64) @ q(P[f"W{l}"]).astype(np.float64).T + P[f"b{l}"])
        Z.append(z)
        H.append(q(silu(z.astype(np.float64))))
    y = f(H[-1].astype(np.float64) @ q(P["W5"]).astype(np.float64).T + P["b5"])
    return y, (H, Z)


def loss_and_grad(p, x, t, bf=True):
    """MSE over the 3 outputs and its gradient (the GPU's forward/backward, restated)."""
    P = unpack(p)
    q = bf16 if bf else (lambda a: np.asarray(a, dtype=np.float64))
    f = (lambda a: np.asarray(a, dtype=np.float32)) if bf else (lambda a: a)
    y, (H, Z) = forward(p, x, bf)
    n = y.shape[0]
    e = y.astype(np.float64) - np.asarray(t, dtype=np.float64)[:, :NOUT]
    loss = float((e * e).sum() / (3.0 * n))
    dZ = f(2.0 * e / (3.0 * n))
    g = {}
    for l in range(5, 0, -1):
        g[f"W{l}"] = q(dZ).astype(np.float64).T @ H[l - 1].astype(np.float64)
        g[f"b{l}"] = dZ.astype(np.float64).sum(axis=0)
        if l == 1:
            break
        dH = q(dZ).astype(np.float64) @ q(P[f"W{l}"]).astype(np.float64)
        dZ = f(dH * dsilu(Z[l - 2].astype(np.float64)))
    return loss, pack({k: np.asarray(v, dtype=np.float64) for k, v in g.items()}).astype(np.float64)


def init_params(seed=0):
    rng = np.random.default_rng(seed)
    d = {}
    for name, shape in LAYOUT:
        if name.startswith("W"):
            fan_in = shape[1]
            gain = 1.0 if name == "W5" else 2.0
            d[name] = rng.normal(0.0, np.sqrt(gain / fan_in), shape)
        else:
            d[name] = np.zeros(shape)
    return pack(d)
