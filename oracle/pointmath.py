"""Independent numpy restatement of the per-point formulas of the MPM step.

TEST INFRASTRUCTURE ONLY (imported by tests/).  It shares no code with the
library: every function is written from the reference's Julia source, cited
per function, vectorised over arrays of inputs, with Julia's evaluation order
(left-to-right association, x^2 = x*x and x^3 = (x*x)*x as Base.literal_pow
gives them, no fused multiply-add; numpy rounds every elementwise operation on
its own).  tests/test_pointmath.py holds the library's scalar header
(csrc/ep_scalar.h, compiled on the host by oracle/scalar_probe.cpp) to it:
bit for bit where the Julia expression fixes every rounding, within a stated
tolerance where the reference calls LAPACK/BLAS or Base.log/exp (eigen,
matrix-vector products, the LU solve).

Reference files (paths within the ElastoPlasm.jl project):
  bsmpm.jl   src/home/program/workflow/shpfun/basis/bsmpm.jl
  gimpm.jl   src/home/program/workflow/shpfun/basis/gimpm.jl
  smpm.jl    src/home/program/workflow/shpfun/basis/smpm.jl
  DP.jl      src/home/program/workflow/elastoplast/plast/retmap/DP.jl
  J2.jl      src/home/program/workflow/elastoplast/plast/retmap/J2.jl
  MCRetMap   src/home/program/workflow/elastoplast/plast/retmap/MCRetMap.jl
  camC       src/home/program/workflow/elastoplast/plast/retmap/camC.zip: camC/camCmodRetMap.jl
  elast.jl   src/home/program/workflow/elastoplast/elast/elast.jl
  setup_cmpr src/home/program/utils/setup/setup_cmpr.jl
"""
from __future__ import annotations

import math

import numpy as np

F = np.float64


def _cube(x):
    return (x * x) * x


def _select(conds, vals):
    """Julia if / elseif / ... / end with a zero default: the first true condition wins."""
    out = np.zeros(np.broadcast(*conds).shape, dtype=F)
    done = np.zeros(out.shape, dtype=bool)
    for c, v in zip(conds, vals):
        take = c & ~done
        out = np.where(take, v, out)
        done |= c
    return out


# ---------------------------------------------------------------------------
# Cubic B-spline pieces t1..t4 (bsmpm.jl:1-62).  Each returns (phi, dphi/dxi).
# ---------------------------------------------------------------------------
def _pieces(x):
    x = np.asarray(x, dtype=F)
    x2, x3 = x * x, _cube(x)
    return x, x2, x3


def bs_t1(xi):
    """t1_ϕ∂ϕ (bsmpm.jl:1-17): the boundary-node piece."""
    x, x2, x3 = _pieces(xi)
    c = [(-2.0 <= x) & (x <= -1.0), (-1.0 <= x) & (x <= 0.0), (0.0 <= x) & (x <= 1.0), (1.0 <= x) & (x <= 2.0)]
    phi = _select(c, [(((1.0 / 6.0) * x3 + x2) + 2.0 * x) + 4.0 / 3.0,
                      ((-1.0 / 6.0) * x3 + x) + 1.0,
                      ((1.0 / 6.0) * x3 - x) + 1.0,
                      (((-1.0 / 6.0) * x3 + x2) - 2.0 * x) + 4.0 / 3.0])
    dphi = _select(c, [((3.0 / 6.0) * x2 + 2.0 * x) + 2.0,
                       (-3.0 / 6.0) * x2 + 1.0,
                       (3.0 / 6.0) * x2 - 1.0,
                       ((-3.0 / 6.0) * x2 + 2.0 * x) - 2.0])
    return phi, dphi


def bs_t2(xi):
    """t2_ϕ∂ϕ (bsmpm.jl:18-31): the node one cell inside the left boundary."""
    x, x2, x3 = _pieces(xi)
    c = [(-1.0 <= x) & (x <= 0.0), (0.0 <= x) & (x <= 1.0), (1.0 <= x) & (x <= 2.0)]
    phi = _select(c, [((-1.0 / 3.0) * x3 - x2) + 2.0 / 3.0,
                      ((1.0 / 2.0) * x3 - x2) + 2.0 / 3.0,
                      (((-1.0 / 6.0) * x3 + x2) - 2.0 * x) + 4.0 / 3.0])
    dphi = _select(c, [(-3.0 / 3.0) * x2 - 2.0 * x,
                       (3.0 / 2.0) * x2 - 2.0 * x,
                       ((-3.0 / 6.0) * x2 + 2.0 * x) - 2.0])
    return phi, dphi


def bs_t3(xi):
    """t3_ϕ∂ϕ (bsmpm.jl:32-47): an interior node."""
    x, x2, x3 = _pieces(xi)
    c = [(-2.0 <= x) & (x <= -1.0), (-1.0 <= x) & (x <= 0.0), (0.0 <= x) & (x <= 1.0), (1.0 <= x) & (x <= 2.0)]
    phi = _select(c, [(((1.0 / 6.0) * x3 + x2) + 2.0 * x) + 4.0 / 3.0,
                      ((-1.0 / 2.0) * x3 - x2) + 2.0 / 3.0,
                      ((1.0 / 2.0) * x3 - x2) + 2.0 / 3.0,
                      (((-1.0 / 6.0) * x3 + x2) - 2.0 * x) + 4.0 / 3.0])
    dphi = _select(c, [((3.0 / 6.0) * x2 + 2.0 * x) + 2.0,
                       (-3.0 / 2.0) * x2 - 2.0 * x,
                       (3.0 / 2.0) * x2 - 2.0 * x,
                       ((-3.0 / 6.0) * x2 + 2.0 * x) - 2.0])
    return phi, dphi


def bs_t4(xi):
    """t4_ϕ∂ϕ (bsmpm.jl:48-61): the node one cell inside the right boundary."""
    x, x2, x3 = _pieces(xi)
    c = [(-2.0 <= x) & (x <= -1.0), (-1.0 <= x) & (x <= 0.0), (0.0 <= x) & (x <= 1.0)]
    phi = _select(c, [(((1.0 / 6.0) * x3 + x2) + 2.0 * x) + 4.0 / 3.0,
                      ((-1.0 / 2.0) * x3 - x2) + 2.0 / 3.0,
                      ((1.0 / 3.0) * x3 - x2) + 2.0 / 3.0])
    dphi = _select(c, [((3.0 / 6.0) * x2 + 2.0 * x) + 2.0,
                       (-3.0 / 2.0) * x2 - 2.0 * x,
                       (3.0 / 3.0) * x2 - 2.0 * x])
    return phi, dphi


INVALID = -1


def bs_class(xn, xB0, xB1, dx):
    """The piece selection of ϕ∂ϕ (bsmpm.jl:63-76) by exact comparison of the node coordinate with
    the boundary table: 0 = t1, 1 = t2, 2 = t3, 3 = t4, INVALID = the reference's "Invalid position"."""
    xn = np.asarray(xn, dtype=F)
    c = [xn == xB0, xn == (xB0 + dx), ((xB0 + dx) < xn) & (xn < (xB1 - dx)), xn == (xB1 - dx), xn == xB1]
    out = np.full(xn.shape, INVALID, dtype=np.int64)
    done = np.zeros(xn.shape, dtype=bool)
    for c_, k in zip(c, (0, 1, 2, 3, 0)):
        out = np.where(c_ & ~done, k, out)
        done |= c_
    return out


def bspline(xi, xn, xB0, xB1, dx):
    """ϕ∂ϕ(ξ, xn, xB, Δx) (bsmpm.jl:63-78): value and derivative over Δx; NaN where the reference
    raises "Invalid position"."""
    cls = bs_class(xn, xB0, xB1, dx)
    parts = [bs_t1(xi), bs_t2(xi), bs_t3(xi), bs_t4(xi)]
    phi = np.full(cls.shape, np.nan)
    dphi = np.full(cls.shape, np.nan)
    for k in range(4):
        phi = np.where(cls == k, parts[k][0], phi)
        dphi = np.where(cls == k, parts[k][1], dphi)
    return phi, dphi / dx


# ---------------------------------------------------------------------------
# GIMP and linear bases.
# ---------------------------------------------------------------------------
def jl_sign(x):
    """Julia `sign` of a Float64: ±1, and ±0 / NaN unchanged."""
    x = np.asarray(x, dtype=F)
    return np.where(x > 0.0, 1.0, np.where(x < 0.0, -1.0, x))


def gimp(dx, h, lp):
    """S∂S(δx, h, lp) (gimpm.jl:1-14)."""
    dx = np.asarray(dx, dtype=F)
    a = np.abs(dx)
    c1 = a < lp
    c2 = (a >= lp) & (a <= (h - lp))
    c3 = (a >= (h - lp)) & (a < (h + lp))
    r = (h + lp) - a
    S = _select([c1, c2, c3], [1.0 - ((4.0 * (dx * dx) + (2.0 * lp) * (2.0 * lp)) / ((8.0 * h) * lp)),
                               1.0 - (a / h),
                               (r * r) / ((4.0 * h) * lp)])
    dS = _select([c1, c2, c3], [-((8.0 * dx) / ((8.0 * h) * lp)),
                                jl_sign(dx) * (-1.0 / h),
                                (-jl_sign(dx) * r) / ((2.0 * h) * lp)])
    return S, dS


def hat(dx, h):
    """N∂N(δx, h) (smpm.jl:1-10)."""
    dx = np.asarray(dx, dtype=F)
    c1 = (-h < dx) & (dx <= 0.0)
    c2 = (0.0 < dx) & (dx <= h)
    N = _select([c1, c2], [1.0 + dx / h, 1.0 - dx / h])
    dN = _select([c1, c2], [np.full(dx.shape, 1.0 / h), np.full(dx.shape, -1.0 / h)])
    return N, dN


def weights_2d(xp, xn, h, basis, xB=None, lp=None):
    """The 2d stencil weight of one (point, node) pair: bsmpm_2d (bsmpm.jl:95-113, ξ = (x_p - x_n)/h),
    gimpm_2d (gimpm.jl:31-47, δ = x_p - x_n with the point's ℓ) or smpm_2d (smpm.jl, δ = x_p - x_n).
    xp, xn: (2, n); returns (N, ∂N/∂x, ∂N/∂z)."""
    xp, xn = np.asarray(xp, dtype=F), np.asarray(xn, dtype=F)
    if basis == "bsmpm":
        fx, gx = bspline((xp[0] - xn[0]) / h[0], xn[0], xB[0][0], xB[0][1], h[0])
        fz, gz = bspline((xp[1] - xn[1]) / h[1], xn[1], xB[1][0], xB[1][1], h[1])
    elif basis == "gimpm":
        fx, gx = gimp(xp[0] - xn[0], h[0], lp[0])
        fz, gz = gimp(xp[1] - xn[1], h[1], lp[1])
    else:
        fx, gx = hat(xp[0] - xn[0], h[0])
        fz, gz = hat(xp[1] - xn[1], h[1])
    return fx * fz, gx * fz, fx * gz


# ---------------------------------------------------------------------------
# Elastic stiffness (setup_cmpr.jl:21-48).
# ---------------------------------------------------------------------------
def elastic_stiffness(E, nu, ndim):
    """(Kc, Gc, Del) of get_elastic_stiffness: Del = E/((1+ν)(1-2ν)) .* D."""
    Kc, Gc = E / (3.0 * (1.0 - 2.0 * nu)), E / (2.0 * (1.0 + nu))
    i, I = 1.0 - nu, (1.0 - 2.0 * nu) / 2.0
    if ndim == 2:
        D = np.array([[i, nu, 0.0], [nu, i, 0.0], [0.0, 0.0, I]])
    else:
        D = np.zeros((6, 6))
        D[:3, :3] = nu
        D[[0, 1, 2], [0, 1, 2]] = i
        D[[3, 4, 5], [3, 4, 5]] = I
    return Kc, Gc, (E / ((1.0 + nu) * (1.0 - 2.0 * nu))) * D


# ---------------------------------------------------------------------------
# Drucker-Prager (DP.jl:1-100), vectorised over points: s is (nstr, n).
# ---------------------------------------------------------------------------
def dp_trial(s):
    """σTr (DP.jl:1-12): P, τ0, τII."""
    s = np.asarray(s, dtype=F)
    if s.shape[0] == 3:
        P = (s[0] + s[1]) / 2.0
        t0 = np.stack([s[0] - P, s[1] - P, s[2] - 0.0])
        tII = np.sqrt(0.5 * (t0[0] * t0[0] + t0[1] * t0[1]) + t0[2] * t0[2])
    else:
        P = ((s[0] + s[1]) + s[2]) / 3.0
        t0 = np.stack([s[0] - P, s[1] - P, s[2] - P, s[3] - 0.0, s[4] - 0.0, s[5] - 0.0])
        tII = np.sqrt(((((0.5 * ((t0[0] * t0[0] + t0[1] * t0[1]) + t0[2] * t0[2]) + t0[3] * t0[3])
                         + t0[4] * t0[4]) + t0[5] * t0[5])))
    return P, t0, tII


def dp_material(tphi, sphi, cphi, c, nstr, tpsi=0.0, spsi=0.0):
    """materialParam (DP.jl:13-24) with tan/sin/cos of ϕ given (ψ = 0 in the reference, DP.jl:37)."""
    if nstr == 3:
        den = np.sqrt(9.0 + (12.0 * tphi) * tphi)
        eta = (3.0 * tphi) / den
        etaB = (3.0 * tpsi) / np.sqrt(9.0 + (12.0 * tpsi) * tpsi)
        xi = (3.0 * c) / den
    else:
        sq3 = np.sqrt(3.0)
        eta = (6.0 * sphi) / (sq3 * (3.0 + sphi))
        etaB = (6.0 * spsi) / (sq3 * (3.0 + spsi))
        xi = ((6.0 * c) * cphi) / (sq3 * (3.0 + sphi))
    return eta, etaB, xi


def dp_return(s, ep2, c0, cr, tphi, sphi, cphi, Hp, Kc, Gc, ep1):
    """The closed-form return of finite_DP / infinitesimal_DP (DP.jl:33-62, 69-98) on Voigt stresses
    s (nstr, n): returns (s', Δλ, ϵpII[1]')."""
    s = np.array(s, dtype=F)
    nstr = s.shape[0]
    D = 2 if nstr == 3 else 3
    c = c0 + Hp * ep2
    c = np.where(c < cr, cr, c)
    P, t0, tII = dp_trial(s)
    eta, etaB, xi = dp_material(tphi, sphi, cphi, c, nstr)
    sm, tP = xi / eta, xi - eta * (xi / eta)
    fs = (tII + eta * P) - xi
    sq = np.sqrt(1.0 + eta * eta)
    h = (tII - tP) - sq * (P - sm)
    shear = ((fs > 0.0) & (P < sm)) | ((h > 0.0) & (P >= sm))
    apex = (h <= 0.0) & (P >= sm)
    dlam = np.zeros_like(P)
    out = s.copy()
    ep1 = np.array(ep1, dtype=F)
    with np.errstate(divide="ignore", invalid="ignore"):
        dl = fs / (Gc + (Kc * eta) * etaB)
        Pn = P - (Kc * etaB) * dl
        tn = xi - eta * (P - (Kc * etaB) * dl)
        r = tn / tII
        for i in range(nstr):
            out[i] = np.where(shear, t0[i] * r + (Pn if i < D else 0.0), out[i])
        dlam = np.where(shear, dl, dlam)
        ep1 = np.where(shear, ep1 + dl * np.sqrt((1.0 / 3.0) + (2.0 / 9.0) * (etaB * etaB)), ep1)
        dl2 = (P - sm) / Kc
        Pn2 = sm - P
        r2 = 0.0 / tII
        for i in range(nstr):
            out[i] = np.where(apex, t0[i] * r2 + (Pn2 if i < D else 0.0), out[i])
        dlam = np.where(apex, dl2, dlam)
        ep1 = np.where(apex, ep1 + (np.sqrt(2.0) * dl2) / 3.0, ep1)
    return out, dlam, ep1


# ---------------------------------------------------------------------------
# Small matrix products as Julia forms them for 2x2 and 3x3 Float64 matrices (LinearAlgebra's
# gemm_wrapper! hands them to matmul2x2!/matmul3x3!: C[i,j] = A[i,1]B[1,j] + A[i,2]B[2,j] (+ A[i,3]B[3,j])
# left to right); batched over the leading axis.
# ---------------------------------------------------------------------------
def jl_matmul(A, B, ta=False, tb=False):
    A = np.swapaxes(A, -1, -2) if ta else A
    B = np.swapaxes(B, -1, -2) if tb else B
    D = A.shape[-1]
    C = np.empty(np.broadcast_shapes(A.shape, B.shape), dtype=F)
    for i in range(D):
        for j in range(D):
            acc = A[..., i, 0] * B[..., 0, j]
            for k in range(1, D):
                acc = acc + A[..., i, k] * B[..., k, j]
            C[..., i, j] = acc
    return C


def matvec(Del, v):
    """Del * v for a batch of Voigt vectors v (n, nstr); the reference's product goes through BLAS
    gemv, whose summation order is not fixed, so this is compared within a tolerance."""
    return np.einsum("ij,nj->ni", Del, v)


# ---------------------------------------------------------------------------
# J2 (J2.jl:1-76), restated with the intended fields (the reference's kernels do not run: they read
# mpts.cᵣ/mpts.c₀ instead of mpts.s.*, write ϵpII[p,1]); batched over points, s is (n, nstr).
# ---------------------------------------------------------------------------
def j2_yield(s, kappa):
    """get_J2 + yield_J2 (J2.jl:1-20): f = sqrt(2 J2) - κ and n = ξ/|ξ| (2d ignores σzz: P = (σxx+σyy)/2)."""
    s = np.asarray(s, dtype=F)
    if s.shape[-1] == 3:
        P = (s[:, 0] + s[:, 1]) / 2.0
        x = np.stack([s[:, 0] - P, s[:, 1] - P, s[:, 2] - 0.0], axis=1)
        J2 = 0.5 * ((x[:, 0] * x[:, 0] + x[:, 1] * x[:, 1]) + 2.0 * (x[:, 2] * x[:, 2]))
    else:
        P = ((s[:, 0] + s[:, 1]) + s[:, 2]) / 3.0
        x = np.stack([s[:, 0] - P, s[:, 1] - P, s[:, 2] - P, s[:, 3] - 0.0, s[:, 4] - 0.0, s[:, 5] - 0.0], axis=1)
        J2 = 0.5 * (((((x[:, 0] * x[:, 0] + x[:, 1] * x[:, 1]) + x[:, 2] * x[:, 2]) + 2.0 * (x[:, 3] * x[:, 3]))
                     + 2.0 * (x[:, 4] * x[:, 4])) + 2.0 * (x[:, 5] * x[:, 5]))
    xn = np.sqrt(2.0 * J2)
    return xn - kappa, x / xn[:, None]


def j2_return(s, ep2, c0, cr, Hp, Del, ftol=1e-9, itmax=20):
    """The cutting-plane loop of finite_J2 / infinitesimal_J2 (J2.jl:21-76): Δλ = f/(nᵀ Del n),
    σ -= Δλ Del n, γ += Δλ, κ = max(cr, c0 + Hp γ), while |f| > ftol and it < 20.
    Returns (σ', γ, yielded)."""
    sig = np.array(s, dtype=F)
    g = np.array(ep2, dtype=F)
    kappa = np.maximum(cr, c0 + Hp * g)
    f, n = j2_yield(sig, kappa)
    yielded = f > 0.0
    act = yielded.copy()
    it = 1
    while it < itmax:
        act &= np.abs(f) > ftol
        if not act.any():
            break
        den = np.einsum("ni,ij,nj->n", n, Del, n)
        dl = np.where(act, f / den, 0.0)
        sig = np.where(act[:, None], sig - dl[:, None] * matvec(Del, n), sig)
        g = np.where(act, g + dl, g)
        kappa = np.maximum(cr, c0 + Hp * g)
        f2, n2 = j2_yield(sig, kappa)
        f = np.where(act, f2, f)
        n = np.where(act[:, None], n2, n)
        it += 1
    return sig, g, yielded


# ---------------------------------------------------------------------------
# Mohr-Coulomb (MCRetMap.jl:1-54) and modified Cam-Clay (camC.zip: camC/camCmodRetMap.jl), restated
# with the Solid's fields (the reference's functions are commented out of plast.jl:14-15,28-29);
# batched over points, s is (n, nstr).  A point leaves the iteration when its own test fails.
# ---------------------------------------------------------------------------
def mc_return(s, ep2, c0, cr, sphi, cphi, Hp, Del, ftol=1e-6, itmax=10_000):
    r"""MCRetMap! on plane-strain Voigt stresses (n, 3): ψ = 0.5°, H = cos ϕ Hp, c = max(c0 + Hp ϵII, cr),
    f = τII + σm sin ϕ - c cos ϕ on the Mohr circle of (σxx, σyy, σxy); cutting plane
    Δγ = f / (H + ∂fᵀ Del ∂g), Δσ = Δγ Del ∂g, Δϵ += Del \ Δσ, ϵII = ϵII0 + sqrt(2/3 (Δϵ1² + Δϵ2² + 2Δϵ3²)).
    Returns (σ', ϵII, status) with status 1 yielded, 0 elastic, -1 over the iteration limit."""
    psi = 0.5 * math.pi / 180.0
    spsi = math.sin(psi)
    sig = np.array(s, dtype=F)
    e0 = np.asarray(ep2, dtype=F)
    sphi, cphi = np.asarray(sphi, dtype=F), np.asarray(cphi, dtype=F)
    H = cphi * Hp

    def circle(x):
        sm = 0.5 * (x[:, 0] + x[:, 1])
        return sm, np.sqrt(0.25 * (x[:, 0] - x[:, 1]) ** 2 + x[:, 2] ** 2)

    c = np.maximum(c0 + Hp * e0, cr)
    sm, tII = circle(sig)
    f = tII + sm * sphi - c * cphi
    yielded = f > 0.0
    act = yielded.copy()
    de = np.zeros_like(sig)
    g = e0.copy()
    status = yielded.astype(np.int32)
    it = 0
    while True:
        act &= np.abs(f) > ftol
        if not act.any():
            break
        it += 1
        a = (sig[:, 0] - sig[:, 1]) / (4.0 * tII)
        df = np.stack([a + sphi / 2.0, -a + sphi / 2.0, sig[:, 2] / tII], axis=1)
        dg = np.stack([a + spsi / 2.0, -a + spsi / 2.0, sig[:, 2] / tII], axis=1)
        den = np.einsum("ni,ij,nj->n", df, Del, dg)
        dgam = np.where(act, f / (H + den), 0.0)
        ds = dgam[:, None] * np.einsum("ij,nj->ni", Del, dg)
        de = de + np.linalg.solve(Del, ds.T).T
        g = np.where(act, e0 + np.sqrt((2.0 / 3.0) * (de[:, 0] ** 2 + de[:, 1] ** 2 + 2.0 * de[:, 2] ** 2)), g)
        c = np.maximum(c0 + Hp * g, cr)
        sig = np.where(act[:, None], sig - ds, sig)
        sm2, t2 = circle(sig)
        f = np.where(act, t2 + sm2 * sphi - c * cphi, f)
        sm, tII = np.where(act, sm2, sm), np.where(act, t2, tII)
        if it > itmax:
            status = np.where(act, -1, status)
            break
    return sig, g, status


def camc_return(s, ep2, epV, Kc, Del):
    """camCRetMap! of camCmodRetMap.jl with its constants (χ = 3/2, Pt = Kc/10, a0 = Pt + Kc/10, β = 1,
    M = 6 sin ϕcs / (3 - sin ϕcs) with ϕcs = 20°, ζ = 0, at most 19 iterations while |f| > 1e-6) and the
    yield function its derivative and envelope use, f = (P - Pt + a)²/b² + (q/M)² - a².
    P, q, n as camCParam (2d: P = (σxx+σyy)/2); ∂f/∂σ = ∂f/∂P/3 on the normal components + √χ ∂f/∂q n.
    Returns (σ', ϵpII, ϵpV, yielded)."""
    chi, Pt = 1.5, Kc / 10.0
    a0, beta = Pt + Kc / 10.0, 1.0
    phics = 20.0 * math.pi / 180.0
    M = 6.0 * math.sin(phics) / (3.0 - math.sin(phics))
    sig = np.array(s, dtype=F)
    nstr = sig.shape[1]
    nnorm = 2 if nstr == 3 else 3
    w2 = np.array([1.0, 1.0, 2.0] if nstr == 3 else [1.0, 1.0, 1.0, 2.0, 2.0, 2.0])

    def param(x):
        P = x[:, :nnorm].sum(axis=1) / nnorm
        xi = x.copy()
        xi[:, :nnorm] -= P[:, None]
        xn = np.sqrt(2.0 * (0.5 * (xi ** 2 * w2).sum(axis=1)))
        return P, np.sqrt(chi) * xn, xi / xn[:, None]

    def yield_(P, q, a):
        b = np.where(P < Pt - a, beta, 1.0)
        return (P - Pt + a) ** 2 / b ** 2 + (q / M) ** 2 - a ** 2, b

    ev = np.array(epV, dtype=F)
    g = np.array(ep2, dtype=F)
    a = a0 * np.exp(-0.0 * ev)
    P, q, n = param(sig)
    f, b = yield_(P, q, a)
    yielded = f > 0.0
    act = yielded.copy()
    for _ in range(19):
        act &= np.abs(f) > 1e-6
        if not act.any():
            break
        dfdp = (2.0 / b ** 2) * (P - Pt + a)
        dfdq = 2.0 * q / M ** 2
        df = np.sqrt(chi) * dfdq[:, None] * n
        df[:, :nnorm] += (dfdp / 3.0)[:, None]
        dl = np.where(act, f / np.einsum("ni,ij,nj->n", df, Del, df), 0.0)
        sig = np.where(act[:, None], sig - dl[:, None] * np.einsum("ij,nj->ni", Del, df), sig)
        ev = np.where(act, ev + dl * dfdp, ev)
        g = np.where(act, g + dl * dfdq, g)
        a = a0 * np.exp(-0.0 * ev)
        P2, q2, n2 = param(sig)
        f2, b2 = yield_(P2, q2, a)
        P, q, f, b = (np.where(act, u, v) for u, v in ((P2, P), (q2, q), (f2, f), (b2, b)))
        n = np.where(act[:, None], n2, n)
    return sig, np.where(yielded, g, ep2), np.where(yielded, ev, epV), yielded


# ---------------------------------------------------------------------------
# Elastic predictors (elast.jl:1-80), batched: tensors (n, D, D) row-major in the last two axes,
# Voigt vectors (n, nstr).
# ---------------------------------------------------------------------------
def voigt(T, chi):
    """mutate(ϵ, Χ, :voigt) (elast.jl:14-32): (xx, yy, Χ xy) / (xx, yy, zz, Χ yz, Χ xz, Χ xy)."""
    if T.shape[-1] == 2:
        return np.stack([T[:, 0, 0], T[:, 1, 1], chi * T[:, 0, 1]], axis=1)
    return np.stack([T[:, 0, 0], T[:, 1, 1], T[:, 2, 2], chi * T[:, 1, 2], chi * T[:, 0, 2], chi * T[:, 0, 1]],
                    axis=1)


def tensor(v, chi):
    """mutate(ϵ, Χ, :tensor) (elast.jl:14-32)."""
    n = v.shape[0]
    if v.shape[-1] == 3:
        T = np.empty((n, 2, 2))
        T[:, 0, 0], T[:, 1, 1] = v[:, 0], v[:, 1]
        T[:, 0, 1] = T[:, 1, 0] = chi * v[:, 2]
        return T
    T = np.empty((n, 3, 3))
    T[:, 0, 0], T[:, 1, 1], T[:, 2, 2] = v[:, 0], v[:, 1], v[:, 2]
    T[:, 0, 1] = T[:, 1, 0] = chi * v[:, 5]
    T[:, 0, 2] = T[:, 2, 0] = chi * v[:, 4]
    T[:, 1, 2] = T[:, 2, 1] = chi * v[:, 3]
    return T


def left_cauchy_green(dF, b):
    """b ← ΔF b ΔFᵀ of finite_elast (elast.jl:48): Julia's 3-argument product of equal square
    matrices is (ΔF b) ΔFᵀ."""
    return jl_matmul(jl_matmul(dF, b), dF, tb=True)


def finite_elast(dF, b, Del):
    """finite_elast (elast.jl:45-56): b ← ΔF b ΔFᵀ, ϵ = ½ n diag(log λ) nᵀ, τ = Del voigt(ϵ, 2).
    The eigen decomposition is numpy's (LAPACK) of the symmetric part."""
    bn = left_cauchy_green(dF, b)
    lam, V = np.linalg.eigh(0.5 * (bn + np.swapaxes(bn, 1, 2)))
    eps = 0.5 * np.einsum("nik,nk,njk->nij", V, np.log(lam), V)
    return bn, eps, matvec(Del, voigt(eps, 2.0))


def finite_rebuild_b(tau, Del):
    r"""After a finite-strain return (DP.jl:63-66, J2.jl:43-45): ϵ = tensor(Del \ τ, ½),
    b = n diag(exp 2λ) nᵀ."""
    eps = tensor(np.linalg.solve(Del, tau.T).T, 0.5)
    lam, V = np.linalg.eigh(eps)
    return eps, np.einsum("nik,nk,njk->nij", V, np.exp(2.0 * lam), V)


def infinitesimal_elast(dF, sig, Del):
    """infinitesimal_elast (elast.jl:69-80): ϵ = ½(ΔF + ΔFᵀ) - I, ω = ½(ΔF - ΔFᵀ),
    σJ = σω' + σ'ω, σ += Del voigt(ϵ, 2) .+ voigt(σJ, 1).  Returns (σ', ϵ, ω, σJ, Del voigt(ϵ, 2))."""
    D = dF.shape[-1]
    dFt = np.swapaxes(dF, 1, 2)
    eps = 0.5 * (dF + dFt) - np.eye(D)
    w = 0.5 * (dF - dFt)
    S = tensor(np.asarray(sig, dtype=F), 1.0)
    sJ = jl_matmul(S, w, tb=True) + jl_matmul(S, w, ta=True)
    de = matvec(Del, voigt(eps, 2.0))
    return sig + (de + voigt(sJ, 1.0)), eps, w, sJ, de
