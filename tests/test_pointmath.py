"""The library's per-point arithmetic (csrc/ep_scalar.h, which the FP64 device step and the C++
oracle both compile) against an independent numpy restatement written from the reference's Julia
source (oracle/pointmath.py, which shares no code with the library).

Every function is checked on >= 10^4 random inputs per case plus the branch boundaries the Julia
code tests (the B-spline piece limits and the exact node-class comparisons, the GIMP support
edges, the Drucker-Prager shear / apex / elastic branches).  Where the Julia expression fixes
every rounding (shape functions, the DP return, the infinitesimal strain and spin) the two must
agree bit for bit, so a changed constant, branch or operation order in ep_scalar.h fails here.
Where the reference calls LAPACK/BLAS or Base.log/exp (eigen, Del * v, Del \\ τ) the tolerance is
written beside the assertion.  No GPU: the header is compiled for the host (oracle/scalar_probe.cpp).
"""
import ctypes as C
import math

import numpy as np
import pytest

N = 20_000
D_ = C.POINTER(C.c_double)
I_ = C.POINTER(C.c_int32)


I64, I32, DBL = C.c_int64, C.c_int32, C.c_double
SIGS = {
    "probe_bspline": [I64, D_, D_, DBL, DBL, DBL, D_, D_, I_],
    "probe_gimp": [I64, D_, DBL, D_, D_, D_],
    "probe_hat": [I64, D_, DBL, D_, D_],
    "probe_dp": [I64, I32, D_, D_, D_, D_, D_, D_, D_, DBL, DBL, DBL, D_, D_],
    "probe_j2": [I64, I32, D_, D_, D_, D_, DBL, D_, D_, I_],
    "probe_mc": [I64, D_, D_, D_, D_, D_, D_, DBL, D_, D_, I_],
    "probe_camc": [I64, I32, D_, D_, D_, DBL, D_, D_, I_],
    "probe_finite_elast": [I64, I32, D_, D_, D_, D_, D_],
    "probe_finite_rebuild_b": [I64, I32, D_, D_, D_, D_],
    "probe_infinitesimal_elast": [I64, I32, D_, D_, D_, D_, D_, D_],
    "probe_exp_log": [I64, D_, D_, D_],
    "probe_eig": [I64, I32, D_, D_, D_],
    "probe_det": [I64, I32, D_, D_],
}


@pytest.fixture(scope="module")
def probe(oracle_mod):
    oracle_mod.build()
    lib = C.CDLL(oracle_mod.PROBE)
    for name, args in SIGS.items():
        getattr(lib, name).argtypes = args
        getattr(lib, name).restype = None
    return lib


@pytest.fixture(scope="module")
def pm():
    import pointmath
    return pointmath


def _p(a):
    return a.ctypes.data_as(D_ if a.dtype == np.float64 else I_)


def _bits_equal(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return np.array_equal(a.view(np.int64), b.view(np.int64))


def _slump_axis(nel=640, L=64.1584):
    """The x axis of the scaled-up slump mesh as the library's set-up builds it (Julia range rule)."""
    from epgpu import ic_slump
    ic, _ = ic_slump([L, L / 4.0], [nel, nel // 4], ni=2)
    m = ic["mesh"]
    return np.unique(m.x[0]), float(m.xB[0, 0]), float(m.xB[0, 1]), float(m.h[0])


def _near(vals, rng, n):
    """n inputs concentrated on and around the given branch limits (exact, ±1..4 ulp)."""
    v = rng.choice(np.asarray(vals, dtype=np.float64), size=n)
    k = rng.integers(-4, 5, size=n)
    out = v.copy()
    for s in range(1, 5):
        out = np.where(k >= s, np.nextafter(out, np.inf), out)
        out = np.where(k <= -s, np.nextafter(out, -np.inf), out)
    return out


def test_bspline_pieces_and_classes(probe, pm):
    rng = np.random.default_rng(1)
    xn_axis, xB0, xB1, h = _slump_axis()
    assert xn_axis.size > 600
    # node coordinates: every mesh node, plus coordinates an ulp off the class boundaries (INVALID
    # or a different class), and random points; ξ across all pieces and on the piece limits
    xn = np.concatenate([rng.choice(xn_axis, N), rng.choice([xB0, xB0 + h, xB1 - h, xB1], N // 2),
                         _near([xB0, xB0 + h, xB1 - h, xB1], rng, N // 4), rng.uniform(xB0 - h, xB1 + h, N // 4)])
    xi = np.concatenate([rng.uniform(-2.5, 2.5, xn.size - N), _near([-2.0, -1.0, 0.0, 1.0, 2.0], rng, N)])
    rng.shuffle(xi)
    f = np.zeros_like(xi)
    df = np.zeros_like(xi)
    cls = np.zeros(xi.size, dtype=np.int32)
    probe.probe_bspline(xi.size, _p(xi), _p(xn), xB0, xB1, h, _p(f), _p(df), _p(cls))
    cref = pm.bs_class(xn, xB0, xB1, h)
    assert np.array_equal(np.where(cls == 4, -1, cls), cref)
    for k in range(4):
        assert (cref == k).sum() > 1000, k                     # every piece family exercised
    assert (cref == pm.INVALID).sum() > 100
    ok = cref != pm.INVALID
    fr, dfr = pm.bspline(xi, xn, xB0, xB1, h)
    assert _bits_equal(f[ok], fr[ok]) and _bits_equal(df[ok], dfr[ok])
    # partition of unity over a node's stencil (shpTest.jl:93-113) with the restatement itself
    xp = rng.uniform(xB0, xB1, 2000)
    e = np.clip(np.floor((xp - xB0) / h), 0, xn_axis.size - 2).astype(int)
    tot = np.zeros_like(xp)
    for o in (-1, 0, 1, 2):
        j = np.clip(e + o, 0, xn_axis.size - 1)
        valid = (e + o >= 0) & (e + o < xn_axis.size)
        w, _ = pm.bspline((xp - xn_axis[j]) / h, xn_axis[j], xB0, xB1, h)
        tot += np.where(valid, w, 0.0)
    assert np.abs(tot - 1.0).max() < 1e-13


@pytest.mark.parametrize("h", [1.6039600000000001, 0.1002475])
def test_gimp(probe, pm, h):
    rng = np.random.default_rng(2)
    lp = np.concatenate([np.full(N // 2, h / 4.0), rng.uniform(0.05 * h, 0.5 * h, N // 2)])
    edges = np.stack([lp, h - lp, h + lp, np.zeros_like(lp)])
    dx = np.where(rng.random(N) < 0.5, rng.uniform(-1.6 * h, 1.6 * h, N),
                  edges[rng.integers(0, 4, N), np.arange(N)] * rng.choice([-1.0, 1.0], N))
    dx = np.where(rng.random(N) < 0.3, np.nextafter(dx, rng.choice([-np.inf, np.inf], N)), dx)
    f = np.zeros(N)
    df = np.zeros(N)
    probe.probe_gimp(N, _p(dx), h, _p(lp), _p(f), _p(df))
    fr, dfr = pm.gimp(dx, h, lp)
    assert _bits_equal(f, fr) and _bits_equal(df, dfr)
    a = np.abs(dx)
    for region in (a < lp, (a >= lp) & (a <= h - lp), (a >= h - lp) & (a < h + lp), a >= h + lp):
        assert region.sum() > 500


def test_linear_hat(probe, pm):
    rng = np.random.default_rng(3)
    h = 1.6039600000000001
    dx = np.concatenate([rng.uniform(-1.5 * h, 1.5 * h, N), _near([-h, 0.0, h], rng, N // 4)])
    f = np.zeros_like(dx)
    df = np.zeros_like(dx)
    probe.probe_hat(dx.size, _p(dx), h, _p(f), _p(df))
    fr, dfr = pm.hat(dx, h)
    assert _bits_equal(f, fr) and _bits_equal(df, dfr)


def _dp_inputs(rng, nstr, n):
    """Trial stresses around the cone: elastic, shear-return and apex-return points."""
    c0 = rng.uniform(1e3, 5e4, n)
    cr = np.full(n, 4e3)
    ep2 = np.where(rng.random(n) < 0.5, 0.0, rng.uniform(0.0, 2.0, n))
    phi = np.radians(rng.uniform(5.0, 45.0, n))
    scale = rng.uniform(1e3, 2e5, n)
    s = rng.normal(size=(n, nstr)) * scale[:, None]
    # shift some trials far to the tension side (apex branch) and some far to compression
    shift = np.where(rng.random(n) < 0.25, rng.uniform(1e4, 3e5, n), 0.0) - np.where(
        rng.random(n) < 0.25, rng.uniform(1e4, 3e5, n), 0.0)
    D = 2 if nstr == 3 else 3
    s[:, :D] += shift[:, None]
    return s, ep2, c0, cr, np.tan(phi), np.sin(phi), np.cos(phi)


@pytest.mark.parametrize("nstr", [3, 6])
def test_drucker_prager_return(probe, pm, nstr):
    rng = np.random.default_rng(4 + nstr)
    E, nu = 1.0e6, 0.3
    Kc, Gc, _ = pm.elastic_stiffness(E, nu, 2 if nstr == 3 else 3)
    Hp = -3.0e4
    s, ep2, c0, cr, tp, sp, cp = _dp_inputs(rng, nstr, N)
    ep1 = rng.uniform(0.0, 1.0, N)
    out = np.ascontiguousarray(s.copy())
    e1 = ep1.copy()
    dl = np.zeros(N)
    probe.probe_dp(N, nstr, _p(out), _p(ep2), _p(c0), _p(cr), _p(tp), _p(sp), _p(cp), Hp, Kc, Gc, _p(e1), _p(dl))
    ref, dref, e1ref = pm.dp_return(s.T, ep2, c0, cr, tp, sp, cp, Hp, Kc, Gc, ep1)
    assert _bits_equal(out, ref.T) and _bits_equal(dl, dref) and _bits_equal(e1, e1ref)
    # branch coverage: elastic, shear return, apex (tension) return
    P, _, tII = pm.dp_trial(s.T)
    c = np.maximum(c0 + Hp * ep2, cr)
    eta, _, xi = pm.dp_material(tp, sp, cp, c, nstr)
    apex = (P >= xi / eta) & ((tII - (xi - eta * (xi / eta))) - np.sqrt(1.0 + eta * eta) * (P - xi / eta) <= 0.0)
    assert (dl == 0).sum() > 1000 and ((dl > 0) & ~apex).sum() > 1000 and apex.sum() > 1000


@pytest.mark.parametrize("nstr", [3, 6])
def test_j2_return(probe, pm, nstr):
    rng = np.random.default_rng(10 + nstr)
    n = 5000
    D = 2 if nstr == 3 else 3
    _, _, Del = pm.elastic_stiffness(1.0e7, 0.3, D)
    s = rng.normal(size=(n, nstr)) * rng.uniform(5e3, 1.2e5, n)[:, None]
    c0 = np.full(n, 5.0e4)
    cr = np.full(n, 4.0e3)
    ep2 = rng.uniform(0.0, 0.1, n)
    out = np.ascontiguousarray(s.copy())
    e1 = ep2.copy()
    y = np.zeros(n, dtype=np.int32)
    DelF = np.asfortranarray(Del).ravel(order="F").copy()
    probe.probe_j2(n, nstr, _p(out), _p(ep2), _p(c0), _p(cr), 1.0e5, _p(DelF), _p(e1), _p(y))
    ref, g, yl = pm.j2_return(s, ep2, c0, cr, 1.0e5, Del)
    assert np.array_equal(y.astype(bool), yl) and yl.sum() > 1000 and (~yl).sum() > 500
    # elastic points untouched, bit for bit; returned ones within 1e-12 of the stress scale (the
    # reference's n'Del n and Del n go through BLAS, whose summation order is not fixed)
    assert _bits_equal(out[~yl], s[~yl])
    scale = np.abs(s).max(axis=1)
    assert (np.abs(out - ref).max(axis=1) / scale).max() < 1e-12
    assert (np.abs(e1 - np.where(yl, g, ep2)) / np.maximum(np.abs(g), 1e-300)).max() < 1e-10


def test_mc_return(probe, pm):
    """MCRetMap.jl restated: elastic points untouched bit for bit, returned ones on the Mohr-Coulomb
    surface (|f| <= 1e-6 Pa, the reference's ftol) and within 1e-10 of the numpy restatement (Del ∂g and
    Del \\ Δσ go through BLAS/LAPACK in the reference)."""
    rng = np.random.default_rng(31)
    n = 4000
    _, _, Del = pm.elastic_stiffness(1.0e6, 0.3, 2)
    P = rng.uniform(-3e5, 2e4, n)
    R = rng.uniform(0.0, 1.2e5, n)
    th = rng.uniform(0.0, 2 * np.pi, n)
    s = np.stack([P + R * np.cos(th), P - R * np.cos(th), R * np.sin(th)], axis=1)
    phi = np.radians(rng.choice([20.0, 7.5, 30.0], n))
    sphi, cphi = np.sin(phi), np.cos(phi)
    c0 = rng.uniform(1e3, 4e4, n)
    cr = np.full(n, 4.0e3)
    ep2 = rng.uniform(0.0, 0.2, n)
    out = np.ascontiguousarray(s.copy())
    e1 = np.zeros(n)
    st = np.zeros(n, dtype=np.int32)
    DelF = np.asfortranarray(Del).ravel(order="F").copy()
    probe.probe_mc(n, _p(out), _p(ep2), _p(c0), _p(cr), _p(sphi), _p(cphi), -3.0e4, _p(DelF), _p(e1), _p(st))
    ref, g, sref = pm.mc_return(s, ep2, c0, cr, sphi, cphi, -3.0e4, Del)
    assert np.array_equal(st, sref) and (st == 1).sum() > 1000 and (st == 0).sum() > 500
    y = st == 1
    assert _bits_equal(out[~y], s[~y])
    scale = np.abs(s).max(axis=1)
    assert (np.abs(out - ref).max(axis=1) / scale)[y].max() < 1e-10
    assert (np.abs(e1 - g)[y] / np.maximum(np.abs(g[y]), 1e-300)).max() < 1e-9
    c = np.maximum(c0 + -3.0e4 * e1, cr)
    sm = 0.5 * (out[:, 0] + out[:, 1])
    f = np.sqrt(0.25 * (out[:, 0] - out[:, 1]) ** 2 + out[:, 2] ** 2) + sm * sphi - c * cphi
    assert np.abs(f[y]).max() <= 1e-6


@pytest.mark.parametrize("nstr", [3, 6])
def test_camc_return(probe, pm, nstr):
    """camCmodRetMap.jl restated: 19 cutting-plane steps on yielded points (|f| in Pa² stays above
    1e-6), elastic points untouched bit for bit, returned stress, ϵpII and ϵpV within 1e-9 of the numpy
    restatement, and the yield function reduced by orders of magnitude."""
    rng = np.random.default_rng(40 + nstr)
    n = 4000
    D = 2 if nstr == 3 else 3
    K, _, Del = pm.elastic_stiffness(1.0e6, 0.3, D)
    nn = 2 if nstr == 3 else 3
    s = rng.normal(size=(n, nstr)) * rng.uniform(1e4, 1.5e5, n)[:, None]
    s[:, :nn] += rng.uniform(-3.5e5, 1.2e5, n)[:, None]
    ep2 = rng.uniform(0.0, 0.1, n)
    epv = rng.uniform(-0.01, 0.01, n)
    out = np.ascontiguousarray(s.copy())
    ev = epv.copy()
    e1 = ep2.copy()
    st = np.zeros(n, dtype=np.int32)
    DelF = np.asfortranarray(Del).ravel(order="F").copy()
    probe.probe_camc(n, nstr, _p(out), _p(ep2), _p(ev), K, _p(DelF), _p(e1), _p(st))
    ref, g, evr, yl = pm.camc_return(s, ep2, epv, K, Del)
    assert np.array_equal(st.astype(bool), yl) and yl.sum() > 1000 and (~yl).sum() > 500
    assert _bits_equal(out[~yl], s[~yl]) and _bits_equal(ev[~yl], epv[~yl]) and _bits_equal(e1[~yl], ep2[~yl])
    scale = np.abs(s).max(axis=1)
    assert (np.abs(out - ref).max(axis=1) / scale).max() < 1e-9
    assert np.abs(e1 - g).max() < 1e-9 * max(np.abs(g).max(), 1.0)
    assert np.abs(ev - evr).max() < 1e-9 * max(np.abs(evr).max(), 1.0)


@pytest.mark.parametrize("D", [2, 3])
def test_finite_elastic_predictor(probe, pm, D):
    rng = np.random.default_rng(20 + D)
    n = N
    NS = 3 if D == 2 else 6
    _, _, Del = pm.elastic_stiffness(1.0e6, 0.3, D)
    dF = np.eye(D) + rng.normal(scale=1e-2, size=(n, D, D))
    A = np.eye(D) + rng.normal(scale=5e-2, size=(n, D, D))
    b = A @ np.swapaxes(A, 1, 2)                           # a symmetric positive b_e
    colmaj = lambda T: np.ascontiguousarray(np.swapaxes(T, 1, 2)).reshape(n, -1)   # noqa: E731
    bb = colmaj(b).copy()
    eps = np.zeros((n, D * D))
    tau = np.zeros((n, NS))
    DelF = Del.ravel(order="F").copy()
    probe.probe_finite_elast(n, D, _p(colmaj(dF).copy()), _p(bb), _p(DelF), _p(eps), _p(tau))
    bn, er, tr = pm.finite_elast(dF, b, Del)
    # b = (ΔF b) ΔFᵀ in matmul2x2!/matmul3x3! order: bit for bit
    assert _bits_equal(bb, colmaj(bn))
    # ϵ = ½ log b through the eigen decomposition (LAPACK in the reference, Jacobi here) and Base.log
    # (the library's own log): 1e-13 of |ϵ|; τ = Del voigt(ϵ, 2) within 1e-12 of |τ|
    assert (np.abs(eps - colmaj(er)).max(axis=1) / np.abs(er).reshape(n, -1).max(axis=1)).max() < 1e-12
    assert (np.abs(tau - tr).max(axis=1) / np.abs(tr).max(axis=1)).max() < 1e-11


@pytest.mark.parametrize("D", [2, 3])
def test_finite_rebuild_of_b(probe, pm, D):
    rng = np.random.default_rng(30 + D)
    n = N
    NS = 3 if D == 2 else 6
    _, _, Del = pm.elastic_stiffness(1.0e6, 0.3, D)
    tau = rng.normal(scale=2e4, size=(n, NS))
    eps = np.zeros((n, D * D))
    b = np.zeros((n, D * D))
    probe.probe_finite_rebuild_b(n, D, _p(tau), _p(Del.ravel(order="F").copy()), _p(eps), _p(b))
    er, br = pm.finite_rebuild_b(tau, Del)
    colmaj = lambda T: np.ascontiguousarray(np.swapaxes(T, 1, 2)).reshape(n, -1)   # noqa: E731
    assert (np.abs(eps - colmaj(er)).max(axis=1) / np.abs(er).reshape(n, -1).max(axis=1)).max() < 1e-13
    assert np.abs(b - colmaj(br)).max() < 1e-14 * np.abs(br).max()


@pytest.mark.parametrize("D", [2, 3])
def test_infinitesimal_elastic_predictor(probe, pm, D):
    rng = np.random.default_rng(40 + D)
    n = N
    NS = 3 if D == 2 else 6
    _, _, Del = pm.elastic_stiffness(1.0e7, 0.3, D)
    dF = np.eye(D) + rng.normal(scale=1e-3, size=(n, D, D))
    sig = rng.normal(scale=5e4, size=(n, NS))
    colmaj = lambda T: np.ascontiguousarray(np.swapaxes(T, 1, 2)).reshape(n, -1)   # noqa: E731
    s = sig.copy()
    eps, w, sJ = np.zeros((n, D * D)), np.zeros((n, D * D)), np.zeros((n, D * D))
    probe.probe_infinitesimal_elast(n, D, _p(colmaj(dF).copy()), _p(s), _p(Del.ravel(order="F").copy()),
                                    _p(eps), _p(w), _p(sJ))
    sr, er, wr, sjr, der = pm.infinitesimal_elast(dF, sig, Del)
    # strain, spin and the (identically zero) "Jaumann" term: bit for bit
    assert _bits_equal(eps, colmaj(er)) and _bits_equal(w, colmaj(wr)) and _bits_equal(sJ, colmaj(sjr))
    assert np.abs(sjr).max() == 0.0
    # σ + Del voigt(ϵ, 2): Del * v goes through BLAS in the reference; 2 ulp of the increment's scale
    assert (np.abs(s - sr).max(axis=1) <= 4.5e-16 * (np.abs(sig).max(axis=1) + np.abs(der).max(axis=1))).all()


def test_elastic_stiffness_matches_the_setup(pm):
    from epgpu.ic import get_elastic_stiffness
    for E, nu in ((1.0e6, 0.3), (1.0e7, 0.3), (2.5e7, 0.25)):
        for d in (2, 3):
            K, G, Del = get_elastic_stiffness(E, nu, d)
            Kr, Gr, Dr = pm.elastic_stiffness(E, nu, d)
            assert K == Kr and G == Gr and _bits_equal(np.asarray(Del).reshape(Dr.shape), Dr)


def test_exp_log_eigen_det_against_numpy(probe):
    """The library's own exp/log (Cody-Waite + Taylor, atanh series), Jacobi eigen decomposition and
    LU determinant against numpy (libm and LAPACK): exp/log within 2 ulp, eigen pairs reconstruct the
    matrix to 1e-14 of its norm, det within 1e-14 of the product scale."""
    rng = np.random.default_rng(50)
    x = np.concatenate([rng.uniform(-700.0, 700.0, N), rng.uniform(-1e-3, 1e-3, N),
                        np.exp(rng.uniform(-700, 700, N))])
    ex, lx = np.zeros_like(x), np.zeros_like(x)
    probe.probe_exp_log(x.size, _p(x), _p(ex), _p(lx))
    ulp = lambda v: np.spacing(np.abs(v))                  # noqa: E731
    m = np.abs(x) <= 700.0
    assert (np.abs(ex[m] - np.exp(x[m])) <= 2 * ulp(np.exp(x[m]))).all()
    pos = x > 0
    assert (np.abs(lx[pos] - np.log(x[pos])) <= 2 * ulp(np.log(x[pos])) + 1e-300).all()
    for D in (2, 3):
        A = rng.normal(size=(N, D, D))
        A = A + np.swapaxes(A, 1, 2)
        Ac = np.ascontiguousarray(np.swapaxes(A, 1, 2)).reshape(N, -1)
        lam, V = np.zeros((N, D)), np.zeros((N, D * D))
        probe.probe_eig(N, D, _p(Ac), _p(lam), _p(V))
        Vm = np.swapaxes(V.reshape(N, D, D), 1, 2)
        R = np.einsum("nik,nk,njk->nij", Vm, lam, Vm)
        nrm = np.abs(A).max(axis=(1, 2))
        assert (np.abs(R - A).max(axis=(1, 2)) / nrm).max() < 1e-14
        assert (np.abs(np.sort(lam, axis=1) - np.linalg.eigvalsh(A)).max(axis=1) / nrm).max() < 1e-14
        det = np.zeros(N)
        probe.probe_det(N, D, _p(Ac), _p(det))
        scale = np.abs(A).max(axis=(1, 2)) ** D
        assert (np.abs(det - np.linalg.det(A)) / scale).max() < 1e-14
        assert math.isfinite(det.sum())
