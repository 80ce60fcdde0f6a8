"""Initial conditions of the slump and collapse problems (host side).

This is the set-up half of ``ic_slump(L, nel; kwargs...)``
(script/example/slump.jl:22-49) and ``ic_collapse`` (script/example/collapse.jl:25-57):
the structured mesh (utils/setup/setup_mesh.jl:26-99), the material constants
(utils/setup/setup_cmpr.jl:120-143), the material-point cloud
(utils/setup/mpts/get_slump.jl:18-95, mpts_populate.jl:26-56, setup_mpts.jl:26-163)
and the time windows (utils/setup/setup_time.jl:21-30).

Every array keeps the reference's Julia layout: column-major, so ``x`` is a
``dim x nmp`` matrix stored particle by particle (``order='F'`` here).  Node
ids, element ids and stencils are 1-based ``Int64`` with 0 meaning "no node",
as in the reference.  The arithmetic order of every expression follows the
Julia source so that the resulting coordinates are bit-identical to the
reference's (no fused multiply-adds; ranges via :mod:`epgpu.julia`).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from .config import kwargser
from .julia import frange


def _F(a, dtype=np.float64):
    return np.asfortranarray(np.asarray(a, dtype=dtype))


# ----------------------------------------------------------------------------- mesh
def get_geom(nel, L, instr):
    """Cell size and stencil width (utils/setup/geom/get_geom.jl:21-30)."""
    L = [float(v) for v in L]
    nel = [int(v) for v in nel]
    ndim = len(L)
    if instr["basis"]["which"] == "bsmpm":
        h = [min(L[i] / nel[i], L[i] / 4.0) for i in range(ndim)]
    else:
        h = [L[i] / nel[i] for i in range(ndim)]
    return {"ndim": ndim, "nn": 4 ** ndim, "h": h, "nel": nel, "L": L}


def get_coords(ndim, L, h, ghosts):
    """Node coordinates and counts (utils/setup/mesh/get_coords.jl:22-55).

    Returns ``(x, nel, nno, axes)`` where ``axes[d]`` is the 1-D coordinate
    vector of direction ``d`` (x, [y,] z) and ``x`` the ``dim x nno`` matrix.
    """
    if ndim == 2:
        x = frange(0.0 - ghosts[0], h[0], L[0] + ghosts[0])
        z = frange(0.0 - ghosts[1], h[1], L[1] + ghosts[1])
        nno = [len(x), len(z), len(x) * len(z)]
        nel = [nno[0] - 1, nno[1] - 1, (nno[0] - 1) * (nno[1] - 1)]
        X = np.empty((2, nno[2]), order="F")
        # node id = j + nno_z * i (0-based), z fastest
        X[0, :] = np.repeat(np.asarray(x), len(z))
        X[1, :] = np.tile(np.asarray(z), len(x))
        return X, nel, nno, [np.asarray(x), np.asarray(z)]
    if ndim == 3:
        x = frange(0.0 - ghosts[0], h[0], L[0] + ghosts[0])
        y = frange(0.0 - ghosts[1], h[1], L[1] + ghosts[1])
        z = frange(0.0 - ghosts[2], h[2], (L[2] + 2.0 * h[2]) + ghosts[2])
        nx, ny, nz = len(x), len(y), len(z)
        nno = [nx, ny, nz, nx * ny * nz]
        nel = [nx - 1, ny - 1, nz - 1, (nx - 1) * (ny - 1) * (nz - 1)]
        X = np.empty((3, nno[3]), order="F")
        # node id = jz + nz*ix + nz*nx*ky (0-based)
        X[0, :] = np.tile(np.repeat(np.asarray(x), nz), ny)
        X[1, :] = np.repeat(np.asarray(y), nx * nz)
        X[2, :] = np.tile(np.asarray(z), nx * ny)
        return X, nel, nno, [np.asarray(x), np.asarray(y), np.asarray(z)]
    raise ValueError("only 2d and 3d meshes are built")


def get_bc(xn, instr, ghosts):
    """Roller/fixed Dirichlet masks and boundary coordinates (utils/setup/mesh/get_bc.jl:43-57).

    Membership uses exact ``==`` on the node coordinates, as the reference does.
    """
    ndim, nno = xn.shape
    xB = np.empty((ndim, 2), order="F")
    for d in range(ndim):
        xB[d, 0] = xn[d, :].min() + ghosts[d]
        xB[d, 1] = xn[d, :].max() - ghosts[d]
    bc = np.zeros((ndim, nno), dtype=np.bool_, order="F")
    dirichlet = instr["bcs"]["dirichlet"]
    for d in range(ndim):
        for k in range(2):
            ids = xn[d, :] == xB[d, k]
            kind = dirichlet[d][k]
            if kind == "roller":
                bc[d, ids] = True
            elif kind == "fixed":
                bc[:, ids] = True
    return bc, xB


def e2n(ndim, nno, nel, nn):
    """Element-to-node stencil (utils/setup/mesh/e2n.jl:20-78), 1-based, 0 = none."""
    if ndim == 2:
        nx, nz = nno[0], nno[1]
        ex, ez = nel[0], nel[1]
        i0 = np.repeat(np.arange(1, ex + 1), ez)          # element x index (outer)
        j0 = np.tile(np.arange(1, ez + 1), ex)            # element z index (inner)
        out = np.zeros((nn, nel[-1]), dtype=np.int64, order="F")
        s = 0
        for i in range(-1, 3):
            for j in range(-1, 3):
                jj, ii = j0 + j, i0 + i
                ok = (jj >= 1) & (jj <= nz) & (ii >= 1) & (ii <= nx)
                out[s, :] = np.where(ok, jj + nz * (ii - 1), 0)
                s += 1
        return out
    if ndim == 3:
        nx, ny, nz = nno[0], nno[1], nno[2]
        ex, ey, ez = nel[0], nel[1], nel[2]
        k0 = np.repeat(np.arange(1, ey + 1), ex * ez)
        i0 = np.tile(np.repeat(np.arange(1, ex + 1), ez), ey)
        j0 = np.tile(np.arange(1, ez + 1), ex * ey)
        out = np.zeros((nn, nel[-1]), dtype=np.int64, order="F")
        s = 0
        for k in range(-1, 3):
            for i in range(-1, 3):
                for j in range(-1, 3):
                    jj, ii, kk = j0 + j, i0 + i, k0 + k
                    ok = ((jj >= 1) & (jj <= nz) & (ii >= 1) & (ii <= nx)
                          & (kk >= 1) & (kk <= ny))
                    out[s, :] = np.where(ok, jj + nz * (ii - 1) + nz * nx * (kk - 1), 0)
                    s += 1
        return out
    raise ValueError("only 2d and 3d meshes are built")


@dataclass
class Mesh:
    """Mirror of ``Mesh`` (boot/needs/types.jl:141-168); nodal arrays are column-major."""
    dim: int
    nel: list
    nno: list
    nn: int
    L: np.ndarray
    h: np.ndarray
    x0: np.ndarray
    x: np.ndarray            # dim x nno
    xB: np.ndarray           # dim x 2
    bcs: np.ndarray          # dim x nno Bool
    e2n: np.ndarray          # nn x nel (1-based)
    axes: list               # per-direction node coordinates (x, [y,] z)
    nnel: list               # nonlocal neighbourhood half-width per direction (e2e.jl:24)
    mi: np.ndarray = None
    oobf: np.ndarray = None
    a: np.ndarray = None
    p: np.ndarray = None
    v: np.ndarray = None
    dJ: np.ndarray = None

    @property
    def nnodes(self) -> int:
        return int(self.nno[-1])

    @property
    def ncells(self) -> int:
        return int(self.nel[-1])


def setup_mesh(instr, geom) -> Mesh:
    """Mesh constructor (utils/setup/setup_mesh.jl:26-99), without the unused dense Mᵢⱼ.

    The reference allocates a dense ``nno x nno`` consistent mass matrix that no
    kernel reads (setup_mesh.jl:52); it is 85 GB at nel=[640,160] and is left out.
    """
    buffer = 2.0 if instr["basis"]["ghost"] else 0.0
    ndim = geom["ndim"]
    L, nn, h = geom["L"], geom["nn"], geom["h"]
    ghosts = [buffer * hh for hh in h]
    xn, nel, nno, axes = get_coords(ndim, L, h, ghosts)
    status, xB = get_bc(xn, instr, ghosts)
    ls = float(instr["nonloc"]["ls"])
    nnel = [int(math.ceil(ls / hh)) for hh in h]
    N = nno[-1]
    return Mesh(
        dim=ndim, nel=nel, nno=nno, nn=nn, L=np.asarray(L, dtype=np.float64),
        h=np.asarray(h, dtype=np.float64), x0=xn.min(axis=1).copy(), x=xn, xB=xB,
        bcs=status, e2n=e2n(ndim, nno, nel, nn), axes=axes, nnel=nnel,
        mi=np.zeros(N), oobf=np.zeros((ndim, N), order="F"), a=np.zeros((ndim, N), order="F"),
        p=np.zeros((ndim, N), order="F"), v=np.zeros((ndim, N), order="F"),
        dJ=np.zeros((ndim, N), order="F"),
    )


# ----------------------------------------------------------------------------- material
def get_elastic_stiffness(E, nu, ndim):
    """Bulk/shear moduli and Voigt stiffness (utils/setup/setup_cmpr.jl:21-48)."""
    Kc, Gc = E / (3.0 * (1.0 - 2.0 * nu)), E / (2.0 * (1.0 + nu))
    i, I = 1.0 - nu, (1.0 - 2.0 * nu) / 2.0
    if ndim == 2:
        D = np.array([[i, nu, 0.0], [nu, i, 0.0], [0.0, 0.0, I]])
    elif ndim == 3:
        D = np.array([[i, nu, nu, 0, 0, 0], [nu, i, nu, 0, 0, 0], [nu, nu, i, 0, 0, 0],
                      [0, 0, 0, I, 0, 0], [0, 0, 0, 0, I, 0], [0, 0, 0, 0, 0, I]], dtype=np.float64)
    else:
        raise ValueError("only 2d and 3d")
    fac = E / ((1.0 + nu) * (1.0 - 2.0 * nu))
    return Kc, Gc, np.asfortranarray(fac * D)


def setup_cmpr(mesh, E=1.0e6, nu=0.3, rho0=2700.0, **over):
    """Constitutive constants (utils/setup/setup_cmpr.jl:120-143).

    Keyword overrides (``c0``, ``cr``, ``phi0``, ``phir``, ``Hp``) stand in for the
    configs whose material differs from the slump defaults.
    """
    K, G, Del = get_elastic_stiffness(E, nu, mesh.dim)
    c = math.sqrt((K + 4.0 / 3.0 * G) / rho0)
    cmpr = {
        "E": float(E), "nu": float(nu), "Kc": K, "Gc": G, "Del": Del,
        "Hp": -30.0e3, "c0": 20.0e3, "cr": 4.0e3,
        "phi0": 20.0 * math.pi / 180, "phir": 7.5 * math.pi / 180,
        "rho0": float(rho0), "c": c,
    }
    cmpr.update(over)
    return cmpr


# ----------------------------------------------------------------------------- points
def mpts_populate(mesh, cmpr, instr, ni=2, grf_fn=None):
    """Regular lattice of points, ``ni`` per cell and direction (mpts_populate.jl:26-56)."""
    h, xB = mesh.h, mesh.xB
    ax = []
    for d in range(mesh.dim):
        ax.append(np.asarray(frange(xB[d, 0] + (0.5 * h[d] / ni), h[d] / ni, xB[d, 1])))
    if mesh.dim == 2:
        x, z = ax
        X = np.empty((len(x) * len(z), 2))
        X[:, 0] = np.repeat(x, len(z))            # vec(xp), z fastest
        X[:, 1] = np.tile(z, len(x))
    else:
        x, y, z = ax
        X = np.empty((len(x) * len(y) * len(z), 3))
        X[:, 0] = np.tile(np.repeat(x, len(z)), len(y))
        X[:, 1] = np.repeat(y, len(x) * len(z))
        X[:, 2] = np.tile(z, len(x) * len(y))
    if instr["grf"]["status"]:
        if grf_fn is None:
            from .grf import cohesion_field
            grf_fn = cohesion_field
        c0 = grf_fn(X, cmpr, instr, mesh)
    else:
        c0 = np.ones(X.shape[0]) * cmpr["c0"]
    return {"ni": ni, "x": X, "c0": c0}


def get_slump(mesh, cmpr, instr, ni=2, lz=12.80, grf_fn=None):
    """Slump geometry filter (utils/setup/mpts/get_slump.jl:18-95).

    Only the last of the 200 line points decides (the loop overwrites ``pos``),
    and ``shuffle`` is dropped because its result is unused (get_slump.jl:88).
    """
    out = mpts_populate(mesh, cmpr, instr, ni=ni, grf_fn=grf_fn)
    wl = 0.15 * lz
    X, c0 = out["x"], out["c0"]
    keep = X[:, -1] <= lz - (0.5 * mesh.h[-1] / ni)
    X, c = X[keep], c0[keep]
    xp, zp = X[:, 0], X[:, -1]
    a = -1.25
    xmax = xp.max()
    # LinRange(min, max, 200)[end] == max exactly; x_line = x + 0.5 L1, z_line = a x
    x_last = xmax + 0.5 * mesh.L[0]
    z_last = a * xmax
    dx, dz = xp - x_last, zp - z_last
    s = dx * a + dz * (-1.0)
    pos = (s > 0.0) | (zp < wl)
    X, c = X[pos], c[pos]
    nmp = X.shape[0]
    xpF = np.asfortranarray(X.T)
    coh0 = c.copy()
    cohr = np.ones(nmp) * cmpr["cr"]
    phi = np.ones(nmp) * cmpr["phi0"]
    phi[xpF[-1, :] <= 2 * wl] = cmpr["phir"]
    return {"xp": xpF, "coh0": coh0, "cohr": cohr, "phi": phi, "ni": ni, "nmp": nmp}


@dataclass
class Point:
    """Mirror of ``Point``/``Solid`` (boot/needs/types.jl:38-105), column-major."""
    ndim: int
    nmp: int
    vmax: np.ndarray
    x: np.ndarray
    z0: np.ndarray
    l0: np.ndarray
    l: np.ndarray
    n0: np.ndarray
    n: np.ndarray
    Omega0: np.ndarray
    Omega: np.ndarray
    dJ: np.ndarray
    J: np.ndarray
    # solid phase
    u: np.ndarray
    v: np.ndarray
    p: np.ndarray
    rho0: np.ndarray
    rho: np.ndarray
    c0: np.ndarray
    cr: np.ndarray
    phi: np.ndarray
    dlam: np.ndarray
    epII: np.ndarray         # 2 x nmp
    epV: np.ndarray
    sig: np.ndarray          # nstr x nmp
    tau: np.ndarray
    dvij: np.ndarray         # dim x dim x nmp
    duij: np.ndarray
    dFij: np.ndarray
    Fij: np.ndarray
    bij: np.ndarray
    eij: np.ndarray
    wij: np.ndarray
    sJij: np.ndarray
    p2e: np.ndarray = field(default=None)
    p2n: np.ndarray = field(default=None)
    Bij: np.ndarray = field(default=None)    # dim x dim x nmp, APIC (types.jl:82)
    Dij: np.ndarray = field(default=None)    # dim x dim x nmp, APIC (types.jl:83)

    @property
    def nstr(self) -> int:
        return 3 if self.ndim == 2 else 6

    def copy(self) -> "Point":
        kw = {}
        for k, v in self.__dict__.items():
            kw[k] = v.copy(order="K") if isinstance(v, np.ndarray) else v
        return Point(**kw)


def setup_mpts(mesh, cmpr, geom) -> Point:
    """Material-point state at rest (utils/setup/setup_mpts.jl:26-163)."""
    dim = mesh.dim
    nstr = 3 if dim == 2 else 6
    ni, nmp, xp = geom["ni"], geom["nmp"], geom["xp"]
    n0 = 0.1 * np.ones(nmp)
    l0 = np.empty((dim, nmp), order="F")
    for d in range(dim):
        l0[d, :] = (1.0 * 0.5) * (mesh.h[d] / ni)
    v0 = np.ones(nmp)
    two_l0 = 2 * l0
    v0 = two_l0[0, :].copy()
    for d in range(1, dim):
        v0 = v0 * two_l0[d, :]
    rho0 = np.full(nmp, cmpr["rho0"])
    eye = np.zeros((dim, dim, nmp), order="F")
    for d in range(dim):
        eye[d, d, :] = 1.0
    Z = lambda *s: np.zeros(s, order="F")
    return Point(
        ndim=dim, nmp=nmp, vmax=np.zeros(dim), x=_F(xp), z0=xp[-1, :].copy(),
        l0=l0.copy(order="F"), l=l0.copy(order="F"), n0=n0.copy(), n=n0.copy(),
        Omega0=v0.copy(), Omega=v0.copy(), dJ=np.ones(nmp), J=np.ones(nmp),
        u=Z(dim, nmp), v=Z(dim, nmp), p=Z(dim, nmp), rho0=rho0.copy(), rho=rho0.copy(),
        c0=np.asarray(geom["coh0"], dtype=np.float64).copy(),
        cr=np.asarray(geom["cohr"], dtype=np.float64).copy(),
        phi=np.asarray(geom["phi"], dtype=np.float64).copy(),
        dlam=np.zeros(nmp), epII=Z(2, nmp), epV=np.zeros(nmp),
        sig=Z(nstr, nmp), tau=Z(nstr, nmp),
        dvij=Z(dim, dim, nmp), duij=Z(dim, dim, nmp), dFij=Z(dim, dim, nmp),
        Fij=eye.copy(order="F"), bij=eye.copy(order="F"), eij=Z(dim, dim, nmp),
        wij=Z(dim, dim, nmp), sJij=Z(dim, dim, nmp),
        p2e=np.zeros(nmp, dtype=np.int64), p2n=np.zeros((mesh.nn, nmp), dtype=np.int64, order="F"),
        Bij=Z(dim, dim, nmp), Dij=Z(dim, dim, nmp),
    )


def setup_time(instr, te=0.0, tg=0.0, tep=0.0):
    """Time windows (utils/setup/setup_time.jl:21-30)."""
    return {"t": np.array([0.0, te + tep]), "te": float(te),
            "tg": float(te) if tg > te else float(tg), "tep": float(tep)}


# ----------------------------------------------------------------------------- entry points
def ic_slump(L, nel, ni=2, cmpr_over=None, grf_fn=None, **kwargs):
    """``ic_slump(L, nel; kwargs...)`` (script/example/slump.jl:22-49).

    Returns ``(ic, cfg)`` like the reference: ``ic`` holds ``mesh``, ``mpts``,
    ``cmpr`` and ``time``; ``cfg`` holds ``instr``.  ``ni`` (points per cell and
    direction) is the reference's ``get_slump`` default 2 (configs at 3 pass it
    here).  Plotting and output folders are left out.
    """
    instr = kwargser(kwargs, dim=len(L))
    geom = get_geom(nel, L, instr)
    mesh = setup_mesh(instr, geom)
    cmpr = setup_cmpr(mesh, **(cmpr_over or {}))
    mpts = setup_mpts(mesh, cmpr, get_slump(mesh, cmpr, instr, ni=ni, grf_fn=grf_fn))
    time = setup_time(instr, te=10.0, tg=10.0, tep=5.0)
    ic = {"mesh": mesh, "mpts": mpts, "cmpr": cmpr, "time": time}
    cfg = {"instr": instr, "misc": {"file": f"{mesh.dim}d_{instr['fwrk']['trsfr']}"}}
    return ic, cfg


def get_collapse(mesh, cmpr, ni, l0):
    """Elastic column geometry (utils/setup/mpts/get_collapse.jl:17-48), 2d."""
    h, xB = mesh.h, mesh.xB
    x = np.asarray(frange(xB[0, 0] + (0.5 * h[0] / ni), h[0] / ni, xB[0, 1]))
    z = np.asarray(frange(xB[1, 0] + (0.5 * h[1] / ni), h[1] / ni, l0))
    xp = np.empty((2, len(x) * len(z)), order="F")
    xp[0, :] = np.repeat(x, len(z))
    xp[1, :] = np.tile(z, len(x))
    nmp = xp.shape[1]
    return {"xp": xp, "coh0": np.ones(nmp) * cmpr["c0"], "cohr": np.ones(nmp) * cmpr["cr"],
            "phi": np.ones(nmp) * cmpr["phi0"], "ni": ni, "nmp": nmp}


def ic_collapse(nel, nu, E, rho0, l0, **kwargs):
    """``ic_collapse(nel, ν, E, ρ0, l0; kwargs...)`` (script/example/collapse.jl:25-57), 2d."""
    if len(nel) != 2:
        raise ValueError("the reference builds the collapse in 2d only (get_collapse.jl:25-34)")
    instr = kwargser(kwargs, dim=2)
    L = [10.0, 1.25 * l0]
    h = [L[-1] / nel[-1], L[-1] / nel[-1]]
    nel = [5, int(nel[-1])]
    L = [5 * h[-1], L[-1]]
    geom = {"ndim": 2, "nn": 16, "h": h, "nel": nel, "L": L}
    mesh = setup_mesh(instr, geom)
    cmpr = setup_cmpr(mesh, E=float(E), nu=float(nu), rho0=float(rho0))
    mpts = setup_mpts(mesh, cmpr, get_collapse(mesh, cmpr, 2, float(l0)))
    tg = math.ceil((1.0 / cmpr["c"]) * (2.0 * l0) * 40.0)
    time = setup_time(instr, te=float(tg), tg=float(tg))
    ic = {"mesh": mesh, "mpts": mpts, "cmpr": cmpr, "time": time}
    cfg = {"instr": instr, "misc": {"file": f"{mesh.dim}d_{instr['fwrk']['trsfr']}"}}
    return ic, cfg
