"""CPU restatement of savlot's per-point plot fields (utils/plot.jl:27-135, what_plot_field).

TEST INFRASTRUCTURE ONLY: imported by tests/ as the checker of ``epgpu_fields``.  The product
never imports it.

Each field is the reference's broadcast expression on the downloaded point state, in the same
operation order, element by element in FP64 (numpy rounds every product and sum on its own, as
Julia's broadcasts do):
  P      -(σ[1,:] + σ[2,:])/2/1e3 (2d), -(σ[1,:] + σ[2,:] + σ[3,:])/3/1e3 (3d)   plot.jl:28-35
  sigxx  σ[1,:]/1e3                                                          plot.jl:43-44
  epsxx  ϵ[1,1,:]                                                            plot.jl:53-54
  epII   ϵpII[1,:]                                                           plot.jl:63-64
  epV    ϵpV                                                                 plot.jl:73-74
  du     sqrt(u[1,:]^2 + u[2,:]^2) (the first two components, also in 3d)  plot.jl:83-84
  z0     z0                                                                  plot.jl:93-94
  coh0   c0/1e3                                                              plot.jl:99-100
  phi0   ϕ                                                                   plot.jl:106-107
  n0, n  n (both options show mpts.n)                                        plot.jl:112-123
  J      J                                                                   plot.jl:124-125
  ms     ρ Ω                                                                 plot.jl:130-131
and the scatter coordinates x[1,:] and x[2,:] (2d) or x[3,:] (3d), plot.jl:142-147.
"""
from __future__ import annotations

import numpy as np


def plot_field(m, what: str) -> np.ndarray:
    """One option of what_plot_field on a Point-like state (column-major arrays as downloaded)."""
    sig = np.asarray(m.sig)
    if what == "P":
        if sig.shape[0] == 3:
            return -(sig[0] + sig[1]) / 2 / 1e3
        return -(sig[0] + sig[1] + sig[2]) / 3 / 1e3
    if what == "sigxx":
        return sig[0] / 1e3
    if what == "epsxx":
        return np.asarray(m.eij)[0, 0]
    if what == "epII":
        return np.asarray(m.epII)[0]
    if what == "epV":
        return np.asarray(m.epV)
    if what == "du":
        u = np.asarray(m.u)
        return np.sqrt(u[0] ** 2 + u[1] ** 2)
    if what == "z0":
        return np.asarray(m.z0)
    if what == "coh0":
        return np.asarray(m.c0) / 1e3
    if what == "phi0":
        return np.asarray(m.phi)
    if what in ("n0", "n"):
        return np.asarray(m.n)
    if what == "J":
        return np.asarray(m.J)
    if what == "ms":
        return np.asarray(m.rho) * np.asarray(m.Omega)
    raise ValueError(f"UndefinedPlotOption: {what}")


def plot_coords(m):
    x = np.asarray(m.x)
    return x[0], x[-1]
