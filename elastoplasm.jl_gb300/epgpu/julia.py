"""Julia floating-point range semantics, restated for the host-side set-up.

ElastoPlasm builds every mesh coordinate, material-point lattice and checkpoint
list with Julia ranges, e.g. ``collect(first(x0):h[1]:last(x0))``
(utils/setup/mesh/get_coords.jl:31-33), ``collect(xB+0.5h/ni : h/ni : xB)``
(utils/setup/mpts/mpts_populate.jl:28-29) and
``sort(collect(time.t[1]:freq:time.te))`` (workflow/worflow.jl:24,69).

Julia does not step a float range by repeated addition.  ``a:s:b`` first tries
to express start, step and stop as small rationals (``Base.rat``); when that
succeeds the elements are the rationals ``(start_n + (i-1) step_n)/den``
evaluated in double-double precision, i.e. the correctly rounded decimal
values.  Otherwise it falls back to ``start + (i-1)*step`` with the product
rounded first.  The B-spline basis later compares node coordinates with
``==`` (workflow/shpfun/basis/bsmpm.jl:64-72) and the Dirichlet masks do too
(utils/setup/mesh/get_bc.jl:15), so the exact bits matter: they are
reproduced here with Python floats (IEEE binary64, no fused operations).
"""
from __future__ import annotations

from fractions import Fraction
import math

_MAXINTFLOAT_F32 = 16777216          # maxintfloat(Float32, Int): Base.rat bound
_MAXINTFLOAT_F64 = 2 ** 53           # maxintfloat(Float64, Int)


def _trunc_int(y: float) -> int:
    return int(math.trunc(y))


def rat(x: float) -> tuple[int, int]:
    """Continued-fraction rational approximation (Julia ``Base.rat``)."""
    y = x
    a = d = 1
    b = c = 0
    m = _MAXINTFLOAT_F32
    while abs(y) <= m:
        f = _trunc_int(y)
        y -= f
        a, c = f * a + c, a
        b, d = f * b + d, b
        if not max(abs(a), abs(b)) <= m:
            return c, d
        if b != 0:
            ratio = float(a) / float(b)
        else:
            ratio = math.copysign(math.inf, a) if a != 0 else math.nan
        if ratio == x:
            break
        y = 1.0 / y if y != 0.0 else math.inf
    return a, b


def _tdiv(a: int, b: int) -> int:
    """Julia ``div`` on integers: quotient truncated toward zero."""
    q = abs(a) // abs(b)
    return q if (a >= 0) == (b >= 0) else -q


def _isbetween(a: float, x: float, b: float) -> bool:
    return (a <= x <= b) or (b <= x <= a)


def frange(start: float, step: float, stop: float) -> list[float]:
    """Elements of the Julia range ``start:step:stop`` (all Float64)."""
    start, step, stop = float(start), float(step), float(stop)
    if step == 0.0:
        raise ValueError("range step cannot be zero")
    step_n, step_d = rat(step)
    if step_d != 0 and float(step_n) / float(step_d) == step:
        start_n, start_d = rat(start)
        stop_n, stop_d = rat(stop)
        if (start_d != 0 and stop_d != 0
                and float(start_n) / float(start_d) == start
                and float(stop_n) / float(stop_d) == stop):
            den = start_d * step_d // math.gcd(start_d, step_d)
            m = _MAXINTFLOAT_F64
            if (den != 0 and abs(start * den) <= m and abs(step * den) <= m
                    and den % start_d == 0 and den % step_d == 0):
                start_n = round(start * den)       # ties to even, as Julia
                step_n = round(step * den)
                length = max(0, _tdiv(den * stop_n - stop_d * start_n + step_n * stop_d,
                                      step_n * stop_d))
                if (_isbetween(start, start + (length - 1) * step, stop + step / 2)
                        and not _isbetween(start, start + length * step, stop)):
                    # twice-precision range: elements are the correctly rounded
                    # rationals (start_n + k step_n)/den
                    return [float(Fraction(start_n + k * step_n, den)) for k in range(length)]
    # fallback: take start and step literally
    lf = (stop - start) / step
    if lf < 0:
        length = 0
    elif lf == 0:
        length = 1
    else:
        length = int(round(lf)) + 1
        stop2 = start + (length - 1) * step
        length -= int(start < stop < stop2) + int(start > stop > stop2)
    return [start + (k * step) for k in range(length)]


def linrange(start: float, stop: float, n: int) -> list[float]:
    """Julia ``LinRange(start, stop, n)`` elements: ``(1-t)*a + t*b``, ``t=j/d``."""
    start, stop = float(start), float(stop)
    if n == 1:
        return [start]
    d = n - 1
    out = []
    for j in range(n):
        t = j / d
        out.append((1.0 - t) * start + t * stop)
    return out
