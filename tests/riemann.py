"""Exact solution of the 1D Riemann problem for a calorically perfect gas
(Toro, "Riemann Solvers and Numerical Methods for Fluid Dynamics", ch. 4:
Newton iteration on the pressure function for the star region).  Used to pin
the oracle's shock-tube solution; test infrastructure only."""
import math

import numpy as np


def _fk(p, rk, pk, ck, g):
    if p > pk:  # shock
        A = 2.0 / ((g + 1.0) * rk)
        B = (g - 1.0) / (g + 1.0) * pk
        sq = math.sqrt(A / (p + B))
        return (p - pk) * sq, sq * (1.0 - 0.5 * (p - pk) / (B + p))
    pr = p / pk  # rarefaction
    f = 2.0 * ck / (g - 1.0) * (pr ** ((g - 1.0) / (2.0 * g)) - 1.0)
    return f, 1.0 / (rk * ck) * pr ** (-(g + 1.0) / (2.0 * g))


def star(rl, ul, pl, rr, ur, pr, g):
    cl, cr = math.sqrt(g * pl / rl), math.sqrt(g * pr / rr)
    p = max(1e-8, 0.5 * (pl + pr))
    for _ in range(100):
        fl, dl = _fk(p, rl, pl, cl, g)
        fr, dr = _fk(p, rr, pr, cr, g)
        dp = (fl + fr + ur - ul) / (dl + dr)
        p = max(1e-12, p - dp)
        if abs(dp) < 1e-14 * p:
            break
    fl, _ = _fk(p, rl, pl, cl, g)
    fr, _ = _fk(p, rr, pr, cr, g)
    return p, 0.5 * (ul + ur) + 0.5 * (fr - fl)


def sample(x, t, rl, ul, pl, rr, ur, pr, g=1.4):
    """Density, velocity, pressure at positions x (diaphragm at 0) and time t."""
    ps, us = star(rl, ul, pl, rr, ur, pr, g)
    cl, cr = math.sqrt(g * pl / rl), math.sqrt(g * pr / rr)
    out = np.zeros((3, len(x)))
    for n, xi in enumerate(x):
        s = xi / t
        if s <= us:  # left of contact
            if ps > pl:
                sl = ul - cl * math.sqrt((g + 1) / (2 * g) * ps / pl + (g - 1) / (2 * g))
                if s <= sl:
                    w = (rl, ul, pl)
                else:
                    w = (rl * ((ps / pl + (g - 1) / (g + 1)) / ((g - 1) / (g + 1) * ps / pl + 1)), us, ps)
            else:
                shl = ul - cl
                csl = cl * (ps / pl) ** ((g - 1) / (2 * g))
                stl = us - csl
                if s <= shl:
                    w = (rl, ul, pl)
                elif s >= stl:
                    w = (rl * (ps / pl) ** (1 / g), us, ps)
                else:
                    c = 2 / (g + 1) * (cl + (g - 1) / 2 * (ul - s))
                    w = (rl * (c / cl) ** (2 / (g - 1)), 2 / (g + 1) * (cl + (g - 1) / 2 * ul + s),
                         pl * (c / cl) ** (2 * g / (g - 1)))
        else:
            if ps > pr:
                sr = ur + cr * math.sqrt((g + 1) / (2 * g) * ps / pr + (g - 1) / (2 * g))
                if s >= sr:
                    w = (rr, ur, pr)
                else:
                    w = (rr * ((ps / pr + (g - 1) / (g + 1)) / ((g - 1) / (g + 1) * ps / pr + 1)), us, ps)
            else:
                shr = ur + cr
                csr = cr * (ps / pr) ** ((g - 1) / (2 * g))
                str_ = us + csr
                if s >= shr:
                    w = (rr, ur, pr)
                elif s <= str_:
                    w = (rr * (ps / pr) ** (1 / g), us, ps)
                else:
                    c = 2 / (g + 1) * (cr - (g - 1) / 2 * (ur - s))
                    w = (rr * (c / cr) ** (2 / (g - 1)), 2 / (g + 1) * (-cr + (g - 1) / 2 * ur + s),
                         pr * (c / cr) ** (2 * g / (g - 1)))
        out[:, n] = w
    return out
