"""Exact solution of the 1D Riemann problem for an ideal gas (test
infrastructure only).

Restates the published exact solver (E. F. Toro, *Riemann Solvers and
Numerical Methods for Fluid Dynamics*, 3rd ed., chapter 4): the pressure
function f(p) = f_L(p) + f_R(p) + (u_R - u_L) with shock (Rankine-Hugoniot)
and rarefaction (isentropic) branches, Newton iteration for the star
pressure from the two-rarefaction guess, then sampling of the wave pattern at
x / t.  The reference compares its 3D Sod runs with such a solution
(python/cfdSolver/torchAnalysis.py `exact_riemann_sod`, used by
python/tests/testSolver3D.py:103-121: mean |rho - exact| < 0.04 at 32 cells,
t = 0.08, diaphragm at 1/2, (rho, u, p) = (1, 0, 1) | (0.125, 0, 0.1)).
"""

import numpy as np


def _branch(p, rho, pk, ck, g):
    """f_K(p) and its derivative for side K (shock if p > p_K)."""
    if p > pk:
        a = 2.0 / ((g + 1.0) * rho)
        b = (g - 1.0) / (g + 1.0) * pk
        s = np.sqrt(a / (p + b))
        return (p - pk) * s, s * (1.0 - 0.5 * (p - pk) / (b + p))
    r = p / pk
    f = 2.0 * ck / (g - 1.0) * (r ** ((g - 1.0) / (2.0 * g)) - 1.0)
    return f, 1.0 / (rho * ck) * r ** (-(g + 1.0) / (2.0 * g))


def star_state(left, right, g=1.4, tol=1e-14, max_iter=100):
    """(p*, u*) between the left and right states (rho, u, p)."""
    rl, ul, pl = left
    rr, ur, pr = right
    cl, cr = np.sqrt(g * pl / rl), np.sqrt(g * pr / rr)
    z = (g - 1.0) / (2.0 * g)
    p = ((cl + cr - 0.5 * (g - 1.0) * (ur - ul)) / (cl / pl ** z + cr / pr ** z)) ** (1.0 / z)
    for _ in range(max_iter):
        fl, dl = _branch(p, rl, pl, cl, g)
        fr, dr = _branch(p, rr, pr, cr, g)
        step = (fl + fr + ur - ul) / (dl + dr)
        p_new = max(p - step, tol)
        if abs(p_new - p) <= tol * 0.5 * (p_new + p):
            p = p_new
            break
        p = p_new
    fl, _ = _branch(p, rl, pl, cl, g)
    fr, _ = _branch(p, rr, pr, cr, g)
    return p, 0.5 * (ul + ur) + 0.5 * (fr - fl)


def sample(left, right, x, t, x0=0.5, g=1.4):
    """(rho, u, p) of the exact solution at positions x and time t > 0."""
    rl, ul, pl = left
    rr, ur, pr = right
    cl, cr = np.sqrt(g * pl / rl), np.sqrt(g * pr / rr)
    ps, us = star_state(left, right, g)
    s = (np.asarray(x, float) - x0) / t
    rho, u, p = np.empty_like(s), np.empty_like(s), np.empty_like(s)
    gm, gp = (g - 1.0) / (g + 1.0), (g + 1.0) / (2.0 * g)
    for i, si in enumerate(s):
        if si <= us:  # left of the contact
            if ps > pl:  # left shock
                sl = ul - cl * np.sqrt(gp * ps / pl + (g - 1.0) / (2.0 * g))
                if si <= sl:
                    rho[i], u[i], p[i] = rl, ul, pl
                else:
                    rho[i] = rl * (ps / pl + gm) / (gm * ps / pl + 1.0)
                    u[i], p[i] = us, ps
            else:  # left rarefaction
                head = ul - cl
                cs = cl * (ps / pl) ** ((g - 1.0) / (2.0 * g))
                tail = us - cs
                if si <= head:
                    rho[i], u[i], p[i] = rl, ul, pl
                elif si >= tail:
                    rho[i] = rl * (ps / pl) ** (1.0 / g)
                    u[i], p[i] = us, ps
                else:
                    c = 2.0 / (g + 1.0) * (cl + 0.5 * (g - 1.0) * (ul - si))
                    u[i] = 2.0 / (g + 1.0) * (cl + 0.5 * (g - 1.0) * ul + si)
                    rho[i] = rl * (c / cl) ** (2.0 / (g - 1.0))
                    p[i] = pl * (c / cl) ** (2.0 * g / (g - 1.0))
        else:  # right of the contact
            if ps > pr:  # right shock
                sr = ur + cr * np.sqrt(gp * ps / pr + (g - 1.0) / (2.0 * g))
                if si >= sr:
                    rho[i], u[i], p[i] = rr, ur, pr
                else:
                    rho[i] = rr * (ps / pr + gm) / (gm * ps / pr + 1.0)
                    u[i], p[i] = us, ps
            else:  # right rarefaction
                head = ur + cr
                cs = cr * (ps / pr) ** ((g - 1.0) / (2.0 * g))
                tail = us + cs
                if si >= head:
                    rho[i], u[i], p[i] = rr, ur, pr
                elif si <= tail:
                    rho[i] = rr * (ps / pr) ** (1.0 / g)
                    u[i], p[i] = us, ps
                else:
                    c = 2.0 / (g + 1.0) * (cr - 0.5 * (g - 1.0) * (ur - si))
                    u[i] = 2.0 / (g + 1.0) * (-cr + 0.5 * (g - 1.0) * ur + si)
                    rho[i] = rr * (c / cr) ** (2.0 / (g - 1.0))
                    p[i] = pr * (c / cr) ** (2.0 * g / (g - 1.0))
    return rho, u, p


def sod(x, t, g=1.4):
    """The standard Sod tube: (1, 0, 1) | (0.125, 0, 0.1), diaphragm at 1/2."""
    return sample((1.0, 0.0, 1.0), (0.125, 0.0, 0.1), x, t, 0.5, g)
