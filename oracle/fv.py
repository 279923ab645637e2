"""NumPy restatement of TORCH's Cartesian finite-volume step (the oracle).

Test infrastructure only (see ``oracle/__init__.py``).  Every function names
the reference lines it restates.  Arithmetic is written so that each NumPy
expression performs the same IEEE-754 double operations, in the same order,
as the reference: products and sums are parenthesised the way Python parses
the reference expressions, sums of squares over the component axis are
sequential, and masks are applied with the reference's precedence.

State layout: ``(dim + 2, nz, ny, nx)`` (x fastest), components rho, rho*u,
[rho*v], [rho*w], E.  Boundary names are the reference's session names
(``Open``, ``Reflective``, ``Periodic``, 2D y ``Inflow``) plus the step
functions' aliases.
"""

import numpy as np

FLOOR = 1e-12  # density / pressure floor used throughout the reference
GUARD = 1e-14  # division guard used by the limiters and HLLC

LIMITERS = ("VanLeer", "Albada", "MINBEE", "Superbee", "Unos")

OPEN, REFLECTIVE, PERIODIC, INFLOW = 0, 1, 2, 3
_BC_NAMES = {
    "open": OPEN, "transmissive": OPEN, "outflow": OPEN,
    "reflective": REFLECTIVE, "wall": REFLECTIVE, "slip": REFLECTIVE,
    "periodic": PERIODIC, "wrap": PERIODIC,
    "inflow": INFLOW,
}
DEFAULT_INLET = (1.0, 0.0, 100.0, 101325.0)  # torchSolver2D.py:229


def bc_code(name):
    """Boundary name -> code (torchSolver3D.py:52-61, torchSolver2D.py:191-264)."""
    try:
        return _BC_NAMES[str(name).lower()]
    except KeyError:
        raise ValueError(f"Unknown boundary: {name}") from None


def _sqsum(rows):
    """Sequential sum of squares over the leading axis, as np.sum(x**2, axis=0)."""
    total = rows[0] * rows[0]
    for k in range(1, rows.shape[0]):
        total = total + rows[k] * rows[k]
    return total


# ---------------------------------------------------------------------------
# Ghost cells
# ---------------------------------------------------------------------------

def _axis_map(n, width, code):
    """Source index and ghost mask for one padded axis.

    Open = edge copy, Reflective = mirror ('symmetric'), Periodic = wrap
    (torchSolver3D.py:47-70; torchSolver2D.py:176-266).  Inflow maps like Open;
    its low-side ghosts are replaced by the inlet afterwards.
    """
    i = np.arange(-width, n + width)
    if code in (OPEN, INFLOW):
        src = np.clip(i, 0, n - 1)
    elif code == REFLECTIVE:
        src = np.where(i < 0, -1 - i, np.where(i >= n, 2 * n - 1 - i, i))
    elif code == PERIODIC:
        src = np.mod(i, n)
    else:
        raise ValueError(f"Unknown boundary code {code}")
    return src, (i < 0) | (i >= n), i < 0


def pad(values, bcs_xyz, width, vector, inlet=None):
    """Pad ``width`` ghost layers on every spatial axis.

    vector=True: ``values`` is (nv, *spatial) and Reflective negates the
    normal momentum in that axis' ghosts (torchSolver3D.py:64-69,
    torchSolver2D.py:204-212,252-261).  A y ``Inflow`` boundary (2D only)
    fills the low y ghosts with ``inlet`` (conservative vector for states,
    scalar for padded scalars) (torchSolver2D.py:224-245,647-656).
    """
    out = np.asarray(values)
    lead = 1 if vector else 0
    dim = out.ndim - lead
    for d in range(dim):  # d = 0 is x, the last array axis
        axis = out.ndim - 1 - d
        n = out.shape[axis]
        src, ghost, low = _axis_map(n, width, bcs_xyz[d])
        out = np.take(out, src, axis=axis)
        if vector and bcs_xyz[d] == REFLECTIVE:
            shape = [1] * (out.ndim - 1)
            shape[axis - 1] = -1
            sign = np.where(ghost, -1.0, 1.0).reshape(shape)
            out[d + 1] = out[d + 1] * sign
        if bcs_xyz[d] == INFLOW:
            index = [slice(None)] * out.ndim
            index[axis] = np.nonzero(low)[0]
            if vector:
                fill = np.asarray(inlet, dtype=float).reshape(
                    (-1,) + (1,) * (out.ndim - 1))
                out[tuple(index)] = fill
            else:
                out[tuple(index)] = inlet
    return out


# ---------------------------------------------------------------------------
# Conversions and physical fluxes
# ---------------------------------------------------------------------------

def prim_to_cons(prim, gamma):
    """Primitive -> conservative, any dimension (torchSession.py:146-150,
    torchSolver3D.py:27-34)."""
    prim = np.asarray(prim, dtype=float)
    state = prim.copy()
    state[1:-1] *= prim[0]
    state[-1] = prim[-1] / (gamma - 1) + 0.5 * prim[0] * _sqsum(prim[1:-1])
    return state


def prim_to_cons_2d(prim, gamma):
    """torchSolver2D.py:61-82 (floors rho and p)."""
    rho = np.maximum(prim[0], FLOOR)
    u, v = prim[1], prim[2]
    p = np.maximum(prim[3], FLOOR)
    out = np.empty_like(prim, dtype=float)
    out[0] = rho
    out[1] = rho * u
    out[2] = rho * v
    out[3] = p / (gamma - 1.0) + 0.5 * rho * (u * u + v * v)
    return out


def cons_to_prim_3d(state, gamma):
    """torchSolver3D.py:37-44 (no floors)."""
    prim = state.copy()
    prim[1:4] /= state[0]
    prim[4] = (gamma - 1) * (state[4] - 0.5 * _sqsum(state[1:4]) / state[0])
    return prim


def cons_to_prim_2d(state, gamma):
    """torchSolver2D.py:38-58 (floors rho and p at 1e-12)."""
    rho = np.maximum(state[0], FLOOR)
    u = state[1] / rho
    v = state[2] / rho
    internal = state[3] - 0.5 * rho * (u * u + v * v)
    out = np.empty_like(state)
    out[0] = rho
    out[1] = u
    out[2] = v
    out[3] = np.maximum((gamma - 1.0) * internal, FLOOR)
    return out


def sound_2d(prim, gamma):
    """torchSolver2D.py:85-91."""
    return np.sqrt(gamma * np.maximum(prim[3], FLOOR) / np.maximum(prim[0], FLOOR))


def flux_3d(state, gamma, m):
    """Physical flux along momentum row m (torchSolver3D.py:77-83)."""
    prim = cons_to_prim_3d(state, gamma)
    vel, p = prim[m], prim[4]
    out = state * vel
    out[m] += p
    out[4] = vel * (state[4] + p)
    return out


def physical(state):
    """torchSolver.py:1038-1046: finite, rho > 1e-12, internal energy > 1e-12."""
    return bool(
        np.isfinite(state).all()
        and np.all(state[0] > FLOOR)
        and np.all(state[-1] - 0.5 * _sqsum(state[1:-1]) / state[0] > FLOOR)
    )


# ---------------------------------------------------------------------------
# Limiters
# ---------------------------------------------------------------------------

def _phi_3d(r, limiter):
    """Limiter function of the 3D step (torchSolver3D.py:90-110)."""
    pos = np.maximum(r, 0)
    if limiter == "VanLeer":
        return 2 * pos / (1 + pos)
    if limiter == "Albada":
        return (pos * pos + pos) / (pos * pos + 1)
    if limiter == "MINBEE":
        return np.maximum(0, np.minimum(r, 1))
    if limiter == "Superbee":
        return np.maximum(0, np.maximum(np.minimum(2 * r, 1), np.minimum(r, 2)))
    if limiter == "Unos":
        return np.maximum(0, np.minimum(
            np.minimum(np.minimum(2, 2 * r), (2 + r) / 3), (1 + 2 * r) / 3))
    raise ValueError(f"Unknown limiter: {limiter}")


def _phi_2d(r, limiter):
    """Limiter function of the 2D step (torchSolver2D.py:147-165).

    VanLeer/Albada return 0 where r <= 0 (or NaN); Unos has no (1+2r)/3 bound;
    unknown names fall back to VanLeer.
    """
    lim = limiter.lower()
    if lim in ("minbee", "minmod"):
        return np.maximum(0.0, np.minimum(r, 1.0))
    if lim == "superbee":
        return np.maximum(0.0, np.maximum(np.minimum(2.0 * r, 1.0), np.minimum(r, 2.0)))
    if lim == "unos":
        return np.maximum(0.0, np.minimum(np.minimum(2.0, 2.0 * r), (2.0 + r) / 3.0))
    pos = np.maximum(r, 0.0)
    if lim in ("albada", "vanalbada", "van_albada"):
        return np.where(r > 0.0, (pos * pos + pos) / (pos * pos + 1.0), 0.0)
    return np.where(r > 0.0, 2.0 * pos / (1.0 + pos), 0.0)


def _limited(minus, plus, phi_fn, limiter):
    safe = np.where(np.abs(plus) < GUARD, GUARD, plus)
    return phi_fn(minus / safe, limiter) * plus


def slope_3d(padded, axis, limiter):
    """Limited slope on the active box (padded[..., 1:-1]) along array axis
    ``axis`` (torchSolver3D.py:86-111)."""
    n = padded.shape[axis]
    centre = [slice(None)] + [slice(1, -1)] * (padded.ndim - 1)
    lo, hi = list(centre), list(centre)
    lo[axis] = slice(0, n - 2)
    hi[axis] = slice(2, n)
    c = padded[tuple(centre)]
    return _limited(c - padded[tuple(lo)], padded[tuple(hi)] - c, _phi_3d, limiter)


def slope_2d(arr, axis, limiter):
    """torchSolver2D.py:124-168 (axis 1 = x, axis 0 = y of the spatial dims)."""
    if axis == 1:
        minus = arr[:, :, 1:-1] - arr[:, :, :-2]
        plus = arr[:, :, 2:] - arr[:, :, 1:-1]
    elif axis == 0:
        minus = arr[:, 1:-1, :] - arr[:, :-2, :]
        plus = arr[:, 2:, :] - arr[:, 1:-1, :]
    else:
        raise ValueError("Axis must be 0 or 1.")
    return _limited(minus, plus, _phi_2d, limiter)


# ---------------------------------------------------------------------------
# HLLC
# ---------------------------------------------------------------------------

def hllc(ul, ur, gamma_l=1.4, gamma_r=None):
    """Normal HLLC flux on rows [rho, m_n, m_t..., E] (torchFlux.py:125-248).

    Where no wave-speed mask holds (NaN speeds) the reference leaves the
    output uninitialised; this restatement returns NaN there.
    """
    gl = gamma_l
    gr = gamma_l if gamma_r is None else gamma_r
    g = 0.5 * (gl + gr)
    rl = np.maximum(ul[0], FLOOR)
    rr = np.maximum(ur[0], FLOOR)
    unl = ul[1] / rl
    unr = ur[1] / rr
    utl = ul[2:-1] / rl
    utr = ur[2:-1] / rr
    kel = 0.5 * rl * (unl * unl + _sqsum(utl))
    ker = 0.5 * rr * (unr * unr + _sqsum(utr))
    pl = np.maximum((gl - 1.0) * (ul[-1] - kel), FLOOR)
    pr = np.maximum((gr - 1.0) * (ur[-1] - ker), FLOOR)
    al = np.sqrt(gl * pl / rl)
    ar = np.sqrt(gr * pr / rr)

    fl = np.empty_like(ul)
    fl[0] = rl * unl
    fl[1] = rl * (unl * unl) + pl
    fl[2:-1] = rl * unl * utl
    fl[-1] = unl * (ul[-1] + pl)
    fr = np.empty_like(ur)
    fr[0] = rr * unr
    fr[1] = rr * (unr * unr) + pr
    fr[2:-1] = rr * unr * utr
    fr[-1] = unr * (ur[-1] + pr)

    sql = np.sqrt(rl)
    sqr = np.sqrt(rr)
    inv = 1.0 / (sql + sqr)
    u_roe = (sql * unl + sqr * unr) * inv
    v_roe = (sql * utl + sqr * utr) * inv
    hl = (ul[-1] + pl) / rl
    hr = (ur[-1] + pr) / rr
    h_roe = (sql * hl + sqr * hr) * inv
    ke_roe = 0.5 * (u_roe * u_roe + _sqsum(v_roe))
    a_roe = np.sqrt(np.maximum((g - 1.0) * (h_roe - ke_roe), FLOOR))

    sl = np.minimum(unl - al, u_roe - a_roe)
    sr = np.maximum(unr + ar, u_roe + a_roe)
    den = rl * (sl - unl) - rr * (sr - unr)
    den = np.where(np.abs(den) < GUARD, GUARD, den)
    ss = (pr - pl + rl * unl * (sl - unl) - rr * unr * (sr - unr)) / den

    def star(u, rho, un, ut, p, s):
        d_ss = np.where(np.abs(s - ss) < GUARD, GUARD, s - ss)
        rho_s = np.maximum(rho * ((s - un) / d_ss), FLOOR)
        d_un = np.where(np.abs(s - un) < GUARD, GUARD, s - un)
        out = np.empty_like(u)
        out[0] = rho_s
        out[1] = rho_s * ss
        out[2:-1] = rho_s * ut
        out[-1] = rho_s * (u[-1] / rho + (ss - un) * (ss + p / (rho * d_un)))
        return out

    fsl = fl + sl * (star(ul, rl, unl, utl, pl, sl) - ul)
    fsr = fr + sr * (star(ur, rr, unr, utr, pr, sr) - ur)
    close_l = np.abs(sl - ss) < FLOOR
    close_r = np.abs(sr - ss) < FLOOR
    fsl[:, close_l] = fl[:, close_l]
    fsr[:, close_r] = fr[:, close_r]

    flux = np.full_like(ul, np.nan)
    for mask, value in (
        (0.0 <= sl, fl),
        ((sl <= 0.0) & (0.0 <= ss), fsl),
        ((ss <= 0.0) & (0.0 <= sr), fsr),
        (0.0 >= sr, fr),
    ):
        flux[:, mask] = value[:, mask]
    return flux


_POOL = None
_WORKERS = 1


def set_workers(workers):
    """Evaluate HLLC in ordered 8192-face batches on a thread pool of this size,
    as the reference's Execution.map does (torchExecution.py:17-58,
    torchFlux.py:57-75).  Values are identical for every worker count."""
    global _POOL, _WORKERS
    from concurrent.futures import ThreadPoolExecutor
    if _POOL is not None:
        _POOL.shutdown(wait=True)
        _POOL = None
    _WORKERS = int(workers)
    if _WORKERS > 1:
        _POOL = ThreadPoolExecutor(max_workers=_WORKERS, thread_name_prefix="oracle-flux")


def hllc_grid(left, right, gamma_l, gamma_r=None, direction=0, batch=8192):
    """Rotate Cartesian components into the normal basis, evaluate HLLC and
    rotate back (torchFlux.py:6-77; batching does not change values)."""
    nv = left.shape[0]
    normal = direction + 1
    order = [0, normal] + [m for m in range(1, nv - 1) if m != normal] + [nv - 1]
    gl = np.broadcast_to(gamma_l, left.shape[1:])
    gr = gl if gamma_r is None else np.broadcast_to(gamma_r, left.shape[1:])
    ul = left[order].reshape(nv, -1)
    ur = right[order].reshape(nv, -1)
    gl, gr = gl.ravel(), gr.ravel()
    n = ul.shape[1]
    if _POOL is None or n <= batch:
        value = hllc(ul, ur, gl, gr)
    else:
        value = np.empty((nv, n))
        spans = [(a, min(a + batch, n)) for a in range(0, n, batch)]

        def work(span):
            a, b = span
            return a, b, hllc(ul[:, a:b], ur[:, a:b], gl[a:b], gr[a:b])

        for a, b, v in _POOL.map(work, spans):
            value[:, a:b] = v
    out = np.empty(left.shape)
    out[order] = value.reshape((nv,) + left.shape[1:])
    return out


# ---------------------------------------------------------------------------
# 3D step
# ---------------------------------------------------------------------------

def _faces_3d(array, axis, active):
    """Left/right face operands (torchSolver3D.py:114-119)."""
    inner = slice(1, -1) if active else slice(2, -2)
    left = [slice(None)] + [inner] * 3
    right = list(left)
    left[axis] = slice(None, -1) if active else slice(1, -2)
    right[axis] = slice(1, None) if active else slice(2, -1)
    return array[tuple(left)], array[tuple(right)]


def hydro_3d(state, gamma, spacing, dt, limiter, bcs_xyz, first_order=False):
    """Unsplit MUSCL-Hancock + HLLC step with the whole-step first-order
    Rusanov fallback (torchSolver3D.py:122-203).

    Returns (result, [flux_x, flux_y, flux_z], used_first_order).
    """
    bcs = [bc_code(b) if isinstance(b, str) else b for b in bcs_xyz]
    padded = pad(state, bcs, 2, True)
    gp = pad(np.broadcast_to(gamma, state.shape[1:]), bcs, 2, False)
    active = padded[:, 1:-1, 1:-1, 1:-1]
    ga = gp[1:-1, 1:-1, 1:-1]
    axes = (3, 2, 1)
    if not first_order:
        slopes = [slope_3d(padded, a, limiter) for a in axes]
        predicted = active.copy()
        for m, (s, h) in enumerate(zip(slopes, spacing), 1):
            predicted -= 0.5 * dt / h * (flux_3d(active + 0.5 * s, ga, m)
                                         - flux_3d(active - 0.5 * s, ga, m))
        if any(not physical(predicted + sign * 0.5 * s)
               for s in slopes for sign in (-1, 1)):
            return hydro_3d(state, gamma, spacing, dt, limiter, bcs, True)
    fluxes = []
    for m, axis in enumerate(axes, 1):
        if first_order:
            left, right = _faces_3d(padded, axis, False)
            gl, gr = _faces_3d(gp[None], axis, False)
            gl, gr = gl[0], gr[0]
            pl, pr = cons_to_prim_3d(left, gl), cons_to_prim_3d(right, gr)
            speed = np.maximum(np.abs(pl[m]) + np.sqrt(gl * pl[4] / pl[0]),
                               np.abs(pr[m]) + np.sqrt(gr * pr[4] / pr[0]))
            flux = 0.5 * (flux_3d(left, gl, m) + flux_3d(right, gr, m)
                          - speed * (right - left))
        else:
            pl, pr = _faces_3d(predicted, axis, True)
            sl, sr = _faces_3d(slopes[m - 1], axis, True)
            gl, gr = _faces_3d(ga[None], axis, True)
            flux = hllc_grid(pl + 0.5 * sl, pr - 0.5 * sr, gl[0], gr[0],
                             direction=m - 1)
        fluxes.append(flux)
    result = state.copy()
    for flux, h, axis in zip(fluxes, spacing, axes):
        result -= dt / h * np.diff(flux, axis=axis)
    if not physical(result):
        if not first_order:
            return hydro_3d(state, gamma, spacing, dt, limiter, bcs, True)
        raise RuntimeError("3D hydrodynamic update produced a nonphysical state")
    return result, fluxes, first_order


# ---------------------------------------------------------------------------
# 2D step
# ---------------------------------------------------------------------------

def inlet_state_2d(inlet_primitive=None):
    """Conservative inlet ghost state, always with gamma = 1.4
    (torchSolver2D.py:227-243)."""
    inlet = np.asarray(DEFAULT_INLET if inlet_primitive is None else inlet_primitive,
                       dtype=float)
    if (inlet.shape != (4,) or not np.isfinite(inlet).all() or inlet[0] <= 0
            or inlet[3] <= 0 or inlet[2] < 0):
        raise ValueError("Inlet requires [rho>0, u, v>=0, p>0] in SI")
    return prim_to_cons_2d(inlet[:, None, None], 1.4)[:, 0, 0]


def pad_state_2d(state, bc_x, bc_y, inlet_primitive=None):
    """apply_boundary_conditions_2d (torchSolver2D.py:176-266)."""
    bcs = (bc_code(bc_x), bc_code(bc_y))
    if bcs[0] == INFLOW:
        raise ValueError(f"Unknown x boundary: {bc_x}")
    inlet = inlet_state_2d(inlet_primitive) if bcs[1] == INFLOW else None
    return pad(state, bcs, 2, True, inlet)


def pad_scalar_2d(q, bc_x, bc_y, inlet_value=1.0):
    """pad_scalar_2d (torchSolver2D.py:647-656)."""
    bcs = (bc_code(bc_x), bc_code(bc_y))
    return pad(np.asarray(q, dtype=float), bcs, 2, False, inlet_value)


def _euler_flux_2d(u, gamma, normal):
    """Predictor fluxes euler_flux_x / euler_flux_y (torchSolver2D.py:326-352)."""
    rho = np.maximum(u[0], FLOOR)
    vx = u[1] / rho
    vy = u[2] / rho
    p = np.maximum((gamma - 1.0) * (u[3] - 0.5 * rho * (vx * vx + vy * vy)), FLOOR)
    f = np.empty_like(u)
    if normal == 0:
        f[0] = rho * vx
        f[1] = rho * (vx * vx) + p
        f[2] = rho * vx * vy
        f[3] = vx * (u[3] + p)
    else:
        f[0] = rho * vy
        f[1] = rho * vx * vy
        f[2] = rho * (vy * vy) + p
        f[3] = vy * (u[3] + p)
    return f


def hydro_2d(u_inner, dx, dy, dt, gamma=1.4, limiter="VanLeer", bc_x="Periodic",
             bc_y="Open", inlet_primitive=None):
    """Unsplit 2D MUSCL-Hancock + HLLC with the LLF fallback
    (torchSolver2D.py:274-466).  Returns (u_next, flux_x, flux_y, used_llf)."""
    ny, nx = u_inner.shape[1], u_inner.shape[2]
    u_pad = pad_state_2d(u_inner, bc_x, bc_y, inlet_primitive)
    gpad = pad_scalar_2d(np.broadcast_to(gamma, (ny, nx)), bc_x, bc_y, 1.4)
    g = gpad[1:ny + 3, 1:nx + 3]
    u_act = u_pad[:, 1:ny + 3, 1:nx + 3]
    dxs = slope_2d(u_pad[:, 1:ny + 3, :], 1, limiter)
    dys = slope_2d(u_pad[:, :, 1:nx + 3], 0, limiter)

    u_bar = (u_act
             - (0.5 * dt / dx) * (_euler_flux_2d(u_act + 0.5 * dxs, g, 0)
                                  - _euler_flux_2d(u_act - 0.5 * dxs, g, 0))
             - (0.5 * dt / dy) * (_euler_flux_2d(u_act + 0.5 * dys, g, 1)
                                  - _euler_flux_2d(u_act - 0.5 * dys, g, 1)))
    u_bar[0] = np.maximum(u_bar[0], FLOOR)
    ke = 0.5 * (u_bar[1] * u_bar[1] + u_bar[2] * u_bar[2]) / u_bar[0]
    p_bar = (g - 1.0) * (u_bar[3] - ke)
    u_bar[3] = np.where(p_bar < FLOOR, FLOOR / (g - 1.0) + ke, u_bar[3])

    flux_x = hllc_grid(u_bar[:, 1:ny + 1, :-1] + 0.5 * dxs[:, 1:ny + 1, :-1],
                       u_bar[:, 1:ny + 1, 1:] - 0.5 * dxs[:, 1:ny + 1, 1:],
                       g[1:ny + 1, :-1], g[1:ny + 1, 1:], direction=0)
    flux_y = hllc_grid(u_bar[:, :-1, 1:nx + 1] + 0.5 * dys[:, :-1, 1:nx + 1],
                       u_bar[:, 1:, 1:nx + 1] - 0.5 * dys[:, 1:, 1:nx + 1],
                       g[:-1, 1:nx + 1], g[1:, 1:nx + 1], direction=1)
    u_next = (u_inner - (dt / dx) * (flux_x[:, :, 1:] - flux_x[:, :, :-1])
              - (dt / dy) * (flux_y[:, 1:, :] - flux_y[:, :-1, :]))
    used = False
    if not physical(u_next):
        used = True
        prim = cons_to_prim_2d(u_pad, gpad)
        ux, vy, pressure = prim[1], prim[2], prim[3]
        sound = sound_2d(prim, gpad)
        fx = np.stack((u_pad[1], u_pad[1] * ux + pressure, u_pad[2] * ux,
                       ux * (u_pad[3] + pressure)))
        fy = np.stack((u_pad[2], u_pad[1] * vy, u_pad[2] * vy + pressure,
                       vy * (u_pad[3] + pressure)))
        cx = np.abs(ux) + sound
        cy = np.abs(vy) + sound
        ax = np.maximum(cx[2:-2, 1:-2], cx[2:-2, 2:-1])
        ay = np.maximum(cy[1:-2, 2:-2], cy[2:-1, 2:-2])
        flux_x = 0.5 * (fx[:, 2:-2, 1:-2] + fx[:, 2:-2, 2:-1]
                        - ax * (u_pad[:, 2:-2, 2:-1] - u_pad[:, 2:-2, 1:-2]))
        flux_y = 0.5 * (fy[:, 1:-2, 2:-2] + fy[:, 2:-1, 2:-2]
                        - ay * (u_pad[:, 2:-1, 2:-2] - u_pad[:, 1:-2, 2:-2]))
        u_next = (u_inner - dt / dx * np.diff(flux_x, axis=2)
                  - dt / dy * np.diff(flux_y, axis=1))
    if not physical(u_next):
        raise RuntimeError("Hydrodynamic update produced a nonphysical state")
    return u_next, flux_x, flux_y, used


# ---------------------------------------------------------------------------
# CFL time steps
# ---------------------------------------------------------------------------

def dt_2d(state, spacing, cfl, gamma, bc_x, bc_y, inlet_primitive=None):
    """Session 2D dt on the padded state (torchSession.py:346-355,
    torchSolver2D.py:512-530)."""
    padded = pad_state_2d(state, bc_x, bc_y, inlet_primitive)
    gp = pad_scalar_2d(np.broadcast_to(gamma, state.shape[1:]), bc_x, bc_y, 1.4)
    prim = cons_to_prim_2d(padded, gp)
    a = sound_2d(prim, gp)
    total = np.max((np.abs(prim[1]) + a) / spacing[0]) + np.max(
        (np.abs(prim[2]) + a) / spacing[1])
    if total <= 1e-12:
        return 1e-3
    return float(cfl / total)


def dt_3d(state, spacing, cfl, gamma):
    """Session 3D dt on the interior (torchSession.py:356-360)."""
    p = cons_to_prim_3d(state, gamma)
    sound = np.sqrt(gamma * p[-1] / p[0])
    return cfl / sum(np.max(np.abs(p[m]) + sound) / h for m, h in enumerate(spacing, 1))


def wave_maxima_3d(state, gamma):
    """Per-direction max(|u_d| + a) used by dt_3d (for the GPU epilogue check)."""
    p = cons_to_prim_3d(state, gamma)
    sound = np.sqrt(gamma * p[-1] / p[0])
    return [float(np.max(np.abs(p[m]) + sound)) for m in (1, 2, 3)]


# ---------------------------------------------------------------------------
# Chemistry (Arrhenius / ZND) and species transport
# ---------------------------------------------------------------------------

def gamma_of_lambda(lam):
    """torchSolver.py:71-78."""
    return (4.5 - lam) / (3.5 - lam)


def cons_to_prim_1d(u, gamma):
    """torchSolver.py:117-127."""
    rho = np.maximum(u[0], FLOOR)
    vel = u[1] / rho
    p = np.maximum((u[2] - 0.5 * rho * (vel * vel)) * (gamma - 1.0), FLOOR)
    return np.vstack((rho, vel, p))


def temperature_si(gamma, lam, u):
    """torchSolver.py:90-114 (kelvin, SI H2/O2 molar mass)."""
    prim = cons_to_prim_1d(u, gamma)
    rho = np.maximum(prim[0], FLOOR)
    molar = lam * (2.0 / 3.0) * 2.016 + lam * (1.0 / 3.0) * 32.0 + (1.0 - lam) * 18.016
    return (prim[2] * molar) / (rho * 8314.46)


SI_CHEMISTRY = dict(q_heat=141584000.0, activation_energy=17.15 * 4184.0,
                    pre_exponential=1.76e5)


def react_1d(lam, dt, u, model="arrhenius", beta=None, *, q_heat=141584000.0,
             activation_energy=17.15 * 4184.0, pre_exponential=1.76e5,
             closure="si", gamma=None):
    """Exponential-midpoint Arrhenius / two-stage ZND source on a (3, n)
    state (torchSolver.py:708-789).

    closure='si' is the reference closure: gamma(lambda), T = p M / (rho R_u),
    rate = A exp(-Ea / (8.314 T)).  closure='nondimensional' restates the same
    integrator with T = p / rho at the constant ``gamma`` and
    rate = A exp(-activation_energy / T) (activation_energy is Ea/R); this
    closure has no reference counterpart (parity unpinned).
    """
    if model not in ("arrhenius", "znd"):
        raise ValueError(f"Unknown kinetic model: {model}")
    if (not np.isfinite([dt, q_heat, activation_energy, pre_exponential]).all()
            or min(dt, q_heat, activation_energy, pre_exponential) < 0):
        raise ValueError("Reaction time and constants must be finite and nonnegative")
    lam = np.asarray(lam, dtype=float)
    if np.any(~np.isfinite(lam)) or np.any((lam < 0) | (lam > 1)):
        raise ValueError("Reactant fraction must lie in [0,1]")
    u = np.asarray(u, dtype=float)
    if u.shape != (3, lam.size) or lam.ndim != 1 or not physical(u):
        raise ValueError("Reaction requires a physical (3,n) state and an (n,) reactant fraction")
    beta_n = np.ones_like(lam) if beta is None else np.asarray(beta, dtype=float)
    if (beta_n.shape != lam.shape or not np.isfinite(beta_n).all()
            or np.any((beta_n < 0) | (beta_n > 1))):
        raise ValueError("Induction fraction must have one value in [0,1] per cell")

    def rate_at(lam_now, state):
        if closure == "si":
            t = np.maximum(temperature_si(gamma_of_lambda(lam_now), lam_now, state), FLOOR)
            return pre_exponential * np.exp(-activation_energy / (8.314 * t))
        prim = cons_to_prim_1d(state, gamma)
        t = np.maximum(prim[2] / prim[0], FLOOR)
        return pre_exponential * np.exp(-activation_energy / t)

    def advance(rate, duration):
        if model == "znd":
            active = np.maximum(0.0, duration - beta_n / np.maximum(rate, 1e-300))
            lam_new = lam * np.exp(-5.0 * rate * active)
            beta_new = np.clip(beta_n - rate * duration, 0.0, 1.0)
        else:
            lam_new = lam * np.exp(-rate * duration)
            beta_new = np.zeros_like(beta_n)
        state = np.copy(u)
        state[2] += q_heat * state[0] * (lam - lam_new)
        return lam_new, state, beta_new

    lam_mid, state_mid, _ = advance(rate_at(lam, u), 0.5 * dt)
    return advance(rate_at(lam_mid, state_mid), dt)


def reaction_nd(state, lam, beta, dt, model="arrhenius", **chem):
    """reaction_step_2d / reaction_step_3d (torchSolver2D.py:474-509,
    torchSolver3D.py:225-243): move the transverse kinetic energy out of E,
    react the 1D state, put the energy change back."""
    dim = state.ndim - 1
    nv = dim + 2
    flat = state.reshape(nv, -1)
    if dim == 3:
        e_normal = flat[4] - 0.5 * _sqsum(flat[2:4]) / flat[0]
    else:
        e_normal = flat[3] - 0.5 * (flat[2] * flat[2]) / flat[0]
    normal = np.stack((flat[0], flat[1], e_normal))
    lam_new, reacted, beta_new = react_1d(
        lam.ravel(), dt, normal, model, None if beta is None else beta.ravel(), **chem)
    result = np.array(state, dtype=float, copy=True)
    result[-1] += (reacted[2] - normal[2]).reshape(lam.shape)
    return (result, lam_new.reshape(lam.shape),
            None if beta is None else beta_new.reshape(lam.shape))


def advect_3d(q, old, new, fluxes, dt, spacing, bcs_xyz):
    """First-order upwind species transport with the hydro mass flux
    (torchSolver3D.py:246-256)."""
    bcs = [bc_code(b) if isinstance(b, str) else b for b in bcs_xyz]
    qp = pad(q, bcs, 2, False)
    rhoq = old[0] * q
    for flux, h, axis in zip(fluxes, spacing, (3, 2, 1)):
        left, right = _faces_3d(qp[None], axis, False)
        scalar_flux = flux[0] * np.where(flux[0] >= 0, left[0], right[0])
        rhoq -= dt / h * np.diff(scalar_flux, axis=axis - 1)
    fraction = rhoq / new[0]
    if np.any(fraction < -1e-10) or np.any(fraction > 1 + 1e-10):
        raise RuntimeError("3D scalar transport left the physical interval")
    return np.clip(fraction, 0, 1)


def advect_2d(q, old, new, mass_x, mass_y, dt_dx, dt_dy, bc_x, bc_y):
    """torchSolver2D.py:659-667."""
    padded = pad_scalar_2d(q, bc_x, bc_y)
    fx = mass_x * np.where(mass_x >= 0, padded[2:-2, 1:-2], padded[2:-2, 2:-1])
    fy = mass_y * np.where(mass_y >= 0, padded[1:-2, 2:-2], padded[2:-1, 2:-2])
    rho_q = old[0] * q - dt_dx * np.diff(fx, axis=1) - dt_dy * np.diff(fy, axis=0)
    return np.clip(rho_q / np.maximum(new[0], FLOOR), 0.0, 1.0)


# ---------------------------------------------------------------------------
# 1D chain (session 1D step)
# ---------------------------------------------------------------------------

def bc_1d(u, bc):
    """One ghost cell each side (torchSolver.py:164-186)."""
    if bc == "Reflective":
        left = np.array([[u[0, 0]], [-u[1, 0]], [u[2, 0]]])
        right = np.array([[u[0, -1]], [-u[1, -1]], [u[2, -1]]])
    elif bc == "Periodic":
        left, right = u[:, -1:], u[:, :1]
    elif bc == "Open":
        left, right = u[:, :1], u[:, -1:]
    else:
        raise ValueError(f"Unknown boundary condition option: {bc}")
    return np.hstack((left, u, right))


def scalar_bc_1d(q, bc):
    """torchSolver.py:1121-1122."""
    return np.pad(q, 1, mode="wrap" if bc == "Periodic" else "edge")


def sound_1d(prim, gamma):
    """torchSolver.py:81-87 (pressure floor 0)."""
    return np.sqrt(gamma * np.maximum(prim[2], 0.0) / np.maximum(prim[0], FLOOR))


def flux_1d(u, gamma):
    """u_to_fu_calc (torchSolver.py:145-156)."""
    prim = cons_to_prim_1d(u, gamma)
    return np.vstack((prim[0] * prim[1], prim[0] * (prim[1] * prim[1]) + prim[2],
                      prim[1] * (u[2] + prim[2])))


def _nan0(a):
    a = np.array(a, dtype=float, copy=True)
    a[~np.isfinite(a)] = 0.0
    return a


def _split_gamma(gamma):
    if np.isscalar(gamma):
        return gamma, gamma
    return gamma[:-1], gamma[1:]


def waves_1d(u_bc, gamma, option="Pressure Based"):
    """Interface wave speeds S_L, S_*, S_R (torchSolver.py:283-404)."""
    gl, gr = _split_gamma(gamma)
    with np.errstate(divide="ignore", invalid="ignore"):
        pl_ = cons_to_prim_1d(u_bc[:, :-1], gl)
        rho_l = np.maximum(pl_[0], FLOOR)
        u_l, p_l = pl_[1], pl_[2]
        a_l = sound_1d(pl_, gl)
        e_l_tot = rho_l * (0.5 * (u_l * u_l) + p_l / ((gl - 1.0) * rho_l))
        pr_ = cons_to_prim_1d(u_bc[:, 1:], gr)
        rho_r = np.maximum(pr_[0], FLOOR)
        u_r, p_r = pr_[1], pr_[2]
        a_r = sound_1d(pr_, gr)
        e_r_tot = rho_r * (0.5 * (u_r * u_r) + p_r / ((gr - 1.0) * rho_r))
    if option == "Pressure Based":
        full = cons_to_prim_1d(u_bc, gamma)
        fl_, fr_ = full[:, :-1], full[:, 1:]
        rho_avg = 0.5 * (fr_[0] + fl_[0])
        a_avg = 0.5 * (sound_1d(fl_, gl) + sound_1d(fr_, gr))
        p_s = np.maximum(0.0, 0.5 * (fl_[2] + fr_[2])
                         - 0.5 * (fr_[1] - fl_[1]) * rho_avg * a_avg)
        q_l = np.ones_like(p_s)
        q_r = np.ones_like(p_s)
        ml, mr = p_s > p_l, p_s > p_r
        g_l = gl[ml] if isinstance(gl, np.ndarray) else gl
        g_r = gr[mr] if isinstance(gr, np.ndarray) else gr
        with np.errstate(divide="ignore", invalid="ignore"):
            q_l[ml] = np.sqrt(1.0 + (g_l + 1.0) / (2.0 * g_l) * (p_s[ml] / p_l[ml] - 1.0))
            q_r[mr] = np.sqrt(1.0 + (g_r + 1.0) / (2.0 * g_r) * (p_s[mr] / p_r[mr] - 1.0))
        s_l = u_l - a_l * q_l
        s_r = u_r + a_r * q_r
    elif option == "Enthalpy Based":
        with np.errstate(divide="ignore", invalid="ignore"):
            sq_l, sq_r = np.sqrt(rho_l), np.sqrt(rho_r)
            den = np.maximum(sq_l + sq_r, FLOOR)
            u_avg = (sq_l * u_l + sq_r * u_r) / den
            h_avg = (sq_l * ((e_l_tot + p_l) / rho_l) + sq_r * ((e_r_tot + p_r) / rho_r)) / den
            g_avg = 0.5 * (gl + gr) if isinstance(gl, np.ndarray) else gl
            a_avg = np.sqrt(np.maximum((g_avg - 1.0) * (h_avg - 0.5 * (u_avg * u_avg)), 1e-10))
        s_l = np.minimum(u_l - a_l, u_avg - a_avg)
        s_r = np.maximum(u_r + a_r, u_avg + a_avg)
    else:
        raise ValueError(f"Unknown wave speed calculation option: {option}")
    den = rho_l * (s_l - u_l) - rho_r * (s_r - u_r)
    den = np.where(np.abs(den) < GUARD, GUARD, den)
    s_s = (p_r - p_l + rho_l * u_l * (s_l - u_l) - rho_r * u_r * (s_r - u_r)) / den
    s_s = np.clip(s_s, s_l, s_r)
    return np.vstack((s_l, s_s, s_r))


def limit_1d(delta, di_uw, di_dw, w, limiter):
    """Sweby-bounded limited slope (torchSolver.py:201-275)."""
    with np.errstate(divide="ignore", invalid="ignore"):
        r = _nan0(di_uw / di_dw)
        denom = 1.0 - w + (1.0 + w) * r
        eps_r = _nan0(2.0 / np.where(np.abs(denom) < FLOOR, FLOOR, denom))
        eps = np.zeros_like(delta)
        pos = r > 0
        if limiter == "VanLeer":
            val = _nan0((2.0 * r) / (1.0 + r))
            eps[pos] = np.minimum(val[pos], eps_r[pos])
        elif limiter == "Albada":
            val = _nan0((r * (1.0 + r)) / (1.0 + r * r))
            eps[pos] = np.minimum(val[pos], eps_r[pos])
        elif limiter == "MINBEE":
            p1 = (r > 0) & (r < 1.0)
            p2 = r >= 1.0
            eps[p1] = r[p1]
            eps[p2] = np.minimum(1.0, eps_r[p2])
        elif limiter == "Superbee":
            val = _nan0(np.maximum(0.0, np.maximum(np.minimum(2.0 * r, 1.0),
                                                   np.minimum(r, 2.0))))
            eps[pos] = np.minimum(val[pos], eps_r[pos])
        elif limiter == "Unos":
            eps = np.minimum(np.maximum(0.0, np.minimum(np.minimum(2.0, 2.0 * r),
                                                        (2.0 + r) / 3.0)), eps_r)
        else:
            raise ValueError(f"Unknown slope limiter option: {limiter}")
    eps = np.maximum(0.0, _nan0(eps))
    slope = eps * delta
    bound = 2.0 * np.minimum(np.abs(di_uw), np.abs(di_dw))
    return np.where(di_uw * di_dw > 0, np.sign(di_dw) * np.minimum(np.abs(slope), bound), 0.0)


def reconstruct_1d(u_bc, dt, dx, gamma, limiter, controller):
    """MUSCL + half-step predictor, interleaved [l0, r0, l1, r1, ...]
    (torchSolver.py:412-491)."""
    inner, left, right = u_bc[:, 1:-1], u_bc[:, :-2], u_bc[:, 2:]
    delta = 0.5 * (right - left)
    di_uw = inner - left
    di_dw = right - inner
    g_in = gamma if np.isscalar(gamma) else gamma[1:-1]
    if controller == "Sound Speed Controlled":
        prim = cons_to_prim_1d(inner, g_in)
        a = sound_1d(prim, g_in)
        with np.errstate(divide="ignore", invalid="ignore"):
            mach = np.abs(prim[1]) / np.maximum(a, FLOOR)
        mach[~np.isfinite(mach)] = 0.0
        w = np.clip((1.0 - mach) / (1.0 + mach), -1.0, 1.0)
    elif controller == "w=0":
        w = np.zeros(inner.shape[1])
    else:
        raise ValueError(f"Unknown w_controler option: {controller}")
    lim = limit_1d(delta, di_uw, di_dw, w, limiter)
    u_l = inner - 0.5 * lim
    u_r = inner + 0.5 * lim
    d_fu = -(dt / (2.0 * dx)) * (flux_1d(u_r, g_in) - flux_1d(u_l, g_in))
    out_l = u_l + d_fu
    out_r = u_r + d_fu
    for s in (out_l, out_r):
        p = (g_in - 1.0) * (s[2] - 0.5 * (s[1] * s[1]) / np.maximum(s[0], FLOOR))
        bad = (s[0] <= FLOOR) | (p <= FLOOR) | ~np.isfinite(s).all(axis=0)
        s[:, bad] = inner[:, bad]
    sub = np.empty((3, 2 * inner.shape[1]))
    sub[:, 0::2] = out_l
    sub[:, 1::2] = out_r
    return sub


def hllc_1d(u_sub_bc, waves, gamma, variant="Variante 1 - Original"):
    """HLLC with precomputed wave speeds (torchSolver.py:534-676)."""
    n = waves.shape[1]
    u_l, u_r = u_sub_bc[:, 0::2], u_sub_bc[:, 1::2]
    gl, gr = _split_gamma(gamma)
    pl_ = cons_to_prim_1d(u_l, gl)
    rho_l = np.maximum(pl_[0], FLOOR)
    v_l, p_l = pl_[1], pl_[2]
    e_l_tot = rho_l * (0.5 * (v_l * v_l) + p_l / ((gl - 1.0) * rho_l))
    pr_ = cons_to_prim_1d(u_r, gr)
    rho_r = np.maximum(pr_[0], FLOOR)
    v_r, p_r = pr_[1], pr_[2]
    e_r_tot = rho_r * (0.5 * (v_r * v_r) + p_r / ((gr - 1.0) * rho_r))
    f_l, f_r = flux_1d(u_l, gl), flux_1d(u_r, gr)
    s_l, s_r = waves[0], waves[2]
    den = rho_l * (s_l - v_l) - rho_r * (s_r - v_r)
    den = np.where(abs(den) < GUARD, GUARD, den)
    s_s = np.clip((p_r - p_l + rho_l * v_l * (s_l - v_l) - rho_r * v_r * (s_r - v_r)) / den,
                  s_l, s_r)
    eps = 1e-12
    if variant == "Variante 1 - Original":
        ok_l = np.abs(s_l - s_s) > eps
        ok_r = np.abs(s_r - s_s) > eps
        d_l = np.where(ok_l, s_l - s_s, -eps)
        d_r = np.where(ok_r, s_r - s_s, eps)
        du_l = np.where(np.abs(s_l - v_l) < eps, -eps, s_l - v_l)
        du_r = np.where(np.abs(s_r - v_r) < eps, eps, s_r - v_r)
        t_l = e_l_tot / rho_l + (s_s - v_l) * (s_s + p_l / (rho_l * du_l))
        t_r = e_r_tot / rho_r + (s_s - v_r) * (s_s + p_r / (rho_r * du_r))
        star_l = rho_l * ((s_l - v_l) / d_l) * np.vstack((np.ones(n), s_s, t_l))
        star_l[:, ~ok_l] = u_l[:, ~ok_l]
        star_r = rho_r * ((s_r - v_r) / d_r) * np.vstack((np.ones(n), s_s, t_r))
        star_r[:, ~ok_r] = u_r[:, ~ok_r]
        f_ls = f_l + s_l * (star_l - u_l)
        f_rs = f_r + s_r * (star_r - u_r)
    elif variant == "Variante_2":
        d_s = np.vstack((np.zeros(n), np.ones(n), s_s))
        d_l = np.where(np.abs(s_l - s_s) < eps, np.sign(s_l - s_s + 1e-30) * eps, s_l - s_s)
        d_r = np.where(np.abs(s_r - s_s) < eps, np.sign(s_r - s_s + 1e-30) * eps, s_r - s_s)
        f_ls = (s_s * (s_l * u_l - f_l)
                + s_l * (p_l + rho_l * (s_l - v_l) * (s_s - v_l)) * d_s) / d_l
        f_rs = (s_s * (s_r * u_r - f_r)
                + s_r * (p_r + rho_r * (s_r - v_r) * (s_s - v_r)) * d_s) / d_r
    else:
        raise ValueError(f"Unknown HLLC variant: {variant}")
    out = np.zeros((3, n))
    for mask, value in ((s_l > 0, f_l), ((s_l <= 0) & (s_s > 0), f_ls),
                        ((s_s <= 0) & (s_r >= 0), f_rs), (s_r < 0, f_r)):
        out[:, mask] = value[:, mask]
    return out


def update_1d(u_bc, flux, dt, dx, gamma):
    """Conservative update with the Rusanov fallback (torchSolver.py:692-700,
    1054-1071).  Returns (state, flux, used_fallback)."""
    cand = u_bc[:, 1:-1] + (-(dt / dx) * (flux[:, 1:] - flux[:, :-1]))
    used = False
    if not physical(cand):
        used = True
        prim = cons_to_prim_1d(u_bc, gamma)
        speed = np.abs(prim[1]) + sound_1d(prim, gamma)
        alpha = np.maximum(speed[:-1], speed[1:])
        pf = flux_1d(u_bc, gamma)
        flux = 0.5 * (pf[:, :-1] + pf[:, 1:] - alpha * np.diff(u_bc))
        cand = u_bc[:, 1:-1] + (-(dt / dx) * (flux[:, 1:] - flux[:, :-1]))
    if not physical(cand):
        raise RuntimeError("Hydrodynamic update produced a nonphysical state")
    return cand, flux, used


def dt_1d(state, gamma, dx, cfl, bc, wavespeed="Pressure Based"):
    """Session 1D dt (torchSession.py:338-345; torchSolver.py:684-689,1049-1051)."""
    padded = bc_1d(state, bc)
    gp = gamma if np.isscalar(gamma) else scalar_bc_1d(gamma, bc)
    waves = waves_1d(padded, gp, wavespeed)
    mw = np.max(np.abs(waves))
    dt_w = (cfl * dx) / mw if mw > 0 else 1e-6
    prim = cons_to_prim_1d(padded, gp)
    dt_h = cfl * dx / np.max(np.abs(prim[1]) + sound_1d(prim, gp))
    return min(dt_w, dt_h)


def step_1d(state, dt, dx, gamma, cfl, limiter, controller, variant, wavespeed, bc):
    """Session 1D hydro chain (torchSession.py:413-437)."""
    padded = bc_1d(state, bc)
    gp = gamma if np.isscalar(gamma) else scalar_bc_1d(gamma, bc)
    waves = waves_1d(padded, gp, wavespeed)
    recon = bc_1d(reconstruct_1d(padded, dt, dx, gp, limiter, controller), bc)
    flux = hllc_1d(recon, waves, gp, variant)
    return update_1d(padded, flux, dt, dx, gp)


def advect_1d(q, old, new, mass_flux, dt_dx, bc):
    """torchSolver.py:1125-1132."""
    padded = scalar_bc_1d(q, bc)
    flux = mass_flux * np.where(mass_flux >= 0, padded[:-1], padded[1:])
    rho_q = old[0] * q - dt_dx * np.diff(flux)
    return np.clip(rho_q / np.maximum(new[0], FLOOR), 0.0, 1.0)
