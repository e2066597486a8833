"""Non-uniform meshes for the spot and variance axes.

Host-side, once per engine, as in the reference (FiniteDifference/utils.py).
Both generators return float64 numpy arrays that the engines upload once.
"""
from bisect import bisect_left

import numpy as np
import scipy.optimize


def sinh_space(exact, high, density, size, force_exact=True):
    """Sigmoidal mesh on [0, ~high] clustered around ``exact``.

    Follows FiniteDifference/utils.py:102-147: points K + c*sinh(eps) on a
    uniform eps grid, shifted so the first point is 0; the upper end is nudged
    within [0.95, 1.05]*high by a bounded scalar minimisation (scipy's
    ``fminbound``, as the reference) so a point lands close to ``exact``, which
    is then forced onto the mesh exactly.
    """
    density = float(density)
    if size == 1:
        return np.asarray(exact)

    def newspace(hi):
        deps = 1.0 / size * (np.arcsinh((hi - exact) * (1 / density))
                             - np.arcsinh(-exact / density))
        eps = np.arcsinh(-exact / density) + np.arange(size) * deps
        space = exact + density * np.sinh(eps)
        space -= min(space)
        return space

    def energy(hi):
        space = newspace(hi)
        try:
            best = space[bisect_left(space, exact)]
        except IndexError:
            best = space[-2]
        return abs(exact - best)

    newmax, _, failed, _ = scipy.optimize.fminbound(energy, high * 0.95, high * 1.05,
                                                    full_output=True)
    if failed:
        raise ValueError("Unable to create a suitable space. %s\n%s"
                         % ((exact, high, density, size), newmax))
    space = newspace(newmax)
    if force_exact:
        idx = bisect_left(space, exact)
        if idx < space.size:
            space[idx] = exact
    return space


def exponential_space(low, exact, high, ex, size, force_exact=True):
    """Mesh v_i = l + (i*dv)**ex with ``exact`` forced onto a point.

    Follows FiniteDifference/utils.py:161-190: the upper end is stretched so
    that the last grid point below ``exact`` (in the ex-th root coordinates)
    hits it exactly.
    """
    if size == 1:
        return np.array([exact])
    v = np.zeros(size)
    lo = pow(low, 1. / ex)
    h = pow(high, 1. / ex)
    x = pow(exact, 1. / ex)
    dv = (h - lo) / (size - 1)
    if force_exact:
        j = 0
        for i in range(size):
            if lo + i * dv > x:
                j = i - 1
                break
        if j == 0:
            raise ValueError("Did not find suitable value.")
        dx = x - (lo + j * dv)
        h += (size - 1) * dx / j
    dv = (h - lo) / (size - 1)
    for i in range(size):
        v[i] = lo + pow(i * dv, ex)
    return v


def heston_meshes(spot, strike, variance, nspots, nvols, spot_max, var_max,
                  spotdensity=7.0, varexp=4.0, spot_min=0.0, force_exact=True):
    """Spot and variance meshes of the reference Heston engines.

    FiniteDifference/heston.py:384-406 and FiniteDifferenceEngineGPU.pyx:662-686:
    variance from ``exponential_space(0, v0, var_max, varexp, nvols)``, spot from
    ``sinh_space(K - spot_min, spot_max - spot_min, spotdensity, nspots) + spot_min``
    and the grid point nearest the spot is moved onto the spot.
    """
    vars_ = exponential_space(0.0, variance, var_max, varexp, nvols, force_exact=force_exact)
    spots = sinh_space(strike - spot_min, spot_max - spot_min, spotdensity, nspots,
                       force_exact=force_exact) + spot_min
    spots = np.array(spots, dtype=np.float64)
    spots[np.argmin(np.abs(spots - spot))] = spot
    return spots, np.array(vars_, dtype=np.float64)


# ---- many options at once ---------------------------------------------------
#
# The functions below build the meshes of a whole batch of Heston engines in
# one pass and give, element for element, the same doubles as the per-option
# generators above: every value goes through the same numpy ufuncs (arcsinh,
# sinh) or the same C library pow() with the same operands in the same order,
# only over many options at once. The spot mesh's bounded minimisation runs
# for all options in lockstep, each with its own state.

_SQRT_EPS = np.sqrt(2.2e-16)
_GOLDEN = 0.5 * (3.0 - np.sqrt(5.0))


def _sinh_space_energy(x, exact, density, size, a0):
    """sinh_space's energy(hi) for every option (x = hi): |exact - space[i]|
    with i = bisect_left(space, exact) (space[-2] when i == size), computed
    from the mesh points next to `exact` only. Returns (energy, ok); ok is
    False where the window of candidate points did not bracket `exact` (the
    caller evaluates the whole mesh there)."""
    deps = 1.0 / size * (np.arcsinh((x - exact) * (1 / density)) - a0)
    s0 = exact + density * np.sinh(a0)
    # first index whose point reaches exact, from the inverse map; the window
    # of candidates around it absorbs the rounding of the estimate
    est = np.ceil((np.arcsinh(s0 / density) - a0) / deps)
    est = np.clip(np.nan_to_num(est, nan=0.0, posinf=0.0, neginf=0.0), 0, size - 1)
    W = 3
    offs = np.arange(-W, W + 1)
    cand = est.astype(np.int64)[:, None] + offs[None, :]
    inside = (cand >= 0) & (cand < size[:, None])
    candc = np.where(inside, cand, 0)
    pts = (exact[:, None] + density[:, None] * np.sinh(a0[:, None] + candc * deps[:, None])) \
        - s0[:, None]
    reach = inside & (pts >= exact[:, None])
    anyr = reach.any(axis=1)
    first = np.argmax(reach, axis=1)
    idx = candc[np.arange(x.size), first]
    # the window must show a point below exact before the first one reaching
    # it (or start at index 0), and hold the last index when none reaches it
    lo_ok = (first > 0) | (idx == 0)
    top = np.where(inside, cand, -1).max(axis=1)
    ok = np.where(anyr, lo_ok, top == size - 1)
    best_in = pts[np.arange(x.size), first]
    # bisect_left == size: the reference takes space[-2]
    j2 = size - 2
    last = (exact + density * np.sinh(a0 + j2 * deps)) - s0
    best = np.where(anyr, best_in, last)
    return np.abs(exact - best), ok


def _sinh_space_flat(x, exact, density, size, a0):
    """sinh_space's newspace(hi) for every option, concatenated option after
    option; returns (space, opt, off) with opt the option of each point and
    off the options' start offsets."""
    deps = 1.0 / size * (np.arcsinh((x - exact) * (1 / density)) - a0)
    off = np.concatenate([[0], np.cumsum(size)[:-1]]).astype(np.int64)
    opt = np.repeat(np.arange(size.size), size)
    i = np.arange(opt.size, dtype=np.int64) - off[opt]
    space = exact[opt] + density[opt] * np.sinh(a0[opt] + i * deps[opt])
    space -= np.minimum.reduceat(space, off)[opt]
    return space, opt, off


def _energy_full(x, exact, density, size, a0):
    space, opt, off = _sinh_space_flat(x, exact, density, size, a0)
    idx = np.add.reduceat((space < exact[opt]).astype(np.int64), off)
    best = space[off + np.where(idx < size, idx, size - 2)]
    return np.abs(exact - best)


def sinh_space_batch(exact, high, density, size, force_exact=True, xatol=1e-5, maxiter=500):
    """sinh_space for many options: exact, high, density and size are arrays
    (or scalars broadcast to them). Returns the meshes concatenated option
    after option (size[k] points each); option k's equals
    sinh_space(exact[k], high[k], density[k], size[k]) bit for bit.

    The upper end of every mesh is found by the bounded minimisation the
    reference calls (scipy.optimize.fminbound: Brent's method with golden
    sections and parabolic steps, xatol = 1e-5, 500 evaluations at most),
    restated here over arrays so that all options take their steps together;
    an option stops when its own convergence test says so."""
    exact, high, density, size = np.broadcast_arrays(
        np.asarray(exact, np.float64), np.asarray(high, np.float64),
        np.asarray(density, np.float64), np.asarray(size, np.int64))
    exact, high, density, size = [np.array(a).reshape(-1) for a in (exact, high, density, size)]
    n = exact.size
    if n == 0:
        return np.zeros(0)
    if (size < 2).any():
        raise ValueError("sinh_space_batch: every mesh needs at least 2 points")
    a0 = np.arcsinh(-exact / density)

    def energy(x, rows):
        e, ok = _sinh_space_energy(x, exact[rows], density[rows], size[rows], a0[rows])
        if not ok.all():
            bad = ~ok
            r = rows[bad]
            e[bad] = _energy_full(x[bad], exact[r], density[r], size[r], a0[r])
        return e

    # scipy.optimize._optimize._minimize_scalar_bounded, per option
    a, b = high * 0.95, high * 1.05
    fulc = a + _GOLDEN * (b - a)
    nfc, xf = fulc.copy(), fulc.copy()
    rat = np.zeros(n)
    e = np.zeros(n)
    allrows = np.arange(n)
    fx = energy(xf, allrows)
    num = 1
    fu = np.full(n, np.inf)
    ffulc, fnfc = fx.copy(), fx.copy()
    xm = 0.5 * (a + b)
    tol1 = _SQRT_EPS * np.abs(xf) + xatol / 3.0
    tol2 = 2.0 * tol1
    flag = np.zeros(n, dtype=np.int32)
    active = np.abs(xf - xm) > (tol2 - 0.5 * (b - a))
    with np.errstate(divide="ignore", invalid="ignore"):
        while active.any():
            r_ = np.nonzero(active)[0]
            A, B, XF, FX = a[r_], b[r_], xf[r_], fx[r_]
            NFC, FNFC, FULC, FFULC = nfc[r_], fnfc[r_], fulc[r_], ffulc[r_]
            E, RAT, XM, T1, T2 = e[r_], rat[r_], xm[r_], tol1[r_], tol2[r_]
            para = np.abs(E) > T1
            r = (XF - NFC) * (FX - FFULC)
            q = (XF - FULC) * (FX - FNFC)
            p = (XF - FULC) * q - (XF - NFC) * r
            q = 2.0 * (q - r)
            p = np.where(q > 0.0, -p, p)
            q = np.abs(q)
            r = E
            E_para = RAT
            accept = para & (np.abs(p) < np.abs(0.5 * q * r)) & (p > q * (A - XF)) & \
                (p < q * (B - XF))
            rat_p = (p + 0.0) / q
            x_p = XF + rat_p
            si = np.sign(XM - XF) + ((XM - XF) == 0)
            rat_p = np.where(((x_p - A) < T2) | ((B - x_p) < T2), T1 * si, rat_p)
            golden = ~accept
            E_gold = np.where(XF >= XM, A - XF, B - XF)
            E = np.where(golden, E_gold, E_para)
            RAT = np.where(golden, _GOLDEN * E_gold, rat_p)
            si = np.sign(RAT) + (RAT == 0)
            X = XF + si * np.maximum(np.abs(RAT), T1)
            FU = energy(X, r_)
            num += 1
            better = FU <= FX
            # fu <= fx
            A1 = np.where(X >= XF, XF, A)
            B1 = np.where(X >= XF, B, XF)
            # fu > fx
            A2 = np.where(X < XF, X, A)
            B2 = np.where(X < XF, B, X)
            c1 = (FU <= FNFC) | (NFC == XF)
            c2 = ~c1 & ((FU <= FFULC) | (FULC == XF) | (FULC == NFC))
            a[r_] = np.where(better, A1, A2)
            b[r_] = np.where(better, B1, B2)
            fulc[r_] = np.where(better | c1, NFC, np.where(c2, X, FULC))
            ffulc[r_] = np.where(better | c1, FNFC, np.where(c2, FU, FFULC))
            nfc[r_] = np.where(better, XF, np.where(c1, X, NFC))
            fnfc[r_] = np.where(better, FX, np.where(c1, FU, FNFC))
            xf[r_] = np.where(better, X, XF)
            fx[r_] = np.where(better, FU, FX)
            fu[r_] = FU
            e[r_] = E
            rat[r_] = RAT
            xm[r_] = 0.5 * (a[r_] + b[r_])
            tol1[r_] = _SQRT_EPS * np.abs(xf[r_]) + xatol / 3.0
            tol2[r_] = 2.0 * tol1[r_]
            if num >= maxiter:
                flag[r_] = 1
                break
            active[r_] = np.abs(xf[r_] - xm[r_]) > (tol2[r_] - 0.5 * (b[r_] - a[r_]))
    flag[np.isnan(xf) | np.isnan(fx) | np.isnan(fu)] = 2
    if flag.any():
        k = int(np.nonzero(flag)[0][0])
        raise ValueError("Unable to create a suitable space. %s\n%s"
                         % ((exact[k], high[k], density[k], int(size[k])), xf[k]))
    space, opt, off = _sinh_space_flat(xf, exact, density, size, a0)
    if force_exact:
        idx = np.add.reduceat((space < exact[opt]).astype(np.int64), off)
        rows = np.nonzero(idx < size)[0]
        space[off[rows] + idx[rows]] = exact[rows]
    return space


def heston_meshes_batch(spot, strike, variance, nspots, nvols, spot_max, var_max,
                        spotdensity=7.0, varexp=4.0, spot_min=0.0, threads=0):
    """heston_meshes for n options at once: spot, strike, variance, nspots,
    nvols and spot_max are arrays (or scalars). Returns (spots, vars) as flat
    float64 arrays, option after option (the batch arena's order), each
    option's mesh bit-identical to heston_meshes(...) for it. The variance
    meshes come from the library's host generator (C pow(), the call Python's
    float ** makes), the spot meshes from sinh_space_batch."""
    from . import _lib
    spot, strike, variance, nspots, nvols, spot_max = np.broadcast_arrays(
        np.asarray(spot, np.float64), np.asarray(strike, np.float64),
        np.asarray(variance, np.float64), np.asarray(nspots, np.int64),
        np.asarray(nvols, np.int64), np.asarray(spot_max, np.float64))
    spot, strike, variance, nspots, nvols, spot_max = [
        np.array(a).reshape(-1) for a in (spot, strike, variance, nspots, nvols, spot_max)]
    n = spot.size
    nv32 = np.ascontiguousarray(nvols, dtype=np.int32)
    v0 = np.ascontiguousarray(variance)
    vars_ = np.empty(int(nvols.sum()), dtype=np.float64)
    _lib.call("fdadi_heston_var_meshes", n, v0.ctypes.data, nv32.ctypes.data, float(var_max),
              float(varexp), 1, int(threads), vars_.ctypes.data)
    space = sinh_space_batch(strike - spot_min, spot_max - spot_min, float(spotdensity), nspots)
    space = space + spot_min
    # the grid point nearest the spot is moved onto the spot (first of ties)
    off = np.concatenate([[0], np.cumsum(nspots)[:-1]]).astype(np.int64)
    opt = np.repeat(np.arange(n), nspots)
    far = np.abs(space - spot[opt])
    near = far == np.minimum.reduceat(far, off)[opt]
    pos = np.where(near, np.arange(space.size), space.size)
    space[np.minimum.reduceat(pos, off)] = spot
    return space, vars_


def price_index_batch(spots, vars_, nspots, nvols, spot, variance):
    """price_index for every option of flat concatenated meshes: arena
    offsets (i * nv + j) within each option, by the same rounded bisection."""
    nspots = np.asarray(nspots, np.int64)
    nvols = np.asarray(nvols, np.int64)
    so = np.concatenate([[0], np.cumsum(nspots)])
    vo = np.concatenate([[0], np.cumsum(nvols)])
    spot = np.broadcast_to(np.asarray(spot, np.float64), nspots.shape)
    variance = np.broadcast_to(np.asarray(variance, np.float64), nspots.shape)
    rs = np.round(spots, decimals=4)
    rv = np.round(vars_, decimals=4)
    ts = np.round(spot, decimals=4)
    tv = np.round(variance, decimals=4)
    opt_s = np.repeat(np.arange(nspots.size), nspots)
    opt_v = np.repeat(np.arange(nvols.size), nvols)
    ids = np.bincount(opt_s, weights=(rs < ts[opt_s]), minlength=nspots.size).astype(np.int64)
    idv = np.bincount(opt_v, weights=(rv < tv[opt_v]), minlength=nvols.size).astype(np.int64)
    return ids * nvols + idv


def barrier_spots(strike, barrier, nspots, force_exact=True):
    """Spot mesh of the up-and-out engine: exponential_space(0, K, barrier, 1/3, n)
    (FiniteDifferenceEngineGPU.pyx:670-678)."""
    return exponential_space(0.0, strike, barrier, 1.0 / 3, nspots, force_exact=force_exact)


def price_index(spots, vars_, spot, variance):
    """Grid index of (spot, variance): bisect on meshes rounded to 4 decimals
    (FiniteDifferenceEngineGPU.pyx:727-734, heston.py:461-465)."""
    ids = bisect_left(list(np.round(spots, decimals=4)), np.round(spot, decimals=4))
    idv = bisect_left(list(np.round(vars_, decimals=4)), np.round(variance, decimals=4))
    return ids, idv
