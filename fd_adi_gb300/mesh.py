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
