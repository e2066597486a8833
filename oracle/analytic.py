"""Closed-form and semi-analytic prices (test infrastructure only).

* ``bs_call``: Black-Scholes call and delta, FiniteDifference/blackscholes.py:42-58.
* ``heston_cos``: the Fang-Oosterlee COS price of a Heston call as the reference's
  ``HestonCos`` computes it (FiniteDifference/heston.py:490-693): N = 256 cosine
  terms, truncation L = 12 on the cumulants c1, c2 (heston.py:643-666), half
  weight on the k = 0 term (:684), K exp(-rT) scaling and clipping at 0
  (:691-693). The reference evaluates it with numexpr; this is plain numpy.
"""
import numpy as np
from scipy.stats import norm


def bs_call(spot, strike, r, var, T):
    s = np.asarray(spot, dtype=float)
    vol = np.maximum(1e-10, np.sqrt(var))
    if T == 0:
        d1 = np.inf
    else:
        s = s + np.finfo(np.atleast_1d(s).dtype).tiny
        d1 = (np.log(s / float(strike)) + (r + 0.5 * vol ** 2) * T) / (vol * np.sqrt(T))
    d2 = d1 - vol * np.sqrt(T)
    return norm.cdf(d1) * s - norm.cdf(d2) * strike * np.exp(-r * T), norm.cdf(d1)


def _xi(k, a, b, c, d):
    kp = k * np.pi / (b - a)
    caba = (c - a) * kp
    daba = (d - a) * kp
    return (((np.cos(daba) + kp * np.sin(daba)) * np.exp(d)
             - (np.cos(caba) + kp * np.sin(caba)) * np.exp(c)) / (1 + kp ** 2))


def _psi(k, a, b, c, d):
    b_a = b - a
    kpi = k * np.pi
    with np.errstate(divide="ignore", invalid="ignore"):
        kp = kpi / b_a
        ret = (np.sin((d - a) * kp) - np.sin((c - a) * kp)) * b_a / kpi
    return np.concatenate([np.broadcast_to(d - c, ret[..., :1].shape), ret[..., 1:]], axis=-1)


def _cf(omega, r, var, T, kappa, theta, sigma, rho):
    p10 = kappa - (1j * rho * sigma) * omega
    D = np.sqrt(p10 ** 2 + (omega ** 2 + 1j * omega) * sigma ** 2)
    p1p = p10 + D
    p1m = p10 - D
    G = p1m / p1p
    p0 = np.exp(-D * T)
    p2 = 1 - G * p0
    return (np.exp(1j * omega * r * T + var / sigma ** 2 * ((1 - p0) / p2) * p1m)
            * np.exp((kappa * theta) / sigma ** 2 * (T * p1m - 2 * np.log(p2 / (1 - G)))))


def heston_cos(spot, strike, r, variance, T, kappa, theta, sigma, rho, N=256):
    """Heston call price(s); ``spot`` and ``variance`` may be arrays (result
    shape [len(spot), len(variance)])."""
    S = np.atleast_1d(np.asarray(spot, dtype=float))
    var = np.atleast_1d(np.asarray(variance, dtype=float))
    K = float(strike)
    L = 12
    x = np.log(S / K)[np.newaxis, :, np.newaxis]
    var = var[:, np.newaxis, np.newaxis]
    vt = var - theta
    e1 = np.exp(-kappa * T)
    p1 = (sigma * T * kappa * e1 * (8 * kappa * rho - 4 * sigma)) * vt
    p2 = (kappa * rho * sigma * (1 - e1) * 8) * (-vt + var)
    p3 = 2 * theta * kappa * T * (-4 * kappa * rho * sigma + sigma ** 2 + 4 * kappa ** 2)
    p4 = sigma ** 2 * ((-vt - var) * np.exp(-2 * kappa * T) + theta * (6 * e1 - 7) + 2 * var)
    p5 = (8 * kappa ** 2 * (1 - e1)) * vt
    c2 = 0.125 * kappa ** (-3) * (p1 + p2 + p3 + p4 + p5)
    c1 = r * T + (-vt) * (1 - e1) / (2 * kappa) - 0.5 * theta * T
    Lc2 = L * np.sqrt(np.abs(c2))
    a = x + c1 - Lc2
    b = x + c1 + Lc2
    k = np.arange(N)[np.newaxis, np.newaxis, :]
    U = 2. / (b - a) * (_xi(k, a, b, 0, b) - _psi(k, a, b, 0, b))
    cf = _cf(k * np.pi / (b - a), r, var, T, kappa, theta, sigma, rho)
    cf[:, :, 0] *= 0.5
    ret = ((cf * np.exp(1j * k * np.pi * (x - a) / (b - a))) * U).real
    ret = K * np.exp(-r * T) * ret.sum(axis=-1)
    ret[np.isnan(ret)] = 0
    return np.maximum(0, ret).T
