"""Laplace quadrature of the orbital-energy denominator (minimax fit).

    1/y ~ sum_{t=1..k} w_t exp(-a_t y),   y in [ymin, ymax]

megalochem obtains (a_t, w_t) from a Fortran minimax library
(src/math/laplace/minimax.hpp:75-92, src/math/laplace/src/laplace_minimax.F90)
that implements the Remez algorithm of Takatsuka, Ten-no and Hackbusch
(J. Chem. Phys. 129, 044112 (2008)) with Newton-Maehly extremum search
(Helmich-Paris and Visscher, J. Comput. Phys. 321, 927 (2016)).  This module
restates that published algorithm in FP64:

  * scale to x = y / ymin in [1, R], R = ymax / ymin;
  * the best approximation g(x) = sum_t w_t exp(-a_t x) of 1/x in the
    maximum norm makes the error eta = g - 1/x equioscillate on 2k+1 points
    1 = x_0 < x_1 < ... < x_2k = R:  eta(x_i) = (-1)^i E;
  * Remez: locate the 2k-1 interior extrema of eta for the current
    parameters, then solve the 2k+1 equations eta(x_i) = (-1)^i E for
    (w, a, E) by a damped Newton iteration; repeat until the extremal
    errors are level;
  * start values: the library reads tabulated parameters; here a sinc
    quadrature of 1/x = int exp(s - x e^s) ds refined by least squares,
    continued in R from a short interval when needed.
The result is scaled back: a_t / ymin, w_t / ymin.  The Laplace interval is
[2(e_lumo - e_homo), 2(e_max - e_min)] (src/mp/mp_compute.cpp:64-69).
"""
from __future__ import annotations

import numpy as np
from scipy.optimize import brentq, least_squares


def _eta(x, w, a):
    return np.exp(-np.outer(x, a)) @ w - 1.0 / x


def _deta(x, w, a):
    return -(np.exp(-np.outer(x, a)) * a) @ w + 1.0 / (x * x)


def _extrema(w, a, R, ngrid=4000):
    """Alternation set of eta: the end points and the interior extrema (sign
    changes of eta' on a log grid, refined by Brent's method); runs of equal
    sign keep their largest |eta|, and surplus points are dropped from the
    end with the smaller |eta| (the Remez exchange rule)."""
    k2 = 2 * len(w) + 1
    x = np.exp(np.linspace(0.0, np.log(R), ngrid))
    d = _deta(x, w, a)
    pts = [1.0]
    for i in np.nonzero(np.sign(d[:-1]) * np.sign(d[1:]) < 0)[0]:
        pts.append(brentq(lambda t: _deta(np.array([t]), w, a)[0], x[i], x[i + 1], xtol=1e-14 * x[i]))
    pts.append(R)
    pts = np.array(pts)
    e = _eta(pts, w, a)
    keep = [0]
    for i in range(1, len(pts)):
        j = keep[-1]
        if np.sign(e[i]) == np.sign(e[j]):
            if abs(e[i]) > abs(e[j]):
                keep[-1] = i
        else:
            keep.append(i)
    while len(keep) > k2:
        keep.pop(0 if abs(e[keep[0]]) < abs(e[keep[-1]]) else -1)
    return pts[keep]


def _newton(xs, w, a, E, iters=60):
    """Solve eta(x_i) = (-1)^i E, i = 0..2k, for (log w, log a, E)."""
    k = len(w)
    sgn = (-1.0) ** np.arange(len(xs))
    p = np.concatenate([np.log(w), np.log(a), [E]])

    def resid(p):
        ww, aa = np.exp(p[:k]), np.exp(p[k:2 * k])
        return _eta(xs, ww, aa) - sgn * p[-1]

    r = resid(p)
    for _ in range(iters):
        ww, aa = np.exp(p[:k]), np.exp(p[k:2 * k])
        ex = np.exp(-np.outer(xs, aa))
        Jm = np.empty((len(xs), 2 * k + 1))
        Jm[:, :k] = ex * ww                        # d/d log w
        Jm[:, k:2 * k] = -ex * ww * aa * xs[:, None]  # d/d log a
        Jm[:, -1] = -sgn
        step = np.linalg.lstsq(Jm, -r, rcond=None)[0]
        lam = 1.0
        n0 = np.linalg.norm(r)
        while lam > 1e-6:
            pn = p + lam * step
            rn = resid(pn)
            if np.all(np.isfinite(rn)) and np.linalg.norm(rn) < n0:
                break
            lam *= 0.5
        else:
            break
        p, r = pn, rn
        if np.linalg.norm(lam * step) < 1e-15 * (1 + np.linalg.norm(p)):
            break
    return np.exp(p[:k]), np.exp(p[k:2 * k]), p[-1]


def _max_error(w, a, R, xs):
    x = np.concatenate([xs, np.exp(np.linspace(0.0, np.log(R), 20000))])
    return float(np.max(np.abs(_eta(x, w, a))))


def _remez(w, a, R, xs=None, iters=60, tol=1e-10):
    """Remez iteration from (w, a); xs: a reference set to use while the
    current parameters do not yet show 2k+1 alternation points.  Returns
    (w, a, max error, alternation set) or None."""
    k = len(w)
    for _ in range(iters):
        cand = _extrema(w, a, R)
        if len(cand) == 2 * k + 1:
            xs = cand
            e = np.abs(_eta(xs, w, a))
            if (e.max() - e.min()) / e.max() < tol:
                break
        elif xs is None:
            return None
        e = _eta(xs, w, a)
        w, a, _ = _newton(xs, w, a, float(np.mean(np.abs(e)) * np.sign(e[0])))
        if not (np.all(np.isfinite(w)) and np.all(np.isfinite(a))):
            return None
    if len(_extrema(w, a, R)) != 2 * k + 1:
        return None
    return w, a, _max_error(w, a, R, xs), xs


def _start(k, R):
    """Sinc-quadrature start refined by least squares on a log grid."""
    lo, hi = -np.log(R) - 2.5, 2.0
    s = np.linspace(lo, hi, k)
    h = (hi - lo) / max(k - 1, 1)
    w, a = h * np.exp(s), np.exp(s)
    x = np.exp(np.linspace(0.0, np.log(R), 40 * k))

    def f(p):
        return _eta(x, np.exp(p[:k]), np.exp(p[k:]))

    p = least_squares(f, np.concatenate([np.log(w), np.log(a)]), xtol=1e-15, ftol=1e-15,
                      gtol=1e-15, max_nfev=4000).x
    return np.exp(p[:k]), np.exp(p[k:])


def minimax_unit(k, R):
    """Best k-term exponential sum for 1/x on [1, R] in the maximum norm:
    (w, a, max error)."""
    if k < 1 or R <= 1.0:
        raise ValueError("need k >= 1 and R > 1")
    res = _remez(*_start(k, R), R)
    if res is not None:
        return res[:3]
    # continuation in R from an interval where the start value converges;
    # each step seeds the Remez iteration with the previous alternation set
    # mapped onto the new interval (log x scaled by log R_new / log R_old)
    for R0 in (100.0 * k, 1000.0 * k, 10.0 * k):
        res = _remez(*_start(k, R0), R0)
        Rprev = R0
        for Ri in np.exp(np.linspace(np.log(R0), np.log(R), 48)[1:]):
            if res is None:
                break
            xs = np.exp(np.log(res[3]) * (np.log(Ri) / np.log(Rprev)))
            res = _remez(res[0], res[1], Ri, xs)
            Rprev = Ri
        if res is not None:
            return res[:3]
    raise RuntimeError(f"minimax fit failed at k={k}, R={R:.4g}")


def laplace_points(k, ymin, ymax):
    """(alpha, omega, err) for 1/y on [ymin, ymax]: exponents, weights and the
    maximum absolute error of 1/y."""
    if not (0 < ymin < ymax):
        raise ValueError("need 0 < ymin < ymax")
    w, a, err = minimax_unit(k, ymax / ymin)
    order = np.argsort(a)
    return a[order] / ymin, w[order] / ymin, err / ymin
