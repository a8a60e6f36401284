"""Exact solution of the one-dimensional Riemann problem for two ideal gases
(test infrastructure, no GPU).

Restated from the published method of E. F. Toro, "Riemann Solvers and
Numerical Methods for Fluid Dynamics" (3rd ed., Springer 2009), chapter 4:
the star-region pressure is the root of f_L(p) + f_R(p) + u_R - u_L = 0
(shock branch where p exceeds the side's pressure, isentropic rarefaction
branch otherwise), found by Newton iteration from the two-rarefaction guess;
the solution is then sampled at x / t.  Each side keeps its own ratio of
specific heats, so a contact between two different gases is exact as well
(the five-equation model's two-material shock tubes).
"""
from __future__ import annotations

import math

import numpy as np


def _side(p, rho_k, p_k, g):
    """f_K(p) and its derivative for one side (rho_k, p_k, gamma g)."""
    c = math.sqrt(g * p_k / rho_k)
    if p > p_k:  # shock
        A = 2.0 / ((g + 1.0) * rho_k)
        B = (g - 1.0) / (g + 1.0) * p_k
        q = math.sqrt(A / (B + p))
        return (p - p_k) * q, q * (1.0 - 0.5 * (p - p_k) / (B + p))
    r = p / p_k  # rarefaction
    return 2.0 * c / (g - 1.0) * (r ** ((g - 1.0) / (2.0 * g)) - 1.0), r ** (-(g + 1.0) / (2.0 * g)) / (rho_k * c)


def star_state(left, right):
    """(p*, u*) of the Riemann problem left = (rho, u, p, gamma), right = the same."""
    rl, ul, pl, gl = left
    rr, ur, pr, gr = right
    cl, cr = math.sqrt(gl * pl / rl), math.sqrt(gr * pr / rr)
    if 2.0 * cl / (gl - 1.0) + 2.0 * cr / (gr - 1.0) <= ur - ul:
        raise ValueError("the data generate vacuum")
    # two-rarefaction guess (exact when both waves are rarefactions and the gases agree)
    z = (gl - 1.0) / (2.0 * gl)
    p = ((cl + cr - 0.5 * (gl - 1.0) * (ur - ul)) / (cl / pl**z + cr / pr**z)) ** (1.0 / z)
    p = max(p, 1e-12 * min(pl, pr))
    for _ in range(100):
        fl, dl = _side(p, rl, pl, gl)
        fr, dr = _side(p, rr, pr, gr)
        p_new = max(p - (fl + fr + ur - ul) / (dl + dr), 1e-12 * min(pl, pr))
        if abs(p_new - p) <= 1e-14 * (p_new + p):
            p = p_new
            break
        p = p_new
    fl, _ = _side(p, rl, pl, gl)
    fr, _ = _side(p, rr, pr, gr)
    return p, 0.5 * (ul + ur) + 0.5 * (fr - fl)


def _sample_side(s, rho_k, u_k, p_k, g, p_s, u_s, sign):
    """The solution at speed s on one side of the contact (sign -1 left, +1 right)."""
    c = math.sqrt(g * p_k / rho_k)
    gm, gp = g - 1.0, g + 1.0
    if p_s > p_k:  # shock
        S = u_k + sign * c * math.sqrt(gp / (2.0 * g) * p_s / p_k + gm / (2.0 * g))
        if sign * (s - S) >= 0.0:
            return rho_k, u_k, p_k
        r = p_s / p_k
        return rho_k * (r + gm / gp) / (gm / gp * r + 1.0), u_s, p_s
    c_s = c * (p_s / p_k) ** (gm / (2.0 * g))
    head = u_k + sign * c
    tail = u_s + sign * c_s
    if sign * (s - head) >= 0.0:
        return rho_k, u_k, p_k
    if sign * (s - tail) <= 0.0:
        return rho_k * (p_s / p_k) ** (1.0 / g), u_s, p_s
    # inside the fan
    w = 2.0 / gp - sign * gm / (gp * c) * (u_k - s)
    return rho_k * w ** (2.0 / gm), 2.0 / gp * (-sign * c + 0.5 * gm * u_k + s), p_k * w ** (2.0 * g / gm)


def sample(left, right, x, t, x0=0.5):
    """Density, velocity, pressure and the material (0 left of the contact,
    1 right) at the points x at time t > 0, the discontinuity initially at x0."""
    p_s, u_s = star_state(left, right)
    out = np.empty((4, len(x)))
    for i, xi in enumerate(np.asarray(x, dtype=np.float64)):
        s = (xi - x0) / t
        if s <= u_s:
            out[:3, i] = _sample_side(s, left[0], left[1], left[2], left[3], p_s, u_s, -1.0)
            out[3, i] = 0.0
        else:
            out[:3, i] = _sample_side(s, right[0], right[1], right[2], right[3], p_s, u_s, 1.0)
            out[3, i] = 1.0
    return out
