"""Test infrastructure: exact solutions for known-answer tests of the Hydro
scheme, the cases of the reference's exact-solution harness
(attic/GA.reproduce/massive-test.cu:52-118): entropy wave, sound wave, Sod's
shock tube, and rotated ("oblique") versions.

The exact solution of the 1-D Riemann problem of an ideal gas is the
published algorithm (E. F. Toro, Riemann Solvers and Numerical Methods for
Fluid Dynamics, ch. 4: Newton iteration on the pressure function for p*,
then sampling the self-similar solution at S = x / t), which the
reference's harness also calls (attic/GA.reproduce/riemann-solver.h:91).
"""
from __future__ import annotations

import math

import numpy as np


def _f(p, rho, pk, ck, g):
    """Toro's pressure function f_K(p) and its derivative."""
    if p > pk:                                   # shock
        A = 2.0 / ((g + 1.0) * rho)
        B = (g - 1.0) / (g + 1.0) * pk
        s = math.sqrt(A / (p + B))
        return (p - pk) * s, s * (1.0 - 0.5 * (p - pk) / (B + p))
    r = p / pk                                   # rarefaction
    return (2.0 * ck / (g - 1.0) * (r ** ((g - 1.0) / (2.0 * g)) - 1.0),
            1.0 / (rho * ck) * r ** (-(g + 1.0) / (2.0 * g)))


def star_state(L, R, g):
    """(p*, u*) of the Riemann problem with states L, R = (rho, u, p)."""
    rl, ul, pl = L
    rr, ur, pr = R
    cl, cr = math.sqrt(g * pl / rl), math.sqrt(g * pr / rr)
    p = max(1e-12, 0.5 * (pl + pr))
    for _ in range(100):
        fl, dl = _f(p, rl, pl, cl, g)
        fr, dr = _f(p, rr, pr, cr, g)
        dp = (fl + fr + ur - ul) / (dl + dr)
        pn = max(1e-12, p - dp)
        if abs(pn - p) <= 1e-14 * (pn + p):
            p = pn
            break
        p = pn
    fl, _ = _f(p, rl, pl, cl, g)
    fr, _ = _f(p, rr, pr, cr, g)
    return p, 0.5 * (ul + ur) + 0.5 * (fr - fl)


def sample(L, R, g, S):
    """(rho, u, p) of the self-similar solution at speeds S = x / t."""
    S = np.asarray(S, float)
    rl, ul, pl = L
    rr, ur, pr = R
    cl, cr = math.sqrt(g * pl / rl), math.sqrt(g * pr / rr)
    ps, us = star_state(L, R, g)
    rho, u, p = np.empty_like(S), np.empty_like(S), np.empty_like(S)
    gm, gp = (g - 1.0) / (g + 1.0), (g + 1.0)
    for side in (0, 1):
        sel = S <= us if side == 0 else S > us
        rk, uk, pk, ck = (rl, ul, pl, cl) if side == 0 else (rr, ur, pr, cr)
        sgn = -1.0 if side == 0 else 1.0     # left waves move with -c, right with +c
        s = S[sel]
        if ps > pk:                           # shock
            ss = uk + sgn * ck * math.sqrt((g + 1) / (2 * g) * ps / pk + (g - 1) / (2 * g))
            rs = rk * (ps / pk + gm) / (gm * ps / pk + 1.0)
            outside = s <= ss if side == 0 else s >= ss
            r_ = np.where(outside, rk, rs)
            u_ = np.where(outside, uk, us)
            p_ = np.where(outside, pk, ps)
        else:                                 # rarefaction
            cs = ck * (ps / pk) ** ((g - 1) / (2 * g))
            head = uk + sgn * ck
            tail = us + sgn * cs
            rs = rk * (ps / pk) ** (1.0 / g)
            if side == 0:
                outside, star = s <= head, s > tail
                c = 2.0 / gp * (ck + 0.5 * (g - 1) * (uk - s))
                uf = 2.0 / gp * (ck + 0.5 * (g - 1) * uk + s)
            else:
                outside, star = s >= head, s < tail
                c = 2.0 / gp * (ck - 0.5 * (g - 1) * (uk - s))
                uf = 2.0 / gp * (-ck + 0.5 * (g - 1) * uk + s)
            rf = rk * (c / ck) ** (2.0 / (g - 1))
            pf = pk * (c / ck) ** (2.0 * g / (g - 1))
            r_ = np.where(outside, rk, np.where(star, rs, rf))
            u_ = np.where(outside, uk, np.where(star, us, uf))
            p_ = np.where(outside, pk, np.where(star, ps, pf))
        rho[sel], u[sel], p[sel] = r_, u_, p_
    return rho, u, p


SOD_L = (1.0, 0.0, 1.0)
SOD_R = (0.125, 0.0, 0.1)


def sod_periodic(x, t, g):
    """Sod's problem twice on the periodic unit interval: the left state in
    [1/4, 3/4), the right state outside, so a mirrored problem sits at 1/4
    and Sod's own at 3/4 (valid while the waves stay apart, t <= 0.12)."""
    x = np.asarray(x, float)
    rho, u, p = sample(SOD_L, SOD_R, g, (x - 0.75) / t)
    left = x < 0.5
    r2, u2, p2 = sample(SOD_L, SOD_R, g, (0.25 - x[left]) / t)
    rho[left], u[left], p[left] = r2, -u2, p2
    return rho, u, p


def entropy_wave(x, y, t, vx=1.0, vy=0.0, kx=1, ky=0):
    """Density 2 + sin(2 pi (kx x + ky y) - phase) advected with (vx, vy) at
    unit pressure (the harness's EntropyWave, periodic wave numbers)."""
    ph = 2 * math.pi * (kx * (x - vx * t) + ky * (y - vy * t))
    return 2.0 + np.sin(ph), np.full_like(ph, vx), np.full_like(ph, vy), np.ones_like(ph)


def sound_wave(x, t, g, amplitude=1e-5):
    """The harness's SoundWave (linear acoustics, unit sound speed)."""
    c = 1.0
    rho0, p0 = g, 1.0                         # c^2 = g p0 / rho0 = 1
    vx = amplitude * np.sin(2 * math.pi * (x - c * t))
    return rho0 + rho0 / c * vx, vx, np.zeros_like(vx), p0 + g * p0 / c * vx
