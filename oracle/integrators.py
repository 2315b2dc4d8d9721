"""Oracle explicit integrators (test infrastructure only).

SSPRK33 follows the Shu-Osher form with OrdinaryDiffEq's evaluation order
(OrdinaryDiffEqSSPRK ``perform_step!`` for ``SSPRK33``: ``tmp = uprev + dt*k``,
``tmp = (3*uprev + tmp + dt*k)/4``, ``u = (uprev + 2*tmp + 2*dt*k)/3``; called in the
reference at ``benchmark/weno/suite.jl:291-295``).  Tsit5 uses Tsitouras' 2011
tableau with the standard PI step-size controller and Hairer's initial step
heuristic, the algorithm OrdinaryDiffEq documents (adaptive trajectories are
therefore *not* pinned to OrdinaryDiffEq bit for bit).
"""
from __future__ import annotations

import math

import numpy as np

# Tsitouras (2011), "Runge-Kutta pairs of order 5(4) satisfying only the first column
# simplifying assumption", Comput. Math. Appl. 62:770-775.
TSIT5_C = [0.0, 0.161, 0.327, 0.9, 0.9800255409045097, 1.0, 1.0]
TSIT5_A = [
    [],
    [0.161],
    [-0.008480655492356989, 0.335480655492357],
    [2.897153057105493, -6.359448489975075, 4.3622954328695815],
    [5.325864828439257, -11.748883564062828, 7.4955393428898365, -0.09249506636175525],
    [5.86145544294642, -12.92096931784711, 8.159367898576159, -0.071584973281401,
     -0.028269050394068383],
    [0.09646076681806523, 0.01, 0.4798896504144996, 1.379008574103742, -3.290069515436081,
     2.324710524099774],
]
TSIT5_BTILDE = [-0.00178001105222577714, -0.0008164344596567469, 0.007880878010261995,
                -0.1447110071732629, 0.5823571654525552, -0.45808210592918697,
                0.015151515151515152]


def ssprk33(f, u0, t0, dt, nsteps):
    """Fixed-step SSPRK33; ``f(u, t)`` returns du."""
    u = np.array(u0, dtype=np.float64, copy=True)
    t = float(t0)
    for _ in range(int(nsteps)):
        k = f(u, t)
        tmp = u + dt * k
        k = f(tmp, t + dt)
        tmp = (3 * u + tmp + dt * k) / 4
        k = f(tmp, t + dt / 2)
        u = (u + 2 * tmp + 2 * dt * k) / 3
        t = t + dt
    return u, t


def _norm(x):
    return math.sqrt(float(np.mean(x * x)))


def tsit5(f, u0, t0, t1, abstol, reltol, dt0=None, maxiters=10 ** 7,
          beta1=0.14, beta2=0.08, qmin=0.2, qmax=10.0, gamma=0.9, qoldinit=1e-4):
    """Adaptive Tsit5 with the PI controller (beta1 = 7/(10*5), beta2 = 2/(5*5)).

    Returns (u(t1), stats) with stats = {naccept, nreject, nf}.
    """
    u = np.array(u0, dtype=np.float64, copy=True)
    t = float(t0)
    nf = 0
    k1 = f(u, t)
    nf += 1
    if dt0 is None:
        sk = abstol + np.abs(u) * reltol
        d0 = _norm(u / sk)
        d1 = _norm(k1 / sk)
        h0 = 1e-6 if (d0 < 1e-5 or d1 < 1e-5) else 0.01 * d0 / d1
        h0 = min(h0, t1 - t0)
        u1 = u + h0 * k1
        f1 = f(u1, t + h0)
        nf += 1
        d2 = _norm((f1 - k1) / sk) / h0
        m = max(d1, d2)
        h1 = max(1e-6, h0 * 1e-3) if m <= 1e-15 else (0.01 / m) ** (1.0 / 5.0)
        dt = min(100 * h0, h1, t1 - t0)
    else:
        dt = float(dt0)
    qold = qoldinit
    naccept = nreject = 0
    it = 0
    while t < t1 and it < maxiters:
        it += 1
        if t + dt > t1:
            dt = t1 - t
        ks = [k1]
        for i in range(1, 7):
            y = u.copy()
            for j, a in enumerate(TSIT5_A[i]):
                y = y + (dt * a) * ks[j]
            kk = f(y, t + TSIT5_C[i] * dt)
            nf += 1
            ks.append(kk)
        unew = y
        err = np.zeros_like(u)
        for j in range(7):
            err = err + (dt * TSIT5_BTILDE[j]) * ks[j]
        sc = abstol + np.maximum(np.abs(u), np.abs(unew)) * reltol
        EEst = _norm(err / sc)
        q11 = EEst ** beta1
        if EEst <= 1.0:
            q = q11 / (qold ** beta2)
            q = max(1.0 / qmax, min(1.0 / qmin, q / gamma))
            u = unew
            t = t + dt
            k1 = ks[6]
            qold = max(EEst, qoldinit)
            dt = dt / q
            naccept += 1
        else:
            q = min(1.0 / qmin, q11 / gamma)
            dt = dt / q
            nreject += 1
    return u, {"naccept": naccept, "nreject": nreject, "nf": nf, "t": t}
