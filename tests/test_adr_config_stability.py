"""The 3-D advection-diffusion-reaction configuration is ill-posed as stated.

u_t = div(K grad u) + 0.3 u_xy - (1, 0.5, 0) . grad u - 0.5 u^2 with K ~ 0.01: the second-order
part has the diffusion tensor [[K, 0.15, 0], [0.15, K, 0], [0, 0, K]], indefinite for K < 0.15,
so the equation is backward-parabolic along the (1, -1, 0) diagonal.  Its discretisation (the
reference's stencils: second-order centered diffusion and mixed term, first-order upwinding)
has Fourier modes near kx dx = ky dx = pi/2 that grow by ~8 % per SSPRK33 step at the
configuration's dt, whatever the grid.  From the Gaussian initial state the reference's
discretisation therefore leaves O(1) and overflows: at 256^3 between steps 400 and 500 (the
configuration asks for 500), at 32^3 within 200.  Every implementation that rounds
differently from another diverges from it by that growth, so long-horizon trajectory
comparisons of this configuration are bounded by it, not by the implementations.

CPU only: the symbol in closed form, and the C/OpenMP restatement of the reference's
discretisation (oracle/c) stepped from u0 at 32^3.
"""
import math

import numpy as np

from molgpu import lower, problems
from oracle.c_port import ADR3D


def _growth_per_step(N, K=0.01, cmix=0.3, cx=1.0, cy=0.5):
    """max over the (theta_x, theta_y) grid (theta_z = 0) of |R(dt * lambda)|, lambda the symbol
    of the semi-discrete operator with constant K, R SSPRK33's stability polynomial."""
    _, _, ex = problems.adr3d(N=N, nz_pts=N + 2)
    dt, dx = ex["dt"], 1.0 / N
    th = np.linspace(-math.pi, math.pi, 181)
    tx, ty = np.meshgrid(th, th, indexing="ij")
    lam = (K * (2 * np.cos(tx) - 2 + 2 * np.cos(ty) - 2) / dx ** 2
           - cmix * np.sin(tx) * np.sin(ty) / dx ** 2                     # centered Dx(Dy(u))
           - cx * (1 - np.exp(-1j * tx)) / dx - cy * (1 - np.exp(-1j * ty)) / dx)   # backward upwind
    z = dt * lam
    R = 1 + z + z ** 2 / 2 + z ** 3 / 6
    return float(np.max(np.abs(R)))


def test_symbol_grows_at_every_resolution():
    for N in (32, 64, 256):
        g = _growth_per_step(N)
        assert 1.05 < g < 1.12, (N, g)
    # 500 steps at 256^3 amplify round-off (1e-16) past O(1)
    assert _growth_per_step(256) ** 500 > 1e16


def test_reference_discretisation_blows_up_from_u0():
    sys_, disc, ex = problems.adr3d(N=32, nz_pts=34)
    lw = lower(sys_.to_spec(disc))
    port = ADR3D(lw)
    u = np.array(lw.u0, copy=True)
    assert np.max(np.abs(u)) <= 1.0
    u = port.ssprk33(u, ex["dt"], 25)
    assert np.all(np.isfinite(u)) and np.max(np.abs(u)) < 1.2
    with np.errstate(all="ignore"):
        u = port.ssprk33(u, ex["dt"], 175)
    assert not np.all(np.isfinite(u)) or np.max(np.abs(u)) > 100.0
