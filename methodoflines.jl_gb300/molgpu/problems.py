"""The benchmark problem families, written against the MethodOfLines-style API.

Each builder returns ``(pdesys, disc, extras)``; ``extras`` carries the seeded
synthetic inputs (targets, step sizes) the workloads use.  All random inputs
come from ``numpy.random.Generator(PCG64(seed))`` in Float64.

1. heat1d        u_t = D u_xx on [0,1], Dirichlet 0, u0 = sin(pi x)
2. brusselator   2-D periodic Brusselator with the reference test's forcing
                 (test/Brusselator/brusselator_eq.jl:8-58)
3. burgers       u_t = -u u_x + nu u_xx, periodic, WENO5 (Convection_WENO tests)
4. nonlinear_diffusion   u_t = div(u^2 grad u) + k u (1-u), Neumann 0 (ensemble member)
5. adr3d         u_t = div(K grad u) + 0.3 u_xy - c.grad u - lambda u^2, periodic x,y, Dirichlet z
6. stretched_reaction_diffusion   u_t = u_xx - k u^2 + s(x), grid clustered at both ends
                 (a grid given as points), Robin left, Neumann right
7. neumann_cosine                 u_t = u_xx on [0, pi], homogeneous Neumann, u0 = cos x
                 (test/Diffusion/MOL_1D_Linear_Diffusion.jl, Test 03), points given as a vector
8. stretched_2d                   u_t = u_xx + u_yy + 0.1 u, x stretched (Robin/Neumann),
                 y uniform (Dirichlet with data)
9. burgers_weno_dirichlet         u_t = -u u_x, u0 = x, Dirichlet x/(t+1) at both ends, WENO
                 (test/Burgers/burgers_eq.jl:56-104; exact solution x/(t+1))
10. viscous_burgers_weno_bounded  u_t = -u u_x + nu u_xx, Dirichlet data, WENO on [0, 1]
11. burgers_weno_channel          2-D u_t = -u u_x - 0.5 u_y + nu lap u, WENO, x bounded
                 (Dirichlet), y periodic
12. neumann_cosine_edge           u_t = u_xx on an edge-aligned grid of [0, 1], u_x = 0,
                 u0 = cos(pi x) (the reference's Test 03 with grid_align = edge_align)
13. robin_2d_edge                 2-D reaction-diffusion on an edge-aligned grid, time- and
                 coordinate-dependent Robin, Neumann and Dirichlet rows
14. convection_nonuniform         u_t = -v u_x on clustered grids (first-order upwinding on a
                 nonuniform grid; test/Convection_NU/MOL_1D_Linear_Convection_NonUniform.jl)
15. weno_convection_mms           u_t = -v u_x with WENO on grids given as points (uniform points,
                 sinh, tanh): test/Convection_WENO/MOL_1D_WENO_NU_Convergence.jl
16. burgers_nonuniform_upwind     u_t = -u u_x, u0 = x, first-order upwinding on a perturbed
                 grid (test/Burgers/burgers_eq.jl:106-152)
"""
from __future__ import annotations

import math

import numpy as np

from .api import MOLFiniteDifference, UpwindScheme, WENOScheme, edge_align
from .symbolic import (Differential, Eq, Field, Interval, IV, Param, PDESystem, cos, exp, register, sin, sqrt)


def _rng(seed):
    return np.random.Generator(np.random.PCG64(seed))


def heat1d(n: int = 101, D: float = 1.0):
    x, t = IV("x"), IV("t")
    u = Field("u")
    Dt, Dxx = Differential(t), Differential(x) ** 2
    Dp = Param("D", D)
    eq = Eq(Dt(u(x, t)), Dp * Dxx(u(x, t)))
    bcs = [Eq(u(x, 0.0), sin(math.pi * x)), Eq(u(0.0, t), 0.0), Eq(u(1.0, t), 0.0)]
    sys = PDESystem([eq], bcs, [(t, Interval(0.0, 0.1)), (x, Interval(0.0, 1.0))], [t, x], [u(x, t)], [Dp])
    disc = MOLFiniteDifference({x: n}, t, approx_order=2)
    return sys, disc, {}


def brusselator(N: int = 256, forcing: bool = True, t_end: float = 11.5):
    """dx = dy = 1/N on [0,1]^2, periodic: N unknowns per dimension and field."""
    x, y, t = IV("x"), IV("y"), IV("t")
    u, v = Field("u"), Field("v")
    Dt = Differential(t)
    Dxx, Dyy = Differential(x) ** 2, Differential(y) ** 2
    alpha = Param("alpha", 10.0)

    def lap(w):
        return Dxx(w) + Dyy(w)

    U, V = u(x, y, t), v(x, y, t)
    f = ((((x - 0.3) ** 2 + (y - 0.6) ** 2) <= 0.1 ** 2) * (t >= 1.1)) * 5.0
    rhs_u = 1.0 + V * U ** 2 - 4.4 * U + alpha * lap(U)
    if forcing:
        rhs_u = rhs_u + f
    eqs = [Eq(Dt(U), rhs_u), Eq(Dt(V), 3.4 * U - V * U ** 2 + alpha * lap(V))]
    bcs = [
        Eq(u(x, y, 0.0), 22 * (y * (1 - y)) ** 1.5),
        Eq(u(0.0, y, t), u(1.0, y, t)),
        Eq(u(x, 0.0, t), u(x, 1.0, t)),
        Eq(v(x, y, 0.0), 27 * (x * (1 - x)) ** 1.5),
        Eq(v(0.0, y, t), v(1.0, y, t)),
        Eq(v(x, 0.0, t), v(x, 1.0, t)),
    ]
    sys = PDESystem(eqs, bcs, [(x, Interval(0.0, 1.0)), (y, Interval(0.0, 1.0)), (t, Interval(0.0, t_end))],
                    [x, y, t], [U, V], [alpha])
    disc = MOLFiniteDifference({x: 1.0 / N, y: 1.0 / N}, t, approx_order=2)
    dx = 1.0 / N
    return sys, disc, {"dt_ssprk": dx * dx / (8 * 10.0)}


def burgers_ic_coeffs(seed: int = 1):
    r = _rng(seed)
    ks = np.arange(1, 9)
    a = r.normal(0.0, 1.0 / ks)
    phi = r.uniform(0.0, 2 * math.pi, size=8)
    return ks, a, phi


def burgers(npts: int = 65537, nu: float = 1e-3, seed: int = 1, target_seed: int = 2):
    """Periodic [0, 2 pi], `npts` grid points (npts - 1 unknowns), WENO5 convection."""
    x, t = IV("x"), IV("t")
    u = Field("u")
    Dt, Dx, Dxx = Differential(t), Differential(x), Differential(x) ** 2
    nup = Param("nu", nu)
    U = u(x, t)
    eq = Eq(Dt(U), -U * Dx(U) + nup * Dxx(U))
    ks, a, phi = burgers_ic_coeffs(seed)
    ic = None
    for k, ak, pk in zip(ks, a, phi):
        term = float(ak) * sin(float(k) * x + float(pk))
        ic = term if ic is None else ic + term
    L = 2 * math.pi
    bcs = [Eq(u(x, 0.0), ic), Eq(u(0.0, t), u(L, t))]
    sys = PDESystem([eq], bcs, [(t, Interval(0.0, 1.0)), (x, Interval(0.0, L))], [t, x], [U], [nup])
    disc = MOLFiniteDifference({x: npts}, t, approx_order=2, advection_scheme=WENOScheme(1e-6))
    # seeded target for the adjoint misfit
    kt, at, pt = burgers_ic_coeffs(target_seed)
    dx = L / (npts - 1)
    xs = np.arange(1, npts) * dx
    target = sum(float(ak) * np.sin(float(k) * xs + float(pk)) for k, ak, pk in zip(kt, at, pt))
    u0 = sum(float(ak) * np.sin(float(k) * xs + float(pk)) for k, ak, pk in zip(ks, a, phi))
    dt = 0.4 / (np.max(np.abs(u0)) / dx + 2 * nu / dx ** 2)
    return sys, disc, {"target": target, "dt": float(dt)}


def random_fourier_2d(seed: int, nmodes: int = 16, kmax: int = 4):
    """Unit-variance sum of nmodes cosines with integer wavenumbers |k| <= kmax."""
    r = _rng(seed)
    kx = r.integers(-kmax, kmax + 1, size=nmodes)
    ky = r.integers(-kmax, kmax + 1, size=nmodes)
    zero = (kx == 0) & (ky == 0)
    kx[zero] = 1
    c = r.normal(size=nmodes)
    ph = r.uniform(0, 2 * math.pi, size=nmodes)
    scale = 1.0 / math.sqrt(0.5 * float(np.sum(c * c)))
    return kx, ky, c * scale, ph


def nonlinear_diffusion(n: int, k: float, seed: int):
    """One ensemble member: n x n grid points on the unit square, Neumann 0 on every face."""
    x, y, t = IV("x"), IV("y"), IV("t")
    u = Field("u")
    Dt, Dx, Dy = Differential(t), Differential(x), Differential(y)
    kp = Param("k", k)
    U = u(x, y, t)
    eq = Eq(Dt(U), Dx(U ** 2 * Dx(U)) + Dy(U ** 2 * Dy(U)) + kp * U * (1 - U))
    kx, ky, c, ph = random_fourier_2d(seed)
    g = None
    for a, b, cc, p in zip(kx, ky, c, ph):
        term = float(cc) * cos(2 * math.pi * float(a) * x + 2 * math.pi * float(b) * y + float(p))
        g = term if g is None else g + term
    bcs = [Eq(u(x, y, 0.0), 0.5 + 0.1 * g),
           Eq(Dx(u(0.0, y, t)), 0.0), Eq(Dx(u(1.0, y, t)), 0.0),
           Eq(Dy(u(x, 0.0, t)), 0.0), Eq(Dy(u(x, 1.0, t)), 0.0)]
    sys = PDESystem([eq], bcs, [(x, Interval(0.0, 1.0)), (y, Interval(0.0, 1.0)), (t, Interval(0.0, 1.0))],
                    [x, y, t], [U], [kp])
    disc = MOLFiniteDifference({x: n, y: n}, t, approx_order=2)
    return sys, disc, {}


def coefficient_system(n: int = 24):
    """Two coupled fields on [0,1]^2 with coordinate-dependent diffusivities beside constant
    first-derivative terms, one diffusivity scaled by a parameter, and Dirichlet, Neumann and
    Robin rows:
        u_t = Dx(K1 Dx u) + Dy(kp K2 Dy u) + 0.7 Dx(u) - v
        v_t = Dx(K2 Dx v) + Dy(K1 Dy v) - 0.4 Dy(v) + u v
    K1 = 0.5 + 0.3 sin(2 pi x) cos(pi y), K2 = 1 + 0.2 x y (registered functions of the
    coordinates, evaluated on the host at the faces)."""
    x, y, t = IV("x"), IV("y"), IV("t")
    u, v = Field("u"), Field("v")
    Dt, Dx, Dy = Differential(t), Differential(x), Differential(y)
    K1 = register("K1", lambda X, Y: 0.5 + 0.3 * np.sin(2 * math.pi * X) * np.cos(math.pi * Y))
    K2 = register("K2", lambda X, Y: 1.0 + 0.2 * X * Y)
    kp = Param("kp", 0.8)
    U, V = u(x, y, t), v(x, y, t)
    eq1 = Eq(Dt(U), Dx(K1(x, y) * Dx(U)) + Dy(kp * K2(x, y) * Dy(U)) + 0.7 * Dx(U) - V)
    eq2 = Eq(Dt(V), Dx(K2(x, y) * Dx(V)) + Dy(K1(x, y) * Dy(V)) - 0.4 * Dy(V) + U * V)
    bcs = [Eq(u(x, y, 0.0), 1.0 + 0.2 * y + 0.1 * sin(math.pi * x) * sin(math.pi * y)),
           Eq(v(x, y, 0.0), 0.5 + 0.1 * cos(math.pi * x) * cos(2 * math.pi * y)),
           Eq(u(0.0, y, t), 1.0 + 0.2 * y), Eq(Dx(u(1.0, y, t)), 0.0),
           Eq(u(x, 0.0, t) + 0.5 * Dy(u(x, 0.0, t)), 1.0), Eq(u(x, 1.0, t), 1.2),
           Eq(Dx(v(0.0, y, t)), 0.0), Eq(Dx(v(1.0, y, t)), 0.0), Eq(Dy(v(x, 0.0, t)), 0.0),
           Eq(Dy(v(x, 1.0, t)), 0.0)]
    sys = PDESystem([eq1, eq2], bcs, [(x, Interval(0.0, 1.0)), (y, Interval(0.0, 1.0)), (t, Interval(0.0, 1.0))],
                    [x, y, t], [U, V], [kp])
    disc = MOLFiniteDifference({x: n, y: n}, t, approx_order=2)
    h = 1.0 / (n - 1)
    return sys, disc, {"dt": 0.1 * h * h}


def ensemble_members(count: int = 4096, seed_n: int = 7, seed_k: int = 8, nmin: int = 32, nmax: int = 512):
    """(n_i, k_i, ic seed) of the ensemble: n log-uniform on [nmin, nmax], k uniform on [0, 2]."""
    rn = _rng(seed_n)
    rk = _rng(seed_k)
    ns = np.rint(np.exp(rn.uniform(math.log(nmin), math.log(nmax), size=count))).astype(int)
    ks = rk.uniform(0.0, 2.0, size=count)
    return [(int(ns[i]), float(ks[i]), 1000 + i) for i in range(count)]


def _kfield_modes(seed: int = 11, nmodes: int = 64, ell: float = 0.1):
    r = _rng(seed)
    kap = r.normal(0.0, 1.0 / ell, size=(nmodes, 3))
    kx = np.rint(kap[:, 0] / (2 * math.pi))
    ky = np.rint(kap[:, 1] / (2 * math.pi))
    kz = kap[:, 2]
    ph = r.uniform(0, 2 * math.pi, size=nmodes)
    return kx, ky, kz, ph


def make_kfield(seed: int = 11, sigma: float = 1.0, mean: float = 0.01):
    """Log-normal diffusivity K = mean * exp(sigma g - sigma^2/2); g unit-variance random Fourier field."""
    kx, ky, kz, ph = _kfield_modes(seed)
    amp = math.sqrt(2.0 / len(kx))

    def K(X, Y, Z):
        g = np.zeros(np.broadcast(X, Y, Z).shape)
        for a, b, c, p in zip(kx, ky, kz, ph):
            g = g + amp * np.cos(2 * math.pi * a * X + 2 * math.pi * b * Y + c * Z + p)
        return mean * np.exp(sigma * g - 0.5 * sigma * sigma)
    return K


def adr3d(N: int = 256, nz_pts: int = 258, seed_k: int = 11, target_seed: int = 12):
    """256^3 unknowns by default: x, y periodic (N+1 points), z Dirichlet (nz_pts points, nz_pts-2 interior)."""
    x, y, z, t = IV("x"), IV("y"), IV("z"), IV("t")
    u = Field("u")
    Dt, Dx, Dy, Dz = Differential(t), Differential(x), Differential(y), Differential(z)
    Kfun = make_kfield(seed_k)
    K = register("K", Kfun)
    U = u(x, y, z, t)
    lam = Param("lambda", 0.5)
    eq = Eq(Dt(U), Dx(K(x, y, z) * Dx(U)) + Dy(K(x, y, z) * Dy(U)) + Dz(K(x, y, z) * Dz(U))
            + 0.3 * Dx(Dy(U)) - 1.0 * Dx(U) - 0.5 * Dy(U) - lam * U ** 2)
    r2 = (x - 0.3) ** 2 + (y - 0.5) ** 2 + (z - 0.5) ** 2
    ic = exp(-1.0 * r2 / (2 * 0.05 ** 2))
    bcs = [Eq(u(x, y, z, 0.0), ic), Eq(u(0.0, y, z, t), u(1.0, y, z, t)), Eq(u(x, 0.0, z, t), u(x, 1.0, z, t)),
           Eq(u(x, y, 0.0, t), 0.0), Eq(u(x, y, 1.0, t), 0.0)]
    sys = PDESystem([eq], bcs, [(x, Interval(0.0, 1.0)), (y, Interval(0.0, 1.0)), (z, Interval(0.0, 1.0)),
                                (t, Interval(0.0, 1.0))], [x, y, z, t], [U], [lam])
    disc = MOLFiniteDifference({x: 1.0 / N, y: 1.0 / N, z: nz_pts}, t, approx_order=2,
                               advection_scheme=UpwindScheme(1))
    dx = 1.0 / N
    dz = 1.0 / (nz_pts - 1)
    kmax = 0.01 * math.exp(1.0 * 3 * math.sqrt(1.0) - 0.5)  # generous bound of the field
    dt = 0.4 / (1.5 / dx + 2 * (3 * kmax + 0.3) / min(dx, dz) ** 2)
    rt = _rng(target_seed)
    return sys, disc, {"dt": float(dt), "target_seed": target_seed, "K": Kfun, "rng_target": rt}


def stretched_points(n: int, lo: float = 0.0, hi: float = 1.0, beta: float = 2.5) -> np.ndarray:
    """n points on [lo, hi] clustered towards both ends (tanh stretching of k / (n - 1))."""
    s = np.arange(n, dtype=np.float64) / (n - 1)
    x = lo + (hi - lo) * 0.5 * (1.0 + np.tanh(beta * (s - 0.5)) / math.tanh(0.5 * beta))
    x[0], x[-1] = lo, hi
    return x


def stretched_reaction_diffusion(n: int = 201, order: int = 2, beta: float = 2.5):
    """Reaction-diffusion on a grid given as points (nonuniform centered operators,
    centered_diff_weights.jl:77-153), Robin row at x = 0 and Neumann row at x = 1."""
    x, t = IV("x"), IV("t")
    u = Field("u")
    Dt, Dx, Dxx = Differential(t), Differential(x), Differential(x) ** 2
    k = Param("k", 2.0)
    eq = Eq(Dt(u(x, t)), Dxx(u(x, t)) - k * u(x, t) * u(x, t) + sin(math.pi * x))
    bcs = [Eq(u(x, 0.0), 1.0 + 0.5 * cos(3.0 * x)), Eq(2.0 * u(0.0, t) + 3.0 * Dx(u(0.0, t)), k * t),
           Eq(Dx(u(1.0, t)), 0.5)]
    sys = PDESystem([eq], bcs, [(t, Interval(0.0, 1.0)), (x, Interval(0.0, 1.0))], [t, x], [u(x, t)], [k])
    pts = stretched_points(n, 0.0, 1.0, beta)
    disc = MOLFiniteDifference({x: pts}, t, approx_order=order)
    h = float(np.min(np.diff(pts)))
    return sys, disc, {"dt": 0.1 * h * h, "points": pts}


def neumann_cosine(n: int = 300, order: int = 8):
    """u_t = u_xx, u0 = cos x, u_x = 0 at both ends of [0, pi]: the reference's linear-diffusion
    Test 03 (exact solution exp(-t) cos x), with the grid given as its n points."""
    x, t = IV("x"), IV("t")
    u = Field("u")
    Dt, Dx, Dxx = Differential(t), Differential(x), Differential(x) ** 2
    eq = Eq(Dt(u(x, t)), Dxx(u(x, t)))
    bcs = [Eq(u(x, 0.0), cos(x)), Eq(Dx(u(0.0, t)), 0.0), Eq(Dx(u(math.pi, t)), 0.0)]
    sys = PDESystem([eq], bcs, [(t, Interval(0.0, 1.0)), (x, Interval(0.0, math.pi))], [t, x], [u(x, t)], [])
    pts = np.array([math.pi * k / (n - 1) for k in range(n)])
    disc = MOLFiniteDifference({x: pts}, t, approx_order=order)
    h = math.pi / (n - 1)
    return sys, disc, {"dt": 0.05 * h * h, "points": pts}


def stretched_2d(nx: int = 48, ny: int = 40, order: int = 2, beta: float = 2.0):
    """2-D diffusion with x on stretched points (nonuniform) and y uniform."""
    x, y, t = IV("x"), IV("y"), IV("t")
    u = Field("u")
    Dt, Dx, Dxx, Dyy = Differential(t), Differential(x), Differential(x) ** 2, Differential(y) ** 2
    eq = Eq(Dt(u(x, y, t)), Dxx(u(x, y, t)) + Dyy(u(x, y, t)) + 0.1 * u(x, y, t))
    bcs = [Eq(u(x, y, 0.0), 1.0 + 0.3 * cos(2.0 * x) * sin(3.0 * y)),
           Eq(u(0.0, y, t) + 0.5 * Dx(u(0.0, y, t)), 1.0), Eq(Dx(u(1.0, y, t)), 0.0),
           Eq(u(x, 0.0, t), 1.0), Eq(u(x, 1.0, t), 1.0 + t)]
    sys = PDESystem([eq], bcs, [(t, Interval(0.0, 1.0)), (x, Interval(0.0, 1.0)), (y, Interval(0.0, 1.0))],
                    [t, x, y], [u(x, y, t)], [])
    pts = stretched_points(nx, 0.0, 1.0, beta)
    disc = MOLFiniteDifference({x: pts, y: 1.0 / (ny - 1)}, t, approx_order=order)
    h = min(float(np.min(np.diff(pts))), 1.0 / (ny - 1))
    return sys, disc, {"dt": 0.1 * h * h, "points": pts}


def burgers_weno_dirichlet(dx: float = 0.05):
    """Inviscid Burgers with WENO on a bounded interval: the interior stops two points from
    each end and points 2 and n-1 are extrapolated (WENO.jl:94, generate_bc_eqs.jl:336-392)."""
    x, t = IV("x"), IV("t")
    u = Field("u")
    Dt, Dx = Differential(t), Differential(x)
    eq = Eq(Dt(u(x, t)), -u(x, t) * Dx(u(x, t)))
    bcs = [Eq(u(x, 0.0), 1.0 * x), Eq(u(0.0, t), 0.0 / (t + 1.0)), Eq(u(1.0, t), 1.0 / (t + 1.0))]
    sys = PDESystem([eq], bcs, [(t, Interval(0.0, 6.0)), (x, Interval(0.0, 1.0))], [t, x], [u(x, t)], [])
    disc = MOLFiniteDifference({x: dx}, t, advection_scheme=WENOScheme())
    return sys, disc, {"dt": 0.2 * dx}


def viscous_burgers_weno_bounded(n: int = 257, nu: float = 2e-3, order: int = 2):
    """u_t = -u u_x + nu u_xx on [0, 1], u0 = 0.5 + 0.4 sin(2 pi x) with time-dependent
    Dirichlet data at both ends, WENO advection."""
    x, t = IV("x"), IV("t")
    u = Field("u")
    Dt, Dx, Dxx = Differential(t), Differential(x), Differential(x) ** 2
    nup = Param("nu", nu)
    eq = Eq(Dt(u(x, t)), -u(x, t) * Dx(u(x, t)) + nup * Dxx(u(x, t)))
    bcs = [Eq(u(x, 0.0), 0.5 + 0.4 * sin(2.0 * math.pi * x)), Eq(u(0.0, t), 0.5 + 0.2 * t),
           Eq(u(1.0, t), 0.5 - 0.1 * t)]
    sys = PDESystem([eq], bcs, [(t, Interval(0.0, 1.0)), (x, Interval(0.0, 1.0))], [t, x], [u(x, t)], [nup])
    disc = MOLFiniteDifference({x: n}, t, approx_order=order, advection_scheme=WENOScheme())
    h = 1.0 / (n - 1)
    return sys, disc, {"dt": 0.4 / (1.0 / h + 2.0 * nu / h ** 2)}


def burgers_weno_channel(nx: int = 65, ny: int = 49, nu: float = 2e-3):
    """2-D WENO advection with x bounded (Dirichlet, extrapolated points 2 and n-1) and y
    periodic."""
    x, y, t = IV("x"), IV("y"), IV("t")
    u = Field("u")
    Dt, Dx, Dy = Differential(t), Differential(x), Differential(y)
    Dxx, Dyy = Differential(x) ** 2, Differential(y) ** 2
    eq = Eq(Dt(u(x, y, t)), -u(x, y, t) * Dx(u(x, y, t)) - 0.5 * Dy(u(x, y, t))
            + nu * (Dxx(u(x, y, t)) + Dyy(u(x, y, t))))
    bcs = [Eq(u(x, y, 0.0), 0.6 + 0.3 * sin(2.0 * math.pi * x) * cos(2.0 * math.pi * y)),
           Eq(u(0.0, y, t), 0.6), Eq(u(1.0, y, t), 0.6 + 0.1 * t),
           Eq(u(x, 0.0, t), u(x, 1.0, t))]
    sys = PDESystem([eq], bcs, [(t, Interval(0.0, 1.0)), (x, Interval(0.0, 1.0)), (y, Interval(0.0, 1.0))],
                    [t, x, y], [u(x, y, t)], [])
    disc = MOLFiniteDifference({x: nx, y: ny}, t, advection_scheme=WENOScheme())
    h = min(1.0 / (nx - 1), 1.0 / (ny - 1))
    return sys, disc, {"dt": 0.3 / (1.5 / h + 4.0 * nu / h ** 2)}


def neumann_cosine_edge(dx: float = 0.01, order: int = 8):
    """u_t = u_xx on an edge-aligned grid (cell centres plus ghost points) of [0, 1] with
    u_x = 0 at both faces; exact solution exp(-pi^2 t) cos(pi x)."""
    x, t = IV("x"), IV("t")
    u = Field("u")
    Dt, Dx, Dxx = Differential(t), Differential(x), Differential(x) ** 2
    eq = Eq(Dt(u(x, t)), Dxx(u(x, t)))
    bcs = [Eq(u(x, 0.0), cos(math.pi * x)), Eq(Dx(u(0.0, t)), 0.0), Eq(Dx(u(1.0, t)), 0.0)]
    sys = PDESystem([eq], bcs, [(t, Interval(0.0, 1.0)), (x, Interval(0.0, 1.0))], [t, x], [u(x, t)], [])
    disc = MOLFiniteDifference({x: dx}, t, approx_order=order, grid_align=edge_align)
    return sys, disc, {"dt": 0.05 * dx * dx}


def robin_2d_edge(dx: float = 0.025, dy: float = 0.03125, order: int = 4):
    """Reaction-diffusion on an edge-aligned 2-D grid: Robin row with data depending on t and
    y at x = 0, Neumann at x = 1, Dirichlet with data in y."""
    x, y, t = IV("x"), IV("y"), IV("t")
    u = Field("u")
    Dt, Dx = Differential(t), Differential(x)
    Dxx, Dyy = Differential(x) ** 2, Differential(y) ** 2
    k = Param("k", 1.0)
    eq = Eq(Dt(u(x, y, t)), Dxx(u(x, y, t)) + Dyy(u(x, y, t)) - k * u(x, y, t) * u(x, y, t))
    bcs = [Eq(u(x, y, 0.0), 1.0 + 0.3 * cos(2.0 * x) * sin(3.0 * y)),
           Eq(2.0 * u(0.0, y, t) + 0.5 * Dx(u(0.0, y, t)), 1.0 + t * y), Eq(Dx(u(1.0, y, t)), 0.2),
           Eq(u(x, 0.0, t), 1.0), Eq(u(x, 1.0, t), 1.0 + t)]
    sys = PDESystem([eq], bcs, [(t, Interval(0.0, 1.0)), (x, Interval(0.0, 1.0)), (y, Interval(0.0, 1.0))],
                    [t, x, y], [u(x, y, t)], [k])
    disc = MOLFiniteDifference({x: dx, y: dy}, t, approx_order=order, grid_align=edge_align)
    h = min(dx, dy)
    return sys, disc, {"dt": 0.1 * h * h}


def cluster_grid(kind: str, n: int = 101, a: float = 0.0, b: float = 1.0) -> np.ndarray:
    """Clustered grids of the reference's nonuniform convection tests: "symmetric" (sinh
    stretching 7), "left"/"right" (geometric spacing, ratio 1000) and "chebyshev" nodes."""
    if kind == "symmetric":
        xi = np.array([-1.0 + 2.0 * k / (n - 1) for k in range(n)])
        x = a + (b - a) * (np.sinh(7.0 * xi) / math.sinh(7.0) + 1.0) / 2.0
    elif kind in ("left", "right"):
        m = n - 1
        r = 1000.0 ** (1.0 / (m - 1))
        dx = np.array([r ** k for k in range(m)])
        if kind == "right":
            dx = dx[::-1]
        dx = dx * ((b - a) / np.sum(dx))
        x = a + np.concatenate([[0.0], np.cumsum(dx)])
    elif kind == "chebyshev":
        k = np.arange(1, n + 1)
        x = np.sort((a + b) / 2 + (b - a) / 2 * np.cos(math.pi * (2 * k - 1) / (2 * n)))
    else:
        raise ValueError(kind)
    x[0], x[-1] = a, b
    return x


def convection_nonuniform(kind: str = "symmetric", n: int = 101, v: float = 1.0):
    """u_t = -v u_x, u0 = sin(2 pi x), exact translating-sine data at both ends, first-order
    upwinding on a clustered grid given as points."""
    x, t = IV("x"), IV("t")
    u = Field("u")
    Dt, Dx = Differential(t), Differential(x)
    vp = Param("v", v)
    eq = Eq(Dt(u(x, t)), -vp * Dx(u(x, t)))
    bcs = [Eq(u(x, 0.0), sin(2.0 * math.pi * x)), Eq(u(0.0, t), sin(2.0 * math.pi * (0.0 - v * t))),
           Eq(u(1.0, t), sin(2.0 * math.pi * (1.0 - v * t)))]
    sys = PDESystem([eq], bcs, [(t, Interval(0.0, 0.25)), (x, Interval(0.0, 1.0))], [t, x], [u(x, t)], [vp])
    pts = cluster_grid(kind, n)
    disc = MOLFiniteDifference({x: pts}, t, advection_scheme=UpwindScheme())
    return sys, disc, {"dt": 0.25 * float(np.min(np.diff(pts))) / abs(v), "points": pts}


WENO_MMS_ALPHA = 0.15


def weno_mms_exact(x, t, v=1.0, L=2 * math.pi):
    return np.sin(2 * math.pi * (x - v * t) / L) + WENO_MMS_ALPHA * np.sin(4 * math.pi * (x - v * t) / L)


def weno_grid(kind: str, n: int, a: float = 0.0, b: float = 2 * math.pi) -> np.ndarray:
    """Grids of the reference's nonuniform WENO convergence test: "uniform" (the points of
    range(a, b, length = n) given as a vector), "sinh" (stretch 4), "tanh" (stretch 2)."""
    xi = np.array([-1.0 + 2.0 * k / (n - 1) for k in range(n)])
    if kind == "uniform":
        x = a + (b - a) * (xi + 1.0) / 2.0
    elif kind == "sinh":
        x = a + (b - a) * (np.sinh(4.0 * xi) / math.sinh(4.0) + 1.0) / 2.0
    elif kind == "tanh":
        x = a + (b - a) * (np.tanh(2.0 * xi) / math.tanh(2.0) + 1.0) / 2.0
    else:
        raise ValueError(kind)
    x[0], x[-1] = a, b
    return x


def weno_convection_mms(kind: str = "sinh", n: int = 81, v: float = 1.0):
    """u_t = -v u_x on [0, 2 pi] with WENO on a grid given as points and the manufactured
    solution sin(2 pi (x - v t)/L) + 0.15 sin(4 pi (x - v t)/L) as Dirichlet data."""
    x, t = IV("x"), IV("t")
    u = Field("u")
    Dt, Dx = Differential(t), Differential(x)
    L = 2 * math.pi
    a = WENO_MMS_ALPHA

    def ex(xx, tt):
        return sin(2 * math.pi * (xx - v * tt) / L) + a * sin(4 * math.pi * (xx - v * tt) / L)
    eq = Eq(Dt(u(x, t)), -v * Dx(u(x, t)))
    bcs = [Eq(u(x, 0.0), ex(x, 0.0)), Eq(u(0.0, t), ex(0.0, t)), Eq(u(L, t), ex(L, t))]
    sys = PDESystem([eq], bcs, [(t, Interval(0.0, 0.05)), (x, Interval(0.0, L))], [t, x], [u(x, t)], [])
    pts = weno_grid(kind, n)
    disc = MOLFiniteDifference({x: pts}, t, advection_scheme=WENOScheme())
    return sys, disc, {"dt": 0.01 * float(np.min(np.diff(pts))) / abs(v), "points": pts}


def burgers_nonuniform_upwind(seed: int = 0):
    """The reference's nonuniform Burgers test: 0:0.05:1 with the inner points moved by
    +-0.001 (seeded here with PCG64), u0 = x, Dirichlet x/(t+1), first-order upwinding."""
    x, t = IV("x"), IV("t")
    u = Field("u")
    Dt, Dx = Differential(t), Differential(x)
    eq = Eq(Dt(u(x, t)), -u(x, t) * Dx(u(x, t)))
    bcs = [Eq(u(x, 0.0), 1.0 * x), Eq(u(0.0, t), 0.0 / (t + 1.0)), Eq(u(1.0, t), 1.0 / (t + 1.0))]
    sys = PDESystem([eq], bcs, [(t, Interval(0.0, 1.0)), (x, Interval(0.0, 1.0))], [t, x], [u(x, t)], [])
    pts = np.array([k * 0.05 for k in range(21)])
    pts[1:-1] += _rng(seed).choice([0.001, -0.001], size=19)
    disc = MOLFiniteDifference({x: pts}, t, advection_scheme=UpwindScheme(1))
    return sys, disc, {"dt": 0.2 * float(np.min(np.diff(pts))), "points": pts}


NLD_C, NLD_H = 50.0, 0.5


def nonlinear_diffusion_nu_exact(x, t):
    """u = (x + h) / (2 sqrt(c - t)), the exact solution of u_t = (u^2 u_x)_x the reference's
    nonuniform nonlinear-diffusion test uses (test/Nonlinear_Diffusion_NU, Test 01a)."""
    return 0.5 * (np.asarray(x) + NLD_H) / math.sqrt(NLD_C - t)


def nonlinear_diffusion_nonuniform(order: int = 2, seed: int = 0, coefficient: str = "u2"):
    """u_t = Dx(a Dx(u)) on the points of 0:0.01:2 with the inner points moved by +-0.001
    (seeded here with PCG64), Dirichlet rows from the exact solution at both ends: the
    nonlinear Laplacian on a nonuniform grid (nonlinear_laplacian.jl:28-103 with the per-point
    half-offset tables of half_offset_weights.jl:72-150).  coefficient "u2" is the reference
    test's a = u^2; "x" gives a = 1 + x, a function of the interpolated half-point coordinate."""
    from .lowering import grid_points
    x, t = IV("x"), IV("t")
    u = Field("u")
    Dt, Dx = Differential(t), Differential(x)
    a = u(x, t) ** 2 if coefficient == "u2" else 1.0 + x
    eq = Eq(Dt(u(x, t)), Dx(a * Dx(u(x, t))))
    k = 0.5 / math.sqrt(NLD_C)
    bcs = [Eq(u(x, 0.0), k * (x + NLD_H)),
           Eq(u(0.0, t), 0.5 * (0.0 + NLD_H) / sqrt(NLD_C - t)),
           Eq(u(2.0, t), 0.5 * (2.0 + NLD_H) / sqrt(NLD_C - t))]
    sys = PDESystem([eq], bcs, [(t, Interval(0.0, 2.0)), (x, Interval(0.0, 2.0))], [t, x], [u(x, t)], [])
    pts = np.array(grid_points(0.0, 0.01, 2.0), dtype=np.float64)
    pts[1:-1] += _rng(seed).choice([0.001, -0.001], size=len(pts) - 2)
    disc = MOLFiniteDifference({x: pts}, t, approx_order=order)
    h = float(np.min(np.diff(pts)))
    amax = 1.0 + 2.0 if coefficient == "x" else (0.5 * (2.0 + NLD_H) / math.sqrt(NLD_C - 2.0)) ** 2
    return sys, disc, {"dt": 0.2 * h * h / amax, "points": pts}


def mixed_nonuniform(nx: int = 21, ny: int = 17, order: int = 2):
    """u_t = Dxx u + Dyy u + 0.3 Dx(Dy(u)) with x on stretched points and y on a grid clustered
    at its low end: the mixed derivative as the product of the two dimensions' per-point
    first-derivative rows (2nd_order_mixed_deriv.jl:5-22 through centered_difference.jl:32-56).
    Dirichlet rows hold x^2 y^2 on every face, so that state is exact data for the tables."""
    x, y, t = IV("x"), IV("y"), IV("t")
    u = Field("u")
    Dt, Dx, Dy = Differential(t), Differential(x), Differential(y)
    eq = Eq(Dt(u(x, y, t)), (Dx ** 2)(u(x, y, t)) + (Dy ** 2)(u(x, y, t)) + 0.3 * Dx(Dy(u(x, y, t))))
    bcs = [Eq(u(x, y, 0.0), x * x * y * y), Eq(u(0.0, y, t), 0.0), Eq(u(1.0, y, t), y * y),
           Eq(u(x, 0.0, t), 0.0), Eq(u(x, 1.0, t), x * x)]
    sys = PDESystem([eq], bcs, [(t, Interval(0.0, 1.0)), (x, Interval(0.0, 1.0)), (y, Interval(0.0, 1.0))],
                    [t, x, y], [u(x, y, t)], [])
    px, py = stretched_points(nx), cluster_grid("left", ny)
    disc = MOLFiniteDifference({x: px, y: py}, t, approx_order=order)
    h = min(float(np.min(np.diff(px))), float(np.min(np.diff(py))))
    return sys, disc, {"dt": 0.1 * h * h, "points": (px, py)}


def spherical_laplacian(dr: float = 0.1, order: int = 4, scale: float = 1.0):
    """u_t = scale / r^2 * Dr(r^2 Dr(u)) on [0, 1], u0 = sin(r)/r, Dr(u) = 0 at r = 0 and
    u = e^(-scale t) sin(1) at r = 1: the reference's spherical-Laplacian tests
    (test/Diffusion/MOL_1D_Linear_Diffusion.jl, Tests 07 and 08), discretised through its
    spherical_diffusion rule (spherical_laplacian.jl)."""
    r, t = IV("r"), IV("t")
    u = Field("u")
    Dt, Dr = Differential(t), Differential(r)
    eq = Eq(Dt(u(r, t)), scale / r ** 2 * Dr(r ** 2 * Dr(u(r, t))))
    bcs = [Eq(u(r, 0.0), sin(r) / r), Eq(Dr(u(0.0, t)), 0.0), Eq(u(1.0, t), exp(-scale * t) * math.sin(1.0))]
    sys = PDESystem([eq], bcs, [(t, Interval(0.0, 1.0)), (r, Interval(0.0, 1.0))], [t, r], [u(r, t)], [])
    disc = MOLFiniteDifference({r: dr}, t, approx_order=order)
    return sys, disc, {"dt": 0.1 * dr * dr / scale}
