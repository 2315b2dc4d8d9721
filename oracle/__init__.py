"""CPU oracle for the method-of-lines hot path (test infrastructure only).

This package restates, on the CPU and in plain Python/numpy, the discretisation
MethodOfLines.jl performs inside ``discretize(pdesys, MOLFiniteDifference(...))``
and the explicit integrators that call the generated ``f!``.  It exists only to
check the GPU product: tests, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` leg of ``bench.py`` may import it; the product package never
does.

Parity status: the Fornberg weights and the centered/upwind weight tables are
pinned against the known answers committed in the reference's own tests
(``test/Components/MOLfornberg_weights.jl``, ``test/shared/finite_diff_schemes.jl``)
and the periodic index wrap against ``test/Components/utils_test.jl``; the
Brusselator RHS is pinned against the reference's generated equations at
dx = 1/4 (``docs/src/generated/bruss_ode_eqs.md``) and its hand-written loop RHS
(``test/Brusselator/brusselator_eq.jl:80-105``); the heat equation against its
exact solution.  The reference itself (Julia) cannot run in this container.
"""
