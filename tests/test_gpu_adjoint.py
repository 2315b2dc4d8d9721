"""Discrete adjoint on the GPU: VJP and checkpointed reverse sweep against finite differences.

Bar: gradients match central finite differences to 1e-6 relative.
"""
import numpy as np
import pytest

from molgpu import Plan, lower, problems

pytestmark = pytest.mark.gpu

FD_TOL = 1e-6


def _plan(name, **kw):
    sys_, disc, ex = getattr(problems, name)(**kw)
    lw = lower(sys_.to_spec(disc))
    return Plan(lw), lw, ex


def _rhs(plan, u, p=None, t=0.3):
    du = np.zeros_like(u)
    plan.rhs(du, u, p, t)
    return du


@pytest.mark.parametrize("name,kw", [("heat1d", dict(n=21)), ("brusselator", dict(N=12)), ("burgers", dict(npts=65)),
                                     ("nonlinear_diffusion", dict(n=11, k=1.2, seed=1000)),
                                     ("adr3d", dict(N=8, nz_pts=10))])
def test_vjp_matches_finite_differences(gpu_lib, name, kw):
    plan, lw, _ = _plan(name, **kw)
    rng = np.random.default_rng(3)
    u = lw.u0 * (1 + 0.1 * rng.standard_normal(lw.n_unknowns)) + 0.05 * rng.standard_normal(lw.n_unknowns)
    lam = rng.standard_normal(lw.n_unknowns)
    v = rng.standard_normal(lw.n_unknowns)
    lam_u = np.zeros(lw.n_unknowns)
    lam_p = np.zeros(max(len(lw.param_names), 1))
    plan.vjp(lam, u, None, 0.3, lam_u=lam_u, lam_p=lam_p)
    h = 1e-6 * max(1.0, float(np.max(np.abs(u))))
    fd = lam @ (_rhs(plan, u + h * v) - _rhs(plan, u - h * v)) / (2 * h)
    assert abs(lam_u @ v - fd) <= FD_TOL * max(abs(fd), 1e-12 * np.linalg.norm(lam_u) * np.linalg.norm(v)), (lam_u @ v, fd)
    for k in range(len(lw.param_names)):
        p0 = lw.param_values.copy()
        hp = 1e-6 * max(1.0, abs(p0[k]))
        pp, pm = p0.copy(), p0.copy()
        pp[k] += hp
        pm[k] -= hp
        fdp = lam @ (_rhs(plan, u, pp) - _rhs(plan, u, pm)) / (2 * hp)
        assert abs(lam_p[k] - fdp) <= FD_TOL * max(abs(fdp), 1e-9), (k, lam_p[k], fdp)
    plan.close()


def test_vjp_aux_gradient_face_diffusivity(gpu_lib):
    """dL/dK on the face arrays of the 3-D diffusivity (the config's dL/dK)."""
    plan, lw, _ = _plan("adr3d", N=8, nz_pts=10)
    rng = np.random.default_rng(5)
    u = lw.u0 + 0.05 * rng.standard_normal(lw.n_unknowns)
    lam = rng.standard_normal(lw.n_unknowns)
    tot = sum(a.size for a in lw.aux)
    lam_aux = np.zeros(tot)
    plan.vjp(lam, u, None, 0.1, lam_u=np.zeros(lw.n_unknowns), lam_aux=lam_aux)
    dirs = [rng.standard_normal(a.size) * (a != 0) for a in lw.aux]
    h = 1e-7

    def with_aux(sign):
        import copy
        lw2 = copy.copy(lw)
        lw2.aux = [a + sign * h * d for a, d in zip(lw.aux, dirs)]
        p = Plan(lw2)
        out = _rhs(p, u, None, 0.1)
        p.close()
        return out

    fd = lam @ (with_aux(+1) - with_aux(-1)) / (2 * h)
    got = lam_aux @ np.concatenate(dirs)
    assert abs(got - fd) <= FD_TOL * abs(fd), (got, fd)


def _loss(plan, u0, dt, n, target, p=None):
    u = u0.copy()
    plan.step_ssprk33(u, dt, n, t0=0.0, p=p)
    return 0.5 * float(np.sum((u - target) ** 2)), u


@pytest.mark.parametrize("nsnap", [2, 5, 0])
def test_adjoint_burgers_matches_finite_differences(gpu_lib, nsnap):
    plan, lw, ex = _plan("burgers", npts=65)
    rng = np.random.default_rng(7)
    target = ex["target"][: lw.n_unknowns] if ex["target"].size == lw.n_unknowns else rng.standard_normal(lw.n_unknowns)
    dt, n = ex["dt"], 40
    g = np.zeros(lw.n_unknowns)
    gp = np.zeros(1)
    uT = np.zeros(lw.n_unknowns)
    loss, nfw = plan.adjoint_ssprk33(lw.u0, dt, n, target, nsnap=nsnap, uT=uT, dLdu0=g, dLdp=gp)
    L0, uref = _loss(plan, lw.u0, dt, n, target)
    assert abs(loss - L0) <= 1e-12 * L0
    assert np.allclose(uT, uref, rtol=0, atol=1e-13 * np.max(np.abs(uref)))
    v = rng.standard_normal(lw.n_unknowns)
    h = 1e-6
    fd = (_loss(plan, lw.u0 + h * v, dt, n, target)[0] - _loss(plan, lw.u0 - h * v, dt, n, target)[0]) / (2 * h)
    assert abs(g @ v - fd) <= FD_TOL * abs(fd), (g @ v, fd)
    nu = lw.param_values[0]
    hp = 1e-6 * nu
    fdp = (_loss(plan, lw.u0, dt, n, target, np.array([nu + hp]))[0] -
           _loss(plan, lw.u0, dt, n, target, np.array([nu - hp]))[0]) / (2 * hp)
    assert abs(gp[0] - fdp) <= FD_TOL * abs(fdp), (gp[0], fdp)
    assert nfw >= n


def test_adjoint_checkpoint_schedules_agree(gpu_lib):
    plan, lw, ex = _plan("burgers", npts=129)
    target = np.zeros(lw.n_unknowns)
    dt, n = ex["dt"], 57
    grads = []
    for ns in (2, 3, 8, n + 1, 0):  # 0: every state and stage value kept, nothing recomputed
        g = np.zeros(lw.n_unknowns)
        gp = np.zeros(1)
        plan.adjoint_ssprk33(lw.u0, dt, n, target, nsnap=ns, dLdu0=g, dLdp=gp)
        grads.append((g, gp))
    for g, gp in grads[1:]:
        assert np.allclose(g, grads[0][0], rtol=1e-11, atol=1e-14)
        assert np.allclose(gp, grads[0][1], rtol=1e-11)


def test_adjoint_adr3d_dLdK(gpu_lib):
    plan, lw, ex = _plan("adr3d", N=8, nz_pts=10)
    rng = np.random.default_rng(12)
    target = rng.standard_normal(lw.n_unknowns) * 0.01
    dt, n = ex["dt"], 8
    tot = sum(a.size for a in lw.aux)
    gaux = np.zeros(tot)
    loss, _ = plan.adjoint_ssprk33(lw.u0, dt, n, target, nsnap=3, dLdaux=gaux)
    dirs = [rng.standard_normal(a.size) * (a != 0) for a in lw.aux]
    h = 1e-7

    def L_with(sign):
        import copy
        lw2 = copy.copy(lw)
        lw2.aux = [a + sign * h * d for a, d in zip(lw.aux, dirs)]
        p = Plan(lw2)
        val = _loss(p, lw.u0, dt, n, target)[0]
        p.close()
        return val

    fd = (L_with(+1) - L_with(-1)) / (2 * h)
    got = gaux @ np.concatenate(dirs)
    assert abs(got - fd) <= FD_TOL * abs(fd), (got, fd)


@pytest.mark.parametrize("nsnap", [3, 0])
def test_adjoint_graph_capture_matches_stream_launches(gpu_lib, monkeypatch, nsnap):
    """On a capturable stream the reverse sweep is recorded into CUDA graphs; the gradient
    equals the one from plain stream launches (same kernels, atomics in another order)."""
    torch = pytest.importorskip("torch")
    plan, lw, ex = _plan("burgers", npts=129)
    rng = np.random.default_rng(3)
    target = rng.standard_normal(lw.n_unknowns)
    dt, n = ex["dt"], 300
    out = {}
    for mode in ("1", "0"):
        monkeypatch.setenv("MOL_ADJOINT_GRAPHS", mode)
        st = torch.cuda.Stream()
        plan.set_stream(st.cuda_stream)
        g = np.zeros(lw.n_unknowns)
        gp = np.zeros(1)
        uT = np.zeros(lw.n_unknowns)
        loss, nfw = plan.adjoint_ssprk33(lw.u0, dt, n, target, nsnap=nsnap, uT=uT, dLdu0=g, dLdp=gp)
        out[mode] = (loss, nfw, g, gp, uT)
    plan.set_stream(0)
    a, b = out["1"], out["0"]
    assert a[0] == b[0] and a[1] == b[1]
    assert np.array_equal(a[4], b[4])
    assert np.allclose(a[2], b[2], rtol=1e-12, atol=1e-15 * np.max(np.abs(b[2])))
    assert np.allclose(a[3], b[3], rtol=1e-12)


def test_adjoint_with_face_pass_matches(gpu_lib, monkeypatch):
    """The adjoint's forward stages through the face pass give the gradient of the stages
    evaluating their own faces (3-D ADR, dL/dK on the faces)."""
    out = {}
    for mode in ("1", "0"):
        monkeypatch.setenv("MOL_FACE_PASS", mode)
        plan, lw, ex = _plan("adr3d", N=8, nz_pts=10)
        target = np.random.default_rng(5).standard_normal(lw.n_unknowns) * 1e-3
        gaux = np.zeros(sum(plan.aux_sizes))
        g = np.zeros(lw.n_unknowns)
        loss, _ = plan.adjoint_ssprk33(lw.u0, ex["dt"], 6, target, nsnap=3, dLdu0=g, dLdaux=gaux)
        out[mode] = (loss, g, gaux)
        plan.close()
    assert out["1"][0] == out["0"][0]
    assert np.allclose(out["1"][1], out["0"][1], rtol=1e-12, atol=1e-18)
    assert np.allclose(out["1"][2], out["0"][2], rtol=1e-12, atol=1e-18)
