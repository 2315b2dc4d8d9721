"""Argument checks of the Python binding: the library trusts the pointers and element counts
it is given, so a wrong dtype, length, layout or a read-only output is refused on the host
before any call into the library (no GPU needed)."""
import numpy as np
import pytest
import torch

from molgpu.api import Batch, Plan, _ptr


def test_accepts_float64_and_float32_arrays_of_the_right_length():
    _, f32 = _ptr(np.zeros(5), 5, "u")
    assert f32 is False
    _, f32 = _ptr(np.zeros(5, dtype=np.float32), 5, "u")
    assert f32 is True
    _, f32 = _ptr(torch.zeros(5, dtype=torch.float64), 5, "u")
    assert f32 is False
    assert _ptr(None, 5, "p") == (None, None)


@pytest.mark.parametrize("bad, err", [
    (np.zeros(5, dtype=np.int64), TypeError),
    (np.zeros(4), ValueError),
    (np.zeros(10)[::2], ValueError),
    ([0.0] * 5, TypeError),
    (torch.zeros(5, dtype=torch.int32), TypeError),
    (torch.zeros(6, dtype=torch.float64), ValueError),
    (torch.zeros(10, dtype=torch.float64)[::2], ValueError),
])
def test_rejects_wrong_dtype_length_or_layout(bad, err):
    with pytest.raises(err):
        _ptr(bad, 5, "u")


def test_rejects_mixed_precision_and_read_only_outputs():
    with pytest.raises(TypeError):
        _ptr(np.zeros(5), 5, "u", f32=True)
    ro = np.zeros(5)
    ro.setflags(write=False)
    _ptr(ro, 5, "u")
    with pytest.raises(ValueError):
        _ptr(ro, 5, "du", out=True)


def _detached_plan(n=6, nparams=2, naux=3):
    """A Plan object without a library handle: every check below must fire before the
    library is reached."""
    plan = object.__new__(Plan)
    plan._h = None
    plan.n, plan.nparams, plan.naux = n, nparams, naux
    return plan


def test_plan_methods_check_their_arguments_first():
    plan = _detached_plan()
    good, short = np.zeros(6), np.zeros(5)
    with pytest.raises(ValueError):
        plan.rhs(np.zeros(6), short, None, 0.0)
    with pytest.raises(TypeError):
        plan.rhs(np.zeros(6, dtype=np.float32), good, None, 0.0)
    with pytest.raises(ValueError):
        plan.rhs(np.zeros(6), good, np.zeros(3), 0.0)
    with pytest.raises(ValueError):
        plan.step_ssprk33(short, 1e-3, 2)
    with pytest.raises(ValueError):
        plan.solve_tsit5(short, 0.0, 1.0, 1e-8, 1e-8)
    with pytest.raises(ValueError):
        plan.vjp(good, good, None, 0.0, lam_aux=np.zeros(2))
    with pytest.raises(ValueError):
        plan.adjoint_ssprk33(good, 1e-3, 4, short)
    with pytest.raises(ValueError):
        plan.adjoint_ssprk33(good, 1e-3, 4, good, dLdp=np.zeros(1))


def test_batch_checks_the_packed_state_and_one_step_per_instance():
    batch = object.__new__(Batch)
    batch._h = None
    batch.n = 3
    batch.offsets = np.array([0, 4, 9, 16], dtype=np.int64)
    with pytest.raises(ValueError):
        batch.step_ssprk33(np.zeros(15), np.ones(3), 1)
    with pytest.raises(ValueError):
        batch.step_ssprk33(np.zeros(16), np.ones(2), 1)


def test_a_count_of_zero_leaves_the_array_unchecked_in_length():
    """A plan without parameters reads no p: any float array (or None) is accepted."""
    _ptr(np.zeros(1), 0, "lam_p")
