"""Stacks that are not finite and positive are refused with the first bad
index, by the small path, a new plan, a kept plan's restack and a resident
plan, and a refused call leaves the next valid call's result untouched
(the reference requires S_i > 0, src/cpu/icm.h)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [50, 20000])
@pytest.mark.parametrize("bad", [0.0, -1.0, np.nan, np.inf])
def test_bad_stack_refused_with_its_index(gpu_icm, n, bad):
    from icm_gb300 import ICMError
    rng = np.random.default_rng(n)
    S = 1e3 * np.exp(rng.standard_normal(n))
    P = 0.9 ** np.arange(max(1, n // 10))
    ref = gpu_icm.gpu_equity(S, P)          # also leaves a kept plan of this shape
    i = n // 3
    Sb = S.copy()
    Sb[i] = bad
    Sb[-1] = bad                             # the first bad index is reported
    with pytest.raises(ICMError, match=rf"S\[{i}\]"):
        gpu_icm.gpu_equity(Sb, P)
    assert np.array_equal(gpu_icm.gpu_equity(S, P), ref)


def test_bad_stack_refused_by_plan_creation(gpu_icm):
    from icm_gb300 import ICMError
    S = np.linspace(1.0, 2.0, 9000)
    S[4321] = np.nan
    with pytest.raises(ICMError):
        gpu_icm.GpuPlan(S, 100)
