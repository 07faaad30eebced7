"""Grid-size convergence searches on the device (pypo_gb300.converge) against
the reference's own System.autoConverge / convergeOnTarget results
(tests/golden/golden_converge.npz) and, trial for trial, their CPU
restatement on the FP64 oracle (oracle/converge.py)."""
import numpy as np
import pytest

from oracle import converge as OC
from tests.test_converge import CASES, case

pytestmark = pytest.mark.gpu


def _dev(cuda, f7, fields):
    import torch
    return torch.tensor(f7, device=cuda), torch.tensor(np.ascontiguousarray(fields), device=cuda)


@pytest.mark.parametrize("key", CASES)
def test_auto_converge_matches_reference(cuda, lib, key):
    """The reference's grid size, and trial for trial the oracle
    restatement's powers."""
    from pypo_gb300 import converge
    g, f7, grid, fields, dish, _, k = case(key)
    d7, dfields = _dev(cuda, f7, fields)
    ref, ref_powers = OC.auto_converge(f7, grid, fields, dish, k)
    for precision in ("fp64", "mixed"):
        size, powers = converge.auto_converge(d7, grid, dfields, dish, k, precision=precision, full_output=True)
        assert np.array_equal(size, g[key + "__auto"]), (precision, size)
        assert len(powers) == len(ref_powers)
        np.testing.assert_allclose(powers, ref_powers, rtol=1e-9 if precision == "fp64" else 1e-5)


def test_auto_converge_rejects_an_aoe_target(cuda, lib):
    from pypo_gb300 import converge, surfaces as SF
    from pypo_gb300._lib import POError
    g, f7, grid, fields, _, _, k = case("uv_xy")
    d7, dfields = _dev(cuda, f7, fields)
    with pytest.raises(POError, match="AoE"):
        converge.auto_converge(d7, grid, dfields, SF.farfield([5, 5], [-1, 1], [-1, 1]), k)


@pytest.mark.parametrize("key", CASES)
def test_converge_on_target_matches_reference(cuda, lib, key):
    """Feed -> dish (the scatterer) -> a plane behind the feed (the target),
    both axes with the bisection: the reference's grid size, and trial for
    trial the oracle restatement's differences."""
    from pypo_gb300 import converge
    g, f7, grid, fields, dish, tgt, k = case(key)
    d7, dfields = _dev(cuda, f7, fields)
    ref, ref_trials = OC.converge_on_target(f7, grid, fields, dish, tgt, k)
    for precision in ("fp64", "mixed"):
        size, trials = converge.converge_on_target(d7, grid, dfields, dish, tgt, k, precision=precision,
                                                   full_output=True)
        assert np.array_equal(size, g[key + "__on_target"]), (precision, size, trials)
        assert [t[:2] for t in trials] == [t[:2] for t in ref_trials]
        np.testing.assert_allclose([t[2] for t in trials], [t[2] for t in ref_trials],
                                   rtol=1e-8 if precision == "fp64" else 1e-3, atol=1e-9)
