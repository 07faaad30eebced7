"""Grid-size convergence searches on the device (pypo_gb300.converge) against
their CPU restatement on the FP64 oracle (oracle/converge.py): the same
trials, the same measured powers or differences, the same grid sizes."""
import numpy as np
import pytest

from oracle import converge as OC

pytestmark = pytest.mark.gpu

LAM = 2.0
K = 2 * np.pi / LAM


def _feed(cuda, n=21):
    """A Gaussian feed (lambda 2 mm, w0 6 mm) on an n x n plane of +-15 mm:
    device grid, its grid mode and counts, the device fields."""
    from pypo_gb300 import beams, engine, surfaces as SF
    plane = SF.plane([n, n], gmode=0, lims_a=[-15.0, 15.0])
    g7 = engine.generate_grid_dev(plane, device=cuda)
    fields, _ = beams.gauss_beam_dev(g7, LAM, 6.0, 0.0, 4 * np.pi)
    return g7, (0, n, n), fields


@pytest.mark.parametrize("gmode", [1, 0])
def test_auto_converge_matches_oracle(cuda, lib, gmode):
    from pypo_gb300 import configs, converge
    g7, grid, fields = _feed(cuda)
    target = configs.dish_facing_feed(60.0, 120.0, 11, gmode=gmode)
    for precision in ("fp64", "mixed"):
        size, powers = converge.auto_converge(g7, grid, fields, target, K, precision=precision, full_output=True)
        ref, ref_powers = OC.auto_converge(g7.cpu().numpy(), grid, fields.cpu().numpy(), target, K)
        assert np.array_equal(size, ref), (precision, size, ref)
        assert len(powers) == len(ref_powers)
        np.testing.assert_allclose(powers, ref_powers, rtol=1e-9 if precision == "fp64" else 1e-5)


def test_auto_converge_rejects_an_aoe_target(cuda, lib):
    from pypo_gb300 import converge, surfaces as SF
    from pypo_gb300._lib import POError
    g7, grid, fields = _feed(cuda)
    with pytest.raises(POError, match="AoE"):
        converge.auto_converge(g7, grid, fields, SF.farfield([5, 5], [-1, 1], [-1, 1]), K)


@pytest.mark.parametrize("gmode", [1, 0])
def test_converge_on_target_matches_oracle(cuda, lib, gmode):
    """Feed -> dish (the scatterer) -> a plane near the focus of the dish's
    reflection (the target), both axes, with the bisection."""
    from pypo_gb300 import configs, converge, surfaces as SF
    g7, grid, fields = _feed(cuda)
    scat = configs.dish_facing_feed(60.0, 120.0, 10, gmode=gmode)
    tgt = SF.translate(SF.plane([5, 5], gmode=gmode, lims_a=[0.0, 20.0] if gmode == 1 else [-20.0, 20.0]),
                       dz=-150.0)
    for precision in ("fp64", "mixed"):
        size, trials = converge.converge_on_target(g7, grid, fields, scat, tgt, K, precision=precision,
                                                   full_output=True)
        ref, ref_trials = OC.converge_on_target(g7.cpu().numpy(), grid, fields.cpu().numpy(), scat, tgt, K)
        assert np.array_equal(size, ref), (precision, size, ref, trials, ref_trials)
        assert [t[:2] for t in trials] == [t[:2] for t in ref_trials]
        np.testing.assert_allclose([t[2] for t in trials], [t[2] for t in ref_trials],
                                   rtol=1e-8 if precision == "fp64" else 1e-3, atol=1e-9)
