"""Surface errors: the reference's uncorrelated normal-direction error
(mt19937 with a fresh normal distribution per point, InterfaceReflector.cpp:
852-866, Random.h:112-116) and the correlated spectral synthesis built on the
same generator, in their three statements: the product's host code
(po_correlated_error), the device kernels (po_generate_grid_dev with rms,
po_correlated_error_dev) and the oracle's numpy (oracle/grids.py, pinned to
the reference's own perturbed grid and to mt19937's known answer).
CPU tests: host against oracle. GPU tests: device against oracle, and a
perturbed-dish chain that never leaves the device."""
import numpy as np
import pytest

from oracle import grids as OG


def _dish(n=61):
    return OG.generate(OG.paraboloid(400.0, [n, n], gmode=1, lims_a=[0.0, 300.0]))


def test_host_correlated_error_matches_oracle(lib):
    from pypo_gb300 import engine
    g7 = np.ascontiguousarray(_dish())
    ref = OG.correlated_error(g7[0], g7[1], 0.05, 30.0, seed=4, n_modes=512)
    got = engine.correlated_error(g7.copy(), 0.05, 30.0, seed=4, n_modes=512)
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-13 * np.abs(ref).max())
    # apply: the points move along their normals by delta, nothing else changes
    moved = g7.copy()
    d = engine.correlated_error(moved, 0.05, 30.0, seed=4, n_modes=512, apply=True)
    np.testing.assert_allclose(moved[:3], g7[:3] + d[None, :] * g7[3:6], rtol=0, atol=1e-13 * 300)
    np.testing.assert_array_equal(moved[3:], g7[3:])


def test_host_correlated_error_rejects_bad_arguments(lib):
    from pypo_gb300 import engine
    from pypo_gb300._lib import POError
    g7 = np.ascontiguousarray(_dish(5))
    with pytest.raises(POError, match="corr_len"):
        engine.correlated_error(g7, 0.05, 0.0, seed=1)
    with pytest.raises(POError, match="n_modes"):
        engine.correlated_error(g7, 0.05, 30.0, seed=1, n_modes=0)


def test_correlated_error_statistics():
    """Variance rms^2 and the Gaussian covariance at one correlation length,
    averaged over seeds (the oracle's synthesis; the host and device equal it)."""
    x, y = np.meshgrid(np.linspace(0, 600, 121), np.linspace(0, 600, 121))
    x, y = x.ravel(), y.ravel()
    var = cov = 0.0
    seeds = range(30)
    for s in seeds:
        d = OG.correlated_error(x, y, 1.0, 30.0, s, 256).reshape(121, 121)
        var += (d * d).mean()
        cov += (d[:, :-6] * d[:, 6:]).mean()   # lag 30 mm along x
    var /= len(seeds)
    cov /= len(seeds)
    assert abs(var - 1.0) < 0.1, var
    assert abs(cov - np.exp(-0.5)) < 0.1, cov


@pytest.mark.gpu
def test_device_normal_deviates_match_oracle(cuda, lib):
    """Many 624-word blocks of the device generator (a 400 x 500 grid with
    rms error) against the oracle's mt19937 and polar method."""
    from pypo_gb300 import engine
    d = OG.plane([400, 500], gmode=0, lims_a=[-1.0, 1.0], rms=0.7, rms_seed=12345)
    got = engine.generate_grid_dev(d, device=cuda).cpu().numpy()
    flat = OG.generate(dict(d, rms=0.0))
    dev = got[2] - flat[2]   # a plane's normal is +z: the deviates are the z offsets
    ref = OG.normal_deviates(12345, 400 * 500, 0.7)
    np.testing.assert_allclose(dev, ref, rtol=0, atol=1e-14)


@pytest.mark.gpu
def test_device_correlated_error_matches_oracle(cuda, lib):
    import torch
    from pypo_gb300 import engine
    g7 = _dish(201)
    ref = OG.correlated_error(g7[0], g7[1], 0.05, 30.0, seed=9, n_modes=700)
    t = torch.tensor(g7, device=cuda)
    got = engine.correlated_error_dev(t, 0.05, 30.0, seed=9, n_modes=700, apply=True).cpu().numpy()
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-13 * np.abs(ref).max())
    moved = t.cpu().numpy()
    np.testing.assert_allclose(moved[:3], g7[:3] + ref[None, :] * g7[3:6], rtol=0, atol=1e-12)


@pytest.mark.gpu
def test_perturbed_dish_chain_stays_on_the_device(cuda, lib):
    """The differentiation configuration's first stage from a device-resident
    perturbed dish: grid, correlated error and feed made on the device, then
    the propagation; equal to the host-built inputs' propagation."""
    import torch
    from pypo_gb300 import beams, configs, engine
    c = configs.dish_chain(scale=0.2)
    dish = configs.dish_facing_feed(400.0, 600.0, c["dish_grid"][1])
    d7 = engine.generate_grid_dev(dish, device=cuda)
    delta = engine.correlated_error_dev(d7, c["lam"] / 40.0, 30.0, seed=4, apply=True)
    np.testing.assert_allclose(delta.cpu().numpy(), c["delta"], rtol=0, atol=1e-13 * np.abs(c["delta"]).max())
    f7 = torch.tensor(c["feed7"], device=cuda)
    _, fcur = beams.gauss_beam_dev(f7, c["lam"], 10.0, 0.0, 4 * np.pi)
    got = engine.propagate_dev("JM", f7, fcur, *c["feed_grid"], d7, c["k"])
    host7 = c["dish7"].copy()
    host7[:3] += c["delta"][None, :] * host7[3:6]
    ref = engine.propagate("JM", c["feed7"], c["feed_cur"], *c["feed_grid"], host7, c["k"])
    rel = np.linalg.norm(got.cpu().numpy() - ref) / np.linalg.norm(ref)
    assert rel <= 1e-6, rel
