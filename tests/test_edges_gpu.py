"""GPU edge cases against the oracle: single source / target, ragged tiles,
far-field direction counts around the two-per-thread CTA width, multi-chunk
source splits, empty sources and targets, M = 0 kernels, large phases
(kR ~ 1e3-1e4 rad, the regime of the benchmark configurations), determinism
and the device error word."""
import numpy as np
import pytest

from tests.common import PHASE_TOL, REL_L2_TOL, errors

pytestmark = pytest.mark.gpu


def _random_case(rng, ns_shape, nt, z=3.0):
    from pypo_gb300 import engine, surfaces as SF
    src = SF.paraboloid(1.0, list(ns_shape), gmode=1, lims_a=[0.1, 2.0])
    s7 = engine.generate_grid(src)
    t7 = np.zeros((7, nt))
    t7[0] = rng.uniform(-2, 2, nt)
    t7[1] = rng.uniform(-2, 2, nt)
    t7[2] = z + rng.uniform(-0.3, 0.3, nt)
    t7[5] = -1.0
    t7[6] = 1.0
    cur = rng.standard_normal((12, s7.shape[1]))
    return src, s7, t7, cur


def _check(mode, s7, cur, gmode, ncx, ncy, t7, k, oracle_mod, t=-1.0):
    from pypo_gb300 import engine
    got = engine.propagate(mode, s7, cur, gmode, ncx, ncy, t7, k, 1.0, t)
    ref = oracle_mod.run(mode, s7, cur, gmode, ncx, ncy, t7, k, 1.0, t)
    e, p = errors(got, ref, mode)
    assert e <= REL_L2_TOL and p <= PHASE_TOL, f"{mode}: rel L2 {e:.2e} phase {p:.2e}"
    return got


@pytest.mark.parametrize("ns_shape,nt", [((2, 2), 7), ((3, 4), 1), ((17, 23), 257), ((31, 33), 300),
                                         ((64, 41), 5)])
def test_sizes_against_oracle(cuda, lib, oracle_mod, ns_shape, nt):
    rng = np.random.default_rng(sum(ns_shape) * 1000 + nt)
    src, s7, t7, cur = _random_case(rng, ns_shape, nt)
    for mode in ("EH", "JM", "EHP", "scalar"):
        c = cur[:2] if mode == "scalar" else cur
        _check(mode, s7, c, 1, *ns_shape, t7, 5.0, oracle_mod)


def test_single_source_point(cuda, lib, oracle_mod):
    """One source element (explicit point, unit weight) against many targets."""
    rng = np.random.default_rng(4)
    s7 = np.array([[0.1], [-0.2], [0.05], [0.0], [0.0], [1.0], [0.01]])
    t7 = np.zeros((7, 50))
    t7[0:2] = rng.uniform(-1, 1, (2, 50))
    t7[2] = rng.uniform(0.5, 2.0, 50)
    t7[5] = 1.0
    cur = rng.standard_normal((12, 1))
    for mode in ("EH", "JMEH", "scalar"):
        c = cur[:2] if mode == "scalar" else cur
        _check(mode, s7, c, -1, 0, 0, t7, 7.0, oracle_mod)


def test_many_source_chunks(cuda, lib, oracle_mod):
    """Few targets, many sources: the source axis is split over many CTAs."""
    rng = np.random.default_rng(11)
    src, s7, t7, cur = _random_case(rng, (120, 171), 40)
    from pypo_gb300 import engine
    engine.propagate("EH", s7, cur, 1, 120, 171, t7, 4.0)
    assert engine.last_launches() >= 5
    _check("EH", s7, cur, 1, 120, 171, t7, 4.0, oracle_mod)
    _check("EH", s7, cur, 1, 120, 171, t7, 4.0, oracle_mod, t=1.0)


@pytest.mark.parametrize("ns_shape,nt", [((2, 2), 1), ((3, 4), 7), ((17, 23), 255), ((31, 33), 257),
                                         ((64, 41), 513)])
def test_far_field_sizes_against_oracle(cuda, lib, oracle_mod, ns_shape, nt):
    """Far field, two directions per thread: counts below, at and just past
    the 256 directions of a CTA."""
    rng = np.random.default_rng(sum(ns_shape) * 100 + nt)
    src, s7, _, cur = _random_case(rng, ns_shape, 1)
    t7 = np.zeros((7, nt))
    # directions around -z and (every other one) around +z: both sides of the sources
    t7[0] = np.pi - rng.uniform(0.0, 0.6, nt)
    t7[0][::2] = rng.uniform(0.0, 0.6, (nt + 1) // 2)
    t7[1] = rng.uniform(0.0, 2 * np.pi, nt)
    t7[5], t7[6] = 1.0, 1.0
    for t in (-1.0, 1.0):
        _check("FF", s7, cur, 1, *ns_shape, t7, 5.0, oracle_mod, t)


def test_empty_targets_give_empty_outputs(cuda, lib):
    import torch
    from pypo_gb300 import engine
    rng = np.random.default_rng(2)
    src, s7, _, cur = _random_case(rng, (5, 6), 1)
    for mode in ("EH", "JM", "JMEH", "EHP", "FF", "scalar"):
        c = cur[:2] if mode == "scalar" else cur
        for prec in ("mixed", "fp64"):
            out = engine.propagate(mode, s7, c, 1, 5, 6, np.zeros((7, 0)), 5.0, precision=prec)
            assert out.shape == (engine.n_out(mode), 0)
    # and the device-pointer entry
    d = lambda a: torch.tensor(a, device=cuda)
    out = engine.propagate_dev("EH", d(s7), d(cur), 1, 5, 6, d(np.zeros((7, 0))), 5.0)
    torch.cuda.synchronize()
    assert tuple(out.shape) == (12, 0)


def test_empty_source_gives_zero(cuda, lib):
    from pypo_gb300 import engine
    t7 = np.zeros((7, 10))
    t7[2] = 1.0
    for prec in ("mixed", "fp64"):
        out = engine.propagate("EH", np.zeros((7, 0)), np.zeros((12, 0)), -1, 0, 0, t7, 1.0, precision=prec)
        assert np.all(out == 0)


def test_m_zero_kernel_matches_general_kernel(cuda, lib, oracle_mod):
    """With M == 0 the host picks the kernel without magnetic terms."""
    rng = np.random.default_rng(3)
    src, s7, t7, cur = _random_case(rng, (29, 30), 200)
    cur[6:] = 0.0
    got = _check("EH", s7, cur, 1, 29, 30, t7, 6.0, oracle_mod)
    assert np.abs(got[6:]).max() > 0   # H from J alone is not zero


def _plane_sources(rng, n, facing):
    """n explicit source points on z = 0 in [-1, 1]^2, unit normal +z or -z
    per point (facing: bool array), random weights and currents."""
    s7 = np.zeros((7, n))
    s7[0:2] = rng.uniform(-1, 1, (2, n))
    s7[5] = np.where(facing, 1.0, -1.0)
    s7[6] = rng.uniform(0.5, 1.5, n) * 1e-3
    return s7, rng.standard_normal((12, n))


def test_lit_tiles_give_the_bits_of_the_per_pair_test(cuda, lib):
    """A source tile proven lit for a CTA's targets skips the per-pair
    illumination test. One more target in the same CTA, lit by every source
    but too close to the source plane for the proof's margin, turns the proof
    off for the whole CTA (the grid frame is unchanged: the target is inside
    the scene's box). The other targets' fields are the same bits."""
    from pypo_gb300 import engine
    rng = np.random.default_rng(21)
    s7, cur = _plane_sources(rng, 1000, np.ones(1000, bool))
    cur[6:] = 0.0                                    # the proof serves the M = 0 kernels
    t7 = np.zeros((7, 100))
    t7[0:2] = rng.uniform(-0.9, 0.9, (2, 100))
    t7[2] = rng.uniform(0.5, 2.0, 100)
    t7[5] = -1.0
    near = t7[:, :1].copy()
    near[2] = 1e-9                                   # n.d = 1e-9 mm > 0: lit, but inside the margin
    k = 2 * np.pi / 0.05
    for mode in ("EH", "JM", "JMEH", "EHP"):
        a = engine.propagate(mode, s7, cur, -1, 0, 0, t7, k)
        b = engine.propagate(mode, s7, cur, -1, 0, 0, np.concatenate([t7, near], axis=1), k)
        assert np.array_equal(a, b[:, :100]), mode
    # far field: directions within 30 deg of +z, and one 1e-7 rad inside the horizon
    d = np.zeros((7, 300))
    d[0] = rng.uniform(0, np.radians(30), 300)
    d[1] = rng.uniform(0, 2 * np.pi, 300)
    edge = d[:, :1].copy()
    edge[0] = np.pi / 2 - 1e-7
    a = engine.propagate("FF", s7, cur, -1, 0, 0, d, k)
    b = engine.propagate("FF", s7, cur, -1, 0, 0, np.concatenate([d, edge], axis=1), k)
    assert np.array_equal(a, b[:, :300])


def test_lit_far_field_adjoint_tiles_give_the_bits_of_the_per_pair_test(cuda, lib):
    """The far-field adjoint's lit-tile proof: one more direction in the last
    tile, 1e-7 rad inside the horizon and with a zero cotangent, turns the
    proof off for that tile; the gradients are the same bits."""
    from pypo_gb300 import engine
    rng = np.random.default_rng(23)
    s7, cur = _plane_sources(rng, 1000, np.ones(1000, bool))
    cur[6:] = 0.0
    d = np.zeros((7, 300))
    d[0] = rng.uniform(0, np.radians(30), 300)
    d[1] = rng.uniform(0, 2 * np.pi, 300)
    edge = d[:, :1].copy()
    edge[0] = np.pi / 2 - 1e-7
    cot = rng.standard_normal((12, 300))
    k = 2 * np.pi / 0.05
    a = engine.adjoint("FF", s7, cur, -1, 0, 0, d, k, cot, want=("cur", "ds"))
    b = engine.adjoint("FF", s7, cur, -1, 0, 0, np.concatenate([d, edge], axis=1), k,
                       np.concatenate([cot, np.zeros((12, 1))], axis=1), want=("cur", "ds"))
    assert np.array_equal(a["cur"], b["cur"]) and np.array_equal(a["ds"], b["ds"])


def test_tiles_facing_both_ways_against_oracle(cuda, lib, oracle_mod):
    """Sources that face the targets, sources that face away, and a tile that
    holds both: lit tiles take the proven path, the others the per-pair
    test; near and far field against the oracle."""
    rng = np.random.default_rng(22)
    facing = np.arange(700) < 300                     # tiles 0-1 face +z, tile 2 mixed, 3-5 face -z
    s7, cur = _plane_sources(rng, 700, facing)
    t7 = np.zeros((7, 150))
    t7[0:2] = rng.uniform(-1, 1, (2, 150))
    t7[2] = rng.uniform(0.3, 1.5, 150)
    t7[5] = -1.0
    k = 2 * np.pi / 0.1
    d = np.zeros((7, 260))
    d[0] = rng.uniform(0, np.radians(60), 260)
    d[1] = rng.uniform(0, 2 * np.pi, 260)
    from pypo_gb300 import engine
    rel = lambda a, b: np.linalg.norm(a - b) / np.linalg.norm(b)
    for m_zero in (True, False):                      # with and without the proof
        c = cur.copy()
        if m_zero:
            c[6:] = 0.0
        for mode in ("EH", "JM"):
            got = _check(mode, s7, c, -1, 0, 0, t7, k, oracle_mod)
            assert np.abs(got).max() > 0
        _check("FF", s7, c, -1, 0, 0, d, k, oracle_mod)
        # far-field adjoint: mixed (lit tiles proven or not) against the FP64 adjoint
        cot = rng.standard_normal((12, 260))
        gm = engine.adjoint("FF", s7, c, -1, 0, 0, d, k, cot, want=("cur", "ds"))
        gd = engine.adjoint("FF", s7, c, -1, 0, 0, d, k, cot, precision="fp64", want=("cur", "ds"))
        assert rel(gm["cur"], gd["cur"]) <= 1e-5 and rel(gm["ds"], gd["ds"]) <= 1e-4, m_zero


def test_magnetic_current_found_past_the_host_prefix(cuda, lib, oracle_mod):
    """The host-buffer entries settle M = 0 from the first 4096 magnetic
    values on the host, and the device checks the rest: a single non-zero M
    at the last source must still select the kernel with magnetic terms."""
    rng = np.random.default_rng(31)
    src, s7, t7, cur = _random_case(rng, (64, 80), 120)
    cur[6:] = 0.0
    cur[11, -1] = 0.7                                  # Mz (im) of the last source only
    _check("EH", s7, cur, 1, 64, 80, t7, 6.0, oracle_mod)
    from pypo_gb300 import engine
    cot = rng.standard_normal((12, t7.shape[1]))
    g = engine.adjoint("EH", s7, cur, 1, 64, 80, t7, 6.0, cot)
    g0 = engine.adjoint("EH", s7, np.where(np.arange(12)[:, None] >= 6, 0.0, cur), 1, 64, 80, t7, 6.0, cot)
    assert not np.allclose(g["ds"], g0["ds"], rtol=0, atol=0)   # the last source's M term is in


def test_far_field_far_off_origin(cuda, lib, oracle_mod):
    """FF keeps the coordinate origin as phase reference; a displaced dish."""
    from pypo_gb300 import engine, surfaces as SF
    src = SF.translate(SF.paraboloid(100.0, [25, 24], gmode=1, lims_a=[0, 60]), 40.0, -30.0, 25.0)
    s7 = engine.generate_grid(src)
    ff = engine.generate_grid(SF.farfield([9, 7], [-3, 3], [-2, 2]))
    rng = np.random.default_rng(8)
    cur = rng.standard_normal((12, s7.shape[1]))
    for t in (-1.0, 1.0):
        _check("FF", s7, cur, 1, 25, 24, ff, 2 * np.pi / 1.0, oracle_mod, t)


def test_large_phase_nearfield(cuda, lib, oracle_mod):
    """Paraboloid D = 1000 mm, f = 500 mm at 1 mm wavelength (kR ~ 3e3 rad),
    focal-plane targets: the benchmark's EH regime on a reduced grid."""
    from pypo_gb300 import engine, surfaces as SF
    src = SF.paraboloid(500.0, [61, 60], gmode=1, lims_a=[0, 500])
    s7 = engine.generate_grid(src)
    tgt = SF.translate(SF.plane([11, 11], gmode=0, lims_a=[-50, 50]), dz=500.0)
    t7 = engine.generate_grid(tgt)
    r = np.hypot(s7[0], s7[1])
    amp = np.exp(-0.5 * np.log(10) * (r / 500.0) ** 2)
    phase = np.random.default_rng(2).normal(0, 0.05, r.size)
    cur = np.zeros((12, r.size))
    cur[0] = amp * np.cos(phase)
    cur[3] = amp * np.sin(phase)
    k = 2 * np.pi / 1.0
    for mode in ("EH", "JM"):
        _check(mode, s7, cur, 1, 61, 60, t7, k, oracle_mod)


def test_large_phase_farfield(cuda, lib, oracle_mod):
    """Paraboloid D = 2000 mm, f = 800 mm at 1 mm wavelength (k r' ~ 6e3 rad)."""
    from pypo_gb300 import engine, surfaces as SF
    src = SF.paraboloid(800.0, [41, 40], gmode=1, lims_a=[0, 1000])
    s7 = engine.generate_grid(src)
    ff = engine.generate_grid(SF.farfield([9, 9], [-0.5, 0.5], [-0.5, 0.5]))
    r = np.hypot(s7[0], s7[1])
    cur = np.zeros((12, r.size))
    cur[0] = np.exp(-0.5 * np.log(10) * (r / 1000.0) ** 2)
    _check("FF", s7, cur, 1, 41, 40, ff, 2 * np.pi, oracle_mod)


def test_large_scene_nearfield_within_limit(cuda, lib, oracle_mod):
    """Targets 30 m from a 2 m dish at 0.5 mm wavelength: R ~ 1.2e5 turns
    (kR ~ 7.5e5 rad), frame half-extent 3e4 wavelengths, inside the mixed
    path's measured range. Forward against the oracle, adjoint against the
    FP64 adjoint."""
    from pypo_gb300 import engine, surfaces as SF
    s7 = engine.generate_grid(SF.paraboloid(800.0, [41, 40], gmode=1, lims_a=[0, 1000]))
    t7 = engine.generate_grid(SF.translate(SF.plane([7, 7], gmode=0, lims_a=[-2000, 2000]), dz=3.0e4))
    t7[3:6] *= -1.0
    rng = np.random.default_rng(21)
    cur = rng.standard_normal((12, s7.shape[1]))
    k = 2 * np.pi / 0.5
    assert engine.mixed_extent("EH", s7, t7, k) <= engine.MIXED_EXTENT_LIMIT
    for mode in ("EH", "JM"):
        _check(mode, s7, cur, 1, 41, 40, t7, k, oracle_mod)
        # the library's frame (computed on the device) has the host planner's extent
        assert engine.last_extent() == pytest.approx(engine.mixed_extent(mode, s7, t7, k), rel=1e-12)
    cot = rng.standard_normal((12, t7.shape[1]))
    gm = engine.adjoint("EH", s7, cur, 1, 41, 40, t7, k, cot, precision="mixed")
    gd = engine.adjoint("EH", s7, cur, 1, 41, 40, t7, k, cot, precision="fp64")
    rel = lambda a, b: np.linalg.norm(a - b) / np.linalg.norm(b)
    assert rel(gm["cur"], gd["cur"]) <= REL_L2_TOL
    assert rel(gm["ds"], gd["ds"]) <= 1e-4 and rel(gm["dt"], gd["dt"]) <= 1e-4


def test_large_scene_farfield_within_limit(cuda, lib, oracle_mod):
    """A 2 m dish 27 m from the coordinate origin (the far field's phase
    reference) at 0.5 mm wavelength: source coordinates up to 4.6e4
    wavelengths, inside the mixed path's measured range."""
    from pypo_gb300 import engine, surfaces as SF
    src = SF.translate(SF.paraboloid(800.0, [41, 40], gmode=1, lims_a=[0, 1000]), 2.2e4, -1.4e4, 8.0e3)
    s7 = engine.generate_grid(src)
    ff = engine.generate_grid(SF.farfield([9, 9], [-1.0, 1.0], [-1.0, 1.0]))
    k = 2 * np.pi / 0.5
    assert engine.mixed_extent("FF", s7, ff, k) <= engine.MIXED_EXTENT_LIMIT
    cur = np.random.default_rng(22).standard_normal((12, s7.shape[1]))
    for t in (-1.0, 1.0):
        _check("FF", s7, cur, 1, 41, 40, ff, k, oracle_mod, t)


def test_deterministic_and_clean_error_word(cuda, lib):
    import torch
    from pypo_gb300 import engine
    rng = np.random.default_rng(1)
    src, s7, t7, cur = _random_case(rng, (40, 50), 333)
    a = engine.propagate("JMEH", s7, cur, 1, 40, 50, t7, 3.0)
    b = engine.propagate("JMEH", s7, cur, 1, 40, 50, t7, 3.0)
    np.testing.assert_array_equal(a, b)
    assert engine.device_error(torch.cuda.current_stream()) == 0


def test_scene_beyond_the_mixed_range_warns(cuda, lib):
    """The host-buffer entries warn after a mixed-precision call whose frame
    half-extent (read back from the device) is beyond the measured range;
    the FP64 path does not."""
    import warnings
    from pypo_gb300 import engine, surfaces as SF
    s7 = engine.generate_grid(SF.paraboloid(50.0, [5, 6], gmode=1, lims_a=[0, 20]))
    t7 = engine.generate_grid(SF.translate(SF.plane([3, 3], gmode=0, lims_a=[-10, 10]), dz=2.0e5))   # 1e5 wavelengths
    t7[3:6] *= -1.0
    cur = np.random.default_rng(1).standard_normal((12, s7.shape[1]))
    k = 2 * np.pi / 1.0
    with pytest.warns(RuntimeWarning, match="fp64"):
        engine.propagate("EH", s7, cur, 1, 5, 6, t7, k)
    assert engine.last_extent() == pytest.approx(engine.mixed_extent("EH", s7, t7, k), rel=1e-12)
    with warnings.catch_warnings():
        warnings.simplefilter("error")
        engine.propagate("EH", s7, cur, 1, 5, 6, t7, k, precision="fp64")
    assert engine.last_extent() == 0.0
    ff = engine.generate_grid(SF.farfield([3, 3], [-1, 1], [-1, 1]))
    engine.propagate("FF", s7, cur, 1, 5, 6, ff, k)
    assert engine.last_extent() == pytest.approx(engine.mixed_extent("FF", s7, ff, k), rel=1e-12)


@pytest.mark.parametrize("grid,radius", [((41, 40), 1000.0), ((61, 60), 120.0)])
def test_far_field_adjoint_tile_offsets_against_oracle(cuda, lib, oracle_mod, grid, radius):
    """The far-field adjoint works on Hilbert-ordered source tiles, the
    centre's phase folded into the cotangents. On a dish of 41 x 40 sources
    over 2 m at 1 mm the tiles span hundreds of turns and store split
    offsets (wide). On 61 x 60 over 240 mm they stay within 64 turns and
    take the FP32 offset phase (narrow). Both are checked against the
    oracle's FP64 adjoint, M = 0 and M != 0, in both time directions."""
    from pypo_gb300 import engine, surfaces as SF
    rng = np.random.default_rng(int(radius))
    s7 = engine.generate_grid(SF.paraboloid(800.0, list(grid), gmode=1, lims_a=[0, radius]))
    ff = engine.generate_grid(SF.farfield([9, 8], [-1.0, 1.0], [-1.0, 1.0]))
    k = 2 * np.pi
    rel = lambda a, b: np.linalg.norm(a - b) / np.linalg.norm(b)
    for m_zero in (True, False):
        cur = rng.standard_normal((12, s7.shape[1]))
        if m_zero:
            cur[6:] = 0.0
        cot = rng.standard_normal((12, ff.shape[1]))
        for t in (-1.0, 1.0):
            gm = engine.adjoint("FF", s7, cur, 1, *grid, ff, k, cot, t_dir=t, want=("cur", "ds"))
            go = oracle_mod.adjoint("FF", s7, cur, 1, *grid, ff, k, cot, t_dir=t)
            assert rel(gm["cur"], go["cur"]) <= REL_L2_TOL, (grid, m_zero, t, rel(gm["cur"], go["cur"]))
            assert rel(gm["ds"], go["ds"]) <= 1e-4, (grid, m_zero, t, rel(gm["ds"], go["ds"]))
