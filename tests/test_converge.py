"""Grid-size convergence searches, CPU side: their restatement on the FP64
oracle (oracle/converge.py) against the reference's own System.autoConverge
and System.convergeOnTarget run on the same feed, dish and target
(tests/golden/golden_converge.npz, made by make_golden.py)."""
import numpy as np
import pytest

from oracle import converge as OC
from tests.common import GOLDEN, from_json

CASES = ["uv_xy", "uv_uv", "xy_xy", "xy_uv"]   # dish grid mode _ target grid mode


def case(key):
    """Feed grid (host), its (gmode, ncx, ncy), fields, dish, target, k of a golden case."""
    from pypo_gb300 import engine
    g = np.load(GOLDEN / "golden_converge.npz")
    feed = from_json(str(g[key + "__feed_json"]))
    f7 = engine.generate_grid(feed)
    grid = (int(feed["gmode"]), *(int(v) for v in feed["gridsize"]))
    return (g, f7, grid, g[key + "__fields"], from_json(str(g[key + "__dish_json"])),
            from_json(str(g[key + "__target_json"])), float(g[key + "__k"]))


@pytest.fixture(scope="module")
def oracle_lib():
    from oracle import oracle as O
    if not O.LIB_PATH.exists():
        O.build()
    return O.load()


@pytest.mark.parametrize("key", CASES)
def test_oracle_searches_match_reference(key, oracle_lib):
    g, f7, grid, fields, dish, tgt, k = case(key)
    size, _ = OC.auto_converge(f7, grid, fields, dish, k)
    assert np.array_equal(size, g[key + "__auto"]), (size, g[key + "__auto"])
    size, _ = OC.converge_on_target(f7, grid, fields, dish, tgt, k)
    assert np.array_equal(size, g[key + "__on_target"]), (size, g[key + "__on_target"])
