"""The CPU side's workload builders (oracle/workloads.py) give the same inputs
as the product's (pypo_gb300/configs.py), so that both arms of the benchmark
time the same problem; and the oracle's Gaussian feed matches the
reference's makeGaussBeam (golden vectors)."""
import numpy as np
import pytest

from common import GOLDEN, from_json
from oracle import grids as OG, workloads as OW


def _close(a, b, rel=1e-13):
    np.testing.assert_allclose(a, b, rtol=0, atol=rel * max(1.0, float(np.abs(b).max())))


def test_oracle_gauss_beam_matches_reference():
    g = np.load(GOLDEN / "golden_gauss.npz")
    s7 = OG.generate(from_json(str(g["plane_json"])))
    f, c = OW.gauss_beam(s7, 3.0, 10.0, 0.0, 4 * np.pi)
    _close(f, g["fields"])
    _close(c, g["currents"])
    s7b = OG.generate(OG.plane([15, 15], gmode=0, lims_a=[-20, 20]))
    _, c2 = OW.gauss_beam(s7b, 1.0, 5.0, 50.0, 1.0, mode=2)
    _close(c2, g["currents2"])


@pytest.mark.parametrize("name,scale", [("dish_eh", 1.0), ("dish_ff", 0.25), ("feed_dish_jm", 1.0)])
def test_workloads_equal_the_products(lib, name, scale):
    from pypo_gb300 import configs
    a = OW.WORKLOADS[name](scale=scale)
    b = configs.WORKLOADS[name](scale=scale)
    for key in ("mode", "gmode", "ncx", "ncy", "pairs"):
        assert a[key] == b[key], key
    assert a["k"] == b["k"]
    for key in ("s7", "t7", "cur"):
        _close(a[key], b[key])


@pytest.mark.parametrize("name", ["cassegrain", "dish_chain"])
def test_chain_stages_equal_the_products(lib, name):
    from pypo_gb300 import configs
    a = OW.CHAINS[name](scale=0.2)
    b = getattr(configs, name)(scale=0.2)
    for key, v in a.items():
        if isinstance(v, np.ndarray):
            _close(v, b[key])
        else:
            assert v == b[key], key
