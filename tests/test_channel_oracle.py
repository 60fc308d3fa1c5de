"""The channel-flow oracle (dry wall rows, pressure-periodic ghosts) against
fixtures generated from the reference's own scripts
(tests/golden/make_golden_channel.py)."""

import os

import numpy as np
import pytest

from oracle import channel

GOLD = os.path.join(os.path.dirname(__file__), "golden", "reference_channel.npz")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


def test_bounce_back_variants_bit_exact(gold):
    f = gold["bb_in"].copy()
    channel.bounce_back_walls(f, 0.1, interior=True)
    np.testing.assert_array_equal(f, gold["bb_interior_uw0.1"])
    f = gold["bb_in"].copy()
    channel.bounce_back_walls(f, 0.1, interior=False, clear=True)
    np.testing.assert_array_equal(f, gold["bb_cleared_uw0.1"])


def test_pressure_periodic(gold):
    f = gold["pp_in"].copy()
    channel.pressure_periodic(f, 1.001, 0.999)
    np.testing.assert_allclose(f, gold["pp_out"], rtol=0, atol=1e-15)


@pytest.mark.parametrize("relax", [0.5, 1.3])
def test_driver_loops(gold, relax):
    one, zero = np.ones((14, 12)), np.zeros((14, 12))
    from oracle import d2q9
    for name, step, n, start in (
            ("poiseuille", lambda f: channel.poiseuille_step(f, relax, 1.001, 0.999), 300, "eq"),
            ("couette", lambda f: channel.couette_step(f, relax, 0.1), 300, "eq")):
        f = d2q9.equilibrium(one, zero, zero) if start == "eq" else np.ones((9, 14, 12))
        for _ in range(n):
            step(f)
        ref = gold["%s_%g" % (name, relax)]
        assert np.isfinite(ref).all()
        np.testing.assert_allclose(f, ref, rtol=0, atol=1e-12, err_msg=name)
