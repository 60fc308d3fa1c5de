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


def test_solid_mask_equals_wall_rows_for_uniform_flow():
    """For wall rows and a state uniform along x, the link-wise mask reflection
    gives the scripts' same-column wall reflection on every fluid row."""
    rng = np.random.default_rng(4)
    col = 0.02 + 0.2 * rng.random((9, 1, 10))
    f = np.repeat(col, 8, axis=1)
    solid = np.zeros((8, 10), dtype=bool)
    solid[:, 0] = solid[:, -1] = True
    a, b = f.copy(), f.copy()
    channel.bounce_back_walls(a, 0.0, interior=False)
    channel.solid_bounce_back(b, solid)
    np.testing.assert_array_equal(a[:, :, 1:-1], b[:, :, 1:-1])


def test_solid_bounce_back_conserves_fluid_mass():
    """Stream, then reflect at an obstacle and closed walls: the fluid nodes
    hold exactly the mass they held before the stream."""
    from oracle import d2q9
    rng = np.random.default_rng(5)
    nx, ny = 12, 9
    solid = np.zeros((nx, ny), dtype=bool)
    solid[0, :] = solid[-1, :] = solid[:, 0] = solid[:, -1] = True
    solid[5:7, 3:6] = True
    f = 0.02 + 0.2 * rng.random((9, nx, ny))
    f[:, solid] = 0.0
    m0 = f[:, ~solid].sum()
    d2q9.stream(f)
    channel.solid_bounce_back(f, solid, periodic=True)
    assert abs(f[:, ~solid].sum() - m0) < 1e-12
