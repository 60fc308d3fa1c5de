"""Channel-flow operators (dry wall rows, pressure-periodic ghosts) on the
device against the oracle and the reference-generated fixtures, and the
Couette / Poiseuille profiles against their analytic solutions."""

import os

import numpy as np
import pytest
import torch

from latticeboltzmann_gb300 import Channel
from oracle import channel as och
from oracle import d2q9

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden", "reference_channel.npz")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


def T(a, dev, dtype=torch.float64):
    return torch.from_numpy(np.ascontiguousarray(a)).to(device=dev, dtype=dtype)


def test_bounce_back_matches_reference_bit_exact(cuda, gold):
    f = T(gold["bb_in"], cuda)
    Channel.bounce_back(f, 0.1, interior=True)
    np.testing.assert_array_equal(f.cpu().numpy(), gold["bb_interior_uw0.1"])
    f = T(gold["bb_in"], cuda)
    Channel.bounce_back(f, 0.1, interior=False, clear=True)
    np.testing.assert_array_equal(f.cpu().numpy(), gold["bb_cleared_uw0.1"])


@pytest.mark.parametrize("ny", [2, 3, 4, 9])
@pytest.mark.parametrize("interior,clear", [(True, False), (False, True), (False, False)])
def test_bounce_back_small_heights_match_oracle(cuda, ny, interior, clear):
    rng = np.random.default_rng(ny)
    f = rng.random((9, 6, ny))
    ref = f.copy()
    och.bounce_back_walls(ref, 0.07, interior=interior, clear=clear)
    g = T(f, cuda)
    Channel.bounce_back(g, 0.07, interior=interior, clear=clear)
    np.testing.assert_array_equal(g.cpu().numpy(), ref)


def test_pressure_periodic_matches_reference(cuda, gold):
    f = T(gold["pp_in"], cuda)
    Channel.pressure_periodic(f, 1.001, 0.999)
    np.testing.assert_allclose(f.cpu().numpy(), gold["pp_out"], rtol=0, atol=1e-15)


@pytest.mark.parametrize("relax", [0.5, 1.3])
def test_driver_loops_match_reference(cuda, gold, relax):
    f = Channel.poiseuille_flow(14, 12, relax, 1.001, 0.999, 300, device=cuda)
    np.testing.assert_allclose(f.cpu().numpy(), gold["poiseuille_%g" % relax], rtol=0, atol=1e-12)
    f = Channel.couette_flow(14, 12, relax, 0.1, 300, interior=True, device=cuda)
    np.testing.assert_allclose(f.cpu().numpy(), gold["couette_%g" % relax], rtol=0, atol=1e-12)


def test_float32_channel_close_to_oracle(cuda):
    f = Channel.poiseuille_flow(20, 16, 1.1, 1.002, 0.998, 200, dtype=torch.float32, device=cuda)
    ref = d2q9.equilibrium(np.ones((20, 16)), np.zeros((20, 16)), np.zeros((20, 16)))
    for _ in range(200):
        och.poiseuille_step(ref, 1.1, 1.002, 0.998)
    assert np.abs(f.double().cpu().numpy() - ref).max() < 2e-6


def test_couette_profile_is_linear(cuda):
    """Steady Couette flow (every column bounced back): the wall lies half a
    cell outside the first and last fluid rows."""
    nx, ny, uw = 8, 34, 0.05
    f = Channel.couette_flow(nx, ny, 1.0, uw, 12000, device=cuda)
    _, ux, _ = d2q9.macroscopic(f.cpu().numpy())
    prof = ux[nx // 2, 1:-1]
    ana = Channel.couette_profile(ny, uw).numpy()
    assert np.abs(prof - ana).max() < 1e-3 * uw, np.abs(prof - ana).max()


def test_poiseuille_profile_is_parabolic(cuda):
    nx, ny, om = 42, 22, 1.0
    f = Channel.poiseuille_flow(nx, ny, om, 1.001, 0.999, 12000, device=cuda)
    _, ux, _ = d2q9.macroscopic(f.cpu().numpy())
    prof = ux[nx // 2, 1:-1]
    ana = Channel.poiseuille_profile(nx, ny, om, 1.001, 0.999).numpy()
    assert np.abs(prof - ana).max() < 0.05 * ana.max(), (prof.max(), ana.max())
    # symmetric about the channel centre
    assert np.abs(prof - prof[::-1]).max() < 1e-6 * ana.max()


@pytest.mark.parametrize("dt", [torch.float64, torch.float32])
@pytest.mark.parametrize("periodic", [True, False])
def test_solid_bounce_back_matches_oracle(cuda, dt, periodic):
    rng = np.random.default_rng(7)
    nx, ny = 23, 17
    solid = rng.random((nx, ny)) < 0.25
    f = (0.02 + 0.2 * rng.random((9, nx, ny))).astype(np.float64 if dt == torch.float64 else np.float32)
    ref = f.copy()
    och.solid_bounce_back(ref, solid, periodic=periodic)
    g = torch.from_numpy(f).to(cuda)
    Channel.solid_bounce_back(g, torch.from_numpy(solid).to(cuda), periodic=periodic)
    np.testing.assert_array_equal(g.cpu().numpy(), ref)


def test_obstacle_box_run_matches_oracle_and_keeps_mass(cuda):
    """A closed box with an obstacle, 200 steps of stream + solid bounce-back +
    collide on the device: equal to the oracle, fluid mass conserved."""
    from latticeboltzmann_gb300 import Collision, Streaming
    rng = np.random.default_rng(8)
    nx, ny = 20, 14
    solid = np.zeros((nx, ny), dtype=bool)
    solid[0, :] = solid[-1, :] = solid[:, 0] = solid[:, -1] = True
    solid[8:11, 5:9] = True
    rho = 1 + 0.01 * rng.standard_normal((nx, ny))
    ux, uy = 0.02 * rng.standard_normal((nx, ny)), 0.02 * rng.standard_normal((nx, ny))
    f = d2q9.equilibrium(rho, ux, uy)
    f[:, solid] = 0.0
    ref = f.copy()
    m0 = ref[:, ~solid].sum()
    g = torch.from_numpy(f).to(cuda)
    mask = torch.from_numpy(solid).to(cuda)
    for _ in range(200):
        d2q9.stream(ref)
        och.solid_bounce_back(ref, solid)
        ref[:, solid] = 0.0
        fl = ref[:, ~solid]
        r, x, y = d2q9.macroscopic(fl)
        ref[:, ~solid] = fl + 1.2 * (d2q9.equilibrium(r, x, y) - fl)
        Streaming.stream(g)
        Channel.solid_bounce_back(g, mask)
        g[:, mask] = 0.0
        fluid = g[:, ~mask]
        Collision.collide(fluid, 1.2)
        g[:, ~mask] = fluid
    out = g.cpu().numpy()
    assert np.abs(out - ref).max() < 1e-13
    assert abs(out[:, ~solid].sum() - m0) < 1e-11
