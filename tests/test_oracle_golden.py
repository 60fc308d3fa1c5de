"""Pins the CPU oracle (numpy restatement and C port) to the reference's own outputs.

The fixture ``tests/golden/reference_d2q9.npz`` was produced by
``tests/golden/make_golden.py`` running the reference's numpy functions
(cavity_opt1.py, cavity_opt0.py, shear_wave_opt1.py, PyLB/Streaming.py and the
oracles of tests/02-CollideTest.py) on seeded inputs.
"""

import numpy as np
import pytest

from oracle import d2q9 as oracle
from oracle import port

SBB_CASES = [(dt, sz, u) for dt in ("float64", "float32") for sz in ("6x5", "8x8", "2x3") for u in ("0", "0.1")]


@pytest.mark.parametrize("shape", ["2x2", "7x5"])
def test_equilibrium_vs_collide_test_oracle(golden, shape):
    # tests/02-CollideTest.py:94-102 compares at 1e-7 absolute
    rho, ux, uy = (golden["eq_in_%s_%s" % (k, shape)] for k in ("rho", "ux", "uy"))
    ref = golden["eq_out_" + shape]
    assert np.abs(oracle.equilibrium(rho, ux, uy) - ref).max() < 1e-15
    assert np.abs(oracle.equilibrium_cxx(rho, ux, uy) - ref).max() < 1e-15
    f = np.zeros((9, rho.size))
    port.equilibrium(rho.ravel(), ux.ravel(), uy.ravel(), f)
    assert np.abs(f.reshape(ref.shape) - ref).max() < 1e-15


@pytest.mark.parametrize("omega", [0.5, 1.7])
def test_collide_vs_collide_test_oracle(golden, omega):
    ref = golden["col_out_%g" % omega]
    a = golden["col_in"].copy()
    oracle.collide(a, omega)
    b = golden["col_in"].copy()
    oracle.collide_cxx(b.reshape(9, -1), omega)
    c = golden["col_in"].copy()
    port.collide(c.reshape(9, -1), omega)
    for x in (a, b, c):
        assert np.abs(x - ref).max() < 1e-14


@pytest.mark.parametrize("dt", ["float64", "float32"])
def test_numpy_collide_bit_exact(golden, dt):
    f = golden["npcol_%s_in" % dt].copy()
    rho, ux, uy = oracle.collide(f, np.array(1.7, dtype=dt))
    assert f.dtype == np.dtype(dt)
    np.testing.assert_array_equal(f, golden["npcol_%s_out" % dt])
    np.testing.assert_array_equal(ux, golden["npcol_%s_ux" % dt])
    np.testing.assert_array_equal(uy, golden["npcol_%s_uy" % dt])


def test_periodic_stream_bit_exact(golden):
    f = golden["stream_in"].copy()
    oracle.stream(f)
    np.testing.assert_array_equal(f, golden["stream_out"])
    g = golden["stream_in"].copy()
    port.stream(g)
    np.testing.assert_array_equal(g, golden["stream_out"])


@pytest.mark.parametrize("dt,size,u0", SBB_CASES)
def test_stream_and_bounce_back_bit_exact(golden, dt, size, u0):
    key = "sbb_%s_%s_u%s" % (dt, size, u0)
    f = golden[key + "_in"].copy()
    oracle.stream_and_bounce_back(f, float(u0))
    np.testing.assert_array_equal(f, golden[key + "_out"])
    g = golden[key + "_in"].copy()
    port.stream_and_bounce_back(g, float(u0))
    np.testing.assert_array_equal(g, golden[key + "_out"])


@pytest.mark.parametrize("dt", ["float64", "float32"])
def test_cavity_run_matches_reference_run(golden, dt):
    nx, ny, nsteps = (int(v) for v in golden["cav_%s_cfg" % dt][:3])
    one = np.ones((nx, ny), dtype=dt)
    zero = np.zeros((nx, ny), dtype=dt)
    f = oracle.equilibrium(one, zero, zero)
    mass = []
    for _ in range(nsteps):
        rho, ux, uy = oracle.cavity_step(f, np.array(1.7, dtype=dt), 0.1)
        mass.append(float(np.sum(f, dtype=np.float64)))
    # the numpy restatement reproduces the reference run bit for bit
    np.testing.assert_array_equal(f, golden["cav_%s_f" % dt])
    np.testing.assert_array_equal(np.array(mass), golden["cav_%s_mass" % dt])
    # the C port follows the native operation order: equal to rounding
    g = port.cavity_run(oracle.equilibrium(one, zero, zero), 1.7, 0.1, nsteps, nthreads=2)
    tol = 1e-13 if dt == "float64" else 5e-6
    assert np.abs(g - golden["cav_%s_f" % dt]).max() < tol


def test_moving_lid_mass_drift_is_the_references(golden):
    # the reference's lid does not conserve mass (corner overwrite + wrapped
    # lid density); the oracle must show the same drift
    m = golden["cav_float64_mass"]
    assert m[-1] - m[0] > 1e-3
    nx, ny = 24, 16
    f = oracle.equilibrium(np.ones((nx, ny)), np.zeros((nx, ny)), np.zeros((nx, ny)))
    m0 = f.sum()
    oracle.cavity_step(f, 1.7, 0.1)
    assert abs(f.sum() - m0 - (m[0] - nx * ny)) < 1e-12


@pytest.mark.parametrize("dt", ["float64", "float32"])
def test_resting_walls_conserve_mass(golden, dt):
    f = golden["cavrest_%s_f" % dt]
    m0 = float(golden["cavrest_%s_m0" % dt])
    tol = 1e-10 if dt == "float64" else 1e-3
    assert abs(float(np.sum(f, dtype=np.float64)) - m0) < tol


def test_einsum_twin_agrees(golden):
    rho, u = golden["opt0_eq_rho"], golden["opt0_eq_u"]
    assert np.abs(oracle.equilibrium(rho, u[0], u[1]) - golden["opt0_eq_out"]).max() < 1e-15


def test_shear_wave_amplitude_series(golden):
    nx, ny, nsteps = (int(v) for v in golden["shear_cfg"][:3])
    omega = float(golden["shear_cfg"][3])
    f = oracle.shear_wave_init(nx, ny, amplitude=1.0, along="y")
    uy_k = np.sin(2 * np.pi / nx * np.arange(nx))
    ampl = []
    for _ in range(nsteps):
        rho, ux, uy = oracle.periodic_step(f, omega)
        ampl.append((uy[:, ny // 2] * uy_k).sum() * 2 / nx)
    assert np.abs(np.array(ampl) - golden["shear_ampl"]).max() < 1e-13
    assert np.abs(f - golden["shear_f"]).max() < 1e-13


def test_streaming_invariants():
    # tests/simpleFlowsTest.py:176-196: a 9x9 periodic grid returns after 9 steps
    f = np.zeros((9, 9, 9))
    f[:, 4, 4] = 1
    for _ in range(9):
        oracle.stream(f)
    assert (f[:, 4, 4] == 1).all() and f.sum() == 9
    # tests/simpleFlowsTest.py:260-297: channel i moves by c_i
    for i in range(1, 9):
        g = np.zeros((9, 9, 9))
        g[i, 4, 4] = 1
        oracle.stream(g)
        assert g[i, 4 + oracle.CX[i], 4 + oracle.CY[i]] == 1


def test_chapman_enskog_beats_equilibrium_on_a_steady_cavity():
    """The oracle's Chapman-Enskog start of a converged 24x24 cavity (wall-density-1
    lid) is closer to the converged populations than the plain equilibrium
    of the same fields, in the interior and overall."""
    n, re, u = 24, 30.0, 0.05
    om = 2 * re / (6 * n * u + re)
    f = oracle.equilibrium(np.ones((n, n)), np.zeros((n, n)), np.zeros((n, n)))
    for _ in range(6000):
        oracle.cavity_ladd_step(f, om, u)
    r, ux, uy = oracle.macroscopic(f)
    feq = oracle.equilibrium(r, ux, uy)
    fce = oracle.chapman_enskog(r, ux, uy, om, periodic=False, u0=u, post_collision=True)
    inner = (slice(None), slice(2, -2), slice(2, -2))
    assert np.abs(fce - f)[inner].max() < 0.6 * np.abs(feq - f)[inner].max()
    assert np.linalg.norm(fce - f) < np.linalg.norm(feq - f)
    # a uniform flow has no gradients: CE start == equilibrium
    one = np.ones((5, 7))
    np.testing.assert_allclose(oracle.chapman_enskog(one, 0.03 * one, -0.01 * one, 1.2, periodic=True),
                               oracle.equilibrium(one, 0.03 * one, -0.01 * one), atol=1e-16)


@pytest.mark.parametrize("impl", ["numpy", "c_port"])
def test_equilibrium_moments(impl):
    """Equilibrium moments (the invariants the reference's collide tests rely
    on): sum f = rho, sum c f = rho u, and sum c_a c_b f = rho (u_a u_b +
    delta_ab / 3), in both restatements."""
    rng = np.random.default_rng(5)
    rho = 1 + 0.05 * rng.standard_normal((6, 7))
    ux, uy = 0.1 * rng.standard_normal((6, 7)), 0.1 * rng.standard_normal((6, 7))
    if impl == "numpy":
        f = oracle.equilibrium(rho, ux, uy)
    else:
        f = np.empty((9, 6, 7))
        port.equilibrium(rho.ravel(), ux.ravel(), uy.ravel(), f.reshape(9, -1), nthreads=1)
    cx, cy = oracle.CX[:, None, None], oracle.CY[:, None, None]
    assert np.allclose(f.sum(axis=0), rho, rtol=0, atol=1e-15)
    assert np.allclose((cx * f).sum(axis=0), rho * ux, rtol=0, atol=1e-15)
    assert np.allclose((cy * f).sum(axis=0), rho * uy, rtol=0, atol=1e-15)
    assert np.allclose((cx * cx * f).sum(axis=0), rho * (ux * ux + 1 / 3), rtol=0, atol=1e-14)
    assert np.allclose((cy * cy * f).sum(axis=0), rho * (uy * uy + 1 / 3), rtol=0, atol=1e-14)
    assert np.allclose((cx * cy * f).sum(axis=0), rho * ux * uy, rtol=0, atol=1e-14)
