"""Precision of the fused solver against float64 runs of the oracle.

Stated tolerances (lid-driven cavity, omega = 1.7, u0 = 0.1, from rest;
relative L2 error of the velocity field against the float64 oracle, the
tolerance of the benchmark spec being 1e-6 for FP32):

* f64 storage:     populations within 1e-12 absolute of the float64 oracle
                   (64^2, 1000 steps).
* f32dev storage:  FP32 deviations h = f - w, FP32 arithmetic in the
                   momentum-exact pair form: <= 2.5e-7 after every checkpoint
                   up to 20,000 steps at 256^2 (measured 1e-7; at 1024^2 the
                   error stays below 1e-6 up to 7,500 steps and at 8192^2 up
                   to 5,000, where the unsteady flow starts to amplify
                   differences), and <= 2e-7 after 1000 steps at 64^2.
* f32 storage:     <= 1.2e-6 after 1000 steps at 64^2 and <= 1.8e-6 at 256^2
                   up to 20,000 steps: the FP32 rounding of the populations
                   f themselves (~3e-8 at 0.44) is the floor (FP64 arithmetic
                   with FP32 populations gives 9e-7 at 64^2); at most a
                   quarter of the error of the reference's own float32
                   arithmetic (cavity_opt1.py with dtype=float32, 6.2e-6).
* f16dev storage:  rel-L2(u) <= 2e-3    (half deviations f_i - w_i)
* bf16dev storage: rel-L2(u) <= 1.5e-2  (bfloat16 deviations)
"""

import numpy as np
import pytest
import torch

import latticeboltzmann_gb300 as PyLB
from oracle import d2q9 as oracle
from oracle import port

pytestmark = pytest.mark.gpu

NX, NY, OMEGA, U0, STEPS = 64, 64, 1.7, 0.1, 1000


def rel_l2_u(f, f_ref):
    _, ux, uy = oracle.macroscopic(np.asarray(f, dtype=np.float64))
    _, rx, ry = oracle.macroscopic(f_ref)
    return np.sqrt(((ux - rx) ** 2 + (uy - ry) ** 2).sum() / (rx ** 2 + ry ** 2).sum())


@pytest.fixture(scope="module")
def ref64():
    f = oracle.equilibrium(np.ones((NX, NY)), np.zeros((NX, NY)), np.zeros((NX, NY)))
    return port.cavity_run(f, OMEGA, U0, STEPS, nthreads=0)


@pytest.fixture(scope="module")
def ref32_error(ref64):
    # the reference's own float32 arithmetic (numpy, cavity_opt1.py order)
    one = np.ones((NX, NY), np.float32)
    zero = np.zeros((NX, NY), np.float32)
    f = oracle.equilibrium(one, zero, zero)
    om = np.array(OMEGA, dtype=np.float32)
    for _ in range(STEPS):
        oracle.cavity_step(f, om, U0)
    return rel_l2_u(f, ref64)


def run(storage, cuda, steps=STEPS, nx=NX, ny=NY, omega=OMEGA):
    lat = PyLB.Lattice(nx, ny, omega, boundary="cavity", u0=U0, storage=storage, device=cuda)
    lat.step(steps)
    return lat


def test_f64_matches_oracle(cuda, ref64):
    lat = run("f64", cuda)
    assert np.abs(lat.populations().cpu().numpy() - ref64).max() < 1e-12


def test_f32_error_bound(cuda, ref64, ref32_error):
    """FP32 populations: the floor is their own rounding (measured 9.5e-7)."""
    lat = run("f32", cuda)
    err = rel_l2_u(lat.populations().cpu().numpy(), ref64)
    assert err <= 1.2e-6, err
    assert err <= 0.25 * ref32_error, (err, ref32_error)


def test_f32dev_error_bound(cuda, ref64):
    """FP32 deviation storage, pair-form collision (momentum changes only by
    the final roundings): measured 9.1e-8, the rounding of the stored
    deviations (an FP64-arithmetic emulation gives 7.7e-8); the directly
    evaluated equilibrium it replaced gave 3.9e-6."""
    e32 = rel_l2_u(run("f32", cuda).populations().cpu().numpy(), ref64)
    edev = rel_l2_u(run("f32dev", cuda).populations(torch.float64).cpu().numpy(), ref64)
    assert edev <= 2e-7, edev
    assert edev <= 0.25 * e32, (edev, e32)


def test_fp32_meets_1e6_velocity_tolerance_256(cuda):
    """The stated step count: a 256^2 cavity (omega 1.7, u0 0.1, Re ~ 870)
    stays within 1e-6 relative L2 of the FP64 oracle's velocity up to 20,000
    steps in FP32-deviation storage (bound 2.5e-7, measured <= 1.07e-7 at
    every checkpoint); FP32 population storage stays within 1.8e-6 (its own
    rounding floor, measured <= 1.66e-6)."""
    n = 256
    f64 = oracle.equilibrium(np.ones((n, n)), np.zeros((n, n)), np.zeros((n, n)))
    lats = {s: run(s, cuda, steps=0, nx=n, ny=n) for s in ("f32dev", "f32")}
    done = 0
    for mark in (1000, 5000, 20000):
        port.cavity_run(f64, OMEGA, U0, mark - done, nthreads=0)
        errs = {}
        for s, lat in lats.items():
            lat.step(mark - done)
            errs[s] = rel_l2_u(lat.populations(torch.float64).cpu().numpy(), f64)
        done = mark
        assert errs["f32dev"] <= 2.5e-7, (mark, errs)
        assert errs["f32"] <= 1.8e-6, (mark, errs)


@pytest.mark.parametrize("storage,tol,mtol", [("f16dev", 2e-3, 0.05), ("bf16dev", 1.5e-2, 0.05)])
def test_16bit_deviation_storage_error_bound(cuda, ref64, storage, tol, mtol):
    """16-bit deviation storage: velocity error and mass drift against float64.

    The reference's moving lid injects mass (0.70 in this run); the 16-bit runs
    must reproduce that drift within 5%: the rest population absorbs each
    node's rounding residual (a CPU emulation of the kernels' deviation-form
    arithmetic: 0.1% for half, 0.5% for bfloat16; bfloat16 without the
    correction: 42%)."""
    lat = run(storage, cuda)
    f = lat.populations(torch.float64).cpu().numpy()
    err = rel_l2_u(f, ref64)
    assert err <= tol, (storage, err)
    m_ref = ref64.sum() - NX * NY
    m = float(lat.mass_momentum()[0]) - NX * NY
    assert abs(m - m_ref) <= mtol * abs(m_ref), (m, m_ref)


@pytest.mark.parametrize("storage", ["f32", "f16dev", "bf16dev", "f32dev"])
def test_resting_walls_conserve_mass(cuda, storage):
    """With resting walls the cavity conserves mass exactly in exact arithmetic.

    The reference's own float32 arithmetic drifts by about 1e-2 here (numpy
    order) or 1.6e-3 (native C++ order); the moment-preserving store keeps
    the drift at the rounding of one population per node and step.
    """
    lat = PyLB.Lattice(48, 40, 1.2, boundary="cavity", u0=0.0, storage=storage, device=cuda)
    rng = np.random.default_rng(3)
    rho = torch.from_numpy(1 + 0.01 * rng.standard_normal((48, 40))).to(cuda)
    lat.equilibrium(rho=rho)
    m0 = float(lat.mass_momentum()[0])
    lat.step(500)
    m1 = float(lat.mass_momentum()[0])
    # CPU emulation of the same arithmetic: f32 5e-6, f16dev 3.4e-5, bf16dev 1.1e-3
    # (deviation-form 16-bit collision with the stored-value mass fix)
    tol = {"f32": 1e-4, "f16dev": 1e-3, "bf16dev": 4e-2, "f32dev": 1e-5}[storage]
    assert abs(m1 - m0) < tol, (storage, m1 - m0)


def test_shear_wave_viscosity(cuda):
    """Velocity shear wave on a periodic lattice decays at nu = (1/omega - 1/2)/3."""
    nx, ny, omega, steps = 64, 32, 1.0, 400
    f0 = oracle.shear_wave_init(nx, ny, amplitude=0.01, along="y")
    lat = PyLB.Lattice(nx, ny, omega, boundary="periodic", storage="f64", device=cuda).load(torch.from_numpy(f0))
    k = 2 * np.pi / nx
    x = np.arange(nx)
    amps = []
    for _ in range(steps // 20):
        lat.step(20)
        _, _, uy = lat.macroscopic()
        amps.append((uy.cpu().numpy()[:, ny // 2] * np.sin(k * x)).sum() * 2 / nx)
    t = 20 * np.arange(1, len(amps) + 1)
    nu = -np.polyfit(t, np.log(amps), 1)[0] / k ** 2
    assert abs(nu - PyLB.viscosity_from_omega(omega)) / PyLB.viscosity_from_omega(omega) < 0.02


def test_density_wave_config_matches_oracle(cuda):
    """Periodic density wave 256 x 128, omega = 1.0, FP64, 10,000 steps.

    The GPU series of the first density mode equals the oracle's (C port,
    FP64) to 1e-12, and both fit the acoustic damping G = nu k^2 with
    nu within 2% of (1/omega - 1/2)/3 (the remaining 1.3% is a property of
    the lattice method at this wavenumber, identical in the oracle) and the
    sound speed within 1e-4 of 1/sqrt(3).
    """
    from latticeboltzmann_gb300 import studies
    nx, ny, omega, steps, every = 256, 128, 1.0, 10000, 10
    t, a, fit = studies.density_wave(nx, ny, omega, steps, every=every, device=cuda)
    f = oracle.density_wave_init(nx, ny, 0.01)
    k = 2 * np.pi / nx
    x = np.arange(nx)
    ref = [((f.sum(axis=0).mean(axis=1)) * np.sin(k * x)).sum() * 2 / nx]
    for _ in range(steps // every):
        port.periodic_run(f, omega, every, nthreads=0)
        ref.append(((f.sum(axis=0).mean(axis=1)) * np.sin(k * x)).sum() * 2 / nx)
    assert np.abs(np.array(ref) - a).max() < 1e-12
    assert abs(fit["rel_err_nu"]) < 0.02, fit
    assert abs(fit["cs_fit"] / fit["cs_theory"] - 1) < 1e-4, fit


@pytest.mark.parametrize("storage,tol", [("f16dev", 2e-3), ("bf16dev", 1.5e-2)])
def test_16bit_stochastic_rounding_error_bound(cuda, ref64, storage, tol):
    """Stochastic rounding of 16-bit storage (same case as above).  At 1024^2,
    omega = 1.0 it keeps the velocity error 100x lower than round-to-nearest
    after 50,000 steps; here it must meet the same bound and reproduce the
    float64 mass drift within 5% (rounding to nearest: 10% / 30%)."""
    lat = PyLB.Lattice(NX, NY, OMEGA, boundary="cavity", u0=U0, storage=storage, device=cuda,
                       rounding="stochastic", seed=11)
    lat.step(STEPS)
    err = rel_l2_u(lat.populations(torch.float64).cpu().numpy(), ref64)
    assert err <= tol, (storage, err)
    m_ref = ref64.sum() - NX * NY
    m = float(lat.mass_momentum()[0]) - NX * NY
    assert abs(m - m_ref) <= 0.05 * abs(m_ref), (m, m_ref)


@pytest.mark.gpu
def test_precision_study_rows_and_perturbed_control(cuda):
    """The precision study's rows: FP32 error against FP64 is small but not
    zero, and the FP64 control run started 1e-12 away from the reference
    separates from it (the flow amplifies differences) but stays far closer
    than FP32 after a few hundred steps of a small cavity."""
    from latticeboltzmann_gb300 import studies
    rows = studies.precision(n=48, omegas=(1.7,), steps=400, storages=("f32", "f64+perturb"), device=cuda,
                             checkpoints=(200, 400))
    assert [(r["steps"], r["storage"]) for r in rows] == [(200, "f32"), (200, "f64+perturb"), (400, "f32"),
                                                          (400, "f64+perturb")]
    for r in rows:
        assert r["fp64_finite"] and r["rel_l2_u"] is not None
    f32 = [r["rel_l2_u"] for r in rows if r["storage"] == "f32"]
    ctl = [r["rel_l2_u"] for r in rows if r["storage"] == "f64+perturb"]
    assert all(0 < e < 1e-4 for e in f32)
    assert all(0 < e < 1e-8 for e in ctl)
