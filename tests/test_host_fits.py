"""Host-side helpers of the studies, checked on the CPU.

* A11/A12: the viscosity of an omega (shear_wave_decay.py:162) and the omega
  of a Reynolds number (slidingLid.py:28) are inverse to each other through
  nu = u L / Re.
* The damped-cosine fit of the density-wave study (config 1) recovers the
  parameters of an analytic series exactly, and on the oracle's own FP64 run
  of a small periodic lattice gives the acoustic speed and a viscosity close
  to (1/omega - 1/2)/3.
* The log-linear shear-decay fit of the batch study (config 4)
  (shear_wave_decay.py:526: nu = -ln(a/a0) / (k^2 t)).
* The seeded uneven batch of config 4.
"""

import math

import numpy as np
import pytest

from latticeboltzmann_gb300 import batch as B
from latticeboltzmann_gb300 import studies
from latticeboltzmann_gb300.solver import omega_from_reynolds, viscosity_from_omega
from oracle import d2q9 as oracle


@pytest.mark.parametrize("re,u,n", [(10.0, 0.1, 256), (1000.0, 0.05, 1024), (137.0, 0.08, 64)])
def test_reynolds_and_viscosity_are_inverse(re, u, n):
    om = omega_from_reynolds(re, u, n)
    assert 0 < om < 2
    assert viscosity_from_omega(om) == pytest.approx(u * n / re, rel=1e-12)
    assert viscosity_from_omega(1.0) == pytest.approx(1.0 / 6.0, rel=1e-15)


def test_damped_cosine_fit_recovers_an_analytic_series():
    nx, omega = 64, 1.3
    k = 2 * math.pi / nx
    t = np.arange(0, 600, 3, dtype=np.float64)
    A, G, w, phi = 0.01, 2.1e-3, 0.97 * k / math.sqrt(3), 0.2
    a = A * np.exp(-G * t) * np.cos(w * t + phi)
    fit = studies.fit_damped_cosine(t, a, nx, omega)
    assert fit["amplitude"] == pytest.approx(A, rel=1e-6)
    assert fit["damping"] == pytest.approx(G, rel=1e-6)
    assert fit["frequency"] == pytest.approx(w, rel=1e-6)
    assert fit["nu_fit"] == pytest.approx(G / (k * k), rel=1e-6)


def test_damped_cosine_fit_on_the_oracle_density_wave():
    # a small periodic lattice, FP64 oracle, first density mode every step
    nx, ny, omega, steps = 32, 2, 1.0, 400
    f = oracle.density_wave_init(nx, ny, eps=0.01)
    x = np.arange(nx)
    mode = lambda g: (g.sum(axis=0).mean(axis=1) * np.sin(2 * np.pi * x / nx)).sum() * 2 / nx
    series = [mode(f)]
    for _ in range(steps):
        oracle.periodic_step(f, omega)
        series.append(mode(f))
    fit = studies.fit_damped_cosine(np.arange(steps + 1, dtype=np.float64), np.array(series), nx, omega)
    assert fit["cs_fit"] == pytest.approx(fit["cs_theory"], rel=2e-2)
    assert abs(fit["rel_err_nu"]) < 0.1


def test_shear_decay_fit():
    ny, nu = 48, 0.05
    k = 2 * math.pi / ny
    t = np.arange(0, 2000, 50, dtype=np.float64)
    a = 0.05 * np.exp(-nu * k * k * t)
    assert B.fit_viscosity(t, a, ny) == pytest.approx(nu, rel=1e-10)
    # samples below the noise floor are left out; fewer than three left: nan
    noisy = a.copy()
    noisy[10:] = 1e-9
    assert B.fit_viscosity(t, noisy, ny) == pytest.approx(nu, rel=1e-10)
    assert math.isnan(B.fit_viscosity(t[:2], a[:2], ny))


def test_seeded_uneven_batch():
    sizes, om = B.random_shear_batch(512, seed=0)
    again, om2 = B.random_shear_batch(512, seed=0)
    assert sizes == again and np.array_equal(om, om2)
    nx = np.array([s[0] for s in sizes])
    ny = np.array([s[1] for s in sizes])
    assert len(sizes) == 512
    assert nx.min() >= 32 and nx.max() <= 1024 and ny.min() >= 16 and ny.max() <= 512
    assert om.min() >= 0.3 and om.max() <= 1.9
    # log-uniform: the median sits near the geometric mean of the range
    assert 100 < np.median(nx) < 330 and 50 < np.median(ny) < 165


def test_surrogate_training_parameters():
    """The surrogate's data set: Re log-uniform over [10, 1000], lid speed
    uniform over [0.05, 0.1], reproducible from the seed."""
    from latticeboltzmann_gb300 import surrogate as S
    re, u = S.sample_parameters(2000, seed=0)
    re2, u2 = S.sample_parameters(2000, seed=0)
    assert np.array_equal(re, re2) and np.array_equal(u, u2)
    assert re.min() >= 10 and re.max() <= 1000 and u.min() >= 0.05 and u.max() <= 0.1
    # log-uniform: log10(Re) has mean ~2 and each decade holds about half
    assert abs(np.log10(re).mean() - 2.0) < 0.05
    assert 0.45 < (re < 100).mean() < 0.55
    assert abs(u.mean() - 0.075) < 0.002
