"""Two fused steps per launch (k_step2) against two single steps.

The two-step kernel keeps the intermediate step in shared memory, stored in
the storage's own codes, and computes each cell with the single-step
kernel's arithmetic, so the populations after any number of steps equal the
single-step path's bit for bit: lattices of one and several blocks in x and
y (blocks of 16-128 rows x 128 columns, periodic block neighbours across the
seams), both wall types, FP32 and f32dev storage, even and odd step counts
(an odd count ends with one single step)."""

import numpy as np
import pytest
import torch

import latticeboltzmann_gb300 as PyLB
from latticeboltzmann_gb300 import _lib
from oracle import d2q9 as oracle

pytestmark = pytest.mark.gpu


@pytest.fixture
def two_step(cuda):
    saved = _lib.get_tuning(_lib.TUNE_TWO_STEP)
    yield
    _lib.set_tuning(_lib.TUNE_TWO_STEP, saved)


def state(nx, ny, seed):
    rng = np.random.default_rng(seed)
    f = oracle.equilibrium(1 + 0.02 * rng.standard_normal((nx, ny)), 0.04 * rng.standard_normal((nx, ny)),
                           0.04 * rng.standard_normal((nx, ny)))
    return f * (1 + 0.01 * rng.standard_normal(f.shape))


def run(nx, ny, storage, boundary, steps, two, f0, cuda):
    _lib.set_tuning(_lib.TUNE_TWO_STEP, int(two))
    lat = PyLB.Lattice(nx, ny, 1.6, boundary=boundary, u0=0.09, storage=storage, device=cuda)
    lat.load(torch.from_numpy(f0))
    spl = lat.steps_per_launch
    lat.step(steps)
    torch.cuda.synchronize()
    _lib.device_status()
    return lat.state.clone(), spl


@pytest.mark.parametrize("storage", ["f32", "f32dev"])
@pytest.mark.parametrize("boundary", ["cavity", "periodic"])
@pytest.mark.parametrize("nx,ny", [(16, 128), (16, 256), (48, 512), (32, 384), (128, 256), (160, 1024), (256, 512)])
@pytest.mark.parametrize("steps", [2, 5])
def test_two_steps_per_launch_equal_single_steps(two_step, cuda, storage, boundary, nx, ny, steps):
    f0 = state(nx, ny, nx + ny)
    a, spl_a = run(nx, ny, storage, boundary, steps, True, f0, cuda)
    b, spl_b = run(nx, ny, storage, boundary, steps, False, f0, cuda)
    assert spl_a == 2 and spl_b == 1
    assert torch.equal(a, b)


def test_steps_per_launch_where_the_kernel_does_not_apply(two_step, cuda):
    _lib.set_tuning(_lib.TUNE_TWO_STEP, 1)
    assert PyLB.Lattice(17, 256, 1.0, device=cuda).steps_per_launch == 1      # nx not a multiple of 16
    assert PyLB.Lattice(16, 250, 1.0, device=cuda).steps_per_launch == 1      # ny not a multiple of 128
    assert PyLB.Lattice(16, 256, 1.0, storage="f64", device=cuda).steps_per_launch == 1
    assert PyLB.Lattice(16, 256, 1.0, storage="f16dev", device=cuda).steps_per_launch == 1
    assert PyLB.Lattice(16, 256, 1.0, boundary="cavity-ladd", device=cuda).steps_per_launch == 1
    assert PyLB.Lattice(16, 256, 1.0, device=cuda).steps_per_launch == 2
    # a lattice where it does not apply still steps (single steps)
    f0 = state(17, 256, 3)
    a, _ = run(17, 256, "f32", "cavity", 4, True, f0, cuda)
    b, _ = run(17, 256, "f32", "cavity", 4, False, f0, cuda)
    assert torch.equal(a, b)


def test_two_step_cavity_against_the_oracle(two_step, cuda):
    """FP64 oracle steps against the FP32 two-step path: the FP32 rounding
    level after 6 steps (the same bound as the single-step kernel)."""
    nx, ny = 32, 256
    f0 = state(nx, ny, 7)
    a, spl = run(nx, ny, "f32", "cavity", 6, True, f0, cuda)
    assert spl == 2
    ref = f0.copy()
    for _ in range(6):
        oracle.cavity_step(ref, 1.6, 0.09)
    assert np.abs(a.double().cpu().numpy() - ref).max() < 2e-6
