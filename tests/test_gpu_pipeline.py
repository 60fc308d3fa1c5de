"""The shared-memory-pipelined step kernel against the register kernel and the oracle.

Both kernels evaluate the same arithmetic on the same values, so their outputs
must agree bit for bit; the pipelined kernel's tiles (1024 FP32 cells, 2048
16-bit cells, 512 FP64 cells per row segment) are exercised with rows shorter
than, equal to and not a multiple of a tile.  The failure path is tested with a
producer that delivers nothing: the consumers' bounded waits expire, the
kernel records the timeout, and the context stays usable.
"""

import numpy as np
import pytest
import torch

import latticeboltzmann_gb300 as PyLB
from latticeboltzmann_gb300 import _lib
from oracle import d2q9 as oracle

pytestmark = pytest.mark.gpu

SIZES = [(3, 8), (17, 40), (64, 1032), (33, 2048), (7, 5000), (130, 3000), (2, 16)]


@pytest.fixture
def tuning(cuda):
    keys = [_lib.TUNE_KERNEL, _lib.TUNE_STAGES, _lib.TUNE_WAIT_LIMIT, _lib.TUNE_TEST_STALL_PRODUCER]
    saved = {k: _lib.get_tuning(k) for k in keys}
    yield _lib
    for k, v in saved.items():
        _lib.set_tuning(k, v)


def random_state(nx, ny, seed):
    rng = np.random.default_rng(seed)
    return oracle.equilibrium(1 + 0.02 * rng.standard_normal((nx, ny)), 0.03 * rng.standard_normal((nx, ny)),
                              0.03 * rng.standard_normal((nx, ny)))


def run_with(kernel, storage, boundary, f0, steps, cuda):
    _lib.set_tuning(_lib.TUNE_KERNEL, _lib.KERNELS[kernel])
    nx, ny = f0.shape[1:]
    lat = PyLB.Lattice(nx, ny, 1.45, boundary=boundary, u0=0.08, storage=storage, device=cuda)
    lat.load(torch.from_numpy(f0))
    lat.step(steps)
    torch.cuda.synchronize()
    return lat


@pytest.mark.parametrize("storage", ["f32", "f64", "f16dev", "bf16dev", "f32dev"])
@pytest.mark.parametrize("boundary", ["cavity", "cavity-ladd", "periodic"])
@pytest.mark.parametrize("nx,ny", SIZES)
def test_pipelined_equals_register_kernel(tuning, cuda, storage, boundary, nx, ny):
    f0 = random_state(nx, ny, nx * 7 + ny)
    a = run_with("register", storage, boundary, f0, 3, cuda)
    b = run_with("pipelined", storage, boundary, f0, 3, cuda)
    _lib.device_status()
    assert torch.equal(a.state, b.state)
    if storage == "f64":
        ref = f0.copy()
        for _ in range(3):
            if boundary == "cavity":
                oracle.cavity_step(ref, 1.45, 0.08)
            elif boundary == "cavity-ladd":
                oracle.cavity_ladd_step(ref, 1.45, 0.08)
            else:
                oracle.periodic_step(ref, 1.45)
        assert np.abs(b.populations().cpu().numpy() - ref).max() < 1e-13


@pytest.mark.parametrize("nx,ny", [(17, 40), (33, 2048), (130, 3000)])
@pytest.mark.parametrize("stages", [2, 3, 6])
def test_pipelined_stream_operators(tuning, cuda, nx, ny, stages):
    tuning.set_tuning(_lib.TUNE_KERNEL, _lib.KERNELS["pipelined"])
    tuning.set_tuning(_lib.TUNE_STAGES, stages)
    f0 = np.random.default_rng(ny).random((9, nx, ny))
    g = torch.from_numpy(f0).to(cuda)
    PyLB.stream(g)
    ref = f0.copy()
    oracle.stream(ref)
    np.testing.assert_array_equal(g.cpu().numpy(), ref)
    g = torch.from_numpy(f0).to(cuda)
    PyLB.Streaming.stream_and_bounce_back(g, 0.1)
    ref = f0.copy()
    oracle.stream_and_bounce_back(ref, 0.1)
    assert np.abs(g.cpu().numpy() - ref).max() < 1e-15
    _lib.device_status()


def test_timeout_is_reported_and_context_survives(tuning, cuda):
    tuning.set_tuning(_lib.TUNE_KERNEL, _lib.KERNELS["pipelined"])
    lat = PyLB.Lattice(64, 4096, 1.2, boundary="periodic", storage="f32", device=cuda)
    _lib.device_status()  # clean slate
    tuning.set_tuning(_lib.TUNE_WAIT_LIMIT, 2000)
    tuning.set_tuning(_lib.TUNE_TEST_STALL_PRODUCER, 1)
    lat.step(1)
    with pytest.raises(_lib.LBGBTimeout):
        _lib.device_status()
    # the status word was reset by the read; normal operation resumes
    tuning.set_tuning(_lib.TUNE_TEST_STALL_PRODUCER, 0)
    tuning.set_tuning(_lib.TUNE_WAIT_LIMIT, 1 << 22)
    lat2 = PyLB.Lattice(64, 4096, 1.2, boundary="periodic", storage="f32", device=cuda)
    lat2.step(2)
    _lib.device_status()
    f = lat2.populations().cpu().numpy()
    # the rest state (float32 weights) is a fixed point
    assert np.abs(f - oracle.W_I.astype(np.float32)[:, None, None]).max() == 0


@pytest.mark.parametrize("storage", ["f16dev", "bf16dev"])
@pytest.mark.parametrize("boundary", ["cavity", "periodic"])
@pytest.mark.parametrize("nx,ny", [(17, 40), (64, 1032), (130, 3000)])
def test_stochastic_rounding_kernels_agree(tuning, cuda, storage, boundary, nx, ny):
    """Stochastic rounding draws its bits from (seed, step, cell, channel):
    both kernels round every value identically."""
    f0 = random_state(nx, ny, ny)
    out = []
    for kernel in ("register", "pipelined"):
        _lib.set_tuning(_lib.TUNE_KERNEL, _lib.KERNELS[kernel])
        lat = PyLB.Lattice(nx, ny, 1.45, boundary=boundary, u0=0.08, storage=storage, device=cuda,
                           rounding="stochastic", seed=7)
        lat.load(torch.from_numpy(f0))
        lat.step(4)
        out.append(lat)
    _lib.device_status()
    assert torch.equal(out[0].state, out[1].state)
    assert int(out[0]._step_ctr.item()) == 4


@pytest.mark.parametrize("storage", ["f16dev", "bf16dev"])
def test_stochastic_rounding_is_reproducible_and_seeded(cuda, storage):
    f0 = random_state(48, 64, 1)

    def run(seed, graph=False):
        lat = PyLB.Lattice(48, 64, 1.3, boundary="cavity", u0=0.1, storage=storage, device=cuda,
                           rounding="stochastic", seed=seed)
        lat.load(torch.from_numpy(f0))
        if graph:
            replay = lat.capture(4)
            for _ in range(3):
                replay()
        else:
            lat.step(12)
        torch.cuda.synchronize()
        return lat.state.clone()

    a, b, c = run(1), run(1), run(2)
    assert torch.equal(a, b)
    assert not torch.equal(a, c)
    # graph replays advance the device step counter: same result as eager steps
    assert torch.equal(run(1, graph=True), a)
