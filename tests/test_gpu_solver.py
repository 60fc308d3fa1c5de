"""The device-resident solver: fused steps, CUDA-graph replay, storage round trips,
vector-width dispatch (row lengths that are and are not multiples of the vector
width) and full-size properties at the benchmark's grid."""

import numpy as np
import pytest
import torch

import latticeboltzmann_gb300 as PyLB
from oracle import d2q9 as oracle

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("storage", ["f32", "f64", "f16dev", "bf16dev", "f32dev"])
@pytest.mark.parametrize("boundary", ["cavity", "periodic"])
def test_graph_replay_equals_eager(cuda, storage, boundary):
    a = PyLB.Lattice(96, 72, 1.6, boundary=boundary, u0=0.1, storage=storage, device=cuda)
    b = PyLB.Lattice(96, 72, 1.6, boundary=boundary, u0=0.1, storage=storage, device=cuda)
    replay = b.capture(10)
    for _ in range(3):
        replay()
    a.step(30)
    torch.cuda.synchronize()
    assert a.steps_taken == b.steps_taken == 30
    assert torch.equal(a.state, b.state)


@pytest.mark.parametrize("storage", ["f32", "f16dev", "bf16dev", "f32dev"])
@pytest.mark.parametrize("ny", [16, 17, 24, 31, 128, 200])
def test_vector_and_scalar_paths_agree(cuda, storage, ny):
    """Row lengths that are not multiples of the vector width take the scalar
    kernel; both must match the float64 oracle equally well."""
    nx = 21
    rng = np.random.default_rng(ny)
    rho = 1 + 0.02 * rng.standard_normal((nx, ny))
    ux = 0.03 * rng.standard_normal((nx, ny))
    uy = 0.03 * rng.standard_normal((nx, ny))
    f0 = oracle.equilibrium(rho, ux, uy)
    ref = f0.copy()
    for _ in range(8):
        oracle.cavity_step(ref, 1.4, 0.1)
    lat = PyLB.Lattice(nx, ny, 1.4, boundary="cavity", u0=0.1, storage=storage, device=cuda)
    lat.load(torch.from_numpy(f0))
    lat.step(8)
    err = np.abs(lat.populations(torch.float64).cpu().numpy() - ref).max()
    tol = {"f32": 2e-6, "f16dev": 2e-4, "bf16dev": 2e-3, "f32dev": 2e-7}[storage]
    assert err < tol, err


def test_storage_round_trip(cuda):
    rng = np.random.default_rng(1)
    f = oracle.equilibrium(1 + 0.01 * rng.standard_normal((40, 48)), 0.02 * rng.standard_normal((40, 48)),
                           0.02 * rng.standard_normal((40, 48)))
    # half an ulp of |h| < 2^-5: 2^-17 in half, 2^-14 in bfloat16; f32: 2^-25 of f < 1
    # f32dev: half an ulp of |h| < 2^-5 in float, plus the rounding of f - w itself
    for storage, tol in (("f32", 3e-8), ("f16dev", 2.0 ** -17), ("bf16dev", 2.0 ** -14), ("f32dev", 2.0 ** -29)):
        lat = PyLB.Lattice(40, 48, 1.0, boundary="periodic", storage=storage, device=cuda).load(torch.from_numpy(f))
        back = lat.populations(torch.float64).cpu().numpy()
        assert np.abs(back - f).max() < tol, storage


def test_equilibrium_initialisation_is_exact_at_rest(cuda):
    lat = PyLB.Lattice(33, 20, 1.0, boundary="cavity", storage="f64", device=cuda)
    f = lat.populations().cpu().numpy()
    assert np.abs(f - oracle.W_I[:, None, None]).max() == 0
    rho, ux, uy = lat.macroscopic()
    w_sum = 0.0
    for w in oracle.W_I:  # the float64 weights do not sum to exactly 1
        w_sum += w
    assert float(rho.min()) == float(rho.max()) == w_sum and float(ux.abs().max()) == 0.0


def test_bad_configuration_rejected(cuda):
    with pytest.raises(ValueError):
        PyLB.Lattice(1, 8, 1.0, boundary="cavity", device=cuda)
    with pytest.raises(ValueError):
        PyLB.Lattice(8, 8, 1.0, storage="f8", device=cuda)
    lat = PyLB.Lattice(8, 8, 1.0, device=cuda)
    with pytest.raises(ValueError):
        lat.capture(3)
    with pytest.raises(ValueError):
        lat.load(torch.zeros(9, 8, 9))


@pytest.mark.parametrize("storage", ["f32", "f16dev", "f32dev"])
def test_full_size_cavity_properties(cuda, storage):
    """Size-independent properties at the benchmark grid (8192^2).

    * With a resting lid the rest state is an exact fixed point (bit-exact).
    * One step from rest with a moving lid: interior nodes stay at rest, the
      lid row gains x momentum 2 * u0/6 per interior column and u0/6 at each
      corner column (where the side wall overrides one Ladd term), i.e.
      (u0/3)(n-1) in total; mass and y momentum do not change.
    """
    n = 8192
    lat = PyLB.Lattice(n, n, 1.7, boundary="cavity", u0=0.0, storage=storage, device=cuda)
    s0 = lat.state.clone()
    lat.step(2)
    assert torch.equal(lat.state, s0)
    del s0, lat
    u0 = 0.1
    lat = PyLB.Lattice(n, n, 1.7, boundary="cavity", u0=u0, storage=storage, device=cuda)
    m0 = float(lat.mass_momentum()[0])
    lat.step(1)
    mass, px, py = lat.mass_momentum().cpu().numpy()
    fp32 = storage in ("f32", "f32dev")
    rel = 1e-6 if fp32 else 2e-3
    # 16-bit: every lid cell carries the same state, so the rounding of its
    # rest population (the only value not conserved exactly) repeats across
    # the 8192 columns: bound 8192 * half an ulp of |h_0| < 2^-9
    assert abs(mass - m0) < (1e-3 if fp32 else n * 2.0 ** -21)
    assert abs(px - u0 / 3 * (n - 1)) < rel * u0 / 3 * n
    # y momentum is zero in exact arithmetic; 16-bit rounding of the six
    # channels with cy != 0 repeats in every lid column: <= n * 6 * 2^-17
    assert abs(py) < (1e-3 if fp32 else n * 6 * 2.0 ** -17)


@pytest.mark.parametrize("storage", ["f32", "f64"])
@pytest.mark.parametrize("boundary", ["cavity", "cavity-ladd", "periodic"])
@pytest.mark.parametrize("nx,ny,blocks", [(64, 96, 5), (37, 40, 16), (3, 8, 16), (130, 2048, 7), (8, 8, 1)])
@pytest.mark.parametrize("copy_streams", [1, 2, 4])
def test_step_host_equals_device_step(cuda, storage, boundary, nx, ny, blocks, copy_streams):
    """The pipelined host step (row blocks; uploads, updates and downloads on
    separate streams, one or several per copy direction) gives the populations
    of the fused device step bit for bit, and leaves the device state equal."""
    rng = np.random.default_rng(nx + ny)
    f0 = oracle.equilibrium(1 + 0.01 * rng.standard_normal((nx, ny)), 0.03 * rng.standard_normal((nx, ny)),
                            0.03 * rng.standard_normal((nx, ny)))
    dt = torch.float32 if storage == "f32" else torch.float64
    a = PyLB.Lattice(nx, ny, 1.3, boundary=boundary, u0=0.07, storage=storage, device=cuda).load(torch.from_numpy(f0))
    b = PyLB.Lattice(nx, ny, 1.3, boundary=boundary, u0=0.07, storage=storage, device=cuda).load(torch.from_numpy(f0))
    host = torch.from_numpy(f0).to(dt).pin_memory()
    a.step(3)
    b.step_host(host, n=3, blocks=blocks, copy_streams=copy_streams)
    torch.cuda.synchronize()
    assert torch.equal(host, a.state.cpu())
    assert torch.equal(b.state, a.state)
    assert b.steps_taken == 3


def test_step_host_rejects_bad_buffers(cuda):
    lat = PyLB.Lattice(16, 16, 1.0, storage="f32", device=cuda)
    with pytest.raises(ValueError):
        lat.step_host(torch.zeros(9, 16, 16))  # not pinned
    with pytest.raises(ValueError):
        lat.step_host(torch.zeros(9, 16, 16, dtype=torch.float64).pin_memory())
    with pytest.raises(ValueError):
        PyLB.Lattice(16, 16, 1.0, storage="f16dev", device=cuda).step_host(torch.zeros(9, 16, 16).pin_memory())


@pytest.mark.parametrize("storage", ["bf16dev", "f16dev"])
def test_16bit_storage_at_16384(cuda, storage):
    """16-bit storage at the 16384^2 grid of the precision study (two 4.8 GB
    buffers): the rest state is an exact fixed point, and one step from rest
    with the wall-density-1 lid conserves mass to the rounding of one rest
    population per lid cell and moves x momentum 2 u0/6 per lid cell."""
    n = 16384
    lat = PyLB.Lattice(n, n, 1.7, boundary="cavity-ladd", u0=0.0, storage=storage, device=cuda)
    s0 = lat.state.clone()
    lat.step(2)
    assert torch.equal(lat.state, s0)
    del s0, lat
    u0 = 0.1
    lat = PyLB.Lattice(n, n, 1.7, boundary="cavity-ladd", u0=u0, storage=storage, device=cuda)
    m0 = float(lat.mass_momentum()[0])
    lat.step(1)
    mass, px, py = lat.mass_momentum().cpu().numpy()
    # FP16 keeps each node's mass up to the rounding of its rest population
    # (|h_0| < 2^-5: half an ulp is 2^-16 unscaled); bfloat16 (8 bits, no
    # mass fix) rounds every changed population of a lid cell (|h| < 2^-5)
    half_ulp = 2.0 ** -16 if storage == "f16dev" else 9 * 2.0 ** -14
    assert abs(mass - m0) < n * half_ulp
    assert abs(px - u0 / 3 * n) < (2e-3 if storage == "f16dev" else 1e-2) * u0 / 3 * n
    assert abs(py) < n * 6 * (2.0 ** -17 if storage == "f16dev" else 2.0 ** -13)
