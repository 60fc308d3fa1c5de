"""Parity of the CUDA operators with the oracle and the reference's golden outputs.

Tolerances: float64 kernels agree with the float64 oracle to 1e-13 absolute
(the reference's own test uses 1e-7, tests/02-CollideTest.py:102); pure data
movement (streaming, bounce-back without lid) is bit-exact; float32 kernels
agree with the float32 oracle to a few float32 ulps of the populations.
"""

import numpy as np
import pytest
import torch

import latticeboltzmann_gb300 as PyLB
from latticeboltzmann_gb300 import _lib
from oracle import d2q9 as oracle

pytestmark = pytest.mark.gpu

SIZES = [(2, 2), (2, 3), (5, 7), (8, 8), (33, 17), (24, 16), (64, 128), (37, 256), (3, 260), (130, 96)]


def T(a, dev):
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def rand_pops(rng, nx, ny, dtype=np.float64):
    return (0.02 + 0.2 * rng.random((9, nx, ny))).astype(dtype)


@pytest.mark.parametrize("shape", ["2x2", "7x5"])
def test_equilibrium_golden(cuda, golden, shape):
    rho, ux, uy = (golden["eq_in_%s_%s" % (k, shape)] for k in ("rho", "ux", "uy"))
    ref = golden["eq_out_" + shape]
    f = torch.zeros((9, rho.size), dtype=torch.float64, device=cuda)
    assert PyLB.equilibrium(T(rho.ravel(), cuda), T(ux.ravel(), cuda), T(uy.ravel(), cuda), f) is None
    assert np.abs(f.cpu().numpy().reshape(ref.shape) - ref).max() < 1e-13
    f32 = torch.zeros((9, rho.size), dtype=torch.float32, device=cuda)
    PyLB.Collision.equilibrium(*(T(a.ravel().astype(np.float32), cuda) for a in (rho, ux, uy)), f32)
    assert np.abs(f32.cpu().numpy().reshape(ref.shape) - ref).max() < 2e-6
    # the native kernel's operation order: bit for bit in both precisions
    for dt, g in ((np.float64, f), (np.float32, f32)):
        args = [a.ravel().astype(dt) for a in (rho, ux, uy)]
        np.testing.assert_array_equal(g.cpu().numpy(), oracle.equilibrium_cxx(*args))


def test_equilibrium_scalar_overload(cuda):
    e = PyLB.equilibrium(1.0, 0.05, -0.02)
    assert e.shape == (9,) and e.dtype == torch.float32 and e.is_cuda
    ref = oracle.equilibrium(np.array(1.0), np.array(0.05), np.array(-0.02))
    assert np.abs(e.cpu().numpy() - ref).max() < 1e-7
    e64 = PyLB.equilibrium(torch.tensor(1.0, dtype=torch.float64, device=cuda), 0.05, -0.02)
    assert e64.dtype == torch.float64 and np.abs(e64.cpu().numpy() - ref).max() < 1e-15
    np.testing.assert_array_equal(e64.cpu().numpy(), oracle.equilibrium_cxx(np.array(1.0), np.array(0.05),
                                                                            np.array(-0.02)))


@pytest.mark.parametrize("omega", [0.5, 1.7])
def test_collide_golden(cuda, golden, omega):
    ref = golden["col_out_%g" % omega]
    f = T(golden["col_in"], cuda)
    PyLB.collide(f.reshape(9, -1), omega)
    assert np.abs(f.cpu().numpy() - ref).max() < 1e-13


@pytest.mark.parametrize("n", [0, 1, 3, 4, 5, 17, 1000, 4099])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_collide_ragged_and_strided(cuda, n, dtype):
    rng = np.random.default_rng(n)
    f = (0.02 + 0.2 * rng.random((9, n))).astype(dtype)
    ref = f.copy()
    if n:
        oracle.collide_cxx(ref, 1.3)
    g = T(f, cuda)
    PyLB.collide(g, 1.3)
    # the native kernel's operations in its order, each rounded on its own:
    # bit for bit in float32 and float64
    if n:
        np.testing.assert_array_equal(g.cpu().numpy(), ref)
    # channel rows spaced wider than N (a view into a bigger buffer), odd stride
    big = torch.zeros((9, n + 3), dtype=g.dtype, device=cuda)
    big[:, :n] = T(f, cuda)
    view = big[:, :n]
    PyLB.collide(view, 1.3)
    if n:
        np.testing.assert_array_equal(view.cpu().numpy(), ref)
    assert (big[:, n:] == 0).all()


def _same_bits(a, b):
    """Bit-identical arrays, except that any NaN equals any NaN (the payload
    of a generated NaN differs between the host CPU and the GPU)."""
    na, nb = np.isnan(a), np.isnan(b)
    np.testing.assert_array_equal(na, nb)
    iv = np.uint32 if a.dtype == np.float32 else np.uint64
    np.testing.assert_array_equal(a[~na].view(iv), b[~nb].view(iv))


def _wide(rng, shape, dtype):
    """Magnitudes from 2^-100 to 2^100 of both signs, a quarter of typical
    populations (0.02 .. 0.22) and 1 % exact zeros."""
    f = np.where(rng.random(shape) < 0.3, -1.0, 1.0) * np.exp2(rng.uniform(-100, 100, shape))
    typical = 0.02 + 0.2 * rng.random(shape)
    pick = rng.random(shape[-1]) < 0.25
    f[..., pick] = typical[..., pick]
    f[..., rng.random(shape[-1]) < 0.01] = 0.0
    return f.astype(dtype)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_native_divisions_bit_exact_over_wide_ranges(cuda, dtype):
    """The native operators divide by 9, 36, 6 and rho through the correctly
    rounded reciprocal with Markstein's correction inside a safe operand range
    and by the IEEE division outside it (and x/2 as x*0.5): bit for bit the
    IEEE results of the numpy restatement, including signed zeros, subnormal
    and overflowing intermediates."""
    rng = np.random.default_rng(11)
    n = 1 << 20
    f = _wide(rng, (9, n), dtype)
    ref = f.copy()
    with np.errstate(all="ignore"):
        oracle.collide_cxx(ref, 1.3)
    g = T(f, cuda)
    PyLB.collide(g, 1.3)
    _same_bits(g.cpu().numpy(), ref)
    rho, ux, uy = (_wide(rng, (n,), dtype) for _ in range(3))
    out = torch.empty((9, n), dtype=g.dtype, device=cuda)
    PyLB.equilibrium(T(rho, cuda), T(ux, cuda), T(uy, cuda), out)
    with np.errstate(all="ignore"):
        _same_bits(out.cpu().numpy(), oracle.equilibrium_cxx(rho, ux, uy))


@pytest.mark.parametrize("n", [1, 5, 4099])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_collide_keep_mass_option(cuda, n, dtype):
    """keep_mass=True: the fused solver's collision.  float32 writes the rest
    population as f_0 + sum_{i>0}(f_i - f_i'), a few ulps of 1 away from the
    native value, and keeps each node's mass closer than the native order."""
    rng = np.random.default_rng(n + 7)
    f = (0.02 + 0.2 * rng.random((9, n))).astype(dtype)
    ref = f.copy()
    oracle.collide_cxx(ref, 1.3)
    g = T(f, cuda)
    PyLB.collide(g, 1.3, keep_mass=True)
    out = g.cpu().numpy()
    tol = 1e-15 if dtype == np.float64 else 6e-7
    assert np.abs(out - ref).max() < tol
    if dtype == np.float32:
        m0 = f.astype(np.float64).sum(axis=0)
        assert np.abs(out.astype(np.float64).sum(axis=0) - m0).max() <= np.abs(
            ref.astype(np.float64).sum(axis=0) - m0).max() + 1e-7
    with pytest.raises(ValueError):
        _lib.call("lbgb_collide_ex", g.data_ptr(), n, n, _lib.F32 if dtype == np.float32 else _lib.F64, 1.3, 6,
                  torch.cuda.current_stream().cuda_stream)


def test_collide_rejects_bad_dtype_and_layout(cuda):
    with pytest.raises(TypeError):
        PyLB.collide(torch.zeros((9, 8), dtype=torch.float16, device=cuda), 1.0)
    with pytest.raises(TypeError):
        PyLB.collide(torch.zeros((8, 9), device=cuda).t(), 1.0)
    with pytest.raises(ValueError):
        PyLB.collide(torch.zeros((8, 8), device=cuda), 1.0)


def test_stream_golden(cuda, golden):
    f = T(golden["stream_in"], cuda)
    PyLB.stream(f)
    np.testing.assert_array_equal(f.cpu().numpy(), golden["stream_out"])


@pytest.mark.parametrize("nx,ny", SIZES + [(1, 1), (1, 9), (9, 1)])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_stream_periodic_bit_exact(cuda, nx, ny, dtype):
    rng = np.random.default_rng(nx * 1000 + ny)
    f = rand_pops(rng, nx, ny, dtype)
    ref = f.copy()
    oracle.stream(ref)
    g = T(f, cuda)
    PyLB.stream(g)
    np.testing.assert_array_equal(g.cpu().numpy(), ref)


@pytest.mark.parametrize("key", ["sbb_%s_%s_u%s" % (d, s, u) for d in ("float64", "float32")
                                 for s in ("6x5", "8x8", "2x3") for u in ("0", "0.1")])
def test_stream_bounce_back_golden(cuda, golden, key):
    u0 = float(key.rsplit("_u", 1)[1])
    f = T(golden[key + "_in"], cuda)
    PyLB.Streaming.stream_and_bounce_back(f, u0)
    out = f.cpu().numpy()
    ref = golden[key + "_out"]
    if u0 == 0.0:
        np.testing.assert_array_equal(out, ref)  # pure data movement
    else:
        tol = 1e-15 if out.dtype == np.float64 else 1e-7
        assert np.abs(out - ref).max() < tol


@pytest.mark.parametrize("nx,ny", SIZES)
@pytest.mark.parametrize("u0", [0.0, 0.1, -0.07])
def test_stream_bounce_back_sizes(cuda, nx, ny, u0):
    rng = np.random.default_rng(7 * nx + ny)
    f = rand_pops(rng, nx, ny)
    ref = f.copy()
    oracle.stream_and_bounce_back(ref, u0)
    g = T(f, cuda)
    PyLB.Streaming.stream_and_bounce_back(g, u0)
    assert np.abs(g.cpu().numpy() - ref).max() < 1e-15
    g2 = T(f, cuda)
    if u0 == 0.0:
        PyLB.Streaming.bounce_back(g2)
    else:
        PyLB.Streaming.moving_wall(g2, u0)
    assert torch.equal(g, g2)


def test_stream_bounce_back_rejects_degenerate(cuda):
    with pytest.raises(ValueError):
        PyLB.Streaming.stream_and_bounce_back(torch.zeros((9, 1, 8), dtype=torch.float64, device=cuda))
    with pytest.raises(ValueError):
        PyLB.Streaming.stream_and_bounce_back(torch.zeros((9, 8, 1), dtype=torch.float64, device=cuda))


@pytest.mark.parametrize("dt", ["float64", "float32"])
def test_cavity_run_golden_operator_path(cuda, golden, dt):
    """The reference's cavity loop (stream_and_bounce_back + collide) through the
    drop-in operators reproduces the reference's own 200-step run."""
    nx, ny, nsteps = (int(v) for v in golden["cav_%s_cfg" % dt][:3])
    f = torch.empty((9, nx, ny), dtype=getattr(torch, dt), device=cuda)
    one = torch.ones(nx * ny, dtype=f.dtype, device=cuda)
    zero = torch.zeros(nx * ny, dtype=f.dtype, device=cuda)
    PyLB.equilibrium(one, zero, zero, f.reshape(9, -1))
    mass = []
    for _ in range(nsteps):
        PyLB.Streaming.stream_and_bounce_back(f)
        PyLB.collide(f.reshape(9, -1), 1.7)
        mass.append(PyLB.mass_momentum(f)[0])
    out = f.cpu().numpy()
    ref = golden["cav_%s_f" % dt]
    if dt == "float64":
        assert np.abs(out - ref).max() < 1e-13
        assert np.abs(torch.stack(mass).cpu().numpy() - golden["cav_float64_mass"]).max() < 1e-10
    else:
        assert np.abs(out - ref).max() < 2e-5


@pytest.mark.parametrize("boundary", ["cavity", "cavity-ladd", "periodic"])
@pytest.mark.parametrize("nx,ny", [(24, 16), (33, 17), (5, 7), (64, 128), (130, 96), (2, 2)])
def test_fused_equals_operator_sequence_f64(cuda, boundary, nx, ny):
    rng = np.random.default_rng(nx + 100 * ny)
    f = rand_pops(rng, nx, ny)
    ref = f.copy()
    for _ in range(5):
        if boundary == "cavity":
            oracle.cavity_step(ref, 1.3, 0.1)
        elif boundary == "cavity-ladd":
            oracle.cavity_ladd_step(ref, 1.3, 0.1)
        else:
            oracle.periodic_step(ref, 1.3)
    lat = PyLB.Lattice(nx, ny, 1.3, boundary=boundary, u0=0.1, storage="f64", device=cuda)
    lat.load(T(f, cuda))
    lat.step(5)
    assert np.abs(lat.populations().cpu().numpy() - ref).max() < 1e-13


@pytest.mark.parametrize("nx,ny", [(64, 128), (33, 17), (130, 96)])
def test_macroscopic_and_mass_momentum(cuda, nx, ny):
    rng = np.random.default_rng(11)
    f = rand_pops(rng, nx, ny)
    rho, ux, uy = PyLB.macroscopic(T(f, cuda))
    r_ref, ux_ref, uy_ref = oracle.macroscopic(f)
    assert np.abs(rho.cpu().numpy() - r_ref).max() < 1e-14
    assert np.abs(ux.cpu().numpy() - ux_ref).max() < 1e-14
    assert np.abs(uy.cpu().numpy() - uy_ref).max() < 1e-14
    mm = PyLB.mass_momentum(T(f, cuda)).cpu().numpy()
    ref = [f.sum(), (oracle.CX[:, None, None] * f).sum(), (oracle.CY[:, None, None] * f).sum()]
    assert np.abs(mm - ref).max() < 1e-9
    # fixed reduction order: bit-identical on repeat
    assert torch.equal(PyLB.mass_momentum(T(f, cuda)), PyLB.mass_momentum(T(f, cuda)))


def test_io_from_device(cuda, tmp_path):
    rng = np.random.default_rng(5)
    a = rng.random((13, 7)).astype(np.float32)
    fn = str(tmp_path / "uy.npy")
    PyLB.IO.save_mpiio(None, fn, T(a, cuda))
    np.testing.assert_array_equal(np.load(fn), a)


@pytest.mark.parametrize("boundary", ["periodic", "cavity", "cavity-ladd"])
@pytest.mark.parametrize("nx,ny", [(2, 2), (17, 33), (64, 40)])
@pytest.mark.parametrize("post", [0, 1])
def test_chapman_enskog_matches_oracle(cuda, boundary, nx, ny, post):
    rng = np.random.default_rng(nx * ny + post)
    rho = 1 + 0.01 * rng.standard_normal((nx, ny))
    ux, uy = 0.05 * rng.standard_normal((nx, ny)), 0.05 * rng.standard_normal((nx, ny))
    ref = oracle.chapman_enskog(rho, ux, uy, 1.37, periodic=boundary == "periodic", u0=0.08, post_collision=bool(post))
    out = torch.empty((9, nx, ny), dtype=torch.float64, device=cuda)
    r, x, y = (T(a, cuda) for a in (rho, ux, uy))
    _lib.call("lbgb_chapman_enskog", r.data_ptr(), x.data_ptr(), y.data_ptr(), out.data_ptr(), nx, ny, 1.37, 0.08,
              _lib.BOUNDARY_CODES[boundary], post, _lib.F64, torch.cuda.current_stream().cuda_stream)
    assert np.abs(out.cpu().numpy() - ref).max() < 1e-14
    # the same through the solver (post-collision form, FP32 storage)
    lat = PyLB.Lattice(nx, ny, 1.37, boundary=boundary, u0=0.08, storage="f32", device=cuda)
    lat.chapman_enskog(r, x, y)
    ref1 = oracle.chapman_enskog(rho, ux, uy, 1.37, periodic=boundary == "periodic",
                                 u0=0.08 if boundary != "periodic" else 0.0, post_collision=True)
    assert np.abs(lat.populations(torch.float64).cpu().numpy() - ref1).max() < 1e-6


@pytest.mark.parametrize("dt", ["f64", "f32"])
@pytest.mark.parametrize("nx,ny", [(64, 64), (7, 50), (3, 1)])
def test_fft_amplitude_matches_numpy(cuda, dt, nx, ny):
    """The reference's decay diagnostic 2/ny max|fft(ux[nx/2, :])|
    (shear_wave_decay.py:155-158) on the device, against numpy.fft."""
    rng = np.random.default_rng(nx * ny)
    l = np.arange(ny)
    ux = 0.05 * np.sin(2 * np.pi * 3 * l / ny)[None, :] + 0.01 * rng.standard_normal((nx, ny))
    f = oracle.equilibrium(1 + 0.01 * rng.standard_normal((nx, ny)), ux, 0.01 * rng.standard_normal((nx, ny)))
    f = f.astype(np.float64 if dt == "f64" else np.float32)
    _, u, _ = oracle.macroscopic(f.astype(np.float64))
    ref = np.max(2 / ny * np.abs(np.fft.fft(u[nx // 2, :])))
    got = float(PyLB.fft_amplitude(T(f, cuda)))
    assert abs(got - ref) <= (1e-12 if dt == "f64" else 1e-6) * max(ref, 1e-3), (got, ref)
