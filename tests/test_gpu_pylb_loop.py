"""The reference's driver loops, unchanged but for numpy -> torch, through the
``PyLB`` package name.

``import PyLB as D2Q9`` and ``from PyLB.IO import save_mpiio`` are the imports
of simulators/parallel_lid_drive_cavity/cavity_opt2.py:42-43; the loop bodies
are those of cavity_opt2.py:266-283 (equilibrium start, stream and
bounce-back, collide, velocity dumps) and of
simulators/serial_shear_wave/Python/shear_wave_opt2.py:85-99 (periodic stream,
collide, shear amplitude).  The operators round like the reference's native
path, so the populations equal the oracle's C port of that path bit for bit in
float32 and float64, at a size below and above the pipelined kernel's
threshold (64K cells).
"""

import numpy as np
import pytest
import torch

import PyLB as D2Q9
from PyLB.IO import save_mpiio
from PyLB.Streaming import c_ic, stream, stream_and_bounce_back
from oracle import d2q9 as oracle
from oracle import port

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,nsteps", [(48, 60), (256, 12)])
@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_cavity_opt2_loop(cuda, tmp_path, n, nsteps, dtype):
    nx = ny = n
    omega, dump_freq = 1.7, 5
    c = torch.from_numpy(c_ic).to(device=cuda, dtype=dtype)
    f_ikl = torch.zeros((9, nx, ny), dtype=dtype, device=cuda)
    D2Q9.equilibrium(torch.ones((nx, ny), dtype=dtype, device=cuda).reshape(-1),
                     torch.zeros((nx, ny), dtype=dtype, device=cuda).reshape(-1),
                     torch.zeros((nx, ny), dtype=dtype, device=cuda).reshape(-1),
                     f_ikl.reshape(9, -1))
    ref = f_ikl.cpu().numpy().copy()
    dumps = {}
    for i in range(nsteps):
        stream_and_bounce_back(f_ikl)
        D2Q9.collide(f_ikl.reshape(9, -1), omega)
        if i % dump_freq == 0:
            rho_kl = torch.sum(f_ikl, dim=0)
            u_ckl = torch.einsum("ikl,ic->ckl", f_ikl, c) / rho_kl
            fn = str(tmp_path / ("ux_%d.npy" % i))
            save_mpiio(None, fn, u_ckl[0])
            dumps[i] = fn
    # the oracle's C port of the native path: stream + bounce-back pass, then
    # collide pass, every operation rounded on its own
    for i in range(nsteps):
        port.cavity_run(ref, omega, 0.1, 1, nthreads=0)
        if i in dumps:
            _, ux, _ = oracle.macroscopic(ref.astype(np.float64))
            got = np.load(dumps[i])
            assert got.dtype == np.dtype(str(dtype).split(".")[1]) and got.shape == (nx, ny)
            tol = 1e-6 if dtype == torch.float32 else 1e-15
            assert np.abs(got - ux).max() < tol
    np.testing.assert_array_equal(f_ikl.cpu().numpy(), ref)


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_shear_wave_opt2_loop(cuda, dtype):
    nx = ny = 64
    omega, nsteps = 1.0, 40
    x_k = torch.arange(nx, dtype=dtype, device=cuda)
    wavevector = 2 * np.pi / nx
    uy_k = torch.sin(wavevector * x_k)
    c = torch.from_numpy(c_ic).to(device=cuda, dtype=dtype)
    f_ikl = torch.arange(9 * nx * ny, dtype=dtype, device=cuda).reshape(9, nx, ny)
    D2Q9.equilibrium(torch.ones((nx, ny), dtype=dtype, device=cuda).reshape(-1),
                     torch.zeros((nx, ny), dtype=dtype, device=cuda).reshape(-1),
                     uy_k.expand(ny, nx).T.contiguous().reshape(-1),
                     f_ikl.reshape(9, -1))
    ref = f_ikl.cpu().numpy().copy()
    ampl = []
    for i in range(nsteps):
        stream(f_ikl)
        D2Q9.collide(f_ikl.reshape(9, -1), omega)
        ampl += [float(((c[:, 1] @ f_ikl[:, :, ny // 2] / f_ikl[:, :, ny // 2].sum(dim=0)) * uy_k).sum() * 2 / nx)]
    port.periodic_run(ref, omega, nsteps, nthreads=0)
    np.testing.assert_array_equal(f_ikl.cpu().numpy(), ref)
    # the reference's Fourier analysis of the (large-amplitude) shear wave
    assert np.isfinite(ampl).all() and ampl[0] > 0
