"""Host-side checks that need no GPU: the C ABI library loads and exports every
symbol of include/lbgb.h, the Python signatures agree with the header, and
the operators reject what the reference's pybind11 binding rejects."""

import os
import re

import numpy as np
import pytest
import torch

import latticeboltzmann_gb300 as PyLB
from latticeboltzmann_gb300 import IO, _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    src = open(os.path.join(ROOT, "include", "lbgb.h")).read()
    return re.findall(r"^LBGB_API\s+[\w\s*]*?\b(lbgb_\w+)\s*\(", src, flags=re.M)


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(_lib.LIB_PATH):
        from latticeboltzmann_gb300 import _build
        _build.build()
    return _lib.load()


def test_header_declares_entry_points():
    names = header_symbols()
    assert len(names) >= 12
    assert set(names) == set(_lib.SIGNATURES), "Python signature table and header disagree"


def test_library_exports_every_header_symbol(lib):
    for name in header_symbols():
        assert hasattr(lib, name), name


def test_version_and_error_buffer(lib):
    assert lib.lbgb_version() >= 10000
    # an invalid call fails on the host before any CUDA work and sets a message
    rc = lib.lbgb_stream_bounce_back(None, None, 1, 1, 0.1, 0, None)
    assert rc == _lib.EINVAL
    assert "cavity" in _lib.last_error()
    rc = lib.lbgb_collide(None, 4, 4, 7, 1.0, None)
    assert rc == _lib.EDTYPE
    with pytest.raises(TypeError):
        _lib.check(rc)


def test_host_validation_before_any_launch(lib):
    rc = lib.lbgb_step_fused(1 << 20, (1 << 20) + 64, 8, 8, _lib.PERIODIC, 1.0, 0.0, _lib.F32, None)
    assert rc == _lib.EINVAL and "overlap" in _lib.last_error()
    rc = lib.lbgb_mass_momentum(1 << 20, 16, 16, _lib.F32, 1 << 24, None, 0, None)
    assert rc == _lib.EWORKSPACE
    rc = lib.lbgb_collide(None, 16, 8, _lib.F32, 1.0, None)
    assert rc == _lib.EINVAL


def test_inplace_stream_and_fused_gemm_validation_before_any_launch(lib):
    """The in-place streams and the fused GEMM reject bad arguments on the
    host, before any launch (no GPU needed)."""
    f, ws = 1 << 24, 1 << 30  # aligned fake device addresses: never dereferenced here
    need = lib.lbgb_stream_inplace_workspace_bytes(64, 64, _lib.F32)
    rc = lib.lbgb_stream_periodic_inplace(None, 64, 64, _lib.F32, ws, need, None)
    assert rc == _lib.EINVAL and "null" in _lib.last_error()
    rc = lib.lbgb_stream_periodic_inplace(f, 64, 64, 9, ws, need, None)
    assert rc == _lib.EDTYPE
    rc = lib.lbgb_stream_periodic_inplace(f, 64, 64, _lib.F32, ws, need - 1, None)
    assert rc == _lib.EINVAL and "workspace" in _lib.last_error()
    rc = lib.lbgb_stream_bounce_back_inplace(f, 64, 64, 0.1, _lib.F32, ws + 8, need, None)
    assert rc == _lib.EINVAL and "16-byte" in _lib.last_error()
    rc = lib.lbgb_stream_bounce_back_inplace(f, 1, 64, 0.1, _lib.F32, ws, need, None)
    assert rc == _lib.EINVAL and "cavity" in _lib.last_error()
    rc = lib.lbgb_stream_periodic_inplace(f + 2, 64, 64, _lib.F32, ws, need, None)
    assert rc == _lib.EINVAL and "aligned" in _lib.last_error()
    # fused GEMM: sizes, then layouts it cannot take (nothing launched)
    rc = lib.lbgb_gemm_bf16_bias_act(0, 32, 16, f, 16, 1, f, 16, ws, 32, 1.0, 0.0, None, 1, 0, None, None)
    assert rc == _lib.EINVAL
    rc = lib.lbgb_gemm_bf16_bias_act(64, 32, 16, f, 1, 64, f, 16, ws, 32, 1.0, 0.0, None, 1, 0, None, None)
    assert rc == _lib.EUNSUPPORTED
    rc = lib.lbgb_gemm_bf16_bias_act(64, 32, 16, f, 16, 1, f, 16, ws + 4, 32, 1.0, 0.0, None, 1, 0, None, None)
    assert rc == _lib.EUNSUPPORTED


def test_workspace_size_is_small(lib):
    assert 0 < lib.lbgb_mass_momentum_workspace_bytes() <= 1 << 20


@pytest.mark.parametrize("code,size", [(0, 4), (1, 8), (2, 2), (3, 2), (4, 4)])
def test_inplace_stream_workspace_bytes(lib, code, size):
    """Edge records of the in-place streams: 6 rows per 16-row tile and 6
    columns per 512-byte tile column (4.7 % of an FP32 lattice, 5.2 % FP64)."""
    nx = ny = 8192
    ty = 512 // size
    rows = 6 * (nx // 16) * ny
    cols = 6 * (ny // ty) * nx
    assert lib.lbgb_stream_inplace_workspace_bytes(nx, ny, code) == (rows + cols) * size
    assert (rows + cols) * size < 0.053 * 9 * nx * ny * size
    assert lib.lbgb_stream_inplace_workspace_bytes(1, 1, code) == (6 + 6) * size + (16 - 6 * size % 16) % 16
    assert lib.lbgb_stream_inplace_workspace_bytes(0, 5, code) == 0
    assert lib.lbgb_stream_inplace_workspace_bytes(5, 5, 9) == 0


@pytest.mark.parametrize("bad", [np.zeros((9, 16)), torch.zeros(9, 16), [0.0] * 9])
def test_no_cpu_path(bad):
    with pytest.raises(TypeError):
        PyLB.collide(bad, 1.0)
    with pytest.raises(TypeError):
        PyLB.stream(bad)
    with pytest.raises(TypeError):
        PyLB.Streaming.stream_and_bounce_back(bad)


def test_c_ic_matches_reference_layout():
    assert PyLB.Streaming.c_ic.shape == (9, 2)
    assert PyLB.Streaming.c_ic[5].tolist() == [1, 1]
    assert PyLB.Streaming.c_ic[8].tolist() == [1, -1]


def test_reynolds_relation():
    # omega = 2 Re / (6 L u + Re)  <=>  nu = u L / Re
    om = PyLB.omega_from_reynolds(1000, 0.1, 300)
    assert abs(PyLB.viscosity_from_omega(om) - 0.1 * 300 / 1000) < 1e-15


def reference_header(dtype, shape):
    # the padding rule of PyLB/IO.py:55-61, restated
    from numpy.lib.format import dtype_to_descr, magic
    m = magic(1, 0)
    d = str({"descr": dtype_to_descr(np.dtype(dtype)), "fortran_order": False, "shape": shape})
    while (len(d) + len(m) + 2) % 16 != 15:
        d += " "
    d += "\n"
    return m + np.int16(len(d)).tobytes() + d.encode("latin-1")


@pytest.mark.parametrize("dtype,shape", [(np.float64, (300, 300)), (np.float32, (7, 5)), (np.float32, (0, 3))])
def test_npy_header_layout(dtype, shape):
    h = IO.npy_header(dtype, shape)
    assert h == reference_header(dtype, shape)
    assert len(h) % 16 == 0


def test_save_npy_round_trip(tmp_path):
    a = np.arange(35, dtype=np.float32).reshape(7, 5) / 3
    fn = str(tmp_path / "ux.npy")
    IO.save_mpiio(None, fn, a)
    b = np.load(fn)
    np.testing.assert_array_equal(a, b)

    class OneRank:
        def Get_size(self):
            return 1

    IO.save_mpiio(OneRank(), fn, a.astype(np.float64))
    assert np.load(fn).dtype == np.float64

    class TwoRanks:
        def Get_size(self):
            return 2

    with pytest.raises(NotImplementedError):
        IO.save_mpiio(TwoRanks(), fn, a)


def test_reference_package_name_imports():
    """``importlib.import_module("PyLB")`` succeeds (tests/01-ImportTest.py:36-44)
    and the reference's imports (cavity_opt2.py:42-43) resolve to the GPU
    operators."""
    import importlib
    mod = importlib.import_module("PyLB")
    import PyLB as D2Q9
    from PyLB.IO import save_mpiio
    from PyLB.Streaming import c_ic, stream, stream_and_bounce_back
    assert mod is D2Q9
    assert D2Q9.collide is PyLB.collide and D2Q9.equilibrium is PyLB.equilibrium and D2Q9.stream is stream
    assert D2Q9.Collision.collide is PyLB.Collision.collide
    assert stream_and_bounce_back is PyLB.Streaming.stream_and_bounce_back
    assert save_mpiio is IO.save_mpiio
    assert c_ic.shape == (9, 2)
    # host arrays are rejected like the binding rejects a wrong type: no CPU path
    with pytest.raises(TypeError):
        D2Q9.collide(np.zeros((9, 4)), 1.0)
