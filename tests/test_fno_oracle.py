"""The float64 FNO of the oracle: its factorised spectral convolution equals
the numpy.fft definition, and its hand-derived gradients equal central finite
differences."""

import numpy as np
import pytest

from oracle import fno


@pytest.mark.parametrize("pad", [None, (40, 32), (36, 30)])
def test_factorised_spectral_conv_equals_fft(pad):
    rng = np.random.default_rng(0)
    B, C, O, H, W, m = 2, 3, 4, 32, 24, 5
    Hp, Wp = pad if pad else (None, None)
    v = rng.standard_normal((B, C, H, W))
    Rr = rng.standard_normal((C, O, 2 * m, m))
    Ri = rng.standard_normal((C, O, 2 * m, m))
    mats = fno.dft_mats(H, W, m, Hp, Wp)
    out, _ = fno.spectral_forward(v, Rr, Ri, mats)
    ref = fno.fft_spectral_reference(v, Rr, Ri, m, Hp, Wp)
    assert np.abs(out - ref).max() < 1e-12


def test_gradients_match_finite_differences():
    rng = np.random.default_rng(1)
    H = W = 16
    m = 4
    p = fno.init_params(rng, width=6, modes=m, layers=2, hidden=10)
    a = rng.standard_normal((2, 4, H, W))
    target = rng.standard_normal((2, 3, H, W))
    mats = fno.dft_mats(H, W, m, 20, 24)
    loss, g, _ = fno.loss_and_grads(p, a, target, mats, layers=2)
    for name in ["P", "pb", "W0", "b1", "Rr0", "Ri1", "Q1", "q2b"]:
        x = p[name]
        for idx in [tuple(rng.integers(0, s) for s in x.shape) for _ in range(3)]:
            old = x[idx]
            eps = 1e-6
            x[idx] = old + eps
            lp, _, _ = fno.loss_and_grads(p, a, target, mats, layers=2)
            x[idx] = old - eps
            lm, _, _ = fno.loss_and_grads(p, a, target, mats, layers=2)
            x[idx] = old
            fd = (lp - lm) / (2 * eps)
            assert abs(fd - g[name][idx]) <= 1e-6 * max(1.0, abs(fd)), (name, idx, fd, g[name][idx])


@pytest.mark.parametrize("H,W,m,pad", [(20, 28, 5, 0.25), (256, 256, 12, 0.25), (32, 24, 4, 0.0)])
def test_product_dft_matrices_equal_oracle(H, W, m, pad):
    """The network's transform matrices and padded period (host side of
    latticeboltzmann_gb300.fno) are the oracle's."""
    from latticeboltzmann_gb300 import fno as F
    Hp, Wp = F.padded_size(H, pad), F.padded_size(W, pad)
    assert (Hp, Wp) == (fno.padded_size(H, pad), fno.padded_size(W, pad))
    assert Hp % 8 == 0 or pad == 0
    assert np.array_equal(F.ky_modes(Hp, m), fno.ky_modes(Hp, m))
    fw, G, iw = F.dft_matrices(H, W, m, Hp, Wp)
    ofw, ch, sh, oiw = fno.dft_mats(H, W, m, Hp, Wp)
    np.testing.assert_allclose(fw, ofw, atol=1e-15)
    np.testing.assert_allclose(G, np.concatenate([ch, sh]), atol=1e-15)
    np.testing.assert_allclose(iw, oiw, atol=1e-15)
