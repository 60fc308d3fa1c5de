"""FP64 numpy Fourier neural operator -- TEST INFRASTRUCTURE ONLY.

The checker for the GPU surrogate (latticeboltzmann_gb300/fno.py): the same
architecture, the same factorisation of the spectral convolution into real
discrete-Fourier-transform products, and a backward pass derived by hand, all
in float64.  Its spectral convolution is itself checked against numpy.fft in
tests/test_fno_oracle.py.

Architecture (4 Fourier layers, width 32, 12 modes):
    v0 = P a + p                      (a: 4 input channels per grid point)
    v_{l+1} = act(W_l v_l + b_l + K_l v_l),  act = GELU for l < 3, identity for l = 3
    out = Q2 GELU(Q1 v_4 + q1) + q2   (3 output channels)
K_l: keep the Fourier modes kx < m (last axis, real transform) and
ky in [0, m) U [H-m, H) (first axis) of every channel, mix channels per mode
with complex weights R_l[c, o, ky, kx], transform back.

Layout: arrays are (B, C, H, W), W the contiguous axis.
"""

import numpy as np

SQ2PI = np.sqrt(2.0 / np.pi)


def gelu(x):
    return 0.5 * x * (1.0 + np.tanh(SQ2PI * (x + 0.044715 * x ** 3)))


def gelu_grad(x):
    t = np.tanh(SQ2PI * (x + 0.044715 * x ** 3))
    return 0.5 * (1.0 + t) + 0.5 * x * (1.0 - t * t) * SQ2PI * (1.0 + 3 * 0.044715 * x * x)


def ky_modes(H, m):
    return np.concatenate([np.arange(m), np.arange(H - m, H)])


def dft_mats(H, W, m, Hp=None, Wp=None):
    """Real matrices of the factorised transform over a zero-padded period.

    The field (H, W) is read as the corner of a (Hp, Wp) zero-padded field
    (Hp >= H, Wp >= W; default no padding) and only the H x W corner of the
    result is kept, so the convolution is not forced to be periodic over the
    cavity.  Padding costs nothing here: it only changes the frequencies.
    fw  (2m, W):  rows kx: cos(2 pi kx w/Wp), rows m+kx: -sin(...)       (forward, along W)
    ch, sh (2m, H): cos / sin(2 pi ky h/Hp) for the kept ky               (along H, both ways)
    iw  (W, 2m):  inverse along W: c_kx cos / -c_kx sin, c_0 = 1, c_kx = 2, scaled by 1/(Hp Wp)
    """
    Hp = H if Hp is None else Hp
    Wp = W if Wp is None else Wp
    w = np.arange(W)
    kx = np.arange(m)
    ang = 2 * np.pi * np.outer(kx, w) / Wp
    fw = np.concatenate([np.cos(ang), -np.sin(ang)], axis=0)
    ky = ky_modes(Hp, m)
    angh = 2 * np.pi * np.outer(ky, np.arange(H)) / Hp
    ch, sh = np.cos(angh), np.sin(angh)
    c = np.where(kx == 0, 1.0, 2.0)
    iw = np.concatenate([(c[:, None] * np.cos(ang)).T, (-c[:, None] * np.sin(ang)).T], axis=1) / (Hp * Wp)
    return fw, ch, sh, iw


def padded_size(n, pad_frac):
    """Padded period for a side of n cells: n (1 + pad_frac), rounded up to a multiple of 8."""
    return int(-(-round(n * (1 + pad_frac)) // 8) * 8) if pad_frac > 0 else n


def spectral_forward(v, Rr, Ri, mats):
    """K v for v (B, C, H, W); returns out (B, O, H, W) and the cache for backward."""
    fw, ch, sh, iw = mats
    m = fw.shape[0] // 2
    x1 = np.einsum("bchw,kw->bchk", v, fw)                 # (B,C,H,2m): [re kx | im kx]
    a, b = x1[..., :m], x1[..., m:]
    # along H with e^{-i theta}: re = a cos + b sin, im = b cos - a sin
    xr = np.einsum("bchk,yh->bcyk", a, ch) + np.einsum("bchk,yh->bcyk", b, sh)
    xi = np.einsum("bchk,yh->bcyk", b, ch) - np.einsum("bchk,yh->bcyk", a, sh)
    # complex mixing per mode: Y = sum_c R[c,o] X[c]
    yr = np.einsum("bcyk,coyk->boyk", xr, Rr) - np.einsum("bcyk,coyk->boyk", xi, Ri)
    yi = np.einsum("bcyk,coyk->boyk", xr, Ri) + np.einsum("bcyk,coyk->boyk", xi, Rr)
    # back along H with e^{+i theta}: re = yr cos - yi sin, im = yr sin + yi cos
    zr = np.einsum("boyk,yh->bohk", yr, ch) - np.einsum("boyk,yh->bohk", yi, sh)
    zi = np.einsum("boyk,yh->bohk", yr, sh) + np.einsum("boyk,yh->bohk", yi, ch)
    z = np.concatenate([zr, zi], axis=-1)                  # (B,O,H,2m)
    out = np.einsum("bohk,wk->bohw", z, iw)
    return out, (v, xr, xi)


def spectral_backward(dout, Rr, Ri, mats, cache):
    fw, ch, sh, iw = mats
    m = fw.shape[0] // 2
    v, xr, xi = cache
    dz = np.einsum("bohw,wk->bohk", dout, iw)
    dzr, dzi = dz[..., :m], dz[..., m:]
    dyr = np.einsum("bohk,yh->boyk", dzr, ch) + np.einsum("bohk,yh->boyk", dzi, sh)
    dyi = -np.einsum("bohk,yh->boyk", dzr, sh) + np.einsum("bohk,yh->boyk", dzi, ch)
    dRr = np.einsum("boyk,bcyk->coyk", dyr, xr) + np.einsum("boyk,bcyk->coyk", dyi, xi)
    dRi = -np.einsum("boyk,bcyk->coyk", dyr, xi) + np.einsum("boyk,bcyk->coyk", dyi, xr)
    dxr = np.einsum("boyk,coyk->bcyk", dyr, Rr) + np.einsum("boyk,coyk->bcyk", dyi, Ri)
    dxi = -np.einsum("boyk,coyk->bcyk", dyr, Ri) + np.einsum("boyk,coyk->bcyk", dyi, Rr)
    da = np.einsum("bcyk,yh->bchk", dxr, ch) - np.einsum("bcyk,yh->bchk", dxi, sh)
    db = np.einsum("bcyk,yh->bchk", dxr, sh) + np.einsum("bcyk,yh->bchk", dxi, ch)
    dx1 = np.concatenate([da, db], axis=-1)
    dv = np.einsum("bchk,kw->bchw", dx1, fw)
    return dv, dRr, dRi


def pointwise(W, b, v):
    return np.einsum("oc,bchw->bohw", W, v) + b[None, :, None, None]


def init_params(rng, width=32, modes=12, layers=4, hidden=128, cin=4, cout=3):
    def lin(o, i):
        s = 1.0 / np.sqrt(i)
        return rng.uniform(-s, s, (o, i)), rng.uniform(-s, s, o)
    p = {}
    p["P"], p["pb"] = lin(width, cin)
    for l in range(layers):
        p["W%d" % l], p["b%d" % l] = lin(width, width)
        s = 1.0 / (width * width)
        p["Rr%d" % l] = s * rng.uniform(0, 1, (width, width, 2 * modes, modes))
        p["Ri%d" % l] = s * rng.uniform(0, 1, (width, width, 2 * modes, modes))
    p["Q1"], p["q1b"] = lin(hidden, width)
    p["Q2"], p["q2b"] = lin(cout, hidden)
    return p


def forward(p, a, mats, layers=4):
    cache = {"a": a}
    v = pointwise(p["P"], p["pb"], a)
    cache["v0"] = v
    for l in range(layers):
        s, sc = spectral_forward(v, p["Rr%d" % l], p["Ri%d" % l], mats)
        z = pointwise(p["W%d" % l], p["b%d" % l], v) + s
        cache["s%d" % l] = sc
        cache["z%d" % l] = z
        v = gelu(z) if l < layers - 1 else z
        cache["v%d" % (l + 1)] = v
    h = pointwise(p["Q1"], p["q1b"], v)
    cache["h"] = h
    g = gelu(h)
    cache["g"] = g
    out = pointwise(p["Q2"], p["q2b"], g)
    return out, cache


def loss_and_grads(p, a, target, mats, layers=4):
    """Mean squared error and its gradient with respect to every parameter."""
    out, c = forward(p, a, mats, layers)
    diff = out - target
    loss = float(np.mean(diff ** 2))
    d = 2.0 * diff / diff.size
    g = {}

    def pw_back(W, x, dy, name_w, name_b):
        g[name_w] = np.einsum("bohw,bchw->oc", dy, x)
        g[name_b] = dy.sum(axis=(0, 2, 3))
        return np.einsum("oc,bohw->bchw", W, dy)

    dg = pw_back(p["Q2"], c["g"], d, "Q2", "q2b")
    dh = dg * gelu_grad(c["h"])
    dv = pw_back(p["Q1"], c["v%d" % layers], dh, "Q1", "q1b")
    for l in reversed(range(layers)):
        dz = dv * gelu_grad(c["z%d" % l]) if l < layers - 1 else dv
        dvs, g["Rr%d" % l], g["Ri%d" % l] = spectral_backward(dz, p["Rr%d" % l], p["Ri%d" % l], mats, c["s%d" % l])
        dv = pw_back(p["W%d" % l], c["v%d" % l], dz, "W%d" % l, "b%d" % l) + dvs
    pw_back(p["P"], c["a"], dv, "P", "pb")
    return loss, g, out


def fft_spectral_reference(v, Rr, Ri, m, Hp=None, Wp=None):
    """The same spectral convolution written with numpy.fft (for the check):
    zero-pad to (Hp, Wp), transform, mix the kept modes, transform back, crop."""
    B, C, H, W = v.shape
    Hp = H if Hp is None else Hp
    Wp = W if Wp is None else Wp
    vp = np.zeros((B, C, Hp, Wp))
    vp[:, :, :H, :W] = v
    vh = np.fft.rfft2(vp, axes=(2, 3))
    ky = ky_modes(Hp, m)
    X = vh[:, :, ky, :m]
    R = Rr + 1j * Ri
    Y = np.einsum("bcyk,coyk->boyk", X, R)
    full = np.zeros((B, R.shape[1], Hp, Wp // 2 + 1), dtype=complex)
    full[:, :, ky, :m] = Y
    return np.fft.irfft2(full, s=(Hp, Wp), axes=(2, 3))[:, :, :H, :W]
