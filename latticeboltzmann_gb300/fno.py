"""Fourier neural operator surrogate of the steady lid-driven cavity.

Maps (Re, lid speed) to steady density and velocity fields; the cavity solver
then starts from those fields in their Chapman-Enskog state instead of from
rest (the reference always starts from rest,
simulators/parallel_lid_drive_cavity/cavity_opt1.py:333-335, and has no
learned part).  Training and inference run on this package's own CUDA
kernels: the BF16 tensor-core GEMM (tcgen05, FP32 accumulation in tensor
memory) for every contraction and small element-wise kernels for the rest.

Architecture: 4 Fourier layers, width 32, 12 modes per axis, BF16 weights and
activations, FP32 accumulation, FP32 master weights updated by Adam.
    v0 = P a + p
    v_{l+1} = act(W_l v_l + b_l + K_l v_l),  act = GELU (tanh form) except after the last layer
    out = Q2 GELU(Q1 v_L + q1) + q2
K_l is the spectral convolution: the field is read as the corner of a
zero-padded (Hp, Wp) period (so the convolution is not periodic over the
cavity), the modes kx < 12 and ky in [0, 12) U [Hp-12, Hp) are mixed across
channels with complex weights, and the result is transformed back.  The real
transforms are dense products with small cos/sin matrices -- GEMMs with
2*12 = 24 or 48 columns -- so the spectral path runs on the tensor cores too.

Layout: activations are channel-major, (C, B, H, W) with W contiguous, so
that a pointwise layer is one GEMM over N = B*H*W columns and the transform
along W is one GEMM over C*B*H rows.  For a cavity, H is the x axis (nx) and
W the y axis (ny, the lid at the last index), matching the (nx, ny) fields of
the solver.

Inputs (4 channels): x and y cell-centre coordinates in (0, 1), log Re and
the lid speed, each scaled to [-1, 1] over the training ranges.  Outputs
(3 channels): (rho - 1) / u0^2, ux / u0, uy / u0.
"""

import json
import math

import numpy as np
import torch

from . import _lib

# GEMM engines: tensor cores (the TMA pipeline where both operands are
# K-major, else the staged kernel), CUDA cores, the staged tensor-core kernel
ENGINE_TENSOR_CORES, ENGINE_CUDA_CORES, ENGINE_STAGED = 0, 1, 2
RE_RANGE = (10.0, 1000.0)
U_RANGE = (0.05, 0.1)


def padded_size(n, pad_frac):
    """Padded period of a side of n cells: n (1 + pad_frac) rounded up to a multiple of 8."""
    return int(-(-round(n * (1 + pad_frac)) // 8) * 8) if pad_frac > 0 else n


def ky_modes(hp, m):
    return np.concatenate([np.arange(m), np.arange(hp - m, hp)])


def dft_matrices(H, W, m, Hp, Wp):
    """(fw (2m, W), G (4m, H), iw (W, 2m)) in float64.

    fw rows kx: cos(2 pi kx w / Wp), rows m + kx: -sin(...): the forward
    transform along W; G rows: cos(2 pi ky h / Hp) for the 2m kept ky, then
    the sines: both transforms along H; iw: the inverse along W of a real
    field (weights 1 for kx = 0, else 2) with the 1 / (Hp Wp) normalisation.
    """
    kx = np.arange(m)
    ang = 2 * np.pi * np.outer(kx, np.arange(W)) / Wp
    fw = np.concatenate([np.cos(ang), -np.sin(ang)], axis=0)
    angh = 2 * np.pi * np.outer(ky_modes(Hp, m), np.arange(H)) / Hp
    G = np.concatenate([np.cos(angh), np.sin(angh)], axis=0)
    c = np.where(kx == 0, 1.0, 2.0)
    iw = np.concatenate([(c[:, None] * np.cos(ang)).T, (-c[:, None] * np.sin(ang)).T], axis=1) / (Hp * Wp)
    return fw, G, iw


def _ptr(t, offset=0):
    return t.data_ptr() + offset * t.element_size()


class FNO2d:
    """The surrogate network, its training step and its inference.

    Parameters live in one flat FP32 buffer (with a BF16 copy for the GEMMs
    and Adam moments beside it), so that one kernel launch updates them all.
    """

    def __init__(self, width=32, modes=12, layers=4, hidden=128, cin=4, cout=3, pad=0.25, device=None, seed=0,
                 engine=ENGINE_TENSOR_CORES, max_splits=1024):
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        if self.device.type != "cuda":
            raise TypeError("FNO2d runs on a CUDA device (there is no CPU path)")
        _lib.load()
        self.width, self.modes, self.layers, self.hidden, self.cin, self.cout = width, modes, layers, hidden, cin, cout
        self.pad, self.engine = float(pad), int(engine)
        if max_splits < 1 or max_splits & (max_splits - 1):
            raise ValueError("max_splits must be a power of two")
        self.max_splits = int(max_splits)  # weight gradients: split-K count over the pixels
        # bias + activation in the epilogue of each layer's last GEMM (tensor-
        # core engine; 16 x 256^2: training step 3.95 against 4.03 ms, forward
        # 1.54 against 1.62 ms with a separate pass)
        self.fused_epilogue = True
        shapes = [("P", (width, cin)), ("pb", (width,))]
        for l in range(layers):
            shapes += [("W%d" % l, (width, width)), ("b%d" % l, (width,)),
                       ("Rr%d" % l, (width, width, 2 * modes, modes)), ("Ri%d" % l, (width, width, 2 * modes, modes))]
        shapes += [("Q1", (hidden, width)), ("q1b", (hidden,)), ("Q2", (cout, hidden)), ("q2b", (cout,))]
        self.shapes = dict(shapes)
        self.offsets, off = {}, 0
        for name, shp in shapes:
            self.offsets[name] = off
            off += -(-int(np.prod(shp)) // 8) * 8  # every tensor starts on 16 bytes of its BF16 copy
        self.numel = off
        f32 = dict(dtype=torch.float32, device=self.device)
        self.flat = torch.zeros(off, **f32)
        self.grad = torch.zeros(off, **f32)
        self.m = torch.zeros(off, **f32)
        self.v = torch.zeros(off, **f32)
        self.flat_bf16 = torch.zeros(off, dtype=torch.bfloat16, device=self.device)
        self.adam_steps = 0
        self.out_scale = np.ones(cout)  # network output c is target channel c / out_scale[c]
        self._mats, self._ws = {}, {}
        self.init_params(np.random.default_rng(seed))

    # ------------------------------------------------------------ parameters
    def view(self, name, buf=None):
        buf = self.flat if buf is None else buf
        o = self.offsets[name]
        shp = self.shapes[name]
        return buf[o:o + int(np.prod(shp))].view(shp)

    def init_params(self, rng):
        """Uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) for the pointwise layers, and
        spectral weights uniform in [0, 1/width^2) (the usual FNO scales)."""
        p = {}
        for name, shp in self.shapes.items():
            if name.startswith("R"):
                p[name] = rng.uniform(0, 1.0 / (self.width * self.width), shp)
            else:
                fan_in = {"P": self.cin, "pb": self.cin, "Q1": self.width, "q1b": self.width, "Q2": self.hidden,
                          "q2b": self.hidden}.get(name, self.width)
                s = 1.0 / math.sqrt(fan_in)
                p[name] = rng.uniform(-s, s, shp)
        self.load_params(p)

    def load_params(self, params):
        for name, x in params.items():
            self.view(name).copy_(torch.as_tensor(np.asarray(x), dtype=torch.float32))
        self._refresh_bf16()
        return self

    def params(self):
        """Parameters as float64 numpy arrays, keyed like the shapes."""
        return {name: self.view(name).double().cpu().numpy() for name in self.shapes}

    def grads(self):
        return {name: self.view(name, self.grad).double().cpu().numpy() for name in self.shapes}

    def _refresh_bf16(self):
        _lib.call("lbgb_fno_to_bf16", self.flat.data_ptr(), self.flat_bf16.data_ptr(), self.numel, self._s())

    def _s(self):
        return torch.cuda.current_stream(self.device).cuda_stream

    def state_dict(self):
        return {"config": dict(width=self.width, modes=self.modes, layers=self.layers, hidden=self.hidden,
                               cin=self.cin, cout=self.cout, pad=self.pad),
                "params": self.params(), "adam_steps": self.adam_steps}

    def save(self, path, bf16=False, meta=None):
        """Weights, configuration and output scales in one .npz file.

        bf16=True stores the matrices as the BF16 values the GEMMs compute
        with and the biases (used in FP32) as they are: half the size, and
        inference from the file equals the trained network's; FP32 masters
        otherwise.  ``meta``: a JSON-serialisable dict stored beside them
        (e.g. the held-out cases of the training run)."""
        sd = self.state_dict()
        extra = {"meta": json.dumps(meta)} if meta is not None else {}
        if bf16:
            bits = lambda v: torch.from_numpy(v.astype(np.float32)).to(torch.bfloat16).view(torch.int16).numpy()
            params = {("b_" + k if v.ndim >= 2 else "p_" + k): (bits(v) if v.ndim >= 2 else v.astype(np.float32))
                      for k, v in sd["params"].items()}
        else:
            params = {"p_" + k: v.astype(np.float32) for k, v in sd["params"].items()}
        np.savez(path, config=json.dumps(sd["config"]), out_scale=np.asarray(self.out_scale, dtype=np.float64),
                 **extra, **params)

    @classmethod
    def load(cls, path, device=None, engine=ENGINE_TENSOR_CORES):
        z = np.load(path)
        net = cls(device=device, engine=engine, **json.loads(str(z["config"])))
        net.out_scale = np.asarray(z["out_scale"], dtype=np.float64)
        params = {k[2:]: z[k] for k in z.files if k.startswith("p_")}
        for k in z.files:
            if k.startswith("b_"):
                params[k[2:]] = torch.from_numpy(z[k]).view(torch.bfloat16).float().numpy()
        net.meta = json.loads(str(z["meta"])) if "meta" in z.files else None
        return net.load_params(params)

    # ------------------------------------------------------------ plumbing
    def _gemm(self, m, n, k, A, a, B, b, C, c, batch=1, beta=0.0, bf16_out=False):
        _lib.call("lbgb_gemm_bf16", m, n, k, A, a[0], a[1], a[2], B, b[0], b[1], b[2], C, c[0], c[1], c[2], batch,
                  1.0, beta, int(bf16_out), self.engine, self._s())

    def _gemm_bias_act(self, m, n, k, A, a, B, b_cs, C, c_rs, bias, rows_per_bias, channels, cols, act, vb):
        """C = A B + C, C += bias per channel (rows_per_bias rows of C each),
        vb = BF16(act(C)): with ``fused_epilogue`` (default) one launch of the
        TMA pipeline when it takes the operands, else the GEMM and
        lbgb_fno_bias_act."""
        s = self._s()
        if self.engine == ENGINE_TENSOR_CORES and self.fused_epilogue:
            rc = _lib.load().lbgb_gemm_bf16_bias_act(m, n, k, A, a[0], a[1], B, b_cs, C, c_rs, 1.0, 1.0, bias,
                                                     rows_per_bias, act, vb, s)
            if rc != _lib.EUNSUPPORTED:
                _lib.check(rc, "lbgb_gemm_bf16_bias_act")
                return
        self._gemm(m, n, k, A, (a[0], a[1], 0), B, (1, b_cs, 0), C, (c_rs, 1, 0), beta=1.0)
        _lib.call("lbgb_fno_bias_act", C, bias, None, None, vb, channels, cols, act, s)

    def _splits(self, K):
        """Split count of a weight gradient over K pixels: the largest power of
        two up to ``max_splits`` that divides K and leaves >= 256 per split."""
        s = self.max_splits
        while s > 1 and (K % s or K // s < 256):
            s //= 2
        return s

    def _wgrad(self, M, Nn, K, A, B, dst, c_rs, c_cs, ws):
        """dst (M x Nn) = A (M x K, K contiguous) @ B^T (B: Nn x K, K contiguous),
        split along K into batched partial products and then summed."""
        S = self._splits(K)
        ks = K // S
        parts = ws["parts"]
        self._gemm(M, Nn, ks, A, (K, 1, ks), B, (1, K, ks), _ptr(parts), (c_rs, c_cs, M * Nn), batch=S)
        _lib.call("lbgb_fno_sum_splits", _ptr(parts), dst, S, M * Nn, 0.0, self._s())

    def matrices(self, H, W):
        key = (H, W)
        if key not in self._mats:
            Hp, Wp = padded_size(H, self.pad), padded_size(W, self.pad)
            if Hp < 2 * self.modes or Wp // 2 + 1 < self.modes:
                raise ValueError("grid %dx%d too small for %d modes" % (H, W, self.modes))
            fw, G, iw = dft_matrices(H, W, self.modes, Hp, Wp)
            # G and iw also transposed: the backward products that read them
            # along their other axis then have both operands K-major (the
            # GEMM's TMA pipeline)
            self._mats[key] = tuple(torch.as_tensor(x, dtype=torch.bfloat16, device=self.device).contiguous()
                                    for x in (fw, G, iw, G.T, iw.T))
        return self._mats[key]

    def _workspace(self, B, H, W, train):
        key = (B, H, W, train)
        if key in self._ws:
            return self._ws[key]
        # keep at most a couple of shapes alive
        if len(self._ws) > 2:
            self._ws.clear()
        N = B * H * W
        C, L, m = self.width, self.layers, self.modes
        q2, m2 = 4 * m, 2 * m
        bf = dict(dtype=torch.bfloat16, device=self.device)
        f32 = dict(dtype=torch.float32, device=self.device)
        ws = {"ab": torch.empty(self.cin, N, **bf),
              "vb": [torch.empty(C, N, **bf) for _ in range(L + 1)],
              "z": [torch.empty(C, N, **f32) for _ in range(L if train else 1)],
              "Pm": [torch.empty(C * B * m2 * q2, **f32) for _ in range(L if train else 1)],
              "X1p": torch.empty(C * B * m2 * H, **bf),
              "Ym": torch.empty(C * B * q2 * m2, **bf),
              "Z": torch.empty(C * B * H * m2, **bf),
              "h": torch.empty(self.hidden, N, **f32),
              "gb": torch.empty(self.hidden, N, **bf),
              "out": torch.empty(self.cout, N, **f32)}
        if train:
            ws.update({"d": torch.empty(self.cout, N, **f32), "db": torch.empty(self.cout, N, **bf),
                       "dh": torch.empty(self.hidden, N, **f32), "dhb": torch.empty(self.hidden, N, **bf),
                       "dv": torch.empty(C, N, **f32),
                       "dzb": torch.empty(C, N, **bf), "dYm": torch.empty(C * B * q2 * m2, **f32),
                       "dP": torch.empty(C * B * m2 * q2, **bf),
                       "parts": torch.empty(self.max_splits * max(self.hidden * C, C * C, C * self.cin,
                                                                    self.cout * self.hidden), **f32),
                       "mse": torch.empty(1024, dtype=torch.float64, device=self.device),
                       "rowsum": torch.empty(64 * max(self.hidden, C, self.cout), **f32)})
        self._ws[key] = ws
        return ws

    # ------------------------------------------------------------ network
    def forward(self, a, train=False):
        """a: float32 (cin, B, H, W) on the device -> float32 (cout, B, H, W)."""
        if a.dtype != torch.float32 or a.dim() != 4 or a.shape[0] != self.cin or not a.is_contiguous():
            raise ValueError("expected a contiguous float32 (%d, B, H, W) input" % self.cin)
        _, B, H, W = a.shape
        N = B * H * W
        ws = self._workspace(B, H, W, train)
        self._shape = (B, H, W)
        fw, G, iw, _, _ = self.matrices(H, W)
        C, m = self.width, self.modes
        q2, m2 = 4 * m, 2 * m
        s = self._s()
        pb = self.flat_bf16
        _lib.call("lbgb_fno_to_bf16", a.data_ptr(), ws["ab"].data_ptr(), a.numel(), s)
        z0 = ws["z"][0]
        # lifting: v0 = P a + p
        self._gemm(N, C, self.cin, _ptr(ws["ab"]), (1, N, 0), _ptr(pb, self.offsets["P"]), (1, self.cin, 0),
                   _ptr(z0), (1, N, 0))
        _lib.call("lbgb_fno_bias_act", _ptr(z0), _ptr(self.flat, self.offsets["pb"]), None, None,
                  _ptr(ws["vb"][0]), C, N, 0, s)
        for l in range(self.layers):
            v = ws["vb"][l]
            z = ws["z"][l] if train else ws["z"][0]
            Pm = ws["Pm"][l] if train else ws["Pm"][0]
            # pointwise branch: z = W_l v
            self._gemm(N, C, C, _ptr(v), (1, N, 0), _ptr(pb, self.offsets["W%d" % l]), (1, C, 0), _ptr(z), (1, N, 0))
            # spectral branch: W-transform (per channel-sample plane), written as (C, B, 2m, H)
            self._gemm(H, m2, W, _ptr(v), (W, 1, H * W), _ptr(fw), (1, W, 0), _ptr(ws["X1p"]), (1, H, m2 * H),
                       batch=C * B, bf16_out=True)
            # H-transform of every (c, b, kx part) row: P (C, B, 2m, 4m)
            self._gemm(C * B * m2, q2, H, _ptr(ws["X1p"]), (H, 1, 0), _ptr(G), (1, H, 0), _ptr(Pm), (q2, 1, 0))
            _lib.call("lbgb_fno_mix", _ptr(Pm), _ptr(pb, self.offsets["Rr%d" % l]), _ptr(pb, self.offsets["Ri%d" % l]),
                      _ptr(ws["Ym"]), C, C, B, 2 * m, m, s)
            # inverse along H: Z (C, B, H, 2m)
            self._gemm(H, m2, q2, _ptr(G), (1, H, 0), _ptr(ws["Ym"]), (m2, 1, q2 * m2), _ptr(ws["Z"]),
                       (m2, 1, H * m2), batch=C * B, bf16_out=True)
            # inverse along W, added onto the pointwise branch, then bias and
            # activation (in the GEMM's epilogue where the TMA pipeline runs)
            self._gemm_bias_act(C * B * H, W, m2, _ptr(ws["Z"]), (m2, 1), _ptr(iw), m2, _ptr(z), W,
                                _ptr(self.flat, self.offsets["b%d" % l]), B * H, C, N, int(l < self.layers - 1),
                                _ptr(ws["vb"][l + 1]))
        # projection
        h = ws["h"]
        self._gemm(N, self.hidden, C, _ptr(ws["vb"][self.layers]), (1, N, 0), _ptr(pb, self.offsets["Q1"]),
                   (1, C, 0), _ptr(h), (1, N, 0))
        _lib.call("lbgb_fno_bias_act", _ptr(h), _ptr(self.flat, self.offsets["q1b"]), None, None, _ptr(ws["gb"]),
                  self.hidden, N, 1, s)
        out = ws["out"]
        self._gemm(N, self.cout, self.hidden, _ptr(ws["gb"]), (1, N, 0), _ptr(pb, self.offsets["Q2"]),
                   (1, self.hidden, 0), _ptr(out), (1, N, 0))
        _lib.call("lbgb_fno_bias_act", _ptr(out), _ptr(self.flat, self.offsets["q2b"]), None, None, None,
                  self.cout, N, 0, s)
        return out.view(self.cout, B, H, W)

    def loss_and_backward(self, a, target, weight=None):
        """Mean squared error of forward(a) against target (cout, B, H, W) and
        its gradient with respect to every parameter into ``self.grad``.
        ``weight``: optional contiguous float32 (cout, B) device tensor, a
        weight per (channel, sample) plane.  Returns the loss as a device
        scalar (float64)."""
        out = self.forward(a, train=True)
        B, H, W = self._shape
        N = B * H * W
        ws = self._ws[(B, H, W, True)]
        if target.shape != out.shape or target.dtype != torch.float32 or not target.is_contiguous():
            raise ValueError("target must be a contiguous float32 tensor of shape %s" % (tuple(out.shape),))
        s = self._s()
        nparts = 1024
        if weight is None:
            _lib.call("lbgb_fno_mse", _ptr(out), _ptr(target), _ptr(ws["d"]), _ptr(ws["mse"]), nparts, out.numel(),
                      s)
        else:
            if (tuple(weight.shape) != (self.cout, B) or weight.dtype != torch.float32 or not weight.is_contiguous()
                    or weight.device != out.device):
                raise ValueError("weight must be a contiguous float32 (%d, %d) device tensor" % (self.cout, B))
            _lib.call("lbgb_fno_mse_weighted", _ptr(out), _ptr(target), _ptr(weight), H * W, _ptr(ws["d"]),
                      _ptr(ws["mse"]), nparts, out.numel(), s)
        loss = ws["mse"].sum() / out.numel()
        self.backward(ws["d"])
        return loss

    def backward(self, d):
        """Gradients from d = dLoss/dout (cout, N) FP32 of the last training forward."""
        B, H, W = self._shape
        N = B * H * W
        ws = self._ws[(B, H, W, True)]
        fw, G, iw, Gt, iwt = self.matrices(H, W)
        C, m, hid = self.width, self.modes, self.hidden
        q2, m2 = 4 * m, 2 * m
        s = self._s()
        pb, g = self.flat_bf16, self.grad
        o = self.offsets
        _lib.call("lbgb_fno_to_bf16", _ptr(d), _ptr(ws["db"]), self.cout * N, s)
        # out = Q2 g + q2
        self._wgrad(hid, self.cout, N, _ptr(ws["gb"]), _ptr(ws["db"]), _ptr(g, o["Q2"]), 1, hid, ws)
        _lib.call("lbgb_fno_row_sum", _ptr(d), _ptr(g, o["q2b"]), _ptr(ws["rowsum"]), self.cout, N, s)
        dh = ws["dh"]
        self._gemm(N, hid, self.cout, _ptr(ws["db"]), (1, N, 0), _ptr(pb, o["Q2"]), (hid, 1, 0), _ptr(dh), (1, N, 0))
        _lib.call("lbgb_fno_gelu_back", _ptr(dh), _ptr(ws["h"]), _ptr(dh), _ptr(ws["dhb"]), hid * N, s)
        # h = Q1 v_L + q1
        self._wgrad(hid, C, N, _ptr(ws["dhb"]), _ptr(ws["vb"][self.layers]), _ptr(g, o["Q1"]), C, 1, ws)
        _lib.call("lbgb_fno_row_sum", _ptr(dh), _ptr(g, o["q1b"]), _ptr(ws["rowsum"]), hid, N, s)
        dv = ws["dv"]
        self._gemm(N, C, hid, _ptr(ws["dhb"]), (1, N, 0), _ptr(pb, o["Q1"]), (C, 1, 0), _ptr(dv), (1, N, 0))
        dzb = ws["dzb"]
        for l in reversed(range(self.layers)):
            if l == self.layers - 1:
                _lib.call("lbgb_fno_to_bf16", _ptr(dv), _ptr(dzb), C * N, s)
            else:
                _lib.call("lbgb_fno_gelu_back", _ptr(dv), _ptr(ws["z"][l]), _ptr(dv), _ptr(dzb), C * N, s)
            v = ws["vb"][l]
            self._wgrad(C, C, N, _ptr(dzb), _ptr(v), _ptr(g, o["W%d" % l]), C, 1, ws)
            _lib.call("lbgb_fno_row_sum", _ptr(dv), _ptr(g, o["b%d" % l]), _ptr(ws["rowsum"]), C, N, s)
            # spectral branch, transposed step by step
            self._gemm(C * B * H, m2, W, _ptr(dzb), (W, 1, 0), _ptr(iwt), (1, W, 0), _ptr(ws["Z"]), (m2, 1, 0),
                       bf16_out=True)
            self._gemm(q2, m2, H, _ptr(G), (H, 1, 0), _ptr(ws["Z"]), (m2, 1, H * m2), _ptr(ws["dYm"]),
                       (m2, 1, q2 * m2), batch=C * B)
            _lib.call("lbgb_fno_mix_back", _ptr(ws["dYm"]), _ptr(ws["Pm"][l]), _ptr(pb, o["Rr%d" % l]),
                      _ptr(pb, o["Ri%d" % l]), _ptr(ws["dP"]), _ptr(g, o["Rr%d" % l]), _ptr(g, o["Ri%d" % l]),
                      C, C, B, 2 * m, m, s)
            self._gemm(C * B * m2, H, q2, _ptr(ws["dP"]), (q2, 1, 0), _ptr(Gt), (1, q2, 0), _ptr(ws["X1p"]),
                       (H, 1, 0), bf16_out=True)
            # pointwise branch: dv = W^T dz, then the spectral branch's input gradient on top
            self._gemm(N, C, C, _ptr(dzb), (1, N, 0), _ptr(pb, o["W%d" % l]), (C, 1, 0), _ptr(dv), (1, N, 0))
            self._gemm(H, W, m2, _ptr(ws["X1p"]), (1, H, m2 * H), _ptr(fw), (W, 1, 0), _ptr(dv), (W, 1, H * W),
                       batch=C * B, beta=1.0)
        # lifting
        _lib.call("lbgb_fno_to_bf16", _ptr(dv), _ptr(dzb), C * N, s)
        self._wgrad(C, self.cin, N, _ptr(dzb), _ptr(ws["ab"]), _ptr(g, o["P"]), self.cin, 1, ws)
        _lib.call("lbgb_fno_row_sum", _ptr(dv), _ptr(g, o["pb"]), _ptr(ws["rowsum"]), C, N, s)

    def adam(self, lr, b1=0.9, b2=0.999, eps=1e-8, weight_decay=0.0):
        """One Adam step on the FP32 master weights; refreshes the BF16 copy."""
        self.adam_steps += 1
        _lib.call("lbgb_fno_adam", _ptr(self.flat), _ptr(self.grad), _ptr(self.m), _ptr(self.v),
                  _ptr(self.flat_bf16), self.numel, lr, b1, b2, eps, self.adam_steps, weight_decay, self._s())

    # ------------------------------------------------------------ cavity use
    def inputs(self, re, u_lid, nx, ny):
        """Input channels (4, B, nx, ny) for lid-driven cavities (re[b], u_lid[b])."""
        re = torch.as_tensor(np.atleast_1d(re), dtype=torch.float32, device=self.device)
        u = torch.as_tensor(np.atleast_1d(u_lid), dtype=torch.float32, device=self.device)
        B = re.numel()
        a = torch.empty(self.cin, B, nx, ny, dtype=torch.float32, device=self.device)
        a[0] = ((torch.arange(nx, device=self.device, dtype=torch.float32) + 0.5) / nx)[None, :, None]
        a[1] = ((torch.arange(ny, device=self.device, dtype=torch.float32) + 0.5) / ny)[None, None, :]
        lo, hi = math.log(RE_RANGE[0]), math.log(RE_RANGE[1])
        a[2] = (2 * (torch.log(re) - lo) / (hi - lo) - 1)[:, None, None]
        a[3] = (2 * (u - U_RANGE[0]) / (U_RANGE[1] - U_RANGE[0]) - 1)[:, None, None]
        return a

    @staticmethod
    def targets(fields, u_lid):
        """Network targets (3, B, nx, ny) from steady fields (B, 3, nx, ny) of (rho, ux, uy)."""
        u = torch.as_tensor(np.atleast_1d(u_lid), dtype=torch.float32, device=fields.device)[:, None, None]
        t = torch.empty((3,) + (fields.shape[0],) + tuple(fields.shape[2:]), dtype=torch.float32,
                        device=fields.device)
        t[0] = (fields[:, 0] - 1) / (u * u)
        t[1] = fields[:, 1] / u
        t[2] = fields[:, 2] / u
        return t

    def predict(self, re, u_lid, nx, ny):
        """Predicted steady (rho, ux, uy), each (B, nx, ny) float32 on the device."""
        out = self.forward(self.inputs(re, u_lid, nx, ny))
        sc = [float(x) for x in self.out_scale]
        u = torch.as_tensor(np.atleast_1d(u_lid), dtype=torch.float32, device=self.device)[:, None, None]
        return 1 + out[0] * (sc[0] * u * u), out[1] * (sc[1] * u), out[2] * (sc[2] * u)


def main(argv=None):
    """Time training steps (forward, backward, Adam) and inference of the
    network on synthetic inputs: ``python -m latticeboltzmann_gb300.fno``."""
    import argparse
    import time
    ap = argparse.ArgumentParser(description=main.__doc__)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--engine", choices=["tensor", "staged", "cuda"], default="tensor",
                    help="tensor: TMA pipeline where both operands are K-major, else the staged kernel; "
                         "staged: the staged tcgen05 kernel for every product; cuda: CUDA cores")
    ap.add_argument("--max-splits", type=int, default=1024, help="split-K count cap of the weight gradients")
    ap.add_argument("--unfused", action="store_true",
                    help="bias and activation as a separate pass after the layer's last GEMM (for comparison)")
    args = ap.parse_args(argv)
    dev = torch.device("cuda", torch.cuda.current_device())
    engine = {"tensor": ENGINE_TENSOR_CORES, "staged": ENGINE_STAGED, "cuda": ENGINE_CUDA_CORES}[args.engine]
    net = FNO2d(device=dev, engine=engine, max_splits=args.max_splits)
    net.fused_epilogue = not args.unfused
    rng = np.random.default_rng(0)
    re = np.exp(rng.uniform(math.log(RE_RANGE[0]), math.log(RE_RANGE[1]), args.batch))
    a = net.inputs(re, rng.uniform(*U_RANGE, args.batch), args.n, args.n)
    t = torch.randn(net.cout, args.batch, args.n, args.n, device=dev)
    for _ in range(args.warmup):
        net.loss_and_backward(a, t)
        net.adam(1e-3)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        net.loss_and_backward(a, t)
        net.adam(1e-3)
    torch.cuda.synchronize(dev)
    train = (time.perf_counter() - t0) / max(args.steps, 1)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        net.forward(a)
    torch.cuda.synchronize(dev)
    fwd = (time.perf_counter() - t0) / max(args.steps, 1)
    print(json.dumps({"batch": args.batch, "n": args.n, "engine": args.engine, "max_splits": net.max_splits,
                      "fused_epilogue": net.fused_epilogue,
                      "train_step_ms": round(train * 1e3, 3),
                      "forward_ms": round(fwd * 1e3, 3), "params": int(sum(np.prod(s) for s in net.shapes.values()))}))


if __name__ == "__main__":
    main()
