"""Device-resident D2Q9 solver around the fused stream-collide kernel.

The reference's time loop calls ``stream_and_bounce_back`` then ``collide`` on
one host array per step (simulators/parallel_lid_drive_cavity/cavity_opt2.py:
272-283; periodic: simulators/serial_shear_wave/Python/shear_wave_opt2.py:
94-99).  ``Lattice`` keeps two population buffers in HBM and advances them with
one fused pull-stream + collide launch per step (ping-pong, no copies); the
stored state after each step is post-collision, as in the reference.

Storage: ``f32``/``f64`` store f; ``f16dev``/``bf16dev`` store f_i - w_i in 16
bits with FP32 arithmetic (half the bytes per lattice update).
"""

import ctypes

import torch

from . import _lib
from ._tensor import require_cuda

_RAW = {"f32": torch.float32, "f64": torch.float64, "f16dev": torch.int16, "bf16dev": torch.int16,
        "f32dev": torch.float32}
_REAL = {"f32": torch.float32, "f64": torch.float64, "f16dev": torch.float32, "bf16dev": torch.float32,
         "f32dev": torch.float32}


def omega_from_reynolds(re, lid_velocity, length):
    """Relaxation parameter for a cavity of side ``length`` at Reynolds number ``re``.

    ``nu = u L / Re`` and ``omega = 1 / (3 nu + 1/2)``, i.e. the relation
    ``omega = 2 Re / (6 L u + Re)`` of simulators/simple_flows/slidingLid.py:28.
    """
    return 2.0 * re / (6.0 * length * lid_velocity + re)


def viscosity_from_omega(omega):
    """Kinematic viscosity of the BGK lattice fluid, ``(1/omega - 1/2) / 3``."""
    return (1.0 / omega - 0.5) / 3.0


class Lattice:
    """A ``(9, nx, ny)`` D2Q9 lattice resident on one GPU.

    Parameters
    ----------
    nx, ny : int
        Grid size (``ny`` is the fast axis; the cavity lid is at ``l = ny-1``).
    omega : float
        BGK relaxation parameter.
    boundary : {"cavity", "cavity-ladd", "periodic"}
        ``cavity``: bounce-back on four walls, lid moving with ``u0`` in +x,
        with the reference's lid term 6 w rho_lid u0 (cavity_opt1.py:225-239).
        ``cavity-ladd``: the same walls, lid term 6 w u0 (wall density 1) at
        every lid node; unlike the reference's lid it conserves mass and has a
        steady state.
    u0 : float
        Lid velocity (cavity only).
    storage : {"f32", "f64", "f16dev", "bf16dev", "f32dev"}
    device : torch device (CUDA).
    rounding : {"nearest", "stochastic"}
        How 16-bit storage rounds (FP32/FP64 ignore it).  Stochastic rounding
        is unbiased, so rounding errors do not add up in slowly varying flows;
        its random bits are a hash of (seed, step, cell, channel).
    seed : int
        Seed of the stochastic rounding.
    """

    def __init__(self, nx, ny, omega, boundary="cavity", u0=0.1, storage="f32", device=None, rounding="nearest",
                 seed=0):
        if storage not in _RAW:
            raise ValueError("storage must be one of %s" % sorted(_RAW))
        if boundary not in _lib.BOUNDARY_CODES:
            raise ValueError("boundary must be one of %s" % sorted(_lib.BOUNDARY_CODES))
        if nx <= 0 or ny <= 0:
            raise ValueError("grid must be positive, got %d x %d" % (nx, ny))
        if boundary != "periodic" and (nx < 2 or ny < 2):
            raise ValueError("the cavity needs nx >= 2 and ny >= 2")
        self.nx, self.ny = int(nx), int(ny)
        self.omega = float(omega)
        self.u0 = float(u0) if boundary != "periodic" else 0.0
        self.boundary = boundary
        self.storage = storage
        self.code = _lib.STORAGE_CODES[storage]
        self.bcode = _lib.BOUNDARY_CODES[boundary]
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        if self.device.type != "cuda":
            raise TypeError("Lattice lives on a CUDA device (there is no CPU path)")
        shape = (9, self.nx, self.ny)
        self._buf = [torch.empty(shape, dtype=_RAW[storage], device=self.device),
                     torch.empty(shape, dtype=_RAW[storage], device=self.device)]
        self._cur = 0
        self._ws = None
        self.steps_taken = 0
        if rounding not in ("nearest", "stochastic"):
            raise ValueError("rounding must be 'nearest' or 'stochastic'")
        self.rounding = rounding
        self.seed = int(seed) & 0xffffffff
        # device step index read by stochastic rounding (advanced on the device)
        self._step_ctr = torch.zeros(1, dtype=torch.int64, device=self.device)
        self.equilibrium()

    # ------------------------------------------------------------------ state
    @property
    def cells(self):
        return self.nx * self.ny

    @property
    def bytes_per_cell_update(self):
        """Algorithmic HBM bytes per cell and launch: 9 loads + 9 stores (one
        step per launch; two where ``steps_per_launch`` is 2)."""
        return 18 * self._buf[0].element_size()

    @property
    def steps_per_launch(self):
        """Steps that ``step(n)`` advances per launch for n >= 2: 2 where the
        two-step kernel applies to this lattice (FP32 or f32dev storage,
        periodic or cavity walls, nx a multiple of 16, ny of 128), else 1."""
        if self.rounding == "stochastic" and self.storage in ("f16dev", "bf16dev"):
            return 1
        return int(_lib.load().lbgb_steps_per_launch(self.nx, self.ny, self.bcode, self.code))

    @property
    def state(self):
        """The raw storage tensor holding the current populations."""
        return self._buf[self._cur]

    def _stream(self):
        return torch.cuda.current_stream(self.device).cuda_stream

    def load(self, f):
        """Set the populations from a float tensor ``(9, nx, ny)`` on any device.

        A host tensor of the storage's own dtype is copied straight into the
        device state (asynchronously when it is pinned); anything else goes
        through a conversion on the device.
        """
        f = torch.as_tensor(f)
        if tuple(f.shape) != (9, self.nx, self.ny):
            raise ValueError("expected populations of shape %s, got %s" % ((9, self.nx, self.ny), tuple(f.shape)))
        if self.storage in ("f32", "f64") and f.dtype == self.state.dtype and f.is_contiguous():
            self.state.copy_(f, non_blocking=f.device.type == "cpu" and f.is_pinned())
            return self
        # deviation storages take a float64 input as it is (f - w in FP64, then rounded)
        dev = self.storage in ("f32dev", "f16dev", "bf16dev")
        real = torch.float64 if dev and f.dtype == torch.float64 else _REAL[self.storage]
        src = f.to(device=self.device, dtype=real).contiguous()
        if self.storage in ("f32", "f64"):
            self.state.copy_(src)
        else:
            code = _lib.F64 if real == torch.float64 else _lib.F32
            _lib.call("lbgb_convert", src.data_ptr(), code, self.cells, self.state.data_ptr(), self.code,
                      self.cells, self.cells, self._stream())
        return self

    def _fill_real(self):
        """Arithmetic type of the fields and start populations: FP64 for f64 and
        for every deviation storage (whose h = f - w must not inherit the
        rounding of an FP32 population: at rest h is then exactly 0, not the
        ~1e-8 of w_i in FP32), FP32 for f32."""
        return torch.float32 if self.storage == "f32" else torch.float64

    def _fields(self, rho, ux, uy):
        real = self._fill_real()
        shape = (self.nx, self.ny)

        def field(v, default):
            if v is None:
                return torch.full(shape, default, dtype=real, device=self.device)
            v = torch.as_tensor(v, dtype=real, device=self.device)
            return v.expand(shape).contiguous()

        return field(rho, 1.0), field(ux, 0.0), field(uy, 0.0)

    def _set_from(self, fill):
        """Run ``fill(out_ptr, code)`` into the state (through an FP32 or FP64
        temporary for the deviation storages)."""
        real = self._fill_real()
        code = _lib.F64 if real == torch.float64 else _lib.F32
        if self.storage in ("f32", "f64"):
            fill(self.state.data_ptr(), code)
        else:
            tmp = torch.empty((9, self.nx, self.ny), dtype=real, device=self.device)
            fill(tmp.data_ptr(), code)
            _lib.call("lbgb_convert", tmp.data_ptr(), code, self.cells, self.state.data_ptr(), self.code,
                      self.cells, self.cells, self._stream())
        return self

    def equilibrium(self, rho=None, ux=None, uy=None):
        """Set the populations to the equilibrium of (rho, ux, uy) (default: rest)."""
        r, x, y = self._fields(rho, ux, uy)
        return self._set_from(lambda out, code: _lib.call(
            "lbgb_equilibrium", r.data_ptr(), x.data_ptr(), y.data_ptr(), out, self.cells, self.cells, code,
            self._stream()))

    def chapman_enskog(self, rho=None, ux=None, uy=None):
        """Set the populations from the flow (rho, ux, uy) with its first-order
        Chapman-Enskog non-equilibrium part at this lattice's omega, in the
        post-collision form f^eq + (1 - omega) f^neq that a step leaves: the
        start that lets a predicted steady field skip the initial transient."""
        r, x, y = self._fields(rho, ux, uy)
        return self._set_from(lambda out, code: _lib.call(
            "lbgb_chapman_enskog", r.data_ptr(), x.data_ptr(), y.data_ptr(), out, self.nx, self.ny, self.omega,
            self.u0, self.bcode, 1, code, self._stream()))

    def populations(self, dtype=None, out=None):
        """The populations f as a float tensor ``(9, nx, ny)`` (decoded for 16-bit storage).

        ``out``: a preallocated tensor (e.g. pinned host memory) of the
        storage's dtype to copy into, asynchronously on the current stream.
        """
        if out is not None:
            if self.storage not in ("f32", "f64") or out.dtype != self.state.dtype:
                out.copy_(self.populations(dtype=out.dtype))
            else:
                out.copy_(self.state, non_blocking=out.device.type == "cpu" and out.is_pinned())
            return out
        if self.storage in ("f32", "f64") and dtype is None:
            return self.state.clone()
        dtype = dtype or torch.float32
        out = torch.empty((9, self.nx, self.ny), dtype=dtype, device=self.device)
        dst = _lib.F64 if dtype == torch.float64 else _lib.F32
        _lib.call("lbgb_convert", self.state.data_ptr(), self.code, self.cells, out.data_ptr(), dst, self.cells,
                  self.cells, self._stream())
        return out

    # ------------------------------------------------------------------ host-resident populations
    def step_host(self, f, n=1, blocks=48, check=True, copy_streams=1):
        """Advance populations that live in host memory by ``n`` steps, in place.

        ``f``: a pinned, contiguous ``(9, nx, ny)`` host tensor of the storage's
        dtype (f32 or f64 storage).  Each step copies f to the device, steps
        and copies the result back -- what the reference's drivers do with
        their host array every step -- but by blocks of rows on separate
        streams, so that the upload of block j+1, the update of block j and
        the download of block j-1 overlap (the host link carries both
        directions at once).  Block 0 is updated last: its rows read the last
        row across the periodic seam (and the lid density does at the
        corners).  The device state ends up holding the same populations as
        ``f``.  At 8192^2 FP32, 32-64 blocks run at 15.3 ms per step (8
        blocks: 18.0 ms; the transfers alone take 14.1 ms at the link's
        two-way rate with one copy stream per direction).

        copy_streams: streams per direction; block j is copied on stream
        j mod copy_streams, so that several copy engines can serve one
        direction.

        check=True (default): wait for the last download and raise
        LBGBTimeout if a bounded device-side wait of a step gave up, so that
        ``f`` is complete and valid when the call returns; check=False
        returns at once, with the downloads still in flight on the current
        stream.
        """
        if self.storage not in ("f32", "f64"):
            raise ValueError("step_host needs f32 or f64 storage (the host array holds the populations as they are)")
        if (not isinstance(f, torch.Tensor) or f.device.type != "cpu" or not f.is_pinned() or not f.is_contiguous()
                or f.dtype != self.state.dtype or tuple(f.shape) != (9, self.nx, self.ny)):
            raise ValueError("step_host: f must be a pinned, contiguous %s tensor of shape %s" % (
                self.state.dtype, (9, self.nx, self.ny)))
        nx, ny = self.nx, self.ny
        nb = max(1, min(int(blocks), nx))
        k = max(1, int(copy_streams))
        edges = [nx * j // nb for j in range(nb + 1)]
        if getattr(self, "_hstreams_k", 0) != k:
            self._hstreams = ([torch.cuda.Stream(self.device) for _ in range(k)],
                              [torch.cuda.Stream(self.device) for _ in range(k)])
            self._hstreams_k = k
        s_in, s_out = self._hstreams
        s_cmp = torch.cuda.current_stream(self.device)
        order = list(range(1, nb)) + [0]
        ev = lambda: torch.cuda.Event()
        for _ in range(int(n)):
            a, b = self._buf[self._cur], self._buf[1 - self._cur]
            # this step's uploads overwrite rows that the last step read
            # (device buffer) and wrote (host array)
            for si in s_in:
                si.wait_stream(s_cmp)
                for so in s_out:
                    si.wait_stream(so)
            ev_in = []
            for j in range(nb):
                st = s_in[j % k]
                _lib.call("lbgb_copy_rows", a.data_ptr(), f.data_ptr(), nx, ny, edges[j], edges[j + 1], self.code,
                          st.cuda_stream)
                e = ev()
                e.record(st)
                ev_in.append(e)
            for j in order:
                # rows of blocks j-1, j, j+1 (with wrap) must be on the device
                for need in {j, j + 1 if j + 1 < nb else 0, j - 1 if j > 0 else nb - 1}:
                    s_cmp.wait_event(ev_in[need])
                _lib.call("lbgb_step_fused_rows", a.data_ptr(), b.data_ptr(), nx, ny, edges[j], edges[j + 1],
                          self.bcode, self.omega, self.u0, self.code, s_cmp.cuda_stream)
                e = ev()
                e.record(s_cmp)
                so = s_out[j % k]
                so.wait_event(e)
                _lib.call("lbgb_copy_rows", f.data_ptr(), b.data_ptr(), nx, ny, edges[j], edges[j + 1], self.code,
                          so.cuda_stream)
            self._cur = 1 - self._cur
            self.steps_taken += 1
        for so in s_out:
            s_cmp.wait_stream(so)
        if check:
            _lib.device_status()
        return f

    def check(self):
        """Synchronize and raise LBGBTimeout if a bounded device-side wait of
        a step launched so far gave up (the populations are then incomplete).
        ``step`` stays asynchronous; call this where the caller synchronizes
        anyway (before reading results)."""
        _lib.device_status()
        return self

    # ------------------------------------------------------------------ stepping
    def step(self, n=1):
        """Advance ``n`` time steps (one fused launch each)."""
        if n <= 0:
            return self
        which = ctypes.c_int(0)
        a, b = self._buf[self._cur], self._buf[1 - self._cur]
        if self.rounding == "stochastic" and self.storage in ("f16dev", "bf16dev"):
            _lib.call("lbgb_run_fused_sr", a.data_ptr(), b.data_ptr(), self.nx, self.ny, self.bcode, self.omega,
                      self.u0, self.code, int(n), self.seed, self._step_ctr.data_ptr(), ctypes.byref(which),
                      self._stream())
        else:
            _lib.call("lbgb_run_fused", a.data_ptr(), b.data_ptr(), self.nx, self.ny, self.bcode, self.omega,
                      self.u0, self.code, int(n), ctypes.byref(which), self._stream())
        if which.value == 1:
            self._cur = 1 - self._cur
        self.steps_taken += n
        return self

    def capture(self, n):
        """Capture ``n`` steps into a CUDA graph; returns a callable replaying them.

        ``n`` must be even so that the state returns to the same buffer after
        each replay (the graph bakes the buffer addresses in).
        """
        if n <= 0 or n % 2:
            raise ValueError("capture: n must be a positive even number")
        # load the kernel variant outside the capture: one step on a two-row
        # copy with the same row length (same vector width, same template)
        warm = [torch.zeros((9, 2, self.ny), dtype=_RAW[self.storage], device=self.device) for _ in range(2)]
        _lib.call("lbgb_step_fused", warm[0].data_ptr(), warm[1].data_ptr(), 2, self.ny, self.bcode, self.omega,
                  self.u0, self.code, self._stream())
        if self.rounding == "stochastic" and self.storage in ("f16dev", "bf16dev"):
            ctr = torch.zeros(1, dtype=torch.int64, device=self.device)
            _lib.call("lbgb_run_fused_sr", warm[0].data_ptr(), warm[1].data_ptr(), 2, self.ny, self.bcode,
                      self.omega, self.u0, self.code, 1, self.seed, ctr.data_ptr(), ctypes.byref(ctypes.c_int(0)),
                      self._stream())
        torch.cuda.current_stream(self.device).synchronize()
        s = torch.cuda.Stream(device=self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        g = torch.cuda.CUDAGraph()
        cur = self._cur
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                self.step(n)
        # capture recorded launches only; restore the bookkeeping
        self._cur = cur
        self.steps_taken -= n
        torch.cuda.current_stream(self.device).wait_stream(s)
        lattice = self

        def replay():
            g.replay()
            lattice.steps_taken += n

        replay.graph = g
        return replay

    # ------------------------------------------------------------------ diagnostics
    def macroscopic(self):
        """(rho, ux, uy), each ``(nx, ny)``, from the current populations."""
        real = torch.float64 if self.storage == "f64" else torch.float32
        rho = torch.empty((self.nx, self.ny), dtype=real, device=self.device)
        ux = torch.empty_like(rho)
        uy = torch.empty_like(rho)
        _lib.call("lbgb_macroscopic", self.state.data_ptr(), rho.data_ptr(), ux.data_ptr(), uy.data_ptr(),
                  self.cells, self.cells, self.code, self._stream())
        return rho, ux, uy

    def mass_momentum(self):
        """Total (mass, x momentum, y momentum) as a float64 CUDA tensor, FP64 sums."""
        if self._ws is None:
            nbytes = _lib.load().lbgb_mass_momentum_workspace_bytes()
            self._ws = torch.empty(nbytes // 8 + 1, dtype=torch.float64, device=self.device)
        out = torch.empty(3, dtype=torch.float64, device=self.device)
        _lib.call("lbgb_mass_momentum", self.state.data_ptr(), self.cells, self.cells, self.code, out.data_ptr(),
                  self._ws.data_ptr(), self._ws.numel() * 8, self._stream())
        return out


def mass_momentum(f):
    """Total (mass, x momentum, y momentum) of a float32/float64 ``(9, ...)`` CUDA tensor."""
    from ._tensor import population_view, storage_code, stream_handle
    n, cs = population_view(f, "mass_momentum")
    code = storage_code(f, "mass_momentum")
    nbytes = _lib.load().lbgb_mass_momentum_workspace_bytes()
    ws = torch.empty(nbytes // 8 + 1, dtype=torch.float64, device=f.device)
    out = torch.empty(3, dtype=torch.float64, device=f.device)
    _lib.call("lbgb_mass_momentum", f.data_ptr(), n, cs, code, out.data_ptr(), ws.data_ptr(), ws.numel() * 8,
              stream_handle(f))
    return out


def macroscopic(f):
    """(rho, ux, uy) of a float32/float64 ``(9, nx, ny)`` or ``(9, N)`` CUDA tensor."""
    from ._tensor import population_view, storage_code, stream_handle
    n, cs = population_view(f, "macroscopic")
    code = storage_code(f, "macroscopic")
    shape = tuple(f.shape[1:])
    rho = torch.empty(shape, dtype=f.dtype, device=f.device)
    ux = torch.empty_like(rho)
    uy = torch.empty_like(rho)
    if n:
        _lib.call("lbgb_macroscopic", f.data_ptr(), rho.data_ptr(), ux.data_ptr(), uy.data_ptr(), n, cs, code,
                  stream_handle(f))
    return rho, ux, uy


def fft_amplitude(f, row=None):
    """2/ny * max_k |FFT(ux[row, :])| of a float32/float64 ``(9, nx, ny)`` CUDA
    tensor (row defaults to nx // 2): the decay amplitude of the shear-wave
    scripts (simulators/simple_flows/shear_wave_decay.py:155-158), computed on
    the device.  Returns a float64 device scalar."""
    from ._tensor import storage_code, stream_handle
    if not isinstance(f, torch.Tensor) or f.device.type != "cuda":
        raise TypeError("fft_amplitude: expected a CUDA tensor (there is no CPU path)")
    if f.dim() != 3 or f.shape[0] != 9 or not f.is_contiguous():
        raise ValueError("fft_amplitude: expected a contiguous (9, nx, ny) tensor")
    code = storage_code(f, "fft_amplitude")
    nx, ny = int(f.shape[1]), int(f.shape[2])
    out = torch.empty((), dtype=torch.float64, device=f.device)
    _lib.call("lbgb_row_fft_amplitude", f.data_ptr(), nx, ny, nx // 2 if row is None else int(row), code,
              out.data_ptr(), stream_handle(f))
    return out
