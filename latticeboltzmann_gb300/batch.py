"""Many independent D2Q9 lattices of uneven size advanced together.

The reference runs one lattice per process and repeats a script per
parameter set (e.g. simulators/serial_shear_wave/Python/shear_wave_opt2.py,
simulators/simple_flows/shear_wave_decay.py:479-548 loops over omega).  Here
all instances share one population buffer and one launch per step
(``lbgb_batch_step``) walks a packed queue of warp tasks; a CUDA graph
captures many steps, and an autotuner picks cells per lane, rows per task and
the grid shape for the given set of instances.
"""

import ctypes
import math
import time

import numpy as np
import torch

from . import _lib
from .solver import _RAW, viscosity_from_omega

INSTANCE_DTYPE = np.dtype([("offset", "<i8"), ("nx", "<i4"), ("ny", "<i4"), ("omega", "<f8"), ("u0", "<f8"),
                           ("vec", "<i4"), ("cell_base", "<u4")])
assert INSTANCE_DTYPE.itemsize == 40

_TUNE_CACHE = {}


def _sm_count(device):
    return torch.cuda.get_device_properties(device).multi_processor_count


class BatchedLattice:
    """Independent lattices ``sizes[b] = (nx_b, ny_b)`` with relaxation ``omegas[b]``.

    boundary: "periodic" (the default; shear-wave studies), "cavity" (the
    reference's lid) or "cavity-ladd" (wall-density-1 lid, steady states);
    lid velocity ``u0``, a scalar or one per instance.  storage as for ``Lattice``.
    """

    def __init__(self, sizes, omegas, boundary="periodic", u0=0.0, storage="f32", device=None):
        if len(sizes) == 0 or len(sizes) != len(omegas):
            raise ValueError("need one omega per instance and at least one instance")
        if storage not in _RAW:
            raise ValueError("storage must be one of %s" % sorted(_RAW))
        if boundary not in _lib.BOUNDARY_CODES:
            raise ValueError("boundary must be one of %s" % sorted(_lib.BOUNDARY_CODES))
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        if self.device.type != "cuda":
            raise TypeError("BatchedLattice lives on a CUDA device (there is no CPU path)")
        self.sizes = [(int(a), int(b)) for a, b in sizes]
        for nx, ny in self.sizes:
            if nx <= 0 or ny <= 0 or (boundary != "periodic" and (nx < 2 or ny < 2)):
                raise ValueError("invalid instance size %dx%d" % (nx, ny))
        self.omegas = np.asarray(omegas, dtype=np.float64)
        self.n = len(self.sizes)
        self.boundary, self.storage = boundary, storage
        self.code = _lib.STORAGE_CODES[storage]
        self.bcode = _lib.BOUNDARY_CODES[boundary]
        u0s = np.broadcast_to(np.asarray(u0, dtype=np.float64), (self.n,)) if boundary != "periodic" \
            else np.zeros(self.n)
        self.u0s = np.array(u0s, dtype=np.float64)
        raw = _RAW[storage]
        es = torch.empty(0, dtype=raw).element_size()
        self.vw = 16 // es
        table = np.zeros(self.n, dtype=INSTANCE_DTYPE)
        off, cell = 0, 0
        for b, (nx, ny) in enumerate(self.sizes):
            table[b] = (off, nx, ny, self.omegas[b], self.u0s[b], self.vw if ny % self.vw == 0 else 1, cell)
            off += -(-9 * nx * ny // self.vw) * self.vw  # next instance starts on a 16-byte boundary
            cell += nx * ny
        self.total = off
        self.cells = cell
        self._table_np = table
        self._tables = {}
        self._buf = [torch.zeros(self.total, dtype=raw, device=self.device) for _ in range(2)]
        self._cur = 0
        self.steps_taken = 0
        n_sm = _sm_count(self.device)
        self.config = {"flat": True, "vector": False, "rows": 2, "threads": 256, "blocks": n_sm * 8}
        self._tasks = {}
        self._amp = torch.empty(self.n, dtype=torch.float64, device=self.device)
        self._partials = torch.empty(self.n * _lib.DIAG_CHUNKS, dtype=torch.float64, device=self.device)
        self.active = np.ones(self.n, dtype=bool)  # instances that still advance
        self._u_prev = None

    # ------------------------------------------------------------ tables and queues
    def _table(self, vector):
        if vector not in self._tables:
            t = self._table_np.copy()
            if not vector:
                t["vec"] = 1
            self._tables[vector] = torch.from_numpy(t.view(np.uint8).copy()).to(self.device)
        return self._tables[vector]

    def task_queue(self, vector=True, rows=1, flat=False):
        """The packed task queue, int32 (n_tasks, 4).

        Segment tasks: (instance, row, column, 0), one warp per ``rows`` rows
        of a 32*V-cell segment.  Flat tasks: (instance, 0, first cell, 0), one
        warp per 32*``rows`` consecutive cells of the flattened grid.
        """
        key = (bool(vector), int(rows), bool(flat), None)
        if key not in self._tasks:
            parts = []
            for b, (nx, ny) in enumerate(self.sizes):
                if flat:
                    c0 = np.arange(0, nx * ny, 32 * rows, dtype=np.int64)
                    q = np.zeros((c0.size, 4), dtype=np.int32)
                    q[:, 0] = b
                    q[:, 2] = c0
                    parts.append(q)
                    continue
                v = self.vw if (vector and ny % self.vw == 0) else 1
                ks = np.arange(0, nx, rows, dtype=np.int32)
                zs = np.arange(0, ny, 32 * v, dtype=np.int32)
                kk, zz = np.meshgrid(ks, zs, indexing="ij")
                q = np.zeros((kk.size, 4), dtype=np.int32)
                q[:, 0] = b
                q[:, 1] = kk.ravel()
                q[:, 2] = zz.ravel()
                parts.append(q)
            q = np.concatenate(parts)
            self._tasks[key] = torch.from_numpy(q).to(self.device)
        return self._tasks[key]

    # ------------------------------------------------------------ state
    @property
    def state(self):
        return self._buf[self._cur]

    def _stream(self):
        return torch.cuda.current_stream(self.device).cuda_stream

    def _slice(self, b, buf=None):
        buf = self.state if buf is None else buf
        nx, ny = self.sizes[b]
        off = int(self._table_np["offset"][b])
        return buf[off:off + 9 * nx * ny]

    def equilibrium(self, fields):
        """Set instance b to the equilibrium of ``fields(b) -> (rho, ux, uy)`` ((nx, ny) tensors)."""
        return self._init(fields, False)

    def chapman_enskog(self, fields):
        """Set instance b to the post-collision Chapman-Enskog state of
        ``fields(b) -> (rho, ux, uy)`` at its own omega and lid speed
        (equilibrium plus (1 - omega) times the first-order non-equilibrium
        part): the warm start of a predicted flow."""
        return self._init(fields, True)

    def _init(self, fields, ce):
        # FP64 fields for f64 and for every deviation storage (see Lattice._fill_real)
        real = torch.float32 if self.storage == "f32" else torch.float64
        code = _lib.F64 if real == torch.float64 else _lib.F32
        for b, (nx, ny) in enumerate(self.sizes):
            rho, ux, uy = (torch.as_tensor(x, dtype=real, device=self.device).expand(nx, ny).contiguous()
                           for x in fields(b))
            n = nx * ny
            direct = self.storage in ("f32", "f64")
            out = self._slice(b) if direct else torch.empty(9 * n, dtype=real, device=self.device)
            if ce:
                _lib.call("lbgb_chapman_enskog", rho.data_ptr(), ux.data_ptr(), uy.data_ptr(), out.data_ptr(), nx, ny,
                          float(self.omegas[b]), float(self.u0s[b]), self.bcode, 1, code, self._stream())
            else:
                _lib.call("lbgb_equilibrium", rho.data_ptr(), ux.data_ptr(), uy.data_ptr(), out.data_ptr(), n, n,
                          code, self._stream())
            if not direct:
                _lib.call("lbgb_convert", out.data_ptr(), code, n, self._slice(b).data_ptr(), self.code, n, n,
                          self._stream())
        return self

    def shear_wave(self, amplitude=0.05):
        """u_x(l) = amplitude sin(2 pi l / ny) at unit density in every instance."""
        def fields(b):
            nx, ny = self.sizes[b]
            l = torch.arange(ny, dtype=torch.float64, device=self.device)
            return 1.0, (amplitude * torch.sin(2 * math.pi * l / ny))[None, :], 0.0
        return self.equilibrium(fields)

    def load(self, b, f):
        """Set instance b from a float tensor (9, nx, ny) (FP32 or FP64, any device)."""
        nx, ny = self.sizes[b]
        n = nx * ny
        f = torch.as_tensor(f).to(self.device)
        if tuple(f.shape) != (9, nx, ny) or f.dtype not in (torch.float32, torch.float64):
            raise ValueError("expected a float32/float64 tensor of shape %s" % ((9, nx, ny),))
        f = f.contiguous()
        src = _lib.F64 if f.dtype == torch.float64 else _lib.F32
        _lib.call("lbgb_convert", f.data_ptr(), src, n, self._slice(b).data_ptr(), self.code, n, n, self._stream())
        return self

    def populations(self, b, dtype=torch.float64):
        """Instance b as a (9, nx, ny) float tensor."""
        nx, ny = self.sizes[b]
        n = nx * ny
        out = torch.empty((9, nx, ny), dtype=dtype, device=self.device)
        dst = _lib.F64 if dtype == torch.float64 else _lib.F32
        _lib.call("lbgb_convert", self._slice(b).data_ptr(), self.code, n, out.data_ptr(), dst, n, n,
                  self._stream())
        return out

    # ------------------------------------------------------------ stepping
    def set_active(self, mask):
        """Advance only the instances where ``mask`` is true (the others keep
        their state: their tasks leave the queue)."""
        mask = np.asarray(mask, dtype=bool).copy()
        other = self._buf[1 - self._cur]
        for b in np.nonzero(self.active & ~mask)[0]:
            # both ping-pong buffers hold the frozen state from now on
            self._slice(int(b), other).copy_(self._slice(int(b)))
        self.active = mask
        self._tasks = {k: v for k, v in self._tasks.items() if k[3] is None}

    def _queue(self, cfg):
        flat = bool(cfg.get("flat", False))
        full = self.task_queue(cfg["vector"], cfg["rows"], flat)
        if self.active.all():
            return full
        key = (bool(cfg["vector"]), int(cfg["rows"]), flat, self.active.tobytes())
        if key not in self._tasks:
            keep = torch.from_numpy(self.active).to(self.device)[full[:, 0].long()]
            self._tasks[key] = full[keep].contiguous()
        return self._tasks[key]

    def _launch(self, src, dst, cfg):
        flat = bool(cfg.get("flat", False))
        tasks = self._queue(cfg)
        if tasks.shape[0] == 0:
            # nothing advances: keep the ping-pong consistent with a copy
            dst.copy_(src)
            return
        _lib.call("lbgb_batch_step", src.data_ptr(), dst.data_ptr(), self.total, self._table(cfg["vector"]).data_ptr(),
                  self.n, tasks.data_ptr(), tasks.shape[0], cfg["rows"], self.bcode, self.code, cfg["threads"],
                  cfg["blocks"], int(flat), self._stream())

    def step(self, n=1, config=None):
        cfg = config or self.config
        for _ in range(int(n)):
            self._launch(self._buf[self._cur], self._buf[1 - self._cur], cfg)
            self._cur = 1 - self._cur
        self.steps_taken += int(n)
        return self

    def capture(self, n):
        """CUDA graph of ``n`` (even) steps; returns a callable replaying them."""
        if n <= 0 or n % 2:
            raise ValueError("capture: n must be a positive even number")
        self.task_queue(self.config["vector"], self.config["rows"], self.config.get("flat", False))  # outside the capture
        self._table(self.config["vector"])
        # load the kernel outside the capture: two steps on a copy of the state
        saved = self.state.clone()
        cur, taken = self._cur, self.steps_taken
        self.step(2)
        self._buf[cur].copy_(saved)
        self._cur, self.steps_taken = cur, taken
        torch.cuda.synchronize(self.device)
        s = torch.cuda.Stream(device=self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        g = torch.cuda.CUDAGraph()
        cur, taken = self._cur, self.steps_taken
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                self.step(n)
        self._cur, self.steps_taken = cur, taken
        torch.cuda.current_stream(self.device).wait_stream(s)
        batch = self

        def replay():
            g.replay()
            batch.steps_taken += n

        replay.graph = g
        return replay

    # ------------------------------------------------------------ diagnostics
    def shear_amplitudes(self, out=None):
        """Per-instance amplitude of the u_x ~ sin(2 pi l / ny) mode (float64 device tensor)."""
        out = self._amp if out is None else out
        _lib.call("lbgb_batch_shear_amplitude", self.state.data_ptr(), self.total, self._table(True).data_ptr(),
                  self.n, self.code, out.data_ptr(), self._partials.data_ptr(), self._stream())
        return out

    def velocity_change(self):
        """Per-instance max |u - u_prev| since the previous call (FP32 device
        tensor; inf on the first call), and u_prev <- u."""
        out = torch.empty(self.n, dtype=torch.float32, device=self.device)
        first = self._u_prev is None
        if first:
            self._u_prev = torch.zeros(2 * self.cells, dtype=torch.float32, device=self.device)
        _lib.call("lbgb_batch_velocity_change", self.state.data_ptr(), self.total, self._table(True).data_ptr(),
                  self.n, self.code, self._u_prev.data_ptr(), self.cells, out.data_ptr(), self._partials.data_ptr(),
                  self._stream())
        if first:
            out.fill_(float("inf"))
        return out

    def fields(self, b):
        """(rho, ux, uy) of instance b as float32 (nx, ny) tensors."""
        from .solver import macroscopic
        f = self.populations(b, torch.float32)
        return macroscopic(f)

    # ------------------------------------------------------------ tuning
    def candidates(self):
        """Launch shapes the autotuner times: row segments (vector or scalar
        lanes, 1-4 rows per task) and flat cell runs (1-8 rounds of 32 cells),
        each with 128/256 threads and 4/8/16 CTAs per SM."""
        n_sm = _sm_count(self.device)
        out = []
        shapes = [(False, v, r) for v in (True, False) for r in (1, 2, 4)] + [(True, False, r) for r in (1, 2, 4, 8)]
        for flat, vector, rows in shapes:
            for threads in (128, 256):
                for per_sm in (4, 8, 16):
                    out.append({"flat": flat, "vector": vector, "rows": rows, "threads": threads,
                                "blocks": n_sm * per_sm})
        return out

    def autotune(self, steps=10, warmup=3, candidates=None):
        """Time every candidate launch configuration on this batch and keep the fastest.

        Results are cached per (instance sizes, storage, boundary) for the
        process.  Returns (best config, {config: ms per step}).  The state is
        saved and restored, so tuning does not advance the simulation.
        """
        key = (tuple(self.sizes), self.storage, self.boundary)
        if key in _TUNE_CACHE:
            self.config = dict(_TUNE_CACHE[key][0])
            return _TUNE_CACHE[key]
        saved = self.state.clone()
        cur, taken = self._cur, self.steps_taken
        timings = {}
        stream = torch.cuda.current_stream(self.device)
        for cfg in (candidates or self.candidates()):
            self.step(warmup, cfg)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            self.step(steps, cfg)
            e1.record(stream)
            e1.synchronize()
            timings[tuple(sorted(cfg.items()))] = e0.elapsed_time(e1) / steps
        best = min(timings, key=timings.get)
        self.config = dict(best)
        self._buf[cur].copy_(saved)
        self._cur, self.steps_taken = cur, taken
        _TUNE_CACHE[key] = (dict(best), timings)
        return _TUNE_CACHE[key]


def fit_viscosity(times, amps, ny, floor=1e-4):
    """nu from a log-linear fit of a shear-mode amplitude series, a(t) ~ exp(-nu k^2 t).

    Uses the samples whose amplitude is above ``floor`` times the first one
    (FP32 rounding sets the noise floor); returns nan with fewer than 3.
    """
    t = np.asarray(times, dtype=np.float64)
    a = np.asarray(amps, dtype=np.float64)
    good = a > floor * a[0]
    if good.sum() < 3:
        return float("nan")
    k = 2 * math.pi / ny
    slope = np.polyfit(t[good], np.log(a[good]), 1)[0]
    return float(-slope / (k * k))


def random_shear_batch(n=512, seed=0, nx_range=(32, 1024), ny_range=(16, 512), omega_range=(0.3, 1.9)):
    """The seeded uneven batch: nx, ny log-uniform, omega uniform."""
    rng = np.random.default_rng(seed)
    nx = np.rint(np.exp(rng.uniform(np.log(nx_range[0]), np.log(nx_range[1]), n))).astype(int)
    ny = np.rint(np.exp(rng.uniform(np.log(ny_range[0]), np.log(ny_range[1]), n))).astype(int)
    om = rng.uniform(omega_range[0], omega_range[1], n)
    return list(zip(nx.tolist(), ny.tolist())), om


def shear_study(n=512, steps=5000, every=10, seed=0, amplitude=0.05, storage="f32", device=None, tune=True):
    """Batched shear-wave study (512 uneven lattices by default): fit the
    viscosity of every instance from its decay series."""
    sizes, om = random_shear_batch(n, seed)
    bl = BatchedLattice(sizes, om, boundary="periodic", storage=storage, device=device).shear_wave(amplitude)
    tuned = bl.autotune() if tune else None
    hist = torch.empty((steps // every + 1, n), dtype=torch.float64, device=bl.device)
    bl.shear_amplitudes(hist[0])
    replay = bl.capture(every) if every % 2 == 0 else None
    torch.cuda.synchronize(bl.device)
    t0 = time.perf_counter()
    for i in range(1, steps // every + 1):
        if replay is not None:
            replay()
        else:
            bl.step(every)
        bl.shear_amplitudes(hist[i])
    torch.cuda.synchronize(bl.device)
    elapsed = time.perf_counter() - t0
    h = hist.cpu().numpy()
    t = np.arange(h.shape[0]) * every
    nu_fit = np.array([fit_viscosity(t, h[:, b], sizes[b][1]) for b in range(n)])
    nu_th = viscosity_from_omega(om)
    return {"sizes": sizes, "omegas": om, "nu_fit": nu_fit, "nu_theory": nu_th, "times": t, "amplitudes": h,
            "elapsed_s": elapsed, "cells": bl.cells, "steps": steps,
            "mlups_incl_diagnostics": bl.cells * steps / elapsed / 1e6, "config": bl.config,
            "tuning": tuned[1] if tuned else None}


def omega_for(re, u_lid, length):
    """Relaxation parameter of a cavity of side ``length`` at Reynolds number re."""
    return 2.0 * re / (6.0 * length * u_lid + re)


def _run_to_steady(bl, tol, every, max_steps, log=None, what="", patience=0):
    """Step the active instances of bl until max|u^(t+every) - u^t| < tol;
    converged instances leave the queue.

    patience > 0: an instance whose change has not dropped below 0.9 x its
    best for ``patience`` checks in a row stops as stalled (its storage's
    rounding floor lies above tol).  Returns (steps per instance: the step
    count at convergence, -1 if max_steps passed, -2 if stalled; the last
    velocity change; the step count at which each instance stalled)."""
    bl.velocity_change()
    n = bl.n
    state = np.where(bl.active, 0, 3)  # 0 running, 1 converged, 2 stalled, 3 not run
    steps = np.where(state == 3, 0, -1).astype(np.int64)
    change = np.full(n, np.inf)
    best = np.full(n, np.inf)
    since = np.zeros(n, dtype=np.int64)
    stalled_at = np.zeros(n, dtype=np.int64)
    done = 0
    while done < max_steps and (state == 0).any():
        bl.step(every)
        done += every
        ch = bl.velocity_change().cpu().numpy()
        # the copy above synchronized: a bounded device-side wait that gave
        # up (incomplete populations) raises here instead of being reported
        # as a result
        _lib.device_status()
        live = state == 0
        change[live] = ch[live]
        conv = live & (ch < tol)
        steps[conv] = done
        state[conv] = 1
        stall = np.zeros(n, dtype=bool)
        if patience:
            going = live & ~conv
            better = going & (ch < 0.9 * best)
            best[better] = ch[better]
            since[better] = 0
            since[going & ~better] += 1
            stall = going & (since >= patience)
            state[stall] = 2
            steps[stall] = -2
            stalled_at[stall] = done
        if conv.any() or stall.any():
            bl.set_active(state == 0)
        if log is not None and done % (every * 50) == 0:
            log("steady_cavities%s: %d steps, %d/%d converged, %d stalled" % (
                what, done, int((state == 1).sum()), n, int((state == 2).sum())))
    return steps, change, stalled_at


def steady_cavities(re, u_lid, n=256, tol=1e-7, every=1000, max_steps=1_000_000, storage="f32", device=None,
                    tune=True, log=None, boundary="cavity-ladd", start=None, refine=None, switch_tol=None,
                    patience=30, info=None):
    """Run lid-driven cavities (n x n) to steady state, all in one batch.

    The default lid is the wall-density-1 one: the reference's lid adds mass
    every step, so above Re ~ 100 its cavities never settle.

    start: None (rest) or ``start(b) -> (rho, ux, uy)`` (n x n tensors), a
    predicted flow from which instance b starts in its Chapman-Enskog state.
    Steady: max over the cavity of |u^(t+every) - u^t| < tol.  Converged
    instances leave the task queue.

    refine: None, or a wider storage ("f64") for the instances the first
    storage cannot bring to tol: with switch_tol = None (adaptive) an
    instance moves to ``refine`` once its change has stalled for
    ``patience`` checks (FP32 storage stalls near 1e-6 per 1000 steps above
    Re ~ 200 at 256^2, FP32 deviations near 1e-7); with a switch_tol every
    instance runs in ``storage`` down to max(tol, switch_tol) and finishes in
    ``refine``.

    Returns (fields float32 (N, 3, n, n) of rho, ux, uy; steps to convergence
    per instance, summed over both phases, -1 if a phase hit max_steps; wall
    seconds from the first step to the last check).  ``info`` (a dict), when
    given, receives the per-phase steps and last velocity changes.
    """
    re = np.asarray(re, dtype=np.float64)
    u_lid = np.asarray(u_lid, dtype=np.float64)
    om = omega_for(re, u_lid, n)
    sizes = [(n, n)] * len(re)
    bl = BatchedLattice(sizes, om, boundary=boundary, u0=u_lid, storage=storage, device=device)
    if start is None:
        bl.equilibrium(lambda b: (1.0, 0.0, 0.0))
    if tune:
        bl.autotune(steps=3, warmup=1)
    if start is not None:
        bl.chapman_enskog(start)
    torch.cuda.synchronize(bl.device)
    t0 = time.perf_counter()
    adaptive = refine is not None and switch_tol is None
    tol1 = tol if refine is None or adaptive else max(tol, switch_tol)
    steps, change, stalled_at = _run_to_steady(bl, tol1, every, max_steps, log, "", patience if adaptive else 0)
    if info is not None:
        info["phase1_steps"], info["phase1_change"] = steps.copy(), change.copy()
    need = (steps == -2) if adaptive else (steps >= 0 if (refine is not None and tol1 > tol) else None)
    if need is not None and need.any():
        bl2 = BatchedLattice(sizes, om, boundary=boundary, u0=u_lid, storage=refine, device=device)
        for b in range(len(re)):
            bl2.load(b, bl.populations(b, torch.float64))
        del bl
        if tune:
            bl2.autotune(steps=3, warmup=1)
        bl2.set_active(need)
        s2, change2, _ = _run_to_steady(bl2, tol, every, max_steps, log, " (%s)" % refine)
        change = np.where(need, change2, change)
        if info is not None:
            info["phase2_steps"], info["phase2_change"] = np.where(need, s2, 0), change2.copy()
        base = stalled_at if adaptive else steps
        steps = np.where(need, np.where(s2 >= 0, base + s2, -1), steps)
        bl = bl2
    if info is not None:
        info["change"] = change
    torch.cuda.synchronize(bl.device)
    wall = time.perf_counter() - t0
    out = torch.empty((len(re), 3, n, n), dtype=torch.float32, device=bl.device)
    for b in range(len(re)):
        r, x, y = bl.fields(b)
        out[b, 0], out[b, 1], out[b, 2] = r, x, y
    return out, steps, wall
