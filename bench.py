#!/usr/bin/env python
"""Benchmark of the D2Q9 hot path: fused stream + bounce-back/moving lid + collide.

Workload (default): lid-driven cavity, 8192 x 8192 cells, FP32 populations,
omega = 1.7, lid velocity 0.1, from rest at equilibrium.  One step = one
fused pull-stream + collide update of the whole lattice; the solver runs two
steps per kernel launch where its two-step kernel applies (FP32 and f32dev
storage: one read and one write of the lattice per two steps), else one.
Metric: MLUPS (million lattice-cell updates per second, physical cells only).

Lines printed (rank 0, one JSON line):
  value      device-timed MLUPS, populations resident in HBM (CUDA events on
             the launching stream, barrier + synchronize on both sides)
  e2e        MLUPS through the public API with the populations in pinned host
             memory: every step copies them host->device, runs the step, and
             copies them back, inside the timed region (Lattice.step_host:
             the three overlap by blocks of rows); e2e.link is the ceiling
             the host link sets, the same bytes copied both ways at once
  roofline   HBM roofline of the fused kernel: the lattice bytes of one
             launch (72 B/cell FP32, 36 B 16-bit deviations; a launch is two
             steps for the two-step kernel) over its CUDA-event launch time
  cpu_baseline  the oracle's C port of the reference step on the host cores;
             cpu_baseline.numpy_opt1: the reference's numpy step, one process
             per host core
  fp16_store FP32 against FP16/BF16 deviation storage (round to nearest and
             stochastic) on the 16384^2 cavity: CUDA-event MLUPS, HBM
             fraction and clock record per storage, ratio to FP32, and each
             mode's error against an FP64 run (1024^2, 1000 steps)
  operator_path  MLUPS of the reference's loop body through the drop-in
             operators (stream_and_bounce_back in place, then collide),
             next to the fused step
  warm_start cavity time to steady state (max |du| < 1e-7 per 1000 steps),
             cold from rest against warm from the committed surrogate's
             prediction, for fixed held-out cases at 256^2 and 1024^2: steps,
             wall seconds and their ratios

``--impl reference`` times the CPU implementation of the reference step (the
C port of the oracle; the reference's own C++ extension needs Eigen, which is
not available) on all host cores, on the same workload.

Multi-GPU (torchrun): replicas only -- every rank runs its own lattice; value
= total cells updated by all ranks / max time over ranks.
"""

import argparse
import json
import os
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "MLUPS (D2Q9 BGK fused stream-collide, lid-driven cavity)"
UNIT = "MLUPS"


def parse(argv=None):
    p = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=1000)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--nx", type=int, default=8192)
    p.add_argument("--ny", type=int, default=8192)
    p.add_argument("--storage", choices=["f32", "f16dev", "bf16dev", "f64", "f32dev"], default="f32")
    p.add_argument("--boundary", choices=["cavity", "periodic"], default="cavity")
    p.add_argument("--omega", type=float, default=1.7)
    p.add_argument("--u0", type=float, default=0.1)
    p.add_argument("--e2e-steps", type=int, default=5)
    p.add_argument("--copy-streams", type=int, default=1,
                   help="streams per copy direction of the end-to-end host step (and of its link bound)")
    p.add_argument("--cpu-seconds", type=float, default=10.0, help="bound of the CPU-baseline sample")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--kernel", choices=["auto", "register", "pipelined"], default="auto",
                   help="step kernel: shared-memory pipelined, register/shuffle, or automatic choice")
    p.add_argument("--stages", type=int, default=0, help="pipeline stages (0: library default)")
    p.add_argument("--rounding", choices=["nearest", "stochastic"], default="nearest",
                   help="rounding of 16-bit storage")
    p.add_argument("--workload", choices=["cavity", "batched-shear"], default="cavity",
                   help="cavity: one lattice (default); batched-shear: 512 uneven periodic shear-wave lattices "
                        "advanced by one launch per step (autotuned)")
    p.add_argument("--no-extras", action="store_true",
                   help="skip the 16-bit storage comparison, the operator-path timing and the warm-start study")
    p.add_argument("--extras", default="operator_path,fp16_store,warm_start",
                   help="comma-separated extras to run (cavity workload): operator_path, fp16_store, warm_start")
    p.add_argument("--store-n", type=int, default=16384, help="lattice side of the 16-bit storage comparison")
    p.add_argument("--store-steps", type=int, default=60, help="timed steps per storage in that comparison")
    p.add_argument("--warm-cases", type=int, default=8, help="held-out cavities timed cold and warm at 256^2")
    p.add_argument("--warm-cases-large", type=int, default=2, help="held-out cavities timed at 1024^2")
    return p.parse_args(argv)


# ---------------------------------------------------------------- distributed
class Dist:
    """Rank bookkeeping; N>1 runs replicas (no data-path collective)."""

    def __init__(self, backend=None):
        import torch.distributed as dist
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local_rank = int(os.environ.get("LOCAL_RANK", "0"))
        self.dist = dist if self.world > 1 else None
        if self.dist is not None and not dist.is_initialized():
            dist.init_process_group(backend=backend or "nccl")

    def barrier(self):
        if self.dist is not None:
            self.dist.barrier()

    def max(self, x, device=None):
        if self.dist is None:
            return float(x)
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64, device=device)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x, device=None):
        if self.dist is None:
            return float(x)
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64, device=device)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.dist is not None and self.dist.is_initialized():
            self.dist.destroy_process_group()


def aggregate_mlups(cells_per_rank, steps, seconds_per_rank, d, device=None):
    """Whole-job MLUPS: all ranks' cell updates over the slowest rank's time."""
    total = d.sum(cells_per_rank * steps, device)
    t = d.max(seconds_per_rank, device)
    return total / t / 1e6, t


# ---------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        import tempfile
        fd, self.path = tempfile.mkstemp(prefix="lbgb_clocks_", suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        time.sleep(0.25)

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append({"sm": float(parts[1]), "max": float(parts[2]), "power": float(parts[3]),
                             "hw": parts[5], "hwt": parts[6], "swt": parts[7], "pcap": parts[8]})
            except ValueError:
                continue
        os.remove(self.path)
        if not rows:
            return None
        import statistics
        reasons = set()
        for r in rows:
            for k, name in (("hw", "hw_slowdown"), ("hwt", "hw_thermal_slowdown"), ("swt", "sw_thermal_slowdown"),
                            ("pcap", "sw_power_cap")):
                if r[k].lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(r["sm"] for r in rows), "sm_max_mhz": max(r["max"] for r in rows),
                "power_w_max": max(r["power"] for r in rows), "samples": len(rows), "reasons": sorted(reasons)}


# ---------------------------------------------------------------- peaks, profiles
def hbm_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs, copy burst)"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profiled_traffic(storage, boundary, cells, kernel="k_step_pipe"):
    """DRAM bytes per launch of the fused kernel from the committed ncu summary,
    scaled from the captured grid to ``cells`` (traffic is proportional to cells)."""
    path = os.path.join(ROOT, "profiles", "k_step_traffic.json")
    try:
        with open(path) as fh:
            rows = json.load(fh)
    except (OSError, ValueError):
        return None, None
    for r in rows:
        if (r.get("storage") == storage and r.get("boundary") == boundary
                and r.get("kernel", "k_step_pipe") == kernel):
            return r["dram_bytes_per_launch"] * cells / r["cells"], r
    return None, None


# ---------------------------------------------------------------- CPU baseline
def _cpu_lattice(rows, ny, storage):
    import numpy as np
    from oracle import port
    dt = np.float64 if storage == "f64" else np.float32
    a = np.empty((9, rows, ny), dtype=dt)
    z = np.zeros(rows * ny, dtype=dt)
    port.equilibrium(np.ones(rows * ny, dtype=dt), z, z, a.reshape(9, -1), nthreads=0)
    return a, np.empty_like(a)


def cpu_port_sample(nx, ny, omega, u0, storage, boundary, budget_s):
    """Time the oracle's C port of the reference step on all host cores.

    The sample is whole-lattice steps for about ``budget_s`` seconds; if one
    whole-lattice step takes more than a third of the budget, a strip of rows
    is used instead.  Returns (MLUPS, cores, sample description).
    """
    from oracle import port
    cores = port.max_threads()
    rows = nx
    while True:
        a, b = _cpu_lattice(rows, ny, storage)
        t0 = time.perf_counter()
        port.run_raw(a, b, boundary, omega, u0, 1)
        t1 = time.perf_counter() - t0
        if t1 <= budget_s / 3 or rows <= 64:
            break
        rows = max(64, int(rows * (budget_s / 3) / t1))
    steps = max(1, int(budget_s / max(t1, 1e-6)))
    t0 = time.perf_counter()
    port.run_raw(a, b, boundary, omega, u0, steps)
    el = time.perf_counter() - t0
    mlups = rows * ny * steps / el / 1e6
    sample = "%d steps of a %d x %d %s lattice (%s), %.1f s on %d host threads; C port of the reference step " \
             "(stream + bounce-back pass, then collide pass)" % (steps, rows, ny, boundary, storage, el, cores)
    return mlups, cores, sample


def cpu_model():
    """The host CPU's model name (lscpu), or the machine type."""
    import platform
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    return platform.machine()


def _numpy_opt1_worker(job):
    """One process of the numpy sample, pinned to its own core: the oracle's
    numpy step (the reference's opt1 arithmetic, bit for bit) on its own strip,
    started at the common wall-clock time ``go``; returns its end time."""
    rows, ny, omega, u0, boundary, steps, go, core = job
    if core is not None and hasattr(os, "sched_setaffinity"):
        try:
            os.sched_setaffinity(0, {core})
        except OSError:
            pass
    import numpy as np
    from oracle import d2q9
    one, zero = np.ones((rows, ny), np.float32), np.zeros((rows, ny), np.float32)
    f = d2q9.equilibrium(one, zero, zero)
    om = np.float32(omega)
    while time.time() < go:
        time.sleep(0.001)
    for _ in range(steps):
        if boundary == "periodic":
            d2q9.periodic_step(f, om)
        else:
            d2q9.cavity_step(f, om, u0)
    return time.time()


def numpy_opt1_sample(ny, omega, u0, boundary, rows=128, steps=12):
    """The reference's numpy step (opt1) on the host: one single-threaded
    process per core, each on its own ``rows`` x ``ny`` strip, all started at
    one wall-clock time; MLUPS = all processes' cell updates / (last end -
    start).  The pool is spawned (the parent has a CUDA context)."""
    import multiprocessing as mp
    cores = sorted(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else list(range(os.cpu_count() or 1))
    n = len(cores)
    ctx = mp.get_context("spawn")
    with ctx.Pool(n) as pool:
        pool.map(abs, range(n), chunksize=1)  # start every worker (interpreter + numpy import) first
        go = time.time() + 2.0
        jobs = [(rows, ny, omega, u0, boundary, steps, go, c) for c in cores]
        ends = pool.map(_numpy_opt1_worker, jobs, chunksize=1)
    el = max(ends) - go
    mlups = n * rows * ny * steps / el / 1e6
    script = "shear_wave_opt1.py" if boundary == "periodic" else "cavity_opt1.py"
    sample = "%d processes x %d steps of a %d x %d %s strip (f32), %.1f s; numpy step of the reference's " \
             "%s arithmetic, one process pinned to each core of %s" % (n, steps, rows, ny, boundary, el, script,
                                                                      cpu_model())
    return mlups, n, sample


def run_reference(args):
    d = Dist(backend="gloo")
    if d.rank != 0:
        d.close()
        return 0
    from oracle import port
    nx, ny = args.nx, args.ny
    cores = port.max_threads()
    # bounded sample: the whole lattice if all steps fit about two minutes,
    # else a strip of rows of it
    rows = nx
    a, b = _cpu_lattice(rows, ny, args.storage)
    t0 = time.perf_counter()
    port.run_raw(a, b, args.boundary, args.omega, args.u0, 1)
    t1 = time.perf_counter() - t0
    budget = 120.0
    if t1 * (args.steps + args.warmup) > budget:
        rows = max(64, int(nx * budget / (t1 * (args.steps + args.warmup))))
        a, b = _cpu_lattice(rows, ny, args.storage)
    if args.warmup > 1:
        port.run_raw(a, b, args.boundary, args.omega, args.u0, args.warmup - 1)
    t0 = time.perf_counter()
    port.run_raw(a, b, args.boundary, args.omega, args.u0, args.steps)
    el = time.perf_counter() - t0
    mlups = rows * ny * args.steps / el / 1e6
    sample = "each step: one %s step of a %d x %d strip of the %d x %d lattice (%s), C port of the reference " \
             "step on %d host threads" % (args.boundary, rows, ny, nx, ny, args.storage, cores)
    line = {
        "impl": "reference", "metric": METRIC, "value": round(mlups, 3), "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(el / args.steps * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.storage == "f64" else "f32", "data": "synthetic (cavity from rest at equilibrium)",
        "config": workload_config(args),
        "cpu_baseline": {"value": round(mlups, 3), "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": round(mlups, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    d.close()
    return 0


def workload_config(args):
    kind = "lid-driven cavity" if args.boundary == "cavity" else "periodic"
    return {"workload": "D2Q9 BGK %s %dx%d, %s populations, omega=%g%s" % (
        kind, args.nx, args.ny, args.storage, args.omega, (", u_lid=%g" % args.u0) if args.boundary == "cavity" else ""),
        "nx": args.nx, "ny": args.ny, "storage": args.storage, "boundary": args.boundary, "omega": args.omega,
        "u_lid": args.u0 if args.boundary == "cavity" else None,
        "l2": "inputs larger than L2 (each population buffer %.2f GB vs 129 MB L2); no flush" % (
            9 * args.nx * args.ny * {"f32": 4, "f64": 8}.get(args.storage, 2) / 1e9),
        "parallelism": "replicas (one lattice per GPU)"}


# ---------------------------------------------------------------- our arm
def run_ours(args):
    import torch
    d = Dist()
    dev = torch.device("cuda", d.local_rank)
    torch.cuda.set_device(dev)
    import latticeboltzmann_gb300 as PyLB
    from latticeboltzmann_gb300 import _lib

    _lib.set_tuning(_lib.TUNE_KERNEL, _lib.KERNELS[args.kernel])
    if args.stages:
        _lib.set_tuning(_lib.TUNE_STAGES, args.stages)
    lat = PyLB.Lattice(args.nx, args.ny, args.omega, boundary=args.boundary, u0=args.u0, storage=args.storage,
                       device=dev, rounding=args.rounding)
    stream = torch.cuda.current_stream(dev)
    # one launch per event: two steps each where the two-step kernel applies
    chunk = lat.steps_per_launch if args.steps % lat.steps_per_launch == 0 else 1
    launches = args.steps // chunk
    for _ in range(args.warmup):  # warm-up launches of the timed kernel
        lat.step(chunk)
    torch.cuda.synchronize(dev)

    clocks = ClockSampler(d.local_rank)
    if d.rank == 0:
        clocks.start()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(launches + 1)]
    d.barrier()
    torch.cuda.synchronize(dev)
    ev[0].record(stream)
    for i in range(launches):
        lat.step(chunk)
        ev[i + 1].record(stream)
    torch.cuda.synchronize(dev)
    d.barrier()
    clk = clocks.stop() if d.rank == 0 else None
    _lib.device_status()  # raises if a bounded device-side wait gave up
    per_launch_ms = [ev[i].elapsed_time(ev[i + 1]) for i in range(launches)]
    total_s = ev[0].elapsed_time(ev[-1]) / 1e3
    mlups, t_max = aggregate_mlups(lat.cells, args.steps, total_s, d, dev)

    # end to end through the public API with host-resident populations
    e2e = None
    if not args.no_e2e:
        host_path = args.storage in ("f32", "f64")
        host = torch.empty((9, args.nx, args.ny), dtype=lat.state.dtype if host_path else torch.float32,
                           pin_memory=True)
        lat.populations(out=host)
        torch.cuda.synchronize(dev)

        def e2e_step():
            if host_path:
                # upload, update and download pipelined by row blocks (public
                # API); the device status is checked once after the loop
                lat.step_host(host, check=False, copy_streams=args.copy_streams)
            else:
                lat.load(host)
                lat.step(1)
                lat.populations(out=host)

        for _ in range(2):
            e2e_step()
        torch.cuda.synchronize(dev)
        d.barrier()
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            e2e_step()
        torch.cuda.synchronize(dev)
        el = time.perf_counter() - t0
        _lib.device_status()
        d.barrier()
        e_mlups, _ = aggregate_mlups(lat.cells, args.e2e_steps, el, d, dev)
        nbytes = host.numel() * host.element_size()
        link_s = host_link_seconds(host, dev, streams=args.copy_streams)
        bound = lat.cells / link_s / 1e6
        e2e = {"value": round(e_mlups, 3), "unit": UNIT, "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
               "steps": args.e2e_steps,
               "path": ("Lattice.step_host(pinned host): row blocks uploaded, updated and downloaded, %d copy "
                        "stream(s) per direction" % args.copy_streams)
               if host_path else "Lattice.load(pinned host) + Lattice.step + Lattice.populations(out=pinned host)",
               "link": {"two_way_gbs": round(2 * nbytes / link_s / 1e9, 1), "bound": round(bound, 1),
                        "frac": round(e_mlups / d.world / bound, 4),
                        "how": "one step's upload and download as concurrent copy-engine copies on %d stream(s) "
                               "per direction, no compute" % args.copy_streams}}
        del host

    if d.rank != 0:
        d.close()
        return 0

    bpc = lat.bytes_per_cell_update  # per cell and launch: one read and one write of the lattice
    avg_launch_s = sum(per_launch_ms) / len(per_launch_ms) / 1e3
    achieved = bpc * lat.cells / avg_launch_s / 1e9
    peak, peak_src = hbm_peak()
    kname = "k_step2" if chunk == 2 else "k_step_pipe"
    traffic, prof = profiled_traffic(args.storage, args.boundary, lat.cells, kname)
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": None if traffic is None else round(traffic),
                "algorithmic_bytes": bpc * lat.cells, "steps_per_launch": chunk,
                "bytes_per_cell_update": bpc / chunk,
                "kernel": ("k_step2 (two fused steps per launch: pull stream + bounce-back/lid + BGK, the "
                           "intermediate step in shared memory)" if chunk == 2 else
                           "k_step (fused pull stream + bounce-back/lid + BGK)"),
                "peak_source": peak_src,
                "traffic_source": None if prof is None else prof.get("source")}
    extras = {}
    want = set() if args.no_extras else {x.strip() for x in args.extras.split(",") if x.strip()}
    unknown = want - {"operator_path", "fp16_store", "warm_start"}
    if unknown:
        raise SystemExit("bench.py: unknown extras %s" % sorted(unknown))
    if args.boundary == "cavity":
        if "operator_path" in want:
            extras["operator_path"] = operator_path(args, dev)
        if "fp16_store" in want:
            extras["fp16_store"] = storage_comparison(args, dev, d.local_rank)
        if "warm_start" in want:
            extras["warm_start"] = warm_start(args, dev)
    cpu = None
    if not args.no_cpu_baseline:
        c_mlups, cores, sample = cpu_port_sample(args.nx, args.ny, args.omega, args.u0, args.storage, args.boundary,
                                                 args.cpu_seconds)
        cpu = {"value": round(c_mlups, 3), "unit": UNIT, "cores": cores, "kind": "port", "sample": sample,
               "cpu_model": cpu_model()}
        if args.storage == "f32" and args.boundary in ("cavity", "periodic"):
            try:
                n_mlups, n_cores, n_sample = numpy_opt1_sample(args.ny, args.omega, args.u0, args.boundary)
                cpu["numpy_opt1"] = {"value": round(n_mlups, 3), "unit": UNIT, "cores": n_cores, "sample": n_sample}
            except Exception as e:  # a baseline that could not run is reported, not hidden
                cpu["numpy_opt1"] = {"error": "%s: %s" % (type(e).__name__, e)}
    line = {
        "metric": METRIC, "value": round(mlups, 1), "unit": UNIT, "n_gpus": d.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(t_max / args.steps * 1e3, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64" if args.storage == "f64" else "f32",
        "data": "synthetic (cavity from rest at equilibrium)", "config": workload_config(args),
        "e2e": e2e, "gpu_launches": launches, "roofline": roofline, "cpu_baseline": cpu, "clocks": clk,
        "hbm_gbs": round(achieved, 1),
    }
    line.update(extras)
    print(json.dumps(line), flush=True)
    d.close()
    return 0


def time_storage(n, storage, dev, steps, warmup, gpu_index, omega=1.7, u0=0.1, rounding="nearest"):
    """CUDA-event MLUPS of the fused cavity step at n x n in one storage (one
    launch per step), with the clock record of its own timed region."""
    import torch
    import latticeboltzmann_gb300 as PyLB
    from latticeboltzmann_gb300 import _lib
    lat = PyLB.Lattice(n, n, omega, boundary="cavity", u0=u0, storage=storage, device=dev, rounding=rounding)
    stream = torch.cuda.current_stream(dev)
    lat.step(warmup)
    torch.cuda.synchronize(dev)
    clocks = ClockSampler(gpu_index)
    clocks.start()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
    ev[0].record(stream)
    for i in range(steps):
        lat.step(1)
        ev[i + 1].record(stream)
    torch.cuda.synchronize(dev)
    clk = clocks.stop()
    _lib.device_status()
    total_s = ev[0].elapsed_time(ev[-1]) / 1e3
    bpc = lat.bytes_per_cell_update
    achieved = bpc * lat.cells * steps / total_s / 1e9
    peak, _ = hbm_peak()
    out = {"mlups": round(lat.cells * steps / total_s / 1e6, 1), "ms_per_step": round(total_s / steps * 1e3, 4),
           "bytes_per_cell": bpc, "achieved_gbs": round(achieved, 1), "frac": round(achieved / peak, 4),
           "rounding": rounding if storage in ("f16dev", "bf16dev") else None, "steps": steps, "clocks": clk}
    del lat
    torch.cuda.empty_cache()
    return out


def storage_comparison(args, dev, gpu_index):
    """FP32 against 16-bit deviation storage on the n x n cavity (the
    reference's cavity_opt1.py:177-245 lid, omega 1.7, u0 0.1), plus the
    error of each 16-bit mode against an FP64 run of the same kernel at
    1024^2 after 1000 steps (relative L2 of u, total-mass drift)."""
    from latticeboltzmann_gb300 import studies
    n = args.store_n
    rows = {}
    for storage, rounding in (("f32", "nearest"), ("f16dev", "nearest"), ("bf16dev", "nearest"),
                              ("f16dev", "stochastic"), ("bf16dev", "stochastic")):
        key = storage + ("+sr" if rounding == "stochastic" else "")
        rows[key] = time_storage(n, storage, dev, args.store_steps, max(3, args.warmup), gpu_index,
                                 rounding=rounding)
    f32 = rows["f32"]["mlups"]
    err = {}
    for r in studies.precision(n=1024, omegas=(1.7,), steps=1000, storages=("f32", "f32dev", "f16dev", "bf16dev",
                                                                            "f16dev+sr", "bf16dev+sr"),
                               device=dev, checkpoints=(1000,)):
        err[r["storage"]] = {"rel_l2_u": r["rel_l2_u"], "mass_drift": round(r["mass_drift"], 6),
                             "mass_drift_fp64": round(r["mass_drift_fp64"], 6)}
    return {"workload": "cavity %dx%d, omega 1.7, u_lid 0.1, from rest; 16-bit storage holds f_i - w_i, "
                        "FP32 arithmetic" % (n, n),
            "rows": rows, "ratio_vs_f32": {k: round(v["mlups"] / f32, 3) for k, v in rows.items() if k != "f32"},
            "error_vs_fp64": {"case": "cavity 1024^2, omega 1.7, u_lid 0.1, 1000 steps, against the FP64 "
                                      "kernel (itself within 1e-12 of the FP64 oracle)", "by_storage": err}}


WEIGHTS = os.path.join(ROOT, "latticeboltzmann_gb300", "weights", "fno_cavity256_bf16.npz")


def weight_files():
    """The committed network and any further ensemble members
    (fno_cavity256_bf16_m<k>.npz, trained on the same data and split)."""
    import glob
    extra = sorted(glob.glob(os.path.join(os.path.dirname(WEIGHTS), "fno_cavity256_bf16_m*.npz")))
    return [WEIGHTS] + extra


def warm_start(args, dev):
    """Time to steady state of the lid-driven cavity started from rest (cold)
    and from the surrogate's prediction in its Chapman-Enskog state (warm; the
    wall time includes the network's inference and the start kernel), for a
    fixed set of the trained network's held-out (Re, u_lid) pairs: evenly
    spaced in Re at 256^2, and the lowest-Re ones evaluated at 1024^2.
    Steady: max |u(t+1000) - u(t)| < 1e-7 (the reference's cold start is
    cavity_opt1.py:333-335).  Each cavity runs alone, in FP32-deviation
    storage (FP64 only if its change stalls above the tolerance)."""
    import numpy as np
    import torch
    from latticeboltzmann_gb300 import surrogate as S
    from latticeboltzmann_gb300.fno import FNO2d
    if not os.path.exists(WEIGHTS):
        return {"unavailable": "no trained weights at %s" % os.path.relpath(WEIGHTS, ROOT)}
    files = weight_files()
    members = [FNO2d.load(p, device=dev) for p in files]
    meta = members[0].meta or {}
    re, u = np.asarray(meta.get("held_out_re", [])), np.asarray(meta.get("held_out_u", []))
    if re.size == 0:
        return {"unavailable": "the weights file names no held-out cases"}
    if any(list((m.meta or {}).get("held_out_re", [])) != re.tolist() for m in members[1:]):
        return {"unavailable": "the ensemble members were not trained on the same held-out split"}
    net = members[0] if len(members) == 1 else S.Ensemble(members)
    order = np.argsort(re)
    pick = order[np.linspace(0, len(order) - 1, min(args.warm_cases, len(order))).astype(int)]
    keys = ("epochs", "train_s", "val_rel_l2_u", "val_rel_l2_rho", "samples", "train_seed")
    out = {"weights": [os.path.relpath(p, ROOT) for p in files], "tol": 1e-7,
           "network": [{k: (m.meta or {}).get(k) for k in keys} for m in members]}
    for n, sel in ((256, pick), (1024, order[:args.warm_cases_large])):
        if len(sel) == 0:
            continue
        rows = S.single_case_timing(net, re[sel], u[sel], n, dev, max_steps=600_000 if n == 256 else 1_500_000)
        cold = sum(r["cold_s"] for r in rows)
        warm = sum(r["warm_s"] for r in rows)
        out["n%d" % n] = {"cases": [{k: (round(v, 4) if isinstance(v, float) else v) for k, v in r.items()}
                                    for r in rows],
                          "cold_s": round(cold, 3), "warm_s": round(warm, 3),
                          "wall_ratio": round(cold / warm, 3) if warm > 0 else None,
                          "steps_ratio": round(sum(r["cold_steps"] for r in rows) /
                                               max(1, sum(r["warm_steps"] for r in rows)), 3)}
    del net
    torch.cuda.empty_cache()
    return out


def operator_path(args, dev):
    """MLUPS of the reference's loop body through the drop-in operators
    (cavity_opt2.py:276-277): Streaming.stream_and_bounce_back (in place:
    edge records, then tiles streamed through shared memory) then
    Collision.collide, on the benchmark lattice in FP32.  144 algorithmic
    bytes per cell per step (stream 72, collide 72; the edge records add
    ~7 more) against the fused step's 72."""
    import torch
    import latticeboltzmann_gb300 as PyLB
    from latticeboltzmann_gb300 import _lib
    nx, ny = args.nx, args.ny
    f = torch.empty((9, nx, ny), dtype=torch.float32, device=dev)
    one = torch.ones(nx * ny, dtype=torch.float32, device=dev)
    zero = torch.zeros(nx * ny, dtype=torch.float32, device=dev)
    PyLB.equilibrium(one, zero, zero, f.reshape(9, -1))
    del one, zero
    stream = torch.cuda.current_stream(dev)

    def step():
        PyLB.Streaming.stream_and_bounce_back(f, args.u0)
        PyLB.collide(f.reshape(9, -1), args.omega)

    def timed(fn):
        for _ in range(max(3, args.warmup)):
            fn()
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize(dev)
        _lib.device_status()
        return e0.elapsed_time(e1) / 1e3

    steps = max(5, min(args.steps, 20))
    secs = timed(step)
    s_secs = timed(lambda: PyLB.Streaming.stream_and_bounce_back(f, args.u0))
    peak, _ = hbm_peak()
    del f
    torch.cuda.empty_cache()
    return {"mlups": round(nx * ny * steps / secs / 1e6, 1), "ms_per_step": round(secs / steps * 1e3, 4),
            "bytes_per_cell": 144, "frac": round(144 * nx * ny * steps / secs / 1e9 / peak, 4), "steps": steps,
            "stream_only": {"mlups": round(nx * ny * steps / s_secs / 1e6, 1),
                            "ms": round(s_secs / steps * 1e3, 4), "bytes_per_cell": 72,
                            "frac": round(72 * nx * ny * steps / s_secs / 1e9 / peak, 4)},
            "launches_per_step": 3,
            "path": "PyLB.Streaming.stream_and_bounce_back (in place: k_ip_save + k_ip_stream) + PyLB.collide, "
                    "float32 (%dx%d)" % (nx, ny)}


def host_link_seconds(host, dev, reps=3, streams=1):
    """Seconds for one step's host traffic with nothing else running: the upload
    of ``host`` and a download of the same size as concurrent copies, each
    direction split over ``streams`` streams -- the ceiling of any per-step
    host round trip with that many copy streams."""
    import torch
    scratch = torch.empty(host.shape, dtype=host.dtype, device=dev)
    dev_buf = torch.empty_like(scratch)
    back = torch.empty(host.shape, dtype=host.dtype, pin_memory=True)
    k = max(1, int(streams))
    ups = [torch.cuda.Stream(dev) for _ in range(k)]
    downs = [torch.cuda.Stream(dev) for _ in range(k)]
    parts = list(zip(torch.chunk(scratch.view(-1), k), torch.chunk(host.view(-1), k),
                     torch.chunk(back.view(-1), k), torch.chunk(dev_buf.view(-1), k)))
    cur = torch.cuda.current_stream(dev)

    def once():
        for su, sd, (sc, h, bk, db) in zip(ups, downs, parts):
            su.wait_stream(cur)
            sd.wait_stream(cur)
            with torch.cuda.stream(su):
                sc.copy_(h, non_blocking=True)
            with torch.cuda.stream(sd):
                bk.copy_(db, non_blocking=True)
        for st in ups + downs:
            cur.wait_stream(st)

    once()
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for _ in range(reps):
        once()
    torch.cuda.synchronize(dev)
    el = (time.perf_counter() - t0) / reps
    del scratch, dev_buf, back
    return el


def run_batched(args):
    """512 uneven periodic shear-wave lattices (nx 32..1024, ny 16..512 log-uniform,
    omega 0.3..1.9, seeded) advanced together; MLUPS over all instances' cells."""
    import torch
    d = Dist()
    dev = torch.device("cuda", d.local_rank)
    torch.cuda.set_device(dev)
    from latticeboltzmann_gb300 import batch as B
    from latticeboltzmann_gb300 import _lib
    sizes, om = B.random_shear_batch(512, seed=0)
    bl = B.BatchedLattice(sizes, om, boundary="periodic", storage=args.storage, device=dev).shear_wave(0.05)
    best, timings = bl.autotune()
    stream = torch.cuda.current_stream(dev)
    for _ in range(args.warmup):
        bl.step(1)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    d.barrier()
    torch.cuda.synchronize(dev)
    ev[0].record(stream)
    bl.step(args.steps)
    ev[1].record(stream)
    torch.cuda.synchronize(dev)
    d.barrier()
    _lib.device_status()
    secs = ev[0].elapsed_time(ev[1]) / 1e3
    mlups, t_max = aggregate_mlups(bl.cells, args.steps, secs, d, dev)
    if d.rank == 0:
        bpc = 18 * torch.empty(0, dtype=bl.state.dtype).element_size()
        achieved = bpc * bl.cells / (secs / args.steps) / 1e9
        peak, peak_src = hbm_peak()
        print(json.dumps({
            "metric": "MLUPS (512 batched uneven D2Q9 shear-wave lattices, one launch per step)",
            "value": round(mlups, 1), "unit": UNIT, "n_gpus": d.world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(t_max / args.steps * 1e3, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if args.storage == "f64" else "f32", "data": "synthetic (seeded batch)",
            "config": {"workload": "512 periodic shear-wave lattices, nx log-uniform 32..1024, ny 16..512, "
                                   "omega 0.3..1.9, seed 0, %s" % args.storage, "cells": bl.cells,
                       "launch": bl.config},
            "gpu_launches": args.steps,
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "traffic": None, "peak_source": peak_src,
                         "kernel": "k_batch_step_flat / k_batch_step (autotuned)"},
        }), flush=True)
    d.close()
    return 0


def main(argv=None):
    args = parse(argv)
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batched-shear":
        return run_batched(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
