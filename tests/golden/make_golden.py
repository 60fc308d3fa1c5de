"""Generate the golden fixtures in this folder from the reference's own code.

Run once where the reference checkout is present (it does not travel):

    python tests/golden/make_golden.py /path/to/LatticeBoltzmann

The reference's numpy functions are lifted out of its scripts with ``ast``:
function definitions and the module-level constants they use are executed in
a fresh namespace; the MPI driver, argv parsing and main loop are dropped.
At one MPI rank the reference's ``communicate()`` is an exact no-op
(``Create_cart(periods=False)`` gives PROC_NULL neighbours), so dropping it
changes nothing.  Sources used:

* ``simulators/parallel_lid_drive_cavity/cavity_opt1.py`` -- ``equilibrium``,
  ``collide``, ``stream``, ``stream_and_bounce_back`` (float64 and float32);
* ``simulators/parallel_lid_drive_cavity/cavity_opt0.py`` -- einsum-form twins;
* ``simulators/serial_shear_wave/Python/shear_wave_opt1.py`` -- periodic run
  and its amplitude diagnostic;
* ``PyLB/Streaming.py`` -- ``stream`` (imported as a plain file);
* ``tests/02-CollideTest.py`` -- ``d2q9_equilibrium_ref``,
  ``d2q9_collide_ref`` (the reference test-suite's own oracles).

Every input is drawn from ``numpy.random.default_rng`` with the seed stored
next to it, so each fixture also records how to regenerate its inputs.
"""

import ast
import os
import sys
from enum import IntEnum

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _lift(path, dtype, keep_names=()):
    """Execute the function defs and simple constants of a reference script."""
    src = open(path).read()
    tree = ast.parse(src)
    body = []
    for node in tree.body:
        if isinstance(node, ast.FunctionDef):
            body.append(node)
        elif isinstance(node, ast.Assign):
            names = [t.id for t in node.targets if isinstance(t, ast.Name)]
            if names and all(n in keep_names for n in names):
                body.append(node)
    mod = ast.Module(body=body, type_ignores=[])
    ns = {"np": np, "IntEnum": IntEnum, "dtype": np.dtype(dtype)}
    exec(compile(mod, path, "exec"), ns)
    return ns


def lift_cavity(ref, name, dtype):
    path = os.path.join(ref, "simulators/parallel_lid_drive_cavity", name)
    return _lift(path, dtype, keep_names=("D", "c_ic", "w_0", "w_1234", "w_5678", "w_i"))


def lift_shear(ref, dtype):
    path = os.path.join(ref, "simulators/serial_shear_wave/Python/shear_wave_opt1.py")
    ns = _lift(path, dtype, keep_names=("c_ic",))
    # the script's weights are dtype(...) scalars of its module-level dtype
    ns["w_0"], ns["w_1234"], ns["w_5678"] = (np.dtype(dtype).type(4 / 9),
                                              np.dtype(dtype).type(1 / 9),
                                              np.dtype(dtype).type(1 / 36))
    return ns


def lift_collide_test(ref):
    path = os.path.join(ref, "tests/02-CollideTest.py")
    return _lift(path, np.float64, keep_names=("c_ic", "w_i"))


def lift_streaming(ref):
    path = os.path.join(ref, "PyLB/Streaming.py")
    ns = {"__name__": "reference_streaming"}
    exec(compile(open(path).read(), path, "exec"), ns)
    return ns


def main(ref):
    out = {}
    ct = lift_collide_test(ref)
    st = lift_streaming(ref)

    # 1. equilibrium, collide vs the reference test-suite oracles (float64)
    seed = 1001
    rng = np.random.default_rng(seed)
    for shape in [(2, 2), (7, 5)]:
        rho = np.abs(rng.random(shape))
        ux = rng.random(shape)
        uy = rng.random(shape)
        tag = "%dx%d" % shape
        out["eq_in_rho_" + tag] = rho
        out["eq_in_ux_" + tag] = ux
        out["eq_in_uy_" + tag] = uy
        out["eq_out_" + tag] = ct["d2q9_equilibrium_ref"](rho, np.array([ux, uy]))
    f = np.abs(rng.random((9, 4, 4)))
    out["col_in"] = f
    for om in (0.5, 1.7):
        c = f.copy()
        ct["d2q9_collide_ref"](c, om)
        out["col_out_%g" % om] = c
    out["seed_collide_test"] = np.array(seed)

    # 2. periodic stream (PyLB.Streaming.stream), odd sizes
    rng = np.random.default_rng(2002)
    f = rng.random((9, 5, 7))
    out["stream_in"] = f
    g = f.copy()
    st["stream"](g)
    out["stream_out"] = g
    out["seed_stream"] = np.array(2002)

    # 3. stream_and_bounce_back / collide / equilibrium of cavity_opt1, f64 and f32
    for dt in (np.float64, np.float32):
        tagd = np.dtype(dt).name
        cav = lift_cavity(ref, "cavity_opt1.py", dt)
        rng = np.random.default_rng(3003)
        for (nx, ny) in [(6, 5), (8, 8), (2, 3)]:
            f = rng.random((9, nx, ny)).astype(dt)
            for u0 in (0.0, 0.1):
                g = f.copy()
                cav["stream_and_bounce_back"](g, u0)
                key = "sbb_%s_%dx%d_u%g" % (tagd, nx, ny, u0)
                out[key + "_in"] = f
                out[key + "_out"] = g
        # numpy-order collide (returns rho, ux, uy)
        f = (rng.random((9, 6, 4)) * 0.2 + 0.02).astype(dt)
        g = f.copy()
        rho, ux, uy = cav["collide"](g, np.array(1.7, dtype=dt))
        out["npcol_%s_in" % tagd] = f
        out["npcol_%s_out" % tagd] = g
        out["npcol_%s_rho" % tagd] = rho
        out["npcol_%s_ux" % tagd] = ux
        out["npcol_%s_uy" % tagd] = uy

        # a short cavity run from rest, in the reference's step order
        nx, ny, nsteps = 24, 16, 200
        f = cav["equilibrium"](np.ones((nx, ny), dtype=dt), np.zeros((nx, ny), dtype=dt),
                               np.zeros((nx, ny), dtype=dt))
        omega = np.array(1.7, dtype=dt)
        mass = []
        for _ in range(nsteps):
            cav["stream_and_bounce_back"](f)
            rho, ux, uy = cav["collide"](f, omega)
            mass.append(float(np.sum(f, dtype=np.float64)))
        out["cav_%s_f" % tagd] = f
        out["cav_%s_ux" % tagd] = ux
        out["cav_%s_uy" % tagd] = uy
        out["cav_%s_mass" % tagd] = np.array(mass)
        out["cav_%s_cfg" % tagd] = np.array([nx, ny, nsteps, 1.7, 0.1])
        # same with a resting lid: mass must be conserved
        f = cav["equilibrium"](np.ones((nx, ny), dtype=dt), np.zeros((nx, ny), dtype=dt),
                               np.zeros((nx, ny), dtype=dt))
        f[:, nx // 3, ny // 2] *= 1.5
        m0 = float(np.sum(f, dtype=np.float64))
        for _ in range(50):
            cav["stream_and_bounce_back"](f, 0.0)
            cav["collide"](f, omega)
        out["cavrest_%s_f" % tagd] = f
        out["cavrest_%s_m0" % tagd] = np.array(m0)

    # 4. einsum-form twins of cavity_opt0 must agree with opt1 (float64)
    cav0 = lift_cavity(ref, "cavity_opt0.py", np.float64)
    rng = np.random.default_rng(4004)
    rho = 1 + 0.1 * rng.random((5, 6))
    u = 0.05 * (rng.random((2, 5, 6)) - 0.5)
    out["opt0_eq_rho"] = rho
    out["opt0_eq_u"] = u
    out["opt0_eq_out"] = cav0["equilibrium"](rho, u)

    # 5. periodic shear wave of shear_wave_opt1 (float64): amplitude series
    sw = lift_shear(ref, np.float64)
    nx = ny = 32
    omega = 0.3
    uy_k = np.sin(2 * np.pi / nx * np.arange(nx))
    f = sw["equilibrium"](np.ones((nx, ny)), np.zeros_like(uy_k).reshape((nx, 1)),
                          uy_k.reshape((nx, 1)))
    ampl = []
    for _ in range(100):
        sw["stream"](f)
        rho, ux, uy = sw["collide"](f, omega)
        ampl.append((uy[:, ny // 2] * uy_k).sum() * 2 / nx)
    out["shear_f"] = f
    out["shear_ampl"] = np.array(ampl)
    out["shear_cfg"] = np.array([nx, ny, 100, omega])

    np.savez_compressed(os.path.join(HERE, "reference_d2q9.npz"), **out)
    print("wrote %d arrays" % len(out))


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("LB_REFERENCE")
    if not ref:
        sys.exit("usage: %s REFERENCE_CHECKOUT (or set LB_REFERENCE)" % sys.argv[0])
    main(ref)
