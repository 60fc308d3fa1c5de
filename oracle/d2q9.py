"""CPU oracle for the D2Q9 BGK hot path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` may import this module, and only as the checker (or as the
timed CPU baseline).  The product (``latticeboltzmann_gb300``) never calls it.

This is a numpy restatement of the reference's hot-path arithmetic, written
in pull form.  Citations are to files of IMTEK-Simulation/LatticeBoltzmann:

* lattice constants: ``PyLB/Streaming.py:28-29``,
  ``simulators/parallel_lid_drive_cavity/cavity_opt1.py:72,88-96``;
* ``equilibrium`` (numpy op order): ``cavity_opt1.py:100-132``;
* ``equilibrium_cxx`` / ``collide_cxx`` (C++ op order of the native
  extension): ``c/d2q9.h:59-81`` and ``c/d2q9.h:121-131``;
* ``collide`` (numpy op order): ``cavity_opt1.py:134-160``;
* ``stream`` (periodic): ``PyLB/Streaming.py:33-46``;
* ``stream_and_bounce_back`` (half-way bounce-back, Ladd moving lid, with the
  reference's corner and lid-density behaviour): ``cavity_opt1.py:177-245``.

Parity pin: ``tests/golden/make_golden.py`` runs the reference's own numpy
functions (extracted from the scripts above and from
``tests/02-CollideTest.py``) on seeded inputs and commits the outputs as
``tests/golden/*.npz``; ``tests/test_oracle_golden.py`` checks this module
against them.
"""

import numpy as np

# Channel order 0, E, N, W, S, NE, NW, SW, SE (PyLB/Streaming.py:28-29).
CX = np.array([0, 1, 0, -1, 0, 1, -1, -1, 1], dtype=np.int64)
CY = np.array([0, 0, 1, 0, -1, 1, 1, -1, -1], dtype=np.int64)
C_IC = np.stack([CX, CY], axis=1)
W_I = np.array([4 / 9, 1 / 9, 1 / 9, 1 / 9, 1 / 9, 1 / 36, 1 / 36, 1 / 36, 1 / 36])
OPP = np.array([0, 3, 4, 1, 2, 7, 8, 5, 6], dtype=np.int64)
E, N, W, S, NE, NW, SW, SE = range(1, 9)


def equilibrium(rho, ux, uy):
    """Equilibrium populations, numpy operation order of cavity_opt1.py:100-132.

    Returns a new array of shape ``(9,) + rho.shape`` in the inputs' dtype.
    """
    dt = np.result_type(rho, ux, uy)
    w0, w1, w5 = (dt.type(4 / 9), dt.type(1 / 9), dt.type(1 / 36))
    uu = ux ** 2 + uy ** 2
    out = []
    for i in range(9):
        # python ints keep numpy's weak scalar promotion (float32 stays float32)
        cu = int(CX[i]) * ux + int(CY[i]) * uy if i else None
        w = w0 if i == 0 else (w1 if i < 5 else w5)
        if i == 0:
            out.append(w * rho * (1 - 3 / 2 * uu))
        else:
            out.append(w * rho * (1 + 3 * cu + 9 / 2 * cu ** 2 - 3 / 2 * uu))
    return np.array(out, dtype=dt)


def equilibrium_cxx(rho, ux, uy):
    """Equilibrium in the operation order of the native kernel (c/d2q9.h:59-81).

    ``ux`` and ``uy`` are scaled by 3 first; ``uu = (ux^2 + uy^2)/6``;
    ``f_i = w_i rho (1 + cu + cu^2/2 - uu)``.
    """
    rho = np.asarray(rho)
    dt = np.result_type(rho, ux, uy)
    rho = rho.astype(dt, copy=False)
    w0 = 4 * rho / dt.type(9)
    w1 = rho / dt.type(9)
    w5 = rho / dt.type(36)
    ux = np.asarray(ux, dtype=dt) * dt.type(3)
    uy = np.asarray(uy, dtype=dt) * dt.type(3)
    cu5, cu6, cu7, cu8 = ux + uy, -ux + uy, -ux - uy, ux - uy
    uu = (ux * ux + uy * uy) / dt.type(6)
    one, half = dt.type(1), dt.type(2)
    return np.array([
        w0 * (one - uu),
        w1 * (one + ux + ux * ux / half - uu),
        w1 * (one + uy + uy * uy / half - uu),
        w1 * (one - ux + ux * ux / half - uu),
        w1 * (one - uy + uy * uy / half - uu),
        w5 * (one + cu5 + cu5 * cu5 / half - uu),
        w5 * (one + cu6 + cu6 * cu6 / half - uu),
        w5 * (one + cu7 + cu7 * cu7 / half - uu),
        w5 * (one + cu8 + cu8 * cu8 / half - uu),
    ], dtype=dt)


def macroscopic(f):
    """Density and velocity of populations ``f`` (cavity_opt1.py:154-156)."""
    rho = np.sum(f, axis=0)
    ux = (f[1] - f[3] + f[5] - f[6] - f[7] + f[8]) / rho
    uy = (f[2] - f[4] + f[5] + f[6] - f[7] - f[8]) / rho
    return rho, ux, uy


def collide(f, omega):
    """BGK collision in place, numpy order (cavity_opt1.py:134-160).

    Returns ``(rho, ux, uy)`` computed before the relaxation.
    """
    rho, ux, uy = macroscopic(f)
    f += omega * (equilibrium(rho, ux, uy) - f)
    return rho, ux, uy


def eigen_sum9(v):
    """Sum of the nine rows of ``v`` in the order Eigen 3.4.0 (the reference's
    pinned, un-vendored dependency, setup.py:32) reduces a fixed-size
    9-vector: the unrolled reduction splits a run of n coefficients into its
    first n//2 and the rest and adds the two sums, i.e.
    ``((v0+v1)+(v2+v3)) + ((v4+v5)+(v6+(v7+v8)))``."""
    def part(a, n):
        if n == 1:
            return v[a]
        h = n // 2
        return part(a, h) + part(a + h, n - h)
    return part(0, 9)


def collide_cxx(f2d, omega):
    """BGK collision in place on a ``(9, N)`` view, C++ order (c/d2q9.h:121-131).

    The density is ``f_i.sum()`` of a fixed-size Eigen vector (``eigen_sum9``);
    returns ``None`` like the native binding.
    """
    dt = f2d.dtype
    omega = dt.type(omega)
    rho = eigen_sum9(f2d)
    ux = (f2d[1] - f2d[3] + f2d[5] - f2d[6] - f2d[7] + f2d[8]) / rho
    uy = (f2d[2] - f2d[4] + f2d[5] + f2d[6] - f2d[7] - f2d[8]) / rho
    feq = equilibrium_cxx(rho, ux, uy)
    f2d += omega * (feq - f2d)


def _pull_periodic(g):
    """Raw periodic pull: ``out_i(k, l) = g_i((k - cx_i) mod nx, (l - cy_i) mod ny)``."""
    _, nx, ny = g.shape
    k = np.arange(nx)
    l = np.arange(ny)
    out = np.empty_like(g)
    for i in range(9):
        out[i] = g[i][np.ix_((k - CX[i]) % nx, (l - CY[i]) % ny)]
    return out


def stream(f):
    """Periodic streaming in place (PyLB/Streaming.py:33-46)."""
    f[...] = _pull_periodic(f)


def lid_density(g, pulled):
    """Lid density per column ``k`` at the top row (cavity_opt1.py:206-210).

    Sum, in the reference's order, of the pre-stream outgoing NW, N, NE at the
    top row and the raw periodic pull (before any wall overwrite) of NW, N, NE,
    W, 0, E at the top row.  At ``k = 0`` and ``k = nx - 1`` the raw pull reads
    across the periodic seam -- the reference does the same.
    """
    t = g.shape[2] - 1
    return (g[NW, :, t] + g[N, :, t] + g[NE, :, t]
            + pulled[NW, :, t] + pulled[N, :, t] + pulled[NE, :, t]
            + pulled[W, :, t] + pulled[0, :, t] + pulled[E, :, t])


def stream_and_bounce_back(f, u0=0.1):
    """Stream with half-way bounce-back on four walls and a moving lid, in place.

    Pull-form restatement of cavity_opt1.py:177-245 (identical in
    cavity_opt0.py:155-223 and cavity_opt2.py:109-177).  ``g`` is the
    pre-stream state; every node is a fluid node and the walls sit half a
    cell outside the array.

    * a population whose source lies inside the array is pulled from there;
    * a population whose source lies outside through the bottom and/or a
      side wall is bounced back from the same node: ``f_i = g_opp(i)``;
    * a population whose source lies outside only through the top (lid) gets
      ``f_S = g_N``, ``f_SE = g_NW + 6 w_SE rho_lid u0``,
      ``f_SW = g_NE - 6 w_SW rho_lid u0``;
    * the diagonals that leave through the top AND a side (SE at the top-left
      node, SW at the top-right node) get plain bounce-back, without the lid
      term, because the side-wall writes come last in the reference.
    """
    _, nx, ny = f.shape
    if nx < 2 or ny < 2:
        raise ValueError("stream_and_bounce_back needs nx >= 2 and ny >= 2")
    g = f.copy()
    pulled = _pull_periodic(g)
    dt = f.dtype
    w = W_I.astype(dt)
    rho_lid = lid_density(g, pulled)
    f[...] = pulled
    t, r = ny - 1, nx - 1
    # bottom wall (l = 0): N, NE, NW come from below
    f[N, :, 0] = g[S, :, 0]
    f[NE, :, 0] = g[SW, :, 0]
    f[NW, :, 0] = g[SE, :, 0]
    # lid (l = ny-1): S, SE, SW come from above
    f[S, :, t] = g[N, :, t]
    f[SE, :, t] = g[NW, :, t] + 6 * w[SE] * rho_lid * u0
    f[SW, :, t] = g[NE, :, t] - 6 * w[SW] * rho_lid * u0
    # left wall (k = 0): E, NE, SE come from the left; overrides the lid at (0, t)
    f[E, 0, :] = g[W, 0, :]
    f[NE, 0, :] = g[SW, 0, :]
    f[SE, 0, :] = g[NW, 0, :]
    # right wall (k = nx-1): W, NW, SW; overrides the lid at (r, t)
    f[W, r, :] = g[E, r, :]
    f[NW, r, :] = g[SE, r, :]
    f[SW, r, :] = g[NE, r, :]


def stream_and_bounce_back_ladd(f, u0=0.1):
    """Standard Ladd moving wall with wall density 1 (boundary code 2).

    Not in the reference; the kernels offer it for steady-state work because
    the reference's lid term 6 w rho_lid u0 uses a rho_lid that reads across
    the periodic seam and skips the corners, which makes the cavity gain mass
    and leaves it without a steady state.  Here every lid node, both corners
    included, gets f_S = g_N, f_SE = g_NW + 6 w u0 and f_SW = g_NE - 6 w u0
    (w = 1/36); the rest is stream_and_bounce_back with a resting lid.
    """
    _, nx, ny = f.shape
    if nx < 2 or ny < 2:
        raise ValueError("stream_and_bounce_back needs nx >= 2 and ny >= 2")
    t = ny - 1
    g_nw, g_ne = f[NW, :, t].copy(), f[NE, :, t].copy()
    stream_and_bounce_back(f, 0.0)
    lid = 6 * W_I.astype(f.dtype)[SE] * u0
    f[SE, :, t] = g_nw + lid
    f[SW, :, t] = g_ne - lid


def cavity_ladd_step(f, omega, u0=0.1):
    """One cavity step with the wall-density-1 lid (stream_and_bounce_back_ladd)."""
    stream_and_bounce_back_ladd(f, u0)
    return collide(f, omega)


def _grad(u, axis, periodic, wall_lo=0.0, wall_hi=0.0):
    """d u / d axis: central differences; at a cavity wall the quadratic through
    the wall value half a cell out and the next two nodes."""
    n = u.shape[axis]
    if n < 2:
        return np.zeros_like(u)
    if periodic:
        return 0.5 * (np.roll(u, -1, axis) - np.roll(u, 1, axis))
    u = np.moveaxis(u, axis, 0)
    g = np.empty_like(u)
    g[1:-1] = 0.5 * (u[2:] - u[:-2])
    g[0] = -4.0 / 3.0 * wall_lo + u[0] + u[1] / 3.0
    g[-1] = 4.0 / 3.0 * wall_hi - u[-1] - u[-2] / 3.0
    return np.moveaxis(g, 0, axis)


def chapman_enskog(rho, ux, uy, omega, periodic=False, u0=0.0, post_collision=False):
    """Equilibrium plus first-order Chapman-Enskog non-equilibrium populations.

    f_i = f_i^eq - (3 w_i rho / omega) (c_ia c_ib - delta_ab/3) d_a u_b (c_s^2 = 1/3);
    post_collision: f^eq + (1 - omega) f^neq, the state a step leaves.
    Not in the reference (its cavity starts from rest, cavity_opt1.py:333-335);
    the warm start of a predicted flow uses it.  For the cavity the lid (l = ny-1)
    moves with (u0, 0) and the other walls rest.
    """
    dxux = _grad(ux, 0, periodic)
    dxuy = _grad(uy, 0, periodic)
    dyux = _grad(ux, 1, periodic, 0.0, u0)
    dyuy = _grad(uy, 1, periodic)
    f = equilibrium(rho, ux, uy)
    scale = (1.0 - omega) if post_collision else 1.0
    for i in range(9):
        ex, ey = float(CX[i]), float(CY[i])
        q = (ex * ex - 1.0 / 3.0) * dxux + ex * ey * (dxuy + dyux) + (ey * ey - 1.0 / 3.0) * dyuy
        f[i] -= scale * 3.0 * W_I[i] * rho / omega * q
    return f


def cavity_step(f, omega, u0=0.1):
    """One cavity time step in the reference's order (cavity_opt1.py:341-343)."""
    stream_and_bounce_back(f, u0)
    return collide(f, omega)


def periodic_step(f, omega):
    """One periodic time step (shear_wave_opt1.py:170-172)."""
    stream(f)
    return collide(f, omega)


def shear_wave_init(nx, ny, amplitude=1.0, dtype=np.float64, along="y"):
    """Shear-wave initial state at rest density.

    ``along="y"``: ``uy(k) = A sin(2 pi k / nx)`` (shear_wave_opt1.py:157-163);
    ``along="x"``: ``ux(l) = A sin(2 pi l / ny)``.
    """
    rho = np.ones((nx, ny), dtype=dtype)
    ux = np.zeros((nx, ny), dtype=dtype)
    uy = np.zeros((nx, ny), dtype=dtype)
    if along == "y":
        uy[:] = (amplitude * np.sin(2 * np.pi * np.arange(nx) / nx)).astype(dtype)[:, None]
    else:
        ux[:] = (amplitude * np.sin(2 * np.pi * np.arange(ny) / ny)).astype(dtype)[None, :]
    return equilibrium(rho, ux, uy)


def density_wave_init(nx, ny, eps=0.01, dtype=np.float64):
    """``rho(k) = 1 + eps sin(2 pi k / nx)``, zero velocity, at equilibrium."""
    rho = np.ones((nx, ny), dtype=dtype) + (eps * np.sin(2 * np.pi * np.arange(nx) / nx)).astype(dtype)[:, None]
    z = np.zeros((nx, ny), dtype=dtype)
    return equilibrium(rho, z, z)
