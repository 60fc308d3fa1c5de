"""Channel flows with dry wall rows ("convention B") -- TEST INFRASTRUCTURE ONLY.

numpy restatement of the boundary operators of the reference's simple-flow
scripts, the checker of latticeboltzmann_gb300/Channel.py:

* simulators/simple_flows/PoiseuilleFlow.py:59-75 ``bounce_back(grid, uw)``:
  the first and last rows (y = 0, y = ny-1) are wall rows; after a push
  stream the populations that entered them are reflected into the adjacent
  fluid rows, columns 1 .. nx-2 only; the top wall moves with uw
  (SW and SE gain -uw/6 and +uw/6).
* simulators/simple_flows/CouetteFlow.py:106-119 ``bounce_back(grid, uw)``:
  the same reflection over every column, then the wall entries are cleared.
* simulators/simple_flows/PoiseuilleFlow.py:76-88
  ``periodic_boundary_with_pressure_variations``: ghost columns x = 0 and
  x = nx-1 get the equilibrium at the inlet/outlet density and the velocity
  of the opposite interior column, plus that column's non-equilibrium part.
* the drivers ``couette_flow`` / ``poiseuille_flow`` (PoiseuilleFlow.py:91-147)
  as step functions over the oracle's stream and BGK collide.

Channels: 0 rest, 1 E, 2 N, 3 W, 4 S, 5 NE, 6 NW, 7 SW, 8 SE (as everywhere).
"""

import numpy as np

from . import d2q9


def bounce_back_walls(f, uw=0.0, interior=True, clear=False):
    """Dry-wall bounce-back of the wall rows y = 0 and y = ny-1, in place."""
    _, nx, ny = f.shape
    cols = slice(1, nx - 1) if interior else slice(None)
    t = ny - 1
    f[2, cols, 1] = f[4, cols, 0]
    f[5, cols, 1] = f[7, cols, 0]
    f[6, cols, 1] = f[8, cols, 0]
    if clear:
        f[4, cols, 0] = 0
        f[7, cols, 0] = 0
        f[8, cols, 0] = 0
    f[4, cols, t - 1] = f[2, cols, t]
    f[7, cols, t - 1] = f[5, cols, t] - uw / 6
    f[8, cols, t - 1] = f[6, cols, t] + uw / 6
    if clear:
        f[2, cols, t] = 0
        f[5, cols, t] = 0
        f[6, cols, t] = 0


def pressure_periodic(f, rho_in, rho_out):
    """Pressure-periodic ghost columns x = 0 (inlet) and x = nx-1 (outlet), in place."""
    rho, ux, uy = d2q9.macroscopic(f)
    feq = d2q9.equilibrium(rho, ux, uy)
    a = d2q9.equilibrium(np.full(f.shape[2], rho_in), ux[-2, :], uy[-2, :]) + (f[:, -2, :] - feq[:, -2, :])
    b = d2q9.equilibrium(np.full(f.shape[2], rho_out), ux[1, :], uy[1, :]) + (f[:, 1, :] - feq[:, 1, :])
    f[:, 0, :] = a
    f[:, -1, :] = b


def push_stream(f):
    """Periodic push stream (the scripts' np.roll by +c_i) -- the same map as d2q9.stream."""
    d2q9.stream(f)


def couette_step(f, omega, uw):
    """One step of PoiseuilleFlow.py's couette_flow: collide, stream, wall bounce-back."""
    d2q9.collide(f, omega)
    push_stream(f)
    bounce_back_walls(f, uw, interior=True)
    return f


def poiseuille_step(f, omega, rho_in, rho_out, uw=0.0):
    """One step of PoiseuilleFlow.py's poiseuille_flow: pressure ghosts, stream, walls, collide."""
    pressure_periodic(f, rho_in, rho_out)
    push_stream(f)
    bounce_back_walls(f, uw, interior=True)
    d2q9.collide(f, omega)
    return f


def couette_step_cleared(f, omega, uw):
    """One step in the order of CouetteFlow.py's fast_calc (stream, collide,
    bounce-back over every column with the wall entries cleared), with the
    correct BGK equilibrium: that script's own equilibrium_on_array
    (CouetteFlow.py:79-82) has ux + uy in channels 6 and 8, a bug not
    reproduced here."""
    push_stream(f)
    d2q9.collide(f, omega)
    bounce_back_walls(f, uw, interior=False, clear=True)
    return f


def solid_bounce_back(f, solid, periodic=True):
    """Link-wise dry-node bounce-back around solid nodes (a boolean (nx, ny)
    mask), in place: f_opp(i)(x - c_i) <- f_i(x) for solid x and fluid x - c_i.
    (A generalisation of the scripts' wall and obstacle reflections, which copy
    diagonals within one column; for rows of solid nodes and flow uniform along
    them the two agree.)"""
    _, nx, ny = f.shape
    src = f.copy()
    for k, l in zip(*np.nonzero(solid)):
        for i in range(1, 9):
            ks, ls = k - int(d2q9.CX[i]), l - int(d2q9.CY[i])
            if periodic:
                ks, ls = ks % nx, ls % ny
            elif not (0 <= ks < nx and 0 <= ls < ny):
                continue
            if not solid[ks, ls]:
                f[d2q9.OPP[i], ks, ls] = src[i, k, l]
