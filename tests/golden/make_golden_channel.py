"""Golden fixtures of the channel-flow boundary operators, from the reference's
own scripts (run where the reference checkout is present; it does not travel):

    python tests/golden/make_golden_channel.py /path/to/LatticeBoltzmann

Functions are lifted with ``ast`` (function definitions plus the module-level
constants they read; plotting, printing and the script bodies are dropped):

* ``simulators/simple_flows/PoiseuilleFlow.py`` -- ``bounce_back`` (columns
  1 .. nx-2), ``periodic_boundary_with_pressure_variations``, ``stream``,
  ``caluculate_real_values``, ``collision`` and the loops of ``couette_flow``
  and ``poiseuille_flow``;
* ``simulators/simple_flows/CouetteFlow.py`` -- ``bounce_back`` (every
  column, wall entries cleared).  Its ``fast_calc`` loop is not a fixture:
  that script's ``equilibrium_on_array`` (CouetteFlow.py:79-82) uses
  ux + uy where channels 6 (NW) and 8 (SE) need uy - ux and ux - uy, so it
  is not the BGK operator of the rest of the reference.

Inputs come from ``numpy.random.default_rng`` with the seeds stored beside
them.  Output: ``reference_channel.npz`` next to this script.
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_golden import _lift  # noqa: E402


def main(ref):
    pois = _lift(os.path.join(ref, "simulators/simple_flows/PoiseuilleFlow.py"), np.float64,
                 keep_names=("relaxation", "velocity_set", "rho_null", "diff"))
    cou = _lift(os.path.join(ref, "simulators/simple_flows/CouetteFlow.py"), np.float64,
                keep_names=("relaxation", "velocity_set", "channels"))
    out = {}
    seed = 11
    rng = np.random.default_rng(seed)
    f = 0.02 + 0.2 * rng.random((9, 12, 10))
    out["seed"] = np.array(seed)
    out["bb_in"] = f.copy()
    g = f.copy()
    pois["bounce_back"](g, 0.1)
    out["bb_interior_uw0.1"] = g
    g = f.copy()
    cou["bounce_back"](g, 0.1)
    out["bb_cleared_uw0.1"] = g
    # near-equilibrium state for the pressure ghosts
    rho = 1 + 0.01 * rng.standard_normal((12, 10))
    ux = 0.02 * rng.standard_normal((12, 10))
    uy = 0.02 * rng.standard_normal((12, 10))
    f = pois["equilibrium_on_array"](rho, ux, uy) + 0.001 * rng.standard_normal((9, 12, 10))
    out["pp_in"] = f.copy()
    g = f.copy()
    pois["periodic_boundary_with_pressure_variations"](g, 1.001, 0.999)
    out["pp_out"] = g
    # the drivers' loops on a 14 x 12 grid (ghost columns / wall rows included)
    for relax in (0.5, 1.3):
        pois["relaxation"] = relax
        cou["relaxation"] = relax
        one, zero = np.ones((14, 12)), np.zeros((14, 12))
        grid = pois["equilibrium_on_array"](one, zero, zero)
        for _ in range(300):
            pois["periodic_boundary_with_pressure_variations"](grid, 1.001, 0.999)
            pois["stream"](grid)
            pois["bounce_back"](grid, 0.0)
            r, x, y = pois["caluculate_real_values"](grid)
            pois["collision"](grid, r, x, y)
        out["poiseuille_%g" % relax] = grid
        grid = pois["equilibrium_on_array"](one, zero, zero)
        for _ in range(300):
            r, x, y = pois["caluculate_real_values"](grid)
            pois["collision"](grid, r, x, y)
            pois["stream"](grid)
            pois["bounce_back"](grid, 0.1)
        out["couette_%g" % relax] = grid
    np.savez_compressed(os.path.join(HERE, "reference_channel.npz"), **out)
    print("wrote", os.path.join(HERE, "reference_channel.npz"), sorted(out))


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("LB_REFERENCE")
    if not ref:
        sys.exit("usage: %s REFERENCE_CHECKOUT (or set LB_REFERENCE)" % sys.argv[0])
    main(ref)
