"""Channel flows with dry wall rows: Couette and pressure-driven Poiseuille.

The reference's simple-flow scripts use a second boundary convention next to
the cavity's half-way bounce-back: the first and last rows of the grid are
wall rows; after a push stream the populations that entered a wall row are
copied back into the adjacent fluid row as their opposites
(simulators/simple_flows/PoiseuilleFlow.py:59-75, CouetteFlow.py:106-119),
and a pressure difference drives the flow through ghost columns at the ends
(PoiseuilleFlow.py:76-88).  These operators act in place on a CUDA
``(9, nx, ny)`` float32/float64 tensor, like the rest of the package, and
compose with ``Streaming.stream`` and ``Collision.collide``; ``couette_flow``
and ``poiseuille_flow`` run the scripts' loops (PoiseuilleFlow.py:91-147) on
the device with two ping-pong buffers.
"""

import torch

from . import _lib
from ._tensor import lattice, storage_code, stream_handle

__all__ = ["bounce_back", "solid_bounce_back", "pressure_periodic", "couette_flow", "poiseuille_flow",
           "couette_profile", "poiseuille_profile"]


def bounce_back(f, uw=0.0, interior=True, clear=False):
    """Reflect what entered the wall rows y = 0 and y = ny-1 back into the fluid.

    The top wall moves with ``uw`` in +x.  ``interior``: columns 1 .. nx-2
    only (PoiseuilleFlow.py, whose end columns are pressure ghosts); else every
    column.  ``clear``: zero the reflected wall entries (CouetteFlow.py).
    """
    nx, ny = lattice(f, "bounce_back")
    code = storage_code(f, "bounce_back")
    _lib.call("lbgb_wall_bounce_back", f.data_ptr(), nx, ny, float(uw), int(bool(interior)), int(bool(clear)),
              code, stream_handle(f))


def solid_bounce_back(f, solid, periodic=True):
    """Return every population that streamed into a solid node to the fluid
    node it came from, reversed (link-wise dry-node bounce-back), in place.

    ``solid``: a CUDA bool/uint8 tensor (nx, ny), nonzero where the node is
    solid (an obstacle, or walls of any shape).  The obstacle channel of the
    reference (experimantal_flows/obstacle_canal.py:413-458) reflects around a
    rectangle the same way, copying diagonals within one column.
    """
    nx, ny = lattice(f, "solid_bounce_back")
    code = storage_code(f, "solid_bounce_back")
    if not isinstance(solid, torch.Tensor) or solid.device != f.device or tuple(solid.shape) != (nx, ny):
        raise ValueError("solid_bounce_back: solid must be an (nx, ny) tensor on the populations' device")
    m = solid.to(torch.uint8).contiguous()
    _lib.call("lbgb_solid_bounce_back", f.data_ptr(), m.data_ptr(), nx, ny, int(bool(periodic)), code,
              stream_handle(f))


def pressure_periodic(f, rho_in, rho_out):
    """Set the inlet (x = 0) and outlet (x = nx-1) ghost columns from the
    prescribed densities and the opposite interior columns' velocity and
    non-equilibrium part."""
    nx, ny = lattice(f, "pressure_periodic")
    code = storage_code(f, "pressure_periodic")
    _lib.call("lbgb_pressure_periodic", f.data_ptr(), nx, ny, float(rho_in), float(rho_out), code,
              stream_handle(f))


class _Loop:
    """Two device buffers and the per-step kernels of a channel run."""

    def __init__(self, nx, ny, dtype, device):
        from .Collision import equilibrium
        dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.nx, self.ny = nx, ny
        self.a = torch.empty((9, nx, ny), dtype=dtype, device=dev)
        self.b = torch.empty_like(self.a)
        n = nx * ny
        equilibrium(torch.ones(n, dtype=dtype, device=dev), torch.zeros(n, dtype=dtype, device=dev),
                    torch.zeros(n, dtype=dtype, device=dev), self.a.view(9, -1))
        self.code = storage_code(self.a, "channel")

    def stream(self):
        _lib.call("lbgb_stream_periodic", self.a.data_ptr(), self.b.data_ptr(), self.nx, self.ny, self.code,
                  stream_handle(self.a))
        self.a, self.b = self.b, self.a

    def collide(self, omega):
        n = self.nx * self.ny
        _lib.call("lbgb_collide", self.a.data_ptr(), n, n, self.code, float(omega), stream_handle(self.a))


def couette_flow(nx, ny, omega, uw, steps, interior=False, dtype=torch.float64, device=None):
    """Couette flow between a resting bottom wall row and a top wall row moving
    with ``uw``, periodic in x; the step of PoiseuilleFlow.py's couette_flow
    (collide, stream, bounce back).  ``interior=True`` reproduces that
    script's bounce-back, which skips the first and last column.  Returns the
    populations (9, nx, ny) after ``steps`` steps from rest."""
    run = _Loop(nx, ny, dtype, device)
    for _ in range(steps):
        run.collide(omega)
        run.stream()
        bounce_back(run.a, uw, interior=interior)
    return run.a


def poiseuille_flow(nx, ny, omega, rho_in, rho_out, steps, uw=0.0, dtype=torch.float64, device=None):
    """Pressure-driven channel: ghost columns at x = 0 and nx-1, wall rows at
    y = 0 and ny-1; the step of PoiseuilleFlow.py's poiseuille_flow (pressure
    ghosts, stream, bounce back, collide).  Returns the populations after
    ``steps`` steps from rest."""
    run = _Loop(nx, ny, dtype, device)
    for _ in range(steps):
        pressure_periodic(run.a, rho_in, rho_out)
        run.stream()
        bounce_back(run.a, uw, interior=True)
        run.collide(omega)
    return run.a


def couette_profile(ny, uw):
    """Analytic Couette profile u_x(y) on the fluid rows 1 .. ny-2: the walls
    sit half a cell beyond the first and last fluid rows."""
    y = torch.arange(1, ny - 1, dtype=torch.float64)
    return uw * (y - 0.5) / (ny - 2)


def poiseuille_profile(nx, ny, omega, rho_in, rho_out):
    """Analytic Poiseuille profile u_x(y) on the fluid rows: the pressure drop
    c_s^2 (rho_in - rho_out) over the nx - 2 fluid columns, walls half a cell
    beyond the first and last fluid rows (the analytic curve of
    PoiseuilleFlow.py:149-153)."""
    nu = (1.0 / omega - 0.5) / 3.0
    h = ny - 2
    y = torch.arange(h, dtype=torch.float64) + 0.5
    g = (rho_in - rho_out) / 3.0 / (nx - 2)
    return g / (2 * nu) * y * (h - y)
