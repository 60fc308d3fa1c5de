"""Measured studies on the device-resident solver.

``density_wave``    periodic lattice, rho(x) = 1 + eps sin(2 pi x/nx), u = 0:
                    records the first Fourier mode of the density along x and
                    fits A exp(-G t) cos(c_s k t + phi); for D2Q9 BGK the
                    acoustic damping rate is G = nu k^2 with
                    nu = (1/omega - 1/2)/3 (the viscosity relation of
                    simulators/simple_flows/shear_wave_decay.py:162).
``shear_wave``      periodic lattice, u_x = A sin(2 pi y/ny): the velocity mode
                    decays as exp(-nu k^2 t) (shear_wave_decay.py:72-76,167).
``precision``       the lid-driven cavity in FP32 / FP16 / BF16 storage against
                    an FP64 run of the same kernel: relative L2 error of the
                    velocity field and the drift of the total mass.

Command line: ``python -m latticeboltzmann_gb300.studies {density,precision}``
prints one JSON line per result.
"""

import argparse
import json
import math
import time

import numpy as np
import torch

from .solver import Lattice, viscosity_from_omega

CS = 1.0 / math.sqrt(3.0)


def _density_mode(lat):
    rho, _, _ = lat.macroscopic()
    prof = rho.double().mean(dim=1)          # average over y
    x = torch.arange(lat.nx, dtype=torch.float64, device=prof.device)
    k = 2 * math.pi / lat.nx
    return float((prof * torch.sin(k * x)).sum() * 2 / lat.nx)


def density_wave(nx=256, ny=128, omega=1.0, steps=10000, eps=0.01, storage="f64", every=1, device=None):
    """Acoustic decay of a periodic density wave (256 x 128, omega 1.0, FP64
    by default); returns the series and the fit."""
    lat = Lattice(nx, ny, omega, boundary="periodic", storage=storage, device=device)
    x = torch.arange(nx, dtype=torch.float64, device=lat.device)
    rho = (1 + eps * torch.sin(2 * math.pi * x / nx))[:, None].expand(nx, ny)
    lat.equilibrium(rho=rho)
    t, a = [0], [_density_mode(lat)]
    t0 = time.perf_counter()
    for s in range(every, steps + 1, every):
        lat.step(every)
        t.append(s)
        a.append(_density_mode(lat))
    elapsed = time.perf_counter() - t0
    t, a = np.array(t, dtype=np.float64), np.array(a)
    fit = fit_damped_cosine(t, a, nx, omega)
    fit.update({"elapsed_s": elapsed, "nx": nx, "ny": ny, "omega": omega, "steps": steps, "storage": storage})
    return t, a, fit


def fit_damped_cosine(t, a, nx, omega):
    """Least-squares fit of a(t) = A exp(-G t) cos(w t + phi)."""
    from scipy.optimize import curve_fit
    k = 2 * math.pi / nx
    nu = viscosity_from_omega(omega)

    def model(tt, A, G, w, phi):
        return A * np.exp(-G * tt) * np.cos(w * tt + phi)

    p0 = [a[0], nu * k * k, CS * k, 0.0]
    p, _ = curve_fit(model, t, a, p0=p0, maxfev=20000)
    A, G, w, phi = p
    return {"amplitude": float(A), "damping": float(G), "frequency": float(w),
            "nu_fit": float(G / (k * k)), "nu_theory": nu, "cs_fit": float(w / k), "cs_theory": CS,
            "rel_err_nu": float(G / (k * k) / nu - 1.0)}


def shear_wave(nx=64, ny=128, omega=1.0, steps=2000, amplitude=0.05, storage="f64", every=50, device=None):
    """Velocity shear wave u_x(y); returns the fitted viscosity."""
    lat = Lattice(nx, ny, omega, boundary="periodic", storage=storage, device=device)
    y = torch.arange(ny, dtype=torch.float64, device=lat.device)
    k = 2 * math.pi / ny
    lat.equilibrium(ux=(amplitude * torch.sin(k * y))[None, :].expand(nx, ny))
    ts, amps = [], []
    for s in range(every, steps + 1, every):
        lat.step(every)
        _, ux, _ = lat.macroscopic()
        amps.append(float((ux.double().mean(dim=0) * torch.sin(k * y)).sum() * 2 / ny))
        ts.append(s)
    ts, amps = np.array(ts, dtype=np.float64), np.array(amps)
    good = amps > 1e-6 * amplitude
    slope = np.polyfit(ts[good], np.log(amps[good]), 1)[0]
    return {"nu_fit": float(-slope / k ** 2), "nu_theory": viscosity_from_omega(omega)}


def _u64(lat):
    """Velocity of the stored populations, decoded and computed in FP64 (an
    FP32 velocity would add its own rounding, ~1e-7 relative, to the error
    being measured)."""
    from .solver import macroscopic
    _, ux, uy = macroscopic(lat.populations(torch.float64))
    return ux, uy


def _rel_l2_u(lat, ux_ref, uy_ref):
    ux, uy = _u64(lat)
    num = torch.sqrt(((ux - ux_ref) ** 2 + (uy - uy_ref) ** 2).sum())
    den = torch.sqrt((ux_ref ** 2 + uy_ref ** 2).sum())
    return float(num / den)


def _make(n, omega, u0, variant, device):
    storage, _, mode = variant.partition("+")
    rounding = "stochastic" if mode == "sr" else "nearest"
    lat = Lattice(n, n, omega, boundary="cavity", u0=u0, storage=storage, device=device, rounding=rounding, seed=1)
    if mode in ("perturb", "perturb-centre"):
        # control run: the same arithmetic with the rest population of one node
        # moved by 1e-12 -- how fast the flow itself separates two runs.  The
        # node sits one row below the middle of the lid (in the flow from the
        # first step) or, for "perturb-centre", at the centre of the cavity.
        f = lat.populations(torch.float64)
        f[0, n // 2, n // 2 if mode == "perturb-centre" else n - 2] += 1e-12
        lat.load(f)
    return lat


def precision(n=1024, omegas=(1.0, 1.7, 1.95), steps=50000, u0=0.1,
              storages=("f32", "f16dev", "bf16dev", "f16dev+sr", "bf16dev+sr"), device=None,
              checkpoints=(1000, 5000, 10000, 20000, 50000)):
    """Error of reduced-precision storage against an FP64 run of the same cavity.

    All lattices advance together; at each checkpoint the relative L2 error of
    the velocity field against the FP64 lattice and the mass drift are
    recorded.  A "+sr" suffix selects stochastic rounding of the 16-bit codes;
    "f64+perturb" / "f64+perturb-centre" is an FP64 control run whose start
    differs by 1e-12 in one population next to the lid / at the centre (it
    separates from the reference run only as fast as the flow amplifies small
    differences).
    """
    out = []
    marks = sorted({c for c in checkpoints if c <= steps} | {steps})
    for omega in omegas:
        lats = {"f64": Lattice(n, n, omega, boundary="cavity", u0=u0, storage="f64", device=device)}
        for st in storages:
            lats[st] = _make(n, omega, u0, st, device)
        m0 = {st: float(l.mass_momentum()[0]) for st, l in lats.items()}
        done = 0
        for mark in marks:
            for lat in lats.values():
                lat.step(mark - done)
            done = mark
            ref = lats["f64"]
            ux_ref, uy_ref = _u64(ref)
            finite = bool(torch.isfinite(ux_ref).all())
            m_ref = float(ref.mass_momentum()[0]) - m0["f64"]
            for st in storages:
                lat = lats[st]
                _, ux, _ = lat.macroscopic()
                ok = finite and bool(torch.isfinite(ux).all())
                out.append({"n": n, "omega": omega, "steps": mark, "storage": st, "fp64_finite": finite,
                            "mass_drift_fp64": m_ref, "mass_drift": float(lat.mass_momentum()[0]) - m0[st],
                            "rel_l2_u": _rel_l2_u(lat, ux_ref, uy_ref) if ok else None})
        del lats
    return out


def main(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("study", choices=["density", "shear", "precision"])
    p.add_argument("--n", type=int, default=1024)
    p.add_argument("--steps", type=int, default=0)
    p.add_argument("--omegas", type=str, default="1.0,1.7,1.95")
    p.add_argument("--storages", type=str, default="f32,f16dev,bf16dev,f16dev+sr,bf16dev+sr",
                   help="precision study: comma-separated storages compared with FP64")
    p.add_argument("--checkpoints", type=str, default="1000,5000,10000,20000,50000",
                   help="precision study: comma-separated step counts at which the error is recorded")
    a = p.parse_args(argv)
    if a.study == "density":
        _, _, fit = density_wave(steps=a.steps or 10000)
        print(json.dumps({"study": "density_wave", **fit}))
    elif a.study == "shear":
        print(json.dumps({"study": "shear_wave", **shear_wave(steps=a.steps or 2000)}))
    else:
        for row in precision(n=a.n, omegas=[float(x) for x in a.omegas.split(",")], steps=a.steps or 50000,
                             storages=tuple(a.storages.split(",")),
                             checkpoints=tuple(int(x) for x in a.checkpoints.split(","))):
            print(json.dumps({"study": "precision", **row}))


if __name__ == "__main__":
    main()
