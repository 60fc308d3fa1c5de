"""Surrogate warm start of the lid-driven cavity: training data, training, and
the warm-versus-cold study.

1. Training data: steady cavities from the batched solver (all instances in
   one batch, converged ones leave the queue), Re log-uniform in [10, 1000]
   and lid speed uniform in [0.05, 0.1], omega from Re = u L / nu with L the
   side.  Steady means max over the cavity of |u^(t+1000) - u^t| < 1e-7; FP32
   storage gets there below Re ~ 200, so the batch runs in FP32 down to 1e-6
   and finishes in FP64.
2. Training: the Fourier neural operator of ``fno.py`` on (Re, u) ->
   normalised (rho, ux, uy), Adam with a cosine learning-rate schedule, all on
   the package's kernels.
3. Study: held-out (Re, u) pairs run to the same tolerance from rest (cold)
   and from the predicted fields in their Chapman-Enskog state (warm); steps,
   wall time (the warm side includes inference and the start kernel) and the
   error of the prediction against the converged field.

The reference has no learned part (its cavity always starts from rest,
simulators/parallel_lid_drive_cavity/cavity_opt1.py:333-335).
"""

import argparse
import json
import math
import os
import time

import numpy as np
import torch

from . import _lib
from . import batch as B
from .fno import FNO2d, RE_RANGE, U_RANGE


def sample_parameters(n, seed=0, re_range=RE_RANGE, u_range=U_RANGE):
    """n pairs (Re log-uniform over re_range, lid speed uniform over u_range)."""
    rng = np.random.default_rng(seed)
    re = np.exp(rng.uniform(math.log(re_range[0]), math.log(re_range[1]), n))
    u = rng.uniform(u_range[0], u_range[1], n)
    return re, u


# How the steady runs go: FP32-deviation storage (same speed as FP32, a 10x
# lower rounding floor) straight to the tolerance; an instance whose velocity
# change stalls above it (its floor) finishes in FP64.  set_precision() changes
# it (the first data set was made with FP32 down to 1e-6, then FP64).
PRECISION = {"storage": "f32dev", "switch_tol": None}


def set_precision(storage="f32dev", switch_tol=None):
    PRECISION.update(storage=storage, switch_tol=switch_tol)


def steady_run(re, u, n, start=None, device=None, tol=1e-7, log=None, max_steps=600_000, tune=True):
    """Steady runs of a batch (see PRECISION); returns (fields (N, 3, n, n) FP32, steps, wall s, info)."""
    info = {}
    fields, steps, wall = B.steady_cavities(re, u, n=n, tol=tol, every=1000, max_steps=max_steps,
                                            storage=PRECISION["storage"], device=device, tune=tune, log=log,
                                            start=start, refine="f64", switch_tol=PRECISION["switch_tol"],
                                            info=info)
    return fields, steps, wall, info


def generate(n_samples, n=256, seed=0, device=None, log=None, max_steps=600_000, re_range=RE_RANGE):
    """Steady cavities for n_samples random (Re, u) pairs; instances that did not
    settle within max_steps (or diverged: a 48^2 cavity at Re 1000 is beyond
    the BGK stability limit) carry steps -1."""
    re, u = sample_parameters(n_samples, seed, re_range)
    fields, steps, wall, info = steady_run(re, u, n, device=device, log=log, max_steps=max_steps)
    return {"re": re, "u": u, "fields": fields, "steps": steps, "wall": wall, "info": info}


def sample_weights(t_all, idx, rho_weight=1.0, max_ratio=100.0, re=None, re_exp=0.0):
    """Loss weight of every (channel, sample) plane of the normalised targets
    t_all (3, S, n, n): the inverse of the plane's mean square, so that each
    sample's fields are fit to the same relative accuracy (the density
    channel (rho - 1) / u0^2 is ~100x smaller at Re 1000 than at Re 10, and
    with one weight for all samples the high-Re pressure -- the slowest part
    of those runs to settle -- would hardly count), capped at max_ratio times
    the smallest weight of the channel, scaled to mean 1 over ``idx`` and
    multiplied by (rho_weight, 1, 1).  re_exp > 0: each sample's weights are
    further multiplied by (Re / min Re)^re_exp, scaled to mean 1 over idx --
    the steps to steady grow like Re^0.6, so high-Re accuracy buys the most
    wall time."""
    ms = t_all.pow(2).mean(dim=(2, 3)).double()  # (3, S)
    w = 1.0 / ms.clamp_min(1e-30)
    sel = torch.as_tensor(np.asarray(idx), device=w.device)
    for c in range(w.shape[0]):
        lo = w[c].index_select(0, sel).min()
        w[c] = torch.minimum(w[c], lo * max_ratio)
        w[c] = w[c] / w[c].index_select(0, sel).mean()
    w[0] *= rho_weight
    if re is not None and re_exp:
        r = torch.as_tensor(np.asarray(re, dtype=np.float64), device=w.device)
        g = (r / r.index_select(0, sel).min()) ** re_exp
        w *= (g / g.index_select(0, sel).mean())[None, :]
    return w.float()


def train(net, data, idx, epochs=100, batch=16, lr=1e-3, lr_min=1e-5, log=None, seed=0, val_idx=None,
          seconds=None, weighting="relative", rho_weight=2.0, re_exp=0.0):
    """Adam on the samples ``idx`` of ``data`` (cosine schedule from lr to lr_min).

    weighting: "relative" (each (channel, sample) plane weighted to the same
    relative accuracy, the density channel by rho_weight; sample_weights) or
    "uniform" (one mean squared error over all planes).  seconds: a wall-time
    budget; after the third epoch the epoch count is set to what fits it (at
    most ``epochs``; the time of epochs 1-2 is the estimate, epoch 0 includes
    one-time set-up) and the schedule spans those.  Returns the history of
    (epoch, mean train loss, validation rel-L2 of u, of rho - 1)."""
    device = net.device
    fields = data["fields"]
    n = fields.shape[-1]
    targets = FNO2d.targets(fields, data["u"])  # (3, S, n, n)
    scale = targets[:, idx].reshape(3, -1).std(dim=1).clamp_min(1e-6)
    net.out_scale = scale.cpu().numpy()
    t_all = targets / scale[:, None, None, None]
    a_all = net.inputs(data["re"], data["u"], n, n)
    w_all = sample_weights(t_all, idx, rho_weight, re=data["re"], re_exp=re_exp) if weighting == "relative" else None
    rng = np.random.default_rng(seed)
    steps_per_epoch = max(1, len(idx) // batch)
    total = epochs * steps_per_epoch
    hist = []
    k = 0
    t_start = time.perf_counter()
    t_ep1 = None
    ep = 0
    while ep < epochs:
        perm = rng.permutation(idx)
        acc = torch.zeros((), dtype=torch.float64, device=device)
        for s in range(steps_per_epoch):
            sel = torch.as_tensor(np.sort(perm[s * batch:(s + 1) * batch]), device=device)
            a = a_all.index_select(1, sel).contiguous()
            t = t_all.index_select(1, sel).contiguous()
            w = None if w_all is None else w_all.index_select(1, sel).contiguous()
            acc += net.loss_and_backward(a, t, weight=w)
            cur = lr_min + 0.5 * (lr - lr_min) * (1 + math.cos(math.pi * min(k, total) / total))
            net.adam(cur)
            k += 1
        if seconds is not None and ep == 2:
            torch.cuda.synchronize(device)
            per_epoch = (time.perf_counter() - t_ep1) / 2
            epochs = max(3, min(epochs, int((seconds - (t_ep1 - t_start)) / per_epoch)))
            total = epochs * steps_per_epoch
            if log is not None:
                log("training: %.2f s per epoch, %d epochs in the %.0f s budget" % (per_epoch, epochs, seconds))
        # once per epoch: a GEMM whose bounded wait gave up left weights or
        # gradients incomplete; stop instead of training on them
        _lib.gemm_status()
        if log is not None and (ep % 25 == 0 or ep == epochs - 1):
            if val_idx is not None and len(val_idx):
                vl, vr = evaluate(net, data, val_idx, with_rho=True)
            else:
                vl = vr = float("nan")
            tl = float(acc) / steps_per_epoch
            hist.append((ep, tl, vl, vr))
            log("epoch %d train %.3e val rel-L2 u %.3e rho-1 %.3e lr %.2e" % (ep, tl, vl, vr, cur))
        if seconds is not None and ep == 0:
            # after epoch 0's one-time set-up and its validation pass
            torch.cuda.synchronize(device)
            t_ep1 = time.perf_counter()
        ep += 1
    return hist


def evaluate(net, data, idx, batch=16, with_rho=False):
    """Mean relative L2 error of the predicted velocity over the samples idx
    (and, with_rho, of the predicted rho - 1)."""
    n = data["fields"].shape[-1]
    errs, rerrs = [], []
    for s in range(0, len(idx), batch):
        sel = np.asarray(idx[s:s + batch])
        rho, ux, uy = net.predict(data["re"][sel], data["u"][sel], n, n)
        f = data["fields"][torch.as_tensor(sel, device=net.device)]
        num = ((ux - f[:, 1]) ** 2 + (uy - f[:, 2]) ** 2).sum(dim=(1, 2)).sqrt()
        den = (f[:, 1] ** 2 + f[:, 2] ** 2).sum(dim=(1, 2)).sqrt()
        errs.append((num / den).cpu())
        rnum = ((rho - f[:, 0]) ** 2).sum(dim=(1, 2)).sqrt()
        rden = ((f[:, 0] - 1) ** 2).sum(dim=(1, 2)).sqrt().clamp_min(1e-30)
        rerrs.append((rnum / rden).cpu())
    _lib.gemm_status()
    if with_rho:
        return float(torch.cat(errs).mean()), float(torch.cat(rerrs).mean())
    return float(torch.cat(errs).mean())


def study(net, re, u, n, device=None, tol=1e-7, log=None, max_steps=600_000, reference=None):
    """Warm versus cold start on the pairs (re, u) at n x n, both as one batch.

    Returns a dict with per-instance steps and the wall seconds of each side;
    the warm wall time includes the network's inference and the start
    kernel.  ``reference``: converged fields (N, 3, n, n) to compare the
    prediction with; by default the cold run's own result."""
    _warm_up(net, re, u, n, device, tune=True)
    cold_f, cold_steps, cold_wall, _ = steady_run(re, u, n, device=device, tol=tol, log=log, max_steps=max_steps)
    torch.cuda.synchronize(device)
    t0 = time.perf_counter()
    rho, ux, uy = net.predict(re, u, n, n)
    torch.cuda.synchronize(device)
    t_inf = time.perf_counter() - t0
    warm_f, warm_steps, warm_wall, _ = steady_run(re, u, n, device=device, tol=tol, log=log, max_steps=max_steps,
                                                  start=lambda b: (rho[b], ux[b], uy[b]))
    ref = cold_f if reference is None else reference
    du = ((ux - ref[:, 1]) ** 2 + (uy - ref[:, 2]) ** 2).sum(dim=(1, 2)).sqrt()
    un = (ref[:, 1] ** 2 + ref[:, 2] ** 2).sum(dim=(1, 2)).sqrt()
    dr = (rho - ref[:, 0]).abs().amax(dim=(1, 2))
    # the two steady answers agree to the solver's tolerance
    dfin = ((warm_f[:, 1:] - cold_f[:, 1:]).abs().amax(dim=(1, 2, 3)))
    return {"n": n, "re": np.asarray(re).tolist(), "u": np.asarray(u).tolist(),
            "cold_steps": cold_steps.tolist(), "warm_steps": warm_steps.tolist(),
            "cold_wall_s": cold_wall, "warm_wall_s": warm_wall + t_inf, "inference_s": t_inf,
            "pred_rel_l2_u": (du / un).cpu().numpy().tolist(), "pred_max_abs_rho": dr.cpu().numpy().tolist(),
            "steady_max_abs_du_warm_vs_cold": dfin.cpu().numpy().tolist()}


def _warm_up(net, re, u, n, device, tune):
    """One short untimed steady run and one prediction at this size, so that
    one-time set-up (kernel loading, workspaces, graph capture) is charged to
    neither side of a timing."""
    r0, u0 = np.atleast_1d(re)[:1], np.atleast_1d(u)[:1]
    steady_run(r0, u0, n, device=device, max_steps=2000, tune=tune)
    net.predict(r0, u0, n, n)
    torch.cuda.synchronize(device)


def single_case_timing(net, re, u, n, device=None, tol=1e-7, max_steps=600_000):
    """Wall time of each cavity (re[i], u[i]) run on its own, from rest and from
    the network's prediction (the warm time includes inference and the start
    kernel): what a user solving one cavity sees."""
    rows = []
    _warm_up(net, re, u, n, device, tune=False)
    for r, v in zip(np.atleast_1d(re), np.atleast_1d(u)):
        _, cs, cw, _ = steady_run([r], [v], n, device=device, tol=tol, max_steps=max_steps, tune=False)
        torch.cuda.synchronize(device)
        t0 = time.perf_counter()
        rho, ux, uy = net.predict([r], [v], n, n)
        _, ws, ww, _ = steady_run([r], [v], n, device=device, tol=tol, max_steps=max_steps, tune=False,
                                  start=lambda b: (rho[b], ux[b], uy[b]))
        torch.cuda.synchronize(device)
        warm = time.perf_counter() - t0
        rows.append({"re": float(r), "u": float(v), "cold_steps": int(cs[0]), "warm_steps": int(ws[0]),
                     "cold_s": cw, "warm_s": warm})
    return rows


class Ensemble:
    """Mean of several trained networks' predictions: independent fits make
    partly independent errors, which the mean reduces."""

    def __init__(self, nets):
        self.nets = list(nets)
        self.device = self.nets[0].device

    def predict(self, re, u_lid, nx, ny):
        acc = None
        for net in self.nets:
            p = net.predict(re, u_lid, nx, ny)  # views of the network's workspace
            acc = [x.clone() for x in p] if acc is None else [a.add_(x) for a, x in zip(acc, p)]
        k = 1.0 / len(self.nets)
        return tuple(a.mul_(k) for a in acc)


def load_networks(paths, device):
    """One network (.npz), or the Ensemble of several (a list of paths, or
    one string with comma-separated paths)."""
    if isinstance(paths, str):
        paths = [p for p in paths.split(",") if p]
    nets = [FNO2d.load(p, device=device) for p in paths]
    return nets[0] if len(nets) == 1 else Ensemble(nets)


def study_only(args):
    """Warm-versus-cold study of a trained network on the held-out pairs of
    an earlier run (no data generation, no training)."""
    os.makedirs(args.out, exist_ok=True)
    dev = torch.device("cuda", torch.cuda.current_device())
    logf = open(os.path.join(args.out, "log.txt"), "a")

    def log(m):
        print(m, flush=True)
        logf.write(m + "\n")
        logf.flush()

    net = load_networks(args.weights, dev)
    prev = json.load(open(args.held_out_from))
    val = np.asarray(prev["held_out"])
    re_all, u_all = np.asarray(prev["data_re"]), np.asarray(prev["data_u"])
    res = {"weights": [os.path.basename(p) for p in args.weights.split(",")], "storage": args.storage,
           "switch_tol": args.switch_tol}
    res["study"] = study(net, re_all[val], u_all[val], args.n, dev, max_steps=args.max_steps)
    s = res["study"]
    log("study %d: cold %.1f s, warm %.1f s (inference %.3f s); steps cold %d warm %d (sums)" % (
        args.n, s["cold_wall_s"], s["warm_wall_s"], s["inference_s"], sum(s["cold_steps"]), sum(s["warm_steps"])))
    sel = val[np.argsort(re_all[val])]
    sel = sel[np.linspace(0, len(sel) - 1, min(args.single_cases, len(sel))).astype(int)]
    res["single"] = single_case_timing(net, re_all[sel], u_all[sel], args.n, dev, max_steps=args.max_steps)
    for row in res["single"]:
        log("single %d: Re %.1f u %.3f cold %d steps %.2f s, warm %d steps %.2f s" % (
            args.n, row["re"], row["u"], row["cold_steps"], row["cold_s"], row["warm_steps"], row["warm_s"]))
    if args.study_large:
        low = val[re_all[val] <= 150]
        low = low[np.argsort(re_all[low])]
        sel = low[np.linspace(0, len(low) - 1, min(args.large_cases, len(low))).astype(int)] if len(low) else low
        res["single_large"] = single_case_timing(net, re_all[sel], u_all[sel], args.study_large, dev,
                                                 max_steps=1_500_000)
        for row in res["single_large"]:
            log("single %d: Re %.1f u %.3f cold %d steps %.2f s, warm %d steps %.2f s" % (
                args.study_large, row["re"], row["u"], row["cold_steps"], row["cold_s"], row["warm_steps"],
                row["warm_s"]))
    with open(os.path.join(args.out, "results.json"), "w") as f:
        json.dump(res, f, indent=1)
    return 0


def main(argv=None):
    ap = argparse.ArgumentParser(description="steady-cavity data, surrogate training and warm-start study")
    ap.add_argument("--samples", type=int, default=2000)
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--held-out", type=int, default=64)
    ap.add_argument("--epochs", type=int, default=150)
    ap.add_argument("--train-seconds", type=float, default=None,
                    help="wall-time budget of the training (the epoch count is fitted to it, at most --epochs)")
    ap.add_argument("--weighting", choices=["relative", "uniform"], default="relative",
                    help="loss weights per (channel, sample): same relative accuracy for every sample, or one MSE")
    ap.add_argument("--rho-weight", type=float, default=2.0, help="extra weight of the density channel")
    ap.add_argument("--init", default=None, help="start the training from these weights (.npz) instead of at random")
    ap.add_argument("--re-exp", type=float, default=0.0,
                    help="sample loss weights times (Re / Re_min)^re_exp (0: off)")
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--max-steps", type=int, default=600_000)
    ap.add_argument("--study-large", type=int, default=1024, help="side of the upsampled study (0: skip)")
    ap.add_argument("--large-cases", type=int, default=4)
    ap.add_argument("--single-cases", type=int, default=8, help="held-out cavities timed one at a time")
    ap.add_argument("--seed", type=int, default=0, help="seed of the data set and its held-out split")
    ap.add_argument("--train-seed", type=int, default=None,
                    help="seed of the first network's initialisation and sample order (default: --seed)")
    ap.add_argument("--members", type=int, default=1,
                    help="networks trained one after another (seeds train-seed, train-seed + 1, ...), each with "
                         "the full epoch / time budget; the study uses the mean of their predictions")
    ap.add_argument("--ensemble-with", default=None,
                    help="comma-separated trained networks (.npz) of the same data set and held-out split to add "
                         "to the study's ensemble")
    ap.add_argument("--out", default="surrogate_out")
    ap.add_argument("--storage", default="f32dev", help="storage of the steady runs before any FP64 refinement")
    ap.add_argument("--switch-tol", type=float, default=None,
                    help="run every instance to this change, then FP64 (default: FP64 only where a run stalls)")
    ap.add_argument("--weights", default=None,
                    help="study only: a trained network (.npz), or comma-separated networks whose predictions "
                         "are averaged, instead of training")
    ap.add_argument("--held-out-from", default=None,
                    help="study only: results.json of the training run that holds the held-out (Re, u) pairs")
    args = ap.parse_args(argv)
    set_precision(args.storage, args.switch_tol)
    if args.weights:
        return study_only(args)
    os.makedirs(args.out, exist_ok=True)
    dev = torch.device("cuda", torch.cuda.current_device())
    logf = open(os.path.join(args.out, "log.txt"), "a")

    def log(m):
        print(m, flush=True)
        logf.write(m + "\n")
        logf.flush()

    t0 = time.perf_counter()
    data = generate(args.samples, args.n, args.seed, dev, log, args.max_steps)
    ok = np.nonzero(data["steps"] > 0)[0]
    log("data: %d/%d steady in %.1f s; steps median %d max %d" % (len(ok), args.samples, data["wall"],
                                                                   int(np.median(data["steps"][ok])),
                                                                   int(data["steps"][ok].max())))
    rng = np.random.default_rng(args.seed + 1)
    perm = rng.permutation(ok)
    val, tr = perm[:args.held_out], perm[args.held_out:]
    tseed = args.seed if args.train_seed is None else args.train_seed
    nets, hists, t_train = [], [], 0.0
    for m in range(max(1, args.members)):
        net = FNO2d.load(args.init, device=dev) if args.init else FNO2d(device=dev, seed=tseed + m)
        t1 = time.perf_counter()
        hist = train(net, data, tr, epochs=args.epochs, batch=args.batch, lr=args.lr, log=log, val_idx=val,
                     seconds=args.train_seconds, weighting=args.weighting, rho_weight=args.rho_weight,
                     re_exp=args.re_exp, seed=tseed + m)
        torch.cuda.synchronize()
        t_m = time.perf_counter() - t1
        t_train += t_m
        tag = "" if m == 0 else "_m%d" % m
        net.save(os.path.join(args.out, "fno%s.npz" % tag))
        vu, vr = evaluate(net, data, val, with_rho=True)
        net.save(os.path.join(args.out, "fno_bf16%s.npz" % tag), bf16=True, meta={
            "n": args.n, "samples": args.samples, "seed": args.seed, "train_seed": tseed + m,
            "steady": int(len(ok)),
            "held_out_re": data["re"][val].tolist(), "held_out_u": data["u"][val].tolist(),
            "held_out_cold_steps": data["steps"][val].tolist(), "epochs": int(hist[-1][0]) + 1 if hist else 0,
            "train_s": t_m, "weighting": args.weighting, "rho_weight": args.rho_weight, "re_exp": args.re_exp,
            "val_rel_l2_u": vu, "val_rel_l2_rho": vr,
            "init_epochs": int((getattr(net, "meta", None) or {}).get("epochs", 0)) if args.init else 0,
            "init_train_s": float((getattr(net, "meta", None) or {}).get("train_s", 0.0)) if args.init else 0.0})
        log("training (network %d, seed %d): %.1f s, val rel-L2 u %.3e rho-1 %.3e" % (m, tseed + m, t_m, vu, vr))
        nets.append(net)
        hists.append(hist)
    for path in [p for p in (args.ensemble_with or "").split(",") if p]:
        other = FNO2d.load(path, device=dev)
        if list((other.meta or {}).get("held_out_re", [])) != data["re"][val].tolist():
            raise SystemExit("%s was not trained on this data set and held-out split" % path)
        vu, vr = evaluate(other, data, val, with_rho=True)
        log("ensemble member %s: val rel-L2 u %.3e rho-1 %.3e" % (path, vu, vr))
        nets.append(other)
    net = nets[0] if len(nets) == 1 else Ensemble(nets)
    if len(nets) > 1:
        vu, vr = evaluate(net, data, val, with_rho=True)
        log("ensemble of %d: val rel-L2 u %.3e rho-1 %.3e" % (len(nets), vu, vr))
    hist = hists[0]
    res = {"samples": args.samples, "n": args.n, "steady": int(len(ok)), "data_wall_s": data["wall"],
           "data_steps": data["steps"].tolist(), "data_re": data["re"].tolist(), "data_u": data["u"].tolist(),
           "held_out": val.tolist(), "train_s": t_train, "history": hist, "members": len(nets),
           "histories": hists}

    def dump():
        with open(os.path.join(args.out, "results.json"), "w") as f:
            json.dump(res, f, indent=1)

    dump()
    res["study"] = study(net, data["re"][val], data["u"][val], args.n, dev, log=log, max_steps=args.max_steps,
                         reference=data["fields"][torch.as_tensor(val, device=dev)])
    s = res["study"]
    log("study %d: cold %.1f s, warm %.1f s (inference %.3f s); steps cold %d warm %d (sums)" % (
        args.n, s["cold_wall_s"], s["warm_wall_s"], s["inference_s"], sum(s["cold_steps"]), sum(s["warm_steps"])))
    dump()
    sel = val[np.argsort(data["re"][val])]
    sel = sel[np.linspace(0, len(sel) - 1, min(args.single_cases, len(sel))).astype(int)]
    res["single"] = single_case_timing(net, data["re"][sel], data["u"][sel], args.n, dev, max_steps=args.max_steps)
    for row in res["single"]:
        log("single %d: Re %.1f u %.3f cold %d steps %.2f s, warm %d steps %.2f s" % (
            args.n, row["re"], row["u"], row["cold_steps"], row["cold_s"], row["warm_steps"], row["warm_s"]))
    dump()
    if args.study_large:
        # cost grows like side^3 / Re at fixed Re: the upsampled study keeps to Re <= 150
        low = val[data["re"][val] <= 150]
        low = low[np.argsort(data["re"][low])]
        sel = low[np.linspace(0, len(low) - 1, min(args.large_cases, len(low))).astype(int)] if len(low) else low
        res["study_large"] = study(net, data["re"][sel], data["u"][sel], args.study_large, dev, log=log,
                                   max_steps=1_500_000)
        s = res["study_large"]
        log("study %d: cold %.1f s, warm %.1f s; steps cold %s warm %s" % (
            args.study_large, s["cold_wall_s"], s["warm_wall_s"], s["cold_steps"], s["warm_steps"]))
    res["total_s"] = time.perf_counter() - t0
    dump()


if __name__ == "__main__":
    main()
