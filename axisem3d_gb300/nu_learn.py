"""Learned Fourier order: element features, wisdom labels, GPU training of the Nu network,
and the learned-Nu vs full-Nu experiment.

The reference learns a point-wise Nu field ("wisdom") from the spectra of a full-Nu run
and reuses it in later runs of the same model (SolidPoint.cpp:240-272, NuWisdom.cpp:19-86).
Here a network trained on the wisdom of full-Nu runs of many seeded 3-D models predicts
each element's Nu from local model features for a model it has not seen, so the reduced
run needs no full-Nu run first; a full-Nu run remains the accuracy reference and the fallback.

Features (16 per element, at the element's centre GLL point):
  0 r / R            1 epicentral distance / pi     2 distance to the axis s / R
  3 period / 100 s   4 element size / 100 km        5 Vp / 10 km/s     6 Vs / 10 km/s
  7 source depth / 1000 km
  8-15 azimuthal power of the local dlnVs perturbation on the ring through the centre,
       orders [1,2), [2,4), ..., [128,256), as (log10(P + 1e-12) + 12) / 12
Target: log2(1 + Nu) / log2(1 + Nu_full), Nu = max wisdom Nu over the element's points.
"""
from __future__ import annotations

import json
import math
import time
from pathlib import Path

import numpy as np

from . import solver

NFEAT = 16


def model_strings(seed: int, rms: float = 0.04, lat_km: float = 500.0, rad_km: float = 200.0):
    """Seeded Gaussian-random dlnVs and dlnVp fields (independent seeds), as list entries."""
    return (f"gaussian_random$VS$Ref1D${rms}${lat_km}${rad_km}${seed}",
            f"gaussian_random$VP$Ref1D${rms}${lat_km}${rad_km}${seed + 7919}")


# TIME_DELTA_T_FACTOR of the experiment's runs: with the 3-D models, runs on the default half
# disk at the mesh's CFL step grow unstable once the P wave reaches the core-mantle boundary
# beneath the source; 0.8 of it is stable (full-Nu and learned-Nu runs use the same step)
DT_FACTOR = 0.8


def write_case(d, seed, nu_full, steps, mesh_kw=None, n_stations=20, dt_factor=DT_FACTOR):
    d = solver.write_inputs(d, mesh_kw=mesh_kw, nu=nu_full, steps=steps, n_stations=n_stations, seed=0,
                            models3d=model_strings(seed), lucky=True)
    if dt_factor != 1.0:
        p = Path(d) / "inparam.time_src_recv"
        p.write_text(p.read_text().replace("TIME_DELTA_T_FACTOR 1.0", f"TIME_DELTA_T_FACTOR {dt_factor}"))
    return d


def ring_bands(models, s, z, nphi=512):
    """Band powers (8 octaves of orders 1..255) of the summed dlnVs of `models` on the ring
    of radius s at height z, per element; (E, 8)."""
    E = len(s)
    out = np.zeros((E, 8))
    phi = 2 * np.pi * np.arange(nphi) / nphi
    vs_models = [m for m in models if m.prop == "VS" and m.ref != 0]
    if not vs_models:
        return out
    step = 256
    for a in range(0, E, step):
        b = min(E, a + step)
        xyz = np.stack([s[a:b, None] * np.cos(phi), s[a:b, None] * np.sin(phi),
                        np.broadcast_to(z[a:b, None], (b - a, nphi))], -1)
        d = np.zeros((b - a, nphi))
        for m in vs_models:
            val, inr = m.evaluate(xyz)
            d += np.where(inr, val, 0.0)
        out[a:b] = _band_powers(d)
    return out


def _band_powers(d):
    """Band powers (8 octaves of orders 1..255) of rows of azimuthal samples d (E, nphi)."""
    P = np.abs(np.fft.rfft(d, axis=1) / d.shape[1]) ** 2
    return np.stack([P[:, 2 ** i:2 ** (i + 1)].sum(1) for i in range(8)], 1)


def ring_bands_gpu(models, s, z, nphi=512, device=0):
    """ring_bands with the rings sampled on the GPU (GaussianRandom.evaluate_rings_gpu,
    FP64): the element centres are packed 25 to a row of the sampler's (n, 25) layout."""
    E = len(s)
    vs_models = [m for m in models if m.prop == "VS" and m.ref != 0]
    if not vs_models or E == 0:
        return np.zeros((E, 8))
    n = (E + 24) // 25
    crd = np.zeros((n * 25, 2))
    crd[:E, 0], crd[:E, 1] = s, z
    crd = crd.reshape(n, 25, 2)
    d = np.zeros((E, nphi))
    for m in vs_models:
        if not hasattr(m, "evaluate_rings_gpu"):
            return ring_bands(models, s, z, nphi)
        d += m.evaluate_rings_gpu(crd, nphi, device=device).transpose(0, 2, 1).reshape(n * 25, nphi)[:E]
    return _band_powers(d)


def element_features(sim, period: float = 50.0, gpu: bool = False) -> np.ndarray:
    """The 16 features of every element; gpu samples the rings of the 3-D model on the GPU."""
    c = sim.crds[:, 12]
    s, z = c[:, 0], c[:, 1]
    r = np.hypot(s, z)
    size = np.hypot(*(sim.crds[:, 24] - sim.crds[:, 0]).T) / np.sqrt(2.0)
    f = np.zeros((len(s), NFEAT), np.float32)
    f[:, 0] = r / sim.R
    f[:, 1] = np.arctan2(s, z) / np.pi
    f[:, 2] = s / sim.R
    f[:, 3] = period / 100.0
    f[:, 4] = size / 100e3
    f[:, 5] = sim.vp_e / 1e4
    f[:, 6] = sim.vs_e / 1e4
    f[:, 7] = sim.src_dep / 1e6
    bands = ring_bands_gpu(sim.models, s, z) if gpu else ring_bands(sim.models, s, z)
    f[:, 8:] = (np.log10(bands + 1e-12) + 12.0) / 12.0
    return f


def element_labels(spec, wisdom) -> np.ndarray:
    return np.asarray(wisdom)[spec.e_pts].max(1)


def encode(nu, nu_full):
    return (np.log2(1.0 + np.asarray(nu, np.float64)) / math.log2(1.0 + nu_full)).astype(np.float32)


def decode(y, nu_full, shift=0.0):
    """Nu from the network output, raised by `shift` in the encoded (log2(1 + Nu)) space."""
    nu = (1.0 + nu_full) ** (np.asarray(y, np.float64) + shift) - 1.0
    return np.clip(np.ceil(nu), 1, nu_full).astype(np.int64)


SHIFTS = (0.0, 0.05, 0.1, 0.15, 0.2, 0.3, 0.45, 0.7)


def calibrate_shift(vals, net, nu_full, steps, target, log=print, preloop="gpu"):
    """The smallest encoded-space shift of the predictions whose runs reproduce every
    validation model's full-Nu seismograms within `target` relative L2 (calibration by
    simulation on models the network was not fitted on); vals = [(sim, features, full-Nu
    seismograms, clock of the full-Nu run)].  Returns (shift, largest validation misfit);
    (1.0, 0.0), i.e. full Nu,
    if no shift qualifies."""
    ys = [net.forward(x).cpu().numpy() for _, x, _, _ in vals]
    for sh in SHIFTS:
        worst = 0.0
        for (sim, _, seis_full, clk), y in zip(vals, ys):
            spec = sim.build(nu_elem=decode(y, nu_full, sh), preloop=preloop)
            seis, _, _, upd = run(spec, steps, clk=clk, schedule=LEARNED_SCHEDULE)
            mis = float(np.linalg.norm(seis - seis_full) / np.linalg.norm(seis_full))
            log(f"calibration shift {sh:.2f}: misfit {mis:.4g}, updates/step {upd}")
            worst = max(worst, mis)
            if worst > target:
                break
        if worst <= target:
            return sh, worst
    return 1.0, 0.0


def clock(spec):
    """A run's time step and source time function, to impose on another run of the same model."""
    return float(spec.dt), np.array(spec.stf, copy=True)


# The bucket schedule ax3d_autotune picks on learned-Nu domains (the shortest rings on
# 64-thread CTAs eight per SM, three side streams, merged launches: element pass 5.74 ms
# against 6.04 ms for the library default on the 16 held-out learned models joined), pinned
# for the learned runs so that none pays for trials; full-Nu runs keep the library default.
LEARNED_SCHEDULE = (1.12, 4, 3, True)


def run(spec, steps, learn=None, clk=None, schedule=None):
    """Loop time of one GPU run (first step to seismograms on the host; the pre-loop and
    any network inference are timed by the caller and added for time-to-seismogram).
    learn = (interval, epsilon) turns the wisdom learner on.  clk = clock(other spec) runs
    on that run's time step: the step of Quad::getDeltaT follows the largest velocity on
    each element's Nr slices, so runs of one model at different Nu fields differ in dt by
    up to ~1 %, and seismograms are compared sample by sample on one time axis (the
    full-Nu run's).  schedule: (ratio, policy, side streams, merge) for ax3d_set_schedule,
    else the library default.  Returns (seis, seconds, wisdom or None, unique-point updates
    per step)."""
    import torch
    from .capi import Ax3dDomain
    if clk is not None:
        spec.dt, spec.stf = clk[0], clk[1].copy()
    dom = Ax3dDomain(spec)
    if schedule is not None:
        dom.set_schedule(*schedule)
    if learn:
        dom.set_wisdom_learning(int(learn[0]), float(learn[1]))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    dom.step(steps)
    seis = dom.seismograms(0, steps)
    t = time.perf_counter() - t0
    wis = dom.get_wisdom() if learn else None
    dom.close()
    return seis, t, wis, int(np.asarray(spec.p_nr, np.int64).sum())


def held_out(net, shift, work, n_test=16, nu_full=64, steps=600, eps=1e-3, interval=5, mesh_kw=None, out=None,
             log=print, preloop="gpu", seed0=5000):
    """The network against the plain full-Nu solver on n_test held-out seeded models (seeds
    seed0, seed0 + 1, ...): per model the full-Nu route (pre-loop, loop), the learned route
    from the input files alone (feature pass, features, inference, pre-loop at the predicted
    Nu, loop) and the wisdom route (the model's own full-Nu wisdom reused); then all learned
    models batched into one domain.  Returns the per-model records and the batched figures."""
    work = Path(work)
    if out:
        Path(out).mkdir(parents=True, exist_ok=True)
    tests = []
    seis_l_all, specs_l, pre_l_all = [], [], []
    for i in range(n_test):
        d = write_case(work / f"test{i}", seed0 + i, nu_full, steps, mesh_kw)
        # plain full-Nu route: pre-loop, then the loop
        t0 = time.perf_counter()
        sim = solver.Simulation(d)
        spec_f = sim.build(preloop=preloop)
        pre_f = time.perf_counter() - t0
        seis_f, t_f, _, upd_f = run(spec_f, steps)
        _, t_fl, wis, _ = run(spec_f, steps, learn=(interval, eps))
        # learned route, from the input files alone: the feature pass (mesh, geometry, 1-D
        # material), the features, network inference, the pre-loop at the predicted Nu, the loop
        t0 = time.perf_counter()
        sim_l = solver.Simulation(d)
        sim_l.feature_pass(preloop=preloop)
        x = element_features(sim_l, gpu=preloop == "gpu")
        t_feat = time.perf_counter() - t0
        import torch
        t0 = time.perf_counter()
        y = net.forward(x).cpu().numpy()
        torch.cuda.synchronize()
        t_inf = time.perf_counter() - t0
        nu_e = decode(y, nu_full, shift)
        t0 = time.perf_counter()
        spec_l = sim_l.build(nu_elem=nu_e, preloop=preloop)
        pre_l = time.perf_counter() - t0
        seis_l, t_l, _, upd_l = run(spec_l, steps, clk=clock(spec_f), schedule=LEARNED_SCHEDULE)
        mis = float(np.linalg.norm(seis_l - seis_f) / np.linalg.norm(seis_f))
        # the reference's route without a network: reuse the wisdom of this model's own
        # full run (which must be paid first)
        spec_w = sim.build(nu_elem=np.maximum(element_labels(spec_f, wis), 1), preloop=preloop)
        seis_w, t_w, _, upd_w = run(spec_w, steps, clk=clock(spec_f), schedule=LEARNED_SCHEDULE)
        mis_w = float(np.linalg.norm(seis_w - seis_f) / np.linalg.norm(seis_f))
        tts_f = pre_f + t_f
        tts_l = t_feat + t_inf + pre_l + t_l
        tests.append(dict(seed=seed0 + i, misfit=mis, t_full=t_f, t_full_learning=t_fl, t_learned=t_l,
                          speedup=t_f / t_l, preloop_full=pre_f, preloop_learned=pre_l, features=t_feat,
                          inference=t_inf, tts_full=tts_f, tts_learned=tts_l, tts_speedup=tts_f / tts_l,
                          upd_full=upd_f, upd_learned=upd_l, misfit_wisdom=mis_w, t_wisdom=t_w,
                          mean_nu_pred=float(nu_e.mean()), mean_nu_label=float(element_labels(spec_f, wis).mean())))
        del spec_f, spec_w
        specs_l.append(spec_l)
        seis_l_all.append(seis_l)
        pre_l_all.append(t_feat + t_inf + pre_l)
        log(f"test {i}: misfit {mis:.4f} (wisdom {mis_w:.4f}), full {tts_f:.2f} s (loop {t_f:.2f}), "
            f"learned {tts_l:.2f} s (loop {t_l:.2f}), updates {upd_f} -> {upd_l}")
        if out:
            (Path(out) / "tests_partial.json").write_text(json.dumps(tests, indent=1))
    # all held-out learned-Nu runs batched into one domain
    from . import ensemble
    # one time axis for the batch (the members share it when their full-Nu runs do)
    clk_b = min((clock(sp) for sp in specs_l), key=lambda c: c[0])
    pinned = any(abs(sp.dt - clk_b[0]) > 1e-12 * clk_b[0] for sp in specs_l)
    for sp in specs_l:
        sp.dt, sp.stf = clk_b[0], clk_b[1].copy()
    big, info = ensemble.concat(specs_l)
    seis_b, t_b, _, upd_b = run(big, steps, schedule=LEARNED_SCHEDULE)
    parts = ensemble.split_seismograms(seis_b, info)
    mis_b = max(float(np.linalg.norm(p - s) / np.linalg.norm(s)) for p, s in zip(parts, seis_l_all))
    t_full_sum = sum(t["t_full"] for t in tests)
    tts_full_sum = sum(t["tts_full"] for t in tests)
    tts_batched = sum(pre_l_all) + t_b  # every learned model's features, inference, pre-loop + one batched loop
    return tests, dict(
        elements=int(len(specs_l[0].e_pts)), misfit_max=max(t["misfit"] for t in tests),
        misfit_mean=float(np.mean([t["misfit"] for t in tests])),
        speedup_mean=float(np.mean([t["speedup"] for t in tests])),
        tts_speedup_mean=float(np.mean([t["tts_speedup"] for t in tests])),
        batched_seconds=t_b, batched_vs_sequential_full=t_full_sum / t_b,
        tts_batched_learned_seconds=tts_batched, tts_sequential_full_seconds=tts_full_sum,
        tts_learned_batched_vs_sequential_full=tts_full_sum / tts_batched,
        batched_vs_sequential_learned=sum(t["t_learned"] for t in tests) / t_b,
        batched_split_misfit_max=mis_b, batched_dt_pinned=pinned)


def experiment(work, n_train=64, n_test=16, nu_full=64, steps=600, epochs=200, batch=4096, lr=2e-3,
               eps=1e-3, interval=5, mesh_kw=None, out=None, log=print, target=0.005, preloop="gpu", n_val=1):
    """Train on the wisdom of n_train - n_val full-Nu runs, calibrate the prediction shift on
    the last n_val training models by simulation (misfit <= target, half the 1 % bar),
    evaluate on n_test held-out models.  Every pre-loop runs on the GPU unless preloop =
    "host".  Returns the summary dict (also written to out/summary.json with the parameters
    in out/nu_mlp.npz)."""
    from .nu_mlp import NuMLP
    work = Path(work)
    X, Y, pre = [], [], []
    t_train_runs = 0.0
    vals = []
    for i in range(n_train):
        d = write_case(work / f"train{i}", 1000 + i, nu_full, steps, mesh_kw)
        t0 = time.perf_counter()
        sim = solver.Simulation(d)
        spec = sim.build(preloop=preloop)
        pre.append(time.perf_counter() - t0)
        seis, t, wis, _ = run(spec, steps, learn=(interval, eps))
        t_train_runs += t
        x = element_features(sim, gpu=preloop == "gpu")
        y = encode(np.minimum(element_labels(spec, wis), nu_full), nu_full)
        log(f"train {i}: {t:.2f} s, mean label Nu {np.mean(element_labels(spec, wis)):.1f}")
        if i >= n_train - n_val and n_train > n_val:
            vals.append((sim, x, seis, clock(spec)))  # held out of the fit: calibrates the shift
        else:
            X.append(x)
            Y.append(y)
            del sim
        del spec
        if out:
            Path(out).mkdir(parents=True, exist_ok=True)
            np.savez(Path(out) / "train_data.npz", X=np.concatenate(X), Y=np.concatenate(Y))
    X, Y = np.concatenate(X), np.concatenate(Y)
    net = NuMLP(max_batch=batch, seed=0)
    t0 = time.perf_counter()
    hist = net.fit(X, Y, epochs=epochs, batch=batch, lr=lr, lr_final=lr * 0.05)
    t_fit = time.perf_counter() - t0
    log(f"fit {t_fit:.1f} s, loss {hist[0]:.4g} -> {hist[-1]:.4g}")
    shift, val_misfit = 0.0, None
    if vals:
        shift, val_misfit = calibrate_shift(vals, net, nu_full=nu_full, steps=steps, target=target, log=log,
                                            preloop=preloop)
    tests, res = held_out(net, shift, work, n_test=n_test, nu_full=nu_full, steps=steps, eps=eps, interval=interval,
                          mesh_kw=mesh_kw, out=out, log=log, preloop=preloop)
    summary = dict(
        n_train=n_train, n_test=n_test, nu_full=nu_full, steps=steps,
        epochs=epochs, batch=batch, fit_seconds=t_fit, train_runs_seconds=t_train_runs,
        preloop_seconds_mean=float(np.mean(pre)) if pre else None, loss_first=float(hist[0]), loss_last=float(hist[-1]),
        shift=shift, validation_misfit=val_misfit, target=target, tests=tests, **res)
    if out:
        out = Path(out)
        out.mkdir(parents=True, exist_ok=True)
        (out / "summary.json").write_text(json.dumps(summary, indent=1))
        np.savez(out / "nu_mlp.npz", params=net.get_params(), nu_full=nu_full, shift=shift)
    net.close()
    return summary


def evaluate(params_file, work, n_test=16, steps=600, mesh_kw=None, out=None, log=print, preloop="gpu"):
    """The held-out comparison of a trained network saved by `experiment` (out/nu_mlp.npz:
    parameters, Nu_full, calibrated shift), without training again."""
    from .nu_mlp import NuMLP
    d = np.load(params_file)
    nu_full, shift = int(d["nu_full"]), float(d["shift"])
    net = NuMLP(max_batch=4096, params=d["params"])
    tests, res = held_out(net, shift, work, n_test=n_test, nu_full=nu_full, steps=steps, mesh_kw=mesh_kw,
                          out=out, log=log, preloop=preloop)
    net.close()
    summary = dict(params=str(params_file), n_test=n_test, nu_full=nu_full, steps=steps, shift=shift,
                   tests=tests, **res)
    if out:
        out = Path(out)
        out.mkdir(parents=True, exist_ok=True)
        (out / "summary_eval.json").write_text(json.dumps(summary, indent=1))
    return summary


def compare_schedules(params_file, work, n_test=16, steps=1500, log=print):
    """Loop seconds of the n_test held-out learned-Nu models joined into one domain, and of
    the first model's full-Nu run, under the library's default bucket schedule and under
    LEARNED_SCHEDULE, twice each in turn; the seismograms of the two schedules must agree."""
    from . import ensemble
    from .nu_mlp import NuMLP
    d = np.load(params_file)
    nu_full, shift = int(d["nu_full"]), float(d["shift"])
    net = NuMLP(max_batch=4096, params=d["params"])
    specs, full = [], None
    for i in range(n_test):
        case = write_case(Path(work) / f"test{i}", 5000 + i, nu_full, steps)
        if i == 0:
            full = solver.Simulation(case).build(preloop="gpu")
        sim = solver.Simulation(case)
        sim.feature_pass(preloop="gpu")
        y = net.forward(element_features(sim, gpu=True)).cpu().numpy()
        specs.append(sim.build(nu_elem=decode(y, nu_full, shift), preloop="gpu"))
    net.close()
    clk = min((clock(sp) for sp in specs), key=lambda c: c[0])
    for sp in specs:
        sp.dt, sp.stf = clk[0], clk[1].copy()
    big, _ = ensemble.concat(specs)
    out, seis = {}, {}
    for label, spec in (("batched", big), ("full", full)):
        for _ in range(2):
            for name, sch in (("default", None), ("learned", LEARNED_SCHEDULE)):
                s_, t, _, _ = run(spec, steps, schedule=sch)
                out.setdefault(f"{label}_{name}", []).append(t)
                seis[(label, name)] = s_
                log(f"{label} {name} schedule: {t:.3f} s")
        out[f"{label}_max_diff"] = float(np.abs(seis[(label, "default")] - seis[(label, "learned")]).max())
    return out


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser(description="learned-Nu experiment")
    ap.add_argument("--work", default="/tmp/ax3d_nu_learn")
    ap.add_argument("--out", default="nu_learn_out")
    ap.add_argument("--train", type=int, default=64)
    ap.add_argument("--test", type=int, default=16)
    ap.add_argument("--nu", type=int, default=256)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--epochs", type=int, default=200)
    ap.add_argument("--eps", type=float, default=1e-3)
    ap.add_argument("--val", type=int, default=1, help="training models that calibrate instead of fitting")
    ap.add_argument("--params", default="", help="evaluate this saved network on the held-out models, no training")
    ap.add_argument("--schedules", action="store_true",
                    help="with --params: loop times under the default and the learned-domain schedule")
    a = ap.parse_args()
    if a.params and a.schedules:
        print(json.dumps(compare_schedules(a.params, a.work, a.test, a.steps, log=lambda m: print(m, flush=True))))
        raise SystemExit(0)
    if a.params:
        s = evaluate(a.params, a.work, a.test, a.steps, out=a.out, log=lambda m: print(m, flush=True))
    else:
        s = experiment(a.work, a.train, a.test, a.nu, a.steps, a.epochs, eps=a.eps, out=a.out,
                       log=lambda m: print(m, flush=True), n_val=a.val)
    print(json.dumps({k: v for k, v in s.items() if k != "tests"}))
