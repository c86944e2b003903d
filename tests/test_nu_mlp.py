"""The Nu network: oracle pinned by finite differences; CUDA forward, gradient and Adam
against the oracle; training reduces the loss."""
import re
from pathlib import Path

import numpy as np
import pytest

from oracle import mlp_oracle as MO

ROOT = Path(__file__).resolve().parents[1]


def _data(n, seed):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((n, MO.NIN)).astype(np.float32)
    t = (np.sin(x[:, 0]) + 0.5 * x[:, 1] * x[:, 2] - 0.3 * x[:, 3] ** 2).astype(np.float32)
    return x, t


def _params(seed):
    from axisem3d_gb300.nu_mlp import init_params
    return init_params(seed)


def test_param_layout_matches_header():
    h = (ROOT / "include" / "ax3d.h").read_text()
    assert int(re.search(r"#define AX3D_MLP_NPARAM (\d+)", h).group(1)) == MO.NPARAM == 35329
    from axisem3d_gb300 import nu_mlp
    assert nu_mlp.NPARAM == MO.NPARAM and nu_mlp.OFFSETS["b4"][0] == MO.NPARAM - 1


def test_bf16_rounding_nearest_even():
    v = np.array([1.0, 1 + 2 ** -8, 1 + 3 * 2 ** -8, -2.5 - 2 ** -7, 3.0e38])
    np.testing.assert_array_equal(MO.bf16(v)[:3], [1.0, 1.0, 1.015625])
    assert MO.bf16(v)[3] == -2.5  # -2.5078125 is the midpoint of -2.5 and -2.515625: even is -2.5
    assert np.isfinite(MO.bf16(v)[4])


def test_oracle_gradient_matches_finite_differences():
    x, t = _data(48, 1)
    p = _params(2).astype(np.float64)
    g, _ = MO.gradient(p, x, t, mirror=False)
    rng = np.random.default_rng(3)
    idx = np.concatenate([rng.choice(MO.NPARAM, 40, replace=False), [MO.NPARAM - 1, 0, 2048, 35200]])
    h = 1e-6
    for i in idx:
        d = np.zeros_like(p)
        d[i] = h
        lp = MO.gradient(p + d, x, t, mirror=False)[1]
        lm = MO.gradient(p - d, x, t, mirror=False)[1]
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])) + 1e-8, (i, fd, g[i])


def test_oracle_mirror_close_to_exact():
    x, t = _data(256, 4)
    p = _params(5)
    ge, _ = MO.gradient(p, x, t, mirror=False)
    gm, _ = MO.gradient(p, x, t, mirror=True)
    assert np.linalg.norm(gm - ge) <= 0.05 * np.linalg.norm(ge)


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))


@pytest.mark.gpu
def test_forward_matches_oracle(ax3d_lib):
    from axisem3d_gb300.nu_mlp import NuMLP
    x, _ = _data(1001, 6)   # a ragged last tile
    p = _params(7)
    net = NuMLP(max_batch=1024, params=p)
    y = net.forward(x).cpu().numpy()
    yo = MO.forward(p, x, mirror=True)
    assert rel(y, yo) <= 1e-3, rel(y, yo)


@pytest.mark.gpu
def test_gradient_matches_oracle_and_is_deterministic(ax3d_lib):
    """BF16 storage with FP32 sums vs the FP64 oracle applying the same BF16 roundings:
    relative L2 <= 5e-3 (rounding flips of single activations), loss <= 1e-4."""
    from axisem3d_gb300.nu_mlp import NuMLP
    x, t = _data(2000, 8)
    p = _params(9)
    net = NuMLP(max_batch=2048, params=p)
    g1, l1 = net.gradient(x, t)
    g2, _ = net.gradient(x, t)
    g1, g2 = g1.cpu().numpy(), g2.cpu().numpy()
    assert np.array_equal(g1, g2)
    go, lo = MO.gradient(p, x, t, mirror=True)
    assert rel(g1, go) <= 5e-3, rel(g1, go)
    assert abs(float(l1) - lo) <= 1e-4 * lo
    for name in ("W1", "W2", "W3", "w4", "b1", "b4"):
        from axisem3d_gb300.nu_mlp import OFFSETS
        o, n = OFFSETS[name]
        assert rel(g1[o:o + n], go[o:o + n]) <= 1e-2, name


@pytest.mark.gpu
def test_adam_steps_match_oracle(ax3d_lib):
    import torch
    from axisem3d_gb300.nu_mlp import NuMLP
    x, t = _data(1024, 10)
    p = _params(11)
    net = NuMLP(max_batch=1024, params=p)
    xd, td = torch.as_tensor(x).cuda(), torch.as_tensor(t).cuda()
    opt = MO.Adam(p)
    for _ in range(5):
        net.train_step(xd, td, 1e-3)
        g, _ = MO.gradient(opt.p, x, t, mirror=True)
        opt.step(g, 1e-3)
    pg = net.get_params().astype(np.float64)
    p0 = p.astype(np.float64)
    assert rel(pg - p0, opt.p - p0) <= 5e-2, rel(pg - p0, opt.p - p0)


@pytest.mark.gpu
def test_training_reduces_loss(ax3d_lib):
    from axisem3d_gb300.nu_mlp import NuMLP
    x, t = _data(16384, 12)
    net = NuMLP(max_batch=4096, seed=13)
    hist = net.fit(x, t, epochs=30, batch=1024, lr=3e-3, lr_final=3e-4)
    assert hist[-1] < 0.1 * hist[0], hist
    xv, tv = _data(4096, 14)
    yv = net.forward(xv).cpu().numpy()
    assert np.mean((yv - tv) ** 2) < 0.2 * np.var(tv)


@pytest.mark.gpu
def test_batch_above_max_is_rejected(ax3d_lib):
    from axisem3d_gb300.capi import Ax3dError
    from axisem3d_gb300.nu_mlp import NuMLP
    x, t = _data(200, 15)
    net = NuMLP(max_batch=128)
    with pytest.raises(Ax3dError) as ei:
        net.gradient(x, t)
    assert ei.value.code == 1


@pytest.mark.gpu
def test_learned_nu_gain_on_held_out_model(tmp_path, ax3d_lib, capsys):
    """What the trained network gains over the method without it.  The network is trained on
    the Nu wisdom labels of full-Nu runs (seeded Gaussian-random 3-D models) and predicts the
    Fourier order of every element of a model it has not seen.  Without the network the
    method runs that model at the full Nu (or pays a full-Nu run first to learn its wisdom);
    with it, the run at the predicted orders costs fewer GLL-point x azimuth updates per step
    and its seismograms stay within 1 % relative L2 of the full-Nu run's.  (The network is
    fitted on four models; two more calibrate the shift of its predictions.)"""
    from axisem3d_gb300 import nu_learn
    mesh = dict(n_theta=16, h_mantle=600e3, h_core=700e3, r_c=1500e3)
    s = nu_learn.experiment(tmp_path, n_train=6, n_val=2, n_test=1, nu_full=32, steps=375, epochs=200,
                            batch=512, mesh_kw=mesh, log=lambda m: None)
    t = s["tests"][0]
    with capsys.disabled():
        print(f"\nlearned Nu: misfit {t['misfit']:.4f}, updates/step {t['upd_full']} -> {t['upd_learned']}, "
              f"mean Nu {t['mean_nu_pred']:.1f} (labels {t['mean_nu_label']:.1f}), loss {s['loss_first']:.4g} -> "
              f"{s['loss_last']:.4g}, calibrated shift {s['shift']}")
    assert s["loss_last"] < 0.5 * s["loss_first"]
    assert t["misfit"] <= 0.01
    assert t["upd_learned"] < t["upd_full"]


@pytest.mark.gpu
def test_ring_features_gpu_match_host(ax3d_lib):
    """The band-power features sampled on the GPU (FP64 sampler) equal the host sampling
    (FP32 phases, FP64 sums) on the rings through the element centres of a seeded model."""
    from axisem3d_gb300 import model3d as M3D, nu_learn
    vs, vp = nu_learn.model_strings(1234)
    R = 6371e3
    models = [M3D.GaussianRandom(vs.split("$")[1:], R), M3D.GaussianRandom(vp.split("$")[1:], R)]
    rng = np.random.default_rng(3)
    E = 203  # not a multiple of the sampler's 25-point rows
    r = rng.uniform(3.5e6, R, E)
    th = rng.uniform(0.0, np.pi, E)
    s, z = r * np.sin(th), r * np.cos(th)
    host = nu_learn.ring_bands(models, s, z)
    gpu = nu_learn.ring_bands_gpu(models, s, z)
    fh = (np.log10(host + 1e-12) + 12.0) / 12.0
    fg = (np.log10(gpu + 1e-12) + 12.0) / 12.0
    assert np.abs(fg - fh).max() < 1e-4


def test_feature_pass_matches_build(tmp_path):
    """The learned route's feature pass (mesh, geometry, 1-D material only) gives the element
    features the full pre-loop gives, so the features need no pre-loop at any Nu."""
    from axisem3d_gb300 import nu_learn, solver
    d = nu_learn.write_case(tmp_path / "c", 5000, 16, 10, dict(n_theta=16, h_mantle=600e3, h_core=700e3,
                                                                r_c=1500e3))
    a = solver.Simulation(d)
    a.build()
    b = solver.Simulation(d)
    b.feature_pass()
    np.testing.assert_array_equal(nu_learn.element_features(b), nu_learn.element_features(a))
