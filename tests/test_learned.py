"""The learned form: network kernels against the FP64 CPU network, the feature
kernel against its FP64 restatement, tensor-core inference against the
training kernels' forward pass, and the pass itself against the FP64 path.

Stated tolerances of the learned form (SPRG_LEARNED), on the 64^3 jittered
box with the Gaussian-bump field, against the FP64 path (which equals the
oracle to 1e-10): size field relative error median <= 2e-3 and p99 <= 2e-2
(measured 1.4e-3 and 1.6e-2; the form's target of 1e-2 for the p99 is not
met: with exact sweeps the network's recovered values alone leave 1.65e-2
at 160^3, its prediction of the correction being good to about 7 % RMS),
mark agreement >= 99.5 %, and the network cuts the median error of the
method without it (the cheap least-squares gradient) by 10x or more.  The network's gradient kernels agree with the FP64 CPU network
(same BF16 rounding points) to 1e-3 relative.
"""
import numpy as np
import pytest

from oracle import learned_oracle as lo


def rand_batch(n, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    x = lo.bf16(rng.uniform(-1, 1, size=(n, lo.N_IN)))
    x[:, 3::4] = lo.bf16(rng.normal(0, 1, size=(n, lo.N_IN // 4)))
    y = rng.normal(0, 0.5, size=(n, lo.N_OUT))
    return x, y


def bf16_bits(x):
    return (np.asarray(x, np.float32).view(np.uint32) >> 16).astype(np.uint16)


def test_oracle_gradient_matches_finite_differences():
    from core_gb300 import learned
    p = learned.init_params(1).astype(np.float64)
    x, y = rand_batch(16, 2)
    g, _ = lo.grad(p, x, y, rounding=False)
    rng = np.random.Generator(np.random.PCG64(5))
    idx = np.concatenate([rng.integers(0, lo.N_PARAMS, 40), [lo.N_PARAMS - 1, lo.N_PARAMS - 4]])
    h = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (lo.mse(pp, x, y) - lo.mse(pm, x, y)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(g[i])


def test_parameter_layout():
    from core_gb300 import _lib, learned
    assert learned.N_PARAMS == lo.N_PARAMS == _lib.MLP_PARAMS
    p = learned.init_params(0)
    W1, b1, W2, b2, W3, b3 = learned.unpack(p)
    assert W1.shape == (64, 128) and W3.shape == (3, 64) and b3.shape == (3,)
    for a, b in zip(learned.unpack(p), lo.unpack(p)):
        assert np.array_equal(a, b)


def test_shipped_parameters():
    from core_gb300 import learned
    import os
    if not os.path.exists(learned.PARAMS_FILE):
        pytest.skip("no trained parameters shipped")
    p, meta = learned.load_params()
    assert p.size == lo.N_PARAMS and np.all(np.isfinite(p))
    assert meta.get("pairs", 0) > 0


# ---------------------------------------------------------------------------
@pytest.mark.gpu
def test_gradient_kernel_matches_cpu_network(gpu_lib):
    import torch
    from core_gb300 import learned
    p = learned.init_params(7)
    x, y = rand_batch(200, 8)  # not a multiple of the 64-sample block
    tr = learned.Trainer(p, 200)
    xb = torch.from_numpy(bf16_bits(x).view(np.int16)).cuda()
    yb = torch.from_numpy(y.astype(np.float32)).cuda()
    g = tr.gradient(xb, yb).cpu().numpy().astype(np.float64)
    loss = float(tr.loss.item())
    g_ref, loss_ref = lo.grad(p, x, y.astype(np.float32).astype(np.float64))
    scale = np.abs(g_ref).max()
    assert np.abs(g - g_ref).max() <= 1e-3 * scale
    assert abs(loss - loss_ref) <= 1e-4 * loss_ref


@pytest.mark.gpu
def test_forward_kernel_matches_cpu_network(gpu_lib):
    import torch
    from core_gb300 import learned
    p = learned.init_params(9)
    x, _ = rand_batch(300, 10)
    tr = learned.Trainer(p, 64)
    z = tr.forward(torch.from_numpy(bf16_bits(x).view(np.int16)).cuda()).cpu().numpy()
    z_ref = lo.forward(p, x)["Z3"]
    assert np.abs(z - z_ref).max() <= 1e-3 * (1 + np.abs(z_ref).max())


def small_case(n=10, seed=11):
    from core_gb300 import workload
    m = workload.box(n, jitter=0.2, seed=seed)
    u = workload.bump_field(m.coords, seed=seed)
    return m, u


@pytest.mark.gpu
def test_features_match_restatement(gpu_lib):
    import core_gb300 as cg
    from core_gb300 import learned
    m, u = small_case()
    with cg.Context(m, precision="fp32") as c:
        x_bits, aux = learned.features(c, u)
        listed = c.debug_read("listed", np.uint8, m.n_verts)
    x = lo.bf16_bits_to_f64(x_bits)
    x_ref, aux_ref = lo.features(m.coords, u, m.edge_verts, listed != 0)
    ok = aux_ref[:, 4] == 0
    assert np.array_equal(aux[:, 4] != 0, aux_ref[:, 4] != 0)
    xr = lo.bf16(x_ref)
    # one BF16 unit at the rounding boundaries (FP32 vs FP64 residuals)
    tol = 2.0 ** -7 * np.abs(xr) + 1e-6
    frac_off = np.mean(np.abs(x[ok] - xr[ok]) > tol[ok])
    assert frac_off < 1e-3
    g, g_ref = aux[ok, :3], aux_ref[ok, :3]
    assert np.abs(g - g_ref).max() <= 1e-4 * np.abs(g_ref).max()
    assert np.allclose(aux[ok, 3], aux_ref[ok, 3], rtol=1e-3)


@pytest.mark.gpu
def test_tensor_core_inference_matches_forward_kernel(gpu_lib):
    import torch
    import core_gb300 as cg
    from core_gb300 import learned
    m, u = small_case(12, 13)
    p = learned.init_params(21)
    with cg.Context(m, precision="fp32") as c:
        x_bits, aux = learned.features(c, u)
    with cg.Context(m, precision="fp32") as c:
        c.set_mlp_params(p)
        c.set_precision("learned")
        c.set_learned_options(True, 1e30)  # no output guard: every unflagged vertex answered by the network
        c.estimate_and_mark(u, 0.004)
        rec = c.debug_read("rec16", np.float32, 8 * m.n_verts).reshape(-1, 8)[:, 4:7].astype(np.float64)
    tr = learned.Trainer(p, 64)
    z = tr.forward(torch.from_numpy(x_bits.view(np.int16)).cuda()).cpu().numpy().astype(np.float64)
    ok = aux[:, 4] == 0
    want = aux[ok, :3] + z[ok] * aux[ok, 3:4]
    corr = np.abs(z[ok] * aux[ok, 3:4]).max()
    assert corr > 0
    assert np.abs(rec[ok] - want).max() <= 2e-2 * corr + 1e-6 * np.abs(want).max()


def learned_vs_fp64(n, use_mlp=True, seed=4):
    import core_gb300 as cg
    from core_gb300 import workload
    m = workload.box(n, jitter=0.2, seed=seed)
    u = workload.bump_field(m.coords, seed=seed)
    ratio = 0.008 * n / 160
    with cg.Context(m, precision="fp64") as c:
        s64, f64, *_ = c.estimate_and_mark(u, ratio)
    with cg.Context(m, precision="learned") as c:
        c.set_learned_options(use_mlp, 8.0)
        sl, fl, _, _, info = c.estimate_and_mark(u, ratio)
    fin = np.isfinite(s64) & np.isfinite(sl)
    rel = np.abs(sl[fin] - s64[fin]) / s64[fin]
    return rel, float(np.mean(fl == f64)), info


@pytest.mark.gpu
def test_learned_pass_accuracy_and_ablation(gpu_lib):
    from core_gb300 import learned
    import os
    if not os.path.exists(learned.PARAMS_FILE):
        pytest.skip("no trained parameters shipped")
    rel, agree, info = learned_vs_fp64(64)
    assert np.median(rel) <= 2e-3
    assert np.percentile(rel, 99) <= 2e-2
    assert agree >= 0.995
    assert info["n_learned_fallback"] < 0.05 * 65 ** 3
    # the method without the network (the cheap gradient alone) is far worse
    rel0, agree0, _ = learned_vs_fp64(64, use_mlp=False)
    assert np.median(rel0) >= 10 * np.median(rel)
    assert agree0 < agree
