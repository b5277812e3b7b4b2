"""Learned form: network parameters, training pairs and the training loop.

The network (``csrc/sprg_learned.cu``) predicts the correction from a cheap
least-squares vertex gradient g_c to the SPR recovered gradient eps*:
eps*(v) = g_c + z * s_v / r_v.  Its training pairs come from the method
itself: on config-3-style meshes (unit boxes of n^3 cells, n log-uniform in
[4, 40]; fields of 1-8 Gaussian bumps, widths U[0.02, 0.3], amplitudes
N(0, 1); interior vertices jittered by U(-0.2h, 0.2h) so the network sees the
geometry of the jittered evaluation box) the FP64 path gives eps*, the
library's feature kernel gives the inputs x and (g_c, s_v / r_v), and the
target is z* = (eps* - g_c) / (s_v / r_v).

Training runs on the GPU through the library's own kernels: the fused
forward/backward (``sprg_mlp_grad``, BF16 weights and activations, FP32
accumulation) and Adam (``sprg_mlp_adam``).  torch supplies device memory,
the stream and the minibatch permutation only.

    python -m core_gb300.learned --boxes 192 --steps 6000   # writes spr_mlp.npz
"""
import argparse
import ctypes
import json
import os
import time

import numpy as np

from . import _lib

HERE = os.path.dirname(os.path.abspath(__file__))
PARAMS_FILE = os.path.join(HERE, "spr_mlp.npz")
N_PARAMS = _lib.MLP_PARAMS
N_IN, N_HID, N_OUT = _lib.MLP_INPUTS, 64, 3
# offsets of W1 [64][128], b1, W2 [64][64], b2, W3 [3][64], b3
OFF = {"W1": 0, "b1": N_HID * N_IN}
OFF["W2"] = OFF["b1"] + N_HID
OFF["b2"] = OFF["W2"] + N_HID * N_HID
OFF["W3"] = OFF["b2"] + N_HID
OFF["b3"] = OFF["W3"] + N_OUT * N_HID
assert OFF["b3"] + N_OUT == N_PARAMS


def unpack(p):
    """Views of the parameter vector as (W1, b1, W2, b2, W3, b3)."""
    p = np.asarray(p)
    return (p[OFF["W1"]:OFF["b1"]].reshape(N_HID, N_IN), p[OFF["b1"]:OFF["W2"]],
            p[OFF["W2"]:OFF["b2"]].reshape(N_HID, N_HID), p[OFF["b2"]:OFF["W3"]],
            p[OFF["W3"]:OFF["b3"]].reshape(N_OUT, N_HID), p[OFF["b3"]:])


def init_params(seed=0):
    """Glorot-uniform weights, zero biases (FP32)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    p = np.zeros(N_PARAMS, np.float32)
    for name, (fo, fi) in (("W1", (N_HID, N_IN)), ("W2", (N_HID, N_HID)), ("W3", (N_OUT, N_HID))):
        a = np.sqrt(6.0 / (fi + fo))
        p[OFF[name]:OFF[name] + fo * fi] = rng.uniform(-a, a, fo * fi)
    return p


def save_params(p, path=PARAMS_FILE, meta=None):
    np.savez(path, params=np.asarray(p, np.float32), meta=json.dumps(meta or {}))


def load_params(path=PARAMS_FILE):
    with np.load(path) as z:
        p = z["params"].astype(np.float32)
        meta = json.loads(str(z["meta"])) if "meta" in z else {}
    if p.size != N_PARAMS:
        raise ValueError(f"{path}: {p.size} parameters, expected {N_PARAMS}")
    return p, meta


def default_params():
    """The trained parameters shipped with the package."""
    if not os.path.exists(PARAMS_FILE):
        raise FileNotFoundError(f"{PARAMS_FILE} is missing: train with `python -m core_gb300.learned`")
    return load_params()[0]


# ---------------------------------------------------------------------------
# training pairs
# ---------------------------------------------------------------------------
def box_sizes(n_boxes, seed, lo=4, hi=40):
    rng = np.random.Generator(np.random.PCG64(seed))
    return np.rint(np.exp(rng.uniform(np.log(lo), np.log(hi), n_boxes))).astype(int)


def features(ctx, u):
    """(x [V][128] uint16 BF16 bits, aux [V][5]) of field u through the library."""
    import torch
    V = ctx.mesh.n_verts
    d_u = torch.from_numpy(np.ascontiguousarray(u, np.float64)).cuda()
    d_x = torch.empty(V * N_IN, dtype=torch.int16, device="cuda")
    d_aux = torch.empty(V * _lib.MLP_AUX, dtype=torch.float32, device="cuda")
    ctx.set_stream(torch.cuda.current_stream().cuda_stream)
    ctx.learned_features(d_u.data_ptr(), d_x.data_ptr(), d_aux.data_ptr())
    torch.cuda.synchronize()
    return (d_x.cpu().numpy().view(np.uint16).reshape(V, N_IN),
            d_aux.cpu().numpy().reshape(V, _lib.MLP_AUX))


def training_pairs(n_boxes, seed=3, jitter=0.2, max_vertices=2_000_000):
    """Inputs and targets from the FP64 path on config-3-style boxes."""
    from . import workload
    from .api import Context
    xs, ys = [], []
    total = 0
    for i, n in enumerate(box_sizes(n_boxes, seed)):
        m = workload.box(int(n), jitter=jitter, seed=seed * 100_003 + i)
        u = workload.batched_field(m.coords, seed * 100_003 + i)
        with Context(m, precision="fp64") as c:
            eps = c.recoverField(c.getGradIPField(u))
        with Context(m, precision="fp32") as c:
            x, aux = features(c, u)
        keep = (aux[:, 4] == 0) & (aux[:, 3] > 0)
        z = (eps[keep] - aux[keep, :3]) / aux[keep, 3:4]
        xs.append(x[keep])
        ys.append(z.astype(np.float32))
        total += int(keep.sum())
        if total >= max_vertices:
            break
    return np.concatenate(xs), np.concatenate(ys)


# ---------------------------------------------------------------------------
# training on the GPU with the library's kernels
# ---------------------------------------------------------------------------
class Trainer:
    def __init__(self, params, batch):
        import torch
        self.torch = torch
        self.lib = _lib.load()
        self.batch = batch
        self.P = torch.from_numpy(np.asarray(params, np.float32).copy()).cuda()
        self.m1 = torch.zeros_like(self.P)
        self.m2 = torch.zeros_like(self.P)
        self.grad = torch.zeros_like(self.P)
        self.loss = torch.zeros(1, dtype=torch.float32, device="cuda")
        self.scratch = torch.empty(int(self.lib.sprg_mlp_scratch_bytes(batch)), dtype=torch.uint8, device="cuda")
        self.step_no = 0

    def stream(self):
        return ctypes.c_void_p(self.torch.cuda.current_stream().cuda_stream)

    def gradient(self, xb, yb):
        n = xb.shape[0]
        _lib.check(self.lib.sprg_mlp_grad(self.P.data_ptr(), xb.data_ptr(), yb.data_ptr(), n, self.grad.data_ptr(),
                                          self.loss.data_ptr(), self.scratch.data_ptr(), self.stream()), None)
        return self.grad

    def step(self, xb, yb, lr):
        self.gradient(xb, yb)
        self.step_no += 1
        _lib.check(self.lib.sprg_mlp_adam(self.P.data_ptr(), self.m1.data_ptr(), self.m2.data_ptr(),
                                          self.grad.data_ptr(), lr, 0.9, 0.999, 1e-8, self.step_no, self.stream()),
                   None)

    def forward(self, x):
        torch = self.torch
        n = x.shape[0]
        out = torch.empty(n * N_OUT, dtype=torch.float32, device="cuda")
        scratch = torch.empty(int(self.lib.sprg_mlp_scratch_bytes(n)), dtype=torch.uint8, device="cuda")
        _lib.check(self.lib.sprg_mlp_forward(self.P.data_ptr(), x.data_ptr(), n, out.data_ptr(), scratch.data_ptr(),
                                             self.stream()), None)
        return out.view(n, N_OUT)

    def params(self):
        return self.P.cpu().numpy().copy()


def train(x, y, steps=6000, batch=8192, lr=2e-3, seed=0, params=None, log_every=500):
    """Adam with cosine decay; returns (params, history)."""
    import torch
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    X = torch.from_numpy(np.ascontiguousarray(x).view(np.int16)).cuda()
    Y = torch.from_numpy(np.ascontiguousarray(y, np.float32)).cuda()
    n = X.shape[0]
    tr = Trainer(init_params(seed) if params is None else params, batch)
    hist = []
    perm = torch.randperm(n, device="cuda", generator=g)
    pos = 0
    t0 = time.time()
    for s in range(1, steps + 1):
        if pos + batch > n:
            perm = torch.randperm(n, device="cuda", generator=g)
            pos = 0
        idx = perm[pos:pos + batch]
        pos += batch
        xb, yb = X[idx].contiguous(), Y[idx].contiguous()
        rate = lr * 0.5 * (1 + np.cos(np.pi * (s - 1) / steps))
        tr.step(xb, yb, float(rate))
        if s % log_every == 0 or s == steps:
            hist.append({"step": s, "mse": float(tr.loss.item()) / (3 * xb.shape[0]), "s": round(time.time() - t0, 1)})
    return tr.params(), hist


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--boxes", type=int, default=192)
    ap.add_argument("--max-vertices", type=int, default=2_000_000)
    ap.add_argument("--steps", type=int, default=6000)
    ap.add_argument("--batch", type=int, default=8192)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--seed", type=int, default=3)
    ap.add_argument("--out", default=PARAMS_FILE)
    a = ap.parse_args()
    t0 = time.time()
    x, y = training_pairs(a.boxes, seed=a.seed, max_vertices=a.max_vertices)
    t_data = time.time() - t0
    nval = max(1, x.shape[0] // 20)
    p, hist = train(x[nval:], y[nval:], steps=a.steps, batch=a.batch, lr=a.lr, seed=a.seed)
    import torch
    tr = Trainer(p, a.batch)
    pred = tr.forward(torch.from_numpy(np.ascontiguousarray(x[:nval]).view(np.int16)).cuda()).cpu().numpy()
    rel = float(np.sqrt(np.mean((pred - y[:nval]) ** 2) / np.mean(y[:nval] ** 2)))
    meta = {"pairs": int(x.shape[0]), "boxes": a.boxes, "seed": a.seed, "steps": a.steps, "batch": a.batch,
            "lr": a.lr, "data_s": round(t_data, 1), "val_rel_rms": rel, "history": hist}
    save_params(p, a.out, meta)
    print(json.dumps({k: v for k, v in meta.items() if k != "history"}), flush=True)
    print(json.dumps(hist[-3:]), flush=True)


if __name__ == "__main__":
    main()
