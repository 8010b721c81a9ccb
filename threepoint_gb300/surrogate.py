"""Surrogate of log b_kappa over a box of triangles and cosmologies.

The network (threepoint_gb300.MLP: 8 -> 256 x 4 -> 1, SiLU, BF16 tensor-core
kernels with FP32 accumulation) maps the features

    (log l1, log l2, log l3, Omega_m, sigma_8, h, w, n_s)

each scaled to [-1, 1] over the box below, to the standardised log b_kappa.
Training targets come from the plain FP64 line-of-sight b_kappa of the
library (tp_bkappa_batch), evaluated at triangles with l1, l2 log-uniform on
[10, 4e4], phi uniform on [0, 2 pi) and l3 = |l1 + l2 e^{i phi}| inside the
same range, for Latin-hypercube cosmologies of the box. Points outside the box
(``in_box`` False) are not the network's to answer: the caller evaluates them
with the plain BiHalofit sum.
"""
from __future__ import annotations

import math

import numpy as np

# cosmology box (the Latin hypercube of the benchmark's 4096 cosmologies)
BOX = (("om", 0.2, 0.4), ("sigma8", 0.7, 0.9), ("h", 0.6, 0.8), ("w", -1.2, -0.8), ("ns", 0.92, 1.0))
L_RANGE = (10.0, 4.0e4)
OMB = 0.048


def cosmo_array(cosmos):
    """[n, 5] box parameters of threepoint_gb300.cosmology objects or dicts"""
    get = (lambda c, k: c[k]) if cosmos and isinstance(cosmos[0], dict) else getattr
    return np.array([[float(get(c, k)) for k, _, _ in BOX] for c in cosmos])


def features(ell, cos):
    """[n, 8] scaled features of triangles ell [n, 3] and box parameters
    cos [n, 5] (or [5], shared)"""
    ell = np.asarray(ell, dtype=np.float64).reshape(-1, 3)
    cos = np.broadcast_to(np.asarray(cos, dtype=np.float64), (len(ell), len(BOX)))
    a, b = math.log(L_RANGE[0]), math.log(L_RANGE[1])
    with np.errstate(divide="ignore", invalid="ignore"):
        fl = (2.0 * np.log(ell) - (a + b)) / (b - a)
    lo = np.array([v[1] for v in BOX])
    hi = np.array([v[2] for v in BOX])
    fc = (2.0 * cos - (lo + hi)) / (hi - lo)
    return np.concatenate([fl, fc], axis=1)


def in_box(ell, cos):
    """True where every feature lies in [-1, 1] (the training domain)"""
    f = features(ell, cos)
    return np.all(np.isfinite(f) & (np.abs(f) <= 1.0), axis=1)


def sample_triangles(rng, n):
    """n triangles with l1, l2 log-uniform on L_RANGE, phi uniform, l3 in L_RANGE"""
    out = np.empty((0, 3))
    a, b = math.log(L_RANGE[0]), math.log(L_RANGE[1])
    while len(out) < n:
        m = 2 * (n - len(out)) + 16
        l1 = np.exp(rng.uniform(a, b, m))
        l2 = np.exp(rng.uniform(a, b, m))
        phi = rng.uniform(0.0, 2 * math.pi, m)
        l3 = np.sqrt(np.maximum(l1 * l1 + l2 * l2 + 2 * l1 * l2 * np.cos(phi), 0.0))
        ok = (l3 >= L_RANGE[0]) & (l3 <= L_RANGE[1])
        out = np.concatenate([out, np.stack([l1, l2, l3], 1)[ok]])
    return out[:n]


def lhs_box(n, seed):
    """n Latin-hypercube cosmologies of the box (dicts of cosmology fields)"""
    rng = np.random.default_rng(seed)
    cols = {}
    for name, lo, hi in BOX:
        cols[name] = lo + (rng.permutation(n) + rng.uniform(size=n)) / n * (hi - lo)
    return [dict(h=float(cols["h"][i]), sigma8=float(cols["sigma8"][i]), omb=OMB, omc=float(cols["om"][i]) - OMB,
                 ns=float(cols["ns"][i]), w=float(cols["w"][i]), om=float(cols["om"][i]), ow=1 - float(cols["om"][i]),
                 zmax=3.0) for i in range(n)]


def generate(ctx, cosmos, nz, per_cosmo, seed=0, precision=None):
    """Training points: (features [N, 8], log b_kappa [N]) for per_cosmo
    triangles of each cosmology (dicts or cosmology objects), targets from
    the context's line-of-sight b_kappa (FP64 by default). Non-positive or
    non-finite b_kappa values are dropped."""
    import threepoint_gb300 as tp

    precision = tp.FP64 if precision is None else precision
    objs = [c if isinstance(c, tp.cosmology) else tp.cosmology(**c) for c in cosmos]
    ctx.set_cosmologies(objs, nz)
    rng = np.random.default_rng(seed)
    xs, ys = [], []
    carr = cosmo_array(objs)
    for i in range(len(objs)):
        ell = sample_triangles(rng, per_cosmo)
        bk = ctx.bkappa(ell, cosmo_index=np.full(len(ell), i, dtype=np.int32), precision=precision)
        ok = np.isfinite(bk) & (bk > 0)
        xs.append(features(ell[ok], carr[i]))
        ys.append(np.log(bk[ok]))
    return np.concatenate(xs), np.concatenate(ys)


class Surrogate:
    """Trained network plus the target standardisation."""

    def __init__(self, max_batch=65536, device=0, seed=0):
        import threepoint_gb300 as tp

        self.net = tp.MLP(max_batch=max_batch, device=device)
        self.device = device
        self.max_batch = max_batch
        self.y_mean, self.y_std = 0.0, 1.0
        rng = np.random.default_rng(seed)
        widths = tp.MLP.WIDTHS
        self.net.set_params([(rng.normal(0.0, math.sqrt(2.0 / widths[i]), (widths[i + 1], widths[i])),
                              np.zeros(widths[i + 1])) for i in range(len(widths) - 1)])

    def fit(self, x, y, steps=2000, batch=8192, lr=1e-3, lr_end=1e-5, seed=0, log_every=0):
        """Adam on random minibatches (device-resident data); learning rate
        decays geometrically from lr to lr_end. Returns the loss history
        (standardised units) at log_every steps."""
        import torch

        x = np.asarray(x, dtype=np.float64)
        y = np.asarray(y, dtype=np.float64)
        self.y_mean, self.y_std = float(y.mean()), float(y.std() or 1.0)
        dev = torch.device("cuda", self.device)
        xd = torch.tensor(x, dtype=torch.float32, device=dev)
        yd = torch.tensor((y - self.y_mean) / self.y_std, dtype=torch.float32, device=dev)
        g = torch.Generator(device=dev).manual_seed(seed)
        batch = min(batch, self.max_batch, len(y))
        loss = torch.zeros(1, dtype=torch.float32, device=dev)
        hist = []
        stream = torch.cuda.ExternalStream(self.net.stream_handle, device=dev)
        torch.cuda.synchronize(dev)
        for s in range(steps):
            lr_s = lr * (lr_end / lr) ** (s / max(1, steps - 1))
            with torch.cuda.stream(stream):
                idx = torch.randint(0, len(y), (batch,), device=dev, generator=g)
                xb = xd.index_select(0, idx).contiguous()
                yb = yd.index_select(0, idx).contiguous()
            self.net.train_step_device(xb, yb, lr_s, loss)
            if log_every and (s % log_every == 0 or s == steps - 1):
                self.net.sync()
                hist.append((s, float(loss.item())))
        self.net.sync()
        return hist

    def predict_log(self, x):
        return self.net.forward(x) * self.y_std + self.y_mean

    def bkappa(self, ell, cos):
        """(b_kappa, inside-box mask); NaN outside the box"""
        m = in_box(ell, cos)
        out = np.full(len(m), np.nan)
        if m.any():
            out[m] = np.exp(self.predict_log(features(np.asarray(ell).reshape(-1, 3)[m],
                                                      np.broadcast_to(cos, (len(m), len(BOX)))[m])))
        return out, m

    def evaluate(self, x, y):
        """relative errors of b_kappa = exp(log b_kappa) at held-out points"""
        rel = np.abs(np.expm1(self.predict_log(x) - np.asarray(y)))
        return {"median": float(np.median(rel)), "p99": float(np.quantile(rel, 0.99)), "max": float(rel.max()),
                "points": int(len(rel))}

    def save(self, path):
        np.savez(path, params=self.net.get_params(flat=True), y_mean=self.y_mean, y_std=self.y_std,
                 box=np.array([[lo, hi] for _, lo, hi in BOX]), l_range=np.array(L_RANGE))

    def load(self, path):
        z = np.load(path)
        if not np.allclose(z["box"], [[lo, hi] for _, lo, hi in BOX]) or not np.allclose(z["l_range"], L_RANGE):
            raise ValueError(f"{path}: trained for another box")
        self.net.set_params(z["params"])
        self.y_mean, self.y_std = float(z["y_mean"]), float(z["y_std"])

    def close(self):
        self.net.close()
