"""The FP64 reference of the b_kappa surrogate network: gradients against
finite differences, BF16 rounding against torch's, Adam against torch's."""
import numpy as np
import pytest

from oracle import mlp as M


def small_params(seed=1, widths=(8, 16, 16, 16, 16, 1)):
    return M.init_params(seed, widths)


def test_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    ps = small_params()
    x = rng.uniform(-1, 1, (12, 8))
    t = rng.normal(size=12)
    loss, g = M.loss_and_grads(ps, x, t)
    eps = 1e-6
    for li, (W, b) in enumerate(ps):
        for idx in [(0, 0), (W.shape[0] - 1, W.shape[1] - 1), (W.shape[0] // 2, W.shape[1] // 3)]:
            Wp = W.copy()
            Wp[idx] += eps
            Wm = W.copy()
            Wm[idx] -= eps
            lp = M.loss_and_grads([(Wp, b) if i == li else p for i, p in enumerate(ps)], x, t)[0]
            lm = M.loss_and_grads([(Wm, b) if i == li else p for i, p in enumerate(ps)], x, t)[0]
            assert g[li][0][idx] == pytest.approx((lp - lm) / (2 * eps), rel=1e-5, abs=1e-9)
        bp = b.copy()
        bp[0] += eps
        bm = b.copy()
        bm[0] -= eps
        lp = M.loss_and_grads([(W, bp) if i == li else p for i, p in enumerate(ps)], x, t)[0]
        lm = M.loss_and_grads([(W, bm) if i == li else p for i, p in enumerate(ps)], x, t)[0]
        assert g[li][1][0] == pytest.approx((lp - lm) / (2 * eps), rel=1e-5, abs=1e-9)


def test_bf16_rounding_matches_torch():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(3)
    a = np.concatenate([rng.normal(size=1000) * 10.0 ** rng.integers(-20, 20, 1000),
                        [0.0, -0.0, 1.0, 1.00390625, 1.0078125, 3.0e38, -1e-40]])
    ours = M.bf16(a)
    ref = torch.tensor(a, dtype=torch.float32).to(torch.bfloat16).to(torch.float64).numpy()
    assert np.array_equal(ours, ref)


def test_adam_matches_torch():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(4)
    ps = small_params(2)
    x = rng.uniform(-1, 1, (20, 8))
    t = rng.normal(size=20)
    tp = [(torch.tensor(W, requires_grad=True), torch.tensor(b, requires_grad=True)) for W, b in ps]
    opt = torch.optim.Adam([p for pair in tp for p in pair], lr=1e-2)
    state = {}
    for _ in range(3):
        _, g = M.loss_and_grads(ps, x, t)
        ps = M.adam_step(ps, g, state, lr=1e-2)
        opt.zero_grad()
        h = torch.tensor(x)
        for i, (W, b) in enumerate(tp):
            z = h @ W.T + b
            h = z if i == len(tp) - 1 else torch.nn.functional.silu(z)
        loss = ((h[:, 0] - torch.tensor(t)) ** 2).mean()
        loss.backward()
        opt.step()
    for (W, b), (tW, tb) in zip(ps, tp):
        assert np.allclose(W, tW.detach().numpy(), rtol=1e-10, atol=1e-12)
        assert np.allclose(b, tb.detach().numpy(), rtol=1e-10, atol=1e-12)
