"""The surrogate network's tensor-core kernels against plain PyTorch FP32 (the
GEMM) and the FP64 reference network of oracle/mlp.py (forward, gradients)."""
import numpy as np
import pytest

from oracle import mlp as M

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def net():
    import threepoint_gb300 as tp

    m = tp.MLP(max_batch=4096)
    yield m
    m.close()


@pytest.mark.parametrize("M_,N,K", [(128, 256, 64), (256, 256, 256), (128, 64, 1024), (384, 32, 128)])
def test_gemm_matches_torch_fp32(net, M_, N, K):
    import torch

    g = torch.Generator().manual_seed(M_ + N + K)
    A = torch.randn(M_, K, generator=g).to(torch.bfloat16).cuda()
    B = torch.randn(N, K, generator=g).to(torch.bfloat16).cuda()
    Cm = torch.full((M_, N), float("nan"), dtype=torch.float32, device="cuda")
    net.gemm_device(A, B, Cm)
    ref = A.float() @ B.float().T
    err = (Cm - ref).abs().max().item()
    assert err <= 1e-4 * ref.abs().max().item() + 1e-5, err


def test_gemm_rejects_unsupported_shapes(net):
    import torch

    import threepoint_gb300 as tp

    A = torch.zeros(128, 64, dtype=torch.bfloat16, device="cuda")
    B = torch.zeros(48, 64, dtype=torch.bfloat16, device="cuda")
    Cm = torch.zeros(128, 48, dtype=torch.float32, device="cuda")
    with pytest.raises(tp.ThreepointError):
        net.gemm_device(A, B, Cm)


def params_and_data(n=1000, seed=5):
    rng = np.random.default_rng(seed)
    ps = M.init_params(seed)
    ps = [(W, rng.normal(0, 0.1, b.shape)) for W, b in ps]
    x = rng.uniform(-1, 1, (n, 8))
    t = rng.normal(size=n)
    return ps, x, t


def test_forward_matches_oracle(net):
    ps, x, _ = params_and_data()
    net.set_params(ps)
    y = net.forward(x)
    ref, _ = M.forward(ps, x, round_bf16=True)
    scale = np.abs(ref).max()
    assert np.abs(y - ref).max() < 1e-2 * scale, (np.abs(y - ref).max(), scale)
    # parameters round-trip (FP32 masters)
    back = net.get_params(flat=True)
    assert np.allclose(back, net.flatten(ps).astype(np.float32), rtol=0, atol=0)


def test_gradients_match_oracle(net):
    ps, x, t = params_and_data(2000, 6)
    net.set_params(ps)
    loss, g = net.gradients(x, t)
    lref, gref = M.loss_and_grads(ps, x, t, round_bf16=True)
    assert loss == pytest.approx(lref, rel=1e-2)
    for (gW, gb), (rW, rb) in zip(g, gref):
        for a, r in ((gW, rW), (gb, rb)):
            rel = np.linalg.norm(a - r) / max(np.linalg.norm(r), 1e-30)
            assert rel < 3e-2, rel


def test_training_reduces_loss(net):
    import torch

    rng = np.random.default_rng(7)
    n = 4096
    x = rng.uniform(-1, 1, (n, 8))
    t = np.sin(2 * x[:, 0]) + x[:, 1] * x[:, 2] - 0.5 * x[:, 3] ** 2
    net.set_params(M.init_params(8))
    l0, _ = net.gradients(x, t)
    xd = torch.tensor(x, dtype=torch.float32, device="cuda")
    td = torch.tensor(t, dtype=torch.float32, device="cuda")
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    for _ in range(300):
        net.train_step_device(xd, td, 1e-3, loss)
    net.sync()
    l1, _ = net.gradients(x, t)
    assert l1 < 0.05 * l0, (l0, l1)
