"""The b_kappa surrogate trained on FP64 line-of-sight targets of a few
cosmologies: it learns (held-out error falls well below the untrained
network's) and answers only inside its box."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_surrogate_trains_on_fp64_targets(nz256):
    import threepoint_gb300 as tp
    from threepoint_gb300 import surrogate as S

    cos = S.lhs_box(6, seed=11)
    with tp.Context(0) as ctx:
        x, y = S.generate(ctx, cos[:5], nz256, per_cosmo=8192, seed=1)
        xh, yh = S.generate(ctx, cos[5:], nz256, per_cosmo=4096, seed=2)
    assert len(y) > 0.99 * 5 * 8192 and np.isfinite(y).all()
    sg = S.Surrogate(max_batch=8192, seed=0)
    before = sg.evaluate(xh, yh)
    hist = sg.fit(x, y, steps=1500, batch=8192, lr=2e-3, lr_end=1e-4, log_every=500)
    after = sg.evaluate(xh, yh)
    assert hist[-1][1] < 0.05 * hist[0][1], hist
    assert after["median"] < 0.2 * before["median"], (before, after)
    ell = np.array([[100.0, 200.0, 250.0], [5.0, 200.0, 200.0]])
    v, m = sg.bkappa(ell, S.cosmo_array([tp.cosmology(**cos[5])])[0])
    assert m.tolist() == [True, False] and np.isfinite(v[0]) and np.isnan(v[1])
    sg.close()
