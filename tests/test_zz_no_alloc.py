"""The allocation-free <Map^3> entry point against the regular one.

tp_map3_jobs_noalloc exists for callers that cannot allocate device memory
while they integrate (stream capture, framework-owned allocators); it keeps its
region stores in a fixed device array of the library. This file is collected
last so that a failure here comes after every other test has run.
"""
import ctypes as C
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ARC = 2.9088820866e-4


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


@pytest.fixture(scope="module")
def setup(nz256):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import threepoint_gb300 as tp
    from conftest import COSMO1

    ctx = tp.Context(0)
    ctx.set_cosmology(tp.cosmology(**COSMO1), nz256)
    yield torch, tp, ctx
    ctx.close()


def _run(torch, tp, ctx, fn_name, th, precision, rel_tol=1e-4):
    dev = torch.device("cuda", 0)
    n = len(th)
    jc = torch.zeros(n, dtype=torch.int32, device=dev)
    jt = torch.tensor(th, dtype=torch.float64, device=dev)
    out = torch.full((n,), float("nan"), dtype=torch.float64, device=dev)
    err = torch.zeros(n, dtype=torch.float64, device=dev)
    st = torch.full((n,), -1, dtype=torch.int32, device=dev)
    L = tp.lib()
    args = (ctx._h, _ptr(jc), _ptr(jt), n, 0.0, 2 * math.pi, 1.0, 0.0, rel_tol, precision)
    if fn_name == "noalloc":
        rc = L.tp_map3_jobs_noalloc(*args, _ptr(out), _ptr(err), _ptr(st))
    else:
        rc = L.tp_map3_jobs_device(*args, _ptr(out), _ptr(err), None, None, _ptr(st), None)
    assert rc == 0, L.tp_last_error(ctx._h)
    torch.cuda.synchronize()
    return out.cpu().numpy(), st.cpu().numpy()


@pytest.mark.parametrize("precision", [1, 0])
def test_noalloc_matches_regular_entry_point_twice(setup, precision):
    torch, tp, ctx = setup
    trip = [(16, 16, 16), (8, 16, 16), (4, 8, 16), (2, 2, 2), (1, 1.47, 32), (8, 8, 32)]
    if precision == 0:
        trip = trip[:2] + trip[4:5]
    th = [[a * ARC, b * ARC, c * ARC] for a, b, c in trip]
    ref, st_ref = _run(torch, tp, ctx, "regular", th, precision)
    assert np.all(st_ref == 0)
    for _ in range(2):  # two calls in a row share (and reuse) the same scratch array
        got, st = _run(torch, tp, ctx, "noalloc", th, precision)
        assert np.all(st == 0)
        assert np.allclose(got, ref, rtol=1e-12, atol=0), (got, ref)


def test_noalloc_region_cap_sets_status_bit(setup):
    """An integral that needs more than the entry point's 8192 regions stops
    at the cap: bit 1 of its status is set, its value is still written and the
    call itself returns success."""
    torch, tp, ctx = setup
    th = [[2 * ARC, 2 * ARC, 2 * ARC], [16 * ARC, 16 * ARC, 16 * ARC]]
    got, st = _run(torch, tp, ctx, "noalloc", th, 1, rel_tol=1e-9)
    assert st[0] & 1, st
    assert np.all(np.isfinite(got))
    ref, st_ref = _run(torch, tp, ctx, "regular", th[:1], 1)
    assert st_ref[0] == 0
    assert abs(got[0] / ref[0] - 1) < 1e-3
