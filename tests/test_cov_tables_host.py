"""The argument patterns and multiplicities of the covariance totals
(T1/T2/T4/T5/T6/T7_total, apertureStatisticsCovariance.cu:272-1044) as the
library sums them, against the oracle's restatement, on the host: the term
is replaced by an injective probe of its six radii, so no integral runs."""
import ctypes as C
import itertools

import numpy as np
import pytest

import oracle as O

PROBE = C.CFUNCTYPE(C.c_double, C.POINTER(C.c_double))


def _probe(th):
    # radii are small integers: the base-7 digits identify every ordering exactly
    return float(sum(th[i] * 7.0 ** i for i in range(6)))


def _product_terms(L, term, geom, a, b):
    mult = (C.c_int * 32)()
    idx = (C.c_int * 192)()
    aa = (C.c_double * 3)(*a)
    bb = (C.c_double * 3)(*b)
    n = L.tp_cov_total_terms(term, geom, aa, bb, mult, idx, 32)
    assert n >= 0
    return [(mult[k], tuple(idx[6 * k:6 * k + 6])) for k in range(n)]


@pytest.fixture(scope="module")
def plib():
    import threepoint_gb300 as tp

    L = tp.lib()
    L.tp_cov_total_terms.restype = C.c_int
    L.tp_cov_total_terms.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                     C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_int]
    return L


TRIPLETS = list(itertools.product((1.0, 2.0, 3.0), repeat=3))


@pytest.mark.parametrize("term,geom", [(1, 1), (1, 2), (2, 1), (2, 2), (4, 2)])
def test_t1_t2_t4_totals_match_oracle(plib, term, geom):
    cb = PROBE(lambda p: _probe([p[i] for i in range(6)]))
    for a in TRIPLETS:
        for b in TRIPLETS:
            ref = O.lib().orc_total_probe(term, geom, C.cast(cb, C.c_void_p), O._dp(np.array(a)), O._dp(np.array(b)))
            src = list(a) + list(b)
            got = sum(m * _probe([src[i] for i in ix]) for m, ix in _product_terms(plib, term, geom, a, b))
            assert got == ref, (term, geom, a, b)


@pytest.mark.parametrize("term", [5, 6, 7])
def test_halo_totals_match_oracle(plib, term):
    for a in TRIPLETS:
        for b in TRIPLETS:
            assert _product_terms(plib, term, 1, a, b) == O.halo_total_terms(term, a, b), (term, a, b)
    # T6_total of the infinite survey is 0 (apertureStatisticsCovariance.cu:849-850)
    assert _product_terms(plib, 6, 2, (1.0, 2.0, 3.0), (1.0, 2.0, 3.0)) == []
