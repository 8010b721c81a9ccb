"""Operation count of the reference's per-point formula (TEST INFRASTRUCTURE ONLY).

Restates, in Python over a counting number type, the FP64 chain the reference
evaluates at one <Map^3> cubature point: the Eisenstein & Hu linear P(k)
(cuda_version/bispectrum.cu:602-693; oracle.cpp linear_pk), the mid-bin
interpolation (bispectrum.cu:335-437), E(z) (:921-928), F2 and F2_tree
(:700-719), bispec (:221-291), integrand_bkappa and the 96-node bkappa
(:293-333), uHat and the point of integrand_Map3_kernel
(apertureStatistics.cu:18-22, 138-153). Values and tables come from the
oracle, and tests/test_opcount.py checks that this restatement reproduces the
oracle's numbers, so the counts are those of the oracle's (= the reference's)
operation sequence.

Counted: every floating-point add, subtract, multiply, divide and comparison
on run-time values (constants folded as a compiler folds them), and every call
of pow, exp, log, log10, sqrt, sin, cos, acos, atan2, fabs, each as one call.
``flop_equivalent`` converts calls to FLOPs with the weights of WEIGHTS (a
declared convention, written into roofline.json with the counts).
"""
from __future__ import annotations

import math

# FLOP weight of one call (declared convention)
WEIGHTS = {"add": 1, "mul": 1, "div": 4, "cmp": 1, "fabs": 1, "sqrt": 4, "exp": 16, "log": 16, "log10": 16,
           "pow": 32, "sin": 16, "cos": 16, "acos": 24, "atan2": 24}

COUNTS: dict[str, int] = {}


def reset():
    COUNTS.clear()


def _c(name, n=1):
    COUNTS[name] = COUNTS.get(name, 0) + n


class N:
    """A float whose arithmetic is counted."""

    __slots__ = ("v",)

    def __init__(self, v):
        self.v = float(v.v if isinstance(v, N) else v)

    @staticmethod
    def _v(x):
        return x.v if isinstance(x, N) else float(x)

    def __add__(self, o):
        _c("add")
        return N(self.v + N._v(o))

    __radd__ = __add__

    def __sub__(self, o):
        _c("add")
        return N(self.v - N._v(o))

    def __rsub__(self, o):
        _c("add")
        return N(N._v(o) - self.v)

    def __mul__(self, o):
        _c("mul")
        return N(self.v * N._v(o))

    __rmul__ = __mul__

    def __truediv__(self, o):
        _c("div")
        return N(self.v / N._v(o))

    def __rtruediv__(self, o):
        _c("div")
        return N(N._v(o) / self.v)

    def __neg__(self):
        return N(-self.v)

    def _cmp(self, o, f):
        _c("cmp")
        return f(self.v, N._v(o))

    def __lt__(self, o):
        return self._cmp(o, lambda a, b: a < b)

    def __le__(self, o):
        return self._cmp(o, lambda a, b: a <= b)

    def __gt__(self, o):
        return self._cmp(o, lambda a, b: a > b)

    def __ge__(self, o):
        return self._cmp(o, lambda a, b: a >= b)

    def __float__(self):
        return self.v


def _f1(name, fn):
    def g(x):
        _c(name)
        return N(fn(N._v(x)))

    return g


exp = _f1("exp", math.exp)
log = _f1("log", math.log)
log10 = _f1("log10", math.log10)
sqrt = _f1("sqrt", math.sqrt)
sin = _f1("sin", math.sin)
cos = _f1("cos", math.cos)
acos = _f1("acos", math.acos)
fabs = _f1("fabs", abs)


def pow_(x, y):
    _c("pow")
    return N(math.pow(N._v(x), N._v(y)))


PI = 3.14159265358979323846
NZ = 256


class Model:
    """Cosmology, tables and the GQ96 rule, all as the oracle holds them."""

    def __init__(self, cosmo: dict, arrays: dict, gq_a, gq_w):
        self.c = {k: N(v) for k, v in cosmo.items()}
        self.t = {k: [N(x) for x in arrays[k]] for k in ("f_K", "g", "D1", "r_sigma", "n_eff", "ncur")}
        self.norm = N(arrays["norm"])
        self.z_max = float(cosmo["zmax"])
        self.gq_a, self.gq_w = list(gq_a), list(gq_w)

    # bispectrum.cu:602-693 (Eisenstein & Hu branch)
    def linear_pk(self, k):
        c = self.c
        k = k * c["h"]
        fc = c["omc"] / c["om"]
        fb = c["omb"] / c["om"]
        theta = 2.728 / 2.7
        pc = 0.25 * (5.0 - sqrt(1.0 + 24.0 * fc))
        omh2 = c["om"] * c["h"] * c["h"]
        ombh2 = c["omb"] * c["h"] * c["h"]
        zeq = 2.5e4 * omh2 / math.pow(theta, 4)
        b1 = 0.313 * pow_(omh2, -0.419) * (1.0 + 0.607 * pow_(omh2, 0.674))
        b2 = 0.238 * pow_(omh2, 0.223)
        zd = 1291.0 * pow_(omh2, 0.251) / (1.0 + 0.659 * pow_(omh2, 0.828)) * (1.0 + b1 * pow_(ombh2, b2))
        yd = (1.0 + zeq) / (1.0 + zd)
        sh = 44.5 * log(9.83 / omh2) / sqrt(1.0 + 10.0 * pow_(ombh2, 0.75))
        alnu = (fc * (5.0 - 2.0 * pc) / 5.0 * (1.0 - 0.553 * fb + 0.126 * fb * fb * fb) * pow_(1.0 + yd, -pc) *
                (1.0 + 0.5 * pc * (1.0 + 1.0 / (7.0 * (3.0 - 4.0 * pc))) / (1.0 + yd)))
        geff = omh2 * (sqrt(alnu) + (1.0 - sqrt(alnu)) / (1.0 + pow_(0.43 * k * sh, 4)))
        qeff = k / geff * theta * theta
        L = log(2.718281828 + 1.84 * sqrt(alnu) * qeff / (1.0 - 0.949 * fb))
        C = 14.4 + 325.0 / (1.0 + 60.5 * pow_(qeff, 1.11))
        delk = pow_(self.norm, 2) * pow_(k * 2997.9 / c["h"], 3.0 + c["ns"]) * pow_(L / (L + C * qeff * qeff), 2)
        pk = 2.0 * PI * PI / (k * k * k) * delk
        return c["h"] * c["h"] * c["h"] * pk

    # mid-bin interpolation with the lower neighbour clamped at bin 0
    def interp(self, arr, idx, didx):
        w = 1 - fabs(didx - 0.5)
        iw = 1 - w
        ii = idx
        if didx > 0.5:
            if idx == NZ - 1:
                iw = N(0.0)
            else:
                ii = idx + 1
        elif didx < 0.5:
            ii = max(idx - 1, 0)
        return arr[idx] * w + arr[ii] * iw

    def E(self, z):
        c = self.c
        return sqrt(c["om"] * pow_(1 + z, 3) + c["ow"] * pow_(1 + z, 3 * (1.0 + c["w"])))

    @staticmethod
    def F2_tree(k1, k2, k3):
        c12 = 0.5 * (k3 * k3 - k1 * k1 - k2 * k2) / (k1 * k2)
        return (5.0 / 7.0) + 0.5 * c12 * (k1 / k2 + k2 / k1) + (2.0 / 7.0) * c12 * c12

    def F2(self, k1, k2, k3, z, D1, r_sigma):
        c = self.c
        q3 = k3 * r_sigma
        logsigma8z = log10(D1 * c["sigma8"])
        a = 1.0 / (1.0 + z)
        omz = c["om"] / (c["om"] + c["ow"] * pow_(a, -3.0 * c["w"]))
        dn = pow_(10.0, -0.483 + 0.892 * logsigma8z - 0.086 * omz)
        return self.F2_tree(k1, k2, k3) + dn * q3

    def bispec(self, k1, k2, k3, z, idx, didx):
        c, t = self.c, self.t
        D1 = self.interp(t["D1"], idx, didx)
        r_sigma = self.interp(t["r_sigma"], idx, didx)
        n_eff = self.interp(t["n_eff"], idx, didx)
        q = [None, k1 * r_sigma, k2 * r_sigma, k3 * r_sigma]
        for i in range(1, 4):
            for j in range(i + 1, 4):
                if q[i] < q[j]:
                    q[i], q[j] = q[j], q[i]
        r1 = q[3] / q[1]
        r2 = (q[2] + q[3] - q[1]) / q[1]
        q = [None, k1 * r_sigma, k2 * r_sigma, k3 * r_sigma]
        ls = log10(D1 * c["sigma8"])
        an = pow_(10.0, -2.167 - 2.944 * ls - 1.106 * pow_(ls, 2) - 2.865 * pow_(ls, 3) -
                  0.310 * pow_(r1, pow_(10.0, 0.182 + 0.57 * n_eff)))
        bn = pow_(10.0, -3.428 - 2.681 * ls + 1.624 * pow_(ls, 2) - 0.095 * pow_(ls, 3))
        cn = pow_(10.0, 0.159 - 1.107 * n_eff)
        alphan = pow_(10.0, -4.348 - 3.006 * n_eff - 0.5745 * pow_(n_eff, 2) + pow_(10.0, -0.9 + 0.2 * n_eff) *
                      pow_(r2, 2))
        if alphan > 1.0 - (2.0 / 3.0) * c["ns"]:
            alphan = 1.0 - (2.0 / 3.0) * c["ns"]
        betan = pow_(10.0, -1.731 - 2.845 * n_eff - 1.4995 * pow_(n_eff, 2) - 0.2811 * pow_(n_eff, 3) + 0.007 * r2)
        BS1h = N(1.0)
        for i in range(1, 4):
            BS1h = BS1h * (1.0 / (an * pow_(q[i], alphan) + bn * pow_(q[i], betan)) / (1.0 + 1.0 / (cn * q[i])))
        fn = pow_(10.0, -10.533 - 16.838 * n_eff - 9.3048 * pow_(n_eff, 2) - 1.8263 * pow_(n_eff, 3))
        gn = pow_(10.0, 2.787 + 2.405 * n_eff + 0.4577 * pow_(n_eff, 2))
        hn = pow_(10.0, -1.118 - 0.394 * n_eff)
        mn = pow_(10.0, -2.605 - 2.434 * ls + 5.71 * pow_(ls, 2))
        nn = pow_(10.0, -4.468 - 3.08 * ls + 1.035 * pow_(ls, 2))
        mun = pow_(10.0, 15.312 + 22.977 * n_eff + 10.9579 * pow_(n_eff, 2) + 1.6586 * pow_(n_eff, 3))
        nun = pow_(10.0, 1.347 + 1.246 * n_eff + 0.4525 * pow_(n_eff, 2))
        pn = pow_(10.0, 0.071 - 0.433 * n_eff)
        en = pow_(10.0, -0.632 + 0.646 * n_eff)
        PSE = [None] * 4
        for i in range(1, 4):
            PSE[i] = ((1.0 + fn * pow_(q[i], 2)) / (1.0 + gn * q[i] + hn * pow_(q[i], 2)) * pow_(D1, 2) *
                      self.linear_pk(q[i] / r_sigma) +
                      1.0 / (mn * pow_(q[i], mun) + nn * pow_(q[i], nun)) / (1.0 + pow_(pn * q[i], -3)))
        BS3h = 2.0 * (self.F2(k1, k2, k3, z, D1, r_sigma) * PSE[1] * PSE[2] +
                      self.F2(k2, k3, k1, z, D1, r_sigma) * PSE[2] * PSE[3] +
                      self.F2(k3, k1, k2, z, D1, r_sigma) * PSE[3] * PSE[1])
        for i in range(1, 4):
            BS3h = BS3h * (1.0 / (1.0 + en * q[i]))
        return BS1h + BS3h

    def integrand_bkappa(self, z, l1, l2, l3):
        if z < 1.0e-7:
            return N(0.0)
        didx = z / self.z_max * NZ
        idx = int(didx.v)
        didx = didx - idx
        g = self.interp(self.t["g"], idx, didx)
        fK = self.interp(self.t["f_K"], idx, didx)
        r = pow_(g * (1.0 + z), 3) * self.bispec(l1 / fK, l2 / fK, l3 / fK, z, idx, didx) / fK / self.E(z)
        return r

    def bkappa(self, l1, l2, l3):
        prefactor = 27.0 / 8.0 * pow_(self.c["om"], 3) * math.pow(100.0 / 299792.0, 5)
        cx = N(self.z_max) / 2
        dx = N(self.z_max) / 2
        q = N(0.0)
        for a, w in zip(self.gq_a, self.gq_w):
            q = q + w * (self.integrand_bkappa(cx - dx * a, l1, l2, l3) + self.integrand_bkappa(cx + dx * a, l1, l2, l3))
        return prefactor * (q * dx)

    @staticmethod
    def uHat(eta):
        temp = 0.5 * eta * eta
        return temp * exp(-temp)

    def map3_point(self, l1, l2, phi, th):
        l1, l2, phi = N(l1), N(l2), N(phi)
        l3 = sqrt(l1 * l1 + l2 * l2 + 2 * l1 * l2 * cos(phi))
        return (l1 * l2 * self.bkappa(l1, l2, l3) * self.uHat(l1 * th[0]) * self.uHat(l2 * th[1]) *
                self.uHat(l3 * th[2]))


def flop_equivalent(counts: dict) -> float:
    return float(sum(WEIGHTS[k] * v for k, v in counts.items()))


def count(fn, *args):
    """(value, counts) of one call"""
    reset()
    v = fn(*args)
    return float(v), dict(COUNTS)
