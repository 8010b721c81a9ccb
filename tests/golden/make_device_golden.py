"""Golden vectors from the reference's OWN device code (bispec,
integrand_bkappa, the Gamma integrands), run on a GB300.

The reference's hot functions are __device__-only, so they are pinned in
three steps:

1. ``prepare`` (where the reference tree exists; REF = its cuda_version
   directory): builds the reference's tables with its own host code
   (oracle/_ref/libref_host.so, ``make -C oracle ref REF=...``), compiles its
   device code with the harness kernels of oracle/ref_device.cu into
   oracle/_ref/ref_device.cubin (``make -C oracle refdev REF=...``) and writes
   the inputs to oracle/_ref/device_inputs.npz.
2. ``run`` (on the GPU machine; needs only the two files of step 1, numpy and
   the CUDA driver): loads the cubin through the driver API, uploads the
   constants the reference's copyConstants / set_cosmology /
   compute_weights_bessel upload (bispectrum.cu:90-219, gamma.cu:13-56), runs
   the harness kernels and writes the outputs (default
   gpurun_out/ref_device_out.npz).
3. ``finish``: merges inputs and outputs into tests/golden/reference_device.npz,
   the committed fixture the tests read.

Only z in [dz/2, z_max) is evaluated: below half a bin the reference reads
table index -1 (bispectrum.cu:356-359, 389-392, 421-424).
"""
import ctypes as C
import math
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

REF_DIR = os.path.join(ROOT, "oracle", "_ref")
CUBIN = os.path.join(REF_DIR, "ref_device.cubin")
INPUTS = os.path.join(REF_DIR, "device_inputs.npz")
FIXTURE = os.path.join(HERE, "reference_device.npz")

NZB = 256
H0_OVER_C = 100.0 / 299792.0  # bispectrum.cuh (H0_over_c)
C_OVER_H0 = 2997.92           # bispectrum.cuh (c_over_H0)
ARCMIN = 2.9088820866e-4
COSMO_KEYS = ("h", "sigma8", "omb", "omc", "ns", "w", "om", "ow", "zmax")


def cosmologies():
    """Fiducial (configuration 1), the four corners of the Latin-hypercube box
    that bound Omega_m, sigma_8, h, w and n_s together, and the fiducial
    cosmology with a given linear P(k) table (the matter_power_lin path)."""
    from conftest import COSMO1

    out = [dict(COSMO1)]
    for om, s8, h, w, ns in ((0.2, 0.7, 0.6, -1.2, 0.92), (0.4, 0.9, 0.8, -0.8, 1.0),
                             (0.2, 0.9, 0.8, -0.8, 0.92), (0.4, 0.7, 0.6, -1.2, 1.0)):
        c = dict(h=h, sigma8=s8, omb=0.048, ns=ns, w=w, om=om, zmax=3.0)
        c["ow"], c["omc"] = 1 - om, om - 0.048
        out.append(c)
    out.append(dict(COSMO1))
    return out


def pk_table(tables_host):
    """A given linear P(k) on the convert_Pk grid (helpers.cu:202-214): 256
    values at k = kMin e^{i dk}, dk = ln(kMax/kMin)/256, here the fiducial
    Eisenstein & Hu P(k) times 1 + 0.1 sin(ln k), so a path that ignored the
    table would not match."""
    kmin, kmax = 1e-4, 1e2
    dk = math.log(kmax / kmin) / NZB
    k = kmin * np.exp(dk * np.arange(NZB))
    pk = np.array([tables_host.linear_pk(float(x)) for x in k]) * (1 + 0.1 * np.sin(np.log(k)))
    return pk, dk, kmin, kmax


def triangles():
    """12 triangles of the reference's bispectrum dump grid
    (classed_version/testApertureStatistics_bispectrum.cpp:59-65: ell
    log-spaced 1..1e5, phi on [1e-4, 2 pi - 1e-4]) and 12 random ones with
    ell1, ell2 log-uniform on [10, 4e4]."""
    ls = np.logspace(0, 5, 10)
    phis = np.linspace(1e-4, 2 * np.pi - 1e-4, 10)
    rng = np.random.default_rng(20261204)
    out = []
    while len(out) < 12:
        l1, l2, ph = ls[rng.integers(10)], ls[rng.integers(10)], phis[rng.integers(10)]
        l3 = math.sqrt(l1 * l1 + l2 * l2 + 2 * l1 * l2 * math.cos(ph))
        if l3 > 1e-3 * max(l1, l2):
            out.append((l1, l2, l3))
    while len(out) < 24:
        l1, l2 = np.exp(rng.uniform(math.log(10), math.log(4e4), 2))
        ph = rng.uniform(0, 2 * np.pi)
        l3 = math.sqrt(l1 * l1 + l2 * l2 + 2 * l1 * l2 * math.cos(ph))
        if l3 > 1e-3 * max(l1, l2):
            out.append((l1, l2, l3))
    return np.array(out)


def node_z(zmax, a96):
    """The 96 line-of-sight nodes of GQ96_of_bdelta (bispectrum.cu:299-309) in
    the node order of the GPU tables (j even: cx - dx a, odd: cx + dx a)."""
    cx = dx = zmax / 2
    z = np.empty(96)
    z[0::2] = cx - dx * a96
    z[1::2] = cx + dx * a96
    return z


def safe_nodes(z, zmax):
    f = z / zmax * NZB
    idx = np.floor(f)
    return ~((idx == 0) & (f - idx < 0.5)) & (z < zmax)


def gamma_inputs():
    rng = np.random.default_rng(7)
    tris = np.array([[10.0, 10.0, 10.0], [5.0, 10.0, 10.0], [3.0, 7.0, 9.0]]) * ARCMIN
    dz = 3.0 / NZB
    pts = np.stack([rng.uniform(0.5 * dz + 1e-9, 3.0 - 1e-6, 48), rng.uniform(0, 2 * np.pi, 48),
                    rng.uniform(1e-3, np.pi / 2 - 1e-3, 48)], 1)
    return tris, pts


def prepare(ref_tree):
    import oracle as O
    from conftest import nz_table

    for target in ("ref", "refdev"):
        r = subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), target, "REF=" + ref_tree],
                           capture_output=True, text=True)
        if r.returncode:
            raise SystemExit(r.stdout + r.stderr)
    R = O.ref_lib()
    zs, ns = nz_table()
    nz = O.read_n_of_z(zs, ns, NZB, 3.0)
    a96, w96 = np.zeros(48), np.zeros(48)
    R.ref_gq96(O._dp(a96), O._dp(w96))
    cos = cosmologies()
    tabs, cvec = [], []
    for c in cos:
        R.ref_set_cosmo(*[c[k] for k in COSMO_KEYS])
        out = np.zeros(6 * NZB + 1)
        R.ref_build_tables(O._dp(nz), O._dp(out))
        tabs.append(out)
        cvec.append([c[k] for k in COSMO_KEYS])
    pk, dk, kmin, kmax = pk_table(O.Tables(cos[0], nz))
    pk_given = np.zeros(len(cos), dtype=np.int32)
    pk_given[-1] = 1
    z = node_z(3.0, a96)
    og = O.ogata_weights()  # psi6, prod6, psi2, prod2 (33 each)
    gt, gp = gamma_inputs()
    np.savez(INPUTS, cosmo=np.array(cvec), tables=np.array(tabs), nz=nz, a96=a96, w96=w96, pk=pk,
             pk_grid=np.array([dk, kmin, kmax]), pk_given=pk_given, ell=triangles(), node_z=z,
             node_safe=safe_nodes(z, 3.0), ogata=og, gamma_tri=gt, gamma_pts=gp,
             gamma_cosmo=np.array([0, 1], dtype=np.int32))
    print("wrote", INPUTS, "and", CUBIN)


# ---------------------------------------------------------------------------
# step 2: CUDA driver API (ctypes), no toolkit needed on the GPU machine
class Driver:
    def __init__(self):
        self.cu = C.CDLL("libcuda.so.1")
        self.ok(self.cu.cuInit(0))
        dev = C.c_int()
        self.ok(self.cu.cuDeviceGet(C.byref(dev), 0))
        self.ctx = C.c_void_p()
        self.ok(self.cu.cuDevicePrimaryCtxRetain(C.byref(self.ctx), dev))
        self.ok(self.cu.cuCtxSetCurrent(self.ctx))
        self.mod = C.c_void_p()
        data = open(CUBIN, "rb").read()
        self._img = C.create_string_buffer(data, len(data))
        self.ok(self.cu.cuModuleLoadData(C.byref(self.mod), self._img))

    @staticmethod
    def ok(rc):
        if rc != 0:
            raise RuntimeError(f"CUDA driver error {rc}")

    def set(self, name, arr, ctype=np.float64):
        a = np.ascontiguousarray(np.atleast_1d(arr), dtype=ctype)
        ptr, size = C.c_uint64(), C.c_size_t()
        self.ok(self.cu.cuModuleGetGlobal_v2(C.byref(ptr), C.byref(size), self.mod, name.encode()))
        if size.value != a.nbytes:
            raise RuntimeError(f"{name}: symbol has {size.value} bytes, value {a.nbytes}")
        self.ok(self.cu.cuMemcpyHtoD_v2(ptr, a.ctypes.data_as(C.c_void_p), C.c_size_t(a.nbytes)))

    def alloc(self, nbytes, host=None):
        p = C.c_uint64()
        self.ok(self.cu.cuMemAlloc_v2(C.byref(p), C.c_size_t(max(nbytes, 8))))
        if host is not None:
            h = np.ascontiguousarray(host)
            self.ok(self.cu.cuMemcpyHtoD_v2(p, h.ctypes.data_as(C.c_void_p), C.c_size_t(h.nbytes)))
        return p

    def get(self, p, n):
        out = np.zeros(n)
        self.ok(self.cu.cuMemcpyDtoH_v2(out.ctypes.data_as(C.c_void_p), p, C.c_size_t(out.nbytes)))
        return out

    def free(self, p):
        self.cu.cuMemFree_v2(p)

    def launch(self, name, grid, block, args):
        f = C.c_void_p()
        self.ok(self.cu.cuModuleGetFunction(C.byref(f), self.mod, name.encode()))
        holders = [a if isinstance(a, (C.c_uint64, C.c_int, C.c_double)) else C.c_int(a) for a in args]
        params = (C.c_void_p * len(holders))(*[C.cast(C.byref(h), C.c_void_p) for h in holders])
        self.ok(self.cu.cuLaunchKernel(f, grid, 1, 1, block, 1, 1, 0, None, params, None))
        self.ok(self.cu.cuCtxSynchronize())


def upload_cosmology(D, inp, ci):
    c = dict(zip(COSMO_KEYS, inp["cosmo"][ci]))
    t = inp["tables"][ci]
    # copyConstants (bispectrum.cu:90-98)
    D.set("dev_A96", inp["a96"])
    D.set("dev_W96", inp["w96"])
    D.set("dev_H0_over_c", H0_OVER_C)
    D.set("dev_c_over_H0", C_OVER_H0)
    D.set("dev_n_redshift_bins", NZB, np.int32)
    D.set("dev_n_kbins", NZB, np.int32)
    # set_cosmology (bispectrum.cu:100-219)
    for k, name in (("h", "dev_h"), ("sigma8", "dev_sigma8"), ("omb", "dev_omb"), ("omc", "dev_omc"),
                    ("ns", "dev_ns"), ("w", "dev_w"), ("om", "dev_om"), ("ow", "dev_ow")):
        D.set(name, c[k])
    given = int(inp["pk_given"][ci])
    D.set("dev_Pk_given", given, np.uint8)
    if given:
        dk, kmin, kmax = inp["pk_grid"]
        D.set("dev_dk", dk)
        D.set("dev_k_min", kmin)
        D.set("dev_k_max", kmax)
        D.set("dev_Pk", inp["pk"])
    D.set("dev_norm", t[6 * NZB])
    D.set("dev_dz", c["zmax"] / NZB)
    D.set("dev_z_max", c["zmax"])
    for i, name in enumerate(("dev_f_K_array", "dev_g_array", "dev_D1_array", "dev_r_sigma_array",
                              "dev_n_eff_array", "dev_ncur_array")):
        D.set(name, t[i * NZB:(i + 1) * NZB])
    # compute_weights_bessel (gamma.cu:13-56): Ogata nodes and weights
    og = inp["ogata"]
    D.set("dev_array_psi", og[0])
    D.set("dev_array_product", og[1])
    D.set("dev_array_psi_J2", og[2])
    D.set("dev_array_product_J2", og[3])
    D.set("dev_prec_k", og.shape[1], np.int32)


def run(out_path):
    inp = dict(np.load(INPUTS))
    D = Driver()
    ell, z = inp["ell"], inp["node_z"][inp["node_safe"]]
    nt, nzs = len(ell), len(z)
    res = {}
    d_ell, d_z = D.alloc(ell.nbytes, ell), D.alloc(z.nbytes, z)
    d_b, d_i = D.alloc(8 * nt * nzs), D.alloc(8 * nt * nzs)
    bis, integ = [], []
    for ci in range(len(inp["cosmo"])):
        upload_cosmology(D, inp, ci)
        n = nt * nzs
        D.launch("ref_node_eval", (n + 127) // 128, 128,
                 [d_ell, d_z, C.c_int(nt), C.c_int(nzs), d_b, d_i])
        bis.append(D.get(d_b, n).reshape(nt, nzs))
        integ.append(D.get(d_i, n).reshape(nt, nzs))
    res["bispec"], res["integrand"] = np.array(bis), np.array(integ)
    gp = inp["gamma_pts"]
    d_p, d_o = D.alloc(gp.nbytes, gp), D.alloc(16 * len(gp))
    gam = np.zeros((len(inp["gamma_cosmo"]), len(inp["gamma_tri"]), 2, len(gp)), dtype=np.complex128)
    for a, ci in enumerate(inp["gamma_cosmo"]):
        upload_cosmology(D, inp, int(ci))
        for b, x in enumerate(inp["gamma_tri"]):
            for which in (0, 1):
                D.launch("ref_gamma_points", (len(gp) + 63) // 64, 64,
                         [d_p, C.c_int(len(gp)), C.c_double(x[0]), C.c_double(x[1]), C.c_double(x[2]),
                          C.c_int(which), d_o])
                o = D.get(d_o, 2 * len(gp))
                gam[a, b, which] = o[0::2] + 1j * o[1::2]
    res["gamma"] = gam
    for p in (d_ell, d_z, d_b, d_i, d_p, d_o):
        D.free(p)
    os.makedirs(os.path.dirname(os.path.abspath(out_path)), exist_ok=True)
    np.savez(out_path, **res)
    print("wrote", out_path, {k: v.shape for k, v in res.items()},
          "finite:", all(np.isfinite(v).all() for v in res.values()))


def finish(out_path):
    inp = dict(np.load(INPUTS))
    res = dict(np.load(out_path))
    keep = ("cosmo", "pk", "pk_grid", "pk_given", "ell", "node_z", "node_safe", "ogata", "gamma_tri",
            "gamma_pts", "gamma_cosmo", "tables")
    np.savez_compressed(FIXTURE, **{k: inp[k] for k in keep}, **res)
    print("wrote", FIXTURE, os.path.getsize(FIXTURE), "bytes")


if __name__ == "__main__":
    if len(sys.argv) < 2 or sys.argv[1] not in ("prepare", "run", "finish"):
        raise SystemExit("usage: make_device_golden.py prepare <reference cuda_version dir> | run [out.npz] | "
                         "finish [out.npz]")
    step = sys.argv[1]
    if step == "prepare":
        if len(sys.argv) < 3:
            raise SystemExit("prepare needs the reference's cuda_version directory")
        prepare(sys.argv[2])
    else:
        path = sys.argv[2] if len(sys.argv) > 2 else os.path.join(ROOT, "gpurun_out", "ref_device_out.npz")
        run(path) if step == "run" else finish(path)
