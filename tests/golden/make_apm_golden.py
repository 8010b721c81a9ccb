"""Golden vectors of the reference's FFT aperture-mass measurement
(python_scripts/aperture_mass_computer.py), produced by importing the
reference module itself.

Run where the reference tree exists:

    python tests/golden/make_apm_golden.py <reference python_scripts directory>

The module's top-level imports include packages that are not installed here
(astropy, lenstools, matplotlib) and the reference's own data loaders; the
functions used below (normalize_shear with CIC, Map_fft with a weight grid and
zero padding, extract_Map3_of_field) need only numpy and scipy, so those
imports are given empty stand-in modules before the import. Writes
tests/golden/reference_apm.npz: a seeded synthetic catalogue, the CIC grids,
one aperture-mass map and <Map^3> for the exponential and the polynomial
filter, with per-triplet and common border cuts.
"""
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "reference_apm.npz")

NPIX = 64
FIELDSIZE = 60.0  # arcmin
THETAS = np.array([1.0, 2.0, 4.0])  # arcmin
N_GAL = 5000


def catalogue(seed=2026):
    """Uniform positions on the field; shears = a smooth pattern + noise."""
    rng = np.random.default_rng(seed)
    x = rng.uniform(0.0, FIELDSIZE, N_GAL)
    y = rng.uniform(0.0, FIELDSIZE, N_GAL)
    g = 0.03 * np.exp(2j * np.pi * (x / 23.0 + y / 37.0)) + 0.02 * (x / FIELDSIZE - 0.5) ** 2 + \
        0.3 * (rng.standard_normal(N_GAL) + 1j * rng.standard_normal(N_GAL)) / np.sqrt(2)
    return x, y, g


def import_reference(python_scripts):
    for name in ("astropy", "astropy.convolution", "astropy.units", "astropy.io", "astropy.io.fits", "lenstools",
                 "matplotlib", "matplotlib.pyplot", "matplotlib.colors", "file_loader", "random_fields", "utility"):
        sys.modules.setdefault(name, types.ModuleType(name))
    conv = sys.modules["astropy.convolution"]
    conv.interpolate_replace_nans = conv.Gaussian2DKernel = conv.convolve_fft = None
    sys.modules["matplotlib.colors"].LogNorm = None
    for f in ("get_gamma_millennium", "get_gamma_millennium_shapenoise", "get_kappa_millennium",
              "get_millennium_downsampled_shapenoise", "get_slics", "get_kappa_slics"):
        setattr(sys.modules["file_loader"], f, None)
    sys.modules["random_fields"].create_gaussian_random_field = None
    sys.modules["random_fields"].create_lognormal_random_field = None
    sys.modules["utility"].create_gamma_field = None
    sys.path.insert(0, python_scripts)
    import aperture_mass_computer as A

    return A


def main(python_scripts):
    A = import_reference(python_scripts)
    x, y, g = catalogue()
    ac = A.aperture_mass_computer(NPIX, 1.0, FIELDSIZE)
    shears, norm = ac.normalize_shear(x, y, g)
    out = {"x": x, "y": y, "g": g, "npix": NPIX, "fieldsize": FIELDSIZE, "thetas": THETAS,
           "shears": shears, "norm": norm}
    ac.change_theta_ap(2.0)
    out["map_theta2"] = ac.Map_fft(shears, norm=norm, periodic_boundary=False)
    out["map_theta2_poly"] = A.aperture_mass_computer(NPIX, 2.0, FIELDSIZE, use_polynomial_filter=True).Map_fft(
        shears, norm=norm, periodic_boundary=False)
    for poly in (False, True):
        for same in (False, True):
            key = f"map3_poly{int(poly)}_same{int(same)}"
            out[key] = A.extract_Map3_of_field(shears, NPIX, THETAS, FIELDSIZE, norm=norm,
                                               same_fieldsize_for_all_theta=same, use_polynomial_filter=poly)
    out["map3_catalogue"] = A.extract_Map3(x, y, g, NPIX, THETAS, FIELDSIZE)
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    if len(sys.argv) < 2:
        raise SystemExit("usage: make_apm_golden.py <reference python_scripts directory>")
    main(sys.argv[1])
