"""Seeded synthetic pore images with the shapes and value ranges of the
benchmark configurations (the reference ships no benchmark images).

config1: 128x128, disk radii U[4,10], porosity 0.65, Kn ~0.1, single block
config2: 1024x1024, disk radii U[6,40], porosity U[0.5,0.7], Kn U[0.01,1], 3 levels
config3: 512x512, porosity 0.6 (Shan-Chen adsorption)
config4: side in {128,...,2048}, porosity U[0.45,0.75], 1-3 levels, log-uniform Kn in [0.01, 2]

Local pore size H comes from the reference's skeleton rule; the lattice
spacing dx is then chosen so that the mean Knudsen number over the void
pixels equals the drawn one, and Kn = mfp / (H dx) per pixel
(include/shape.hpp:245-246).
"""
import numpy as np

from .native import generate_disks, pore_properties, units


def image(n, rmin, rmax, porosity, kn_mean, seed):
    pore = generate_disks(n, rmin, rmax, porosity, seed)
    H, kn_unit = pore_properties(pore, 1.0, 1.0)  # kn_unit = 1 / H
    mfp = units()["mfp"]
    void = pore == 1
    dx = mfp * kn_unit[void].mean() / kn_mean
    kn = np.where(void, kn_unit * mfp / dx, 0.0)
    return dict(pore=pore, kn=kn, locpore=H, dx=float(dx), porosity=float(void.mean()), kn_mean=float(kn_mean))


def config1(index=0):
    return image(128, 4, 10, 0.65, 0.1, 1000 + index)


def config2(index=0):
    rng = np.random.default_rng(2000 + index)
    phi = rng.uniform(0.5, 0.7)
    kn = rng.uniform(0.01, 1.0)
    return image(1024, 6, 40, phi, kn, 2000 + index)


def config3(index=0):
    return image(512, 6, 40, 0.6, 0.1, 3000 + index)


def config4(index=0):
    rng = np.random.default_rng(4000 + index)
    n = int(rng.choice([128, 256, 512, 1024, 2048]))
    phi = rng.uniform(0.45, 0.75)
    levels = int(rng.integers(1, 4))
    kn = float(np.exp(rng.uniform(np.log(0.01), np.log(2.0))))
    d = image(n, max(2, n // 256), max(4, n // 32), phi, kn, 4000 + index)
    d["levels"] = levels
    return d
