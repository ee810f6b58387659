"""Generates tests/golden/config3_20000.npz: the FP64 oracle's run of the
config-3 Shan-Chen adsorption workload for its full Nt = 20000 steps.

Test infrastructure: the oracle's restatement (oracle/lbm_oracle.cpp, pinned
against the reference's own adsorption runs) on the grid tables of
mantiis_gb300.HostGrid, on all host cores (tens of minutes).  Workload:
workloads.config3(0) (512x512 seeded disk image, porosity 0.6), the exponential
pseudopotential psi = 0.5 (1 - exp(-rho / 0.5)), G = -4.5 and G_ads = -0.5 in
the common Shan-Chen convention (G_ff = G / 18, G_fs = 3 G_ads in the
reference's), no body force, initial density 0.5 + U[-1e-3, 1e-3] (seed 3000).
The fixture holds the adsorbed-layer density profile (mean density of the
fluid cells at Euclidean wall distance d, d = 1..12, rounded to the nearest
integer), the total mass every 1000 steps, the density residual history, and
rho of every 4th cell at the end.

Usage: python tests/golden/make_config3.py [--steps N]
"""
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from mantiis_gb300 import SIM_ADSORPTION, HostGrid, default_params, workloads  # noqa: E402
from oracle.pyoracle import for_grid  # noqa: E402

KW = dict(psi_form=1, rho_psi=0.5, g_ff=-4.5 / 18, g_fs=-1.5)
DMAX = 12


def wall_distance(pore):
    """Euclidean distance of every pixel to the nearest solid pixel, rounded."""
    from scipy.ndimage import distance_transform_edt

    return np.rint(distance_transform_edt(pore)).astype(np.int64)


def profile(grid, rho, dist):
    """Mean density of the cells at wall distance d = 1..DMAX."""
    d = dist[grid.cells["y"], grid.cells["x"]]
    return np.array([rho[d == k].mean() if (d == k).any() else 0.0 for k in range(1, DMAX + 1)])


def setup():
    img = workloads.config3(0)
    p = default_params(dx=img["dx"], simulation=SIM_ADSORPTION, rho_init=0.5, fbody=0.0, tol=0.0, **KW)
    g = HostGrid(img["pore"], img["kn"], img["locpore"], p)
    rng = np.random.default_rng(3000)
    rho0 = 0.5 + rng.uniform(-1e-3, 1e-3, g.n_cells)
    return img, p, g, rho0


def main():
    steps = int(sys.argv[sys.argv.index("--steps") + 1]) if "--steps" in sys.argv else 20000
    img, p, g, rho0 = setup()
    o = for_grid(g, sim="adsorption", dx=img["dx"], fbody=0.0, rho_init=rho0, threads=os.cpu_count() or 1, **KW)
    mass, done = [rho0.sum()], 0
    while done < steps:
        o.run(1000)
        done += 1000
        f = o.fields()
        mass.append(f["rho"].sum())
        print(f"step {done}  mass {mass[-1]:.15e}  rho {f['rho'].min():.6f}..{f['rho'].max():.6f}", flush=True)
    f = o.fields()
    dist = wall_distance(img["pore"])
    sub = np.arange(0, g.n_cells, 4)
    np.savez_compressed(HERE / "config3_20000.npz", steps=done, profile=profile(g, f["rho"], dist),
                        mass=np.array(mass), residuals=o.residuals(), cells=sub, rho=f["rho"][sub])
    print("written", HERE / "config3_20000.npz")


if __name__ == "__main__":
    main()
