"""Generates tests/golden/steady_mb1024.npz: the FP64 oracle's steady state of
the multi-block image workloads.config2_steady(0) (1024x1024, two levels).

Test infrastructure: it runs the oracle's restatement (oracle/lbm_oracle.cpp,
pinned against the reference's own multi-block code) on the grid tables of
mantiis_gb300.HostGrid (equal to the reference's Grid2D tables) until the
permeability k = <u_x> nu / F_body changes by less than 1e-8 (relative) over
1000 steps, on all host cores; this takes tens of minutes.  The fixture holds
k, the convergence history (k every 500 steps), the pixel-area means of u_x,
u_y and rho over 8x8 pixel blocks, and u_x, u_y, rho of every 8th cell.

Usage: python tests/golden/make_steady.py [--max-steps N]
"""
import os
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from mantiis_gb300 import HostGrid, default_params, workloads  # noqa: E402
from oracle.pyoracle import for_grid  # noqa: E402

CHUNK = 500
TOL = 1e-8


def permeability(grid, ux, fbody):
    """<u_x> over all n x n pixels (a cell counts once per covered pixel, buffer
    cells not at all) times nu = (mean tau_s over non-buffer cells - 1/2) / 3,
    over F_body."""
    c = grid.cells
    real = c["is_buffer"] == 0
    area = np.left_shift(1, 2 * (c["level"] - 1)).astype(np.float64)
    mean_ux = float((ux[real] * area[real]).sum()) / (grid.n * grid.n)
    nu = (float(c["tau"][real].mean()) - 0.5) / 3.0
    return mean_ux * nu / fbody


def block_means(grid, values, block=8):
    """Pixel fields (a cell fills its 2^(l-1) square, solids 0) averaged over
    block x block pixel squares."""
    c = grid.cells
    n = grid.n
    px = np.zeros((n, n))
    for lvl in range(1, grid.max_level + 1):
        m = (c["level"] == lvl) & (c["is_buffer"] == 0)
        s = 1 << (lvl - 1)
        for dy in range(s):
            for dx in range(s):
                px[c["y"][m] + dy, c["x"][m] + dx] = values[m]
    return px.reshape(n // block, block, n // block, block).mean(axis=(1, 3))


def main():
    max_steps = int(sys.argv[sys.argv.index("--max-steps") + 1]) if "--max-steps" in sys.argv else 100000
    img = workloads.config2_steady(0)
    p = default_params(multiblock=1, max_allowed_level=img["levels"], dx=img["dx"], edge_fine=1, tol=0.0)
    g = HostGrid(img["pore"], img["kn"], img["locpore"], p)
    o = for_grid(g, sim="transport", dx=img["dx"], fbody=p.fbody, threads=os.cpu_count() or 1)
    hist, done, t0 = [], 0, time.time()
    while done < max_steps:
        o.run(CHUNK)
        done += CHUNK
        f = o.fields()
        k = permeability(g, f["ux"], p.fbody)
        if not np.isfinite(k):
            raise SystemExit(f"non-finite state after {done} steps")
        hist.append(k)
        change = abs(hist[-1] - hist[-3]) / abs(hist[-1]) if len(hist) >= 3 else 1.0
        print(f"step {done:6d}  k {k:.12e}  change/1000 {change:.3e}  {time.time() - t0:.0f} s", flush=True)
        if change < TOL:
            break
    f = o.fields()
    sub = np.arange(0, g.n_cells, 8)
    np.savez_compressed(HERE / "steady_mb1024.npz", k=k, steps=done, history=np.array(hist), chunk=CHUNK,
                        n_cells=g.n_cells, dx=img["dx"], kn_mean=img["kn_mean"], porosity=img["porosity"],
                        ux_blocks=block_means(g, f["ux"]), uy_blocks=block_means(g, f["uy"]),
                        rho_blocks=block_means(g, f["rho"]), cells=sub, ux=f["ux"][sub], uy=f["uy"][sub],
                        rho=f["rho"][sub])
    print("written", HERE / "steady_mb1024.npz")


if __name__ == "__main__":
    main()
