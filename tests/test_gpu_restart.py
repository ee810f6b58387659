"""Restart from saved populations (mgpu_set_distributions): a run stopped after
k steps, downloaded (mgpu_download_cells, or the f.txt pixel layout of
mgpu_download_pixels on a single-block grid) and restarted in a fresh context
at time step k continues as the uninterrupted run, with the same time counter.
The state is FP32 deviations from w rho0; the FP64 populations f = w rho0 + df
that are saved resolve them to ~1e-17 absolute, so a deviation below ~1e-9 can
come back one FP32 ulp off: populations agree to 1e-13 (bit for bit where no
deviation is that small); residuals (sums of FP32 |u| changes, FP64 atomics)
to 1e-6 relative."""
import numpy as np
import pytest
from conftest import load

from mantiis_gb300 import SIM_ADSORPTION, SIM_COUPLED, MantiisError, Solver, default_params, generate_disks

pytestmark = pytest.mark.gpu


def restart_pair(make, total, split, layout="cells"):
    a = make()
    assert a.run(total) == total
    b = make()
    assert b.run(split) == split
    saved = b.cells(with_f=True)["f"] if layout == "cells" else b.pixels(with_f=True)["f"]
    c = make()
    c.set_distributions(saved, layout=layout, t=split)
    assert c.time == split
    assert c.run(total - split) == total - split
    assert c.time == a.time == total
    fa, fc = a.cells(with_f=True)["f"], c.cells(with_f=True)["f"]
    return a, c, np.abs(fa - fc).max()


@pytest.mark.parametrize("layout", ["cells", "pixels"])
def test_restart_single_block_transport(fixture64, layout):
    p = default_params(dx=1e-9, tol=0.0)
    make = lambda: Solver(fixture64["pore"], fixture64["kn"], fixture64["locpore"], p)  # noqa: E731
    a, c, err = restart_pair(make, 60, 25, layout)
    assert err <= 1e-13
    # residuals 26..60 of the uninterrupted run
    ra, rc = a.residuals(), c.residuals()
    assert len(rc) == 35 and np.allclose(rc, ra[25:], rtol=1e-6, atol=0)


def test_restart_multiblock_three_levels():
    pore = generate_disks(128, 4, 16, 0.6, 77, open_x_edges=True)
    kn = np.where(pore == 1, 0.2, 0.0)
    lp = np.where(pore == 1, 7.73, 0.0)
    p = default_params(dx=1e-9, tol=0.0, multiblock=1, max_allowed_level=3)
    make = lambda: Solver(pore, kn, lp, p)  # noqa: E731
    assert make().info["max_level"] == 3
    a, c, err = restart_pair(make, 40, 17)
    assert err <= 1e-13
    assert np.allclose(c.residuals(), a.residuals()[17:], rtol=1e-9, atol=0)


def test_restart_adsorption(fixture64):
    p = default_params(dx=12e-9, simulation=SIM_ADSORPTION, tol=0.0)
    make = lambda: Solver(fixture64["pore"], fixture64["kn"], fixture64["locpore"], p)  # noqa: E731
    a, c, err = restart_pair(make, 50, 20)
    assert err <= 1e-13
    ra, rc = a.residuals()[20:], c.residuals()
    assert len(rc) == 30
    # a restarted run begins like a fresh one: its first density residual
    # compares the restart state with itself (the reference's 1e-5 floor)
    assert rc[0] == 1e-5 and np.allclose(rc[1:], ra[1:], rtol=1e-9, atol=0)


@pytest.mark.parametrize("split", [100, 110])
def test_restart_coupled(split):
    fx = load("fixture64.npz")
    p = default_params(dx=12e-9, simulation=SIM_COUPLED, tol=0.0)
    make = lambda: Solver(fx["pore"], fx["kn"], fx["locpore"], p)  # noqa: E731
    a, c, err = restart_pair(make, 125, split)
    assert err <= 1e-13


def test_restart_rejects_bad_input(fixture64):
    s = Solver(fixture64["pore"], fixture64["kn"], fixture64["locpore"], default_params(dx=1e-9))
    f = s.cells(with_f=True)["f"]
    with pytest.raises(ValueError):
        s.set_distributions(f[:-1], layout="cells")
    bad = f.copy()
    bad[3, 4] = np.nan
    with pytest.raises(MantiisError):
        s.set_distributions(bad, layout="cells")
    with pytest.raises(MantiisError):
        s.set_distributions(f, layout="cells", t=-1)
