"""The FP64 CPU oracle is pinned against the reference's golden outputs and
against the reference's own multi-block code (fixtures made by
tests/golden/make_golden.py from oracle/_ref)."""
import numpy as np
import pytest
from conftest import load

from mantiis_gb300 import HostGrid, default_params
from oracle.pyoracle import for_grid


def pixels(grid, values, n):
    out = np.zeros(n * n)
    out[grid.cells["y"] * n + grid.cells["x"]] = values
    return out.reshape(n, n)


@pytest.mark.parametrize("sim,dx", [("transport", 1e-9), ("adsorption", 12e-9)])
def test_oracle_reproduces_reference_gold(fixture64, sim, dx):
    # run_tests.sh: 64x64, single block, 100 steps, max abs difference <= 1e-10
    g = HostGrid(fixture64["pore"], fixture64["kn"], fixture64["locpore"], default_params(dx=dx))
    o = for_grid(g, sim=sim, dx=dx)
    assert o.run(100) == 100
    f = o.fields()
    for name in ("ux", "uy", "rho"):
        err = np.abs(pixels(g, f[name], 64) - fixture64[f"{sim}_{name}"]).max()
        assert err <= 1e-10, (sim, name, err)


@pytest.mark.parametrize("case", ["channel64", "block64", "block64b"])
def test_oracle_multiblock_matches_reference_code(case):
    ref = load(f"refgrid_{case}.npz")
    st = load(f"refstate_{case}.npz")
    g = HostGrid(ref["img_pore"], ref["img_kn"], ref["img_locpore"], default_params(multiblock=1))
    assert g.max_level == 2
    o = for_grid(g, sim="transport", dx=1e-9)
    done = 0
    for step in (1, 2, 50):
        o.run(step - done)
        done = step
        f = o.fields()
        for name in ("rho", "ux", "uy"):
            err = np.abs(f[name] - st[f"{name}_{step}"]).max()
            assert err <= 1e-12, (case, step, name, err)
        assert np.abs(f["f"] - st[f"f_{step}"]).max() <= 1e-12
    assert np.allclose(o.residuals(), st["residuals_50"], rtol=1e-9, atol=0)


def test_oracle_three_levels_match_reference_code():
    # the reference's own three-level run (depth limit raised to 3, oracle/_ref
    # ref_driver3) on a 128x128 block geometry whose interpolation stays inside
    # the reference's arrays: the oracle on its own grid tables, 50 coarse steps
    from oracle.pygrid import GridTables

    ref = load("refgrid_block128_l3.npz")
    st = load("refstate_block128_l3.npz")
    g = GridTables(ref["img_pore"], ref["img_kn"], ref["img_locpore"], multiblock=True, max_allowed_level=3)
    assert g.max_level == 3 and g.n_cells == int(ref["n_cells"])
    assert np.array_equal(g.cells["conn"], ref["conn"]) and np.array_equal(g.fine_rows, ref["fine_rows"])
    o = for_grid(g, sim="transport", dx=1e-9)
    done = 0
    for step in (1, 2, 50):
        o.run(step - done)
        done = step
        f = o.fields()
        for name in ("rho", "ux", "uy"):
            err = np.abs(f[name] - st[f"{name}_{step}"]).max()
            assert err <= 1e-12, (step, name, err)
        assert np.abs(f["f"] - st[f"f_{step}"]).max() <= 1e-12
    assert np.allclose(o.residuals(), st["residuals_50"], rtol=1e-9, atol=0)


def test_oracle_break_semantics(fixture64):
    # the loop stops right after the first step whose residual is below tol
    g = HostGrid(fixture64["pore"], fixture64["kn"], fixture64["locpore"], default_params(dx=1e-9))
    o = for_grid(g, sim="transport", dx=1e-9)
    o.run(40)
    r = o.residuals()
    tol = float(r[29]) * 1.0000001  # first residual below tol is that of step 30
    assert (r[:29] > tol).all()
    o2 = for_grid(g, sim="transport", dx=1e-9, tol=tol)
    assert o2.run(100, break_on_tol=True) == 30


def test_oracle_coupled_run_matches_reference_code(fixture64):
    # refstate_coupled64.npz: the reference's own coupled run (oracle/_ref,
    # tests/golden/make_golden.py); at step 100 the run resets u and rho, so
    # only f is compared there
    from mantiis_gb300 import HostGrid, default_params
    from oracle.pyoracle import for_grid

    st = load("refstate_coupled64.npz")
    g = HostGrid(fixture64["pore"], fixture64["kn"], fixture64["locpore"], default_params(dx=12e-9))
    o = for_grid(g, sim="coupled", dx=12e-9)
    done = 0
    for step in (100, 101, 130):
        o.run(step - done, break_on_tol=True)
        done = step
        f = o.fields()
        assert np.abs(f["f"] - st[f"f_{step}"]).max() < 1e-10
        if step > 100:
            assert np.abs(f["ux"] - st[f"ux_{step}"]).max() < 1e-10
            assert np.abs(f["rho"] - st[f"rho_{step}"]).max() < 1e-10
    assert np.allclose(o.residuals()[100:], 1.0)


def test_oracle_matches_reference_on_disk_image():
    # the config-1 disk image (128x128, single block, Kn ~0.1): the reference's
    # own code (refstate_config1_200.npz) after 200 steps
    st = load("refstate_config1_200.npz")
    pore = st["pore"].astype(np.int32)
    dx = float(st["dx"])
    g = HostGrid(pore, st["kn"], st["locpore"], default_params(dx=dx))
    o = for_grid(g, sim="transport", dx=dx)
    assert o.run(200) == 200
    f = o.fields()
    for name in ("rho", "ux", "uy"):
        scale = np.abs(st[name]).max()
        assert np.abs(f[name] - st[name]).max() <= 1e-12 * scale, name
    assert np.allclose(o.residuals(), st["residuals"], rtol=1e-9, atol=0)


def test_oracle_adsorption_matches_reference_on_disk_image():
    # PR-EOS pseudopotential, bounce-back walls and the inlet/outlet on a 128x128
    # seeded disk image at dx = 12 nm: the reference's own run after 100 steps
    from mantiis_gb300 import SIM_ADSORPTION

    st = load("refstate_adsorption128_100.npz")
    p = default_params(dx=12e-9, simulation=SIM_ADSORPTION)
    g = HostGrid(st["pore"].astype(np.int32), st["kn"], st["locpore"], p)
    o = for_grid(g, sim="adsorption", dx=12e-9)
    assert o.run(100) == 100
    f = o.fields()
    for name in ("rho", "ux", "uy"):
        assert np.abs(f[name] - st[name]).max() <= 1e-12 * np.abs(st[name]).max(), name
    assert np.allclose(o.residuals(), st["residuals"], rtol=1e-9, atol=0)


VARIANTS_SB = [(2, 1), (1, 2), (0, 0), (1, 1), (0, 2), (0, 1)]
VARIANTS_MB = [(2, 1), (0, 2), (0, 1)]


@pytest.mark.parametrize("collision,wall,multiblock", [(c, w, 0) for c, w in VARIANTS_SB] +
                         [(c, w, 1) for c, w in VARIANTS_MB])
def test_oracle_variants_match_reference_code(fixture64, collision, wall, multiblock):
    # refstate_variants.npz: the reference's own runs with collision_method
    # 0 BGK / 1 MRT / 2 regularized MRT and wall_boundary 0 BB / 1 MDBB / 2 SRBB
    # (include/coreLB.hpp:678-792, 859-967): single block on the 64x64 test
    # image (100 steps), multi-block on the block64 geometry (50 steps)
    st = load("refstate_variants.npz")
    key = f"{'mb' if multiblock else 'sb'}_c{collision}_w{wall}"
    if multiblock:
        ref = load("refgrid_block64.npz")
        img, steps = (ref["img_pore"], ref["img_kn"], ref["img_locpore"]), 50
    else:
        img, steps = (fixture64["pore"], fixture64["kn"], fixture64["locpore"]), 100
    g = HostGrid(*img, default_params(dx=1e-9, multiblock=multiblock, collision=collision, wall=wall))
    o = for_grid(g, sim="transport", dx=1e-9, collision=collision, wall=wall)
    assert o.run(steps) == steps
    f = o.fields()
    # populations agree to rounding (measured <= 1e-16); the velocities of
    # ~1e-6 are differences of O(0.03) populations, so that rounding shows at
    # 1e-10 of max|u| (measured 8e-11 .. 2.4e-10)
    assert np.abs(f["f"] - st[f"{key}_f"].reshape(-1, 9)).max() <= 1e-15
    assert np.abs(f["rho"] - st[f"{key}_rho"]).max() <= 1e-14 * np.abs(st[f"{key}_rho"]).max()
    for name in ("ux", "uy"):
        scale = np.abs(st[f"{key}_{name}"]).max()
        assert np.abs(f[name] - st[f"{key}_{name}"]).max() <= 2e-9 * scale, name


def test_solid_pixels_on_the_seam_lose_mass_under_the_reference_order():
    # A 128^2 config-4 draw whose x-edge columns the generator's fill made partly
    # solid (config4_steady(186) before its fallback to a 3-column margin: the
    # last of its 400 seeds): under the reference's order a wall link's share at
    # the seam lands in a population that the x-periodic copy then overwrites,
    # and the FP64 restatement of the reference's step loses ~1 % of the mass per
    # 1000 steps while its mean flow runs against the force.  config4_steady
    # now draws such images again, and its image 186 conserves mass.
    import os

    from mantiis_gb300 import workloads
    from mantiis_gb300.surrogate import solver_params

    rng = np.random.default_rng(4500 + 186)
    n = int(rng.choice([128, 256, 512, 1024, 2048]))
    phi = rng.uniform(0.45, 0.75)
    assert int(rng.integers(1, 3)) == 1
    kn = float(np.exp(rng.uniform(np.log(0.01), np.log(0.12))))
    old = workloads.image(n, 2, 4, phi, kn, 4500 + 186 + 100000 * 399, open_x_edges=True)
    old["levels"] = 1
    assert not old["pore"][1:-1][:, [0, 1, n - 2, n - 1]].all()

    def drift_and_flow(d):
        g = HostGrid(d["pore"], d["kn"], d["locpore"], solver_params(d))
        o = for_grid(g, sim="transport", dx=d["dx"], threads=os.cpu_count() or 1)
        keep = g.cells["is_buffer"] == 0
        o.run(1000)
        m0 = o.fields()["rho"][keep].sum()
        o.run(3000)
        f = o.fields()
        return (f["rho"][keep].sum() - m0) / m0, f["ux"][keep].mean()

    drift, ux = drift_and_flow(old)
    assert ux < 0 and drift < -0.02
    new = workloads.config4_steady(186)
    assert new["pore"][1:-1][:, [0, 1, n - 2, n - 1]].all()
    drift, ux = drift_and_flow(new)
    assert ux > 0 and abs(drift) < 1e-10


@pytest.mark.parametrize("index", [83, 149, 186, 190])
def test_config4_steady_keeps_the_seam_void(index):
    # the four of the first 256 config-4 steady draws whose 400 seeds all had
    # solid pixels on the seam are drawn with disks kept off three columns
    from mantiis_gb300 import workloads

    d = workloads.config4_steady(index)
    n = d["pore"].shape[0]
    assert d["pore"][1:-1][:, [0, 1, n - 2, n - 1]].all()
