"""GPU parity of the adsorption step (Shan-Chen pseudopotential force, plain
MRT with the Guo source, bounce-back walls, x-periodic links and the
generalized inlet/outlet) against the reference's gold files and the FP64
oracle.  The 100-step adsorption transient is strongly nonlinear (density
0.11-1.35, |u| up to 0.19); tolerances are stated per test."""
import numpy as np
import pytest
from conftest import load

from mantiis_gb300 import SIM_ADSORPTION, HostGrid, Solver, default_params, generate_disks
from oracle.pyoracle import for_grid
from test_gpu_transport import record

pytestmark = pytest.mark.gpu


def test_adsorption_gold_64(fixture64):
    # test/run_tests.sh adsorption case: dx = 12 nm, 64x64, 100 steps
    p = default_params(dx=12e-9, simulation=SIM_ADSORPTION)
    s = Solver(fixture64["pore"], fixture64["kn"], fixture64["locpore"], p)
    assert s.run(100) == 100
    px = s.pixels()
    umax = np.abs(fixture64["adsorption_ux"]).max()
    e_ux = np.abs(px["ux"] - fixture64["adsorption_ux"]).max() / umax
    e_uy = np.abs(px["uy"] - fixture64["adsorption_uy"]).max() / umax
    e_rho = np.abs(px["rho"] - fixture64["adsorption_rho"]).max() / np.abs(fixture64["adsorption_rho"]).max()
    record("adsorption_gold_64", ux=e_ux, uy=e_uy, rho=e_rho)
    # measured on a GB300: u_x 1.0e-6, u_y 2.3e-6, rho 1.3e-6
    assert e_ux < 1e-5 and e_uy < 2.5e-5 and e_rho < 1.5e-5


def test_adsorption_residuals_vs_oracle(fixture64):
    p = default_params(dx=12e-9, simulation=SIM_ADSORPTION)
    g = HostGrid(fixture64["pore"], fixture64["kn"], fixture64["locpore"], p)
    o = for_grid(g, sim="adsorption", dx=12e-9)
    o.run(60)
    ref = o.residuals()
    s = Solver(fixture64["pore"], fixture64["kn"], fixture64["locpore"], p)
    s.run(60)
    r = s.residuals()
    assert len(r) == 60 and r[0] == 1e-5 == ref[0]
    e = np.abs(r - ref) / ref
    record("adsorption_residuals_64", max_rel=e.max(), median_rel=np.median(e))
    assert np.median(e) < 2e-5  # measured median 1.6e-6 (max 1.4e-5)


def test_exponential_pseudopotential_vs_oracle():
    # the exponential form psi = rho0 (1 - exp(-rho/rho0)) with G = -4.5 and
    # G_ads = -0.5 in the common Shan-Chen convention (weights 1/9, 1/36), initial
    # density 0.5 +- 1e-3.  The reference's force carries -6 G_ff with weights
    # 1/3, 1/12 (18 x the common one) and -G_fs with weights 1/3, 1/12, so
    # G_ff = G / 18 and G_fs = 3 G_ads.
    n = 128
    pore = generate_disks(n, 4, 10, 0.6, 3001)
    kn = np.where(pore == 1, 0.1, 0.0)
    lp = np.where(pore == 1, 7.73, 0.0)
    kw = dict(psi_form=1, rho_psi=0.5, g_ff=-4.5 / 18, g_fs=-1.5)
    p = default_params(dx=1e-9, simulation=SIM_ADSORPTION, rho_init=0.5, fbody=0.0, **kw)
    g = HostGrid(pore, kn, lp, p)
    rng = np.random.default_rng(3)
    rho = 0.5 + rng.uniform(-1e-3, 1e-3, g.n_cells)
    o = for_grid(g, sim="adsorption", dx=1e-9, fbody=0.0, rho_init=rho, **kw)
    o.run(50)
    ref = o.fields()
    s = Solver(pore, kn, lp, p)
    s.set_equilibrium(rho, np.zeros_like(rho), np.zeros_like(rho))
    s.run(50)
    got = s.cells()
    e_rho = np.abs(got["rho"] - ref["rho"]).max() / 0.5
    e_ux = np.abs(got["ux"] - ref["ux"]).max() / max(np.abs(ref["ux"]).max(), 1e-30)
    record("adsorption_exponential_128", rho=e_rho, ux=e_ux)
    # measured rho 5.9e-8; u (no body force: a weak flow of the density
    # noise, relative to its own small maximum) 5.1e-4
    assert e_rho < 6e-7 and e_ux < 5e-3


def test_coupled_run_matches_reference_code(fixture64):
    # the reference's own coupled run (tests/golden/refstate_coupled64.npz):
    # 100 adsorption steps without body force, then regularized MRT + Shan-Chen
    # force + SRBB coupling steps whose velocity residual stays 1
    from mantiis_gb300 import SIM_COUPLED

    st = load("refstate_coupled64.npz")
    p = default_params(dx=12e-9, simulation=SIM_COUPLED)
    s = Solver(fixture64["pore"], fixture64["kn"], fixture64["locpore"], p)
    done = 0
    for step in (100, 101, 130):
        assert s.run(step - done) == step - done
        done = step
        c = s.cells(with_f=True)
        e_f = np.abs(c["f"] - st[f"f_{step}"]).max() / 0.2355
        umax = np.abs(st[f"ux_{step}"]).max()
        e_ux = np.abs(c["ux"] - st[f"ux_{step}"]).max() / umax if step > 100 else 0.0
        e_rho = np.abs(c["rho"] - st[f"rho_{step}"]).max() / np.abs(st[f"rho_{step}"]).max() if step > 100 else 0.0
        record(f"coupled_64_{step}", f=e_f, ux=e_ux, rho=e_rho)
        # measured (worst step): f 3.3e-6, u_x 1.1e-6, rho 1.2e-6
        assert e_f < 3.5e-5 and e_ux < 1.2e-5 and e_rho < 1.5e-5
    r = s.residuals()
    assert len(r) == 130 and np.allclose(r[100:], 1.0)


def test_config3_full_size_vs_oracle():
    # config 3 at full size: 512x512 seeded disk image, porosity 0.6,
    # psi = rho0 (1 - exp(-rho/rho0)), G = -4.5, G_ads = -0.5 (common
    # convention; G_ff = G / 18, G_fs = 3 G_ads in the reference's), initial
    # density 0.5 +- 1e-3, 200 steps: the density field (adsorbed layers) and the
    # total mass against the FP64 oracle
    import os
    from mantiis_gb300 import workloads

    img = workloads.config3(0)
    kw = dict(psi_form=1, rho_psi=0.5, g_ff=-4.5 / 18, g_fs=-1.5)
    p = default_params(dx=img["dx"], simulation=SIM_ADSORPTION, rho_init=0.5, fbody=0.0, tol=0.0, **kw)
    g = HostGrid(img["pore"], img["kn"], img["locpore"], p)
    rng = np.random.default_rng(3000)
    rho = 0.5 + rng.uniform(-1e-3, 1e-3, g.n_cells)
    o = for_grid(g, sim="adsorption", dx=img["dx"], fbody=0.0, rho_init=rho, threads=os.cpu_count() or 1, **kw)
    o.run(200)
    ref = o.fields()
    s = Solver(img["pore"], img["kn"], img["locpore"], p)
    s.set_equilibrium(rho, np.zeros_like(rho), np.zeros_like(rho))
    s.run(200)
    got = s.cells()
    e_rho = np.abs(got["rho"] - ref["rho"]).max() / np.abs(ref["rho"]).max()
    m_gpu, m_ref, m0 = got["rho"].sum(), ref["rho"].sum(), rho.sum()
    record("config3_512_200", rho=e_rho, mass=abs(m_gpu - m_ref) / m_ref, drift_ref=abs(m_ref - m0) / m0,
           rho_span=float(ref["rho"].max() - ref["rho"].min()))
    # measured rho 1.5e-7, mass 1.4e-12
    assert e_rho < 1.5e-6 and abs(m_gpu - m_ref) / m_ref < 1.5e-11


def test_adsorption_disk_image_vs_reference_code():
    # a 128x128 disk image against the reference's own adsorption run
    # (refstate_adsorption128_100.npz): PR-EOS psi, BB walls, inlet/outlet, 100 steps
    st = load("refstate_adsorption128_100.npz")
    p = default_params(dx=12e-9, simulation=SIM_ADSORPTION, tol=0.0)
    s = Solver(st["pore"].astype(np.int32), st["kn"], st["locpore"], p)
    assert s.run(100) == 100
    c = s.cells()
    umax = np.abs(st["ux"]).max()
    e_ux = np.abs(c["ux"] - st["ux"]).max() / umax
    e_rho = np.abs(c["rho"] - st["rho"]).max() / np.abs(st["rho"]).max()
    record("adsorption_disk128_vs_reference_100", ux=e_ux, rho=e_rho)
    assert e_ux < 1e-5 and e_rho < 1.5e-5  # measured u_x 9.0e-7, rho 1.4e-6


@pytest.mark.parametrize("call", ["run", "advance", "advance_graph"])
def test_persistent_adsorption_engine_bit_identical(call):
    # the cooperative launch over many steps (engine 1, the default) and the
    # launches per pass (engine 0) step the same arithmetic: bit-identical
    # states and, for run / advance, the same per-step residuals; on a 512^2
    # config-3 image from a perturbed state, odd step counts (both parities)
    from mantiis_gb300 import workloads

    img = workloads.config3(0)
    kw = dict(psi_form=1, rho_psi=0.5, g_ff=-4.5 / 18, g_fs=-1.5)
    p = default_params(dx=img["dx"], simulation=SIM_ADSORPTION, rho_init=0.5, fbody=0.0, tol=0.0, **kw)
    rng = np.random.default_rng(3001)
    out = {}
    for engine in (0, 1):
        s = Solver(img["pore"], img["kn"], img["locpore"], p)
        s.set_engine(engine)
        n = s.info["n_cells"]
        rho = 0.5 + rng.uniform(-1e-3, 1e-3, n) if engine == 0 else out[0][2]
        s.set_equilibrium(rho, np.zeros(n), np.zeros(n))
        if call == "run":
            assert s.run(37) == 37
            assert s.run(1000) == 1000
        elif call == "advance":
            s.advance(37)
            s.advance(1000)
        else:
            s.advance_graph(37)
            s.advance_graph(1000)
        s.sync()
        launches = s.launches
        out[engine] = (s.cells(with_f=True)["f"], s.residuals(), rho, launches)
        s.close()
    assert np.array_equal(out[0][0], out[1][0])
    if call != "advance_graph":
        assert len(out[0][1]) == len(out[1][1]) == 1037
        assert np.array_equal(out[0][1], out[1][1])
    # one launch per call (and its barrier reset) against four per step
    assert out[1][3] < out[0][3] / 100
