"""GPU parity of the transport step (regularized MRT + SRBB + x-periodic, the
reference's default path) against the reference's gold files, the reference's
own multi-block code and the FP64 oracle.

Tolerances (FP32 deviation storage vs the reference's FP64): velocities are
compared relative to the field's largest magnitude, densities relative to the
inlet density; the bounds are written in each test.
"""
import json
import os

import numpy as np
import pytest
from conftest import ROOT, load

from mantiis_gb300 import HostGrid, Solver, default_params, generate_disks
from oracle.pyoracle import for_grid

pytestmark = pytest.mark.gpu

REPORT = {}


def record(name, **kw):
    REPORT[name] = {k: float(v) for k, v in kw.items()}
    out = os.environ.get("MANTIIS_TEST_REPORT")
    if out:
        with open(out, "w") as fh:
            json.dump(REPORT, fh, indent=1)


def rel_err(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


def test_transport_gold_64(fixture64):
    # test/run_tests.sh transport case: 64x64 single block, 100 steps
    s = Solver(fixture64["pore"], fixture64["kn"], fixture64["locpore"], default_params(dx=1e-9))
    assert s.run(100) == 100
    px = s.pixels()
    e_ux = rel_err(px["ux"], fixture64["transport_ux"])
    e_uy = np.abs(px["uy"] - fixture64["transport_uy"]).max() / np.abs(fixture64["transport_ux"]).max()
    e_rho = np.abs(px["rho"] - fixture64["transport_rho"]).max() / 0.2355
    record("transport_gold_64", ux=e_ux, uy=e_uy, rho=e_rho)
    # measured on a GB300: u_x 4.0e-7, u_y 2.6e-7, rho 7.3e-13
    assert e_ux < 4e-6 and e_uy < 3e-6 and e_rho < 1e-11
    assert s.launches > 0


def test_transport_residuals_and_break(fixture64):
    g = HostGrid(fixture64["pore"], fixture64["kn"], fixture64["locpore"], default_params(dx=1e-9))
    o = for_grid(g, sim="transport", dx=1e-9)
    o.run(300)
    ref = o.residuals()
    s = Solver(fixture64["pore"], fixture64["kn"], fixture64["locpore"], default_params(dx=1e-9))
    s.run(300)
    r = s.residuals()
    assert len(r) == 300
    e = np.abs(r - ref) / ref
    record("transport_residuals_64", max_rel=e.max(), median_rel=np.median(e))
    assert np.median(e) < 2e-5  # measured median 2.3e-6 (max 7.6e-5, late residuals ~1e-9)
    # break: tolerance just above the residual of step 250 in the oracle run
    tol = float(ref[249]) * 1.0001
    first = int(np.argmax(ref < tol)) + 1
    s2 = Solver(fixture64["pore"], fixture64["kn"], fixture64["locpore"], default_params(dx=1e-9, tol=tol))
    done = s2.run(1000)
    record("transport_break_64", oracle_step=first, gpu_step=done)
    assert abs(done - first) <= 2
    assert s2.time == done - 1


@pytest.mark.parametrize("case", ["channel64", "block64", "block64b"])
def test_multiblock_matches_reference_code(case):
    ref = load(f"refgrid_{case}.npz")
    st = load(f"refstate_{case}.npz")
    s = Solver(ref["img_pore"], ref["img_kn"], ref["img_locpore"], default_params(multiblock=1))
    assert s.info["max_level"] == 2
    done = 0
    for step in (1, 2, 50):
        s.advance(step - done)
        done = step
        c = s.cells(with_f=True)
        e_ux = rel_err(c["ux"], st[f"ux_{step}"])
        e_rho = np.abs(c["rho"] - st[f"rho_{step}"]).max() / 0.2355
        e_f = np.abs(c["f"] - st[f"f_{step}"]).max() / 0.2355
        record(f"multiblock_{case}_{step}", ux=e_ux, rho=e_rho, f=e_f)
        # measured (worst case and step): u_x 5.5e-7, rho 1.1e-12, f 4.7e-13
        assert e_ux < 5e-6 and e_rho < 1e-11 and e_f < 5e-12


def test_three_levels_match_reference_code():
    # the reference's own three-level run (depth limit raised to 3, oracle/_ref
    # ref_driver3) on a 128x128 block geometry whose interpolation stays inside
    # the reference's arrays (refstate_block128_l3.npz): 1, 2 and 50 coarse steps
    ref = load("refgrid_block128_l3.npz")
    st = load("refstate_block128_l3.npz")
    s = Solver(ref["img_pore"], ref["img_kn"], ref["img_locpore"], default_params(multiblock=1, max_allowed_level=3))
    assert s.info["max_level"] == 3
    done = 0
    for step in (1, 2, 50):
        s.advance(step - done)
        done = step
        c = s.cells(with_f=True)
        e_ux = rel_err(c["ux"], st[f"ux_{step}"])
        e_rho = np.abs(c["rho"] - st[f"rho_{step}"]).max() / 0.2355
        e_f = np.abs(c["f"] - st[f"f_{step}"]).max() / 0.2355
        record(f"multiblock_block128_l3_{step}", ux=e_ux, rho=e_rho, f=e_f)
        # measured (worst step): u_x 2.8e-7, rho 2.4e-10, f 2.2e-10 (FP32
        # deviations: the coarse level's larger velocities)
        assert e_ux < 3e-6 and e_rho < 2.5e-9 and e_f < 2.5e-9


def oracle_pair(pore, steps, multiblock=0, levels=2, dx=1e-9, kn=None, lp=None, edge_fine=0):
    n = pore.shape[0]
    kn = np.where(pore == 1, 0.1, 0.0) if kn is None else kn
    lp = np.where(pore == 1, 7.73, 0.0) if lp is None else lp
    p = default_params(multiblock=multiblock, max_allowed_level=levels, dx=dx, edge_fine=edge_fine)
    g = HostGrid(pore, kn, lp, p)
    o = for_grid(g, sim="transport", dx=dx)
    o.run(steps)
    s = Solver(pore, kn, lp, p)
    s.advance(steps)
    return o.fields(), s.cells(with_f=True), s


def test_multiblock_test_image_vs_oracle(fixture64):
    # the reference reads outside its arrays here; the oracle applies the same
    # defined rule as the GPU (nominal node position, parent's populations)
    ref, got, s = oracle_pair(fixture64["pore"], 60, multiblock=1, kn=fixture64["kn"], lp=fixture64["locpore"])
    e = rel_err(got["ux"], ref["ux"])
    record("multiblock_testimage_vs_oracle", ux=e)
    assert e < 3e-6  # measured 2.2e-7


# The reference's multi-block scheme is not stable on every image: coarse cells
# facing finer ones across the x-periodic boundary (no buffer cells there) and,
# with three levels, level-2 buffer cells stepped twice between refreshes lose
# populations, and the FP64 oracle diverges as well.  The multi-block cases are
# therefore compared with edge_fine on and, for three levels, over few steps.
@pytest.mark.parametrize("n,levels,steps", [(128, 1, 200), (256, 2, 200), (256, 3, 8)])
def test_disk_images_vs_oracle(n, levels, steps):
    pore = generate_disks(n, 4 if n == 128 else 6, 10 if n == 128 else 30, 0.65, 1000 + n + levels)
    ref, got, s = oracle_pair(pore, steps, multiblock=int(levels > 1), levels=max(levels, 2), edge_fine=int(levels > 1))
    assert s.info["max_level"] == levels
    e = rel_err(got["ux"], ref["ux"])
    e_rho = np.abs(got["rho"] - ref["rho"]).max() / 0.2355
    record(f"disks_{n}_L{levels}_vs_oracle", ux=e, rho=e_rho)
    # measured: u_x 1.9e-7 / 1.2e-7 / 3.3e-7, rho 5.8e-9 / 8.7e-9 / 1.3e-7 (1, 2, 3 levels)
    assert e < 3e-6 and e_rho < {1: 6e-8, 2: 9e-8, 3: 1.5e-6}[levels]


def test_graph_path_matches_stepwise(fixture64):
    p = default_params(dx=1e-9)
    a = Solver(fixture64["pore"], fixture64["kn"], fixture64["locpore"], p)
    b = Solver(fixture64["pore"], fixture64["kn"], fixture64["locpore"], p)
    a.advance(41)
    b.advance_graph(41)
    b.sync()
    ca, cb = a.cells(with_f=True), b.cells(with_f=True)
    assert np.array_equal(ca["f"], cb["f"])


def test_deterministic(fixture64):
    p = default_params(dx=1e-9, multiblock=1)
    runs = []
    for _ in range(2):
        s = Solver(fixture64["pore"], fixture64["kn"], fixture64["locpore"], p)
        s.advance(30)
        runs.append(s.cells(with_f=True)["f"])
    assert np.array_equal(runs[0], runs[1])


@pytest.mark.parametrize("engine,group", [(0, 0), (1, 0), (1, 2)])
def test_batch_matches_single_contexts(fixture64, engine, group):
    # a batch of images with 1, 2 and 3 levels steps each exactly like its own
    # context: per-image launches on concurrent streams (engine 0) and the
    # persistent launch over all images (engine 1, images interleaved all at
    # once or two at a time)
    from mantiis_gb300 import Batch

    imgs = [(fixture64["pore"], fixture64["kn"], fixture64["locpore"], default_params(dx=1e-9))]
    for n, levels, seed in ((128, 2, 11), (256, 3, 12)):
        pore = generate_disks(n, 4 if n == 128 else 6, 10 if n == 128 else 30, 0.65, seed)
        kn = np.where(pore == 1, 0.1, 0.0)
        lp = np.where(pore == 1, 7.73, 0.0)
        imgs.append((pore, kn, lp, default_params(multiblock=1, max_allowed_level=levels, edge_fine=1)))
    solo = [Solver(*a) for a in imgs]
    grouped = [Solver(*a) for a in imgs]
    for s in solo:
        s.advance(9)
    b = Batch(grouped)
    b.set_engine(engine, group)
    b.advance(4)   # the first step from the initial state, then a graph of two, then one
    b.advance(5)
    b.sync()
    for s, g in zip(solo, grouped):
        assert g.time == s.time
        assert np.array_equal(s.cells(with_f=True)["f"], g.cells(with_f=True)["f"])
    obs = b.observables()
    for s, o in zip(solo, obs):
        # same state; the FP64 block sums are added atomically (order varies)
        assert abs(o["mean_ux"] - s.observables()["mean_ux"]) <= 1e-12 * abs(o["mean_ux"])
    assert b.launches > 0


# collision 0 BGK, 1 MRT, 2 regularized MRT; wall 0 BB, 1 MDBB, 2 SRBB
# (include/coreLB.hpp:678-792, 859-967): the variants the reference selects with
# Settings::collision_method / wall_boundary, checked against the FP64 oracle
@pytest.mark.parametrize("collision,wall,multiblock", [(2, 1, 0), (1, 2, 0), (0, 0, 0), (1, 1, 0), (2, 1, 1), (0, 2, 1)])
def test_collision_and_wall_variants_vs_oracle(fixture64, collision, wall, multiblock):
    p = default_params(dx=1e-9, collision=collision, wall=wall, multiblock=multiblock)
    g = HostGrid(fixture64["pore"], fixture64["kn"], fixture64["locpore"], p)
    o = for_grid(g, sim="transport", dx=1e-9, collision=collision, wall=wall)
    o.run(60)
    ref = o.fields()
    s = Solver(fixture64["pore"], fixture64["kn"], fixture64["locpore"], p)
    s.advance(60)
    got = s.cells(with_f=True)
    e = rel_err(got["ux"], ref["ux"])
    e_f = np.abs(got["f"] - ref["f"]).max() / 0.2355
    record(f"variant_c{collision}_w{wall}_mb{multiblock}", ux=e, f=e_f)
    # measured: u_x <= 4.6e-7; f 2.1e-13 single block, 6.6e-8 on the multi-block
    # test image (whose fine-buffer parents meet walls)
    assert e < 5e-6 and e_f < (7e-7 if multiblock else 3e-12)


VARIANTS_SB = [(2, 1), (1, 2), (0, 0), (1, 1), (0, 2), (0, 1)]
VARIANTS_MB = [(2, 1), (0, 2), (0, 1)]


@pytest.mark.parametrize("collision,wall,multiblock", [(c, w, 0) for c, w in VARIANTS_SB] +
                         [(c, w, 1) for c, w in VARIANTS_MB])
def test_variants_vs_reference_code(fixture64, collision, wall, multiblock):
    # BGK / MRT collisions and MDBB / BB walls against the reference's own runs
    # (refstate_variants.npz, oracle/_ref): single block on the 64x64 test image
    # for 100 steps, multi-block on the block64 geometry for 50 steps
    st = load("refstate_variants.npz")
    key = f"{'mb' if multiblock else 'sb'}_c{collision}_w{wall}"
    if multiblock:
        ref = load("refgrid_block64.npz")
        img, steps = (ref["img_pore"], ref["img_kn"], ref["img_locpore"]), 50
    else:
        img, steps = (fixture64["pore"], fixture64["kn"], fixture64["locpore"]), 100
    s = Solver(*img, default_params(dx=1e-9, multiblock=multiblock, collision=collision, wall=wall, tol=0.0))
    assert s.run(steps) == steps
    got = s.cells(with_f=True)
    e_ux = rel_err(got["ux"], st[f"{key}_ux"])
    e_uy = np.abs(got["uy"] - st[f"{key}_uy"]).max() / np.abs(st[f"{key}_ux"]).max()
    e_f = np.abs(got["f"] - st[f"{key}_f"].reshape(-1, 9)).max() / 0.2355
    record(f"variant_ref_{key}", ux=e_ux, uy=e_uy, f=e_f)
    # measured on a GB300: u_x <= 6.5e-7, u_y <= 4.6e-7, f <= 5.0e-13
    assert e_ux < 7e-6 and e_uy < 5e-6 and e_f < 5e-12


def test_plain_paths_agree_and_autotune():
    # the TMA pipeline, the direct 32x8 tiles and the direct 8x4 warp tiles run
    # the same arithmetic on the same slots: bit-identical states; plain_path -1
    # times all three and keeps the fastest
    pore = generate_disks(256, 6, 20, 0.6, 77, open_x_edges=True)
    kn = np.where(pore == 1, 0.1, 0.0)
    lp = np.where(pore == 1, 7.73, 0.0)
    runs = {}
    for path in (0, 1, 2, -1):
        s = Solver(pore, kn, lp, default_params(plain_path=path, multiblock=1, edge_fine=1))
        s.advance(20)
        runs[path] = (s.cells(with_f=True)["f"], s.info)
    assert [runs[k][1]["plain_path"] for k in (0, 1, 2)] == [0, 1, 2]
    assert np.array_equal(runs[0][0], runs[1][0])
    assert np.array_equal(runs[0][0], runs[2][0])
    assert np.array_equal(runs[0][0], runs[-1][0])
    us = runs[-1][1]["autotune_us"]
    assert min(us) > 0
    assert runs[-1][1]["plain_path"] == int(np.argmin(us))
    record("autotune_256", direct_us=us[0], tma_us=us[1], direct8x4_us=us[2])


@pytest.mark.parametrize("sim", ["transport", "adsorption"])
def test_advance_residuals_equal_run(fixture64, sim):
    # mgpu_advance with a residual every step (pairs of steps from a CUDA graph)
    # records the residuals mgpu_run records (FP64 atomic sums: 1e-12)
    from mantiis_gb300 import SIM_ADSORPTION

    kw = dict(dx=12e-9, simulation=SIM_ADSORPTION) if sim == "adsorption" else dict(dx=1e-9)
    a = Solver(fixture64["pore"], fixture64["kn"], fixture64["locpore"], default_params(tol=0.0, **kw))
    b = Solver(fixture64["pore"], fixture64["kn"], fixture64["locpore"], default_params(tol=0.0, check_every=1, **kw))
    assert a.run(31) == 31
    b.advance(31)
    b.sync()
    ra, rb = a.residuals(), b.residuals()
    n = min(len(ra), len(rb))
    assert n >= 30
    assert np.allclose(ra[:n], rb[:n], rtol=1e-12, atol=0)
    assert np.array_equal(a.cells(with_f=True)["f"], b.cells(with_f=True)["f"])


def test_config2_full_size_vs_oracle():
    # the benchmark's own workload at full size: a 1024x1024 config-2 image, 3
    # levels, edge_fine, 6 coarse steps on the GPU against the FP64 oracle
    # (all host cores); populations relative to rho_in, u_x relative to its max
    import os
    from mantiis_gb300 import workloads

    img = workloads.config2(0)
    p = default_params(multiblock=1, max_allowed_level=3, dx=img["dx"], edge_fine=1)
    g = HostGrid(img["pore"], img["kn"], img["locpore"], p)
    o = for_grid(g, sim="transport", dx=img["dx"], threads=os.cpu_count() or 1)
    o.run(6)
    ref = o.fields()
    s = Solver(img["pore"], img["kn"], img["locpore"], p)
    assert s.info["max_level"] == 3
    s.advance(6)
    got = s.cells(with_f=True)
    rho_in = s.info["rho_in"]
    e_f = np.abs(got["f"].reshape(-1) - np.asarray(ref["f"]).reshape(-1)).max() / rho_in
    e_ux = rel_err(got["ux"], ref["ux"])
    record("config2_1024_vs_oracle_6", f=e_f, ux=e_ux)
    assert e_f < 6e-7 and e_ux < 2e-6  # measured f 6.1e-8, u_x 1.7e-7


def test_config1_permeability_vs_oracle():
    # config 1 (128x128 seeded disks, radii U[4,10], porosity 0.65, Kn ~0.1,
    # single block) for its Nt = 5000 steps: the permeability k = <u_x> nu / F
    # of the GPU run within 1e-5 of the FP64 oracle's
    import os
    from mantiis_gb300 import workloads

    img = workloads.config1(0)
    p = default_params(dx=img["dx"], tol=0.0)
    g = HostGrid(img["pore"], img["kn"], img["locpore"], p)
    o = for_grid(g, sim="transport", dx=img["dx"], fbody=p.fbody, threads=os.cpu_count() or 1)
    o.run(5000)
    ref = o.fields()
    s = Solver(img["pore"], img["kn"], img["locpore"], p)
    s.advance(5000)
    k_gpu = s.observables()["permeability"]
    n = img["pore"].shape[0]
    nu = (s.info["tau_mean"] - 0.5) / 3.0
    k_ref = ref["ux"].sum() / (n * n) * nu / p.fbody
    e = abs(k_gpu - k_ref) / abs(k_ref)
    record("config1_permeability_5000", rel=e, k=k_gpu)
    assert e < 6e-6  # measured 5.6e-7; the target is 1e-5


def test_disk_image_vs_reference_code():
    # the config-1 disk image (disks crossing the x-periodic seam) against the
    # reference's own run (refstate_config1_200.npz): 200 steps, FP32 GPU
    st = load("refstate_config1_200.npz")
    p = default_params(dx=float(st["dx"]), tol=0.0)
    s = Solver(st["pore"].astype(np.int32), st["kn"], st["locpore"], p)
    assert s.run(200) == 200
    c = s.cells()
    e_ux = rel_err(c["ux"], st["ux"])
    e_rho = np.abs(c["rho"] - st["rho"]).max() / np.abs(st["rho"]).max()
    record("config1_disk_vs_reference_200", ux=e_ux, rho=e_rho)
    assert e_ux < 1.5e-6 and e_rho < 1e-7  # measured u_x 1.1e-7, rho 8.4e-9
