"""The oracle's own grid construction (oracle/grid_oracle.cpp, oracle/pygrid.py),
which lets bench.py's CPU arm run without any product library:

* pinned to the reference: pore properties against the reference's own
  Shape::calculateProperties (refprops*.npz) and grid tables against the
  reference's own Grid2D / LB2D (refgrid_*.npz), both written by
  tests/golden/make_golden.py from the reference's code;
* equal, table for table and bit for bit, to the product's host grid builder
  on the benchmark's workloads (edge-refined three-level 1024^2 included);
* the CPU arm's input fixture is the GPU arm's first image, and the CPU arm
  maps no library of the package.  No GPU."""
import json
import subprocess
import sys

import numpy as np
import pytest
from conftest import ROOT, load

from oracle import pygrid


def same_tables(a, b):
    """Names of the tables in which two grids differ."""
    bad = [k for k in ("x", "y", "level", "type", "is_buffer", "bnd", "conn", "lin", "tau", "kn", "locpore")
           if not np.array_equal(a.cells[k], b.cells[k])]
    bad += [k for k in a.links if not np.array_equal(a.links[k], b.links[k])]
    bad += [k for k in ("coarse_rows", "fine_rows", "parent_child") if not np.array_equal(getattr(a, k), getattr(b, k))]
    bad += [k for k in ("n_cells", "max_level", "inlet", "inlet2", "outlet", "outlet2") if getattr(a, k) != getattr(b, k)]
    return bad


@pytest.mark.parametrize("dx", [1e-9, 2.3e-9, 7.7e-10])
def test_units_match_product(dx):
    from mantiis_gb300 import units

    assert pygrid.units(dx) == units(dx)
    assert pygrid.units(dx, T=350.0, P=5e6) == units(dx, 350.0, 5e6)


@pytest.mark.parametrize("name", ["fx64", "disks128", "disks256", "bigpores256"])
def test_pore_properties_match_reference(name):
    ref = load("refprops.npz")
    lp, kn = pygrid.pore_properties(ref[f"{name}_pore"], float(ref["dx"]), float(ref["mfp"]))
    assert np.array_equal(lp, ref[f"{name}_locpore"])
    want = ref[f"{name}_kn"]
    assert np.all((kn == 0) == (want == 0))
    nz = want != 0
    # the reference is built with -Ofast: the two divisions of Kn may round apart
    assert np.max(np.abs(kn[nz] - want[nz]) / want[nz]) <= 4.5e-16


@pytest.mark.parametrize("name", ["noise96", "blobs128", "diagonal128"])
def test_pore_properties_match_reference_irregular(name):
    ref = load("refprops_extra.npz")
    lp, _ = pygrid.pore_properties(ref[f"{name}_pore"], float(ref["dx"]), float(ref["mfp"]))
    assert np.array_equal(lp, ref[f"{name}_locpore"])


def compare_with_reference(g, ref):
    c = g.cells
    assert g.n_cells == int(ref["n_cells"]) and g.max_level == int(ref["max_level"])
    assert np.array_equal(np.stack([c["x"], c["y"]], 1), ref["ij"])
    for k in ("level", "type", "is_buffer", "bnd", "lin", "conn", "kn"):
        assert np.array_equal(c[k], ref[k]), k
    for k in ("stream_id", "stream_ic", "stream_loc", "wall_id", "wall_ic", "per_id", "per_i2", "per_ic"):
        assert np.array_equal(g.links[k], ref[k]), k
    for k in ("coarse_rows", "fine_rows", "parent_child"):
        assert np.array_equal(getattr(g, k), ref[k]), k
    assert np.abs(c["tau"] - ref["tau"]).max() <= 1e-12


def test_grid_matches_reference_single_block(fixture64):
    g = pygrid.GridTables(fixture64["pore"], fixture64["kn"], fixture64["locpore"], multiblock=False)
    compare_with_reference(g, load("refgrid_fixture64_sb.npz"))


def test_grid_matches_reference_multiblock(fixture64):
    g = pygrid.GridTables(fixture64["pore"], fixture64["kn"], fixture64["locpore"], multiblock=True,
                          max_allowed_level=2)
    compare_with_reference(g, load("refgrid_fixture64_mb.npz"))


@pytest.mark.parametrize("case", ["channel64", "block64", "block64b"])
def test_grid_matches_reference_block_geometries(case):
    ref = load(f"refgrid_{case}.npz")
    g = pygrid.GridTables(ref["img_pore"], ref["img_kn"], ref["img_locpore"], multiblock=True, max_allowed_level=2)
    compare_with_reference(g, ref)


@pytest.mark.parametrize("levels,edge_fine", [(1, 0), (2, 0), (3, 0), (3, 1)])
def test_grid_matches_product_256(levels, edge_fine):
    from mantiis_gb300 import HostGrid, default_params, workloads

    img = workloads.image(256, 6, 20, 0.6, 0.05, 77)
    p = default_params(multiblock=int(levels > 1), max_allowed_level=max(levels, 2), dx=img["dx"],
                       edge_fine=edge_fine)
    want = HostGrid(img["pore"], img["kn"], img["locpore"], p)
    got = pygrid.GridTables(img["pore"], img["kn"], img["locpore"], multiblock=levels > 1,
                            max_allowed_level=max(levels, 2), edge_fine=edge_fine, dx=img["dx"])
    assert same_tables(got, want) == []


def test_config2_fixture_is_the_benchmark_image():
    """oracle/data holds image 0 of the GPU arm's batch; the oracle derives its
    fields and its three-level edge-refined grid exactly as the product does."""
    from mantiis_gb300 import HostGrid, default_params, workloads

    want = workloads.config2(0)
    got = pygrid.config2_image(0)
    assert np.array_equal(got["pore"], want["pore"])
    assert np.array_equal(got["kn"], want["kn"]) and np.array_equal(got["locpore"], want["locpore"])
    assert got["dx"] == want["dx"] and got["levels"] == 3 and got["edge_fine"] == 1
    g = pygrid.GridTables(got["pore"], got["kn"], got["locpore"], multiblock=True, max_allowed_level=3,
                          edge_fine=True, dx=got["dx"])
    h = HostGrid(want["pore"], want["kn"], want["locpore"],
                 default_params(multiblock=1, max_allowed_level=3, dx=want["dx"], edge_fine=1))
    assert same_tables(g, h) == []
    assert g.lattice_updates() == 1266664.0


def test_reference_arm_loads_no_product_library():
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "3", "--ref-budget", "2"], capture_output=True, text=True, timeout=600,
                         cwd=str(ROOT))
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads([ln for ln in out.stdout.splitlines() if ln.startswith("{")][-1])
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["product_libraries_loaded"] == []
    assert "grid_oracle.cpp" in line["cpu_baseline"]["sample"]


@pytest.mark.parametrize("levels", [2, 3])
def test_grid_matches_reference_disk_image(levels):
    # the reference's own Grid2D on a 256x256 disk image with void x edges: two
    # levels from the unmodified reference, three with its depth limit raised to
    # 3; the fixtures hold every table but the streaming link list
    ref = load(f"refgrid_disks256_l{levels}.npz")
    g = pygrid.GridTables(ref["img_pore"].astype(np.int32), ref["img_kn"], ref["img_locpore"], multiblock=True,
                          max_allowed_level=levels, dx=float(ref["dx"]))
    c = g.cells
    assert g.n_cells == int(ref["n_cells"]) and g.max_level == levels
    assert np.array_equal(np.stack([c["x"], c["y"]], 1), ref["ij"])
    for k in ("level", "type", "is_buffer", "bnd", "lin", "conn", "kn"):
        assert np.array_equal(c[k], ref[k]), k
    for k in ("wall_id", "wall_ic", "per_id", "per_i2", "per_ic"):
        assert np.array_equal(g.links[k], ref[k]), k
    for k in ("coarse_rows", "fine_rows", "parent_child"):
        assert np.array_equal(getattr(g, k), ref[k]), k
    assert np.abs(c["tau"] - ref["tau"]).max() <= 1e-12


@pytest.mark.parametrize("seed", range(12))
def test_grid_and_properties_agree_on_random_images(seed):
    # two independent restatements of the reference's grid construction (the
    # product's host builder and the oracle's) on seeded random disk images:
    # sizes 32..128, porosity 0.45..0.8, void x edges or not, one to three
    # levels, with and without edge_fine; where one rejects an image (an
    # untabulated boundary pattern), so must the other
    from mantiis_gb300 import HostGrid, MantiisError, default_params, generate_disks, pore_properties

    rng = np.random.default_rng(100 + seed)
    n = int(rng.choice([32, 64, 128]))
    pore = generate_disks(n, 2.0, max(3.0, n / 16), float(rng.uniform(0.45, 0.8)), 7000 + seed,
                          open_x_edges=bool(seed % 2))
    lp_a, kn_a = pore_properties(pore, 1e-9, 5e-9)
    lp_b, kn_b = pygrid.pore_properties(pore, 1e-9, 5e-9)
    assert np.array_equal(lp_a, lp_b) and np.array_equal(kn_a, kn_b)
    levels = int(rng.integers(1, 4))
    edge_fine = bool(rng.integers(0, 2)) and levels > 1
    kn = np.where(pore == 1, kn_a, 0.0)
    p = default_params(multiblock=int(levels > 1), max_allowed_level=max(levels, 2), dx=1e-9, edge_fine=int(edge_fine))
    try:
        want = HostGrid(pore, kn, lp_a, p)
    except MantiisError as e:
        with pytest.raises(RuntimeError, match=str(e).split(":")[-1].strip()[:20]):
            pygrid.GridTables(pore, kn, lp_a, multiblock=levels > 1, max_allowed_level=max(levels, 2),
                              edge_fine=edge_fine)
        return
    got = pygrid.GridTables(pore, kn, lp_a, multiblock=levels > 1, max_allowed_level=max(levels, 2),
                            edge_fine=edge_fine)
    assert same_tables(got, want) == []


def test_oracle_tables_hold_the_products_numbers():
    # the oracle's copy of the reference's boundary-type tables and the product's
    # (both written from include/system_files) hold the same numbers
    import re

    def arrays(path, prefix):
        txt = path.read_text()
        out = {}
        for name in ("BND_CODES", "IFSTREAM", "ICSR", "XY_NORM"):
            blk = txt[txt.index(prefix + name):]
            blk = blk[blk.index("=") + 1:blk.index("};")]
            out[name] = [float(v) for v in re.findall(r"-?\d+(?:\.\d+)?(?:[eE]-?\d+)?", blk)]
        return out

    a = arrays(ROOT / "oracle" / "reference_tables.h", "ORACLE_")
    b = arrays(ROOT / "mantiis_gb300" / "csrc" / "boundary_tables.h", "MANTIIS_")
    assert a == b and len(a["BND_CODES"]) == 52 and len(a["IFSTREAM"]) == 52 * 9
