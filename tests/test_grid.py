"""The product's host grid builder reproduces the reference's Grid2D / LB2D
tables (cell order, levels, buffers, neighbours, boundary types, link lists,
interface rows, relaxation times) exactly."""
import numpy as np
import pytest
from conftest import ROOT, load

from mantiis_gb300 import HostGrid, MantiisError, default_params, generate_disks, units


def compare(g, ref):
    c = g.cells
    assert g.n_cells == int(ref["n_cells"]) and g.max_level == int(ref["max_level"])
    assert np.array_equal(np.stack([c["x"], c["y"]], 1), ref["ij"])
    for k in ("level", "type", "is_buffer", "bnd", "lin"):
        assert np.array_equal(c[k], ref[k]), k
    assert np.array_equal(c["conn"], ref["conn"])
    for k in ("stream_id", "stream_ic", "stream_loc", "wall_id", "wall_ic", "per_id", "per_i2", "per_ic"):
        assert np.array_equal(g.links[k], ref[k]), k
    assert np.array_equal(g.coarse_rows, ref["coarse_rows"])
    assert np.array_equal(g.fine_rows, ref["fine_rows"])
    assert np.array_equal(g.parent_child, ref["parent_child"])
    assert np.abs(c["tau"] - ref["tau"]).max() <= 1e-12
    assert np.array_equal(c["kn"], ref["kn"])


def test_single_block_grid(fixture64):
    g = HostGrid(fixture64["pore"], fixture64["kn"], fixture64["locpore"], default_params())
    compare(g, load("refgrid_fixture64_sb.npz"))
    assert g.n_cells == int((fixture64["pore"] == 1).sum())


def test_multiblock_grid_of_test_image(fixture64):
    g = HostGrid(fixture64["pore"], fixture64["kn"], fixture64["locpore"], default_params(multiblock=1))
    compare(g, load("refgrid_fixture64_mb.npz"))
    # the reference's interpolation reads outside its arrays for these parents
    assert g.diagnostics["fine_parent_missing_nbr"] == 8


@pytest.mark.parametrize("case", ["channel64", "block64", "block64b"])
def test_multiblock_grid_block_geometries(case):
    ref = load(f"refgrid_{case}.npz")
    g = HostGrid(ref["img_pore"], ref["img_kn"], ref["img_locpore"], default_params(multiblock=1))
    compare(g, ref)
    assert sum(g.diagnostics.values()) == 0


def test_grid_from_folder_matches_arrays(tmp_path, fixture64):
    for name, arr, fmt in (("pore.dat", fixture64["pore"], "%d"), ("Kn.dat", fixture64["kn"], "%.6e"),
                           ("localporesize.dat", fixture64["locpore"], "%.6e")):
        np.savetxt(tmp_path / name, arr.T.reshape(-1), fmt=fmt)
    a = HostGrid(folder=str(tmp_path) + "/", n=64)
    b = HostGrid(fixture64["pore"], fixture64["kn"], fixture64["locpore"])
    assert np.array_equal(a.cells["conn"], b.cells["conn"])
    assert np.array_equal(a.cells["tau"], b.cells["tau"])


def test_input_errors(tmp_path, fixture64):
    # include/io.hpp:53-72 messages
    with pytest.raises(MantiisError, match="File not found"):
        HostGrid(folder=str(tmp_path) + "/", n=64)
    np.savetxt(tmp_path / "pore.dat", np.ones(100), fmt="%d")
    with pytest.raises(MantiisError, match="Insufficient data"):
        HostGrid(folder=str(tmp_path) + "/", n=64)


def test_unknown_boundary_pattern():
    # an isolated void pixel has a 9-neighbour pattern outside the 52 tabulated types
    p = np.zeros((16, 16), np.int32)
    p[1:4, :] = 1
    p[8, 8] = 1
    with pytest.raises(MantiisError, match="Boundary type is not contained"):
        HostGrid(p, np.full((16, 16), 0.1), np.full((16, 16), 5.0))


def test_multiblock_needs_power_of_two():
    p = np.ones((48, 48), np.int32)
    p[0] = p[-1] = 0
    with pytest.raises(MantiisError, match="divisible by 2"):
        HostGrid(p, np.full((48, 48), 0.1), np.full((48, 48), 5.0), default_params(multiblock=1))


def test_units_match_reference_run():
    # values printed by the reference build for T = 300 K, P = 2 MPa
    u = units(1e-9, 300.0, 2.0e6)
    assert abs(u["rho_in"] - 0.23555454407598886) < 1e-15
    assert abs(u["mfp"] / 7.7308467606585409e-10 - 1) < 1e-14
    assert abs(u["T_lu"] - 0.11479923396990133) < 1e-15


def test_disk_generator():
    a = generate_disks(128, 4, 10, 0.65, 1000)
    b = generate_disks(128, 4, 10, 0.65, 1000)
    assert np.array_equal(a, b)
    assert (a[0] == 0).all() and (a[-1] == 0).all()
    phi = a.mean()
    assert 0.60 < phi <= 0.65
    assert not np.array_equal(a, generate_disks(128, 4, 10, 0.65, 1001))


def test_three_level_grid_builds():
    p = generate_disks(256, 6, 40, 0.6, 2000)
    g = HostGrid(p, np.full(p.shape, 0.1), np.full(p.shape, 7.0), default_params(multiblock=1, max_allowed_level=3))
    assert g.max_level == 3
    lv = g.cells["level"]
    assert (lv == 3).any() and (lv == 2).any() and (lv == 1).any()
    # every interface row points at existing cells
    assert (g.fine_rows[:, 1:] >= 0).all()


@pytest.mark.parametrize("levels", [2, 3])
def test_disk_image_grid_matches_reference(levels):
    # the reference's own Grid2D / LB2D on a 256x256 disk image with void x
    # edges: two levels from the unmodified reference, three with its quadtree
    # depth limit raised to 3 (refgrid_disks256_l<levels>.npz); every table but
    # the streaming link list, which the fixtures leave out
    ref = load(f"refgrid_disks256_l{levels}.npz")
    p = default_params(multiblock=1, max_allowed_level=levels, dx=float(ref["dx"]))
    g = HostGrid(ref["img_pore"].astype(np.int32), ref["img_kn"], ref["img_locpore"], p)
    assert g.max_level == levels
    c = g.cells
    assert g.n_cells == int(ref["n_cells"])
    assert np.array_equal(np.stack([c["x"], c["y"]], 1), ref["ij"])
    for k in ("level", "type", "is_buffer", "bnd", "lin", "conn", "kn"):
        assert np.array_equal(c[k], ref[k]), k
    for k in ("wall_id", "wall_ic", "per_id", "per_i2", "per_ic"):
        assert np.array_equal(g.links[k], ref[k]), k
    for k in ("coarse_rows", "fine_rows", "parent_child"):
        assert np.array_equal(getattr(g, k), ref[k]), k
    assert np.abs(c["tau"] - ref["tau"]).max() <= 1e-12


def test_three_level_block_grid_matches_reference():
    # the three-level block geometry of refstate_block128_l3.npz (the reference's
    # own run with its depth limit raised to 3)
    ref = load("refgrid_block128_l3.npz")
    g = HostGrid(ref["img_pore"], ref["img_kn"], ref["img_locpore"], default_params(multiblock=1, max_allowed_level=3))
    assert g.max_level == 3 and g.n_cells == int(ref["n_cells"])
    c = g.cells
    for k in ("level", "type", "is_buffer", "bnd", "lin", "conn"):
        assert np.array_equal(c[k], ref[k]), k
    for k in ("wall_id", "wall_ic", "per_id", "per_i2", "per_ic"):
        assert np.array_equal(g.links[k], ref[k]), k
    for k in ("coarse_rows", "fine_rows", "parent_child"):
        assert np.array_equal(getattr(g, k), ref[k]), k
    assert np.abs(c["tau"] - ref["tau"]).max() <= 1e-12
    assert sum(g.diagnostics.values()) == 0
