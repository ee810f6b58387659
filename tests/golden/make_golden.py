"""Generates the golden fixtures under tests/golden/ (run in a checkout that has
the reference at REF_DIR and oracle/_ref built: `make -C oracle`).

  fixture64.npz     the reference's 64x64 test inputs (test/test_input_output/
                    {pore,Kn,localporesize}.dat, as row-major images) and its gold
                    outputs gold/{transport,adsorption}/{ux,uy,rho}.txt (100 steps)
  refgrid_<case>.npz  grid tables produced by the reference's own Grid2D / LB2D
                    code (oracle/_ref/ref_driver): the 64x64 test image single-
                    and multi-block, and block geometries multi-block
  refstate_<case>.npz per-cell state of the reference's own solver after some
                    steps for multi-block cases where the reference's
                    interpolation stays inside its arrays
  refstate_coupled64.npz  the reference's coupled run on the 64x64 test image
  refprops.npz      local pore size and Kn from the reference's own
                    Shape::calculateProperties on four pore images
  refprops_extra.npz  the same on three irregular images (noise, blobs,
                    diagonal channels)
  refstate_config1_200.npz  the reference's own run on the config-1 disk image
                    (128x128, single block), cell fields after 200 steps
  refstate_adsorption128_100.npz  the reference's own adsorption run on a
                    128x128 disk image, cell fields after 100 steps
  refstate_variants.npz  the reference's own runs with BGK / MRT collisions and
                    MDBB / BB walls, single block (64x64 test image) and
                    multi-block (block64 geometry)
  refgrid_disks256_l3.npz  grid tables of the reference's own Grid2D / LB2D with
                    the quadtree depth limit raised to 3 (oracle/_ref/ref_driver3)
                    on a 256x256 seeded disk image (void x edges), with the image
                    and its fields
  refgrid_disks256_l2.npz  the unpatched reference's two-level grid of that image
  refgrid_block128_l3.npz, refstate_block128_l3.npz  the same three-level build
                    on a 128x128 block geometry, and the reference's own cell
                    states after 1, 2 and 50 coarse steps

Usage: python tests/golden/make_golden.py REF_DIR [--only properties|properties_extra|disk_state|disk_adsorption|coupled|variants|grid3|grid2_disks|state3]
"""
import os
import struct
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
_ARGS = [a for a in sys.argv[1:] if not a.startswith("--")]
_ONLY = sys.argv[sys.argv.index("--only") + 1] if "--only" in sys.argv else None
if _ONLY:
    _ARGS.remove(_ONLY)
if not _ARGS and not os.environ.get("MANTIIS_REF_DIR"):
    sys.exit("usage: make_golden.py <reference checkout> [--only ...]  (or set MANTIIS_REF_DIR)")
REF = Path(_ARGS[0] if _ARGS else os.environ["MANTIIS_REF_DIR"])
DRIVER = ROOT / "oracle" / "_ref" / "ref_driver"
HOME = ROOT / "oracle" / "_ref" / "home"


def read_col_major(path, n):
    v = np.loadtxt(path)
    return v.reshape(n, n).T.copy()  # data[j*n + i] belongs to row i, column j


def write_col_major(folder, pore, kn, lp):
    folder.mkdir(parents=True, exist_ok=True)
    for name, arr, fmt in (("pore.dat", pore, "%d"), ("Kn.dat", kn, "%.6e"), ("localporesize.dat", lp, "%.6e")):
        np.savetxt(folder / name, arr.T.reshape(-1), fmt=fmt)


def read_dump(path):
    d = path.read_bytes()
    off = 0

    def take(fmt):
        nonlocal off
        v = struct.unpack_from(fmt, d, off)
        off += struct.calcsize(fmt)
        return v

    def vec(dt):
        nonlocal off
        (k,) = take("q")
        a = np.frombuffer(d, dtype=dt, count=k, offset=off).copy()
        off += a.nbytes
        return a

    return take, vec


def read_grid(path):
    take, vec = read_dump(path)
    (n,) = take("q")
    (L,) = take("i")
    g = dict(n_cells=n, max_level=L)
    g["ij"] = vec(np.int32).reshape(-1, 2)
    for k in ("level", "type", "is_buffer", "bnd"):
        g[k] = vec(np.int32)
    g["conn"] = vec(np.int64).reshape(-1, 9)
    for k in ("tau", "kn", "locpore"):
        g[k] = vec(np.float64)
    g["lin"] = vec(np.int64)
    g["stream_id"], g["stream_ic"], g["stream_loc"] = vec(np.int64), vec(np.int32), vec(np.int64)
    g["wall_id"], g["wall_ic"] = vec(np.int64), vec(np.int32)
    g["per_id"], g["per_i2"], g["per_ic"] = vec(np.int64), vec(np.int64), vec(np.int32)
    g["coarse_rows"] = vec(np.int64).reshape(-1, 6)
    g["fine_rows"] = vec(np.int64).reshape(-1, 6)
    g["parent_child"] = vec(np.int64).reshape(-1, 5)
    return g


def read_state(path):
    take, vec = read_dump(path)
    (step,) = take("q")
    s = dict(step=step)
    for k in ("rho", "ux", "uy", "f", "residuals"):
        s[k] = vec(np.float64)
    s["f"] = s["f"].reshape(-1, 9)
    return s


def run_ref(folder, n, steps, multiblock, mode="transport", dx=1e-9, levels=2, dump_steps=(), extra=()):
    exe = DRIVER if levels == 2 else ROOT / "oracle" / "_ref" / "ref_driver3"
    with tempfile.TemporaryDirectory() as dump:
        cmd = [str(exe), "1", "true" if multiblock else "False", str(n), str(folder) + "/", str(steps), "--mode", mode,
               "--dx", repr(dx), "--quiet", "--no-break", "--dump", dump]
        if dump_steps:
            cmd += ["--dump-steps", ",".join(str(s) for s in dump_steps)]
        cmd += [str(a) for a in extra]
        env = dict(os.environ, HOME=str(HOME))
        subprocess.run(cmd, check=True, env=env, stdout=subprocess.DEVNULL)
        grid = read_grid(Path(dump) / "grid.bin")
        states = {s: read_state(Path(dump) / f"state_{s}.bin") for s in dump_steps}
    return grid, states


def block_geometry(n, wall, obst=None):
    p = np.ones((n, n), dtype=np.int32)
    p[:wall, :] = 0
    p[n - wall:, :] = 0
    if obst:
        r0, r1, c0, c1 = obst
        p[r0:r1, c0:c1] = 0
    kn = np.where(p == 1, 0.1, 0.0)
    lp = np.where(p == 1, 7.73, 0.0)
    return p, kn, lp


CASES = {
    # name: (n, wall rows, obstacle rows/cols)
    "channel64": (64, 2, None),
    "block64": (64, 2, (24, 40, 16, 32)),
    "block64b": (64, 1, (20, 44, 8, 40)),
}


def main():
    t = REF / "test" / "test_input_output"
    fx = dict(
        pore=read_col_major(t / "pore.dat", 64).astype(np.int32),
        kn=read_col_major(t / "Kn.dat", 64),
        locpore=read_col_major(t / "localporesize.dat", 64),
    )
    for sim in ("transport", "adsorption"):
        for name in ("ux", "uy", "rho"):
            fx[f"{sim}_{name}"] = np.loadtxt(t / "gold" / sim / f"{name}.txt").reshape(64, 64)
    np.savez_compressed(HERE / "fixture64.npz", **fx)

    with tempfile.TemporaryDirectory() as tmp:
        # multi-block grid of the 64x64 test image (the reference's interpolation
        # reads outside its arrays on this image, so only the grid is kept)
        f = Path(tmp) / "fx64"
        write_col_major(f, fx["pore"], fx["kn"], fx["locpore"])
        grid, _ = run_ref(f, 64, 0, True)
        np.savez_compressed(HERE / "refgrid_fixture64_mb.npz", **grid)
        grid, _ = run_ref(f, 64, 0, False)
        np.savez_compressed(HERE / "refgrid_fixture64_sb.npz", **grid)
        for name, (n, wall, obst) in CASES.items():
            f = Path(tmp) / name
            p, kn, lp = block_geometry(n, wall, obst)
            write_col_major(f, p, kn, lp)
            grid, states = run_ref(f, n, 50, True, dump_steps=(1, 2, 50))
            np.savez_compressed(HERE / f"refgrid_{name}.npz", img_pore=p, img_kn=kn, img_locpore=lp, **grid)
            np.savez_compressed(HERE / f"refstate_{name}.npz",
                                **{f"{k}_{s}": v for s, st in states.items() for k, v in st.items()})
    coupled_fixture(fx)
    properties_fixture(fx)
    disk_state_fixture()
    disk_adsorption_fixture()
    variants_fixture(fx)
    grid3_fixture()
    grid2_disks_fixture()
    state3_fixture()
    print("fixtures written to", HERE)


def coupled_fixture(fx):
    """The reference's coupled run (include/mantiisApp.hpp:376-392) on the 64x64
    test image, single block, dx = 12 nm: 100 adsorption steps without body
    force, then coupling steps; states after 100, 101 and 130 steps."""
    with tempfile.TemporaryDirectory() as tmp:
        f = Path(tmp) / "fx64"
        write_col_major(f, fx["pore"], fx["kn"], fx["locpore"])
        grid, states = run_ref(f, 64, 30, False, mode="coupled", dx=12e-9, dump_steps=(100, 101, 130))
        np.savez_compressed(HERE / "refstate_coupled64.npz",
                            **{f"{k}_{s}": v for s, st in states.items() for k, v in st.items()})


# (collision, wall): 0 BGK, 1 MRT, 2 regularized MRT; 0 BB, 1 MDBB, 2 SRBB
VARIANTS_SB = [(2, 1), (1, 2), (0, 0), (1, 1), (0, 2), (0, 1)]
VARIANTS_MB = [(2, 1), (0, 2), (0, 1)]


def variants_fixture(fx):
    """The reference's own runs with the other collision operators and walls
    (Settings::collision_method / wall_boundary: SRTCollision, include/coreLB.hpp:678-691,
    MRTCollisionNonRegularized :694-742, MDBBWall :936-967, BBWall :859-865):
    single block on the 64x64 test image (100 steps) and multi-block on the
    block64 geometry (50 steps); cell fields and populations at the last step."""
    out = {}
    with tempfile.TemporaryDirectory() as tmp:
        f = Path(tmp) / "fx64"
        write_col_major(f, fx["pore"], fx["kn"], fx["locpore"])
        for c, w in VARIANTS_SB:
            _, st = run_ref(f, 64, 100, False, dump_steps=(100,), extra=("--collision", c, "--wall", w))
            for k in ("rho", "ux", "uy", "f"):
                out[f"sb_c{c}_w{w}_{k}"] = st[100][k]
        n, wall, obst = CASES["block64"]
        p, kn, lp = block_geometry(n, wall, obst)
        f = Path(tmp) / "block64"
        write_col_major(f, p, kn, lp)
        for c, w in VARIANTS_MB:
            _, st = run_ref(f, n, 50, True, dump_steps=(50,), extra=("--collision", c, "--wall", w))
            for k in ("rho", "ux", "uy", "f"):
                out[f"mb_c{c}_w{w}_{k}"] = st[50][k]
    np.savez_compressed(HERE / "refstate_variants.npz", **out)


def disk_state_fixture():
    """The reference's own single-block run on the config-1 disk image
    (128x128, radii U[4,10], porosity 0.65, Kn ~0.1, the package's seeded
    generator and its dx): cell fields after 200 steps."""
    sys.path.insert(0, str(ROOT))
    from mantiis_gb300 import workloads

    img = workloads.config1(0)
    # the values as the reference reads them back from the %.6e text files
    kn = np.vectorize(lambda v: float(f"{v:.6e}"))(img["kn"])
    lp = np.vectorize(lambda v: float(f"{v:.6e}"))(img["locpore"])
    with tempfile.TemporaryDirectory() as tmp:
        f = Path(tmp) / "c1"
        write_col_major(f, img["pore"], kn, lp)
        _, states = run_ref(f, 128, 200, False, dx=img["dx"], dump_steps=(200,))
    st = states[200]
    np.savez_compressed(HERE / "refstate_config1_200.npz", pore=img["pore"].astype(np.uint8), kn=kn, locpore=lp,
                        dx=img["dx"], rho=st["rho"], ux=st["ux"], uy=st["uy"], residuals=st["residuals"])


def disk_adsorption_fixture():
    """The reference's own adsorption run (PR-EOS pseudopotential, bounce-back
    walls, inlet/outlet) on a 128x128 seeded disk image at dx = 12 nm: cell
    fields after 100 steps."""
    sys.path.insert(0, str(ROOT))
    from mantiis_gb300 import workloads

    img = workloads.image(128, 6, 14, 0.6, 0.1, 3100)
    kn = np.vectorize(lambda v: float(f"{v:.6e}"))(img["kn"])
    lp = np.vectorize(lambda v: float(f"{v:.6e}"))(img["locpore"])
    with tempfile.TemporaryDirectory() as tmp:
        f = Path(tmp) / "a1"
        write_col_major(f, img["pore"], kn, lp)
        _, states = run_ref(f, 128, 100, False, mode="adsorption", dx=12e-9, dump_steps=(100,))
    st = states[100]
    np.savez_compressed(HERE / "refstate_adsorption128_100.npz", pore=img["pore"].astype(np.uint8), kn=kn,
                        locpore=lp, rho=st["rho"], ux=st["ux"], uy=st["uy"], residuals=st["residuals"])


def run_ref_properties(pore, dx, mfp):
    """Shape::calculateProperties (include/shape.hpp:127-251) of the reference on
    one pore image: (LocPore, Kn), row-major [row][column]."""
    n = pore.shape[0]
    with tempfile.TemporaryDirectory() as tmp:
        f = Path(tmp) / "img"
        zero = np.zeros((n, n))
        write_col_major(f, pore, zero, zero)
        cmd = [str(DRIVER), "1", "False", str(n), str(f) + "/", "0", "--mode", "properties", "--dx", repr(dx),
               "--mfp", repr(mfp), "--quiet", "--dump", tmp]
        subprocess.run(cmd, check=True, env=dict(os.environ, HOME=str(HOME)), stdout=subprocess.DEVNULL)
        raw = (Path(tmp) / "properties.bin").read_bytes()
    count = int(np.frombuffer(raw[:8], np.int64)[0])
    lp = np.frombuffer(raw[8:8 + 8 * count], np.float64)
    kn = np.frombuffer(raw[16 + 8 * count:16 + 16 * count], np.float64)
    return lp.reshape(n, n).copy(), kn.reshape(n, n).copy()


def disk_image(n, rmin, rmax, porosity, seed, open_x_edges=False):
    """Seeded disk packing of the package's own generator (host code, no GPU)."""
    sys.path.insert(0, str(ROOT))
    from mantiis_gb300 import generate_disks
    return generate_disks(n, rmin, rmax, porosity, seed, open_x_edges=open_x_edges).astype(np.int32)


def properties_fixture(fx):
    """Local pore size and Kn of the reference on four images: the 64x64 test
    image, disk packings at 128 and 256 (the second with void x edges), and a
    256 image of a few large disks whose top and bottom rows are partly void."""
    images = {
        "fx64": fx["pore"].astype(np.int32),
        "disks128": disk_image(128, 4, 16, 0.6, 1),
        "disks256": disk_image(256, 8, 32, 0.6, 2, open_x_edges=True),
    }
    big = disk_image(256, 24, 60, 0.8, 3)
    big[0, 100:180] = 1
    big[255, 40:90] = 1
    images["bigpores256"] = big
    out = {}
    for name, pore in images.items():
        lp, kn = run_ref_properties(pore, 1e-9, 5e-9)
        out[f"{name}_pore"] = pore.astype(np.uint8)
        out[f"{name}_locpore"] = lp
        out[f"{name}_kn"] = kn
    np.savez_compressed(HERE / "refprops.npz", dx=1e-9, mfp=5e-9, **out)
    properties_extra_fixture()


def properties_extra_fixture():
    """Three irregular images for the host pipeline: salt-and-pepper noise (many
    one-pixel pores and tiny components), smoothed random blobs, and thin
    diagonal channels (skeletons that are all diagonal steps)."""
    rng = np.random.default_rng(17)
    images = {"noise96": (rng.random((96, 96)) < 0.58).astype(np.int32)}
    field = rng.random((128, 128))
    for _ in range(6):  # smoothing by neighbour averages on the torus
        field = (field + np.roll(field, 1, 0) + np.roll(field, -1, 0) + np.roll(field, 1, 1)
                 + np.roll(field, -1, 1)) / 5.0
    images["blobs128"] = (field > np.median(field)).astype(np.int32)
    y, x = np.mgrid[0:128, 0:128]
    images["diagonal128"] = (((x + y) % 24) < 5).astype(np.int32)
    for im in images.values():
        im[0, :] = 0
        im[-1, :] = 0
    out = {}
    for name, pore in images.items():
        lp, kn = run_ref_properties(pore, 1e-9, 5e-9)
        out[f"{name}_pore"] = pore.astype(np.uint8)
        out[f"{name}_locpore"] = lp
        out[f"{name}_kn"] = kn
    np.savez_compressed(HERE / "refprops_extra.npz", dx=1e-9, mfp=5e-9, **out)


def grid2_disks_fixture():
    """Two quadtree levels (the reference's own depth limit, unpatched
    ref_driver) on the 256x256 disk image of grid3_fixture; grid only."""
    sys.path.insert(0, str(ROOT))
    from mantiis_gb300 import workloads

    img = workloads.image(256, 6, 20, 0.6, 0.05, 77, open_x_edges=True)
    with tempfile.TemporaryDirectory() as tmp:
        f = Path(tmp) / "disks256"
        write_col_major(f, img["pore"], img["kn"], img["locpore"])
        kn, lp = read_col_major(f / "Kn.dat", 256), read_col_major(f / "localporesize.dat", 256)
        grid, _ = run_ref(f, 256, 0, True, dx=img["dx"], levels=2)
    for k in ("stream_id", "stream_ic", "stream_loc"):
        grid.pop(k)
    grid["conn"] = grid["conn"].astype(np.int32)
    np.savez_compressed(HERE / "refgrid_disks256_l2.npz", img_pore=img["pore"].astype(np.uint8), img_kn=kn,
                        img_locpore=lp, dx=img["dx"], **grid)


def grid3_fixture():
    """Three quadtree levels on a 256x256 disk image (radii 6-20, porosity 0.6,
    seed 77, mean Kn 0.05, the two columns at either x edge void), built by the
    reference's Grid2D with its depth limit raised to 3; grid only.  With solid
    pixels on the x-periodic seam the reference's three-level build ends in a
    segmentation fault (its interface tables then index outside its arrays)."""
    sys.path.insert(0, str(ROOT))
    from mantiis_gb300 import workloads

    img = workloads.image(256, 6, 20, 0.6, 0.05, 77, open_x_edges=True)
    with tempfile.TemporaryDirectory() as tmp:
        f = Path(tmp) / "disks256"
        write_col_major(f, img["pore"], img["kn"], img["locpore"])
        # the fields as the reference read them (7 significant digits)
        kn, lp = read_col_major(f / "Kn.dat", 256), read_col_major(f / "localporesize.dat", 256)
        grid, _ = run_ref(f, 256, 0, True, dx=img["dx"], levels=3)
    # the streaming link lists (330 k links) follow from conn and the boundary
    # types and are left out to keep the file small; the wall and periodic lists stay
    for k in ("stream_id", "stream_ic", "stream_loc"):
        grid.pop(k)
    grid["conn"] = grid["conn"].astype(np.int32)
    np.savez_compressed(HERE / "refgrid_disks256_l3.npz", img_pore=img["pore"].astype(np.uint8), img_kn=kn,
                        img_locpore=lp, dx=img["dx"], **grid)


CASES3 = {
    # name: (n, wall rows, obstacle rows/cols); three quadtree levels, grids on
    # which the reference's interpolation stays inside its arrays
    "block128_l3": (128, 2, (48, 80, 32, 64)),
}


def state3_fixture():
    """The reference's own three-level run (oracle/_ref/ref_driver3, depth limit
    raised to 3) on a block geometry: grid tables and cell states after 1, 2 and
    50 coarse steps."""
    with tempfile.TemporaryDirectory() as tmp:
        for name, (n, wall, obst) in CASES3.items():
            f = Path(tmp) / name
            p, kn, lp = block_geometry(n, wall, obst)
            write_col_major(f, p, kn, lp)
            grid, states = run_ref(f, n, 50, True, levels=3, dump_steps=(1, 2, 50))
            for k in ("stream_id", "stream_ic", "stream_loc"):
                grid.pop(k)
            grid["conn"] = grid["conn"].astype(np.int32)
            np.savez_compressed(HERE / f"refgrid_{name}.npz", img_pore=p, img_kn=kn, img_locpore=lp, **grid)
            np.savez_compressed(HERE / f"refstate_{name}.npz",
                                **{f"{k}_{s}": v for s, st in states.items() for k, v in st.items()})


if __name__ == "__main__":
    if _ONLY:
        fx = dict(np.load(HERE / "fixture64.npz"))
        {"properties": properties_fixture, "coupled": coupled_fixture,
         "properties_extra": lambda _: properties_extra_fixture(),
         "disk_state": lambda _: disk_state_fixture(),
         "disk_adsorption": lambda _: disk_adsorption_fixture(),
         "variants": variants_fixture,
         "grid3": lambda _: grid3_fixture(),
         "grid2_disks": lambda _: grid2_disks_fixture(),
         "state3": lambda _: state3_fixture()}[_ONLY](fx)
    else:
        main()
