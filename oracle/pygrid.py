"""The oracle's own inputs: unit system, pore properties and grid tables.

TEST INFRASTRUCTURE ONLY: imported by tests/ and by bench.py's CPU arm, which
with it builds its grid and steps it with lbm_oracle.cpp without loading any
product library; never by the product.

  units            _GLOBAL_::recompute (include/globalParameters.hpp:180-221)
  pore_properties  Shape::calculateProperties (include/shape.hpp:127-251), in grid_oracle.cpp
  GridTables       Grid2D + LB2D link lists and relaxation times, in grid_oracle.cpp;
                   the attributes Oracle() reads (n, max_level, n_cells, cells,
                   links, coarse_rows, fine_rows, inlet ... outlet2)
  image_fields     per-pixel Kn of a seeded image whose mean Kn is given, as the
                   benchmark workloads define it
  config2_image    the benchmark's first config-2 image from oracle/data
"""
import ctypes as C
import math
from pathlib import Path

import numpy as np

from .pyoracle import OracleGrid, lib as _oracle_lib

HERE = Path(__file__).resolve().parent


class OracleGridOptions(C.Structure):
    _fields_ = [("multiblock", C.c_int), ("max_allowed_level", C.c_int), ("edge_fine", C.c_int),
                ("dx", C.c_double), ("mfp", C.c_double)]


class OracleGridExtra(C.Structure):
    _fields_ = [("lin", C.c_void_p), ("locpore", C.c_void_p), ("n_parent_child", C.c_int64),
                ("parent_child", C.c_void_p), ("buffer_wall_links", C.c_int64)]


_ready = False


def lib():
    global _ready
    L = _oracle_lib()
    if not _ready:
        L.oracle_pore_properties.restype = C.c_int64
        L.oracle_pore_properties.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_void_p, C.c_void_p]
        L.oracle_grid_create.restype = C.c_void_p
        L.oracle_grid_create.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.POINTER(OracleGridOptions)]
        L.oracle_grid_view.argtypes = [C.c_void_p, C.POINTER(OracleGrid), C.POINTER(OracleGridExtra)]
        L.oracle_grid_destroy.argtypes = [C.c_void_p]
        L.oracle_grid_error.restype = C.c_char_p
        _ready = True
    return L


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def units(dx=1e-9, T=300.0, P=2.0e6):
    """Peng-Robinson methane at (T, P) and the lattice conversion factors, in
    the reference's order of operations (include/globalParameters.hpp:50-132
    and :180-221); the cubic's root by Cardano's one-real-root branch
    (include/utils.hpp:571-600), the largest of the roots found
    (include/utils.hpp:226-239, numeric_limits<double>::min() when none)."""
    Cl, T_phy, P_phy = float(dx), float(T), float(P)
    Tc_phy, Pc_phy, d_mol, omega, Mw = 190.564, 4.5992 * 1.0e6, 3.800e-10, 0.011, 16.043 * 1.0e-3
    NA, R_EOS = 6.02214076e23, 8.31446
    a_lu, b_lu, R_lu, Mw_lu = 2.0 / 49.0, 2.0 / 21.0, 1.0, 1.0
    Rs_lu = R_lu / Mw_lu
    pw = math.pow
    k = 0.37464 + 1.54226 * omega - 0.26992 * pw(omega, 2)
    alpha = pw((1 + k * (1 - math.sqrt(T_phy / Tc_phy))), 2)
    a_alpha_lu = a_lu * alpha
    Rs = R_EOS / Mw
    a = 0.45724 * (R_EOS * Tc_phy) * (R_EOS * Tc_phy) / Pc_phy
    aG = a * alpha
    bG = 0.07780 * R_EOS * Tc_phy / Pc_phy
    AG = aG * P_phy / (R_EOS * R_EOS) / (T_phy * T_phy)
    BG = bG * P_phy / R_EOS / T_phy
    ZG3, ZG2 = 1.0, BG - 1
    ZG1 = AG - 3 * (BG * BG) - 2 * BG
    ZG0 = BG * BG * BG + (BG * BG) - AG * BG
    roots = []
    ca, cb, cc, cd = ZG3, ZG2, ZG1, ZG0
    p = (3 * ca * cc - cb * cb) / (3 * ca * ca)
    q = (2 * cb * cb * cb - 9 * ca * cb * cc + 27 * ca * ca * cd) / (27 * ca * ca * ca)
    delta = -4 * p * p * p - 27 * q * q
    if delta < 0:
        u1 = -q / 2 + math.sqrt(q * q / 4 + p * p * p / 27)
        u2 = -q / 2 - math.sqrt(q * q / 4 + p * p * p / 27)
        t = float(np.power(np.float64(u1), 1.0 / 3.0)) + float(np.power(np.float64(u2), 1.0 / 3.0))
        roots.append(t - cb / (3 * ca))
    ZG = 2.2250738585072014e-308
    for r in roots:
        if r > ZG:
            ZG = r
    vG = ZG * R_EOS * T_phy / P_phy
    rho_phy_mol = 1 / vG
    rho_phy = rho_phy_mol * Mw
    C_Rs = Rs / Rs_lu
    b_Rs = 0.07780 * Rs * Tc_phy / Pc_phy
    a_Rs = 0.45724 * pw((Rs * Tc_phy), 2) / Pc_phy
    C_as = a_Rs / a_lu
    C_bs = b_Rs / b_lu
    C_aob = C_as / C_bs
    Ct = Cl / math.sqrt(C_aob)
    CT = 1 / (C_Rs / pw(Cl, 2) * pw(Ct, 2))
    T_lu = T_phy / CT
    C_Mw = Mw / Mw_lu
    Cm = pw(Cl, 3) / C_bs
    Crho = Cm / (Cl * Cl * Cl)
    Cn = Cm / C_Mw
    Cu = Cl / Ct
    Cf = Cm / (pw(Ct, 2) * pw(Cl, 2))
    Crho_mol = Cn / pw(Cl, 3)
    rhoin = rho_phy / Crho
    mfp = 1.0 / (math.sqrt(2.0) * Crho_mol * rhoin / Mw_lu * NA * math.pi * (2 * d_mol / 2.0 + 2 * d_mol / 2.0) *
                 (2 * d_mol / 2.0 + 2 * d_mol / 2.0))
    return dict(rho_in=rhoin, mfp=mfp, T_lu=T_lu, a_alpha_lu=a_alpha_lu, Cu=Cu, Cf=Cf)


def pore_properties(pore, dx, mfp):
    """Local pore size and Kn of every pixel (Shape::calculateProperties)."""
    pore = np.ascontiguousarray(pore, dtype=np.int32)
    n = pore.shape[0]
    if pore.shape != (n, n):
        raise ValueError("pore image must be square")
    lp, kn = np.zeros((n, n)), np.zeros((n, n))
    failed = lib().oracle_pore_properties(_p(pore), n, float(dx), float(mfp), _p(lp), _p(kn))
    if failed < 0:
        raise RuntimeError(lib().oracle_grid_error().decode())
    return lp, kn


def image_fields(pore, kn_mean):
    """Kn and local pore size of a pore image whose lattice spacing makes the
    mean Kn over the void pixels kn_mean (Kn = mfp / (H dx) per pixel,
    include/shape.hpp:245-246; mfp of the default 1 nm spacing)."""
    pore = np.ascontiguousarray(pore, dtype=np.int32)
    H, kn_unit = pore_properties(pore, 1.0, 1.0)  # kn_unit = 1 / H
    mfp = units()["mfp"]
    void = pore == 1
    dx = mfp * kn_unit[void].mean() / kn_mean
    kn = np.where(void, kn_unit * mfp / dx, 0.0)
    return dict(pore=pore, kn=kn, locpore=H, dx=float(dx))


def config2_image(index=0):
    """Config-2 image `index` of the benchmark (1024x1024 seeded disks, three
    quadtree levels) from oracle/data, with its fields derived here."""
    d = np.load(HERE / "data" / f"config2_image{index}.npz")
    n = int(d["n"])
    pore = np.unpackbits(d["pore_bits"])[: n * n].reshape(n, n).astype(np.int32)
    out = image_fields(pore, float(d["kn_mean"]))
    out["levels"] = int(d["levels"])
    out["edge_fine"] = int(d["edge_fine"])
    return out


class GridTables:
    """Grid tables of a pore image from the oracle's Grid2D restatement."""

    def __init__(self, pore, kn, locpore, multiblock=True, max_allowed_level=3, edge_fine=False, dx=1e-9,
                 T=300.0, P=2.0e6):
        pore = np.ascontiguousarray(pore, dtype=np.int32)
        n = pore.shape[0]
        kn = np.ascontiguousarray(kn, dtype=np.float64).reshape(n, n)
        locpore = np.ascontiguousarray(locpore, dtype=np.float64).reshape(n, n)
        opt = OracleGridOptions(1 if multiblock else 0, int(max_allowed_level), 1 if edge_fine else 0, float(dx),
                                units(dx, T, P)["mfp"])
        L = lib()
        h = L.oracle_grid_create(_p(pore), _p(kn), _p(locpore), n, C.byref(opt))
        if not h:
            raise RuntimeError(L.oracle_grid_error().decode())
        try:
            g, e = OracleGrid(), OracleGridExtra()
            L.oracle_grid_view(h, C.byref(g), C.byref(e))
            self._read(g, e)
        finally:
            L.oracle_grid_destroy(h)

    def _read(self, g, e):
        def arr(ptr, count, dt, shape=None):
            out = np.zeros(count, dtype=dt)
            if count:
                C.memmove(out.ctypes.data, ptr, count * out.itemsize)
            return out if shape is None else out.reshape(shape)

        N = int(g.n_cells)
        self.n, self.max_level, self.n_cells = int(g.n), int(g.max_level), N
        c = {k: arr(getattr(g, k), N, np.int32) for k in ("x", "y", "level", "type", "is_buffer", "bnd")}
        c["conn"] = arr(g.conn, 9 * N, np.int64, (N, 9))
        c["tau"], c["kn"] = arr(g.tau, N, np.float64), arr(g.kn, N, np.float64)
        c["locpore"], c["lin"] = arr(e.locpore, N, np.float64), arr(e.lin, N, np.int64)
        self.cells = c
        self.links = dict(stream_id=arr(g.stream_id, g.n_stream, np.int64),
                          stream_ic=arr(g.stream_ic, g.n_stream, np.int32),
                          stream_loc=arr(g.stream_loc, g.n_stream, np.int64),
                          wall_id=arr(g.wall_id, g.n_wall, np.int64), wall_ic=arr(g.wall_ic, g.n_wall, np.int32),
                          per_id=arr(g.per_id, g.n_per, np.int64), per_i2=arr(g.per_i2, g.n_per, np.int64),
                          per_ic=arr(g.per_ic, g.n_per, np.int32))
        self.coarse_rows = arr(g.coarse_rows, 6 * g.n_coarse, np.int64, (int(g.n_coarse), 6))
        self.fine_rows = arr(g.fine_rows, 6 * g.n_fine, np.int64, (int(g.n_fine), 6))
        self.parent_child = arr(e.parent_child, 5 * e.n_parent_child, np.int64, (int(e.n_parent_child), 5))
        self.inlet, self.inlet2, self.outlet, self.outlet2 = (int(v) for v in (g.inlet, g.inlet2, g.outlet,
                                                                                g.outlet2))
        self.buffer_wall_links = int(e.buffer_wall_links)

    def lattice_updates(self):
        """Lattice updates of one coarse step: 2^(max_level - level) per non-buffer cell."""
        c = self.cells
        keep = c["is_buffer"] == 0
        return float(np.sum(np.left_shift(1, self.max_level - c["level"][keep]).astype(np.float64)))
