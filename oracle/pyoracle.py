"""ctypes binding of the FP64 CPU oracle (oracle/lbm_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as the
checker and by bench.py's CPU-baseline leg -- never by the product.

The oracle consumes grid tables (oracle.pygrid.GridTables, a
mantiis_gb300.HostGrid or any object with the same attributes) and restates
the reference time step in FP64.
"""
import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liblbm_oracle.so"


class OracleGrid(C.Structure):
    _fields_ = [
        ("n", C.c_int), ("max_level", C.c_int), ("n_cells", C.c_int64),
        ("x", C.c_void_p), ("y", C.c_void_p), ("level", C.c_void_p), ("type", C.c_void_p),
        ("is_buffer", C.c_void_p), ("bnd", C.c_void_p), ("conn", C.c_void_p), ("tau", C.c_void_p),
        ("kn", C.c_void_p),
        ("n_stream", C.c_int64), ("stream_id", C.c_void_p), ("stream_loc", C.c_void_p), ("stream_ic", C.c_void_p),
        ("n_wall", C.c_int64), ("wall_id", C.c_void_p), ("wall_ic", C.c_void_p),
        ("n_per", C.c_int64), ("per_id", C.c_void_p), ("per_i2", C.c_void_p), ("per_ic", C.c_void_p),
        ("n_coarse", C.c_int64), ("n_fine", C.c_int64), ("coarse_rows", C.c_void_p), ("fine_rows", C.c_void_p),
        ("inlet", C.c_int64), ("inlet2", C.c_int64), ("outlet", C.c_int64), ("outlet2", C.c_int64),
    ]


class OracleParams(C.Structure):
    _fields_ = [
        ("simulation", C.c_int), ("collision", C.c_int), ("wall", C.c_int),
        ("fbody", C.c_double), ("rhoin", C.c_double), ("mfp", C.c_double), ("Cl", C.c_double),
        ("T_lu", C.c_double), ("a_alpha_lu", C.c_double), ("tol", C.c_double),
        ("psi_form", C.c_int), ("rho_psi", C.c_double), ("g_ff", C.c_double), ("g_fs", C.c_double),
    ]


_lib = None


def build():
    subprocess.run(["make", "-s", "-C", str(HERE), "own"], check=True)


def lib():
    global _lib
    if _lib is None:
        build()  # make: rebuilds only what is out of date
        L = C.CDLL(str(LIB))
        L.oracle_create.restype = C.c_void_p
        L.oracle_create.argtypes = [C.POINTER(OracleGrid), C.POINTER(OracleParams), C.c_void_p]
        L.oracle_run.restype = C.c_int
        L.oracle_run.argtypes = [C.c_void_p, C.c_int, C.c_int]
        L.oracle_fields.argtypes = [C.c_void_p] + [C.c_void_p] * 4
        L.oracle_residuals.restype = C.c_int64
        L.oracle_residuals.argtypes = [C.c_void_p, C.c_void_p, C.c_int64]
        L.oracle_destroy.argtypes = [C.c_void_p]
        L.oracle_threads.restype = C.c_int
        L.oracle_threads.argtypes = [C.c_int]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


class Oracle:
    """FP64 reference-algorithm run on a grid (HostGrid tables)."""

    def __init__(self, grid, simulation=0, collision=2, wall=2, fbody=1e-8, rhoin=None, mfp=None, dx=1e-9,
                 T_lu=0.0, a_alpha_lu=0.0, tol=1e-10, psi_form=0, rho_psi=1.0, g_ff=-1.0, g_fs=-12.7,
                 rho_init=None, threads=1):
        c = grid.cells
        self._keep = []

        def keep(a, dt):
            a = np.ascontiguousarray(a, dtype=dt)
            self._keep.append(a)
            return _p(a)

        g = OracleGrid()
        g.n, g.max_level, g.n_cells = grid.n, grid.max_level, grid.n_cells
        for k in ("x", "y", "level", "type", "is_buffer", "bnd"):
            setattr(g, k, keep(c[k], np.int32))
        g.conn = keep(c["conn"], np.int64)
        g.tau = keep(c["tau"], np.float64)
        g.kn = keep(c["kn"], np.float64)
        L = grid.links
        g.n_stream = len(L["stream_id"])
        g.stream_id, g.stream_loc = keep(L["stream_id"], np.int64), keep(L["stream_loc"], np.int64)
        g.stream_ic = keep(L["stream_ic"], np.int32)
        g.n_wall = len(L["wall_id"])
        g.wall_id, g.wall_ic = keep(L["wall_id"], np.int64), keep(L["wall_ic"], np.int32)
        g.n_per = len(L["per_id"])
        g.per_id, g.per_i2 = keep(L["per_id"], np.int64), keep(L["per_i2"], np.int64)
        g.per_ic = keep(L["per_ic"], np.int32)
        g.n_coarse, g.n_fine = len(grid.coarse_rows), len(grid.fine_rows)
        g.coarse_rows = keep(grid.coarse_rows if len(grid.coarse_rows) else np.zeros((1, 6)), np.int64)
        g.fine_rows = keep(grid.fine_rows if len(grid.fine_rows) else np.zeros((1, 6)), np.int64)
        g.inlet, g.inlet2, g.outlet, g.outlet2 = grid.inlet, grid.inlet2, grid.outlet, grid.outlet2
        p = OracleParams(simulation, collision, wall, fbody, rhoin, mfp, dx, T_lu, a_alpha_lu, tol, psi_form,
                         rho_psi, g_ff, g_fs)
        lib().oracle_threads(threads)
        ri = None
        if rho_init is not None:
            ri = keep(rho_init, np.float64)
        self._h = lib().oracle_create(C.byref(g), C.byref(p), ri)
        self.n_cells = grid.n_cells

    def run(self, n, break_on_tol=False):
        return lib().oracle_run(self._h, int(n), 1 if break_on_tol else 0)

    def fields(self):
        N = self.n_cells
        rho, ux, uy, f = np.zeros(N), np.zeros(N), np.zeros(N), np.zeros(9 * N)
        lib().oracle_fields(self._h, _p(rho), _p(ux), _p(uy), _p(f))
        return dict(rho=rho, ux=ux, uy=uy, f=f.reshape(N, 9))

    def residuals(self):
        n = lib().oracle_residuals(self._h, None, 0)
        out = np.zeros(max(n, 1))
        lib().oracle_residuals(self._h, _p(out), n)
        return out[:n]

    def close(self):
        if self._h:
            lib().oracle_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


def for_grid(grid, sim="transport", dx=1e-9, T=300.0, P=2.0e6, fbody=1e-8, **kw):
    """Oracle with the physical constants of (dx, T, P) (the oracle's own
    restatement of the reference's unit system, oracle/pygrid.py)."""
    from .pygrid import units

    u = units(dx, T, P)
    simulation = {"transport": 0, "adsorption": 1, "coupled": 2}[sim]
    if simulation == 1:
        kw.setdefault("collision", 1)
        kw.setdefault("wall", 0)
    return Oracle(grid, simulation=simulation, fbody=fbody, rhoin=u["rho_in"], mfp=u["mfp"], dx=dx,
                  T_lu=u["T_lu"], a_alpha_lu=u["a_alpha_lu"], **kw)
