"""ctypes binding of libmantiis_gpu.so (the C ABI declared in include/mantiis_gpu.h).

The library is built in-tree by mantiis_gb300.build.build(); importing this
module loads it and fails loudly if it is missing.  Solver objects drive the
GPU; HostGrid, units(), pore_properties() and generate_disks() are host-only
and work without a GPU.
"""
import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "lib" / "libmantiis_gpu.so"

SIM_TRANSPORT, SIM_ADSORPTION, SIM_COUPLED = 0, 1, 2
NOALLOC_MAX_CELLS = 1 << 20  # MGPU_NOALLOC_MAX_CELLS


class Params(C.Structure):
    _fields_ = [
        ("simulation", C.c_int),
        ("collision", C.c_int),
        ("wall", C.c_int),
        ("multiblock", C.c_int),
        ("max_allowed_level", C.c_int),
        ("dx", C.c_double),
        ("fbody", C.c_double),
        ("T", C.c_double),
        ("P", C.c_double),
        ("tol", C.c_double),
        ("psi_form", C.c_int),
        ("rho_psi", C.c_double),
        ("g_ff", C.c_double),
        ("g_fs", C.c_double),
        ("rho_init", C.c_double),
        ("rho_noise", C.c_double),
        ("seed", C.c_uint64),
        ("check_every", C.c_int),
        ("edge_fine", C.c_int),
        ("plain_path", C.c_int),
        ("concurrent", C.c_int),
    ]


class Info(C.Structure):
    _fields_ = [
        ("n", C.c_int),
        ("max_level", C.c_int),
        ("n_cells", C.c_int64),
        ("n_buffer_cells", C.c_int64),
        ("n_special", C.c_int64),
        ("lu_per_step", C.c_double),
        ("buffer_lu_per_step", C.c_double),
        ("rho_in", C.c_double),
        ("mfp", C.c_double),
        ("tau_mean", C.c_double),
        ("device_bytes", C.c_int64),
        ("grid_undefined_cases", C.c_int64),
        ("plain_path", C.c_int),
        ("pad_", C.c_int),
        ("autotune_us", C.c_double * 3),
    ]


class MantiisError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"mantiis_gpu error {code}: {msg}")
        self.code = code


_lib = None

P = C.c_void_p
I32P = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
I64P = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
F64P = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")

# every entry point of include/mantiis_gpu.h: name -> (restype, argtypes)
SIGNATURES = {
    "mgpu_default_params": (None, [C.POINTER(Params)]),
    "mgpu_create": (C.c_int, [I32P, F64P, F64P, C.c_int, C.POINTER(Params), C.POINTER(P)]),
    "mgpu_create_from_folder": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(Params), C.POINTER(P)]),
    "mgpu_destroy": (C.c_int, [P]),
    "mgpu_get_info": (C.c_int, [P, C.POINTER(Info)]),
    "mgpu_run": (C.c_int, [P, C.c_int, C.POINTER(C.c_int)]),
    "mgpu_advance": (C.c_int, [P, C.c_int]),
    "mgpu_advance_graph": (C.c_int, [P, C.c_int]),
    "mgpu_sync": (C.c_int, [P]),
    "mgpu_step_level": (C.c_int, [P, C.c_int, C.c_int]),
    "mgpu_level_info": (C.c_int, [P, C.c_int, I64P]),
    "mgpu_time": (C.c_int, [P, C.POINTER(C.c_int64)]),
    "mgpu_residuals": (C.c_int, [P, P, C.c_int64, C.POINTER(C.c_int64)]),
    "mgpu_download_cells": (C.c_int, [P, P, P, P, P]),
    "mgpu_download_pixels": (C.c_int, [P, P, P, P, P]),
    "mgpu_observables": (C.c_int, [P, F64P]),
    "mgpu_reconstructed": (C.c_int, [P, I64P]),
    "mgpu_cell_positions": (C.c_int, [P, P, P, P]),
    "mgpu_set_equilibrium": (C.c_int, [P, F64P, F64P, F64P]),
    "mgpu_set_distributions": (C.c_int, [P, F64P, C.c_int, C.c_int64]),
    "mgpu_set_equilibrium_noalloc": (C.c_int, [P, F64P, F64P, F64P]),
    "mgpu_set_stream": (C.c_int, [P, P]),
    "mgpu_launch_count": (C.c_int64, [P]),
    "mgpu_batch_create": (C.c_int, [C.POINTER(P), C.c_int, C.POINTER(P)]),
    "mgpu_batch_advance": (C.c_int, [P, C.c_int]),
    "mgpu_batch_observables": (C.c_int, [P, F64P]),
    "mgpu_batch_set_stream": (C.c_int, [P, P]),
    "mgpu_batch_set_engine": (C.c_int, [P, C.c_int, C.c_int]),
    "mgpu_set_engine": (C.c_int, [P, C.c_int]),
    "mgpu_batch_sync": (C.c_int, [P]),
    "mgpu_batch_launch_count": (C.c_int64, [P]),
    "mgpu_batch_destroy": (C.c_int, [P]),
    "mgpu_last_error": (C.c_char_p, [P]),
    "mgpu_global_error": (C.c_char_p, []),
    "mgpu_grid_build": (C.c_int, [I32P, F64P, F64P, C.c_int, C.POINTER(Params), C.POINTER(P)]),
    "mgpu_grid_build_from_folder": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(Params), C.POINTER(P)]),
    "mgpu_grid_sizes": (C.c_int, [P, I64P]),
    "mgpu_grid_cells": (C.c_int, [P, P, P, P, P, P, P, P, P, P, P, P]),
    "mgpu_grid_links": (C.c_int, [P, P, P, P, P, P, P, P, P]),
    "mgpu_grid_interfaces": (C.c_int, [P, P, P, P]),
    "mgpu_grid_diagnostics": (C.c_int, [P, I64P]),
    "mgpu_grid_destroy": (C.c_int, [P]),
    "mgpu_host_error": (C.c_char_p, []),
    "mgpu_units": (C.c_int, [C.c_double, C.c_double, C.c_double, F64P]),
    "mgpu_pore_properties": (C.c_int, [I32P, C.c_int, C.c_double, C.c_double, F64P, F64P]),
    "mgpu_pore_properties_gpu": (C.c_int, [I32P, C.c_int, C.c_double, C.c_double, F64P, F64P,
                                           C.POINTER(C.c_int64), C.c_void_p]),
    "mgpu_generate_disks": (C.c_int, [C.c_int, C.c_double, C.c_double, C.c_double, C.c_uint64, I32P]),
    "mgpu_generate_disks_ex": (C.c_int, [C.c_int, C.c_double, C.c_double, C.c_double, C.c_uint64, C.c_int, I32P]),
}


def lib():
    """Loads libmantiis_gpu.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(
                f"{LIB_PATH} is missing: build it with mantiis_gb300.build.build() (nvcc, sm_103a) first")
        L = C.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def default_params(**kw):
    p = Params()
    lib().mgpu_default_params(C.byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise KeyError(f"unknown parameter {k}")
        setattr(p, k, v)
    return p


def units(dx=1e-9, T=300.0, P=2.0e6):
    out = np.zeros(6)
    lib().mgpu_units(dx, T, P, out)
    return dict(rho_in=out[0], mfp=out[1], T_lu=out[2], a_alpha_lu=out[3], Cu=out[4], Cf=out[5])


def _host_check(rc):
    if rc != 0:
        raise MantiisError(rc, lib().mgpu_host_error().decode())


def pore_properties(pore, dx, mfp):
    pore = np.ascontiguousarray(pore, dtype=np.int32)
    n = pore.shape[0]
    lp = np.zeros((n, n))
    kn = np.zeros((n, n))
    _host_check(lib().mgpu_pore_properties(pore.reshape(-1), n, dx, mfp, lp.reshape(-1), kn.reshape(-1)))
    return lp, kn


def pore_properties_gpu(pore, dx, mfp, stream=None, return_iterations=False):
    """pore_properties computed by the GPU kernels on the current device (same
    results bit for bit); optionally also the number of thinning iterations."""
    pore = np.ascontiguousarray(pore, dtype=np.int32)
    n = pore.shape[0]
    if pore.shape != (n, n):
        raise ValueError("pore image must be square")
    lp = np.zeros((n, n))
    kn = np.zeros((n, n))
    it = C.c_int64(0)
    rc = lib().mgpu_pore_properties_gpu(pore.reshape(-1), n, dx, mfp, lp.reshape(-1), kn.reshape(-1),
                                        C.byref(it), stream)
    if rc != 0:
        raise MantiisError(rc, lib().mgpu_global_error().decode())
    return (lp, kn, it.value) if return_iterations else (lp, kn)


def generate_disks(n, rmin, rmax, porosity, seed, periodic_x=False, open_x_edges=False, edge_margin=2):
    """Seeded disk packing; periodic_x wraps the disks across the x-periodic
    edge, open_x_edges keeps disks off the `edge_margin` (2 or 3) columns at
    either x edge."""
    if edge_margin not in (2, 3):
        raise ValueError("edge_margin must be 2 or 3")
    out = np.zeros(n * n, dtype=np.int32)
    flags = (1 if periodic_x else 0) | ((4 if edge_margin == 3 else 2) if open_x_edges else 0)
    _host_check(lib().mgpu_generate_disks_ex(n, rmin, rmax, porosity, seed, flags, out))
    return out.reshape(n, n)


def _image_args(pore, kn, locpore):
    pore = np.ascontiguousarray(pore, dtype=np.int32)
    n = pore.shape[0]
    if pore.shape != (n, n):
        raise ValueError("pore image must be square")
    kn = np.ascontiguousarray(kn, dtype=np.float64).reshape(n, n)
    locpore = np.ascontiguousarray(locpore, dtype=np.float64).reshape(n, n)
    return pore, kn, locpore, n


class HostGrid:
    """Grid tables built on the host (reference cell order); no GPU involved."""

    def __init__(self, pore=None, kn=None, locpore=None, params=None, folder=None, n=None):
        params = params or default_params()
        h = C.c_void_p()
        if folder is not None:
            _host_check(lib().mgpu_grid_build_from_folder(str(folder).encode(), int(n), C.byref(params), C.byref(h)))
        else:
            pore, kn, locpore, n = _image_args(pore, kn, locpore)
            _host_check(lib().mgpu_grid_build(pore.reshape(-1), kn.reshape(-1), locpore.reshape(-1), n,
                                              C.byref(params), C.byref(h)))
        self.n = int(n)
        try:
            self._read(h)
        finally:
            lib().mgpu_grid_destroy(h)

    def _read(self, h):
        L = lib()
        s = np.zeros(12, dtype=np.int64)
        L.mgpu_grid_sizes(h, s)
        N = int(s[0])
        self.n_cells, self.max_level = N, int(s[1])
        self.inlet, self.inlet2, self.outlet, self.outlet2 = (int(v) for v in s[8:12])
        c = {k: np.zeros(N, np.int32) for k in ("x", "y", "level", "type", "is_buffer", "bnd")}
        c["conn"] = np.zeros(9 * N, np.int64)
        for k in ("tau", "kn", "locpore"):
            c[k] = np.zeros(N)
        c["lin"] = np.zeros(N, np.int64)
        L.mgpu_grid_cells(h, *(_ptr(c[k]) for k in ("x", "y", "level", "type", "is_buffer", "bnd", "conn", "tau",
                                                     "kn", "locpore", "lin")))
        c["conn"] = c["conn"].reshape(N, 9)
        self.cells = c
        ns, nw, npr = int(s[2]), int(s[3]), int(s[4])
        k = dict(stream_id=np.zeros(ns, np.int64), stream_ic=np.zeros(ns, np.int32), stream_loc=np.zeros(ns, np.int64),
                 wall_id=np.zeros(nw, np.int64), wall_ic=np.zeros(nw, np.int32), per_id=np.zeros(npr, np.int64),
                 per_i2=np.zeros(npr, np.int64), per_ic=np.zeros(npr, np.int32))
        L.mgpu_grid_links(h, *(_ptr(k[n]) for n in ("stream_id", "stream_ic", "stream_loc", "wall_id", "wall_ic",
                                                     "per_id", "per_i2", "per_ic")))
        self.links = k
        self.coarse_rows = np.zeros((int(s[5]), 6), np.int64)
        self.fine_rows = np.zeros((int(s[6]), 6), np.int64)
        self.parent_child = np.zeros((int(s[7]), 5), np.int64)
        L.mgpu_grid_interfaces(h, _ptr(self.coarse_rows), _ptr(self.fine_rows), _ptr(self.parent_child))
        d = np.zeros(5, np.int64)
        L.mgpu_grid_diagnostics(h, d)
        self.diagnostics = dict(buffer_wall_links=int(d[0]), fine_parent_missing_nbr=int(d[1]),
                                coarse_missing_child=int(d[2]), fine_group_unmatched=int(d[3]),
                                pore_search_failed=int(d[4]))


class Solver:
    """One pore image on the GPU (include/mantiis_gpu.h, mgpu_ctx)."""

    def __init__(self, pore=None, kn=None, locpore=None, params=None, folder=None, n=None, **kw):
        self._h = None
        params = params or default_params()
        for k, v in kw.items():
            setattr(params, k, v)
        self.params = params
        h = C.c_void_p()
        L = lib()
        if folder is not None:
            rc = L.mgpu_create_from_folder(str(folder).encode(), int(n), C.byref(params), C.byref(h))
        else:
            pore, kn, locpore, n = _image_args(pore, kn, locpore)
            rc = L.mgpu_create(pore.reshape(-1), kn.reshape(-1), locpore.reshape(-1), n, C.byref(params), C.byref(h))
        if rc != 0:
            raise MantiisError(rc, L.mgpu_global_error().decode())
        self._h = h
        self.refresh_info()
        self.n = self.info["n"]
        self.n_cells = self.info["n_cells"]

    def refresh_info(self):
        """Re-reads mgpu_get_info (device_bytes grows when buffers are created on
        first use, e.g. by set_equilibrium) into self.info and returns it."""
        inf = Info()
        self._check(lib().mgpu_get_info(self._h, C.byref(inf)))
        self.info = {f: getattr(inf, f) for f, _ in Info._fields_ if f != "pad_"}
        self.info["autotune_us"] = tuple(self.info["autotune_us"])
        return self.info

    def _check(self, rc):
        if rc != 0:
            raise MantiisError(rc, lib().mgpu_last_error(self._h).decode())

    def run(self, n_steps):
        done = C.c_int(0)
        self._check(lib().mgpu_run(self._h, int(n_steps), C.byref(done)))
        return done.value

    def advance(self, n_steps):
        self._check(lib().mgpu_advance(self._h, int(n_steps)))

    def advance_graph(self, n_steps):
        """Enqueues n coarse steps from a captured CUDA graph; returns without waiting."""
        self._check(lib().mgpu_advance_graph(self._h, int(n_steps)))

    def set_engine(self, engine):
        """Adsorption step engine (mgpu_set_engine): 1 (default) the steps of a
        call in one cooperative launch, 0 launches per pass."""
        self._check(lib().mgpu_set_engine(self._h, int(engine)))

    def step_level(self, level, n):
        """Profiling aid: n substeps of one level alone (see mgpu_step_level)."""
        self._check(lib().mgpu_step_level(self._h, int(level), int(n)))

    def level_info(self, level):
        out = np.zeros(4, np.int64)
        self._check(lib().mgpu_level_info(self._h, int(level), out))
        return dict(active=int(out[0]), active_real=int(out[1]), tiles=int(out[2]), substeps=int(out[3]))

    def sync(self):
        self._check(lib().mgpu_sync(self._h))

    @property
    def time(self):
        t = C.c_int64(0)
        lib().mgpu_time(self._h, C.byref(t))
        return t.value

    def residuals(self):
        cnt = C.c_int64(0)
        lib().mgpu_residuals(self._h, None, 0, C.byref(cnt))
        out = np.zeros(cnt.value)
        lib().mgpu_residuals(self._h, _ptr(out), cnt.value, C.byref(cnt))
        return out

    def cells(self, with_f=False, out=None):
        """FP64 fields per cell (mgpu_download_cells); `out` may hold float64
        arrays rho, ux, uy of n_cells each (e.g. views of pinned host memory) to
        read into."""
        N = self.n_cells
        if out is not None:
            rho, ux, uy = (np.ascontiguousarray(out[k]) for k in ("rho", "ux", "uy"))
            if not all(a.dtype == np.float64 and a.size == N for a in (rho, ux, uy)):
                raise ValueError("out arrays must be float64 of n_cells each")
            if any(a is not out[k] for a, k in zip((rho, ux, uy), ("rho", "ux", "uy"))):
                raise ValueError("out arrays must be contiguous")
        else:
            rho, ux, uy = np.zeros(N), np.zeros(N), np.zeros(N)
        f = np.zeros(9 * N) if with_f else None
        self._check(lib().mgpu_download_cells(self._h, _ptr(rho), _ptr(ux), _ptr(uy), _ptr(f)))
        out = dict(rho=rho, ux=ux, uy=uy)
        if with_f:
            out["f"] = f.reshape(N, 9)
        return out

    def pixels(self, with_f=False):
        nn = self.n * self.n
        rho, ux, uy = np.zeros(nn), np.zeros(nn), np.zeros(nn)
        f = np.zeros(9 * nn) if with_f else None
        self._check(lib().mgpu_download_pixels(self._h, _ptr(rho), _ptr(ux), _ptr(uy), _ptr(f)))
        out = dict(rho=rho.reshape(self.n, self.n), ux=ux.reshape(self.n, self.n), uy=uy.reshape(self.n, self.n))
        if with_f:
            out["f"] = f.reshape(self.n, self.n, 9)
        return out

    def observables(self):
        out = np.zeros(4)
        self._check(lib().mgpu_observables(self._h, out))
        return dict(mean_ux=out[0], permeability=out[1], mass=out[2], residual=out[3])

    def cell_positions(self):
        """Top-left pixel (x, y) and level of every cell, in cell order."""
        x, y, lv = (np.zeros(self.n_cells, np.int32) for _ in range(3))
        self._check(lib().mgpu_cell_positions(self._h, _ptr(x), _ptr(y), _ptr(lv)))
        return x, y, lv

    def reconstructed(self):
        out = np.zeros(self.n * self.n, np.int64)
        self._check(lib().mgpu_reconstructed(self._h, out))
        return out.reshape(self.n, self.n)

    def _cell_fields(self, rho, ux, uy):
        a = [np.ascontiguousarray(v, dtype=np.float64).reshape(-1) for v in (rho, ux, uy)]
        for name, v in zip(("rho", "ux", "uy"), a):
            if v.size != self.n_cells:
                raise ValueError(f"{name} holds {v.size} values, expected n_cells = {self.n_cells}")
        return a

    def set_equilibrium(self, rho, ux, uy):
        self._check(lib().mgpu_set_equilibrium(self._h, *self._cell_fields(rho, ux, uy)))

    def set_distributions(self, f, layout="cells", t=0):
        """Restart from populations (mgpu_set_distributions): f of
        download_cells (layout "cells", 9 per cell) or of f.txt / pixels()
        (layout "pixels", 9 per pixel); stepping continues from time step t."""
        f = np.ascontiguousarray(f, dtype=np.float64).reshape(-1)
        want = 9 * (self.n_cells if layout == "cells" else self.n * self.n)
        if layout not in ("cells", "pixels") or f.size != want:
            raise ValueError(f"expected {want} populations for layout {layout!r}, got {f.size}")
        self._check(lib().mgpu_set_distributions(self._h, f, 0 if layout == "cells" else 1, int(t)))

    def set_equilibrium_noalloc(self, rho, ux, uy):
        """set_equilibrium staged through the library's static device array
        (mgpu_set_equilibrium_noalloc): no allocation, at most NOALLOC_MAX_CELLS cells."""
        self._check(lib().mgpu_set_equilibrium_noalloc(self._h, *self._cell_fields(rho, ux, uy)))

    def set_stream(self, stream_handle):
        self._check(lib().mgpu_set_stream(self._h, C.c_void_p(int(stream_handle) if stream_handle else 0)))

    @property
    def launches(self):
        return int(lib().mgpu_launch_count(self._h))

    def close(self):
        if self._h:
            lib().mgpu_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class Batch:
    """Several Solver contexts stepped together (include/mantiis_gpu.h, mgpu_batch):
    one launch per phase over every image, two coarse steps per CUDA graph."""

    def __init__(self, solvers):
        self._h = None
        self.solvers = list(solvers)
        self.stream = None  # as last set (set_stream)
        self.engine = None  # (engine, group) as last set (set_engine)
        arr = (P * len(self.solvers))(*[s._h for s in self.solvers])
        h = C.c_void_p()
        rc = lib().mgpu_batch_create(arr, len(self.solvers), C.byref(h))
        if rc != 0:
            raise MantiisError(rc, lib().mgpu_global_error().decode())
        self._h = h

    def _check(self, rc):
        if rc != 0:
            raise MantiisError(rc, lib().mgpu_global_error().decode())

    def advance(self, n_steps):
        """Enqueues n coarse steps of every image; returns without waiting."""
        self._check(lib().mgpu_batch_advance(self._h, int(n_steps)))

    def observables(self):
        out = np.zeros(4 * len(self.solvers))
        self._check(lib().mgpu_batch_observables(self._h, out))
        o = out.reshape(-1, 4)
        return [dict(mean_ux=r[0], permeability=r[1], mass=r[2], residual=r[3]) for r in o]

    def set_stream(self, stream_handle):
        self._check(lib().mgpu_batch_set_stream(self._h, C.c_void_p(int(stream_handle) if stream_handle else 0)))
        self.stream = stream_handle

    def set_engine(self, engine, group=0):
        """engine 0: per-image phase launches on concurrent streams; 1: one
        persistent launch per coarse step over all images (mgpu_batch_set_engine),
        interleaving `group` images at a time (0 = all)."""
        self._check(lib().mgpu_batch_set_engine(self._h, int(engine), int(group)))
        self.engine = (int(engine), int(group))

    def sync(self):
        self._check(lib().mgpu_batch_sync(self._h))

    @property
    def launches(self):
        return int(lib().mgpu_batch_launch_count(self._h))

    def close(self):
        if self._h:
            lib().mgpu_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
