"""mgpu_set_equilibrium_noalloc (static staging array, no allocation) against
mgpu_set_equilibrium.  Both launch the same kernel on the same FP64 inputs, so
the states agree far inside the tests' tolerance for populations (1e-6 of the
inlet density).  This file is collected last and needs no other test before it."""
import re

import numpy as np
import pytest
from conftest import ROOT

from mantiis_gb300 import Solver, default_params
from mantiis_gb300.native import NOALLOC_MAX_CELLS, MantiisError

RHO_IN = 0.2355


def fields(n, seed):
    rng = np.random.default_rng(seed)
    rho = RHO_IN * (1.0 + 1e-3 * rng.standard_normal(n))
    return rho, 1e-4 * rng.standard_normal(n), 1e-4 * rng.standard_normal(n)


def state_err(a, b):
    ca, cb = a.cells(with_f=True), b.cells(with_f=True)
    e_f = np.abs(ca["f"] - cb["f"]).max() / RHO_IN
    e_ux = np.abs(ca["ux"] - cb["ux"]).max() / max(np.abs(ca["ux"]).max(), 1e-30)
    return e_f, e_ux


def test_max_cells_matches_header():
    text = (ROOT / "include" / "mantiis_gpu.h").read_text()
    m = re.search(r"#define MGPU_NOALLOC_MAX_CELLS \(1 << (\d+)\)", text)
    assert m and NOALLOC_MAX_CELLS == 1 << int(m.group(1))


def test_cell_field_sizes_checked_before_any_call():
    # short arrays would make the C side read past them: the binding refuses
    s = Solver.__new__(Solver)
    s._h, s.n_cells = None, 10
    ok, short = np.zeros(10), np.zeros(9)
    for fn in (s.set_equilibrium, s.set_equilibrium_noalloc):
        with pytest.raises(ValueError, match="expected n_cells = 10"):
            fn(ok, short, ok)


@pytest.mark.gpu
def test_noalloc_matches_set_equilibrium_twice(fixture64):
    import torch

    # multi-block: the kernel also fills the interface buffers
    p = default_params(dx=1e-9, multiblock=1)
    img = (fixture64["pore"], fixture64["kn"], fixture64["locpore"])
    ref, got, other, other_ref = Solver(*img, p), Solver(*img, p), Solver(*img, p), Solver(*img, p)
    n = ref.n_cells
    # set_equilibrium creates its staging buffers on first use; do that before
    # the device's free memory is read
    ref.set_equilibrium(*fields(n, 0))
    other_ref.set_equilibrium(*fields(n, 0))

    def noalloc(s, fl):
        # neither the device's free memory nor the context's own device memory
        # changes across the call
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        bytes_before = s.refresh_info()["device_bytes"]
        s.set_equilibrium_noalloc(*fl)
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info()[0] == free_before
        assert s.refresh_info()["device_bytes"] == bytes_before

    for seed in (1, 2):  # two calls in a row on the same context
        fl = fields(n, seed)
        noalloc(got, fl)
        ref.set_equilibrium(*fl)
        e_f, e_ux = state_err(ref, got)
        assert e_f < 1e-6 and e_ux < 1e-4
        ref.advance(10)
        got.advance(10)
        e_f, e_ux = state_err(ref, got)
        assert e_f < 1e-6 and e_ux < 1e-4
    # a second context on the same device reuses the staging array: its state
    # matches set_equilibrium's on the same fields, and the first context's
    # state is still its own
    fl = fields(n, 3)
    noalloc(other, fl)
    other_ref.set_equilibrium(*fl)
    e_f, e_ux = state_err(other_ref, other)
    assert e_f < 1e-6 and e_ux < 1e-4
    e_f, _ = state_err(ref, got)
    assert e_f < 1e-6


@pytest.mark.gpu
def test_noalloc_rejects_grid_above_limit():
    n = 1100  # channel: 1100 x 1098 fluid cells > 2^20
    pore = np.ones((n, n), np.int32)
    pore[0, :] = pore[-1, :] = 0
    kn = np.where(pore == 1, 0.1, 0.0)
    lp = np.where(pore == 1, 7.73, 0.0)
    s = Solver(pore, kn, lp, default_params(dx=1e-9))
    assert s.n_cells > NOALLOC_MAX_CELLS
    with pytest.raises(MantiisError, match="exceed the static staging area") as ei:
        s.set_equilibrium_noalloc(*fields(s.n_cells, 4))
    assert ei.value.code == -1  # MGPU_E_ARG
