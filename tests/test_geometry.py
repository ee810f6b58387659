"""Local pore size and Knudsen number on the host against the reference's own
Shape::calculateProperties (include/shape.hpp:127-251), run on four images by
tests/golden/make_golden.py (refprops.npz).  No GPU."""
import numpy as np
import pytest
from conftest import load

from mantiis_gb300 import MantiisError, pore_properties

CASES = ("fx64", "disks128", "disks256", "bigpores256")


@pytest.fixture(scope="module")
def refprops():
    return load("refprops.npz")


def check_against_reference(lp, kn, ref, name):
    # LocPore is twice a float distance: identical.  Kn = mfp / LocPore / dx: the
    # reference is built with -Ofast, which may round the two divisions
    # differently, so allow 2 ulp.
    assert np.array_equal(lp, ref[f"{name}_locpore"]), name
    want = ref[f"{name}_kn"]
    assert np.all((kn == 0) == (want == 0)), name
    nz = want != 0
    assert np.max(np.abs(kn[nz] - want[nz]) / want[nz]) <= 4.5e-16, name


@pytest.mark.parametrize("name", CASES)
def test_host_properties_match_reference(refprops, name):
    pore = refprops[f"{name}_pore"].astype(np.int32)
    lp, kn = pore_properties(pore, float(refprops["dx"]), float(refprops["mfp"]))
    check_against_reference(lp, kn, refprops, name)


def test_solid_pixels_get_zero(refprops):
    pore = refprops["bigpores256_pore"].astype(np.int32)
    lp, kn = pore_properties(pore, 1e-9, 5e-9)
    assert np.all(lp[pore != 1] == 0) and np.all(kn[pore != 1] == 0)
    assert np.all(lp[pore == 1] > 0)


def test_too_small_image_rejected():
    with pytest.raises(MantiisError):
        pore_properties(np.ones((3, 3), np.int32), 1e-9, 5e-9)


EXTRA = ("noise96", "blobs128", "diagonal128")


@pytest.mark.parametrize("name", EXTRA)
def test_host_properties_match_reference_irregular(name):
    # salt-and-pepper noise, smoothed blobs, thin diagonal channels
    ref = load("refprops_extra.npz")
    pore = ref[f"{name}_pore"].astype(np.int32)
    lp, kn = pore_properties(pore, float(ref["dx"]), float(ref["mfp"]))
    check_against_reference(lp, kn, ref, name)
