"""GPU pore-property pipeline (mgpu_pore_properties_gpu): bit-packed Zhang-Suen
thinning, exact distance transforms and the nearest-skeleton search give the
reference's LocPore and Kn (refprops.npz, from Shape::calculateProperties,
include/shape.hpp:127-251) and equal the host pipeline bit for bit on larger
and ragged images."""
import numpy as np
import pytest
from conftest import load
from test_geometry import CASES, check_against_reference

from mantiis_gb300 import MantiisError, generate_disks, pore_properties, pore_properties_gpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def refprops():
    return load("refprops.npz")


@pytest.mark.parametrize("name", CASES)
def test_gpu_properties_match_reference(refprops, name):
    pore = refprops[f"{name}_pore"].astype(np.int32)
    lp, kn = pore_properties_gpu(pore, float(refprops["dx"]), float(refprops["mfp"]))
    check_against_reference(lp, kn, refprops, name)


def bit_equal(pore):
    lp_h, kn_h = pore_properties(pore, 2e-9, 6e-9)
    lp_g, kn_g, iters = pore_properties_gpu(pore, 2e-9, 6e-9, return_iterations=True)
    assert np.array_equal(lp_g, lp_h) and np.array_equal(kn_g, kn_h)
    return iters


@pytest.mark.parametrize("n,seed,open_edges", [(100, 7, False), (333, 8, True), (1024, 9, True)])
def test_gpu_equals_host(n, seed, open_edges):
    # 100 and 333: the padded width 3n is not a multiple of the 32-pixel word
    pore = generate_disks(n, max(2, n // 64), max(4, n // 16), 0.6, seed, open_x_edges=open_edges)
    assert bit_equal(pore) >= 1


def test_gpu_edge_images():
    rng = np.random.default_rng(3)
    # salt-and-pepper noise: many tiny components and one-pixel pores
    bit_equal((rng.random((96, 96)) < 0.55).astype(np.int32))
    # all void: no solid pixel, the wall distance is the float maximum
    bit_equal(np.ones((64, 64), np.int32))
    # all solid: nothing to compute
    lp, kn = pore_properties_gpu(np.zeros((64, 64), np.int32), 1e-9, 5e-9)
    assert not lp.any() and not kn.any()
    # smallest accepted side, and pixel values other than 0/1 (not void, but
    # foreground of the wall distance, as in the reference)
    bit_equal(np.array([[0, 1, 1, 0], [1, 1, 1, 1], [1, 2, 1, 1], [0, 1, 1, 0]], np.int32))


def test_gpu_rejects_bad_side():
    with pytest.raises(MantiisError):
        pore_properties_gpu(np.ones((3, 3), np.int32), 1e-9, 5e-9)
