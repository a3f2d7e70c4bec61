"""GPU: the on-device microstructure generators (agb_gen_*) against the host
generators of alamo_gb300.microstructure on the same random draws."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_voronoi_device_equals_host(gpu_lib):
    from alamo_gb300 import microstructure as M
    n = 40
    ddw_h, ids_h, _ = M.voronoi_cubic(n, ngrains=16, seed=11)
    ddw_d, ids_d, _ = M.voronoi_cubic_device(n, ngrains=16, seed=11)
    assert np.array_equal(ids_d.cpu().numpy(), ids_h)           # same grain for every node
    assert np.array_equal(ddw_d.cpu().numpy(), ddw_h)           # gathered moduli, bit for bit


@pytest.mark.parametrize("q", [0, 1, 2, 5])
def test_ellipsoids_device_matches_host(gpu_lib, q):
    from alamo_gb300 import microstructure as M
    n_h, ddw_h, F0_h = M.rve_problem(q, seed=7, edges=(24, 32))
    n_d, ddw_d, F0_d = M.rve_problem_device(q, seed=7, edges=(24, 32))
    assert n_h == n_d and np.array_equal(F0_h, F0_d)
    d = ddw_d.cpu().numpy()
    assert np.abs(d - ddw_h).max() <= 1e-12 * np.abs(ddw_h).max()


def test_sphere_device_matches_host(gpu_lib):
    from alamo_gb300 import microstructure as M
    ddw_h, F0_h = M.sphere_inclusion(32)
    ddw_d, F0_d = M.sphere_inclusion_device(32)
    assert np.abs(ddw_d.cpu().numpy() - ddw_h).max() <= 1e-13
    assert np.abs(F0_d.cpu().numpy() - F0_h).max() <= 1e-16


def test_generator_rejects_bad_arguments(gpu_lib):
    import ctypes
    from alamo_gb300._lib import AGB_BADARG, lib
    n = (ctypes.c_int * 3)(0, 4, 4)
    out = np.zeros(2 * 125)
    assert lib().agb_gen_sphere(n, 0.25, 1, 1, 10, 10, 1e-3, out.ctypes.data_as(ctypes.c_void_p), None, 0,
                                None) == AGB_BADARG
