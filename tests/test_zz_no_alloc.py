"""fsi_mg_subtract_average_noalloc: the mean removal for callers that cannot
allocate GPU memory (their device memory belongs to their own pool, or their
time loop must not pay cudaMalloc's implicit synchronisation).  It works on
the caller's device arrays without a handle and keeps its partial sums in a
fixed array inside the library.

Checked through the C ABI against the handle-based fsi_mg_subtract_average
on the same inputs, on two calls in a row (the second call finds the first
call's partial sums still in the shared array).  This file is collected last
so that a run stopping at the first failure has run every other test.
"""
import ctypes

import numpy as np
import pytest

from flow_structure_interaction_fem_ibm_gb300 import problem as P
from flow_structure_interaction_fem_ibm_gb300.grid import Metrics
from flow_structure_interaction_fem_ibm_gb300.poisson import PoissonSolver

pytestmark = pytest.mark.gpu

TOL = 1e-13   # the tolerance of the handle-based mean-removal parity test


def _dev(a, dtype):
    """Device copy of a Fortran-order array (same memory order) and the tensor."""
    import torch
    t = torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=dtype).transpose())).cuda()
    return t


def _host(t):
    return t.cpu().numpy().transpose()


def _noalloc(lib, pr, p_dev, ib_dev, dx_dev, dy_dev, dz_dev, stream=None):
    import torch
    prm = pr.params
    st = stream if stream is not None else torch.cuda.current_stream()
    rc = lib.fsi_mg_subtract_average_noalloc(
        ctypes.c_void_p(p_dev.data_ptr()), ctypes.c_void_p(ib_dev.data_ptr()),
        ctypes.c_void_p(dx_dev.data_ptr()), ctypes.c_void_p(dy_dev.data_ptr()),
        ctypes.c_void_p(dz_dev.data_ptr()), prm.ndim, prm.nx, prm.ny, prm.nz,
        ctypes.c_void_p(st.cuda_stream))
    assert rc == 0, lib.fsi_mg_last_error().decode()
    torch.cuda.synchronize()


def _case(name):
    if name == "sphere16_tanh":
        return P.sphere(16, seed=2, stretch=1.5)
    if name == "box2d_32":
        return P.box2d(32, seed=9)
    # the largest grid the fixed scratch accepts: (ny-1)*(nz-1) = 256*256 = 65536 rows
    return P.box3d((2, 256, 256), seed=4, stretch=1.5)


@pytest.mark.parametrize("case,own_stream", [("sphere16_tanh", False), ("box2d_32", False),
                                             ("sphere16_tanh", True), ("rows65536", True)])
def test_noalloc_mean_removal_matches_handle_entry_point(gpu_built, case, own_stream):
    import torch
    lib = gpu_built
    pr = _case(case)
    s = PoissonSolver(pr.params, pr.x, pr.y, pr.z).set_boundary(pr.geom)
    ib_dev = _dev(pr.geom.iblank, np.int8)
    dx_dev, dy_dev, dz_dev = (_dev(Metrics(c).dx, np.float64) for c in (pr.x, pr.y, pr.z))
    stream = torch.cuda.Stream() if own_stream else None   # a freshly created non-default stream
    rng = np.random.default_rng(21)
    try:
        for call in range(2):   # two calls in a row share the library's scratch array
            p = np.asfortranarray(rng.standard_normal(pr.shape) + 3.0 * call)
            ref = s.subtracting_average_pressure(p.copy(order="F"))
            p_dev = _dev(p, np.float64)
            torch.cuda.synchronize()
            _noalloc(lib, pr, p_dev, ib_dev, dx_dev, dy_dev, dz_dev, stream)
            got = _host(p_dev)
            assert np.abs(got - ref).max() < TOL, (call, np.abs(got - ref).max())
    finally:
        s.close()


def test_noalloc_mean_removal_rejects_grids_beyond_its_scratch(gpu_built):
    lib = gpu_built
    # 3 x 258 x 258 nodes: (258-1)*(258-1) = 66049 (j,k) rows > 65536
    rc = lib.fsi_mg_subtract_average_noalloc(ctypes.c_void_p(16), ctypes.c_void_p(16), ctypes.c_void_p(16),
                                             ctypes.c_void_p(16), ctypes.c_void_p(16), 3, 3, 258, 258,
                                             ctypes.c_void_p(0))
    assert rc == -1
    assert "65536" in lib.fsi_mg_last_error().decode()
