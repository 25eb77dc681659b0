"""fos_euler_rhs_dev_static -- the residual for callers that cannot allocate device memory
when they evaluate it (their host code owns a fixed device-memory budget, or must not
allocate inside its time loop).  Its scratch is a static device array of the library; the
result must equal fos_euler_rhs_dev's on two calls in a row (the second call sees the
first call's leftovers in the shared array), within the residual tolerance used elsewhere
(1e-11 relative), and grids larger than the array must be refused with a clear error.

Collected last on purpose (file name), so a run that stops at the first failure has run
everything else first."""
import numpy as np
import pytest

from fosolvers_gb300 import mesh as M
from fosolvers_gb300.euler import FLUX_FP32
from helpers import Case, hex_workload, perturbed, rel_err, with_all_conditions

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("flags", [0, FLUX_FP32])
@pytest.mark.parametrize("name", ["sine8", "hex-conds"])
def test_static_scratch_residual_matches_rhs_dev(cuda, flags, name):
    import torch
    wl = (M.make_workload("sine96", scale=8, seed=5) if name == "sine8"  # 3,072 cells
          else with_all_conditions(hex_workload(10, seed=5)))  # warped hexahedra, 480 cells
    c = Case(wl, flags=flags)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    for seed in (1, 2):  # two calls in a row, different states
        y = perturbed(c.y0, c.nC, seed)
        y_ref_order = dev(y)
        yi = torch.empty_like(y_ref_order)
        c.gpu.to_internal(y_ref_order, yi)
        f_dev = torch.empty_like(yi)
        f_static = torch.full_like(yi, float("nan"))
        c.gpu.rhs_dev(0.0, yi, f_dev)
        assert c.gpu.rhs_dev_static(0.0, yi, f_static) == 0
        torch.cuda.synchronize()
        a, b = f_static.cpu().numpy(), f_dev.cpu().numpy()
        assert np.all(np.isfinite(a))
        assert rel_err(a, b) <= 1e-11


@pytest.mark.parametrize("grid", ["cells", "faces"])
def test_static_scratch_refuses_large_grid(cuda, grid):
    """Two limits: 65,536 cells (a 24^3 x 6 tetrahedral box has 82,944) and 147,456 faces (a
    38^3 hexahedral box has 54,872 cells, under the cell limit, and 168,948 faces)."""
    import torch
    from fosolvers_gb300 import _lib
    if grid == "cells":
        c = Case(M.make_workload("sine96", scale=24, seed=5))
    else:
        m = M.box_mesh(38, 38, 38, jitter=0.1, seed=5, cells="hex")
        st = M.sine_state(m.centroids(), 5)
        c = Case(M.Workload("hex38", m, st, np.zeros(0, np.int32), np.zeros(0, np.int32),
                            np.zeros((0, 5)), order=2, dt=5e-4, nsteps=1))
        assert c.nC <= 65536 and c.grid.nP > 147456
    y = torch.zeros(c.N, dtype=torch.float64, device="cuda")
    out = torch.zeros_like(y)
    rc = _lib.lib().fos_euler_rhs_dev_static(c.gpu.handle, 0.0, y.data_ptr(), out.data_ptr())
    assert rc == -1
    msg = _lib.last_error()
    assert "at most 65536 cells and 147456 faces" in msg
    assert (f"{c.nC} cells" in msg) and (f"{c.grid.nP} faces" in msg)
