"""GpuSolver.create on a device that cannot hold the domain: the reference
returns an AllocationFailure (not a throw) after destroying every buffer it had
created (src/lbm/gpu-solver.ts:330-334, src/lbm/gpu-resources.ts:3-5).

The request is a 64 x 16384 x 3968 tunnel (4.16 G cells, just under the 2^32
cell limit) in f32 storage: its population array alone (19 x 4 bytes per cell,
316 GB) is larger than the GPU's whole memory, so the first large allocation
is refused at once and nothing close to the device's capacity is ever held.
The voxel grid (about 33 GB on the device) is built first on the GPU."""
import numpy as np
import pytest

from tests.shapes import box

pytestmark = pytest.mark.gpu

HUGE = (64, 16384, 3968)


def test_allocation_failure_is_returned_and_leaves_nothing_behind():
    torch = pytest.importorskip("torch")
    from pocketwind_gb300 import geometry, solver
    from pocketwind_gb300._lib import AllocationFailure

    torch.cuda.init()
    body = box([20.25, 100.25, 100.25], [28.25, 108.25, 108.25])
    grid = geometry.voxelize(body, None, HUGE, False)
    torch.cuda.synchronize()
    free_before, total = torch.cuda.mem_get_info()
    assert 19 * 4 * HUGE[0] * HUGE[1] * HUGE[2] > total  # the request cannot fit
    params = solver.SolverParams(tau0=0.56, u_in=0.05, precision="f32")
    out = solver.GpuSolver.create(HUGE, grid, params)
    assert isinstance(out, AllocationFailure)
    assert out.kind == "allocation-failure"
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    # everything the failed create had allocated is back (streams, events and
    # the small buffers made before the populations)
    assert free_before - free_after < 64 << 20
    del grid
    # the context is still usable: a small domain steps and keeps rest at rest
    small = (16, 16, 16)
    g = geometry.voxelize(box([4.25, 4.25, 4.25], [8.25, 8.25, 8.25]), None, small, False)
    s = solver.GpuSolver.create(small, g, solver.SolverParams(tau0=0.8, u_in=0.0))
    assert not isinstance(s, Exception)
    s.step(10, True)
    m = s.macros()
    assert np.isfinite(m).all() and np.abs(m[:, 1:]).max() == 0.0
    s.destroy()
