"""GPU tracers against the reference's golden particle vector and the binary32
tracer restatements (particles_update.wgsl, plate_smoke.wgsl, 3-D streaks)."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.shapes import NO_Q

pytestmark = pytest.mark.gpu


def _solver(layout, geometry, boundary, u_in=0.05, **kw):
    from pocketwind_gb300 import geometry as G, solver as S
    grid = G.grid_from_arrays(layout, geometry, boundary)
    return S.GpuSolver.create(layout, grid, S.SolverParams(tau0=0.8, u_in=u_in, **kw))


def _empty(layout):
    cells = layout[0] * layout[1] * layout[2]
    return np.concatenate([np.zeros(cells, np.uint32), np.full(cells, NO_Q, np.uint32)]), np.zeros(0, np.uint32)


def test_particles_golden_vector_on_gpu():
    """tests/browser/particles.spec.ts:19-127"""
    from pocketwind_gb300.tracers import Particles
    g, b = _empty((16, 16, 16))
    s = _solver((16, 16, 16), g, b)
    lin = np.zeros((4096, 4), np.float32)
    for cell in range(4096):
        lin[cell] = (2, (cell % 16) * 0.01, ((cell // 16) % 16) * 0.02, (cell // 256) * 0.03)
    s.write_macros(lin)
    rec0 = np.array([4.25, 5.5, 6.75, 10, 4.25, 5.5, 6.75, 0], np.float32)
    p = Particles(s, rec0, 7, (3.1, 3.1, 10.9, 10.9), (5.0, 5.0))

    def record(steps, age=10, x=4.25, gen=0):
        p.write(np.array([x, 5.5, 6.75, age, x, 5.5, 6.75, gen], np.float32))
        p.update(steps)
        return p.read()[0]

    got = record(2)
    assert np.allclose(got, [4.335, 5.72, 7.155, 11, 4.25, 5.5, 6.75, 0], atol=5e-6)
    s.write_macros(np.tile(np.array([20, 3, 4, 0], np.float32), (4096, 1)))
    assert np.allclose(record(9), [4.85, 6.3, 6.75, 11, 4.25, 5.5, 6.75, 0], atol=5e-6)
    assert list(record(0)) == [4.25, 5.5, 6.75, 11, 4.25, 5.5, 6.75, 0]
    assert list(record(0, 3999)) == [4.25, 5.5, 6.75, 4000, 4.25, 5.5, 6.75, 0]
    expired, outlet, nxt = record(0, 4000), record(0, 10, 14), record(0, 4000, 4.25, 1)
    for r in (expired, outlet, nxt):
        assert r[0] == 2 and r[3] == 0 and list(r[4:7]) == list(r[0:3]) and all(3.1 <= c <= 10.9 for c in r[1:3])
    assert list(expired) == list(outlet) and expired[7] == 1 and nxt[7] == 2
    ref = O.particles_update(np.array([4.25, 5.5, 6.75, 4000, 4.25, 5.5, 6.75, 0], np.float32),
                             np.tile(np.array([20, 3, 4, 0], np.float32), 4096), np.zeros(4096, np.uint32),
                             (16, 16, 16), 7, 0, (3.1, 3.1, 10.9, 10.9), (5.0, 5.0))
    assert np.array_equal(expired, ref)


def _flow_case():
    """A short run of the vehicle case to give the tracers a real wake."""
    from pocketwind_gb300 import meshes
    from pocketwind_gb300.geometry import voxelize
    from pocketwind_gb300 import solver as S
    layout = (128, 64, 64)
    grid = voxelize(meshes.vehicle_case_mesh(128, 64), None, layout, True)
    s = S.GpuSolver.create(layout, grid, S.SolverParams(tau0=0.5 + 3 * 0.00625, u_in=0.05, les=True, operator="reg"))
    s.step(400, True)
    return s, grid


def test_plate_smoke_matches_restatement():
    from pocketwind_gb300.tracers import PlateSmoke
    s, grid = _flow_case()
    flags = grid.flags.copy()
    macros = s.macros().reshape(-1)
    ports = np.array([[60, 5], [60, 9], [-1, -1], [50, 13], [75, 10], [40, 1.5]], np.float32)
    plate = PlateSmoke(s, 32, 36, 64, ports)
    ref = np.zeros((42 * 64, 4), np.float32)
    rake = (2.0, 1.5, 40.0, 8.0)
    for frame in range(40):
        release, releasing = frame // 2, frame % 2 == 0
        plate.advance(release, releasing, rake)
        ref = O.plate_smoke(ref, 42, 64, release, releasing, rake, (128, 64, 64), 32, macros, flags, ports)
    got = plate.read()
    assert np.array_equal(got[:, :3], ref.reshape(-1, 4)[:, :3])
    assert np.allclose(got[:, 3], ref.reshape(-1, 4)[:, 3], rtol=1e-4, atol=0)
    assert (got[:, 3] > 0).sum() > 100


def test_streaks_match_restatement():
    from pocketwind_gb300.tracers import Streaks
    s, grid = _flow_case()
    flags = grid.flags.copy()
    macros = s.macros().reshape(-1)
    rake = (2.0, 20.0, 44.0, 1.5, 30.0)
    st = Streaks(s, 16, 16, 32, rake)
    puffs = np.zeros((16 * 16 * 32, 4), np.float32)
    rel = np.zeros(16 * 16 * 32, np.uint32)
    for frame in range(24):
        st.advance(8.0, frame // 2, frame % 2 == 0)
        puffs, rel = O.streaks(puffs, rel, 16, 16, 32, frame // 2, frame % 2 == 0, rake, 8.0,
                               (128, 64, 64), macros, flags)
    got, got_rel = st.read()
    ref = puffs.reshape(-1, 4)
    assert np.array_equal(got_rel, rel)
    assert np.array_equal(got[:, :3], ref[:, :3])
    assert np.allclose(got[:, 3], ref[:, 3], rtol=1e-4, atol=0)
    assert (got[:, 3] > 0).sum() > 1000


def test_plate_smoke_with_dye_ports_from_geometry():
    """The plate's ports placed by dye_ports (plate-layout.ts:164-225) on the
    voxelized vehicle's centre plane, the rake from rake_span: the kernel
    matches the restatement and the port threads carry live smoke."""
    from pocketwind_gb300 import plate_layout as PL
    from pocketwind_gb300.tracers import PlateSmoke
    s, grid = _flow_case()
    flags = grid.flags.copy()
    macros = s.macros().reshape(-1)
    low, high = PL.rake_span(44.0, 64)
    ports = PL.dye_ports(flags, (128, 64, 64), 32, (low, high)).reshape(-1, 2)
    assert (ports[:, 0] >= 0).sum() >= 4
    plate = PlateSmoke(s, 32, PL.RAKE_THREADS, 64, ports)
    ref = np.zeros((PL.THREADS * 64, 4), np.float32)
    rake = (float(PL.RAKE_X), low, high, 8.0)
    for frame in range(30):
        release, releasing = frame // 2, frame % 2 == 0
        plate.advance(release, releasing, rake)
        ref = O.plate_smoke(ref, PL.THREADS, 64, release, releasing, rake, (128, 64, 64), 32, macros, flags, ports)
    got = plate.read()
    assert np.array_equal(got[:, :3], ref.reshape(-1, 4)[:, :3])
    port_rows = got.reshape(PL.THREADS, 64, 4)[PL.RAKE_THREADS:]
    live = [(port_rows[k, :, 3] > 0).any() for k in range(PL.PORTS) if ports[k, 0] >= 0]
    assert all(live)


def test_particles_seeded_from_geometry_stay_valid():
    """particle_seeds (particle-layout.ts:66-112) on the voxelized vehicle feeds
    the particle kernel; after advection every particle sits on a valid fluid
    node by the reseed rule the kernel applies."""
    from pocketwind_gb300 import meshes, particle_layout as PL
    from pocketwind_gb300.tracers import Particles
    s, grid = _flow_case()
    layout = (128, 64, 64)
    body = meshes.vehicle_case_mesh(128, 64)
    pts = body.positions.reshape(-1, 3)
    data, region, fallback = PL.particle_seeds(grid.flags, layout, pts.min(axis=0), pts.max(axis=0), 4096, 7)
    p = Particles(s, data, 7, region, fallback)
    for _ in range(20):
        p.update(8.0)
    rec = p.read().reshape(-1, 8)
    flags = grid.flags
    bad = 0
    for r in rec[::17]:
        x, y, z, age = (float(v) for v in r[:4])
        n = int(round(x)) + 128 * (int(round(y)) + 64 * int(round(z)))
        flag = int(flags[n]) if 0 <= n < flags.size else 1
        bad += PL.particle_needs_reseed((x, y, z), age, layout, flag)
    assert bad == 0
