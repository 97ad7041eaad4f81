"""Host side of the serving loop (no device): the request stream and the
synthetic scenarios are deterministic and have the stated distributions."""
import numpy as np

from anuga_core_gb300.serve import poisson_requests, delaunay_mesh, scenario_state, MeshCache, Request


def test_poisson_stream_statistics():
    reqs = poisson_requests(n=2000, rate=20.0, seed=99)
    arr = np.array([r.arrival for r in reqs])
    assert np.all(np.diff(arr) >= 0)
    rate = (len(arr) - 1) / (arr[-1] - arr[0])
    assert 18.0 < rate < 22.0
    cells = np.array([r.cells for r in reqs])
    assert cells.min() >= 1e4 and cells.max() <= 2e6
    assert 0.4 < np.mean([r.kind == "rect" for r in reqs]) < 0.6
    fts = np.array([r.finaltime for r in reqs])
    assert fts.min() >= 60 and fts.max() <= 3600
    again = poisson_requests(n=2000, rate=20.0, seed=99)
    assert [r.arrival for r in again] == list(arr)


def test_delaunay_mesh_and_state():
    m = delaunay_mesh(5000, seed=3)
    assert 3500 < len(m) < 6500
    assert "inflow" in m.tag_boundary_cells and "wall" in m.tag_boundary_cells
    z, stage, eta = scenario_state(m, Request(0, 0.0, "delaunay", 5000, 11, 60.0))
    assert np.array_equal(stage, z)
    assert eta.min() >= 0.02 and eta.max() <= 0.05
    c = MeshCache(ladder=[5000.0, 20000.0])
    assert c.snap(6000) == 5000 and c.snap(15000) == 20000


def test_delaunay_mesh_is_well_shaped():
    """No slivers: the smallest inscribed radius stays a fair fraction of the
    lattice spacing (10 m), so the CFL timestep cannot collapse."""
    m = delaunay_mesh(20000, seed=5)
    assert m.radii.min() > 0.5
    assert m.areas.min() > 5.0


def test_mesh_cache_is_shared_safely_between_threads():
    import threading
    c = MeshCache(ladder=[5000.0])
    got = []
    threads = [threading.Thread(target=lambda: got.append(c.get("delaunay", 5000)[0])) for _ in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert len(got) == 4 and all(g is got[0] for g in got)
    # the same key gives the same mesh in a fresh cache
    again = MeshCache(ladder=[5000.0]).get("delaunay", 5000)[0]
    assert np.array_equal(again.nodes, got[0].nodes)
