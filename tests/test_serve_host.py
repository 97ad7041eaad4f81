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


class _FakePool:
    """Stand-in for the device pool with the calls the server makes: each
    scenario needs ceil(finaltime / 0.5) steps and a chunk advances every
    running scenario by up to `chunk` steps; capacity is counted in cells
    rounded up to 256 as the server's admission check does."""

    def __init__(self, cells, slots):
        self.free_cells, self.slots = cells, slots
        self.scn = {}
        self.max_live = 0
        self.next_sid = 0

    def capacity(self):
        return dict(cells=self.free_cells, boundary=1 << 30, halo=1 << 30, scenarios=self.slots - len(self.scn))

    def add(self, mesh, params, T):
        n = T["conn"].shape[0]
        need = ((n + 255) // 256) * 256
        assert need <= self.free_cells and len(self.scn) < self.slots      # the server checked first
        self.free_cells -= need
        sid = self.next_sid
        self.next_sid += 1
        self.scn[sid] = dict(n=n, need=need, steps=0, target=None)
        self.max_live = max(self.max_live, len(self.scn))
        return sid

    def set_field(self, sid, name, values):
        assert len(values) == self.scn[sid]["n"]

    def set_boundary(self, sid, kind, values):
        pass

    def distribute(self, sid):
        pass

    def set_clock(self, sid, time, yield_time, final_time, max_steps=0):
        self.scn[sid]["target"] = int(np.ceil(final_time / 0.5))

    def launch_chunk(self, chunk):
        for s in self.scn.values():
            s["steps"] = min(s["target"], s["steps"] + chunk)

    def wait(self):
        return sum(s["steps"] < s["target"] for s in self.scn.values())

    def stats_all(self, sids):
        from types import SimpleNamespace
        from anuga_core_gb300 import _lib
        st = [SimpleNamespace(reason=_lib.STOP_FINAL if self.scn[s]["steps"] >= self.scn[s]["target"] else 0,
                              total_steps=self.scn[s]["steps"]) for s in sids]
        return st, np.array([x.reason == 0 for x in st])

    def get_field(self, sid, name, out=None):
        return np.zeros(self.scn[sid]["n"])

    def remove(self, sid):
        self.free_cells += self.scn.pop(sid)["need"]

    def close(self):
        pass


def _server(monkeypatch, cells, slots, chunk):
    from anuga_core_gb300 import serve as S, mixed
    fake = _FakePool(cells, slots)
    monkeypatch.setattr(mixed, "Pool", lambda *a, **k: fake)
    srv = S.FloodServer(hbm_bytes=1 << 30, max_scenarios=slots, chunk_steps=chunk,
                        mesh_cache=MeshCache(ladder=[5000.0]))
    return srv, fake


def test_server_serves_every_request_and_accounts_its_time(monkeypatch):
    reqs = poisson_requests(n=12, seed=5, lo=4000, hi=6000, t_lo=10.0, t_hi=40.0)
    srv, fake = _server(monkeypatch, cells=1 << 20, slots=8, chunk=16)
    summ = srv.run(reqs, realtime=True)          # arrivals in real time: the stream spans about 0.6 s
    srv.close()
    assert summ["requests"] == 12 and len({r.rid for r in srv.results}) == 12
    for r in srv.results:
        assert r.arrival <= r.admitted <= r.done and r.latency >= 0
        assert r.steps == int(np.ceil(next(q.finaltime for q in reqs if q.rid == r.rid) / 0.5))
    assert summ["cell_steps"] == sum(r.cells * r.steps for r in srv.results)
    assert summ["chunks"] > 0 and summ["device_s"] >= 0 and summ["admit_s"] >= 0
    assert not fake.scn and fake.free_cells == 1 << 20           # everything retired and released


def test_server_waits_for_capacity_and_keeps_arrival_order(monkeypatch):
    reqs = poisson_requests(n=6, seed=8, lo=4000, hi=6000, t_lo=10.0, t_hi=40.0)
    srv, fake = _server(monkeypatch, cells=5120, slots=8, chunk=8)      # room for one scenario
    srv.run(reqs, realtime=True)
    srv.close()
    assert fake.max_live == 1
    order = [r.rid for r in sorted(srv.results, key=lambda r: r.admitted)]
    assert order == [r.rid for r in sorted(reqs, key=lambda r: r.arrival)]
