"""Continuous-batching server: each request's result is the same alone and in
the mix (bitwise: the device kernels treat every scenario independently, so
sharing the pool, the chunk boundaries and the admission order change
nothing), and requests queue when the pool is full."""
import numpy as np
import pytest

from anuga_core_gb300.serve import FloodServer, MeshCache, Request

pytestmark = pytest.mark.gpu


def _requests(n=16):
    rng = np.random.default_rng(5)
    out = []
    for i in range(n):
        out.append(Request(rid=i, arrival=0.01 * i, kind="rect" if i % 2 == 0 else "delaunay",
                           cells=int(rng.integers(4000, 40000)), seed=1000 + i,
                           finaltime=float(rng.uniform(5.0, 20.0)), inflow_stage=float(rng.uniform(1.0, 2.5))))
    return out


def test_results_same_alone_and_in_the_mix():
    cache = MeshCache(ladder=np.exp(np.linspace(np.log(4000), np.log(40000), 4)))
    reqs = _requests()
    mix = FloodServer(hbm_bytes=64 << 20, max_scenarios=5, chunk_steps=16, keep_results=True, mesh_cache=cache)
    summary = mix.run(reqs, realtime=False)
    assert summary["requests"] == len(reqs)
    got = {r.rid: r for r in mix.results}
    # requests overlapped on the device: more than one admitted before the first finished
    first_done = min(r.done for r in mix.results)
    assert sum(1 for r in mix.results if r.admitted < first_done) > 1
    mix.close()
    for req in reqs:
        alone = FloodServer(hbm_bytes=32 << 20, max_scenarios=1, chunk_steps=1000, keep_results=True,
                            mesh_cache=cache)
        alone.run([Request(**{**req.__dict__, "arrival": 0.0})], realtime=False)
        r = alone.results[0]
        alone.close()
        assert r.steps == got[req.rid].steps, req.rid
        assert np.array_equal(r.stage, got[req.rid].stage), req.rid


def test_admission_waits_for_memory():
    cache = MeshCache(ladder=[30000.0])
    reqs = [Request(rid=i, arrival=0.0, kind="rect", cells=30000, seed=i, finaltime=3.0) for i in range(4)]
    # room for one 30k-cell scenario at a time
    srv = FloodServer(hbm_bytes=14 << 20, max_scenarios=4, chunk_steps=8, keep_results=False, mesh_cache=cache)
    srv.run(reqs, realtime=False)
    res = sorted(srv.results, key=lambda r: r.admitted)
    srv.close()
    assert len(res) == 4
    for a, b in zip(res, res[1:]):
        assert b.admitted >= a.done - 1e-6      # served one after another
