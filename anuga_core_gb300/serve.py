"""Serving: a continuous-batching request loop for flood scenarios.

Requests (a mesh, a seeded bathymetry and inflow, a final time) arrive over
time.  The server keeps one device pool; a request is admitted as soon as a
scenario slot and enough pool memory (cells, boundary edges, halo entries:
its HBM footprint) are free, its state is uploaded once and stays on the GPU
until its final time, and every scenario in the pool advances together in
chunks of device steps (one graph launch per chunk).  Between chunks the host
retires finished scenarios (one D2H read of the final state) and admits new
ones; building the next requests' tables overlaps the running chunk.

Latency of a request = time its result is on the host - its arrival time.
"""
from __future__ import annotations

import concurrent.futures
import dataclasses
import threading
import time

import numpy as np

from . import _lib, mixed
from .domain import FLOW_ALGORITHMS
from .mesh import Mesh, rectangular_cross
from .tables import pack_mixed


@dataclasses.dataclass
class Request:
    rid: int
    arrival: float          # seconds after the stream starts
    kind: str               # "rect" or "delaunay"
    cells: int              # target number of triangles
    seed: int
    finaltime: float        # simulated seconds
    inflow_stage: float = 2.0


def poisson_requests(n=2000, rate=20.0, seed=99, lo=1.0e4, hi=2.0e6, t_lo=60.0, t_hi=3600.0):
    """The request stream: Poisson arrivals, rectangular cross or Delaunay
    meshes (50/50) with log-uniform sizes, final times U(t_lo, t_hi)."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, n)
    arr = np.cumsum(gaps) - gaps[0]
    kinds = np.where(rng.uniform(size=n) < 0.5, "rect", "delaunay")
    cells = np.exp(rng.uniform(np.log(lo), np.log(hi), n)).astype(np.int64)
    fts = rng.uniform(t_lo, t_hi, n)
    inflow = rng.uniform(1.0, 3.0, n)
    return [Request(i, float(arr[i]), str(kinds[i]), int(cells[i]), int(seed * 100000 + i), float(fts[i]),
                    float(inflow[i])) for i in range(n)]


def _size_ladder(lo=1.0e4, hi=2.0e6, steps=12):
    return np.exp(np.linspace(np.log(lo), np.log(hi), steps))


def delaunay_mesh(n_cells, seed, spacing=10.0):
    """Delaunay triangulation of a jittered lattice in a square (about
    n_cells triangles).  Interior points move by up to 0.3 spacing; points on
    the square's sides stay on the lattice, so no triangle degenerates along
    the boundary.  Boundary edges on the west side are tagged 'inflow', the
    others 'wall'."""
    from scipy.spatial import Delaunay
    rng = np.random.default_rng(seed)
    npts = max(int(n_cells // 2), 16)
    side = max(int(np.ceil(np.sqrt(npts))), 3)
    L = (side - 1) * spacing
    gx, gy = np.meshgrid(np.arange(side), np.arange(side), indexing="ij")
    pts = np.stack([gx.ravel(), gy.ravel()], 1).astype(float) * spacing
    interior = (gx.ravel() > 0) & (gx.ravel() < side - 1) & (gy.ravel() > 0) & (gy.ravel() < side - 1)
    pts[interior] += rng.uniform(-0.3, 0.3, (int(interior.sum()), 2)) * spacing
    tri = Delaunay(pts).simplices.astype(np.int64)
    a = pts[tri]
    cr = (a[:, 1, 0] - a[:, 0, 0]) * (a[:, 2, 1] - a[:, 0, 1]) - (a[:, 1, 1] - a[:, 0, 1]) * (a[:, 2, 0] - a[:, 0, 0])
    keep = np.abs(cr) > 1e-6 * spacing * spacing
    tri = tri[keep]
    cr = cr[keep]
    tri[cr < 0] = tri[cr < 0][:, [0, 2, 1]]
    M0 = Mesh(pts, tri)
    bnd = {}
    E = M0.edge_midpoint_coordinates.reshape(-1, 3, 2)
    for (v, e) in M0.boundary:
        bnd[(v, e)] = "inflow" if E[v, e, 0] < 0.01 * L else "wall"
    return Mesh(pts, tri, bnd)


class MeshCache:
    """Meshes and their device tables, one per (kind, size on a log ladder).

    Safe to share between the server's preparation threads: each entry is
    built once, under a lock of its own, and a Delaunay mesh's seed follows
    from its size, so the same key always gives the same mesh."""

    def __init__(self, ladder=None):
        self.ladder = _size_ladder() if ladder is None else np.asarray(ladder)
        self.cache = {}
        self._lock = threading.Lock()
        self._key_locks = {}

    def snap(self, cells):
        return int(self.ladder[np.argmin(np.abs(np.log(self.ladder) - np.log(cells)))])

    def get(self, kind, cells):
        n = self.snap(cells)
        key = (kind, n)
        with self._lock:
            hit = self.cache.get(key)
            if hit is not None:
                return hit
            lock = self._key_locks.setdefault(key, threading.Lock())
        with lock:
            with self._lock:
                hit = self.cache.get(key)
            if hit is not None:
                return hit
            if kind == "rect":
                m = max(int(round(np.sqrt(n / 4.0))), 2)
                p, e, b = rectangular_cross(m, m, 10.0 * m, 10.0 * m)
                mesh = Mesh(p, e, b)
            else:
                mesh = delaunay_mesh(n, seed=7 + n)
            entry = (mesh, pack_mixed(mesh))
            with self._lock:
                self.cache[key] = entry
            return entry


def scenario_state(mesh, req):
    """Seeded bathymetry (slope + bumps), dry start, Manning n."""
    rng = np.random.default_rng(req.seed)
    C = mesh.centroid_coordinates
    x, y = C[:, 0], C[:, 1]
    L = max(x.max() - x.min(), 1.0)
    z = -rng.uniform(0.0005, 0.002) * (x - x.min())
    for _ in range(6):
        cx, cy = rng.uniform(x.min(), x.max()), rng.uniform(y.min(), y.max())
        z = z + rng.uniform(-1.5, 1.5) * np.exp(-((x - cx) ** 2 + (y - cy) ** 2) / (2 * (rng.uniform(0.05, 0.2) * L) ** 2))
    stage = z.copy()                                        # dry start
    eta = rng.uniform(0.02, 0.05, len(z))
    return z, stage, eta


def scenario_boundary(mesh, req):
    kind = np.zeros(mesh.boundary_length, np.int32)
    vals = np.zeros((mesh.boundary_length, 3))
    for tag, ids in mesh.tag_boundary_cells.items():
        if tag in ("left", "inflow"):
            kind[ids] = _lib.BC_DIRICHLET
            vals[ids] = (req.inflow_stage, 0.0, 0.0)
        elif tag == "right":
            kind[ids] = _lib.BC_TRANSMISSIVE
        else:
            kind[ids] = _lib.BC_REFLECTIVE
    return kind, vals


def de1_params():
    p = _lib.Params()
    d = FLOW_ALGORITHMS["DE1"]
    p.g, p.epsilon, p.minimum_allowed_height = 9.8, 1.0e-12, d["minimum_allowed_height"]
    for k in ("beta_w", "beta_w_dry", "beta_uh", "beta_uh_dry", "beta_vh", "beta_vh_dry"):
        setattr(p, k, d[k])
    p.CFL, p.evolve_max_timestep, p.evolve_min_timestep = d["CFL"], 1.0e3, 1.0e-6
    p.extrapolate_velocity_second_order = 1
    p.timestepping_method = 2
    p.max_smallsteps = 50
    p.precision = _lib.AGX_PREC_MIXED
    return p


@dataclasses.dataclass
class Result:
    rid: int
    cells: int
    steps: int
    arrival: float
    admitted: float
    done: float
    stage: np.ndarray = None

    @property
    def latency(self):
        return self.done - self.arrival


class FloodServer:
    """Continuous-batching server over one device pool.

    hbm_bytes: memory budget of the pool (default: 60% of the free device
    memory); the pool's cell/boundary/halo capacities follow from it and
    admission checks a request's footprint against what is free."""

    def __init__(self, hbm_bytes=None, max_scenarios=256, chunk_steps=64, keep_results=False,
                 mesh_cache=None, workers=4):
        if hbm_bytes is None:
            import torch
            free, _total = torch.cuda.mem_get_info()
            hbm_bytes = int(0.6 * free)
        per_cell = mixed.bytes_per_cell()
        cells = int(hbm_bytes // (per_cell + 64))          # + lnk, halo and staging entries
        self.pool = mixed.Pool(cells, max(cells // 16, 4096), max_scenarios)
        self.hbm_bytes = hbm_bytes
        self.chunk = int(chunk_steps)
        self.keep = keep_results
        self.cache = mesh_cache or MeshCache()
        self.params = de1_params()
        self.exec = concurrent.futures.ThreadPoolExecutor(max_workers=workers)
        self.live = {}            # sid -> (request, admitted time, cells)
        self.results = []
        self.cell_steps = 0

    def fits(self, T):
        cap = self.pool.capacity()
        N = T["conn"].shape[0]
        need = ((N + 255) // 256) * 256
        return (cap["scenarios"] > 0 and cap["cells"] >= need and cap["boundary"] >= T["boundary_cell"].shape[0]
                and cap["halo"] >= T["halo_cells"].size)

    def _prepare(self, req):
        mesh, T = self.cache.get(req.kind, req.cells)
        z, stage, eta = scenario_state(mesh, req)
        kind, vals = scenario_boundary(mesh, req)
        return req, mesh, T, z, stage, eta, kind, vals

    def _admit(self, prep, t_now):
        req, mesh, T, z, stage, eta, kind, vals = prep
        sid = self.pool.add(mesh, self.params, T)
        self.pool.set_field(sid, "elev_c", z)
        self.pool.set_field(sid, "stage_c", stage)
        self.pool.set_field(sid, "xmom_c", np.zeros_like(z))
        self.pool.set_field(sid, "ymom_c", np.zeros_like(z))
        self.pool.set_field(sid, "friction_c", eta)
        self.pool.set_boundary(sid, kind, vals)
        self.pool.distribute(sid)
        self.pool.set_clock(sid, 0.0, 1e300, req.finaltime, 0)
        self.live[sid] = (req, t_now, len(mesh))

    def _retire(self, t0):
        sids = sorted(self.live)
        if not sids:
            return
        stats, running = self.pool.stats_all(sids)
        for sid, st, run in zip(sids, stats, running):
            if run:
                continue
            req, t_adm, n = self.live.pop(sid)
            stage = self.pool.get_field(sid, "stage_c") if self.keep else None
            if not self.keep:
                self.pool.get_field(sid, "stage_c")       # the result read (D2H) is part of the latency
            t_done = time.perf_counter() - t0
            if st.reason == _lib.STOP_ERROR:
                self.pool.stats(sid)                      # raises with the device's error
                raise _lib.AgxError(-5, "scenario %d failed on the device" % req.rid)
            self.results.append(Result(req.rid, n, int(st.total_steps), req.arrival, t_adm, t_done, stage))
            self.cell_steps += n * int(st.total_steps)
            self.pool.remove(sid)

    def run(self, requests, realtime=True, max_wall=None):
        """Serve the requests; returns a summary dict (p50/p99 latency,
        aggregate cell-steps/s).  realtime=True admits a request once its
        arrival time has passed on the wall clock; realtime=False replays the
        stream as fast as possible, every request counting as arrived."""
        pending = sorted(requests, key=lambda r: r.arrival)
        futures = {}
        self.device_s = 0.0          # wall time spent in device chunks (launch to completion)
        self.admit_s = 0.0           # in admissions (tables, state and boundary upload)
        self.retire_s = 0.0          # in retirements (statistics, result read, removal)
        self.idle_s = 0.0            # with no scenario on the device (waiting for arrivals)
        self.chunks = 0
        t0 = time.perf_counter()
        i_next = 0
        waiting = []          # prepared, arrived, not yet admitted (in arrival order)
        while i_next < len(pending) or waiting or self.live or futures:
            now = time.perf_counter() - t0
            if max_wall is not None and now > max_wall:
                break
            clock = now if realtime else float("inf")
            # start preparing requests that have arrived (and a few ahead)
            while i_next < len(pending) and (pending[i_next].arrival <= clock or len(futures) < 2):
                r = pending[i_next]
                futures[r.rid] = (r, self.exec.submit(self._prepare, r))
                i_next += 1
            for rid in sorted(futures, key=lambda k: futures[k][0].arrival):
                r, f = futures[rid]
                # replay mode (realtime=False) takes requests strictly in arrival
                # order, so admission does not depend on host thread timing
                if (f.done() or not realtime) and r.arrival <= clock:
                    waiting.append(f.result())
                    del futures[rid]
            waiting.sort(key=lambda p: p[0].arrival)
            ta = time.perf_counter()
            while waiting and self.fits(waiting[0][2]):
                self._admit(waiting.pop(0), time.perf_counter() - t0)
            self.admit_s += time.perf_counter() - ta
            if self.live:
                tc = time.perf_counter()
                self.pool.launch_chunk(self.chunk)
                self.pool.wait()
                tr = time.perf_counter()
                self.device_s += tr - tc
                self.chunks += 1
                self._retire(t0)
                self.retire_s += time.perf_counter() - tr
            else:
                ti = time.perf_counter()
                time.sleep(0.001)
                self.idle_s += time.perf_counter() - ti
        wall = time.perf_counter() - t0
        lat = np.array([r.latency for r in self.results]) if self.results else np.zeros(1)
        return dict(requests=len(self.results), wall_s=wall, p50_s=float(np.percentile(lat, 50)),
                    p99_s=float(np.percentile(lat, 99)), cell_steps=int(self.cell_steps),
                    cell_steps_per_s=self.cell_steps / max(wall, 1e-9), chunks=self.chunks,
                    device_s=self.device_s, device_cell_steps_per_s=self.cell_steps / max(self.device_s, 1e-9),
                    admit_s=self.admit_s, retire_s=self.retire_s, idle_s=self.idle_s)

    def close(self):
        self.exec.shutdown(wait=False)
        self.pool.close()
