"""Edge cases of the mixed-precision pool: a one-triangle mesh (three
boundary edges, a tile holding one cell and 127 unused slots), a completely
dry domain, and meshes whose last tile is partly filled (4, 124, 128 and 132
triangles against 128-cell tiles).

Bars: depths within 1 mm of the plain FP64 form on the same inputs; a dry
domain keeps its stage bitwise and takes one step of the maximum timestep
to reach the yield time, as the plain form does.  Also: a pool refuses a
scenario beyond its capacity and stays usable, and the Domain's one-call
state exchange (set_conserved_state / get_conserved_state) returns the state
it was given on both forms, from pageable and page-locked arrays.
"""
import numpy as np
import pytest

from anuga_core_gb300.mesh import Mesh, rectangular_cross
from helpers import make_domain, random_state

pytestmark = pytest.mark.gpu

DEPTH_TOL = 1.0e-3   # metres


def _depth(d):
    z = d.quantities["elevation"].centroid_values
    return np.maximum(d.quantities["stage"].centroid_values - z, 0.0)


def test_single_triangle_within_1mm_of_plain():
    p = np.array([[0.0, 0.0], [1.0, 0.0], [0.0, 1.0]])
    e = np.array([[0, 1, 2]])
    st = dict(elevation=np.zeros(1), stage=np.full(1, 0.5), xmom=np.full(1, 0.1), ymom=np.zeros(1),
              friction=np.zeros(1))
    kinds = {"exterior": ("reflective", None)}
    res = {}
    for precision in ("fp64", "mixed"):
        d = make_domain(p, e, None, "DE0", st, kinds, precision=precision)
        for _ in d.evolve(yieldstep=0.1, finaltime=0.3):
            pass
        assert abs(d.get_time() - 0.3) < 1e-12
        res[precision] = _depth(d)
    assert np.abs(res["mixed"] - res["fp64"]).max() <= DEPTH_TOL


def test_dry_domain_keeps_its_stage():
    p, e, b = rectangular_cross(5, 5, 10.0, 10.0)
    mesh = Mesh(p, e, b)
    z = mesh.centroid_coordinates[:, 0] * 0.1
    st = dict(elevation=z, stage=z.copy(), xmom=np.zeros_like(z), ymom=np.zeros_like(z), friction=np.zeros_like(z))
    d = make_domain(p, e, b, "DE1", st, {t: ("reflective", None) for t in mesh.tag_boundary_cells},
                    precision="mixed")
    for _ in d.evolve(yieldstep=5.0, finaltime=5.0):
        pass
    assert np.array_equal(d.quantities["stage"].centroid_values, z)
    assert d.total_steps == 1


@pytest.mark.parametrize("m,n", [(1, 1), (31, 1), (8, 4), (11, 3)])
def test_partly_filled_last_tile_within_1mm_of_plain(m, n):
    p, e, b = rectangular_cross(m, n, 4.0 * m, 4.0 * n)
    mesh = Mesh(p, e, b)
    assert len(mesh) == 4 * m * n
    st = random_state(mesh, seed=100 + m + n, dry_fraction=0.3)
    kinds = {t: ("reflective", None) for t in mesh.tag_boundary_cells}
    res = {}
    for precision in ("fp64", "mixed"):
        d = make_domain(p, e, b, "DE1", st, kinds, precision=precision)
        for _ in d.evolve(yieldstep=0.5, finaltime=2.0):
            pass
        res[precision] = (_depth(d), d.quantities["stage"].centroid_values.sum())
    assert np.abs(res["mixed"][0] - res["fp64"][0]).max() <= DEPTH_TOL


def test_pool_rejects_a_scenario_beyond_its_capacity():
    """A scenario larger than the free cells is refused with an error; the
    pool keeps working for scenarios that fit."""
    from anuga_core_gb300 import _lib, mixed
    from anuga_core_gb300.serve import de1_params
    pool = mixed.Pool(256, 4096, 2)
    try:
        free = pool.capacity()["cells"]
        big = Mesh(*rectangular_cross(16, 16, 16.0, 16.0))          # 1024 triangles
        assert len(big) > free
        with pytest.raises(_lib.AgxError):
            pool.add(big, de1_params())
        assert pool.capacity()["cells"] == free
        small = Mesh(*rectangular_cross(2, 2, 2.0, 2.0))           # 16 triangles
        sid = pool.add(small, de1_params())
        z = np.zeros(len(small))
        pool.set_field(sid, "elev_c", z)
        pool.set_field(sid, "stage_c", z + 0.5)
        nb = small.boundary_length
        pool.set_boundary(sid, np.full(nb, _lib.BC_REFLECTIVE, np.int32), np.zeros((nb, 3)))
        pool.distribute(sid)
        pool.set_clock(sid, 0.0, 1e300, 1.0, 0)
        assert pool.advance() == 1                                  # one launch runs to the final time
        assert abs(pool.stats(sid).time - 1.0) < 1e-12
        assert np.allclose(pool.get_field(sid, "stage_c"), 0.5)
    finally:
        pool.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_domain_conserved_state_exchange(precision):
    """Domain.set_conserved_state / get_conserved_state with page-locked and
    pageable arrays: the state set is the state read back and the one the
    quantities show; stepping continues from it."""
    import torch
    from anuga_core_gb300 import workloads
    d = workloads.dam_break(m=20, flow_algorithm="DE1", precision=precision)
    for _ in d.evolve(yieldstep=0.5, finaltime=0.5):
        pass
    n = len(d)
    w0, uh0, vh0 = d.get_conserved_state()
    assert np.array_equal(w0, d.quantities["stage"].centroid_values)
    pin = [torch.empty(n, dtype=torch.float64, pin_memory=True).numpy() for _ in range(3)]
    z = d.quantities["elevation"].centroid_values
    rng = np.random.default_rng(7)
    w = z + np.maximum(w0 - z, 0.0) * (1.0 + 0.01 * rng.random(n))
    for arrs in ([w, uh0 * 0.5, vh0 * 0.5], None):
        if arrs is None:                                   # page-locked input
            for dst, src in zip(pin, [w, uh0 * 0.5, vh0 * 0.5]):
                dst[:] = src
            arrs = pin
        d.set_conserved_state(*arrs)
        got = d.get_conserved_state()
        # the mixed form keeps the depth w - z in FP64: the stage comes back as (w - z) + z
        tol = 0.0 if precision == "fp64" else 1e-12
        assert np.abs(got[0] - w).max() <= tol
        assert np.array_equal(got[1], uh0 * 0.5) and np.array_equal(got[2], vh0 * 0.5)
        assert np.abs(d.quantities["stage"].centroid_values - w).max() <= tol
    for _ in d.evolve(yieldstep=0.5, finaltime=1.0):
        pass
    assert abs(d.get_time() - 1.0) < 1e-12


def test_rk3_boundary_flux_sums_are_per_step():
    """The per-stage boundary flux sums reported after a step (three for
    rk3) are that step's, on both forms: the mixed ones agree with the plain
    FP64 ones to the FP32 flux tolerance and do not accumulate over steps."""
    p, e, b = rectangular_cross(16, 8, 32.0, 16.0)
    mesh = Mesh(p, e, b)
    st = random_state(mesh, seed=21, dry_fraction=0.2)
    kinds = {"left": ("dirichlet", (float(st["stage"].max()) + 0.3, 0.0, 0.0)), "right": ("transmissive", None),
             "top": ("reflective", None), "bottom": ("reflective", None)}
    res = {}
    for precision in ("fp64", "mixed"):
        d = make_domain(p, e, b, "DE2", st, kinds, precision=precision)
        for _ in d.evolve(yieldstep=0.5, finaltime=2.0):
            pass
        assert d.total_steps > 5
        res[precision] = np.asarray(d.boundary_flux_sum, float)[:3]
    scale = np.abs(res["fp64"]).max()
    assert scale > 0.0
    assert np.abs(res["mixed"] - res["fp64"]).max() <= 1e-2 * scale, res
