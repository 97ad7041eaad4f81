"""A multiprocessor-mode adapter for the reference's own Domain.

The reference Domain dispatches each DE phase on ``multiprocessor_mode``;
in mode 4 it calls methods of a ``gpu_interface`` object
(shallow_water/shallow_water_domain.py:1872, 1912, 2037, 2146, 2878-2900;
shallow_water/friction.py:125-147).  ``AGX_interface`` offers the same
methods, under the same names and called the same way, over the plain FP64
kernels of libagx: each call copies in the arrays the phase reads from the
domain's numpy storage, runs the phase on the GPU and copies back what it
writes, so the reference's Python boundary objects, operators and time loop
keep working around it.  A maintainer wires it in with

    domain.set_multiprocessor_mode(4)
    domain.gpu_interface = AGX_interface(domain)

(set before the first evolve).  The arrays it touches are named as the
reference's Quantity storage (quantity.py:59-103) and Domain attributes.
Whole yieldsteps without host round trips are the job of
anuga_core_gb300.Domain; this adapter is the per-phase seam.
"""
from __future__ import annotations

import numpy as np

from . import _lib
from .tables import pack_tables

_FULL = {"stage": "stage", "xmom": "xmomentum", "ymom": "ymomentum", "elev": "elevation", "height": "height",
         "friction": "friction"}
_SLOT = {"c": "centroid_values", "e": "edge_values", "v": "vertex_values", "b": "boundary_values",
         "x": "explicit_update", "s": "semi_implicit_update"}


class AGX_interface:
    def __init__(self, domain):
        self.domain = domain
        d = domain
        p = _lib.Params()
        p.g, p.epsilon, p.minimum_allowed_height = d.g, d.epsilon, d.minimum_allowed_height
        for k in ("beta_w", "beta_w_dry", "beta_uh", "beta_uh_dry", "beta_vh", "beta_vh_dry"):
            setattr(p, k, getattr(d, k))
        p.CFL, p.evolve_max_timestep, p.evolve_min_timestep = d.CFL, d.evolve_max_timestep, d.evolve_min_timestep
        p.extrapolate_velocity_second_order = 1 if d.extrapolate_velocity_second_order else 0
        p.low_froude = int(getattr(d, "low_froude", 0))
        p.timestepping_method = {"euler": 1, "rk2": 2, "rk3": 3}[d.get_timestepping_method()]
        p.use_sloped_mannings = 1 if getattr(d, "use_sloped_mannings", False) else 0
        p.max_smallsteps = int(getattr(d, "max_smallsteps", 50))
        p.precision = _lib.AGX_PREC_FP64
        self.fluxcalls = p.timestepping_method
        self.substep = 0
        self.scn = _lib.Scenario(pack_tables(d.mesh), p)

    def close(self):
        self.scn.close()

    # -- copies between the domain's numpy storage and the device ---------
    def _push(self, loc, names=("stage", "xmom", "ymom")):
        for n in names:
            a = getattr(self.domain.quantities[_FULL[n]], _SLOT[loc])
            self.scn.set("%s_%s" % (n, loc), np.ascontiguousarray(a, np.float64))

    def _pull(self, loc, names=("stage", "xmom", "ymom")):
        for n in names:
            a = getattr(self.domain.quantities[_FULL[n]], _SLOT[loc])
            a[...] = self.scn.get("%s_%s" % (n, loc)).reshape(a.shape)

    # -- the phases, as the reference's Domain calls them ------------------
    def protect_against_infinitesimal_and_negative_heights_kernal(self, *args, **kwargs):
        """protect_new(domain) -> mass error (shallow_water_domain.py:2016-2048)."""
        self._push("c", ("stage", "xmom", "ymom", "elev"))
        mass = self.scn.protect()
        self._pull("c")
        return mass

    def extrapolate_second_order_edge_sw_kernel(self, *args, **kwargs):
        """extrapolate_second_order_edge_sw(domain) (sw_domain_openmp.c:1336-1952):
        edge and vertex values of stage, momenta, bed and height; the
        momenta of cells surrounded by dry cells are zeroed."""
        self._push("c", ("stage", "xmom", "ymom", "elev"))
        self.scn.distribute(with_protect=False)
        self._pull("c", ("stage", "xmom", "ymom", "height"))
        names = ("stage", "xmom", "ymom", "elev", "height")
        self._pull("e", names)
        self._pull("v", names)

    def compute_fluxes_ext_central_kernel(self, *args, **kwargs):
        """compute_fluxes_ext_central(domain, timestep) -> flux timestep
        (sw_domain_openmp.c:456-772), with the boundary values the domain's
        boundary objects wrote; the stages of a step are counted here as the
        reference's static counter counts them (:492-505)."""
        d = self.domain
        self._push("c", ("stage", "xmom", "ymom", "elev", "height"))
        self._push("e", ("stage", "xmom", "ymom", "elev", "height"))
        self._push("b")
        substep = self.substep
        dt = self.scn.compute_fluxes(substep)
        self._pull("x")
        d.max_speed[:] = self.scn.get("max_speed")
        bfs = getattr(d, "boundary_flux_sum", None)
        if bfs is not None and substep < len(bfs):
            bfs[substep] = self.scn.stats().boundary_flux_sum[substep]
        self.substep = (substep + 1) % self.fluxcalls
        return dt if substep == 0 else d.evolve_max_timestep

    def compute_forcing_terms_manning_friction_flat(self, *args, **kwargs):
        """manning_friction_implicit (friction.py:23-72; sw_domain_openmp.c:1954-1986)."""
        self._push("c", ("stage", "xmom", "ymom", "elev", "friction"))
        self._push("s", ("xmom", "ymom"))
        self.scn.compute_forcing()
        self._pull("s", ("xmom", "ymom"))

    compute_forcing_terms_manning_friction_sloped = compute_forcing_terms_manning_friction_flat

    def update_conserved_quantities_kernal(self, *args, **kwargs):
        """Quantity.update for stage and momenta with the domain's timestep,
        then fix_negative_cells (quantity.c:772-818, sw_domain_openmp.c:2037-2056);
        returns the number of cells set to zero depth."""
        d = self.domain
        self._push("c", ("stage", "xmom", "ymom", "elev"))
        self._push("x")
        self._push("s")
        n = self.scn.update_conserved(d.timestep)
        self._pull("c")
        self._pull("s")
        return n
