"""anuga_core_gb300: GPU (GB300, sm_103a) implementation of ANUGA's DE
shallow-water timestep behind the anuga.Domain API.

The user API mirrors the reference package names::

    import anuga_core_gb300 as anuga
    domain = anuga.rectangular_cross_domain(100, 100, len1=100., len2=100.)
    domain.set_flow_algorithm('DE0')
    domain.set_quantity('elevation', lambda x, y: -x / 20)
    ...
    for t in domain.evolve(yieldstep=1.0, finaltime=10.0):
        print(domain.timestepping_statistics())
"""
from .mesh import Mesh, rectangular_cross
from .domain import Domain, rectangular_cross_domain
from .boundaries import (Reflective_boundary, Transmissive_boundary, Dirichlet_boundary, Time_boundary,
                         Transmissive_n_momentum_zero_t_momentum_set_stage_boundary,
                         Transmissive_momentum_set_stage_boundary, Transmissive_stage_zero_momentum_boundary,
                         Time_stage_zero_momentum_boundary, Dirichlet_discharge_boundary,
                         Flather_external_stage_zero_velocity_boundary, Characteristic_stage_boundary,
                         Time_space_boundary, Inflow_boundary, Compute_fluxes_boundary)
from .operators import Inlet_operator, Rate_operator
from .checkpoint import load_checkpoint_file

__all__ = ["Mesh", "rectangular_cross", "Domain", "rectangular_cross_domain", "Reflective_boundary",
           "Transmissive_boundary", "Dirichlet_boundary", "Time_boundary",
           "Transmissive_n_momentum_zero_t_momentum_set_stage_boundary", "Transmissive_momentum_set_stage_boundary",
           "Transmissive_stage_zero_momentum_boundary", "Time_stage_zero_momentum_boundary",
           "Dirichlet_discharge_boundary", "Flather_external_stage_zero_velocity_boundary",
           "Characteristic_stage_boundary", "Time_space_boundary", "Inflow_boundary", "Compute_fluxes_boundary",
           "Rate_operator", "Inlet_operator", "load_checkpoint_file"]
