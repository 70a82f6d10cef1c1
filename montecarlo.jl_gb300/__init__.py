"""GB300-native DQMC sweep for the Hubbard model (MonteCarlo.jl drop-in path).

Host-side mirror of the reference's user API -- ``HubbardModel``, ``DQMC``,
``run`` (the reference's ``run!``) and the Hirsch / Gauss-Hermite fields --
driving the CUDA library ``libdqmc_gb300.so`` through its C ABI
(``include/dqmc_gb300.h``).  The package directory is named
``montecarlo.jl_gb300``; it is imported under the module name
``montecarlo_gb300`` (see ``__graft_entry__.load_package``).
"""
from .lattices import (Bond, Chain, CubicLattice, Honeycomb, Lattice, SquareLattice,  # noqa: F401
                       TriangularLattice, UnitCell)
from .model import (DENSITY_GHQ, DENSITY_HIRSCH, MAGNETIC_GHQ, MAGNETIC_HIRSCH,  # noqa: F401
                    AttractiveHubbardModel, DensityGHQField, DensityHirschField, DQMCParameters,
                    HubbardModel, MagneticGHQField, MagneticHirschField, RepulsiveHubbardModel,
                    generate_chunks, hopping_exponentials)
from .measurements import (LogBinner, double_occupancy as double_occupancy_kernel,  # noqa: F401
                           interaction_energy, occupation_kernel, spin_density_correlation_z,
                           spin_susceptibility_z, structure_factor, time_displaced_sdc_z,
                           susceptibilities, time_displaced_correlations, CORRELATIONS,
                           current_operator, bilinear_correlation, pair_form_factor,
                           pair_correlation, td_arrays, by_distance)
from .dqmc import (DQMC, ExitCode, Measurement, double_occupancy, greens_measurement,  # noqa: F401
                   occupation, spin_density_correlation)


def run(mc, **kwargs):
    """``run!(mc)`` of the reference (DQMC.jl:252)."""
    return mc.run(**kwargs)
from .serving import Request, Server, poisson_stream, request_config, run_ensemble  # noqa: F401
from .tempering import neighbour_partners, run_tempering  # noqa: F401,E402
