"""sunny_gb300 -- GB300-native (sm_103a) spin-dynamics hot path of Sunny.jl behind a C ABI.

The directory is ``sunny.jl_gb300/``; it is imported under the module name
``sunny_gb300`` (see ``__graft_entry__.package()``). Everything that computes runs in
``libsunnygb300.so``; this package only mirrors Sunny's host API.
"""
from .crystal import (Bond, Crystal, bond_parity, lattice_vectors, cubic_crystal, bcc_crystal,
                      fcc_primitive_crystal, diamond_crystal, pyrochlore_crystal, triangular_crystal)
from .operators import (spin_matrices, spin_matrices_of_dim, stevens_matrices_of_dim, rcs_factors,
                        matrix_to_stevens_coefficients, expected_spin, ket_from_dipole,
                        hermitian_basis, tensor_decomposition)
from .system import (System, Moment, Langevin, ImplicitMidpoint, step, energy, energy_per_site,
                     magnetization, energy_grad, set_exchange, set_onsite_coupling, set_field,
                     randomize_spins, polarize_spins, langevin_noise, LocalSampler, propose_uniform,
                     propose_flip, propose_delta, mix_proposals, local_energy_change, local_colors,
                     clone_system, to_inhomogeneous, set_exchange_at, set_onsite_coupling_at,
                     set_vacancy_at, remove_periodicity, minimize_energy, MinimizationResult, enable_dipole_dipole)
from .correlations import (SampledCorrelations, MeasureSpec, ssf_trace, ssf_perp, ssf_custom, add_sample,
                           merge_correlations, compare_correlations, systematic_difference, available_energies, available_wave_vectors,
                           adjusted_dt_and_downsampling_factor, all_dipole_observables, intensities,
                           intensities_static, Intensities)
from .tempering import ReplicaBatch, ParallelTempering, SystemParallelTempering, exchange_round
from .adjoint import SampledCorrelationsAdjoint
from ._abi import SunnyGPUError, load as load_library

__all__ = [n for n in dir() if not n.startswith("_")]
