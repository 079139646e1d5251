"""twoldg: the GB300-native OLDG field step of TreeWaveOLDG.jl.

A Python mirror of the reference package's API for the field right-hand
side and RK4 step (src/evolution.jl, src/stepping.jl, src/sinewave.jl,
src/refinement.jl) over the C ABI of libtwoldg (include/twoldg.h), whose
sm_103a kernels do all the arithmetic.
"""
from .nativebuild import build, lib_path
from .element import Element, element_table
from .forest import Forest, nested_cubes, refine_regions, wave_forest
from .problem import (WaveIntegrator, WaveProblem, check_layout, initial_state, oldg_timestep,
                      quadrature_norm, solve, truncate_stage, truncate_state, wave_energy, wave_integrator,
                      wave_norm, wave_rhs)
from .drivers import (convergence_rate, reflect_errors, reflect_exact, reflect_omega, wave_errors,
                      wave_exact, wave_omega)
from .indicator import modal_indicator, mode_amplitude
from .batch import Batch, fill_batch, sine_ensemble
from .geometry import (PolarAnnulus, annulus_errors, annulus_exact, annulus_forest, annulus_wavenumber,
                       metric_tables, projector_mode)
from .ball import (BallForest, DirichletData, OutgoingPulse, PlaneWave, RadiativeBoundary, SevenPatchBall,
                   SphericalStandingWave, ThirteenPatchBall, radiative_errors, sevenpatch_errors, sevenpatch_exact,
                   sevenpatch_forest, thirteenpatch_forest)

from .regrid import COARSEN, KEEP, REFINE, refine_flags, refine_mark, regrid, transfer_state
from .blast import adaptive_blast, blast_exact, blast_initial, blast_reference, refinement_buffer, uniform_blast

from .extraction import (PlaneExtraction, SphereExtraction, ball_patch_point, harmonic_modes, plane_values,
                         sphere_modes, sphere_rule, sphere_values, spherical_harmonics)
from .transfer import (ParticleSupport, TransferPlan, particle_forces, particle_frame, project_source, reconstruct,
                       reconstruct_gradient, self_inertia, source_pairing, source_rhs, transfer_table)

__all__ = [n for n in dir() if not n.startswith("_")]
