"""GB300-native axisymmetric split-step NLSE propagator (fused silica).

Drop-in for the propagator path of omatousou/Rapport
(``Integrator.propagate`` -> ``step`` -> ``LinearOperator.half_linear``,
``NonlinearOperator.split`` / ``update_plasma``): Python + torch on the host,
hand-written sm_103a CUDA kernels behind the C ABI of ``libnlse.so``.
"""
from .config import Config, n_sellmeier, workload_config
from .grids import ENVELOPES, build_grids, envelope_gaussian_focused, envelope_lens, keldysh_rate
from .operators import LinearOperator, NonlinearOperator
from .integrator import Integrator
from .filament_sim import FIELD_TOGGLES, run
from .sweeps import build_scenarios, energy_scenarios, load_scenario_npz, run_scenarios, summarize

__all__ = ["Config", "n_sellmeier", "workload_config", "build_grids", "envelope_gaussian_focused",
           "envelope_lens", "ENVELOPES", "keldysh_rate", "LinearOperator", "NonlinearOperator",
           "Integrator", "run", "FIELD_TOGGLES", "build_scenarios", "energy_scenarios", "load_scenario_npz",
           "run_scenarios", "summarize"]
