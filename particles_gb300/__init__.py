"""particles_gb300 -- GB300-native test-particle integrator.

The hot path of PARTICLES (adaptive Cash-Karp RK5 / DOP853 step loop,
trilinear gather of U and B, relativistic Lorentz force) as fused sm_103a
CUDA kernels behind a C ABI (include/particles_gb300.h).  This package is the
Python face of that ABI plus the host-side helpers the reference driver
provides (parameter vector, time grid, initial states, synthetic fields).
"""
from . import fields, initial, params
from .integrations import (Ensemble, Fields, OutputStream, carry_buffer, integrate,
                           integrate_dp853, integrate_rk5)
from .params import method_id, pack_params, time_grid

__all__ = [
    "Ensemble", "Fields", "OutputStream", "carry_buffer", "fields", "initial", "integrate", "integrate_dp853",
    "integrate_rk5", "method_id", "pack_params", "params", "time_grid",
]
