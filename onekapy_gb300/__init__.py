"""onekapy_gb300 -- GB300 (sm_103a) engine for OnekaPy's stochastic capture zones.

Reference-compatible modules (same names and signatures as OnekaPy's oneka/):
  model           Model, AquiferError, RangeError
  probabilityfield  ProbabilityField
  capturezone     compute_capturezone, compute_backtrace
  stochastic      create_stochastic_capturezone, generate_random_variate, ...
  deterministic   create_deterministic_capturezone
Engine (device-resident, batched): engine.Site, engine.realize, engine.track.
All compute runs in liboneka_gb300.so (include/oneka_gb300.h); there is no
CPU fallback.
"""
__version__ = "0.1.0"
