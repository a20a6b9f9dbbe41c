"""superspinsim_gb300 -- SuperSpinsim's time-stepping hot path on GB300.

Drop-in for the reference's ``generate_simulator`` / ``simulate`` (numba
kernels replaced by hand-written sm_103a CUDA in libsss.so, called through
ctypes), plus a batched persistent-kernel sweep (``sweep.Sweep``) and
adjoint gradients of integrated readouts (``adjoint.Objective``,
``adjoint.PulseObjective``).
"""
from superspinsim_gb300.generate_simulator import generate_simulator  # noqa: F401
from superspinsim_gb300.program import Program  # noqa: F401
from superspinsim_gb300 import quadratures  # noqa: F401

__version__ = "0.1.0"
