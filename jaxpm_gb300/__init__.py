"""GB300-native particle-mesh engine for JaxPM's force-and-step hot path.

Modules mirror ``jaxpm``'s: ``painting`` (cic_paint, cic_read, cic_paint_dx,
cic_read_dx), ``pm`` (pm_forces, lpt, linear_field), ``ode``
(make_ode_fn, make_diffrax_ode, symplectic_fpm_ode), ``growth``,
``kernels``, ``distributed`` (fft3d, ifft3d, uniform_particles,
normal_field) and ``utils`` (power_spectrum).  ``simulate`` holds the fused
FastPM loop.  All GPU work goes through ``libpmgb.so`` (C ABI in
``include/pmgb.h``), built in-tree by ``jaxpm_gb300.build``.
"""
from . import cosmology, growth  # noqa: F401  (host-side, no GPU needed)

__version__ = "0.1.0"


def library():
    """Loads and returns the ctypes handle of libpmgb.so (raises
    ``PmgbUnavailable`` if it is not built)."""
    from . import _lib
    return _lib.load()
