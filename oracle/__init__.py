"""CPU oracle for the particle-mesh force-and-step path of JaxPM.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and
the ``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may import
this package, and only as the checker or as the timed CPU restatement.  The
product (``jaxpm_gb300``) never imports it and has no CPU fallback.

What it is: a NumPy restatement, in float32 and float64, of the reference's
hot-path algorithm, each function citing the reference file:line it follows
(paths relative to the JaxPM project root):

* ``cic``        -- ``jaxpm/painting.py`` and ``jaxpm/painting_utils.py``
* ``fourier``    -- ``jaxpm/kernels.py``, ``jaxpm/distributed.py:37-42``,
                    ``jaxpm/pm.py:12-58``
* ``cosmology``  -- ``jaxpm/growth.py`` plus the published background,
                    growth-ODE and Eisenstein & Hu (1998) transfer function
                    that JaxPM imports from jax_cosmo
* ``nbody``      -- ``jaxpm/pm.py:61-144``, ``jaxpm/ode.py:13-147``
* ``power``      -- ``jaxpm/utils.py:14-128``

Parity status.  The reference is pure Python/JAX and needs ``jax``,
``jax_cosmo`` and ``jaxdecomp``, none of which can be imported where this
project is built, and the reference ships no golden vectors (its tests
compute every expected value live with FastPM/pmesh).  The oracle is
therefore **parity unpinned** against the running reference.  It is held
instead by analytic known-answer tests (single particles at centres, faces,
corners and periodic wraps; a uniform lattice painting a constant mesh; a
plane-wave density whose force is known in closed form; growth factors of an
Einstein-de Sitter universe) and by the committed fixtures under
``tests/golden/`` that freeze its outputs.

Third-party arithmetic restated here (absent from the reference tree):

* jaxdecomp >= 0.2.9 (``pyproject.toml:17``): ``pfft3d``/``pifft3d`` are taken
  as the unnormalised forward / normalised inverse complex 3-D DFT in natural
  axis order; ``fftfreq3d`` as ``2*pi*fftfreq(n)`` per axis (radians/cell).
* jax_cosmo (unpinned; the reference CI installs a fork): ``Esqr``,
  ``growth_factor``, ``growth_rate``, ``growth_factor_second``,
  ``growth_rate_second``, ``_compute_growth_tables`` and
  ``linear_matter_power`` are restated from the published equations; table
  resolution, integrator and second-order normalisation are this project's
  choice and are documented in ``oracle/cosmology.py``.
"""
