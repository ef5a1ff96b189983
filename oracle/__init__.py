"""CPU oracle for the FastPM particle-mesh hot path — TEST INFRASTRUCTURE ONLY.

Nothing in the shipped package imports this directory.  Only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py`` (its ``cpu_baseline`` leg and its
``--impl reference`` arm) use it, and only as the checker / the timed CPU
restatement of the reference algorithm.

Contents
--------
pmesh_np      numpy restatement of the subset of the third-party ``pmesh``
              package that ``fastpm.core`` / ``fastpm.force`` call (ParticleMesh,
              RealField/ComplexField, r2c/c2r, apply, CIC/TSC paint/readout,
              uniform particle grid, identity domain layout) plus the whitenoise
              generator shared with the device code (Philox4x32-10 per mode).
cosmology_np  ``nbodykit.cosmology`` stand-in: a Cosmology with Om0 and an
              Eisenstein & Hu (1998) no-wiggle linear P(k) normalised to sigma8.
fastpm_np     float64 restatement of fastpm/core.py, fastpm/force/{lpt,gravity,
              kernels}.py and fastpm/background.py (MatterDominated).
power_np      restatement of fastpm/utils.py:power (integer-shell P(k)).

Parity status
-------------
* core.py / force / background / utils.power restatements are PINNED: they are
  compared bit-for-bit (float64, rtol 1e-12) with the reference's own unmodified
  modules run in the build container over the same pmesh stand-in; the outputs
  are committed under tests/golden/ with the script that made them.
* The pmesh subset itself is UNPINNED: pmesh / pfft / nbodykit are not vendored
  by the reference (setup.py:22 lists bare 'pmesh', 'nbodykit') and are absent
  here.  Its conventions (r2c carries 1/N, c2r does not; node-centred cells;
  CIC support 2 / TSC support 3 windows; fftfreq wavenumbers) are the ones the
  reference relies on (fastpm/tests/test_kernel.py:12-13, force/kernels.py).
  The whitenoise random stream is this project's own (pmesh's cannot be
  reproduced without its source), so the oracle's whitenoise is what both the
  oracle and the device code are fed.
"""
