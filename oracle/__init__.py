"""CPU oracle for the Mie hot path -- TEST INFRASTRUCTURE ONLY.

Nothing in the product package (``geosmie_gb300``) imports this package.  It is
used by ``tests/`` as the checker, by ``__graft_entry__.smoke()`` to check one
small GPU invocation, and by ``bench.py`` for the CPU baseline leg and the
``--impl reference`` arm.

Modules
-------
pymie        restatement of pymiecoated (mie_coeffs.py, mie_props.py,
             mie_coated.py): a_n/b_n, efficiencies, pi_n/tau_n, S1/S2.
integration  restatement of the runoptics table builder
             (geosmie/dointegration.py, geosmie/particleparams.py): x grids,
             growth, refractive-index mixing, PSD weights, integratePSD with
             its weighting quirks, phase-function normalisation.
gsf          ctypes front end of ``spher_expan.c``, a C restatement of
             gsf/spher_expan.f (Gauss nodes, interpolation, generalized
             spherical functions, expansion coefficients).

Parity pinning: ``tests/golden/make_golden.py`` imports the reference's own
Python code (pymiecoated, dointegration) and records its outputs as fixtures;
``tests/test_oracle_golden.py`` checks this oracle against those fixtures and
against the known-answer values of pymiecoated/test/test_mie.py.  The GSF
restatement has no reference test or fixture (the Fortran cannot be compiled
here: no Fortran compiler); it is pinned by known answers instead
(Gauss-Legendre nodes, Henyey-Greenstein moments, MATR round trip).
"""
