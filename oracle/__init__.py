"""FP64 CPU oracle for the kinematical spot-pattern path -- TEST INFRASTRUCTURE.

This package is the checker, never the product.  Only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline / reference legs of
``bench.py`` may import it.  The ``diffsims_gb300`` package never imports it and
has no CPU fallback: its compute path is the CUDA library or an error.

What it restates (numpy, float64), with the reference file:line each function
follows, is listed in each function's docstring.  The reference is diffsims
0.7.x (pure Python); citations are paths inside that project.

Pinning: the restatement is checked against the reference's own golden
vectors and known-answer tests (tests/test_oracle_golden.py):

* ``diffsims/tests/generators/old_simulation.npy`` (graphite, 128x128, atol 1e-8)
* spot counts 70 / 250 / 250 (diffsims/tests/generators/test_simulation_generator.py:137-161)
* enumeration sizes and orders (diffsims/tests/crystallography/test_reciprocal_lattice_vector.py:76-116,
  doctest diffsims/crystallography/reciprocal_lattice_vector.py:1107-1127)
* wavelength and intensity KATs (diffsims/tests/utils/test_sim_utils.py:49-60,330-394)
* fixtures produced by running the reference's own ``sim_utils`` and
  ``shape_factor_models`` functions (tests/golden/make_golden.py).

Unpinned (stated, not hidden): the reference's ``inv(stdbase @ recbase)``
re-basing of fractional coordinates (diffsims/utils/sim_utils.py:290-291) is the
identity for every cell whose lattice frame is x || a, z || c* (the frame used
here); for triclinic cells built through orix/diffpy it has not been checked
because orix and diffpy are not installable in the build container.
"""
