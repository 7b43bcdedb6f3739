"""CPU oracle of the CITRUS scatter step: test infrastructure only.

A float64 numpy restatement of the reference's algorithm for the path (cabouman/citrus v0.28.0,
``citrus/scatter_solver``): the wavefront plan and linear-discontinuous sweep, the scattering moments, the Siddon line
integrals, the uncollided fluence and first-collision source with its sampling correction, the collapsed-cone image
and the primary. Each function cites the reference lines it follows.

Only the test suite, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` use this package, always
as the checker; the product (``citrus_gb300``) never imports it. The direction sets and spherical-harmonic tables are
taken from ``citrus_gb300.quadrature`` and the panel arithmetic from ``citrus_gb300.geometry`` (pure float64 numpy
set-up code); those tables are pinned on their own against fixtures generated from the reference
(``tests/golden``), so sharing them does not weaken the check of the path's arithmetic.

Parity is pinned: ``tests/test_oracle_golden.py`` checks every oracle function against the fixtures in
``tests/golden`` produced by ``tests/golden/make_golden.py`` from the reference itself.
"""
