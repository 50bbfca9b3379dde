"""CPU oracle for the far-field butterfly hot path (test infrastructure only).

This package restates, in plain NumPy/SciPy, the reference algorithms of
ButterflyFactorizations.jl that the GPU library replaces: geometry, 2^d cluster
trees, level padding, near/far interaction lists, the PartialQR compressor,
`assemble_BF`, the flat / dictionary matvecs, the materialised adjoint and the
global far-field driver.  Every function cites the reference file:line it
follows.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this package, and there only as the checker.  The
library under ``butterflyfactorizations.jl_gb300/`` never imports it.

Parity status: **parity unpinned**.  The reference is pure Julia (no Julia in
this image) and ships no golden vectors; its tests are tolerance checks against
dense BEAST products (``test/test_subroutines.jl:174-182``).  The oracle is
therefore pinned on (a) those tolerance criteria rerun on the point-Helmholtz
configurations, (b) LAPACK ``zgeqp3`` (via SciPy) for the pivoted QR that
``LowRankApprox.pqr`` performs, and (c) self-consistency between the three
reference matvec orders.
"""
