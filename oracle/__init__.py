"""CPU FP64 oracle for the jQMC walker path -- TEST INFRASTRUCTURE ONLY.

This package is a NumPy restatement of the reference's formulas (each function
cites the reference file:line it follows).  It exists to check the CUDA path:
only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import it, and only as the checker or the timed CPU baseline.
The product path (``jqmc_gb300``) never imports it and has no CPU fallback.

Parity pin: ``tests/golden/make_golden.py`` runs the reference's own functions
(under a NumPy stand-in for JAX, since JAX is not installed) on seeded inputs
and stores their outputs in ``tests/golden/*.npz``; ``tests/test_oracle_golden.py``
checks this oracle against those fixtures.
"""
