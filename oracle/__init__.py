"""CPU oracle for the pairwise-interaction hot path (test infrastructure).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this package, and only as the checker or the timed CPU
reference.  The GPU product has no CPU fallback and never imports it.
"""
