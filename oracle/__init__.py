"""CPU oracle for the supereight2 dense-mapping hot path (test infrastructure only).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline legs of ``bench.py`` import
this package. The product (``supereight2_gb300`` and ``libse_gpu``) never does.
"""
