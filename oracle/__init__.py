"""CPU oracle for the SpMV / power-method path (test infrastructure only).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
may import this package.  It is the checker, never the product: the GPU library
in ``thesis_spmv_gb300`` does not import, link or call it.
"""
