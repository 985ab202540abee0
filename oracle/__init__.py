"""CPU oracle for the PFEM-2 step path (TEST INFRASTRUCTURE ONLY).

Loaded by the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` as the checker.  The product (``gpupfem2_gb300``) never imports it.
"""
