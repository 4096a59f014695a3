"""CPU oracle for the MeshODE deformation hot path (test infrastructure only).

Imported by tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py``; the product path never imports it.
"""
