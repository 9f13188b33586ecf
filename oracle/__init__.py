"""CPU oracle for the batch renderer's draw path.

Test infrastructure: imported only by ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py``.  The product package never
imports it."""
