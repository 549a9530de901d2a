"""Test infrastructure: the CPU oracle of the per-projection-direction distance stage.

This package is the checker, never the product.  Only ``tests/``, ``__graft_entry__.smoke()`` and
``bench.py``'s CPU-baseline / reference arm import it.  The GPU product path in
``manifoldem_python_gb300`` never imports it and fails loudly when its CUDA library is missing.

Parity status: pinned.  ``distance_oracle.pd_op`` is checked against outputs of the reference's own
``getDistanceCTF_local_Conj9combinedS2.op`` run on identical inputs (fixtures in
``tests/golden/``, produced by ``tests/golden/make_golden.py``).
"""
