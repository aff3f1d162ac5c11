"""CPU oracle for the femgl Newton hot path — TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this package, as the checker or the timed CPU baseline.
The product path (the CUDA library and its Python binding) never imports it.

Parity status: the per-quadrature-point physics is pinned against the reference's
own cell kernels compiled unmodified (``oracle/_ref``) and against golden vectors
generated from them (``tests/golden``).  Mesh-level condensation and the Newton
loop restate deal.II/femgl semantics; the reference program itself cannot be built
(no deal.II/Trilinos/p4est), so those levels are pinned by the cell-level golden
matrices and by identities (free-energy gradient, symmetry), not by reference runs.
"""
