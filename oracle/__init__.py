"""CPU oracle for the ceviche Yee-stencil path -- TEST INFRASTRUCTURE ONLY.

This package restates, in numpy/scipy FP64, the reference algorithms that the
GPU library replaces.  It is the checker: only ``tests/``, the
``__graft_entry__.smoke()`` check and ``bench.py``'s CPU-baseline / reference
arm may import it.  The product package (``ceviche_gb300``) never imports it
and has no CPU fallback.

Parity pinning: every function here is checked against fixtures generated by
running the unmodified ceviche 0.1.3 forward code (``tests/golden/``), see
``tests/test_oracle_golden.py``.  Gradients are pinned against central finite
differences of that reference forward code (autograd itself is not available,
so the reference's VJP rules are restated in ``oracle.fdfd`` / ``oracle.fdtd``).

Modules:
    constants  -- ceviche/constants.py:7-11
    fdfd       -- ceviche/derivatives.py:34-216, ceviche/fdfd.py:58-244,
                  ceviche/primitives.py:103-148, ceviche/solvers.py:50-62
    fdtd       -- ceviche/fdtd.py:74-316, ceviche/derivatives.py:16-30,
                  ceviche/utils.py:153-176
"""
