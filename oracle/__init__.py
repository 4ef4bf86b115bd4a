"""TEST INFRASTRUCTURE ONLY — the CPU oracle of the explicit encoding operator.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py`` (the CPU
baseline and the ``--impl reference`` arm) may import this package, and only
as the checker / baseline, never as the product path.

Parity status: pinned by every known-answer test that the reference's own test
suite holds for this path (zero-phase ``op*ones == fill(2,3)`` and unit-weight
normal ``== fill(3,4)``; ``basisfunc_spha(...,17) == [-24,-96]``), by the
reference's deterministic fixture problem restated from its test file, and by
an independent FP64 dense-matrix restatement (``dense.py``) cross-checked
against the blocked C restatement (``hoe_oracle.c``).  The reference itself
(Julia) cannot run in this environment.
"""
