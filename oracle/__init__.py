"""CPU oracle for panoptic-evaluator's hot path.

TEST INFRASTRUCTURE ONLY. This package restates, in numpy and plain Python,
the reference CPU algorithms of AndyBarcia/panoptic-evaluator
(``panoptic_evaluator/evaluator.py``, ``instance.py``, ``combined.py``,
``prefix.py``). Each function cites the reference lines it follows.

Only ``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` /
``--impl reference`` legs of ``bench.py`` may import it, and only as the
checker or the timed CPU baseline. The product package never imports it.

Parity pin: the oracle is checked against golden vectors produced by the
reference's own CPU implementation (``tests/golden/make_golden.py`` imports
the reference and writes ``tests/golden/*.npz``; ``tests/test_oracle.py``
compares).
"""

from . import panoptic, instance, combined, prefix  # noqa: F401
