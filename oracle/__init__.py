"""Test infrastructure: the CPU oracle of the B-spline fitter and the
reference's own CPU fitter compiled from its sources (where present).

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may use this package. It is the checker, never the product."""
