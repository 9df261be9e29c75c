"""Test infrastructure: the CPU oracle of the B-spline fitter, the
reference's own CPU fitter compiled from its sources (where present) and the
reference's own CUDA kernels compiled to PTX (ref_gpu).

Only the tests, ``__graft_entry__.smoke()``, the CPU-baseline leg of
``bench.py`` and its reference arm (``--impl reference``) may use this
package. It is the checker and the baseline, never the product."""
