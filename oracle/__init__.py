"""Oracle package: CPU (NumPy FP64) restatement of the ad-dft plane-wave path.

Test infrastructure only.  ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline legs of ``bench.py`` are the only allowed importers; the GPU
product never imports it.
"""
