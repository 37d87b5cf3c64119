"""CPU oracle for the scattering hot path (test infrastructure only).

This package restates, in numpy, the algorithm of kymatio's 2-D and 1-D
scattering transforms (kymatio 0.4.0.dev0):

* ``oracle.filters``      -- the Morlet/Gabor filter banks
  (kymatio/scattering2d/filter_bank.py, kymatio/scattering1d/filter_bank.py)
* ``oracle.scattering2d`` -- the 2-D cascade and its numpy backend ops
  (kymatio/scattering2d/core/scattering2d.py, .../backend/numpy_backend.py)
* ``oracle.scattering1d`` -- the 1-D cascade, padding and output formatting
  (kymatio/scattering1d/core/scattering1d.py, .../frontend/base_frontend.py)

It is the checker, never the product: only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline / reference arm
may import it.  Fed float64 input it computes in FP64, like the reference's
numpy backend; fed float32 it keeps the reference's float32/complex64
arithmetic.

Parity pinning: ``tests/test_oracle_golden.py`` checks this restatement
against the reference's own golden files (test_data_2d.npz, test_data_1d.npz,
re-exported under tests/golden/) and against outputs of the reference numpy
frontend generated by ``tests/golden/make_golden.py``.
"""
