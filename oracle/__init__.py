"""CPU oracle for the interpolation and block hot path.

TEST INFRASTRUCTURE ONLY. Nothing in the product package imports, links or
executes anything under ``oracle/``; only ``tests/``, ``__graft_entry__.smoke()``
and the ``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` use it, and
only as the checker or as the timed CPU baseline, never as the thing measured
or shipped.

What lives here:

* ``oracle.interp`` -- a vectorised torch-on-CPU restatement of the reference's
  pure-torch interpolation path (``ungrid_torch`` / ``grid_torch`` /
  ``weights_torch`` / ``kaiser_bessel_torch`` in
  ``src/torchlinops/functional/_interp/{ungrid,grid,kernels}.py``), runnable in
  float32 (mirror of the reference arithmetic) or float64 (the FP64 oracle),
  plus the trajectory gradient obtained by autograd through the float64
  restatement.
* ``oracle.blocks`` -- the unfold / fold restatement
  (``src/torchlinops/functional/_unfold/{unfold,fold}.py``).
* ``oracle.binning`` -- bin keys and the stable permutation that the GPU plan
  must reproduce bit-exactly.
* ``oracle.cg`` -- conjugate gradients in float64.

Pinning: ``tests/test_oracle_golden.py`` checks every function here against
golden vectors that ``tests/golden/make_golden.py`` produced by importing and
running the reference itself (torchlinops 0.7.4, CPU path).
"""
