"""CPU oracle for the transport-map path — TEST INFRASTRUCTURE ONLY.

This package restates, in plain FP64 NumPy, the reference's algorithm for
the unbalanced entropic OT transport-map path (wot 1.0.8):

* ``oracle.optimal_transport`` — ``wot/ot/optimal_transport.py`` (the
  growth-iteration driver, the duality-gap solver, the fixed-iteration
  solver and Chizat's primal/dual objectives);
* ``oracle.ot_model``          — ``wot/ot/ot_model.py`` (median-normalised
  squared-Euclidean cost, per-pair orchestration) and ``wot/ot/util.py``
  ``compute_pca`` (restated with an exact SVD; the reference uses
  scikit-learn's randomized SVD, see that module);
* ``oracle.torch_ot``          — the default solver and the cost again, on FP64
  torch tensors in the same operation order, so that the same reference
  arithmetic checks 20,000 x 25,000 and larger problems on a GPU;
* ``oracle.tmap``              — ``wot/tmap/transport_map_model.py``,
  ``wot/tmap/chaining.py``, ``wot/tmap/util.py`` and ``wot/population.py``.

Pinning: the restatement is checked against the reference's own
known-answer test (``tests/test_transport.py``: 3x3 identity coupling at
epsilon=0.01), against the reference's orphan integer transport-map
fixtures (``tests/inputs/transport_maps/*.csv``) and against golden
vectors produced by running the reference's solver module itself
(``tests/golden/make_golden.py``, committed with its outputs).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU
baseline / reference arm may import this package, and only as the
checker or the timed CPU baseline: the product path (``wot_gb300``) never
calls into it.
"""
