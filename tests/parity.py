"""Parity measures shared by the GPU tests, and the bounds they are held to.

A coupling T is compared with the FP64 reference R (the reference's own solver
output, or the oracle's FP64 restatement on the same inputs) three ways:

  coupling_err  max|T - R| / max|R|                                 <= COUPLING_TOL  (1e-4)
  element_err   max |T_ij - R_ij| / |R_ij| over the entries with
                |R_ij| >= ELEMENT_FLOOR * max|R| (1e-6 of the largest) <= ELEMENT_TOL  (1e-4)
  marginal_err  max_i |r_i - r_ref_i| / max_i r_ref_i, for the row
                sums and the column sums                            <= MARGINAL_TOL  (1e-6)

The normalised-max measure alone lets a small entry be wrong by orders of
magnitude; the elementwise one bounds every entry that carries mass down to a
millionth of the largest. FP32 storage of the cost puts a relative error of
about C 2^-24 / eps on each entry's exponent (below 1e-5 for median-normalised
costs at eps >= 0.01), which is what these bounds leave room for.
"""
import numpy as np

COUPLING_TOL = 1e-4
ELEMENT_TOL = 1e-4
ELEMENT_FLOOR = 1e-6
MARGINAL_TOL = 1e-6


# The on-the-fly (tensor-core) form forms every exponent from FP16 hi/lo splits
# of the points (22 significant bits) accumulated in FP32 on the tensor cores:
# an absolute exponent error of about kappa |x| |y| 2^-22, a hundred times the
# streamed form's FP32 storage of C for near neighbours. Its couplings meet
# COUPLING_TOL; its small entries and marginals are held to these bounds, by the
# final epsilon: (element bound, marginal bound).
ONTHEFLY_BOUNDS = {0.05: (1e-4, 2e-5), 0.01: (2e-3, 2e-4)}

# The batched solver's pass sums each exponent as one FP32 fma of the FP32
# weight and cost, relative to the row's offset (its speculative form), so
# FP32 rounding of weights and exponents of tens to hundreds stays in each
# entry (the single-problem passes remove it with split weights and exact
# offset subtraction, at a cost the exp-bound batched pass does not pay). Its
# couplings and entries meet COUPLING_TOL and ELEMENT_TOL; its marginals this:
BATCHED_MARGINAL_TOL = 3e-6


def coupling_err(T, R):
    return float(np.abs(T - R).max() / np.abs(R).max())


def element_err(T, R, floor=ELEMENT_FLOOR):
    T, R = np.asarray(T), np.asarray(R)
    keep = np.abs(R) >= floor * np.abs(R).max()
    return float((np.abs(T[keep] - R[keep]) / np.abs(R[keep])).max())


def marginal_err(T, R):
    r = np.abs(T.sum(1) - R.sum(1)).max() / np.abs(R.sum(1)).max()
    c = np.abs(T.sum(0) - R.sum(0)).max() / np.abs(R.sum(0)).max()
    return float(max(r, c))


def errors(T, R):
    """All three measures, as a dict (for reports)."""
    return {'coupling_max_rel_err': coupling_err(T, R), 'element_max_rel_err': element_err(T, R),
            'marginal_max_rel_err': marginal_err(T, R)}


def assert_parity_onthefly(T, R, eps, what=''):
    """The on-the-fly form's bounds (ONTHEFLY_BOUNDS) at final epsilon eps."""
    el_tol, mg_tol = ONTHEFLY_BOUNDS[eps]
    e = errors(T, R)
    assert e['coupling_max_rel_err'] <= COUPLING_TOL, (what, e)
    assert e['element_max_rel_err'] <= el_tol, (what, e)
    assert e['marginal_max_rel_err'] <= mg_tol, (what, e)
    return e


def assert_parity_batched(T, R, what=''):
    """The batched solver's bounds: COUPLING_TOL, ELEMENT_TOL, BATCHED_MARGINAL_TOL."""
    e = errors(T, R)
    assert e['coupling_max_rel_err'] <= COUPLING_TOL, (what, e)
    assert e['element_max_rel_err'] <= ELEMENT_TOL, (what, e)
    assert e['marginal_max_rel_err'] <= BATCHED_MARGINAL_TOL, (what, e)
    return e


def assert_parity(T, R, marginals=True, what=''):
    """T matches R within the three bounds (marginals optional: a coupling
    returned un-normalised after max_iter is compared entry by entry only)."""
    e = errors(T, R)
    assert e['coupling_max_rel_err'] <= COUPLING_TOL, (what, e)
    assert e['element_max_rel_err'] <= ELEMENT_TOL, (what, e)
    if marginals:
        assert e['marginal_max_rel_err'] <= MARGINAL_TOL, (what, e)
    return e
