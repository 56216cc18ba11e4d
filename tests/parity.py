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


def assert_parity(T, R, marginals=True, what=''):
    """T matches R within the three bounds (marginals optional: a coupling
    returned un-normalised after max_iter is compared entry by entry only)."""
    e = errors(T, R)
    assert e['coupling_max_rel_err'] <= COUPLING_TOL, (what, e)
    assert e['element_max_rel_err'] <= ELEMENT_TOL, (what, e)
    if marginals:
        assert e['marginal_max_rel_err'] <= MARGINAL_TOL, (what, e)
    return e
