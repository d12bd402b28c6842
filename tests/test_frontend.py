"""Front end (the reference's PASIf.py operations, vectorised) on CPU."""
import warnings

import numpy as np
from scipy.sparse import csc_matrix, dia_matrix
from scipy.sparse.linalg import inv

from pasif_gb300.frontend import _neg_inverse


def test_neg_inverse_equals_sparse_inv():
    """-M^-1 of a diagonal M by entry-wise division equals -1 * scipy's sparse
    inv (PASIf.py:609) in format, index arrays and every bit of the values;
    other matrices go through inv itself."""
    rng = np.random.default_rng(0)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        for _ in range(10):
            G = int(rng.integers(1, 800))
            d = rng.uniform(0.01, 100, G) * rng.choice([-1, 1], G) * 10.0 ** rng.integers(-8, 8, G)
            M = dia_matrix((d, [0]), shape=(G, G))
            a, b = _neg_inverse(M), -1. * inv(M)
            assert a.format == b.format
            np.testing.assert_array_equal(a.indptr, b.indptr)
            np.testing.assert_array_equal(a.indices, b.indices)
            np.testing.assert_array_equal(a.data, b.data)
        M = csc_matrix(np.array([[2.0, 1.0], [0.0, 3.0]]))
        np.testing.assert_array_equal(_neg_inverse(M).toarray(), (-1. * inv(M)).toarray())
