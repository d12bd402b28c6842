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


def _random_tensor(rng, n, order, nnz):
    from pasif_gb300.frontend import coo_tensor
    t = coo_tensor([n] * order)
    t.val = rng.normal(size=nnz).tolist()
    t.indices = rng.integers(0, n, size=nnz * order).tolist()
    return t


def _concat_loop(a, b):
    """Pairwise block-diagonal concatenation written as index loops (the
    semantics of PASIf.py:86-100: b's indices shifted by a's dimensions,
    values appended, dimensions summed)."""
    nd = len(a.dimensions)
    val = list(a.val) + list(b.val)
    idx = list(a.indices)
    for e in range(len(b.val)):
        for d in range(nd):
            idx.append(b.indices[e * nd + d] + a.dimensions[d])
    return val, idx, [x + y for x, y in zip(a.dimensions, b.dimensions)]


def test_tensor_concatenation_equals_index_loops():
    """Vectorised block-diagonal concatenation of system tensors (one call for
    all systems, and pairwise concatenateTensor) equals index loops."""
    import copy
    from pasif_gb300.frontend import _concat_tensors
    rng = np.random.default_rng(5)
    for order in (3, 4, 5):
        ts = [_random_tensor(rng, int(rng.integers(1, 6)), order, int(rng.integers(0, 7))) for _ in range(9)]
        ref = copy.deepcopy(ts[0])
        for t in ts[1:]:
            ref.val, ref.indices, ref.dimensions = _concat_loop(ref, t)
        got = _concat_tensors(ts)
        assert got.dimensions == ref.dimensions
        assert got.val == ref.val and got.indices == ref.indices
        pair = copy.deepcopy(ts[0])
        for t in ts[1:]:
            pair.concatenateTensor(t)
        assert pair.dimensions == ref.dimensions
        assert pair.val == ref.val and pair.indices == ref.indices


def test_tensor_diag_scaling_and_offsets():
    """multiplyByDiagMatrix scales each value by the diagonal entry of its
    destination (first) index; offsetDimmension shifts one index position."""
    rng = np.random.default_rng(6)
    t = _random_tensor(rng, 5, 3, 11)
    d = rng.normal(size=5)
    v0, i0 = list(t.val), list(t.indices)
    t.multiplyByDiagMatrix(d)
    assert t.val == [v0[e] * d[i0[3 * e]] for e in range(11)]
    t.offsetDimmension(2, 4)
    assert t.indices == [i0[k] + (4 if k % 3 == 2 else 0) for k in range(33)]
    assert t.getIndicesDim(0) == i0[0::3]


def test_unfold_is_block_diagonal():
    """The unfolded system (PASIf.py:475-605) of several systems: M, B, K are
    the block-diagonal matrices of the per-system ones, force pattern and
    initial conditions stacked."""
    from scipy.linalg import block_diag
    from scipy.sparse import coo_matrix
    from pasif_gb300.frontend import PASIf
    rng = np.random.default_rng(7)
    sizes = [2, 3, 1, 4]
    vecM = [dia_matrix((rng.uniform(1, 2, s), [0]), shape=(s, s)) for s in sizes]
    vecB = [coo_matrix(rng.normal(size=(s, s)) * (rng.random((s, s)) < 0.5)) for s in sizes]
    vecK = [coo_matrix(rng.normal(size=(s, s))) for s in sizes]
    gam = [[_random_tensor(rng, s, 3, 2) for s in sizes], [_random_tensor(rng, s, 4, 3) for s in sizes]]
    vecF = [rng.normal(size=s) for s in sizes]
    vecIC = [rng.normal(size=s) for s in sizes]
    G, M, Bm, Km, ts, F, IC = PASIf._unfold(None, vecM, vecB, vecK, gam, vecF, vecIC)
    assert G == sum(sizes)
    np.testing.assert_array_equal(M.toarray(), block_diag(*[m.toarray() for m in vecM]))
    np.testing.assert_array_equal(Bm.toarray(), block_diag(*[b.toarray() for b in vecB]))
    np.testing.assert_array_equal(Km.toarray(), block_diag(*[k.toarray() for k in vecK]))
    np.testing.assert_array_equal(F, np.concatenate(vecF))
    np.testing.assert_array_equal(IC, np.concatenate(vecIC))
    assert ts[0].dimensions == [G] * 3 and ts[1].dimensions == [G] * 4
