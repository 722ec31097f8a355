"""The standalone device linear system (xg_linsoe_*, the reference's
LinearSOE calls): SparseGenColLinSOE-style assembly checked on the CPU
against a dense assembly, argument checks, and (GPU) the block-Jacobi PCG
solve against a dense solve, with node blocks and with point Jacobi."""
import numpy as np
import pytest

from xara_gb300 import gpu


def _problem(seed=0, nnode=60, nel=70, ndf=3):
    """Element-like contributions: every 'element' couples the dofs of two
    to four nodes with an SPD matrix; some dofs are constrained (-1)."""
    rng = np.random.default_rng(seed)
    n = nnode * ndf
    eq = np.arange(n).reshape(nnode, ndf)
    fixed = rng.choice(nnode, 3, replace=False)
    elems = []
    for _ in range(nel):
        nodes = rng.choice(nnode, rng.integers(2, 5), replace=False)
        ids = eq[nodes].ravel().copy()
        for f in fixed:
            if f in nodes:
                ids[np.nonzero(np.repeat(nodes, ndf) == f)[0]] = -1
        g = rng.normal(size=(len(ids), len(ids)))
        elems.append((g @ g.T + len(ids) * np.eye(len(ids)), ids))
    # every node connected to itself so the matrix is nonsingular
    for i in range(nnode):
        k = np.eye(ndf) * 5.0
        elems.append((k, eq[i].copy()))
    K = np.zeros((n, n))
    pattern = np.eye(n, dtype=bool)          # the element graph (setSize)
    for k, ids in elems:
        v = ids >= 0
        K[np.ix_(ids[v], ids[v])] += k[np.ix_(v, v)]
        pattern[np.ix_(ids[v], ids[v])] = True
    rowptr = np.concatenate([[0], np.cumsum(pattern.sum(1))]).astype(np.int32)
    colidx = np.concatenate([np.nonzero(r)[0] for r in pattern]).astype(np.int32)
    blk = np.arange(0, n + 1, ndf, dtype=np.int32)
    return n, elems, K, rowptr, colidx, blk


def test_assembly_matches_dense():
    n, elems, K, rp, ci, blk = _problem()
    with gpu.LinearSystem(rp, ci, blk) as s:
        for k, ids in elems:
            s.add_a(k, ids)
        rows = np.repeat(np.arange(n), np.diff(rp))
        np.testing.assert_allclose(s.values(), K[rows, ci], rtol=1e-14, atol=1e-12)
        s.add_a(elems[0][0], elems[0][1], fact=-1.0)          # fact scales
        k0, id0 = elems[0]
        v = id0 >= 0
        K2 = K.copy()
        K2[np.ix_(id0[v], id0[v])] -= k0[np.ix_(v, v)]
        np.testing.assert_allclose(s.values(), K2[rows, ci], rtol=1e-13, atol=1e-12)
        s.zero_a()
        assert not s.values().any()
        b = np.arange(n, dtype=float)
        s.set_b(b, 2.0)
        s.add_b(np.ones(3), [0, -1, 5], fact=0.5)
        expect = 2.0 * b
        expect[[0, 5]] += 0.5
        np.testing.assert_array_equal(s.rhs(), expect)
        s.set_b(np.ones(n), 0.0)             # the quick return: B unchanged
        np.testing.assert_array_equal(s.rhs(), expect)
        s.add_b(np.ones(3), [0, 1, 2], fact=0.0)
        np.testing.assert_array_equal(s.rhs(), expect)
        s.zero_b()
        assert not s.rhs().any()


def test_repeated_equation_sums_in_reference_order():
    """An ID that names one equation twice (two nodes of an element tied to
    one master by equalDOF: the PlainHandler's numbering copies the master's
    equation numbers to them) gives that entry several terms in one addA.
    SparseGenColLinSOE::addA (SparseGenColLinSOE.cpp:262-310) walks columns
    outside, rows inside; the sum is bit-identical only in that order."""
    rp = np.array([0, 2, 4], np.int32)
    ci = np.array([0, 1, 0, 1], np.int32)
    ids = np.array([0, 1, 0], np.int32)                # equation 0 twice
    e = 2.0 ** -53
    m = np.array([[1.0, 3.0, -1.0],
                  [5.0, 7.0, 11.0],
                  [e, 13.0, 0.0]])                     # (1 + e) - 1 = 0, (1 - 1) + e = e
    expect = {}
    for i in range(3):                                 # the reference's loop: column i
        for j in range(3):                             # row j
            key = (int(ids[j]), int(ids[i]))
            expect[key] = expect.get(key, 0.0) + m[j, i]
    with gpu.LinearSystem(rp, ci) as s:
        s.add_a(m, ids)
        got = s.values()
    want = np.array([expect[(0, 0)], expect[(0, 1)], expect[(1, 0)], expect[(1, 1)]])
    np.testing.assert_array_equal(got, want)
    # the row-outer order would give another (0,0) entry: the case matters
    row_outer = 0.0
    for i in range(3):
        for j in range(3):
            if ids[i] == 0 and ids[j] == 0:
                row_outer += m[i, j]
    assert row_outer != want[0]


def test_argument_checks():
    n, elems, K, rp, ci, blk = _problem()
    with pytest.raises(gpu.XaraGpuError, match="sorted"):
        bad = ci.copy()
        bad[[0, 1]] = bad[[1, 0]]
        gpu.LinearSystem(rp, bad)
    with pytest.raises(gpu.XaraGpuError, match="blocks"):
        gpu.LinearSystem(rp, ci, np.array([0, 7, n], np.int32))


def test_terms_outside_the_system_are_skipped():
    """SparseGenColLinSOE::addA / addB (SparseGenColLinSOE.cpp:263-350) skip
    an equation number outside 0..n-1 and an entry missing from the pattern
    and add every other term."""
    n, elems, K, rp, ci, blk = _problem()
    j = int(np.setdiff1d(np.arange(n), ci[rp[0]:rp[1]])[0])      # not coupled to 0
    m = np.array([[1.0, 2.0, 3.0], [4.0, 5.0, 6.0], [7.0, 8.0, 9.0]])
    with gpu.LinearSystem(rp, ci) as s:
        s.add_a(m, [0, j, n + 3])
        s.add_b(np.array([1.0, 2.0, 3.0]), [0, j, n])
        vals, b = s.values(), s.rhs()
    want = np.zeros(len(ci))
    want[rp[0] + np.searchsorted(ci[rp[0]:rp[1]], 0)] = 1.0
    want[rp[j] + np.searchsorted(ci[rp[j]:rp[j + 1]], j)] = 5.0
    assert np.array_equal(vals, want)
    wb = np.zeros(n)
    wb[0], wb[j] = 1.0, 2.0
    assert np.array_equal(b, wb)


@pytest.mark.gpu
@pytest.mark.parametrize("blocks", [True, False])
def test_pcg_solve_matches_dense(need_gpu, blocks):
    n, elems, K, rp, ci, blk = _problem(seed=3)
    b = np.random.default_rng(4).normal(size=n)
    with gpu.LinearSystem(rp, ci, blk if blocks else None) as s:
        for k, ids in elems:
            s.add_a(k, ids)
        s.set_b(b)
        x, it, rr = s.solve(rtol=1e-13)
        assert rr <= 1e-13 and it > 0
        np.testing.assert_allclose(x, np.linalg.solve(K, b), rtol=1e-9, atol=1e-12)
        # new values through the same pattern: a second solve uses them
        s.zero_a()
        for k, ids in elems:
            s.add_a(k, ids, fact=2.0)
        x2, _, _ = s.solve(rtol=1e-13)
        np.testing.assert_allclose(x2, 0.5 * np.linalg.solve(K, b), rtol=1e-9, atol=1e-12)


@pytest.mark.gpu
def test_profile_ldl_solve_matches_dense(need_gpu):
    """`system ProfileSPD` on the device: ProfileSPDLinSOE's assembly (the
    row <= col terms) and the device LDL' against a dense solve; a second
    right-hand side reuses the factors, new values refactor."""
    n, elems, K, rp, ci, blk = _problem(seed=5)
    rng = np.random.default_rng(6)
    b1, b2 = rng.normal(size=n), rng.normal(size=n)
    with gpu.LinearSystem(rp, ci, system=gpu.XG_SYSTEM_PROFILE_SPD) as s:
        for k, ids in elems:
            s.add_a(k, ids)
        vals = s.values()
        rows = np.repeat(np.arange(n), np.diff(rp))
        assert not vals[ci > rows].any()                   # only the lower triangle
        s.set_b(b1)
        x1, it, rr = s.solve()
        assert it == 0 and rr == 0.0
        np.testing.assert_allclose(x1, np.linalg.solve(K, b1), rtol=1e-10, atol=1e-13)
        s.set_b(b2)
        x2, _, _ = s.solve()
        np.testing.assert_allclose(x2, np.linalg.solve(K, b2), rtol=1e-10, atol=1e-13)
        s.zero_a()
        for k, ids in elems:
            s.add_a(k, ids, fact=4.0)
        x3, _, _ = s.solve()
        np.testing.assert_allclose(x3, 0.25 * np.linalg.solve(K, b2), rtol=1e-10, atol=1e-13)


@pytest.mark.gpu
def test_profile_ldl_pivot_checks(need_gpu):
    """ProfileSPDLinDirectSolver's checks: a first pivot <= 0 fails the
    solve (XG_ESOLVE naming the equation); a later negative pivot does not."""
    n, elems, K, rp, ci, blk = _problem(seed=7)
    with gpu.LinearSystem(rp, ci, system=gpu.XG_SYSTEM_PROFILE_SPD) as s:
        for k, ids in elems:
            s.add_a(k, ids)
        s.add_a(np.array([[-2.0 * K[0, 0]]]), [0])           # a negative first pivot
        s.set_b(np.ones(n))
        with pytest.raises(gpu.XaraGpuError, match="pivot 0"):
            s.solve()
    with gpu.LinearSystem(rp, ci, system=gpu.XG_SYSTEM_PROFILE_SPD) as s:
        Kn = K.copy()
        for k, ids in elems:
            s.add_a(k, ids)
        last = n - 1
        s.add_a(np.array([[-3.0 * K[last, last]]]), [last])   # indefinite, last pivot < 0
        Kn[last, last] -= 3.0 * K[last, last]
        b = np.random.default_rng(8).normal(size=n)
        s.set_b(b)
        x, _, _ = s.solve()
        np.testing.assert_allclose(x, np.linalg.solve(Kn, b), rtol=1e-9, atol=1e-12)
