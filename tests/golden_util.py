"""Helpers shared by the tests: load a golden fixture and rebuild its model."""
import os

import numpy as np

from xara_gb300 import configs

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# tolerance for floating-point parity (relative, norm-wise per vector; the
# tangent's values also row by row, row_relerr)
RTOL_STATE = 1e-12      # resisting force / tangent values per iteration
RTOL_HISTORY = 1e-8     # converged displacement histories


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False)
    return {k: z[k] for k in z.files}


def model_of(fx):
    builder = getattr(configs, str(fx["builder"]))
    args = tuple(int(a) for a in fx["args"])
    def value(v):
        try:
            f = float(v)
        except ValueError:
            return str(v)
        return int(f) if f.is_integer() else f
    kw = {str(k): value(v) for k, v in zip(fx["kw_keys"], fx["kw_vals"])}
    return builder(*args, **kw)


def relerr(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    den = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (den if den > 0 else 1.0)


def row_relerr(fx, a, b):
    """Largest difference of CSR values a and b in each row over that row's
    largest |b| (the rows of the fixture's pattern; it is symmetric, so the
    column starts are the row pointers): every coefficient is held to the
    scale of its own row, not to the norm of the whole matrix."""
    rp = np.asarray(fx["colstart"])
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    n = len(rp) - 1
    rows = np.repeat(np.arange(n), np.diff(rp))
    dmax = np.zeros(n)
    smax = np.zeros(n)
    np.maximum.at(dmax, rows, np.abs(a - b))
    np.maximum.at(smax, rows, np.abs(b))
    return float((dmax / np.where(smax > 0, smax, 1.0)).max())


def unbalance_solves(fx, desc, phase):
    """Indices of the captured solves whose right-hand side is the unbalance.

    DisplacementControl solves phat once in newStep, then per iteration the
    unbalance and phat (DisplacementControl.cpp:121-250): ordinal 0 and the
    even ordinals are phat solves.
    """
    it = fx["cap_iter"]
    if phase.integrator == 1:
        return np.nonzero(it % 2 == 1)[0]
    return np.arange(len(it))


def external_load(fx, desc, k, eqn, pattern=0):
    """F_ext of captured solve k (a solve of the first phase): lambda times the
    reference loads of that phase's pattern (later patterns are not yet in
    the domain)."""
    neq = len(fx["colstart"]) - 1
    f = np.zeros(neq)
    lam = fx["cap_lambda"][k]
    if desc.load_node is None:
        return f
    for i, n in enumerate(desc.load_node):
        if desc.load_pattern[i] != pattern:
            continue
        idx = np.searchsorted(desc.node_tag, n)
        for j in range(desc.ndf):
            r = eqn[idx * desc.ndf + j]
            if r >= 0:
                f[r] += lam * desc.load_value[i * desc.ndf + j]
    return f


def csc_to_csr_values(fx, vals_csc):
    """The pattern is symmetric, so CSC (column-major) of the reference and
    CSR of this library share index arrays; the values of entry (r, c) sit at
    the same position as those of (c, r).  Map CSC values to CSR order."""
    cs, ri = fx["colstart"], fx["rowidx"]
    n = len(cs) - 1
    cols = np.repeat(np.arange(n), np.diff(cs)).astype(np.int64)
    # CSC position p holds A[ri[p], cols[p]]; keys (col, row) ascend with p.
    key_csc = cols * n + ri
    # CSR position k (same index arrays) holds A[cols[k], ri[k]], which sits
    # at the CSC position whose (col, row) key is (ri[k], cols[k]).
    p = np.searchsorted(key_csc, ri.astype(np.int64) * n + cols)
    return vals_csc[p]


def assemble_elements(desc, eqn, rowptr, colidx, K, P):
    """Assemble per-element global tangents K[ne, ned, ned] and resisting
    forces P[ne, ned] (element order of the description) into CSR values in
    the order of (rowptr, colidx) and the resisting force per equation."""
    ne, ned = P.shape
    nen = ned // desc.ndf
    conn = np.asarray(desc.elem_conn).reshape(ne, nen)
    idx = np.searchsorted(np.asarray(desc.node_tag), conn)
    ids = (idx[:, :, None] * desc.ndf + np.arange(desc.ndf)).reshape(ne, ned)
    ids = np.asarray(eqn)[ids]
    vals = np.zeros(len(colidx))
    resid = np.zeros(len(rowptr) - 1)
    for e in range(ne):
        for a in range(ned):
            r = ids[e, a]
            if r < 0:
                continue
            resid[r] += P[e, a]
            row = colidx[rowptr[r]:rowptr[r + 1]]
            for b in range(ned):
                c = ids[e, b]
                if c >= 0:
                    vals[rowptr[r] + np.searchsorted(row, c)] += K[e, a, b]
    return vals, resid
