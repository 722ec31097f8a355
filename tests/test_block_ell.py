"""The PCG's node-block copy of the matrix (xg_pcg.cu block_ell_layout),
host side: for symmetric node-coupled patterns with diagonal blocks of 1 to
6 equations (ragged: some nodes with fewer free dofs), nodes coupled to
every other node (a multi-point constraint's retained node) and point
Jacobi, the layout's slots, block columns and padded vector reproduce
y = A x, no two CSR entries share a slot, and the chunks cover exactly the
long node rows.  The device SpMV reads the same arrays (tests/test_linsoe.py
and the PCG parity tests run it)."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from xara_gb300 import gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sp = pytest.importorskip("scipy.sparse")


@pytest.fixture(scope="module")
def ell(tmp_path_factory):
    if not os.path.exists(gpu.LIB):
        pytest.skip("libxara_gpu.so not built")
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "include")
    out = str(tmp_path_factory.mktemp("ell") / "libell_driver.so")
    gpudir = os.path.dirname(gpu.LIB)
    cmd = ["g++", "-std=c++17", "-O1", "-fPIC", "-shared", "-w", "-I" + cuda_inc,
           os.path.join(ROOT, "tests", "block_ell", "ell_driver.cpp"), "-o", out, gpu.LIB,
           "-Wl,-rpath," + gpudir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    D = C.CDLL(out)
    D.ell_apply.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                            C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    return D


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def node_pattern(nodes, maxm, long_nodes, seed):
    rng = np.random.default_rng(seed)
    m = 1 + rng.integers(0, maxm, size=nodes)
    blk = np.concatenate([[0], np.cumsum(m)]).astype(np.int32)
    adj = [set() for _ in range(nodes)]
    for i in range(nodes):
        for d in range(-3, 4):
            if 0 <= i + d < nodes:
                adj[i].add(i + d)
                adj[i + d].add(i)
    for _ in range(nodes // 4):
        a, b = rng.integers(0, nodes, size=2)
        adj[a].add(b)
        adj[b].add(a)
    for a in rng.integers(0, nodes, size=long_nodes):
        for b in range(nodes):
            adj[a].add(b)
            adj[b].add(a)
    rows, cols = [], []
    for i in range(nodes):
        for j in adj[i]:
            for r in range(blk[i], blk[i + 1]):
                for c in range(blk[j], blk[j + 1]):
                    rows.append(r)
                    cols.append(c)
    n = int(blk[-1])
    A = sp.csr_matrix((rng.uniform(-1, 1, size=len(rows)), (rows, cols)), shape=(n, n))
    A.sort_indices()
    return A, blk


@pytest.mark.parametrize("nodes,maxm,long_nodes,seed", [
    (1000, 3, 0, 1), (777, 6, 0, 2), (500, 2, 2, 3), (333, 1, 0, 4), (2000, 3, 1, 5)])
def test_layout_reproduces_the_product(ell, nodes, maxm, long_nodes, seed):
    A, blk = node_pattern(nodes, maxm, long_nodes, seed)
    n = A.shape[0]
    x = np.random.default_rng(seed + 10).uniform(-1, 1, size=n)
    y = np.zeros(n)
    kb, chunked, clash = C.c_int(), C.c_int(), C.c_int()
    rp, ci = A.indptr.astype(np.int32), A.indices.astype(np.int32)
    vals = np.ascontiguousarray(A.data)
    assert ell.ell_apply(n, _p(rp), _p(ci), _p(vals), nodes, _p(blk), 96, _p(x), _p(y),
                         C.byref(kb), C.byref(chunked), C.byref(clash)) == 0
    want_kb = {1: 1, 2: 2, 3: 3}.get(int(np.diff(blk).max()), 6)
    assert kb.value == want_kb
    assert clash.value == 0
    # the rows of node rows coupled to more than 96 nodes go to the chunks
    node_of = np.repeat(np.arange(nodes), np.diff(blk))
    coupled = [len(set(node_of[A.indices[A.indptr[blk[i]]:A.indptr[blk[i + 1]]]]))
               for i in range(nodes)]
    assert chunked.value == sum(int(blk[i + 1] - blk[i]) for i in range(nodes) if coupled[i] > 96)
    assert (chunked.value > 0) == (long_nodes > 0)
    np.testing.assert_allclose(y, A @ x, rtol=1e-12, atol=1e-12)
