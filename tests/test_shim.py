"""The `system` shims (include/CudaBJPCGLinSOE.h: SparseGenColLinSOE's
assembly; include/CudaProfileSPDLinSOE.h: ProfileSPDLinSOE's) inside the
reference's own analysis loop.

The shim is compiled against the reference's headers and handed to the
reference harness (oracle/_ref) as a second LinearSOE: the reference's
AnalysisModel graph sizes it, and its integrators and FE_Elements feed it the
same zeroA / zeroB / addA / addB / setB calls they feed the reference's
SparseGenColLinSOE and ProfileSPDLinSOE.  Before every solve the shim's
pattern, assembled values and right-hand side must equal the reference's bit
for bit (the ProfileSPD shim's against ProfileSPDLinSOE's own profile
storage).  Host work only
(the device solve is covered by tests/test_linsoe.py); skipped where the
reference sources or the compiled harness are absent.
"""
import ctypes as C
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import build_ref  # noqa: E402
import ref  # noqa: E402
from xara_gb300 import configs, gpu  # noqa: E402

sp = pytest.importorskip("scipy.sparse")

CAP = 40


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    if not (ref.available() and os.path.isdir(build_ref.DEFAULT_SRC)):
        pytest.skip("reference sources or oracle/_ref/libxara_ref.so absent")
    if not os.path.exists(gpu.LIB):
        pytest.skip("libxara_gpu.so not built")
    out = str(tmp_path_factory.mktemp("shim") / "libshim_driver.so")
    refdir = os.path.dirname(ref.LIB)
    gpudir = os.path.dirname(gpu.LIB)
    cmd = (["g++", "-std=c++17", "-fconcepts", "-O1", "-fPIC", "-shared", "-w",
            "-I" + os.path.join(ROOT, "include")]
           + build_ref.include_flags(build_ref.DEFAULT_SRC)
           + [os.path.join(ROOT, "tests", "shim", "shim_driver.cpp"), "-o", out,
              ref.LIB, gpu.LIB, "-Wl,-rpath," + refdir, "-Wl,-rpath," + gpudir])
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    ref.lib()                                  # the harness instance the driver links
    D = C.CDLL(out)
    D.shim_attach.restype = C.c_void_p
    D.shim_attach.argtypes = [C.c_void_p, C.c_int, C.c_int]
    D.shim_free.argtypes = [C.c_void_p]
    D.shim_sizes.argtypes = [C.c_void_p] + [C.c_void_p] * 4
    D.shim_pattern.argtypes = [C.c_void_p] + [C.c_void_p] * 3
    D.shim_captured.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    return D


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def run_with_shim(D, desc, phases, system=gpu.XG_SYSTEM_BJPCG):
    rec = {}

    def attach(h):
        rec["r"] = D.shim_attach(h, CAP, system)
        assert rec["r"]
        if system == gpu.XG_SYSTEM_PROFILE_SPD:
            ref.lib().xref_capture_profile(C.c_void_p(h), 1)

    run = ref.RefRun(desc, phases, capture=(0, 1 << 20), cap_solves=CAP, attach=attach)
    r = rec["r"]
    neq, nnz, nblk, count = C.c_int(), C.c_int(), C.c_int(), C.c_int()
    D.shim_sizes(r, C.byref(neq), C.byref(nnz), C.byref(nblk), C.byref(count))
    rp = np.zeros(neq.value + 1, np.int32)
    ci = np.zeros(nnz.value, np.int32)
    blk = np.zeros(max(nblk.value + 1, 1), np.int32)
    D.shim_pattern(r, _p(rp), _p(ci), _p(blk))
    A = np.zeros((count.value, nnz.value))
    B = np.zeros((count.value, neq.value))
    D.shim_captured(r, _p(A), _p(B))
    errors = ref.lib().xref_observer_errors(C.c_void_p(run.h))
    D.shim_free(r)
    return run, rp, ci, blk[:nblk.value + 1] if nblk.value else blk[:0], A, B, errors


# (builder, every block a whole node's): the continuum blocks tie their
# loaded edge / face to a master node with equalDOF, so the tied equations
# belong to several DOF groups; those groups' equations get blocks of one
# equation and every other node keeps its node block
MODELS = {
    "quad J2, DisplacementControl": (lambda: configs.quad_block(8, 4, steps=4), False),
    "brick J2, DisplacementControl": (lambda: configs.brick_block(4, 3, 2, steps=3), False),
    "2D steel frame, gravity and pushover": (lambda: configs.steel_frame_2d(2, 3), True),
    "3D RC frame, gravity and pushover": (lambda: configs.rc_frame_3d(1, 1, 2), True),
    "2D steel frame, Newmark with Rayleigh damping":
        (lambda: configs.steel_frame_2d_eq(1, 2, steps=6), True),
    "2D RC frame of Concrete01 and Steel01, gravity and pushover":
        (lambda: configs.rc_frame_2d(2, 3, steps=6), True),
}


def expected_blocks(eqn, n):
    """Block starts the shim should give: a node's free equations form one
    block when they are contiguous, at most six, and no other node shares
    them; all other equations are blocks of one."""
    claims = np.bincount(eqn[eqn >= 0], minlength=n)
    starts = set(range(n))
    for e in eqn:
        f = np.sort(e[e >= 0])
        if f.size and f.size <= 6 and f[-1] - f[0] + 1 == f.size and (claims[f] == 1).all():
            starts -= set(int(x) for x in f[1:])
    return np.array(sorted(starts) + [n], np.int32)


@pytest.mark.parametrize("name", list(MODELS))
def test_shim_assembles_what_the_reference_assembles(driver, name):
    build, whole_nodes = MODELS[name]
    desc, phases = build()
    run, rp, ci, blk, A, B, errors = run_with_shim(driver, desc, phases)
    assert errors == 0
    # pattern: CSR of the symmetric pattern == the reference's CSC
    assert np.array_equal(rp, run.colstart) and np.array_equal(ci, run.rowidx)
    # the same solves were seen, with identical values
    ns = run.cap_A.shape[0]
    assert ns > 0 and A.shape[0] == ns
    n = run.neq
    for k in range(ns):
        ref_csr = sp.csc_matrix((run.cap_A[k], run.rowidx, run.colstart), shape=(n, n)).tocsr()
        ref_csr.sort_indices()
        assert np.array_equal(ref_csr.indptr, rp) and np.array_equal(ref_csr.indices, ci)
        assert np.array_equal(A[k], ref_csr.data), (name, k)
        assert np.array_equal(B[k], run.cap_B[k]), (name, k)
    # preconditioner blocks: node blocks, single equations where nodes share one
    eqn = run.eqn.reshape(desc.num_nodes, desc.ndf)
    assert np.array_equal(blk, expected_blocks(eqn, n))
    sizes = np.diff(blk)
    assert sizes.min() >= 1 and sizes.max() <= desc.ndf
    free = [np.sort(e[e >= 0]) for e in eqn if (e >= 0).any()]
    if whole_nodes:
        assert sorted(int(f[0]) for f in free) == list(blk[:-1])
    else:
        # only the tied edge / face and its master fall back to single equations
        singles = int((sizes == 1).sum())
        tied = int(np.sum(np.bincount(run.eqn[run.eqn >= 0]) > 1))
        assert tied >= 1 and (sizes == desc.ndf).sum() >= len(free) // 2, (singles, tied)


@pytest.mark.parametrize("name", list(MODELS))
def test_profile_shim_assembles_what_profilespd_assembles(driver, name):
    """`system ProfileSPD` on the device (include/CudaProfileSPDLinSOE.h): at
    every solve the values its LDL' reads (the lower triangle, holding the
    terms ProfileSPDLinSOE::addA keeps, row <= col) equal ProfileSPDLinSOE's
    own profile storage bit for bit, profile entries outside the pattern
    included (zero in both), and the right-hand side equals the reference's."""
    L = ref.lib()
    L.xref_profile_layout.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    L.xref_captured_profile.argtypes = [C.c_void_p, C.c_void_p]
    L.xref_capture_profile.argtypes = [C.c_void_p, C.c_int]
    desc, phases = MODELS[name][0]()
    run, rp, ci, blk, A, B, errors = run_with_shim(driver, desc, phases,
                                                   gpu.XG_SYSTEM_PROFILE_SPD)
    assert errors == 0
    n = run.neq
    diag = np.zeros(n, np.int32)
    psize = C.c_int()
    assert L.xref_profile_layout(C.c_void_p(run.h), _p(diag), C.byref(psize)) == 0
    ns = A.shape[0]
    P = np.zeros(ns * psize.value)
    assert L.xref_captured_profile(C.c_void_p(run.h), _p(P)) == ns * psize.value
    P = P.reshape(ns, psize.value)
    rows = np.repeat(np.arange(n), np.diff(rp))
    lower = ci <= rows
    # CSR (c, r), r <= c, sits at profile position iDiagLoc[c] - 1 - (c - r)
    pos = diag[rows[lower]] - 1 - (rows[lower] - ci[lower])
    for k in range(ns):
        mine = np.zeros(psize.value)
        mine[pos] = A[k][lower]
        assert np.array_equal(mine, P[k]), (name, k)
        assert np.array_equal(A[k][~lower], np.zeros((~lower).sum())), (name, k)
        assert np.array_equal(B[k], run.cap_B[k]), (name, k)
