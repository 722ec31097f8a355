"""ctypes binding of ``oracle/_ref/libxara_ref.so`` (test infrastructure).

The library holds the reference's own CPU classes compiled from its sources
(``build_ref.py``) plus the harness in ``ref_harness.cpp``.  It exists only
in the container that has the reference sources; GPU tests use the fixtures
generated from it (``tests/golden/make_golden.py``) and the C restatement in
``xara_oracle.c``.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_ref", "libxara_ref.so")

_lib = None


def available():
    return os.path.exists(LIB)


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(LIB)
        _lib.xref_create.restype = C.c_void_p
        _lib.xref_create.argtypes = [C.c_void_p]
        _lib.xref_destroy.argtypes = [C.c_void_p]
        _lib.xref_run_phase.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int,
                                        C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.xref_numbering.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.xref_pattern.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.xref_num_captured.argtypes = [C.c_void_p]
        _lib.xref_captured.argtypes = [C.c_void_p] + [C.c_void_p] * 6
        _lib.xref_times.argtypes = [C.c_void_p] + [C.c_void_p] * 3
        _lib.xref_j2_path.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                                      C.c_void_p, C.c_void_p]
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class RefRun:
    """Run a model through the reference's analysis loop and keep the record."""

    def __init__(self, desc, phases, capture=(0, 0), cap_solves=0, attach=None):
        """attach(handle), when given, runs after the Domain is built and
        before the first phase (e.g. to hand the harness a second LinearSOE)."""
        L = lib()
        self.desc = desc
        self._s = desc.struct()
        self.h = L.xref_create(C.byref(self._s))
        if not self.h:
            raise RuntimeError("xref_create failed")
        if attach is not None:
            attach(self.h)
        nu = desc.num_nodes * desc.ndf
        self.step_u, self.step_lambda, self.step_iters = [], [], []
        for ph in phases:
            n = ph.num_steps
            su = np.zeros((n, nu))
            sl = np.zeros(n)
            si = np.zeros(n, np.int32)
            ps = ph.struct()
            r = L.xref_run_phase(self.h, C.byref(ps), capture[0], capture[1], cap_solves,
                                 _p(su), _p(sl), _p(si))
            if r != 0:
                raise RuntimeError(f"reference analysis failed: {r}")
            self.step_u.append(su)
            self.step_lambda.append(sl)
            self.step_iters.append(si)
        self.step_u = np.concatenate(self.step_u)
        self.step_lambda = np.concatenate(self.step_lambda)
        self.step_iters = np.concatenate(self.step_iters)
        eqn = np.zeros(nu, np.int32)
        neq, nnz = C.c_int(), C.c_int()
        L.xref_numbering(self.h, _p(eqn), C.byref(neq), C.byref(nnz))
        self.eqn, self.neq, self.nnz = eqn, neq.value, nnz.value
        self.colstart = np.zeros(self.neq + 1, np.int32)
        self.rowidx = np.zeros(self.nnz, np.int32)
        L.xref_pattern(self.h, _p(self.colstart), _p(self.rowidx))
        ns = L.xref_num_captured(self.h)
        self.cap_step = np.zeros(ns, np.int32)
        self.cap_iter = np.zeros(ns, np.int32)
        self.cap_B = np.zeros((ns, self.neq))
        self.cap_A = np.zeros((ns, self.nnz))
        self.cap_X = np.zeros((ns, self.neq))
        self.cap_U = np.zeros((ns, nu))
        L.xref_captured(self.h, _p(self.cap_step), _p(self.cap_iter), _p(self.cap_B),
                        _p(self.cap_A), _p(self.cap_X), _p(self.cap_U))
        self.cap_lambda = np.zeros(ns)
        L.xref_captured_lambda.argtypes = [C.c_void_p, C.c_void_p]
        L.xref_captured_lambda(self.h, _p(self.cap_lambda))
        e, s, t = C.c_double(), C.c_double(), C.c_double()
        L.xref_times(self.h, C.byref(e), C.byref(s), C.byref(t))
        self.elem_seconds, self.solve_seconds, self.step_seconds = e.value, s.value, t.value

    def elem_response(self, U, revert_first=False):
        """Per-element global tangent [ne, ned, ned] and resisting force
        [ne, ned] at trial displacements U (after Domain::revertToLastCommit
        when revert_first)."""
        L = lib()
        L.xref_elem_response.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
        d = self.desc
        ned = (2 if d.elem_type in (3, 4) else 4 if d.elem_type == 1 else 8) * d.ndf
        K = np.zeros((d.num_elems, ned, ned))
        P = np.zeros((d.num_elems, ned))
        U = np.ascontiguousarray(U, np.float64)
        r = L.xref_elem_response(self.h, _p(U), int(revert_first), _p(K), _p(P))
        if r != 0:
            raise RuntimeError(f"reference element response failed: {r}")
        return K, P


def j2_path(dim, param, strain, commit):
    """Stress and tangent of J2PlaneStrain (dim=2) / J2ThreeDimensional (dim=3)."""
    L = lib()
    ns = 3 if dim == 2 else 6
    strain = np.ascontiguousarray(strain, np.float64).reshape(-1, ns)
    npts = strain.shape[0]
    commit = np.ascontiguousarray(commit, np.int32)
    param = np.ascontiguousarray(param, np.float64)
    stress = np.zeros((npts, ns))
    tang = np.zeros((npts, ns, ns))
    L.xref_j2_path(dim, _p(param), npts, _p(strain), _p(commit), _p(stress), _p(tang))
    return stress, tang


def uniaxial_path(kind, param, strain, commit):
    """Stress and tangent of the reference's Steel02 / Concrete02 along a path."""
    L = lib()
    L.xref_uniaxial_path.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                                     C.c_void_p, C.c_void_p]
    strain = np.ascontiguousarray(strain, np.float64)
    commit = np.ascontiguousarray(commit, np.int32)
    param = np.ascontiguousarray(param, np.float64)
    s = np.zeros(len(strain))
    t = np.zeros(len(strain))
    L.xref_uniaxial_path(kind, _p(param), len(strain), _p(strain), _p(commit), _p(s), _p(t))
    return s, t


def ddm_gradient(desc, phases, params, obj):
    """The reference's DDM sensitivity (computeGradients at every step) of J
    = sum over steps and terms of w u(node, dof)^2: params is a list of
    (element tag, name) with name 0 fy, 1 E, 2 b (Steel01), 3 fc, 4 epsco,
    5 fcu (Concrete01); obj = (node tags, dofs, weights).  Returns
    (dJ/dparam, J)."""
    L = lib()
    L.xref_ddm_setup.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int,
                                 C.c_void_p, C.c_void_p, C.c_void_p]
    L.xref_ddm_result.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    tags = np.ascontiguousarray([p[0] for p in params], np.int32)
    names = np.ascontiguousarray([p[1] for p in params], np.int32)
    nodes = np.ascontiguousarray(obj[0], np.int32)
    dofs = np.ascontiguousarray(obj[1], np.int32)
    w = np.ascontiguousarray(obj[2], np.float64)

    def attach(h):
        r = L.xref_ddm_setup(C.c_void_p(h), len(tags), _p(tags), _p(names), len(nodes),
                             _p(nodes), _p(dofs), _p(w))
        if r != 0:
            raise RuntimeError(f"xref_ddm_setup failed: {r}")

    run = RefRun(desc, phases, attach=attach)
    grad = np.zeros(len(tags))
    J = C.c_double()
    L.xref_ddm_result(C.c_void_p(run.h), _p(grad), C.byref(J))
    return grad, J.value, run
