"""ctypes binding of the C oracle ``oracle/xara_oracle.c`` (test infrastructure).

The oracle is the CPU restatement of the reference algorithm; it is the
checker for the CUDA path and the timed CPU baseline.  Only tests, the smoke
check and the benchmark's CPU-baseline leg use it.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "xara_oracle.c")
INC = os.path.join(HERE, "xara_oracle_frame.inc")
LIB = os.path.join(HERE, "libxara_oracle.so")

_lib = None


def build(force=False):
    """Compile the oracle with gcc (seconds); used by __graft_entry__.build()."""
    import platform
    machine = {"x86_64": 62, "aarch64": 183}.get(platform.machine(), -1)
    same_arch = False
    if os.path.exists(LIB):
        with open(LIB, "rb") as f:
            head = f.read(20)
        same_arch = head[:4] == b"\x7fELF" and int.from_bytes(head[18:20], "little") == machine
    newest = max(os.path.getmtime(SRC), os.path.getmtime(INC))
    if not force and same_arch and os.path.getmtime(LIB) >= newest:
        return LIB
    tmp = LIB + ".tmp"
    subprocess.run(["gcc", "-O2", "-fPIC", "-shared", "-std=c11", "-ffp-contract=off",
                    "-o", tmp, SRC, "-lm"], check=True)
    os.replace(tmp, LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        vp = C.c_void_p
        L.xo_create.restype = vp
        L.xo_create.argtypes = [vp]
        L.xo_destroy.argtypes = [vp]
        L.xo_sizes.argtypes = [vp, vp, vp]
        L.xo_numbering.argtypes = [vp, vp]
        L.xo_pattern.argtypes = [vp, vp, vp]
        L.xo_elem_state.argtypes = [vp, vp, vp, vp]
        L.xo_commit.argtypes = [vp]
        L.xo_revert.argtypes = [vp]
        L.xo_work.argtypes = [vp, vp, vp]
        L.xo_soe_solve.argtypes = [vp, vp, vp]
        L.xo_run_phase.argtypes = [vp, vp, vp, vp, vp]
        L.xo_times.argtypes = [vp, vp, vp]
        L.xo_history.argtypes = [vp, vp, vp]
        L.xo_set_history.argtypes = [vp, vp, vp]
        L.xo_j2_path.argtypes = [C.c_int, vp, C.c_int, vp, vp, vp, vp]
        L.xo_uniaxial_path.argtypes = [C.c_int, vp, C.c_int, vp, vp, vp, vp]
        L.xo_uniaxial_init.argtypes = [C.c_int, vp, vp]
        L.xo_uniaxial_trial.argtypes = [C.c_int, vp, vp, C.c_double, vp]
        L.xo_keep_element_matrices.argtypes = [vp, vp, vp]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class OracleModel:
    """A model held by the C oracle: numbering, pattern, element state, solve."""

    def __init__(self, desc):
        L = lib()
        self.desc = desc
        self._s = desc.struct()
        self.h = L.xo_create(C.byref(self._s))
        if not self.h:
            raise ValueError("oracle: unsupported model")
        neq, nnz = C.c_int(), C.c_int()
        L.xo_sizes(self.h, C.byref(neq), C.byref(nnz))
        self.neq, self.nnz = neq.value, nnz.value
        self.nu = desc.num_nodes * desc.ndf

    def close(self):
        if self.h:
            lib().xo_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def numbering(self):
        eqn = np.zeros(self.nu, np.int32)
        lib().xo_numbering(self.h, _p(eqn))
        return eqn

    def pattern(self):
        rp = np.zeros(self.neq + 1, np.int32)
        ci = np.zeros(self.nnz, np.int32)
        lib().xo_pattern(self.h, _p(rp), _p(ci))
        return rp, ci

    def elem_state(self, U):
        U = np.ascontiguousarray(U, np.float64)
        vals = np.zeros(self.nnz)
        resid = np.zeros(self.neq)
        lib().xo_elem_state(self.h, _p(U), _p(vals), _p(resid))
        return vals, resid

    def element_matrices(self, U):
        """Every element's tangent [ne, ned, ned] and resisting force [ne,
        ned] at the trial displacements U (the element state of elem_state)."""
        d = self.desc
        ned = (2 if d.elem_type in (3, 4) else 4 if d.elem_type == 1 else 8) * d.ndf
        K = np.zeros((d.num_elems, ned, ned))
        P = np.zeros((d.num_elems, ned))
        lib().xo_keep_element_matrices(self.h, _p(K), _p(P))
        try:
            self.elem_state(U)
        finally:
            lib().xo_keep_element_matrices(self.h, None, None)
        return K, P

    def commit(self):
        lib().xo_commit(self.h)

    def revert(self):
        lib().xo_revert(self.h)

    def work(self):
        """(material-point updates, section updates) so far."""
        a, b = C.c_longlong(), C.c_longlong()
        lib().xo_work(self.h, C.byref(a), C.byref(b))
        return a.value, b.value

    def soe_solve(self, b):
        """ProfileSPD solve with the tangent of the last element update."""
        b = np.ascontiguousarray(b, np.float64)
        x = np.zeros_like(b)
        r = lib().xo_soe_solve(self.h, _p(b), _p(x))
        if r != 0:
            raise RuntimeError(f"skyline solve failed: {r}")
        return x

    def run(self, phases):
        L = lib()
        us, ls, its = [], [], []
        for ph in phases:
            n = ph.num_steps
            su, sl, si = np.zeros((n, self.nu)), np.zeros(n), np.zeros(n, np.int32)
            ps = ph.struct()
            r = L.xo_run_phase(self.h, C.byref(ps), _p(su), _p(sl), _p(si))
            if r != 0:
                raise RuntimeError(f"oracle analysis failed: {r}")
            us.append(su); ls.append(sl); its.append(si)
        return np.concatenate(us), np.concatenate(ls), np.concatenate(its)

    def times(self):
        e, s = C.c_double(), C.c_double()
        lib().xo_times(self.h, C.byref(e), C.byref(s))
        return e.value, s.value

    def history(self, nip):
        nh = self.desc.num_elems * nip
        ep = np.zeros((nh, 9))
        xi = np.zeros(nh)
        lib().xo_history(self.h, _p(ep), _p(xi))
        return ep, xi

    def set_history(self, ep, xi):
        ep = np.ascontiguousarray(ep, np.float64)
        xi = np.ascontiguousarray(xi, np.float64)
        lib().xo_set_history(self.h, _p(ep), _p(xi))


def j2_path(dim, param, strain, commit):
    L = lib()
    ns = 3 if dim == 2 else 6
    strain = np.ascontiguousarray(strain, np.float64).reshape(-1, ns)
    npts = strain.shape[0]
    commit = np.ascontiguousarray(commit, np.int32)
    param = np.ascontiguousarray(param, np.float64)
    stress = np.zeros((npts, ns))
    tang = np.zeros((npts, ns, ns))
    L.xo_j2_path(dim, _p(param), npts, _p(strain), _p(commit), _p(stress), _p(tang))
    return stress, tang


def uniaxial_path(kind, param, strain, commit):
    """Stress and tangent of Steel02 / Concrete02 / elastic along a strain path."""
    L = lib()
    strain = np.ascontiguousarray(strain, np.float64)
    commit = np.ascontiguousarray(commit, np.int32)
    param = np.ascontiguousarray(param, np.float64)
    s = np.zeros(len(strain))
    t = np.zeros(len(strain))
    L.xo_uniaxial_path(kind, _p(param), len(strain), _p(strain), _p(commit), _p(s), _p(t))
    return s, t


def uniaxial_init(kind, param):
    """Committed record (12 doubles) of a fresh material."""
    h = np.zeros(12)
    lib().xo_uniaxial_init(kind, _p(np.ascontiguousarray(param, np.float64)), _p(h))
    return h


def uniaxial_trial(kind, param, hc, eps):
    """Trial record from a committed record and a trial strain."""
    ht = np.zeros(12)
    hc = np.ascontiguousarray(hc, np.float64)
    lib().xo_uniaxial_trial(kind, _p(np.ascontiguousarray(param, np.float64)), _p(hc),
                            float(eps), _p(ht))
    return ht
