"""ctypes binding of ``libxara_gpu.so`` and the device model handle.

The library is built in-tree by :func:`xara_gb300._build.build` (nvcc,
sm_103a).  Nothing here falls back to a CPU path: a missing library or a
failing CUDA call raises.
"""
import ctypes as C
import os
import re

import numpy as np

from . import _abi
from ._abi import XG_SYSTEM_BJPCG, XG_SYSTEM_PROFILE_SPD, xg_step_stats  # noqa: F401
from ._abi import (XG_REC_ACCEL, XG_REC_DISP, XG_REC_ENVELOPE, XG_REC_NODE,  # noqa: F401
                   XG_REC_VEL)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libxara_gpu.so")
HEADER = os.path.join(HERE, "..", "include", "xara_gpu.h")

_lib = None


class XaraGpuError(RuntimeError):
    """A negative status from the C ABI, with xg_last_error()'s text."""

    def __init__(self, code, msg):
        super().__init__(f"xara_gpu error {code}: {msg}")
        self.code = code


def declared_symbols():
    """Names of the entry points declared in include/xara_gpu.h."""
    with open(HEADER) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(xg_[a-z0-9_]+)\s*\(", text)))


def lib():
    """Load libxara_gpu.so (ImportError when it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB):
        raise ImportError(f"{LIB} not built: run __graft_entry__.build()")
    L = C.CDLL(LIB)
    vp, ip, dp = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double)
    L.xg_last_error.restype = C.c_char_p
    L.xg_model_create.argtypes = [vp, C.POINTER(vp)]
    L.xg_model_destroy.argtypes = [vp]
    L.xg_model_sizes.argtypes = [vp, ip, ip]
    L.xg_model_numbering.argtypes = [vp, vp]
    L.xg_model_pattern.argtypes = [vp, vp, vp]
    L.xg_elemset_set_trial_disp.argtypes = [vp, vp]
    L.xg_elemset_update.argtypes = [vp, vp, vp]
    L.xg_elemset_commit.argtypes = [vp]
    L.xg_elemset_revert.argtypes = [vp]
    L.xg_elemset_revert_to_start.argtypes = [vp]
    L.xg_elemset_get_history.argtypes = [vp, C.c_int, vp, C.c_long]
    L.xg_elemset_set_history.argtypes = [vp, C.c_int, vp, C.c_long]
    L.xg_soe_solve.argtypes = [vp, vp, vp, C.c_double, C.c_int, ip, dp]
    L.xg_analysis_set_phase.argtypes = [vp, vp]
    L.xg_analysis_set_solver.argtypes = [vp, C.c_double, C.c_int]
    L.xg_analysis_set_system.argtypes = [vp, C.c_int]
    L.xg_analyze.argtypes = [vp, C.c_int, vp]
    L.xg_get_disp.argtypes = [vp, vp, dp]
    L.xg_reset.argtypes = [vp]
    L.xg_model_plan.argtypes = [vp, vp, vp, vp, ip, ip]
    _lib = L
    return _lib


def plan(desc):
    """Host-only DOF numbering and CSR pattern (no GPU needed).

    Returns (eqn[num_nodes*ndf], rowptr, colidx) as DOF_Numberer and
    SparseGenColLinSOE would produce them.
    """
    L = lib()
    s = desc.struct()
    neq, nnz = C.c_int(), C.c_int()
    _check(L.xg_model_plan(C.byref(s), None, None, None, C.byref(neq), C.byref(nnz)))
    eqn = np.zeros(desc.num_nodes * desc.ndf, np.int32)
    rp = np.zeros(neq.value + 1, np.int32)
    ci = np.zeros(nnz.value, np.int32)
    _check(L.xg_model_plan(C.byref(s), _p(eqn), _p(rp), _p(ci), C.byref(neq), C.byref(nnz)))
    return eqn, rp, ci


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _check(code):
    if code < 0:
        msg = lib().xg_last_error()
        raise XaraGpuError(code, msg.decode() if msg else "")
    return code


class DeviceModel:
    """A model resident on the GPU: element set, system and Newton driver."""

    def __init__(self, desc):
        L = lib()
        self.desc = desc
        self._s = desc.struct()
        h = C.c_void_p()
        _check(L.xg_model_create(C.byref(self._s), C.byref(h)))
        self.h = h
        neq, nnz = C.c_int(), C.c_int()
        _check(L.xg_model_sizes(self.h, C.byref(neq), C.byref(nnz)))
        self.neq, self.nnz = neq.value, nnz.value
        self.nu = desc.num_nodes * desc.ndf

    def close(self):
        if getattr(self, "h", None):
            lib().xg_model_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- DOF numbering and pattern -----------------------------------------
    def numbering(self):
        eqn = np.zeros(self.nu, np.int32)
        _check(lib().xg_model_numbering(self.h, _p(eqn)))
        return eqn

    def pattern(self):
        rp = np.zeros(self.neq + 1, np.int32)
        ci = np.zeros(self.nnz, np.int32)
        _check(lib().xg_model_pattern(self.h, _p(rp), _p(ci)))
        return rp, ci

    # -- element set ---------------------------------------------------------
    def set_trial_disp(self, U):
        U = np.ascontiguousarray(U, np.float64)
        assert U.size == self.nu
        _check(lib().xg_elemset_set_trial_disp(self.h, _p(U)))

    def update(self, want_vals=True, want_resid=True):
        vals = np.zeros(self.nnz) if want_vals else None
        resid = np.zeros(self.neq) if want_resid else None
        r = lib().xg_elemset_update(self.h, _p(vals), _p(resid))
        if r < 0 and lib().xg_last_error():
            _check(r)
        return vals, resid, r

    def element_matrices(self):
        """Every element's tangent [ne, ned, ned] and resisting force [ne,
        ned] from the last update (xg_elemset_element_matrices)."""
        L = lib()
        L.xg_elemset_element_matrices.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        d = self.desc
        ned = (2 if d.elem_type in (_abi.XG_ELE_FBC2D, _abi.XG_ELE_FBC3D) else
               4 if d.elem_type == _abi.XG_ELE_QUAD else 8) * d.ndf
        K = np.zeros((d.num_elems, ned, ned))
        P = np.zeros((d.num_elems, ned))
        _check(L.xg_elemset_element_matrices(self.h, _p(K), _p(P)))
        return K, P

    def commit(self):
        _check(lib().xg_elemset_commit(self.h))

    def revert(self):
        _check(lib().xg_elemset_revert(self.h))

    def history(self):
        n = 1 << 62
        buf = np.zeros(1)
        r = lib().xg_elemset_get_history(self.h, 0, _p(buf), 0)
        # the error text carries the size; ask with the exact size instead
        nip = 4 if self.desc.elem_type == _abi.XG_ELE_QUAD else 8
        nh = 4 if nip == 4 else 6
        n = self.desc.num_elems * nip * (nh + 1)
        buf = np.zeros(n)
        _check(lib().xg_elemset_get_history(self.h, 0, _p(buf), n))
        del r
        return buf

    # -- recorders ------------------------------------------------------------
    def add_recorder(self, nodes, dofs, response=XG_REC_DISP, kind=XG_REC_NODE, time=False,
                     dT=0.0):
        """`recorder Node|EnvelopeNode <-time> <-dT dT> -node nodes -dof dofs
        disp|vel|accel` (dofs 0-based); recorded on the device after every
        committed step of :meth:`analyze`.  Returns the recorder id."""
        L = lib()
        L.xg_recorder_add.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int,
                                      C.c_void_p, C.c_int, C.c_int, C.c_double,
                                      C.POINTER(C.c_int)]
        nodes = np.ascontiguousarray(nodes, np.int32)
        dofs = np.ascontiguousarray(dofs, np.int32)
        rid = C.c_int()
        _check(L.xg_recorder_add(self.h, int(kind), int(response), _p(nodes), len(nodes),
                                 _p(dofs), len(dofs), 1 if time else 0, float(dT),
                                 C.byref(rid)))
        return rid.value

    def recorder(self, rid):
        """The recorder's rows so far ([rows, cols])."""
        L = lib()
        L.xg_recorder_size.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int),
                                       C.POINTER(C.c_int)]
        L.xg_recorder_read.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int]
        rows, cols = C.c_int(), C.c_int()
        _check(L.xg_recorder_size(self.h, int(rid), C.byref(rows), C.byref(cols)))
        out = np.zeros((rows.value, cols.value))
        _check(L.xg_recorder_read(self.h, int(rid), _p(out), rows.value))
        return out

    def write_recorder(self, rid, path, precision=6):
        """Write the rows as the reference's DataFileStream does."""
        L = lib()
        L.xg_recorder_write.argtypes = [C.c_void_p, C.c_int, C.c_char_p, C.c_int]
        _check(L.xg_recorder_write(self.h, int(rid), str(path).encode(), int(precision)))

    def fiber_records(self):
        """Committed fiber records of a frame model, [fibers x sections, 12]."""
        nf = np.diff(np.asarray(self.desc.sec_fiber_start))[np.asarray(self.desc.elem_mat)]
        n = int(nf.sum()) * self.desc.fbc_num_ip * 12
        buf = np.zeros(max(n, 1))
        _check(lib().xg_elemset_get_history(self.h, 1, _p(buf), n))
        return buf[:n].reshape(-1, 12)

    def set_history(self, buf):
        buf = np.ascontiguousarray(buf, np.float64)
        _check(lib().xg_elemset_set_history(self.h, 0, _p(buf), buf.size))

    # -- linear system -------------------------------------------------------
    def solve(self, b, rtol=1e-12, maxit=20000):
        b = np.ascontiguousarray(b, np.float64)
        x = np.zeros(self.neq)
        it, rr = C.c_int(), C.c_double()
        _check(lib().xg_soe_solve(self.h, _p(b), _p(x), rtol, maxit, C.byref(it), C.byref(rr)))
        return x, it.value, rr.value

    # -- analysis ------------------------------------------------------------
    def set_solver(self, rtol=1e-12, maxit=20000):
        """Block-Jacobi PCG settings (used when the system is XG_SYSTEM_BJPCG)."""
        _check(lib().xg_analysis_set_solver(self.h, rtol, maxit))

    def set_system(self, system):
        """XG_SYSTEM_PROFILE_SPD (device LDL', the default) or XG_SYSTEM_BJPCG."""
        _check(lib().xg_analysis_set_system(self.h, int(system)))

    def set_phase(self, phase):
        self._ps = phase.struct()
        _check(lib().xg_analysis_set_phase(self.h, C.byref(self._ps)))

    def analyze(self, num_steps):
        stats = (xg_step_stats * max(num_steps, 1))()
        r = lib().xg_analyze(self.h, num_steps, stats)
        out = [(s.newton_iters, s.solver_iters, s.status) for s in stats[:num_steps]]
        _check(r)
        return out

    def disp(self):
        u = np.zeros(self.nu)
        lam = C.c_double()
        _check(lib().xg_get_disp(self.h, _p(u), C.byref(lam)))
        return u, lam.value

    def response(self, which=XG_REC_DISP):
        """Committed displacements, velocities or accelerations [nu]."""
        out = np.zeros(self.nu)
        _check(lib().xg_get_response(self.h, int(which), _p(out)))
        return out

    def reset(self):
        _check(lib().xg_reset(self.h))

    def run(self, phases, record=True):
        """Run phases step by step; returns (U per step, lambda per step, stats)."""
        us, ls, stats = [], [], []
        for ph in phases:
            self.set_phase(ph)
            for _ in range(ph.num_steps):
                st = self.analyze(1)
                stats.extend(st)
                if record:
                    u, lam = self.disp()
                    us.append(u)
                    ls.append(lam)
        return (np.array(us) if record else None), np.array(ls), stats


def profile_enable(model, on=True):
    _check(lib().xg_profile_enable(model.h, 1 if on else 0))


def autotune(model, element=True, pcg=True):
    """Start the online autotuner (element kernel block shape, PCG grid)."""
    L = lib()
    L.xg_analysis_autotune.argtypes = [C.c_void_p, C.c_int]
    _check(L.xg_analysis_autotune(model.h, (1 if element else 0) | (2 if pcg else 0)))


def autotune_result(model):
    """(elements per block, PCG rows per block, tunings still sampling)."""
    L = lib()
    L.xg_autotune_result.argtypes = [C.c_void_p] + [C.POINTER(C.c_int)] * 3
    a, b, c = C.c_int(), C.c_int(), C.c_int()
    _check(L.xg_autotune_result(model.h, C.byref(a), C.byref(b), C.byref(c)))
    return a.value, b.value, c.value


def pcg_layout(model):
    """(block order, node-pair blocks, rows left to CSR chunks) of the PCG's
    node-block copy of the tangent; block order 0 before the first PCG solve
    or when no copy was built."""
    L = lib()
    L.xg_model_pcg_layout.argtypes = [C.c_void_p, C.POINTER(C.c_int),
                                      C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]
    kb, nb, nc = C.c_int(), C.c_longlong(), C.c_longlong()
    _check(L.xg_model_pcg_layout(model.h, C.byref(kb), C.byref(nb), C.byref(nc)))
    return kb.value, nb.value, nc.value


def model_stream(model):
    """The model's CUDA stream as an integer handle (cudaStream_t)."""
    L = lib()
    L.xg_model_stream.argtypes = [C.c_void_p, C.POINTER(C.c_void_p)]
    p = C.c_void_p()
    _check(L.xg_model_stream(model.h, C.byref(p)))
    return p.value or 0


def profile_counters(model):
    """(point updates, section updates, element updates) since enabling."""
    L = lib()
    L.xg_profile_counters.argtypes = [C.c_void_p] + [C.POINTER(C.c_longlong)] * 3
    a, b, c = C.c_longlong(), C.c_longlong(), C.c_longlong()
    _check(L.xg_profile_counters(model.h, C.byref(a), C.byref(b), C.byref(c)))
    return a.value, b.value, c.value


def profile_read(model):
    """{kernel group: (milliseconds, launches)} accumulated since enabling."""
    L = lib()
    L.xg_profile_get.argtypes = [C.c_void_p, C.c_int, C.c_char_p, C.c_int,
                                 C.POINTER(C.c_double), C.POINTER(C.c_long)]
    out = {}
    k = 0
    buf = C.create_string_buffer(64)
    while True:
        ms, n = C.c_double(), C.c_long()
        if L.xg_profile_get(model.h, k, buf, 64, C.byref(ms), C.byref(n)) < 0:
            break
        out[buf.value.decode()] = (ms.value, n.value)
        k += 1
    return out


def set_uniaxial_params(model, uni_param):
    """Replace the uniaxial parameters ([num_uni, XG_UNI_NPARAM]) and reset
    the model to its initial state."""
    q = np.ascontiguousarray(uni_param, np.float64).reshape(-1, _abi.XG_UNI_NPARAM)
    L = lib()
    L.xg_model_set_uniaxial_params.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
    _check(L.xg_model_set_uniaxial_params(model.h, _p(q), q.shape[0]))


def adjoint_forward(model, phase, num_steps, ckpt_every, node, dof, weight):
    """Newmark run of num_steps from the initial state with checkpoints every
    ckpt_every steps; returns J = sum over steps and terms of
    weight * u(node, dof)^2."""
    L = lib()
    L.xg_adjoint_forward.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                                     C.POINTER(C.c_double)]
    node = np.ascontiguousarray(node, np.int32)
    dof = np.ascontiguousarray(dof, np.int32)
    weight = np.ascontiguousarray(weight, np.float64)
    obj = _abi.xg_objective_desc(len(node), node.ctypes.data_as(C.POINTER(C.c_int)),
                                 dof.ctypes.data_as(C.POINTER(C.c_int)),
                                 weight.ctypes.data_as(C.POINTER(C.c_double)))
    model._ps = phase.struct()
    J = C.c_double()
    _check(L.xg_adjoint_forward(model.h, C.byref(model._ps), int(num_steps), int(ckpt_every),
                                C.byref(obj), C.byref(J)))
    return J.value


def adjoint_objective_terms(model, num_terms):
    """The last adjoint run's objective, term by term."""
    L = lib()
    L.xg_adjoint_objective_terms.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
    Jk = np.zeros(num_terms)
    _check(L.xg_adjoint_objective_terms(model.h, _p(Jk), int(num_terms)))
    return Jk


def adjoint_backward(model, scale=1.0):
    """dJ/d(parameters 0..2) of every uniaxial material, [num_uni, 3]."""
    L = lib()
    L.xg_adjoint_backward.argtypes = [C.c_void_p, C.c_double, C.c_void_p, C.c_int]
    nu = len(model.desc.uni_type)
    g = np.zeros((nu, 3))
    _check(L.xg_adjoint_backward(model.h, float(scale), _p(g), nu))
    return g


def ddm_forward(model, phase, num_steps, dtheta, node, dof, weight):
    """Newmark or LoadControl run of num_steps from the initial state with the
    direct differentiation along the directions ``dtheta`` [num_dir, num_uni,
    3]; returns (J, dJ[num_dir])."""
    L = lib()
    L.xg_ddm_forward.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                                 C.c_void_p, C.POINTER(C.c_double), C.c_void_p]
    nu = len(model.desc.uni_type)
    dth = np.ascontiguousarray(np.asarray(dtheta, np.float64).reshape(-1, nu, 3))
    node = np.ascontiguousarray(node, np.int32)
    dof = np.ascontiguousarray(dof, np.int32)
    weight = np.ascontiguousarray(weight, np.float64)
    obj = _abi.xg_objective_desc(len(node), node.ctypes.data_as(C.POINTER(C.c_int)),
                                 dof.ctypes.data_as(C.POINTER(C.c_int)),
                                 weight.ctypes.data_as(C.POINTER(C.c_double)))
    model._ps = phase.struct()
    J = C.c_double()
    dJ = np.zeros(dth.shape[0])
    _check(L.xg_ddm_forward(model.h, C.byref(model._ps), int(num_steps), dth.shape[0], _p(dth),
                            C.byref(obj), C.byref(J), _p(dJ)))
    return J.value, dJ


def ddm_objective_terms(model, direction, num_terms):
    """The last DDM run's objective tangent along ``direction``, term by term."""
    L = lib()
    L.xg_ddm_objective_terms.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int]
    out = np.zeros(num_terms)
    _check(L.xg_ddm_objective_terms(model.h, int(direction), _p(out), int(num_terms)))
    return out


def ddm_disp_sensitivity(model, direction):
    """The last DDM run's displacement tangent along ``direction`` after its
    last step, [num_nodes, ndf]."""
    L = lib()
    L.xg_ddm_disp_sensitivity.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
    out = np.zeros((model.desc.num_nodes, model.desc.ndf))
    _check(L.xg_ddm_disp_sensitivity(model.h, int(direction), _p(out)))
    return out


def uniaxial_jvp(kind, param, hc, strain, dstrain, dhc, dq):
    """Host Jacobian-vector product of one material point's trial record: the
    tangent of the trial record [12]."""
    L = lib()
    L.xg_uniaxial_jvp.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_double, C.c_double,
                                  C.c_void_p, C.c_void_p, C.c_void_p]
    q = np.ascontiguousarray(param, np.float64)
    hc = np.ascontiguousarray(hc, np.float64)
    dhc = np.ascontiguousarray(dhc, np.float64)
    dq = np.ascontiguousarray(dq, np.float64)
    dht = np.zeros(12)
    _check(L.xg_uniaxial_jvp(int(kind), _p(q), _p(hc), float(strain), float(dstrain), _p(dhc),
                             _p(dq), _p(dht)))
    return dht


def uniaxial_vjp(kind, param, hc, strain, yb):
    """Host vector-Jacobian product of one material point's trial record:
    (adjoint of the committed record [12], of the strain, of parameters 0-2)."""
    L = lib()
    L.xg_uniaxial_vjp.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_double, C.c_void_p,
                                  C.c_void_p, C.POINTER(C.c_double), C.c_void_p]
    q = np.ascontiguousarray(param, np.float64)
    hc = np.ascontiguousarray(hc, np.float64)
    yb = np.ascontiguousarray(yb, np.float64)
    hb, qb, sb = np.zeros(12), np.zeros(3), C.c_double()
    _check(L.xg_uniaxial_vjp(int(kind), _p(q), _p(hc), float(strain), _p(yb), _p(hb),
                             C.byref(sb), _p(qb)))
    return hb, sb.value, qb


class LinearSystem:
    """A standalone device linear system with the reference's LinearSOE
    calls (``xg_linsoe_*``): CSR pattern with sorted columns, host-side
    addA / addB / setB, and on the device either block-Jacobi PCG
    (``system=XG_SYSTEM_BJPCG``, SparseGenColLinSOE's assembly) or the LDL'
    (``system=XG_SYSTEM_PROFILE_SPD``, ProfileSPDLinSOE's assembly)."""

    def __init__(self, rowptr, colidx, blk_start=None, system=None):
        L = lib()
        L.xg_linsoe_create.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                       C.POINTER(C.c_void_p)]
        L.xg_linsoe_destroy.argtypes = [C.c_void_p]
        for name in ("xg_linsoe_zero_a", "xg_linsoe_zero_b"):
            getattr(L, name).argtypes = [C.c_void_p]
        L.xg_linsoe_add_a.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_double]
        L.xg_linsoe_add_b.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_double]
        L.xg_linsoe_set_b.argtypes = [C.c_void_p, C.c_void_p, C.c_double]
        for name in ("xg_linsoe_get_a", "xg_linsoe_get_b", "xg_linsoe_get_x"):
            getattr(L, name).argtypes = [C.c_void_p, C.c_void_p]
        L.xg_linsoe_solve.argtypes = [C.c_void_p, C.c_double, C.c_int, C.POINTER(C.c_int),
                                      C.POINTER(C.c_double)]
        self._rp = np.ascontiguousarray(rowptr, np.int32)
        self._ci = np.ascontiguousarray(colidx, np.int32)
        self.n = len(self._rp) - 1
        blk = None if blk_start is None else np.ascontiguousarray(blk_start, np.int32)
        h = C.c_void_p()
        _check(L.xg_linsoe_create(self.n, _p(self._rp), _p(self._ci),
                                  _p(blk) if blk is not None else None,
                                  0 if blk is None else len(blk) - 1, C.byref(h)))
        self.h = h
        if system is not None:
            L.xg_linsoe_set_system.argtypes = [C.c_void_p, C.c_int]
            _check(L.xg_linsoe_set_system(self.h, int(system)))

    def close(self):
        if self.h:
            lib().xg_linsoe_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def zero_a(self):
        _check(lib().xg_linsoe_zero_a(self.h))

    def zero_b(self):
        _check(lib().xg_linsoe_zero_b(self.h))

    def add_a(self, m, ids, fact=1.0):
        m = np.ascontiguousarray(m, np.float64)
        ids = np.ascontiguousarray(ids, np.int32)
        _check(lib().xg_linsoe_add_a(self.h, _p(m), _p(ids), len(ids), float(fact)))

    def add_b(self, v, ids, fact=1.0):
        v = np.ascontiguousarray(v, np.float64)
        ids = np.ascontiguousarray(ids, np.int32)
        _check(lib().xg_linsoe_add_b(self.h, _p(v), _p(ids), len(ids), float(fact)))

    def set_b(self, v, fact=1.0):
        v = np.ascontiguousarray(v, np.float64)
        _check(lib().xg_linsoe_set_b(self.h, _p(v), float(fact)))

    def values(self):
        out = np.zeros(len(self._ci))
        _check(lib().xg_linsoe_get_a(self.h, _p(out)))
        return out

    def rhs(self):
        out = np.zeros(self.n)
        _check(lib().xg_linsoe_get_b(self.h, _p(out)))
        return out

    def solve(self, rtol=1e-12, maxit=20000):
        it, rr = C.c_int(), C.c_double()
        _check(lib().xg_linsoe_solve(self.h, float(rtol), int(maxit), C.byref(it), C.byref(rr)))
        x = np.zeros(self.n)
        _check(lib().xg_linsoe_get_x(self.h, _p(x)))
        return x, it.value, rr.value


def set_graph(model, enable=True):
    """Run Newmark steps of many-part models as CUDA graphs (see xg_analysis_set_graph)."""
    L = lib()
    L.xg_analysis_set_graph.argtypes = [C.c_void_p, C.c_int]
    _check(L.xg_analysis_set_graph(model.h, 1 if enable else 0))


def graph_steps(model):
    """Steps that ran as CUDA graphs."""
    L = lib()
    L.xg_analysis_graph_steps.argtypes = [C.c_void_p, C.POINTER(C.c_long)]
    n = C.c_long()
    _check(L.xg_analysis_graph_steps(model.h, C.byref(n)))
    return n.value
