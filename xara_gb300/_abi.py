"""ctypes mirror of ``include/xara_gpu.h`` (model, phase and step structs).

The structs carry raw pointers into numpy arrays; :class:`ModelDesc` and
:class:`PhaseDesc` keep those arrays alive for as long as the struct lives.
"""
import ctypes as C

import numpy as np

XG_ELE_QUAD, XG_ELE_BRICK, XG_ELE_FBC2D, XG_ELE_FBC3D = 1, 2, 3, 4
XG_UNI_STEEL02, XG_UNI_CONCRETE02, XG_UNI_ELASTIC, XG_UNI_STEEL01, XG_UNI_CONCRETE01 = 1, 2, 3, 4, 5
XG_HANDLER_PLAIN, XG_HANDLER_TRANSFORMATION = 0, 1
XG_INT_LOAD_CONTROL, XG_INT_DISP_CONTROL, XG_INT_NEWMARK = 0, 1, 2
XG_TEST_NORM_DISP_INCR, XG_TEST_NORM_UNBALANCE = 0, 1
XG_SYSTEM_BJPCG, XG_SYSTEM_PROFILE_SPD = 0, 1
XG_REC_NODE, XG_REC_ENVELOPE = 0, 1
XG_REC_DISP, XG_REC_VEL, XG_REC_ACCEL = 0, 1, 2
XG_J2_NPARAM = 8
XG_UNI_NPARAM = 12

NEN = {XG_ELE_QUAD: 4, XG_ELE_BRICK: 8, XG_ELE_FBC2D: 2, XG_ELE_FBC3D: 2}

_pd = C.POINTER(C.c_double)
_pi = C.POINTER(C.c_int)


class xg_model_desc(C.Structure):
    _fields_ = [
        ("ndm", C.c_int), ("ndf", C.c_int),
        ("num_nodes", C.c_int), ("node_tag", _pi), ("node_crd", _pd), ("node_mass", _pd),
        ("elem_type", C.c_int), ("num_elems", C.c_int), ("elem_tag", _pi),
        ("elem_conn", _pi), ("elem_mat", _pi), ("thickness", C.c_double),
        ("elem_vecxz", _pd), ("geom_transf", C.c_int), ("fbc_num_ip", C.c_int),
        ("fbc_max_iters", C.c_int), ("fbc_tol", C.c_double),
        ("num_j2", C.c_int), ("j2_param", _pd),
        ("num_uni", C.c_int), ("uni_type", _pi), ("uni_param", _pd),
        ("num_sec", C.c_int), ("sec_fiber_start", _pi), ("fib_y", _pd), ("fib_z", _pd),
        ("fib_area", _pd), ("fib_mat", _pi), ("sec_GJ", _pd),
        ("num_sp", C.c_int), ("sp_node", _pi), ("sp_dof", _pi), ("sp_pattern", _pi),
        ("sp_value", _pd), ("handler", C.c_int),
        ("num_mp", C.c_int), ("mp_retained", _pi), ("mp_constrained", _pi), ("mp_dof", _pi),
        ("num_loads", C.c_int), ("load_node", _pi), ("load_pattern", _pi), ("load_value", _pd),
    ]


class xg_phase_desc(C.Structure):
    _fields_ = [
        ("integrator", C.c_int), ("pattern", C.c_int), ("num_steps", C.c_int),
        ("d_lambda", C.c_double), ("dc_node", C.c_int), ("dc_dof", C.c_int),
        ("dc_incr", C.c_double), ("dt", C.c_double), ("gamma", C.c_double),
        ("beta", C.c_double), ("alpha_m", C.c_double), ("beta_k", C.c_double),
        ("beta_k_init", C.c_double), ("beta_k_comm", C.c_double),
        ("alpha_m_node", _pd), ("beta_k_init_elem", _pd),
        ("gm_dof", C.c_int), ("gm_npts", C.c_int), ("gm_dt", C.c_double),
        ("gm_accel", _pd), ("gm_count", C.c_int), ("gm_node_record", _pi),
        ("test", C.c_int), ("tol", C.c_double),
        ("max_iter", C.c_int), ("load_const", C.c_int),
    ]


class xg_objective_desc(C.Structure):
    _fields_ = [("num_terms", C.c_int), ("node", _pi), ("dof", _pi), ("weight", _pd)]


class xg_step_stats(C.Structure):
    _fields_ = [("newton_iters", C.c_int), ("solver_iters", C.c_int),
                ("elem_iters", C.c_int), ("status", C.c_int)]


def _ptr(a, kind):
    if a is None:
        return None
    if kind == "d":
        return a.ctypes.data_as(_pd)
    return a.ctypes.data_as(_pi)


class ModelDesc:
    """A model in flat structure-of-arrays form plus its ctypes view.

    Every field is a numpy array (int32 or float64) named like the C struct.
    """

    INT_FIELDS = ("node_tag", "elem_tag", "elem_conn", "elem_mat", "uni_type",
                  "sec_fiber_start", "fib_mat", "sp_node", "sp_dof", "sp_pattern",
                  "load_node", "load_pattern", "mp_retained", "mp_constrained", "mp_dof")
    DBL_FIELDS = ("node_crd", "node_mass", "elem_vecxz", "j2_param", "uni_param",
                  "fib_y", "fib_z", "fib_area", "sec_GJ", "sp_value", "load_value")

    def __init__(self, **kw):
        self.ndm = int(kw.pop("ndm"))
        self.ndf = int(kw.pop("ndf"))
        self.elem_type = int(kw.pop("elem_type"))
        self.thickness = float(kw.pop("thickness", 1.0))
        self.geom_transf = int(kw.pop("geom_transf", 0))
        self.fbc_num_ip = int(kw.pop("fbc_num_ip", 5))
        self.fbc_max_iters = int(kw.pop("fbc_max_iters", 10))
        self.fbc_tol = float(kw.pop("fbc_tol", 1e-12))
        self.handler = int(kw.pop("handler", XG_HANDLER_PLAIN))
        self.arrays = {}
        for f in self.INT_FIELDS:
            v = kw.pop(f, None)
            self.arrays[f] = None if v is None else np.ascontiguousarray(v, dtype=np.int32).ravel()
        for f in self.DBL_FIELDS:
            v = kw.pop(f, None)
            self.arrays[f] = None if v is None else np.ascontiguousarray(v, dtype=np.float64).ravel()
        if kw:
            raise TypeError(f"unknown model fields: {sorted(kw)}")
        self.meta = {}
        self._struct = None

    def __getattr__(self, name):
        arrays = self.__dict__.get("arrays")
        if arrays is not None and name in arrays:
            return arrays[name]
        raise AttributeError(name)

    @property
    def num_nodes(self):
        return len(self.arrays["node_tag"])

    @property
    def num_elems(self):
        return len(self.arrays["elem_tag"])

    @property
    def nen(self):
        return NEN[self.elem_type]

    def struct(self):
        a = self.arrays
        s = xg_model_desc()
        s.ndm, s.ndf = self.ndm, self.ndf
        s.num_nodes = self.num_nodes
        s.node_tag, s.node_crd = _ptr(a["node_tag"], "i"), _ptr(a["node_crd"], "d")
        s.node_mass = _ptr(a["node_mass"], "d")
        s.elem_type, s.num_elems = self.elem_type, self.num_elems
        s.elem_tag, s.elem_conn = _ptr(a["elem_tag"], "i"), _ptr(a["elem_conn"], "i")
        s.elem_mat = _ptr(a["elem_mat"], "i")
        s.thickness = self.thickness
        s.elem_vecxz = _ptr(a["elem_vecxz"], "d")
        s.geom_transf, s.fbc_num_ip = self.geom_transf, self.fbc_num_ip
        s.fbc_max_iters, s.fbc_tol = self.fbc_max_iters, self.fbc_tol
        s.num_j2 = 0 if a["j2_param"] is None else len(a["j2_param"]) // XG_J2_NPARAM
        s.j2_param = _ptr(a["j2_param"], "d")
        s.num_uni = 0 if a["uni_type"] is None else len(a["uni_type"])
        s.uni_type, s.uni_param = _ptr(a["uni_type"], "i"), _ptr(a["uni_param"], "d")
        s.num_sec = 0 if a["sec_fiber_start"] is None else len(a["sec_fiber_start"]) - 1
        s.sec_fiber_start = _ptr(a["sec_fiber_start"], "i")
        s.fib_y, s.fib_z = _ptr(a["fib_y"], "d"), _ptr(a["fib_z"], "d")
        s.fib_area, s.fib_mat = _ptr(a["fib_area"], "d"), _ptr(a["fib_mat"], "i")
        s.sec_GJ = _ptr(a["sec_GJ"], "d")
        s.num_sp = 0 if a["sp_node"] is None else len(a["sp_node"])
        s.sp_node, s.sp_dof = _ptr(a["sp_node"], "i"), _ptr(a["sp_dof"], "i")
        s.sp_pattern, s.sp_value = _ptr(a["sp_pattern"], "i"), _ptr(a["sp_value"], "d")
        s.handler = self.handler
        s.num_mp = 0 if a["mp_retained"] is None else len(a["mp_retained"])
        s.mp_retained, s.mp_constrained = _ptr(a["mp_retained"], "i"), _ptr(a["mp_constrained"], "i")
        s.mp_dof = _ptr(a["mp_dof"], "i")
        s.num_loads = 0 if a["load_node"] is None else len(a["load_node"])
        s.load_node, s.load_pattern = _ptr(a["load_node"], "i"), _ptr(a["load_pattern"], "i")
        s.load_value = _ptr(a["load_value"], "d")
        self._struct = s
        return s


class PhaseDesc:
    """One analysis phase (integrator, test, number of steps)."""

    def __init__(self, integrator=XG_INT_LOAD_CONTROL, pattern=0, num_steps=1,
                 d_lambda=0.0, dc_node=0, dc_dof=0, dc_incr=0.0, dt=0.0,
                 gamma=0.5, beta=0.25, alpha_m=0.0, beta_k=0.0, beta_k_init=0.0,
                 beta_k_comm=0.0, gm_dof=0, gm_accel=None, gm_dt=0.0, gm_node_record=None,
                 alpha_m_node=None, beta_k_init_elem=None,
                 test=XG_TEST_NORM_DISP_INCR, tol=1e-10, max_iter=25, load_const=0):
        self.kw = dict(integrator=integrator, pattern=pattern, num_steps=num_steps,
                       d_lambda=d_lambda, dc_node=dc_node, dc_dof=dc_dof, dc_incr=dc_incr,
                       dt=dt, gamma=gamma, beta=beta, alpha_m=alpha_m, beta_k=beta_k,
                       beta_k_init=beta_k_init, beta_k_comm=beta_k_comm, gm_dof=gm_dof,
                       gm_dt=gm_dt, test=test, tol=tol, max_iter=max_iter,
                       load_const=load_const)
        # gm_accel: one record [npts] or one per record index [count, npts]
        self.gm_accel = None if gm_accel is None else np.ascontiguousarray(gm_accel, np.float64)
        self.gm_node_record = None if gm_node_record is None else \
            np.ascontiguousarray(gm_node_record, np.int32)
        self.alpha_m_node = None if alpha_m_node is None else \
            np.ascontiguousarray(alpha_m_node, np.float64)
        self.beta_k_init_elem = None if beta_k_init_elem is None else \
            np.ascontiguousarray(beta_k_init_elem, np.float64)

    def __getattr__(self, name):
        kw = self.__dict__.get("kw")
        if kw is not None and name in kw:
            return kw[name]
        raise AttributeError(name)

    def struct(self):
        s = xg_phase_desc(**self.kw)
        if self.gm_accel is None:
            s.gm_npts, s.gm_count = 0, 0
        else:
            a = self.gm_accel if self.gm_accel.ndim == 2 else self.gm_accel[None, :]
            s.gm_count, s.gm_npts = a.shape
        s.gm_accel = _ptr(self.gm_accel, "d")
        s.gm_node_record = _ptr(self.gm_node_record, "i")
        s.alpha_m_node = _ptr(self.alpha_m_node, "d")
        s.beta_k_init_elem = _ptr(self.beta_k_init_elem, "d")
        self._struct = s
        return s
