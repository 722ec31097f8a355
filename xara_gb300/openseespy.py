"""OpenSeesPy-style commands for the models the device path covers.

The reference's Python interface (SRC/opensees/openseespy.py) forwards
OpenSeesPy calls -- ``model``, ``node``, ``fix``, ``uniaxialMaterial``,
``section``/``fiber``/``patch``/``layer``, ``element``, ``pattern``,
``integrator``, ``analyze``, ``nodeDisp`` ... -- to its Tcl interpreter.  This
module takes the same calls for the hot path's scope and runs them on the
GPU through :class:`xara_gb300.gpu.DeviceModel`::

    from xara_gb300 import openseespy as ops
    ops.model("basic", "-ndm", 2, "-ndf", 3)
    ops.node(1, 0.0, 0.0); ...
    ops.analyze(10)
    ops.nodeDisp(7, 1)

Covered: ``element quad`` (plane strain J2Plasticity), ``element stdBrick``
(J2Plasticity), ``element forceBeamColumn`` (fiber sections of Steel02,
Concrete02, Steel01, Concrete01 and Elastic fibers, Lobatto integration,
Linear and PDelta
transformations; one element type per model), ``fix``, ``equalDOF``,
``mass``, Plain patterns with a Linear series (nodal loads, ``sp``),
``pattern UniformExcitation`` with a Path series, ``rayleigh``,
``constraints Plain|Transformation`` (Transformation with single-point
constraints only: imposed `sp` values, no ``equalDOF``), ``numberer RCM``, ``system
ProfileSPD|CudaBJPCG``, ``test NormDispIncr|NormUnbalance``, ``algorithm
Newton``, ``integrator LoadControl|DisplacementControl|Newmark``,
``loadConst``, ``nodeDisp|nodeVel|nodeAccel``, ``getTime``, ``recorder
Node|EnvelopeNode``.  Anything else raises
``NotImplementedError`` naming the command.

The device model is built at the first ``analyze``.  A command that changes
the model after that (a new load pattern after ``loadConst``, say) rebuilds
it and replays the analysis so far, which gives the same state: the steps
are deterministic and a pattern added later takes no part in the earlier
ones.  Dofs are 1-based as in the reference.
"""
import numpy as np

from . import gpu
from ._abi import (ModelDesc, PhaseDesc, XG_ELE_BRICK, XG_ELE_FBC2D, XG_ELE_FBC3D, XG_ELE_QUAD,
                   XG_HANDLER_PLAIN, XG_HANDLER_TRANSFORMATION, XG_INT_DISP_CONTROL,
                   XG_INT_LOAD_CONTROL, XG_INT_NEWMARK, XG_REC_ACCEL, XG_REC_DISP,
                   XG_REC_ENVELOPE, XG_REC_NODE, XG_REC_VEL, XG_SYSTEM_BJPCG,
                   XG_SYSTEM_PROFILE_SPD, XG_TEST_NORM_DISP_INCR, XG_TEST_NORM_UNBALANCE,
                   XG_UNI_CONCRETE01, XG_UNI_CONCRETE02, XG_UNI_ELASTIC, XG_UNI_NPARAM,
                   XG_UNI_STEEL01, XG_UNI_STEEL02)


class _State:
    def __init__(self):
        self.ndm = self.ndf = None
        self.nodes = {}            # tag -> coordinates
        self.masses = {}           # tag -> ndf values
        self.fixes = []            # (node, dof0)
        self.mps = []              # (retained, constrained, dof0)
        self.nd = {}               # nDMaterial tag -> J2 row
        self.uni = {}              # uniaxialMaterial tag -> (type, row)
        self.sections = {}         # tag -> dict(fibers=[(y, z, A, mat)], GJ)
        self.cur_section = None
        self.transfs = {}          # tag -> (0 Linear | 1 PDelta, vecxz)
        self.integ = {}            # tag -> (section tag, points)
        self.elements = []         # (kind, tag, nodes, attrs)
        self.series = {}           # tag -> (kind, dict)
        self.patterns = []         # dicts: kind, tag, series, loads, sps, dir, factor
        self.cur_pattern = None
        self.rayleigh = (0.0, 0.0, 0.0, 0.0)
        self.handler = XG_HANDLER_PLAIN
        self.system = XG_SYSTEM_PROFILE_SPD
        self.solver = (1e-12, 20000)
        self.test = (XG_TEST_NORM_DISP_INCR, 1e-10, 25)
        self.integrator = None
        self.analysis = None
        self.recorders = []        # dicts
        self.history = []          # ("analyze", phase kwargs, n) | ("loadconst", t)
        self.model = None
        self.built_version = -1
        self.version = 0           # bumped by every command that changes the model
        self.time = 0.0


_S = _State()


def _changed():
    _S.version += 1


def _unsupported(what):
    raise NotImplementedError(f"{what} is outside the device path's scope")


# ---------------------------------------------------------------------------
# model building
# ---------------------------------------------------------------------------
def wipe():
    """Write the recorders' files and clear everything."""
    global _S
    _write_recorders()
    if _S.model is not None:
        _S.model.close()
    _S = _State()


def model(kind, *args):
    if str(kind).lower() not in ("basic", "basicbuilder"):
        _unsupported(f"model {kind}")
    a = [str(x) for x in args]
    _S.ndm = int(a[a.index("-ndm") + 1])
    _S.ndf = int(a[a.index("-ndf") + 1]) if "-ndf" in a else {1: 1, 2: 3, 3: 6}[_S.ndm]
    _changed()


def node(tag, *args):
    args = list(args)
    crd = [float(v) for v in args[:_S.ndm]]
    _S.nodes[int(tag)] = crd
    if "-mass" in [str(a) for a in args]:
        i = [str(a) for a in args].index("-mass")
        _S.masses[int(tag)] = [float(v) for v in args[i + 1:i + 1 + _S.ndf]]
    _changed()


def mass(tag, *values):
    _S.masses[int(tag)] = [float(v) for v in values[:_S.ndf]]
    _changed()


def fix(tag, *flags):
    for d, f in enumerate(flags[:_S.ndf]):
        if int(f):
            _S.fixes.append((int(tag), d))
    _changed()


def equalDOF(retained, constrained, *dofs):
    for d in dofs:
        _S.mps.append((int(retained), int(constrained), int(d) - 1))
    _changed()


def nDMaterial(kind, tag, *args):
    if kind != "J2Plasticity":
        _unsupported(f"nDMaterial {kind}")
    v = [float(a) for a in args]
    # K G sig0 sigInf delta H <eta>; the device row adds rho (unused here)
    row = v[:6] + [v[6] if len(v) > 6 else 0.0, 0.0]
    _S.nd[int(tag)] = row
    _changed()


def uniaxialMaterial(kind, tag, *args):
    v = [float(a) for a in args]
    row = np.zeros(XG_UNI_NPARAM)
    if kind == "Steel02":
        # Fy E b <R0 cR1 cR2 <a1 a2 a3 a4 <sigInit>>> (fedeas.cpp defaults)
        d = [None, None, None, 15.0, 0.925, 0.15, 0.0, 1.0, 0.0, 1.0, 0.0]
        for i, x in enumerate(v[:11]):
            d[i] = x
        row[:11] = d
        _S.uni[int(tag)] = (XG_UNI_STEEL02, row)
    elif kind == "Concrete02":
        row[:7] = v[:7]
        _S.uni[int(tag)] = (XG_UNI_CONCRETE02, row)
    elif kind == "Steel01":
        # fy E0 b <a1 a2 a3 a4> (Steel01.h defaults 0 55 0 55)
        d = [None, None, None, 0.0, 55.0, 0.0, 55.0]
        for i, x in enumerate(v[:7]):
            d[i] = x
        row[:7] = d
        _S.uni[int(tag)] = (XG_UNI_STEEL01, row)
    elif kind == "Concrete01":
        # fpc epsc0 fpcu epscu
        row[:4] = v[:4]
        _S.uni[int(tag)] = (XG_UNI_CONCRETE01, row)
    elif kind == "Elastic":
        row[0] = v[0]
        _S.uni[int(tag)] = (XG_UNI_ELASTIC, row)
    else:
        _unsupported(f"uniaxialMaterial {kind}")
    _changed()


def section(kind, tag, *args):
    if kind not in ("Fiber", "fiberSec"):
        _unsupported(f"section {kind}")
    a = [str(x) for x in args]
    GJ = float(a[a.index("-GJ") + 1]) if "-GJ" in a else 0.0
    _S.sections[int(tag)] = dict(fibers=[], GJ=GJ)
    _S.cur_section = int(tag)
    _changed()


def fiber(y, z, area, mat):
    _S.sections[_S.cur_section]["fibers"].append((float(y), float(z), float(area), int(mat)))
    _changed()


def patch(kind, mat, *args):
    v = [float(a) for a in args]
    if kind == "rect":
        nij, njk = int(v[0]), int(v[1])
        yI, zI, yJ, zJ = v[2:6]
        corners = [(yI, zI), (yJ, zI), (yJ, zJ), (yI, zJ)]
    elif kind == "quad":
        nij, njk = int(v[0]), int(v[1])
        corners = [(v[2], v[3]), (v[4], v[5]), (v[6], v[7]), (v[8], v[9])]
    else:
        _unsupported(f"patch {kind}")
    # QuadPatch::getFibers: bilinear cells, a fiber at each cell's centroid
    # with the cell's area
    (y1, z1), (y2, z2), (y3, z3), (y4, z4) = corners

    def at(s, t):
        return ((1 - s) * (1 - t) * y1 + s * (1 - t) * y2 + s * t * y3 + (1 - s) * t * y4,
                (1 - s) * (1 - t) * z1 + s * (1 - t) * z2 + s * t * z3 + (1 - s) * t * z4)

    for j in range(njk):
        for i in range(nij):
            p = [at(i / nij, j / njk), at((i + 1) / nij, j / njk),
                 at((i + 1) / nij, (j + 1) / njk), at(i / nij, (j + 1) / njk)]
            A = 0.5 * abs(sum(p[k][0] * p[(k + 1) % 4][1] - p[(k + 1) % 4][0] * p[k][1]
                              for k in range(4)))
            cy = sum(q[0] for q in p) / 4
            cz = sum(q[1] for q in p) / 4
            fiber(cy, cz, A, mat)


def layer(kind, mat, *args):
    if kind != "straight":
        _unsupported(f"layer {kind}")
    v = [float(a) for a in args]
    n, A, yS, zS, yE, zE = int(v[0]), v[1], v[2], v[3], v[4], v[5]
    # StraightReinfLayer: bars evenly from start to end (one bar: the middle)
    for i in range(n):
        s = 0.5 if n == 1 else i / (n - 1)
        fiber(yS + s * (yE - yS), zS + s * (zE - zS), A, mat)


def geomTransf(kind, tag, *vecxz):
    t = {"Linear": 0, "PDelta": 1}.get(kind)
    if t is None:
        _unsupported(f"geomTransf {kind}")
    _S.transfs[int(tag)] = (t, [float(v) for v in vecxz[:3]])
    _changed()


def beamIntegration(kind, tag, sec, n):
    if kind != "Lobatto":
        _unsupported(f"beamIntegration {kind}")
    _S.integ[int(tag)] = (int(sec), int(n))
    _changed()


def element(kind, tag, *args):
    a = list(args)
    if kind == "quad":
        nodes = [int(x) for x in a[:4]]
        thick, ptype, mat = float(a[4]), str(a[5]), int(a[6])
        if ptype != "PlaneStrain":
            _unsupported(f"element quad {ptype}")
        _S.elements.append(("quad", int(tag), nodes, dict(thick=thick, mat=mat)))
    elif kind == "stdBrick":
        _S.elements.append(("stdBrick", int(tag), [int(x) for x in a[:8]], dict(mat=int(a[8]))))
    elif kind in ("forceBeamColumn", "nonlinearBeamColumn"):
        i, j = int(a[0]), int(a[1])
        rest = [x for x in a[2:] if not isinstance(x, str)]
        if len(rest) >= 3:       # old syntax: numIntgrPts secTag transfTag
            npts, sec, transf = int(rest[0]), int(rest[1]), int(rest[2])
        else:                    # transfTag integrationTag
            transf = int(rest[0])
            sec, npts = _S.integ[int(rest[1])]
        _S.elements.append(("fbc", int(tag), [i, j], dict(sec=sec, npts=npts, transf=transf)))
    else:
        _unsupported(f"element {kind}")
    _changed()


# ---------------------------------------------------------------------------
# loads
# ---------------------------------------------------------------------------
def timeSeries(kind, tag, *args):
    a = list(args)
    s = [str(x) for x in a]
    if kind in ("Linear", "Constant"):
        f = float(a[s.index("-factor") + 1]) if "-factor" in s else 1.0
        _S.series[int(tag)] = (kind, dict(factor=f))
    elif kind == "Path":
        dt = float(a[s.index("-dt") + 1])
        if "-values" in s:
            i = s.index("-values")
            vals = []
            for x in a[i + 1:]:
                if isinstance(x, str) and x.startswith("-"):
                    break
                vals.append(float(x))
        elif "-filePath" in s:
            vals = list(np.loadtxt(s[s.index("-filePath") + 1]).ravel())
        else:
            _unsupported("timeSeries Path without -values or -filePath")
        f = float(a[s.index("-factor") + 1]) if "-factor" in s else 1.0
        _S.series[int(tag)] = ("Path", dict(dt=dt, values=np.asarray(vals) * f))
    else:
        _unsupported(f"timeSeries {kind}")
    _changed()


def pattern(kind, tag, *args):
    a = list(args)
    s = [str(x) for x in a]
    if kind == "Plain":
        ts = int(a[0])
        if _S.series.get(ts, ("?",))[0] != "Linear":
            _unsupported("a Plain pattern with a series other than Linear")
        p = dict(kind="Plain", tag=int(tag), series=ts, loads=[], sps=[])
    elif kind == "UniformExcitation":
        f = float(a[s.index("-fact") + 1]) if "-fact" in s else 1.0
        ts = int(a[s.index("-accel") + 1])
        p = dict(kind="UniformExcitation", tag=int(tag), dir=int(a[0]) - 1, series=ts, factor=f,
                 loads=[], sps=[])
    else:
        _unsupported(f"pattern {kind}")
    _S.patterns.append(p)
    _S.cur_pattern = p
    _changed()


def load(nodeTag, *values):
    _S.cur_pattern["loads"].append((int(nodeTag), [float(v) for v in values[:_S.ndf]]))
    _changed()


def sp(nodeTag, dof, value):
    _S.cur_pattern["sps"].append((int(nodeTag), int(dof) - 1, float(value)))
    _changed()


def rayleigh(alphaM, betaK, betaKinit, betaKcomm):
    _S.rayleigh = (float(alphaM), float(betaK), float(betaKinit), float(betaKcomm))


# ---------------------------------------------------------------------------
# analysis settings
# ---------------------------------------------------------------------------
def constraints(kind, *args):
    h = {"Plain": XG_HANDLER_PLAIN, "Transformation": XG_HANDLER_TRANSFORMATION}.get(kind)
    if h is None:
        _unsupported(f"constraints {kind}")
    if h != _S.handler:
        _S.handler = h
        _changed()


def numberer(kind, *args):
    if kind != "RCM":
        _unsupported(f"numberer {kind} (the device path numbers with RCM, the default)")


def system(kind, *args):
    if kind == "ProfileSPD":
        _S.system = XG_SYSTEM_PROFILE_SPD
    elif kind == "CudaBJPCG":
        _S.system = XG_SYSTEM_BJPCG
        if len(args) >= 2:
            _S.solver = (float(args[0]), int(args[1]))
    else:
        _unsupported(f"system {kind}")


def test(kind, tol, maxIter, *rest):
    t = {"NormDispIncr": XG_TEST_NORM_DISP_INCR, "NormUnbalance": XG_TEST_NORM_UNBALANCE}.get(kind)
    if t is None:
        _unsupported(f"test {kind}")
    _S.test = (t, float(tol), int(maxIter))


def algorithm(kind, *args):
    if kind != "Newton":
        _unsupported(f"algorithm {kind}")


def integrator(kind, *args):
    if kind == "LoadControl":
        _S.integrator = ("LoadControl", float(args[0]))
    elif kind == "DisplacementControl":
        _S.integrator = ("DisplacementControl", int(args[0]), int(args[1]) - 1, float(args[2]))
    elif kind == "Newmark":
        _S.integrator = ("Newmark", float(args[0]), float(args[1]))
    else:
        _unsupported(f"integrator {kind}")


def analysis(kind, *args):
    if kind not in ("Static", "Transient"):
        _unsupported(f"analysis {kind}")
    _S.analysis = kind


# ---------------------------------------------------------------------------
# the device model
# ---------------------------------------------------------------------------
def build_desc():
    """The model description the commands so far define (no GPU needed)."""
    kinds = {e[0] for e in _S.elements}
    if len(kinds) != 1:
        _unsupported("a model without elements or with several element types")
    kind = kinds.pop()
    tags = sorted(_S.nodes)
    crd = np.asarray([_S.nodes[t] for t in tags], np.float64)
    els = sorted(_S.elements, key=lambda e: e[1])
    kw = dict(ndm=_S.ndm, ndf=_S.ndf, handler=_S.handler, node_tag=tags, node_crd=crd,
              elem_tag=[e[1] for e in els], elem_conn=[e[2] for e in els])
    if _S.masses:
        m = np.zeros((len(tags), _S.ndf))
        for i, t in enumerate(tags):
            if t in _S.masses:
                m[i] = _S.masses[t]
        kw["node_mass"] = m
    if kind in ("quad", "stdBrick"):
        mats = sorted({e[3]["mat"] for e in els})
        kw["elem_type"] = XG_ELE_QUAD if kind == "quad" else XG_ELE_BRICK
        kw["elem_mat"] = [mats.index(e[3]["mat"]) for e in els]
        kw["j2_param"] = np.asarray([_S.nd[t] for t in mats])
        if kind == "quad":
            th = {e[3]["thick"] for e in els}
            if len(th) != 1:
                _unsupported("quads of different thickness")
            kw["thickness"] = th.pop()
    else:
        secs = sorted({e[3]["sec"] for e in els})
        npts = {e[3]["npts"] for e in els}
        tr = {_S.transfs[e[3]["transf"]][0] for e in els}
        if len(npts) != 1 or len(tr) != 1:
            _unsupported("force-based elements with different integration or transformations")
        unis = sorted({f[3] for s in secs for f in _S.sections[s]["fibers"]})
        start, fy_, fz_, fa_, fm_ = [0], [], [], [], []
        for s in secs:
            for y, z, A, mt in _S.sections[s]["fibers"]:
                fy_.append(y)
                fz_.append(z)
                fa_.append(A)
                fm_.append(unis.index(mt))
            start.append(len(fy_))
        kw.update(elem_type=XG_ELE_FBC2D if _S.ndm == 2 else XG_ELE_FBC3D,
                  geom_transf=tr.pop(), fbc_num_ip=npts.pop(),
                  elem_mat=[secs.index(e[3]["sec"]) for e in els],
                  uni_type=[_S.uni[u][0] for u in unis],
                  uni_param=np.asarray([_S.uni[u][1] for u in unis]),
                  sec_fiber_start=start, fib_y=fy_, fib_area=fa_, fib_mat=fm_)
        if _S.ndm == 3:
            kw["fib_z"] = fz_
            kw["sec_GJ"] = [_S.sections[s]["GJ"] for s in secs]
            kw["elem_vecxz"] = [_S.transfs[e[3]["transf"]][1] for e in els]
    # constraints: fixes, then pattern sp (index of its Plain pattern)
    plain = [p for p in _S.patterns if p["kind"] == "Plain"]
    spn = [f[0] for f in _S.fixes]
    spd = [f[1] for f in _S.fixes]
    spp = [-1] * len(_S.fixes)
    spv = [0.0] * len(_S.fixes)
    ln, lp, lv = [], [], []
    for k, p in enumerate(plain):
        for n_, d, v in p["sps"]:
            spn.append(n_)
            spd.append(d)
            spp.append(k)
            spv.append(v)
        for n_, vals in p["loads"]:
            ln.append(n_)
            lp.append(k)
            lv.append(vals + [0.0] * (_S.ndf - len(vals)))
    if spn:
        kw.update(sp_node=spn, sp_dof=spd, sp_pattern=spp, sp_value=spv)
    if ln:
        kw.update(load_node=ln, load_pattern=lp, load_value=lv)
    if _S.mps:
        kw.update(mp_retained=[m_[0] for m_ in _S.mps], mp_constrained=[m_[1] for m_ in _S.mps],
                  mp_dof=[m_[2] for m_ in _S.mps])
    return ModelDesc(**kw)


def _phase(n, dt):
    """The phase of an ``analyze n dt`` with the current settings."""
    plain = [p for p in _S.patterns if p["kind"] == "Plain"]
    pat = len(plain) - 1 if plain else -1
    t, tol, maxit = _S.test
    base = dict(num_steps=n, test=t, tol=tol, max_iter=maxit, pattern=pat)
    ig = _S.integrator
    if ig is None:
        raise RuntimeError("analyze: no integrator")
    if ig[0] == "LoadControl":
        return dict(base, integrator=XG_INT_LOAD_CONTROL, d_lambda=ig[1])
    if ig[0] == "DisplacementControl":
        return dict(base, integrator=XG_INT_DISP_CONTROL, dc_node=ig[1], dc_dof=ig[2],
                    dc_incr=ig[3])
    aM, bK, bK0, bKc = _S.rayleigh
    ph = dict(base, integrator=XG_INT_NEWMARK, dt=float(dt), gamma=ig[1], beta=ig[2],
              alpha_m=aM, beta_k=bK, beta_k_init=bK0, beta_k_comm=bKc)
    ue = [p for p in _S.patterns if p["kind"] == "UniformExcitation"]
    if ue:
        if len(ue) > 1:
            _unsupported("several UniformExcitation patterns")
        kind_, s = _S.series[ue[-1]["series"]]
        if kind_ != "Path":
            _unsupported("UniformExcitation with a series other than Path")
        ph.update(gm_dof=ue[-1]["dir"], gm_accel=s["values"] * ue[-1]["factor"], gm_dt=s["dt"])
    return ph


def _attach_recorders():
    for r in _S.recorders:
        r["id"] = _S.model.add_recorder(r["nodes"], r["dofs"], response=r["response"],
                                        kind=r["kind"], time=r["time"], dT=r["dT"])


def _run(ph_kw, n):
    """0 when all n steps converged, else the library's error code (the
    model is then back at its last committed state)."""
    ph = PhaseDesc(**ph_kw)
    _S.phase = ph                            # keeps the arrays alive
    _S.model.set_phase(ph)
    try:
        _S.model.analyze(int(n))
    except gpu.XaraGpuError as e:
        return e.code
    return 0


def _apply_system():
    """The `system` chosen last (it may change between analyses)."""
    want = (_S.system, _S.solver)
    if getattr(_S, "applied", None) != want:
        _S.model.set_system(_S.system)
        if _S.system == XG_SYSTEM_BJPCG:
            _S.model.set_solver(*_S.solver)
        _S.applied = want


def _ensure_model():
    if _S.model is not None and _S.built_version == _S.version:
        return
    if _S.model is not None:
        _S.model.close()
    _S.model = gpu.DeviceModel(build_desc())
    _S.applied = None
    _apply_system()
    _S.built_version = _S.version
    _attach_recorders()
    for h in _S.history:                     # replay the analysis so far
        if h[0] == "analyze":
            r = _run(h[1], h[2])
            if r != 0:
                raise RuntimeError("replaying the analysis after a model change failed")
        else:
            gpu._check(gpu.lib().xg_analysis_load_const(_S.model.h, h[1]))


def analyze(numIncr=1, dt=0.0, *args):
    """``analyze numIncr <dt>``: 0 on success, < 0 when a step fails (the
    model is then back at its last committed state)."""
    _ensure_model()
    _apply_system()
    ph = _phase(int(numIncr), dt)
    r = _run(ph, int(numIncr))
    if r == 0:
        _S.history.append(("analyze", ph, int(numIncr)))
    _write_recorders()
    return 0 if r == 0 else -1


def loadConst(*args):
    s = [str(a) for a in args]
    t = float(args[s.index("-time") + 1]) if "-time" in s else _S.time
    _S.history.append(("loadconst", t))
    if _S.model is not None:
        import ctypes as C
        L = gpu.lib()
        L.xg_analysis_load_const.argtypes = [C.c_void_p, C.c_double]
        gpu._check(L.xg_analysis_load_const(_S.model.h, t))


# ---------------------------------------------------------------------------
# results
# ---------------------------------------------------------------------------
def _committed():
    u, lam = _S.model.disp()
    return u.reshape(-1, _S.ndf), lam


def nodeDisp(tag, dof=-1):
    u, _ = _committed()
    i = sorted(_S.nodes).index(int(tag))
    return list(u[i]) if int(dof) < 1 else float(u[i, int(dof) - 1])


def _node_response(which, tag, dof):
    u = _S.model.response(which).reshape(-1, _S.ndf)
    i = sorted(_S.nodes).index(int(tag))
    return list(u[i]) if int(dof) < 1 else float(u[i, int(dof) - 1])


def nodeVel(tag, dof=-1):
    return _node_response(XG_REC_VEL, tag, dof)


def nodeAccel(tag, dof=-1):
    return _node_response(XG_REC_ACCEL, tag, dof)


def getTime():
    return _committed()[1] if _S.model is not None else 0.0


def recorder(kind, *args):
    if kind not in ("Node", "EnvelopeNode"):
        _unsupported(f"recorder {kind}")
    a = list(args)
    s = [str(x) for x in a]
    rec = dict(kind=XG_REC_NODE if kind == "Node" else XG_REC_ENVELOPE, time="-time" in s,
               dT=float(a[s.index("-dT") + 1]) if "-dT" in s else 0.0,
               file=s[s.index("-file") + 1] if "-file" in s else None,
               precision=int(a[s.index("-precision") + 1]) if "-precision" in s else 6)

    def ints_after(flag):
        i = s.index(flag) + 1
        out = []
        while i < len(a) and not (isinstance(a[i], str) and not a[i].lstrip("-").isdigit()):
            out.append(int(a[i]))
            i += 1
        return out

    if "-nodeRange" in s:
        lo, hi = ints_after("-nodeRange")[:2]
        rec["nodes"] = [t for t in sorted(_S.nodes) if lo <= t <= hi]
    else:
        rec["nodes"] = ints_after("-node")
    rec["dofs"] = [d - 1 for d in ints_after("-dof")]
    resp = s[-1]
    rec["response"] = {"disp": XG_REC_DISP, "vel": XG_REC_VEL, "accel": XG_REC_ACCEL}.get(resp)
    if rec["response"] is None:
        _unsupported(f"recorder response {resp}")
    _S.recorders.append(rec)
    if _S.model is not None:
        rec["id"] = _S.model.add_recorder(rec["nodes"], rec["dofs"], response=rec["response"],
                                          kind=rec["kind"], time=rec["time"], dT=rec["dT"])
    return len(_S.recorders)


def _write_recorders():
    if _S.model is None:
        return
    for r in _S.recorders:
        if r.get("file") and "id" in r:
            _S.model.write_recorder(r["id"], r["file"], r["precision"])
