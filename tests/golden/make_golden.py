"""Generate the golden fixtures in this folder from the reference itself.

Runs in the container that holds the reference sources: it needs
``oracle/_ref/libxara_ref.so`` (``python oracle/build_ref.py``), i.e. the
reference's own CPU classes (J2Plasticity, FourNodeQuad, Brick, Domain,
PlainHandler, RCM, DOF_Numberer, SparseGenColLinSOE, ProfileSPD,
NewtonRaphson, DisplacementControl, ...) compiled from source.  The GPU machine
has no reference; tests there read these fixtures.

Usage: python tests/golden/make_golden.py        (the small fixtures)
       python tests/golden/make_golden.py c1     (frame3d_c1: the full-size 3D RC
                                                  frame pushover, about half an hour)
       python tests/golden/make_golden.py settle (frame2d_settle_2x3 alone)
       python tests/golden/make_golden.py steel01 (uniaxial paths, Steel01 frames)
       python tests/golden/make_golden.py concrete01 (uniaxial paths, the Steel01 /
           Concrete01 surrogate frame and its DDM gradient)
"""
import os
import sys

import numpy as np

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), "..", ".."))
sys.path.insert(0, ROOT)

from oracle import port, ref  # noqa: E402
from xara_gb300 import configs  # noqa: E402
from xara_gb300._abi import PhaseDesc  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def kw_array(kw):
    """Builder keyword values: numbers as float64, or as text when one is a
    string (golden_util.model_of reads both)."""
    vals = list(kw.values())
    if any(isinstance(v, str) for v in vals):
        return np.array([str(v) for v in vals])
    return np.asarray(vals, np.float64)


def save(name, **arrays):
    path = os.path.join(OUT, name + ".npz")
    np.savez_compressed(path, **arrays)
    print(f"{name}.npz: {os.path.getsize(path) / 1024:.0f} KB")


def j2_paths(seed=1):
    """Random strain paths through J2PlaneStrain / J2ThreeDimensional."""
    rng = np.random.default_rng(seed)
    out = {}
    for dim, ns in ((2, 3), (3, 6)):
        n = 200
        steps = rng.normal(0.0, 6e-4, size=(n, ns))
        strain = np.cumsum(steps, axis=0)
        commit = (rng.random(n) < 0.6).astype(np.int32)
        param = np.array([166.7e9, 76.9e9, 250e6, 300e6, 8.0, 1e9, 0.0, 0.0])
        s, t = ref.j2_path(dim, param, strain, commit)
        out[f"d{dim}_param"] = param
        out[f"d{dim}_strain"] = strain
        out[f"d{dim}_commit"] = commit
        out[f"d{dim}_stress"] = s
        out[f"d{dim}_tangent"] = t
    save("j2_paths", **out)


def uniaxial_paths(seed=2):
    """Random strain paths through Steel02, Concrete02, Steel01 and Concrete01."""
    rng = np.random.default_rng(seed)
    out = {}
    for kind, param, scale in ((1, configs.steel02_row(350e6, 200e9, 0.01), 4e-3),
                               (2, configs.concrete02_row(30e6), 2e-3),
                               (4, configs.steel01_row(350e6, 200e9, 0.01, 0.02, 2.0, 0.03, 3.0),
                                4e-3),
                               (5, configs.concrete01_row(30e6), 2e-3)):
        n = 400
        strain = np.cumsum(rng.normal(0.0, scale / 3, size=n))
        commit = (rng.random(n) < 0.5).astype(np.int32)
        s, t = ref.uniaxial_path(kind, param, strain, commit)
        out.update({f"k{kind}_param": param, f"k{kind}_strain": strain,
                    f"k{kind}_commit": commit, f"k{kind}_stress": s, f"k{kind}_tangent": t})
    save("uniaxial_paths", **out)


def model_fixture(name, builder, args, kw, capture_steps=(), cap_solves=400):
    desc, phases = builder(*args, **kw)
    lo = min(capture_steps) if capture_steps else 0
    hi = max(capture_steps) + 1 if capture_steps else 0
    r = ref.RefRun(desc, phases, capture=(lo, hi), cap_solves=cap_solves)
    keep = np.isin(r.cap_step, np.asarray(capture_steps, np.int32))
    arrays = dict(
        builder=np.array(builder.__name__), args=np.asarray(args),
        kw_keys=np.array(list(kw.keys())), kw_vals=kw_array(kw),
        eqn=r.eqn, colstart=r.colstart, rowidx=r.rowidx,
        step_u=r.step_u, step_lambda=r.step_lambda, step_iters=r.step_iters,
    )
    if capture_steps:
        arrays.update(cap_step=r.cap_step[keep], cap_iter=r.cap_iter[keep],
                      cap_B=r.cap_B[keep], cap_A=r.cap_A[keep], cap_U=r.cap_U[keep],
                      cap_lambda=r.cap_lambda[keep])
        # committed material history at the start of every captured step,
        # from the oracle (itself pinned against the reference by these files)
        if desc.elem_type in (3, 4):       # frames: replay from the start only
            save(name, **arrays)
            return
        nip = 4 if desc.elem_type == 1 else 8
        hist_ep, hist_xi = [], []
        for s in sorted(capture_steps):
            o = port.OracleModel(desc)
            if s > 0:
                o.run([PhaseDesc(**{**phases[0].kw, "num_steps": s})])
            ep, xi = o.history(nip)
            o.close()
            hist_ep.append(ep[:, [0, 4, 8, 1, 5, 6]])  # xx yy zz xy yz zx
            hist_xi.append(xi)
        arrays.update(hist_steps=np.asarray(sorted(capture_steps), np.int32),
                      hist_ep=np.asarray(hist_ep), hist_xi=np.asarray(hist_xi))
    save(name, **arrays)


def revert_fixture(name, builder, args, kw, seed=5, scale=2e-4):
    """Element responses around the end of the first phase: at U + dU, then
    after Domain::revertToLastCommit at U + dU/2 (the committed state's
    bookkeeping: initialFlag, section re-evaluation, fiber records)."""
    desc, phases = builder(*args, **kw)
    r = ref.RefRun(desc, phases[:1])
    u = r.step_u[-1]
    du = scale * np.random.default_rng(seed).normal(size=u.size)
    du[r.eqn < 0] = 0.0
    K1, P1 = r.elem_response(u + du)
    K2, P2 = r.elem_response(u + 0.5 * du, revert_first=True)
    save(name, builder=np.array(builder.__name__), args=np.asarray(args),
         kw_keys=np.array(list(kw.keys())), kw_vals=kw_array(kw),
         eqn=r.eqn, colstart=r.colstart, rowidx=r.rowidx, u=u, du=du,
         K1=K1, P1=P1, K2=K2, P2=P2)


def c1_pushover(name="frame3d_c1", sample=50_000, seed=11, every=10):
    """The 3D RC frame 10x10x20 at full size (6,820 forceBeamColumn elements,
    120 / 64 fibers, P-Delta): gravity by LoadControl, loadConst, then the
    DisplacementControl pushover of the roof corner to 2 % drift in 200
    steps, through the reference's own classes.  Kept: the numbering and
    pattern; the roof node's six displacements and the load factor after
    every step; every free displacement after every ``every``-th step; and
    every solve of the first pushover step (trial displacements, right-hand
    sides, the row maxima of the tangent and the tangent values at
    ``sample`` seeded CSC slots)."""
    desc, phases = configs.rc_frame_3d()
    grav = phases[0].num_steps
    r = ref.RefRun(desc, phases, capture=(grav, grav + 1), cap_solves=64)
    ndf = desc.ndf
    roof = int(np.searchsorted(desc.node_tag, desc.meta["roof"]))
    free = np.nonzero(r.eqn >= 0)[0].astype(np.int32)
    snap = np.arange(every - 1, len(r.step_u), every, dtype=np.int32)
    rng = np.random.default_rng(seed)
    slots = np.sort(rng.choice(r.nnz, size=sample, replace=False)).astype(np.int32)
    cs, ri = r.colstart, r.rowidx
    cols = np.repeat(np.arange(r.neq), np.diff(cs))
    rowmax = np.zeros((len(r.cap_A), r.neq))
    for k, a in enumerate(r.cap_A):
        # the pattern is symmetric: the largest |entry| of row i is that of column i
        rowmax[k] = np.maximum.reduceat(np.abs(a), cs[:-1])
    save(name, builder=np.array("rc_frame_3d"), args=np.asarray([], np.int64),
         kw_keys=np.array([], dtype="<U1"), kw_vals=np.asarray([], np.float64),
         eqn=r.eqn, colstart=cs, rowidx=ri,
         step_lambda=r.step_lambda, step_iters=r.step_iters,
         roof_u=r.step_u[:, roof * ndf:(roof + 1) * ndf],
         free=free, snap_steps=snap, snap_u=r.step_u[snap][:, free],
         cap_step=r.cap_step, cap_iter=r.cap_iter, cap_B=r.cap_B,
         cap_U=r.cap_U[:, free], cap_lambda=r.cap_lambda,
         slot=slots, slot_col=cols[slots].astype(np.int32), cap_A_slot=r.cap_A[:, slots],
         cap_A_rowmax=rowmax,
         ref_seconds=np.array([r.elem_seconds, r.solve_seconds, r.step_seconds]))


def steel01_fixtures():
    """2D steel frames with Steel01 fibers: gravity and pushover (every solve
    of the first gravity step captured) and gravity then a ground motion
    (Newmark, Rayleigh on the initial stiffness)."""
    model_fixture("frame2d_s01_2x3", configs.steel_frame_2d, (2, 3),
                  {"steps": 12, "law": "Steel01"}, capture_steps=(0,))
    model_fixture("frame2d_s01_eq_2x3", configs.steel_frame_2d_eq, (2, 3),
                  {"steps": 150, "law": "Steel01"})


def ddm_fixture(name="ddm_steel01_frame"):
    """The reference's DDM gradient (computeGradients at every step) of the
    summed squared roof drift of configs.ddm_steel01_frame with respect to
    every member's Steel01 fy, E0 and b, and the objective itself."""
    desc, phases = configs.ddm_steel01_frame()
    params = [(int(t), k) for t in desc.elem_tag for k in range(3)]
    obj = (desc.meta["obj_node"], desc.meta["obj_dof"], desc.meta["obj_weight"])
    grad, J, run = ref.ddm_gradient(desc, phases, params, obj)
    save(name, builder=np.array("ddm_steel01_frame"), args=np.asarray([], np.int64),
         kw_keys=np.array([], dtype="<U1"), kw_vals=np.asarray([], np.float64),
         grad=grad.reshape(-1, 3), J=np.array([J]), step_u=run.step_u,
         step_iters=run.step_iters)


def concrete01_fixtures():
    """The Steel01 / Concrete01 surrogate: the 2D RC frame's gravity and
    pushover (every solve of the first gravity step captured), and the
    reference's DDM gradient of the summed squared roof drift of the
    massless ramp with respect to every member's Concrete01 fc, epsco, fcu
    and Steel01 fy, E, b (checked against central differences of the oracle
    before it is written)."""
    model_fixture("frame2d_rc01_2x3", configs.rc_frame_2d, (2, 3), {"steps": 20},
                  capture_steps=(0,))
    desc, phases = configs.ddm_rc01_frame()
    params = [(int(t), k) for t in desc.elem_tag for k in (3, 4, 5, 0, 1, 2)]
    obj = (desc.meta["obj_node"], desc.meta["obj_dof"], desc.meta["obj_weight"])
    grad, J, run = ref.ddm_gradient(desc, phases, params, obj)
    grad = grad.reshape(-1, 3)
    q0 = desc.uni_param.reshape(-1, 12)
    roof = list(desc.node_tag).index(int(obj[0][0]))

    def J_of(q):
        d = configs._with_geometry(desc, uni_param=q)
        o = port.OracleModel(d)
        U, _, _ = o.run(phases)
        o.close()
        return obj[2][0] * np.sum(U[:, 3 * roof] ** 2)

    worst = 0.0
    for k in range(3):
        scale = np.abs(grad[:, k] * q0[:, k]).max()
        for u in np.argsort(np.abs(grad[:, k] * q0[:, k]))[-3:]:
            h = 1e-6 * abs(q0[u, k])
            qp, qm = q0.copy(), q0.copy()
            qp[u, k] += h
            qm[u, k] -= h
            fd = (J_of(qp) - J_of(qm)) / (2 * h)
            worst = max(worst, abs(fd - grad[u, k]) * abs(q0[u, k]) / scale)
    print(f"ddm_rc01_frame: reference DDM against central differences of the oracle: "
          f"{worst:.2e} of each kind's largest scaled entry")
    save("ddm_rc01_frame", builder=np.array("ddm_rc01_frame"), args=np.asarray([], np.int64),
         kw_keys=np.array([], dtype="<U1"), kw_vals=np.asarray([], np.float64),
         grad=grad, J=np.array([J]), step_u=run.step_u, step_iters=run.step_iters,
         fd_check=np.array([worst]))


def settlement_fixture():
    """The 2D steel frame with a support settlement imposed through the
    Transformation handler (gravity and settlement by LoadControl, then the
    pushover), every solve of the first gravity step captured."""
    model_fixture("frame2d_settle_2x3", configs.settlement_frame_2d, (2, 3), {},
                  capture_steps=(0,))


# The recorders of the transient 2D frame fixture: file, envelope, dofs
# (0-based; 5 does not exist in 2D), response (0 disp, 1 vel, 2 accel),
# -time, -dT (in record steps), -precision.
RECORDER_SPECS = [
    ("disp", 0, [0, 1, 2, 5], 0, 1, 0, 6),
    ("env", 1, [0, 2], 0, 1, 0, 10),
    ("env0", 1, [0], 0, 0, 0, 6),
    ("vel", 0, [0], 1, 0, 0, 6),
    ("vel3", 0, [0], 1, 0, 3, 6),
    ("acc", 0, [1], 2, 0, 0, 6),
]


def recorder_fixture(name="recorders_frame2d_eq"):
    """`recorder Node` / `recorder EnvelopeNode` of the reference
    (NodeRecorder, EnvelopeNodeRecorder, DataFileStream) on the transient
    2D steel frame: gravity by LoadControl, loadConst -time 0, 40 Newmark
    steps; the files' lines as the reference wrote them."""
    import ctypes as C
    import tempfile
    desc, phases = configs.steel_frame_2d_eq(2, 3, steps=40)
    tags = np.asarray(desc.arrays["node_tag"])
    nodes = np.array([tags[1], tags[len(tags) // 2], tags[-1]], np.int32)
    dt = phases[-1].dt
    L = ref.lib()
    L.xref_add_node_recorder.argtypes = [C.c_void_p, C.c_char_p, C.c_int, C.c_int, C.c_void_p,
                                         C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_double,
                                         C.c_int]
    L.xref_close_recorders.argtypes = [C.c_void_p]
    tmp = tempfile.mkdtemp()

    def attach(h):
        for f, env, dofs, resp, echo, dsteps, prec in RECORDER_SPECS:
            da = np.array(dofs, np.int32)
            r = L.xref_add_node_recorder(C.c_void_p(h), os.path.join(tmp, f + ".out").encode(),
                                         env, len(nodes), nodes.ctypes.data_as(C.c_void_p),
                                         len(dofs), da.ctypes.data_as(C.c_void_p), resp, echo,
                                         dsteps * dt, prec)
            assert r == 0, f

    run = ref.RefRun(desc, phases, attach=attach)
    L.xref_close_recorders(C.c_void_p(run.h))
    arrays = {"nodes": nodes}
    for f, *_ in RECORDER_SPECS:
        with open(os.path.join(tmp, f + ".out")) as fh:
            arrays[f] = np.array(fh.read().splitlines())
    save(name, **arrays)


def main():
    if not ref.available():
        sys.exit("oracle/_ref/libxara_ref.so missing: run python oracle/build_ref.py")
    if sys.argv[1:] == ["c1"]:
        c1_pushover()
        return
    if sys.argv[1:] == ["recorders"]:
        recorder_fixture()
        return
    if sys.argv[1:] == ["settle"]:
        settlement_fixture()
        return
    if sys.argv[1:] == ["concrete01"]:
        uniaxial_paths()
        concrete01_fixtures()
        return
    if sys.argv[1:] == ["steel01"]:
        uniaxial_paths()
        steel01_fixtures()
        ddm_fixture()
        return
    j2_paths()
    model_fixture("quad_8x4", configs.quad_block, (8, 4), {}, capture_steps=(0, 6))
    model_fixture("quad_64x16", configs.quad_block, (64, 16), {})
    model_fixture("brick_4x3x2", configs.brick_block, (4, 3, 2), {"steps": 5},
                  capture_steps=(0, 2))
    model_fixture("brick_8x8x4", configs.brick_block, (8, 8, 4), {"steps": 10})
    uniaxial_paths()
    model_fixture("frame2d_2x3", configs.steel_frame_2d, (2, 3), {"steps": 10},
                  capture_steps=(0,))
    model_fixture("frame3d_1x1x2", configs.rc_frame_3d, (1, 1, 2),
                  {"col_fibers": 40, "beam_fibers": 24, "steps": 10, "pdelta": 1},
                  capture_steps=(0,))
    model_fixture("frame3d_2x1x3", configs.rc_frame_3d, (2, 1, 3),
                  {"col_fibers": 60, "beam_fibers": 40, "steps": 30, "pdelta": 1})
    model_fixture("frame2d_eq_2x3", configs.steel_frame_2d_eq, (2, 3), {"steps": 150})
    model_fixture("frame2d_pd_2x3", configs.steel_frame_2d, (2, 3), {"steps": 12, "pdelta": 1},
                  capture_steps=(0,))
    revert_fixture("revert_frame2d_2x3", configs.steel_frame_2d, (2, 3), {"steps": 10})
    revert_fixture("revert_frame3d_1x1x2", configs.rc_frame_3d, (1, 1, 2),
                   {"col_fibers": 40, "beam_fibers": 24, "steps": 10, "pdelta": 1})
    revert_fixture("revert_quad_8x4", configs.quad_block, (8, 4), {}, scale=1e-4)
    settlement_fixture()
    steel01_fixtures()
    ddm_fixture()
    concrete01_fixtures()


if __name__ == "__main__":
    main()
