"""The OpenSeesPy-style front-end (xara_gb300.openseespy): command sequences
as a user of the reference's Python interface writes them give the same
model description as the library's builders (CPU), and the same analysis on
the GPU -- including a load pattern defined after loadConst, which rebuilds
the device model and replays the analysis so far."""
import numpy as np
import pytest

from xara_gb300 import configs
from xara_gb300 import openseespy as ops


def _quad_script(nx=8, ny=4, steps=4):
    ops.wipe()
    ops.model("basic", "-ndm", 2, "-ndf", 2)
    for j in range(ny + 1):
        for i in range(nx + 1):
            ops.node(j * (nx + 1) + i + 1, float(i), float(j))
    ops.nDMaterial("J2Plasticity", 1, *configs.J2_STEEL[:6])
    t = 1
    for j in range(ny):
        for i in range(nx):
            n1 = j * (nx + 1) + i + 1
            ops.element("quad", t, n1, n1 + 1, n1 + nx + 2, n1 + nx + 1, 1.0, "PlaneStrain", 1)
            t += 1
    for i in range(nx + 1):
        ops.fix(i + 1, 1, 1)
    master = ny * (nx + 1) + 1
    for i in range(1, nx + 1):
        ops.equalDOF(master, master + i, 2)
    ops.timeSeries("Linear", 1)
    ops.pattern("Plain", 1, 1)
    ops.load(master, 0.0, -1.0)
    ops.constraints("Plain")
    ops.numberer("RCM")
    ops.system("ProfileSPD")
    ops.test("NormDispIncr", 1e-10, 25)
    ops.algorithm("Newton")
    ops.integrator("DisplacementControl", master, 2, -0.005 * ny / steps)
    ops.analysis("Static")
    return master


def _frame_script(bays=2, stories=3, nfib=40, steps=5, grav_steps=4, gravity=-150e3,
                  settle=None):
    """settle: a vertical settlement (metres) of the middle base node, an
    `sp` of the gravity pattern under `constraints Transformation`."""
    ops.wipe()
    ops.model("basic", "-ndm", 2, "-ndf", 3)
    nx = bays + 1
    for j in range(stories + 1):
        for i in range(nx):
            ops.node(j * nx + i + 1, i * 6.0, j * 3.5)
    mid = bays // 2 + 1
    for i in range(nx):
        ops.fix(i + 1, 1, 0 if (settle is not None and i + 1 == mid) else 1, 1)
    ops.uniaxialMaterial("Steel02", 1, 350e6, 200e9, 0.01, 18.0, 0.925, 0.15)
    for tag, dims in ((1, (0.45, 0.3, 0.022, 0.014)), (2, (0.5, 0.2, 0.016, 0.010))):
        ops.section("Fiber", tag)
        for y, A in zip(*configs.wide_flange_fibers(*dims, nfib)):
            ops.fiber(y, 0.0, A, 1)
    ops.geomTransf("Linear", 1)
    ops.beamIntegration("Lobatto", 1, 1, 5)
    ops.beamIntegration("Lobatto", 2, 2, 5)
    t = 1
    for j in range(stories):
        for i in range(nx):
            ops.element("forceBeamColumn", t, j * nx + i + 1, (j + 1) * nx + i + 1, 1, 1)
            t += 1
    for j in range(1, stories + 1):
        for i in range(bays):
            ops.element("forceBeamColumn", t, j * nx + i + 1, j * nx + i + 2, 1, 2)
            t += 1
    ops.timeSeries("Linear", 1)
    ops.pattern("Plain", 1, 1)
    for n in range(nx + 1, (stories + 1) * nx + 1):
        ops.load(n, 0.0, gravity, 0.0)
    if settle is not None:
        ops.sp(mid, 2, settle)
    ops.constraints("Plain" if settle is None else "Transformation")
    ops.numberer("RCM")
    ops.system("ProfileSPD")
    ops.test("NormDispIncr", 1e-10, 50)
    ops.algorithm("Newton")
    ops.integrator("LoadControl", 1.0 / grav_steps)
    ops.analysis("Static")
    roof = stories * nx + 1
    return roof, nx


def _lateral(roof, nx, stories=3, steps=5):
    ops.loadConst("-time", 0.0)
    ops.timeSeries("Linear", 2)
    ops.pattern("Plain", 2, 2)
    for j in range(1, stories + 1):
        ops.load(j * nx + 1, float(j) / stories, 0.0, 0.0)
    ops.integrator("DisplacementControl", roof, 1, 0.02 * stories * 3.5 / steps)


def _same_desc(a, b, skip=()):
    assert (a.ndm, a.ndf, a.elem_type) == (b.ndm, b.ndf, b.elem_type)
    for k, v in b.arrays.items():
        if k in skip or v is None:
            continue
        assert a.arrays[k] is not None, k
        np.testing.assert_array_equal(a.arrays[k], v, err_msg=k)


def test_quad_commands_give_the_builders_model():
    _quad_script()
    d, _ = configs.quad_block(8, 4, steps=4)
    _same_desc(ops.build_desc(), d)
    ops.wipe()


def test_frame_commands_give_the_builders_model():
    roof, nx = _frame_script()
    _lateral(roof, nx)
    d, _ = configs.steel_frame_2d(2, 3, steps=5, grav_steps=4)
    _same_desc(ops.build_desc(), d)
    ops.wipe()


def test_rc01_frame_commands_give_the_builders_model():
    """Steel01 bars and Concrete01 layers (`uniaxialMaterial Concrete01 tag
    fpc epsc0 fpcu epscu`, `Steel01 tag fy E0 b a1 a2 a3 a4`) in layered
    fiber sections give the RC frame builder's model."""
    ops.wipe()
    ops.model("basic", "-ndm", 2, "-ndf", 3)
    bays, stories, nx = 2, 3, 3
    for j in range(stories + 1):
        for i in range(nx):
            ops.node(j * nx + i + 1, i * 6.0, j * 3.5)
    for i in range(nx):
        ops.fix(i + 1, 1, 1, 1)
    ops.uniaxialMaterial("Concrete01", 1, -30e6, -0.002, -6e6, -0.006)
    ops.uniaxialMaterial("Steel01", 2, 420e6, 200e9, 0.01, 0.0, 1.0, 0.0, 1.0)
    for tag, (bw, h, nbar) in ((1, (0.5, 0.5, 3)), (2, (0.4, 0.6, 4))):
        ops.section("Fiber", tag)
        for y in (np.arange(10) + 0.5) * h / 10 - h / 2:
            ops.fiber(y, 0.0, bw * h / 10, 1)
        for y in (h / 2 - 0.05, -(h / 2 - 0.05)):
            ops.fiber(y, 0.0, nbar * 491e-6, 2)
    ops.geomTransf("Linear", 1)
    ops.beamIntegration("Lobatto", 1, 1, 5)
    ops.beamIntegration("Lobatto", 2, 2, 5)
    t = 1
    for j in range(stories):
        for i in range(nx):
            ops.element("forceBeamColumn", t, j * nx + i + 1, (j + 1) * nx + i + 1, 1, 1)
            t += 1
    for j in range(1, stories + 1):
        for i in range(bays):
            ops.element("forceBeamColumn", t, j * nx + i + 1, j * nx + i + 2, 1, 2)
            t += 1
    ops.timeSeries("Linear", 1)
    ops.pattern("Plain", 1, 1)
    for n in range(nx + 1, (stories + 1) * nx + 1):
        ops.load(n, 0.0, -100e3, 0.0)
    ops.constraints("Plain")
    ops.numberer("RCM")
    ops.system("ProfileSPD")
    ops.test("NormDispIncr", 1e-10, 50)
    ops.algorithm("Newton")
    ops.integrator("LoadControl", 0.25)
    ops.analysis("Static")
    _lateral(stories * nx + 1, nx)
    d, _ = configs.rc_frame_2d(2, 3, steps=5, grav_steps=4)
    _same_desc(ops.build_desc(), d)
    ops.wipe()
    with pytest.raises(NotImplementedError, match="Concrete04"):
        ops.uniaxialMaterial("Concrete04", 3, -30e6, -0.002, -0.004, 30e9)


def test_transient_commands_give_the_builders_phase():
    """Masses, a Path series under UniformExcitation, rayleigh and Newmark:
    the description and the transient phase equal the builder's."""
    desc, phases = configs.steel_frame_2d_eq(2, 3, steps=40, dt=0.01, grav_steps=4,
                                             with_gravity=True)
    quake = phases[1]
    roof, nx = _frame_script(grav_steps=4)
    q = desc.uni_param.reshape(-1, 12)[0]                  # the builder's seeded fy and b
    ops.uniaxialMaterial("Steel02", 1, *q[:6])
    tags = list(desc.node_tag)
    mass = desc.node_mass.reshape(-1, 3)
    for t, m in zip(tags, mass):
        if m.any():
            ops.mass(t, *m)
    ops.analysis("Transient")
    ops.loadConst("-time", 0.0)
    ops.timeSeries("Path", 7, "-dt", quake.gm_dt, "-values", *quake.gm_accel)
    ops.pattern("UniformExcitation", 8, 1, "-accel", 7)
    ops.rayleigh(desc.meta["alpha_m"], 0.0, desc.meta["beta_k0"], 0.0)
    ops.integrator("Newmark", 0.5, 0.25)
    ops.test("NormDispIncr", 1e-10, 50)
    _same_desc(ops.build_desc(), desc, skip=("load_node", "load_pattern", "load_value"))
    ph = ops._phase(40, 0.01)
    for k in ("integrator", "num_steps", "dt", "gamma", "beta", "alpha_m", "beta_k_init",
              "gm_dof", "gm_dt", "tol", "max_iter"):
        assert ph[k] == getattr(quake, k), k
    np.testing.assert_array_equal(ph["gm_accel"], quake.gm_accel)
    ops.wipe()


def test_unsupported_commands_are_named():
    ops.wipe()
    ops.model("basic", "-ndm", 2, "-ndf", 3)
    with pytest.raises(NotImplementedError, match="uniaxialMaterial Hysteretic"):
        ops.uniaxialMaterial("Hysteretic", 1, 1.0, 1.0, 0.01)
    with pytest.raises(NotImplementedError, match="algorithm KrylovNewton"):
        ops.algorithm("KrylovNewton")
    ops.wipe()


@pytest.mark.gpu
def test_frame_commands_run_like_the_builders(need_gpu, tmp_path):
    from xara_gb300 import gpu
    roof, nx = _frame_script()
    ops.recorder("Node", "-file", str(tmp_path / "roof.out"), "-time", "-node", roof,
                 "-dof", 1, "disp")
    assert ops.analyze(4) == 0
    _lateral(roof, nx)
    assert ops.analyze(5) == 0               # rebuilds with pattern 2 and replays gravity
    u_ops = ops.nodeDisp(roof, 1)
    lines = (tmp_path / "roof.out").read_text().splitlines()
    ops.wipe()
    desc, phases = configs.steel_frame_2d(2, 3, steps=5, grav_steps=4)
    with gpu.DeviceModel(desc) as m:
        m.set_system(gpu.XG_SYSTEM_PROFILE_SPD)
        U, lam, _ = m.run(phases)
    i = list(desc.node_tag).index(roof)
    assert u_ops == U[-1, i * 3]
    # the recorder: 4 gravity steps and 5 pushover steps, time then roof drift
    assert len(lines) == 9
    assert float(lines[-1].split()[1]) == pytest.approx(U[-1, i * 3], rel=1e-5)


@pytest.mark.gpu
def test_quad_commands_run_like_the_builders(need_gpu):
    from xara_gb300 import gpu
    master = _quad_script()
    assert ops.analyze(4) == 0
    u = ops.nodeDisp(master)
    ops.wipe()
    desc, phases = configs.quad_block(8, 4, steps=4)
    with gpu.DeviceModel(desc) as m:
        U, _, _ = m.run(phases)
    i = list(desc.node_tag).index(master)
    np.testing.assert_array_equal(u, U[-1, 2 * i:2 * i + 2])


@pytest.mark.gpu
def test_transformation_commands_run_like_the_builders(need_gpu):
    """`constraints Transformation` with a support settlement imposed by an
    `sp` inside the gravity pattern: the same displacements, bit for bit, as
    the builder's model of it (configs.settlement_frame_2d).  Ten gravity
    steps, as in the golden fixture: the 3 cm settlement in four steps makes
    the first Newton step diverge, in the reference as in the oracle."""
    from xara_gb300 import gpu
    roof, nx = _frame_script(settle=-0.03, grav_steps=10)
    assert ops.analyze(10) == 0
    _lateral(roof, nx)
    assert ops.analyze(5) == 0
    u_roof = ops.nodeDisp(roof)
    u_mid = ops.nodeDisp(2)
    ops.wipe()
    desc, phases = configs.settlement_frame_2d(2, 3, settlement=-0.03, steps=5, grav_steps=10)
    with gpu.DeviceModel(desc) as m:
        U, _, _ = m.run(phases)
    tags = list(desc.node_tag)
    i, k = tags.index(roof), tags.index(2)
    np.testing.assert_array_equal(u_roof, U[-1, 3 * i:3 * i + 3])
    np.testing.assert_array_equal(u_mid, U[-1, 3 * k:3 * k + 3])
    assert u_mid[1] == pytest.approx(-0.03, rel=1e-12)
