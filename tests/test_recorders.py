"""Node and envelope recorders (recorder/NodeRecorder.cpp,
EnvelopeNodeRecorder.cpp): values gathered on the device after every
committed step, against the displacement history the analysis returns, a
host restatement of the envelope's update rule, the -dT thinning, and the
reference's file format (DataFileStream: blank-separated %g rows), and
against the files of the reference's own recorders on the same analysis."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _envelope(vals, times, echo):
    """EnvelopeNodeRecorder::record (EnvelopeNodeRecorder.cpp:401-468)."""
    n = vals.shape[1]
    w = 2 if echo else 1
    env = np.zeros((3, n * w))
    for k, (v, t) in enumerate(zip(vals, times)):
        for i in range(n):
            c = i * w + (1 if echo else 0)
            if k == 0:
                env[:, c] = v[i], v[i], abs(v[i])
                if echo:
                    env[:, c - 1] = t
                continue
            moved = False
            if env[0, c] > v[i]:
                env[0, c] = v[i]
                if echo:
                    env[0, c - 1] = t
                moved = True
            elif env[1, c] < v[i]:
                env[1, c] = v[i]
                if echo:
                    env[1, c - 1] = t
                moved = True
            if moved and env[2, c] < abs(v[i]):
                env[2, c] = abs(v[i])
                if echo:
                    env[2, c - 1] = t
    return env


def test_node_and_envelope_recorders(need_gpu, tmp_path):
    from xara_gb300 import configs, gpu
    desc, phases = configs.frame_batch(2, steps=30, seed=3)
    tags = np.asarray(desc.arrays["node_tag"])
    nodes = [int(tags[1]), int(tags[len(tags) // 2]), int(tags[-1])]
    dofs = [0, 1, 2, 5]                      # dof 5 does not exist in 2D: recorded as 0
    dt = phases[0].dt
    with gpu.DeviceModel(desc) as m:
        m.set_system(gpu.XG_SYSTEM_PROFILE_SPD)
        r_disp = m.add_recorder(nodes, dofs, time=True)
        r_env = m.add_recorder(nodes, [0, 2], kind=gpu.XG_REC_ENVELOPE, time=True)
        r_env0 = m.add_recorder(nodes, [0], kind=gpu.XG_REC_ENVELOPE)
        r_vel = m.add_recorder(nodes, [0], response=gpu.XG_REC_VEL)
        r_vel3 = m.add_recorder(nodes, [0], response=gpu.XG_REC_VEL, dT=3 * dt)
        r_acc = m.add_recorder(nodes, [1], response=gpu.XG_REC_ACCEL)
        U, lam, _ = m.run(phases)
        rows = m.recorder(r_disp)
        env, env0 = m.recorder(r_env), m.recorder(r_env0)
        vel, vel3, acc = m.recorder(r_vel), m.recorder(r_vel3), m.recorder(r_acc)
        m.write_recorder(r_disp, tmp_path / "disp.out")
        m.write_recorder(r_env, tmp_path / "env.out", precision=10)
        v_end, a_end = m.response(gpu.XG_REC_VEL), m.response(gpu.XG_REC_ACCEL)
        np.testing.assert_array_equal(m.response(gpu.XG_REC_DISP), m.disp()[0])
    ndf = desc.ndf
    idx = [np.searchsorted(tags, n) for n in nodes]
    expect = np.zeros((len(U), len(nodes) * len(dofs)))
    for a, i in enumerate(idx):
        for b, d in enumerate(dofs):
            if d < ndf:
                expect[:, a * len(dofs) + b] = U[:, i * ndf + d]
    assert rows.shape == (len(U), 1 + expect.shape[1])
    np.testing.assert_array_equal(rows[:, 0], lam)           # the committed time
    np.testing.assert_array_equal(rows[:, 1:], expect)
    # envelopes: min, max, max |.| with the times they were reached
    ux = expect[:, [a * len(dofs) + b for a in range(len(nodes)) for b in (0, 2)]]
    np.testing.assert_array_equal(env, _envelope(ux, lam, True))
    np.testing.assert_array_equal(env0, _envelope(expect[:, ::len(dofs)], lam, False))
    # -dT: a row when the time has reached the next stamp (1e-6 dT tolerance)
    keep, nxt = [], 0.0
    for k, t in enumerate(lam):
        if t - nxt >= -3 * dt * 1e-6:
            keep.append(k)
            nxt = t + 3 * dt
    np.testing.assert_array_equal(vel3, vel[keep])
    assert vel.shape == (len(U), len(nodes)) and np.abs(vel).max() > 0
    # the last rows are the committed velocities and accelerations
    np.testing.assert_array_equal(vel[-1], v_end[[i * ndf for i in idx]])
    np.testing.assert_array_equal(acc[-1], a_end[[i * ndf + 1 for i in idx]])
    assert acc.shape == (len(U), len(nodes)) and np.abs(acc).max() > 0
    # DataFileStream: blank-separated values, %g with the precision
    text = (tmp_path / "disp.out").read_text().splitlines()
    assert text == [" ".join(f"{v:.6g}" for v in r) for r in rows]
    text = (tmp_path / "env.out").read_text().splitlines()
    assert text == [" ".join(f"{v:.10g}" for v in r) for r in env]


def test_recorder_files_match_the_reference(need_gpu, tmp_path):
    """The same six recorders as the reference's `recorder Node` /
    `recorder EnvelopeNode` (NodeRecorder, EnvelopeNodeRecorder and
    DataFileStream compiled from its sources; tests/golden/make_golden.py
    recorders) on the transient 2D frame: gravity by LoadControl, loadConst
    -time 0, 40 Newmark steps.  Every file has the reference's lines and
    columns; times and the envelope's time stamps equal; values within the
    printed precision of each column's largest magnitude (roundoff-level
    entries such as 1e-21 vertical drifts print differently)."""
    import os
    from golden_util import GOLDEN
    from xara_gb300 import configs, gpu
    path = os.path.join(GOLDEN, "recorders_frame2d_eq.npz")
    if not os.path.exists(path):
        pytest.skip("recorders_frame2d_eq.npz not generated")
    z = np.load(path)
    specs = [("disp", 0, [0, 1, 2, 5], 0, 1, 0, 6), ("env", 1, [0, 2], 0, 1, 0, 10),
             ("env0", 1, [0], 0, 0, 0, 6), ("vel", 0, [0], 1, 0, 0, 6),
             ("vel3", 0, [0], 1, 0, 3, 6), ("acc", 0, [1], 2, 0, 0, 6)]
    responses = [gpu.XG_REC_DISP, gpu.XG_REC_VEL, gpu.XG_REC_ACCEL]
    desc, phases = configs.steel_frame_2d_eq(2, 3, steps=40)
    nodes = [int(n) for n in z["nodes"]]
    dt = phases[-1].dt
    with gpu.DeviceModel(desc) as m:
        m.set_system(gpu.XG_SYSTEM_PROFILE_SPD)
        ids = {}
        for f, env, dofs, resp, echo, dsteps, prec in specs:
            ids[f] = m.add_recorder(nodes, dofs, response=responses[resp],
                                    kind=gpu.XG_REC_ENVELOPE if env else gpu.XG_REC_NODE,
                                    time=bool(echo), dT=dsteps * dt)
        m.run(phases)
        for f, *rest in specs:
            m.write_recorder(ids[f], tmp_path / (f + ".out"), precision=rest[-1])
    for f, env, dofs, resp, echo, dsteps, prec in specs:
        got = (tmp_path / (f + ".out")).read_text().splitlines()
        want = [str(x) for x in z[f]]
        assert len(got) == len(want), (f, len(got), len(want))
        g = np.array([[float(x) for x in line.split()] for line in got])
        w = np.array([[float(x) for x in line.split()] for line in want])
        assert g.shape == w.shape, f
        tcols = [c for c in range(w.shape[1]) if echo and (env and c % 2 == 0 or not env and c == 0)]
        np.testing.assert_array_equal(g[:, tcols], w[:, tcols])     # times
        vcols = [c for c in range(w.shape[1]) if c not in tcols]
        scale = np.maximum(np.abs(w[:, vcols]).max(axis=0), 1e-300)
        assert np.all(np.abs(g[:, vcols] - w[:, vcols]) <= 2 * 10.0 ** (1 - prec) * scale), f


def test_recorder_rejects_unknown_nodes(need_gpu):
    from xara_gb300 import configs, gpu
    desc, _ = configs.frame_batch(1, steps=5, seed=1)
    with gpu.DeviceModel(desc) as m:
        with pytest.raises(gpu.XaraGpuError, match="no node"):
            m.add_recorder([10 ** 8], [0])
        with pytest.raises(gpu.XaraGpuError):
            m.add_recorder([int(desc.arrays["node_tag"][0])], [0], kind=7)
