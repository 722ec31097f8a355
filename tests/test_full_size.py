"""Parity at the BASELINE sizes.

* Config 1, the 3D RC frame 10x10x20 (6,820 forceBeamColumn elements with
  120- and 64-fiber sections, P-Delta, 14,520 equations): the reference's own
  run of the whole analysis (gravity, loadConst, the DisplacementControl
  pushover to 2 % roof drift in 200 steps) is the fixture
  ``frame3d_c1.npz`` (``tests/golden/make_golden.py c1``).  Checked: the
  numbering and pattern bit for bit; every solve of the first pushover step
  replayed in the reference's order, tangent values entry by entry against
  their row's largest magnitude and the resisting force entry by entry
  against its largest magnitude, within 1e-12; the device analysis's roof
  history, load factors and displacement snapshots within 1e-8.
* Config 2, the stdBrick J2 block 128x128x64 (1,048,576 elements,
  8,388,608 integration points): one element phase at a seeded trial field
  that yields part of the block, against the oracle, entry by entry.
* Config 3, 4,096 frames in one device model: 64 of them, spread over the
  batch, each against its own oracle run over 300 steps of its record.

Tolerances: 1e-12 per entry (state, tangent) relative to the row's largest
magnitude; 1e-8 relative for converged histories (norm-wise per history).
"""
import os

import numpy as np
import pytest

from golden_util import GOLDEN, RTOL_HISTORY, RTOL_STATE, relerr

pytestmark = pytest.mark.gpu

C1 = os.path.join(GOLDEN, "frame3d_c1.npz")


@pytest.fixture(scope="module")
def gpu_mod(need_gpu):
    from xara_gb300 import gpu
    gpu.lib()
    return gpu


@pytest.fixture(scope="module")
def c1():
    if not os.path.exists(C1):
        pytest.skip("frame3d_c1.npz not generated")
    z = np.load(C1)
    return {k: z[k] for k in z.files}


def c1_model():
    from xara_gb300 import configs
    return configs.rc_frame_3d()


def pattern_loads(desc, eqn, neq, pattern):
    f = np.zeros(neq)
    vals = np.asarray(desc.load_value).reshape(-1, desc.ndf)
    for i, n in enumerate(desc.load_node):
        if desc.load_pattern[i] != pattern:
            continue
        idx = int(np.searchsorted(np.asarray(desc.node_tag), n))
        for j in range(desc.ndf):
            r = eqn[idx * desc.ndf + j]
            if r >= 0:
                f[r] += vals[i, j]
    return f


def entrywise(a, b, scale):
    """Largest |a - b| over the scale of each entry."""
    return float(np.max(np.abs(a - b) / np.maximum(scale, 1e-300)))


def test_c1_first_pushover_step_entrywise(gpu_mod, c1):
    """Gravity on the device, then every solve of the first pushover step
    replayed at the reference's trial displacements, in its order (the
    force-based elements iterate from their last trial state): the tangent
    at the 50,000 sampled slots against the row maxima, the resisting force
    P = F_ext - B against its largest entry."""
    desc, phases = c1_model()
    grav = phases[0]
    eqn = c1["eqn"]
    free = c1["free"]
    cs, ri = c1["colstart"], c1["rowidx"]
    slot, scol = c1["slot"], c1["slot_col"]
    srow = ri[slot]
    # gravity, held by loadConst at the factor its last LoadControl step reached
    fgrav = c1["step_lambda"][grav.num_steps - 1] * pattern_loads(desc, eqn, len(cs) - 1, 0)
    phat = pattern_loads(desc, eqn, len(cs) - 1, 1)
    with gpu_mod.DeviceModel(desc) as m:
        assert np.array_equal(m.numbering(), eqn)
        rp, ci = m.pattern()
        assert np.array_equal(rp, cs) and np.array_equal(ci, ri)
        # the device's CSR position of each sampled (row, col) entry
        pos = rp[srow] + np.array([np.searchsorted(ci[rp[r]:rp[r + 1]], c)
                                   for r, c in zip(srow, scol)])
        m.set_phase(grav)
        m.analyze(grav.num_steps)
        u = np.zeros(m.nu)
        last = None
        checked = 0
        for k in range(len(c1["cap_step"])):
            u[free] = c1["cap_U"][k]
            if last is None or not np.array_equal(u, last):
                m.set_trial_disp(u)
                vals, resid, _ = m.update()
                last = u.copy()
            err_a = entrywise(vals[pos], c1["cap_A_slot"][k], c1["cap_A_rowmax"][k][srow])
            assert err_a < RTOL_STATE, (k, err_a)
            if c1["cap_iter"][k] % 2 == 1:         # an unbalance solve: B = F_ext - P
                p_ref = fgrav + c1["cap_lambda"][k] * phat - c1["cap_B"][k]
                err_p = entrywise(resid, p_ref, np.abs(p_ref).max())
                assert err_p < RTOL_STATE, (k, err_p)
            checked += 1
    assert checked >= 5


def test_c1_pushover_history(gpu_mod, c1):
    """The whole analysis on the device (gravity, loadConst, 200
    DisplacementControl steps to 2 % roof drift, device LDL') against the
    reference: roof node history and load factor every step, every free
    displacement every tenth step, Newton iteration counts."""
    desc, phases = c1_model()
    roof_tag = desc.meta["roof"]
    snaps = {int(s): i for i, s in enumerate(c1["snap_steps"])}
    with gpu_mod.DeviceModel(desc) as m:
        m.set_system(gpu_mod.XG_SYSTEM_PROFILE_SPD)
        rid = m.add_recorder([roof_tag], dofs=list(range(6)))
        lam, iters, got = [], [], {}
        step = 0
        for ph in phases:
            m.set_phase(ph)
            for _ in range(ph.num_steps):
                st = m.analyze(1)
                iters.append(st[0][0])
                u, l_ = m.disp()
                lam.append(l_)
                if step in snaps:
                    got[step] = u[c1["free"]]
                step += 1
        roof = m.recorder(rid)[:, -6:]
    assert roof.shape == c1["roof_u"].shape
    assert relerr(roof, c1["roof_u"]) < RTOL_HISTORY
    assert relerr(lam, c1["step_lambda"]) < RTOL_HISTORY
    for s, i in snaps.items():
        assert relerr(got[s], c1["snap_u"][i]) < RTOL_HISTORY, s
    iters = np.asarray(iters)
    assert np.mean(iters == c1["step_iters"]) >= 0.8, (iters, c1["step_iters"])


def brick_field(desc, nx, ny, nz, eps=2.5e-3):
    """Seeded compression with a lateral wave: part of the block yields
    (sigma0 is drawn per element from U[200, 300] MPa)."""
    rng = np.random.default_rng(7)
    crd = desc.node_crd.reshape(-1, 3)
    x, y, z = crd[:, 0] / nx, crd[:, 1] / ny, crd[:, 2] / nz
    shape = 1.0 + 0.6 * np.sin(2 * np.pi * x) * np.cos(np.pi * y)
    u = np.zeros((len(crd), 3))
    u[:, 2] = -eps * nz * z * shape
    u[:, 0] = 0.3 * eps * nx * (x - 0.5) * z
    u[:, 1] = 0.3 * eps * ny * (y - 0.5) * z
    u += rng.normal(0.0, 1e-6, size=u.shape) * (z[:, None] > 0)
    return u.ravel()


def test_c2_element_phase_full_size(gpu_mod):
    """One element phase of the 128x128x64 brick block (1,048,576 bricks,
    263 M tangent entries) on the device and in the oracle: tangent entry
    by entry against its row's largest magnitude, resisting force against
    its largest entry, within 1e-12; most points yield (about 97 %), the
    rest stay elastic."""
    from oracle import port
    from xara_gb300 import configs
    nx, ny, nz = 128, 128, 64
    desc, _ = configs.brick_block(nx, ny, nz, steps=1)
    U = brick_field(desc, nx, ny, nz)
    o = port.OracleModel(desc)
    vo, ro = o.elem_state(U)
    o.commit()
    ep, _ = o.history(8)
    o.close()
    yielded = float(np.mean(np.abs(ep).max(axis=1) > 0))
    assert 0.01 < yielded < 0.999, yielded           # plastic and elastic points both
    with gpu_mod.DeviceModel(desc) as m:
        rp, _ = m.pattern()
        m.set_trial_disp(U)
        v, r, _ = m.update()
    rowmax = np.maximum.reduceat(np.abs(vo), rp[:-1])
    scale = np.repeat(rowmax, np.diff(rp))
    assert entrywise(v, vo, scale) < RTOL_STATE
    assert entrywise(r, ro, np.abs(ro).max()) < RTOL_STATE


def test_c3_batch_frames_against_their_own_runs(gpu_mod):
    """4,096 frames (1-12 bays, 2-20 stories, 40-fiber Steel02 sections,
    each under its own 2,000-step Kanai-Tajimi record) in one device model,
    the first 300 Newmark steps; 64 frames spread over the batch, each run
    alone through the oracle: every frame's displacement history within
    1e-8."""
    from oracle import port
    from xara_gb300 import configs
    from xara_gb300._abi import PhaseDesc
    steps = 300
    desc, phases, parts = configs.frame_batch(4096, steps=2000, seed=0, return_parts=True)
    pick = np.linspace(0, len(parts) - 1, 64).round().astype(int)
    offs = np.concatenate([[0], np.cumsum([d.num_nodes * d.ndf for d, _ in parts])])
    keep = {int(f): [] for f in pick}
    with gpu_mod.DeviceModel(desc) as m:
        m.set_system(gpu_mod.XG_SYSTEM_PROFILE_SPD)
        m.set_phase(phases[0])
        for _ in range(steps):
            m.analyze(1)
            u, _ = m.disp()
            for f in keep:
                keep[f].append(u[offs[f]:offs[f + 1]].copy())
    for f in keep:
        d, p = parts[f]
        o = port.OracleModel(d)
        Uf, _, _ = o.run([PhaseDesc(**{**p[0].kw, "num_steps": steps}, gm_accel=p[0].gm_accel)])
        o.close()
        e = relerr(np.asarray(keep[f]), Uf)
        assert e < RTOL_HISTORY, (f, e)
