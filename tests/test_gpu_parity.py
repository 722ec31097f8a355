"""Parity of the CUDA path (through the C ABI) with the reference.

Golden fixtures come from the reference's own classes; the C oracle covers
the rest.  Floating-point tolerances: resisting force and tangent values per
Newton iteration within a relative 1e-12 (norm-wise per vector), converged
displacement histories within a relative 1e-8.  Integer work (equation
numbers, CSR pattern) is bit-exact.
"""
import numpy as np
import pytest

from golden_util import (RTOL_HISTORY, RTOL_STATE, assemble_elements, csc_to_csr_values,
                         external_load, load, model_of, relerr, row_relerr,
                         unbalance_solves)

pytestmark = pytest.mark.gpu

MODELS = ["quad_8x4", "quad_64x16", "brick_4x3x2", "brick_8x8x4"]


@pytest.fixture(scope="module")
def gpu_mod(need_gpu):
    from xara_gb300 import gpu
    gpu.lib()
    return gpu


@pytest.mark.parametrize("name", MODELS)
def test_device_numbering_and_pattern(gpu_mod, name):
    fx = load(name)
    desc, _ = model_of(fx)
    with gpu_mod.DeviceModel(desc) as m:
        assert np.array_equal(m.numbering(), fx["eqn"])
        rp, ci = m.pattern()
        assert np.array_equal(rp, fx["colstart"])
        assert np.array_equal(ci, fx["rowidx"])


def _history_to_device(desc, ep, xi):
    """Fixture history [npts, 6 (xx yy zz xy yz zx)] -> device SoA layout."""
    nh = 4 if desc.elem_type == 1 else 6
    return np.concatenate([ep[:, c] for c in range(nh)] + [xi])


@pytest.mark.parametrize("name", ["quad_8x4", "brick_4x3x2"])
def test_replay_element_state(gpu_mod, name):
    """Every captured Newton iteration: the device's resisting force and
    tangent from the reference's trial displacements."""
    fx = load(name)
    desc, phases = model_of(fx)
    eqn = fx["eqn"]
    with gpu_mod.DeviceModel(desc) as m:
        checked = 0
        for si, step in enumerate(fx["hist_steps"]):
            m.set_history(_history_to_device(desc, fx["hist_ep"][si], fx["hist_xi"][si]))
            for k in unbalance_solves(fx, desc, phases[0]):
                if fx["cap_step"][k] != step:
                    continue
                m.set_trial_disp(fx["cap_U"][k])
                vals, resid, st = m.update()
                fext = external_load(fx, desc, k, eqn)
                assert relerr(resid, fext - fx["cap_B"][k]) < RTOL_STATE
                ref = csc_to_csr_values(fx, fx["cap_A"][k])
                assert relerr(vals, ref) < RTOL_STATE
                assert row_relerr(fx, vals, ref) < RTOL_STATE
                checked += 1
        assert checked >= 4


@pytest.mark.parametrize("system", ["profile", "pcg"])
@pytest.mark.parametrize("name", MODELS)
def test_displacement_history(gpu_mod, name, system):
    """Whole analysis (DisplacementControl + Newton + the device solver,
    skyline LDL' or block-Jacobi PCG): converged displacements and load
    factors per step vs the reference."""
    fx = load(name)
    desc, phases = model_of(fx)
    with gpu_mod.DeviceModel(desc) as m:
        m.set_system(gpu_mod.XG_SYSTEM_PROFILE_SPD if system == "profile"
                     else gpu_mod.XG_SYSTEM_BJPCG)
        U, lam, stats = m.run(phases)
    assert relerr(U, fx["step_u"]) < RTOL_HISTORY
    assert relerr(lam, fx["step_lambda"]) < RTOL_HISTORY
    iters = np.array([s[0] for s in stats])
    # Newton iteration counts agree except where ||dU|| lands within the PCG
    # tolerance of the 1e-10 test threshold
    assert np.mean(iters == fx["step_iters"]) >= 0.8, (iters, fx["step_iters"])


@pytest.mark.parametrize("name,kb", [("brick_8x8x4", 3), ("quad_64x16", 2),
                                     ("frame3d_2x1x3", 6)])
def test_pcg_node_block_layout(gpu_mod, name, kb):
    """After a PCG solve the tangent's node-block copy has the block order of
    the model's nodes and one block per coupled node pair of the pattern
    (node rows coupled to more than 96 nodes left to the CSR chunks)."""
    fx = load(name)
    desc, phases = model_of(fx)
    with gpu_mod.DeviceModel(desc) as m:
        assert gpu_mod.pcg_layout(m)[0] == 0
        m.set_system(gpu_mod.XG_SYSTEM_BJPCG)
        m.set_phase(phases[0])
        m.analyze(1)
        order, blocks, chunked = gpu_mod.pcg_layout(m)
        rp, ci = m.pattern()
        eqn = np.asarray(m.numbering()).reshape(-1, desc.ndf)
    assert order == kb
    # the node owning each equation: its free dofs, not the equalDOF-tied
    # ones (those carry the retained node's equation)
    tags = list(np.asarray(desc.node_tag))
    tied = set()
    if desc.arrays.get("mp_constrained") is not None:
        for t, d in zip(desc.arrays["mp_constrained"], desc.arrays["mp_dof"]):
            tied.add((tags.index(int(t)), int(d)))
    node_of = np.full(len(rp) - 1, -1)
    for n, row in enumerate(eqn):
        for d, r in enumerate(row):
            if r >= 0 and (n, d) not in tied:
                node_of[r] = n
    assert (node_of >= 0).all()
    pairs = {}
    for r in range(len(rp) - 1):
        pairs.setdefault(node_of[r], set()).update(node_of[ci[rp[r]:rp[r + 1]]].tolist())
    want = sum(len(v) for v in pairs.values() if len(v) <= 96)
    long_rows = sum(int(np.sum(node_of == n)) for n, v in pairs.items() if len(v) > 96)
    assert blocks == want and chunked == long_rows


def test_assembly_is_deterministic(gpu_mod):
    fx = load("brick_4x3x2")
    desc, _ = model_of(fx)
    with gpu_mod.DeviceModel(desc) as m:
        m.set_trial_disp(fx["cap_U"][1])
        v1, r1, _ = m.update()
        v2, r2, _ = m.update()
    assert np.array_equal(v1, v2) and np.array_equal(r1, r2)


@pytest.mark.parametrize("name", ["quad_8x4", "frame3d_2x1x3"])
def test_profile_ldl_against_dense_solve(gpu_mod, name):
    """Device skyline LDL' (envelope tiles, 32 x 32) against a dense solve,
    on a quad tangent and on a 3D frame tangent whose envelope spans several
    tiles; two right-hand sides per factorisation, as DisplacementControl
    uses it."""
    fx = load(name)
    desc, _ = model_of(fx)
    with gpu_mod.DeviceModel(desc) as m:
        m.set_system(gpu_mod.XG_SYSTEM_PROFILE_SPD)
        m.set_trial_disp(fx["step_u"][3] if name.startswith("frame") else fx["cap_U"][1])
        vals, resid, _ = m.update()
        rp, ci = m.pattern()
        n = m.neq
        A = np.zeros((n, n))
        for r in range(n):
            A[r, ci[rp[r]:rp[r + 1]]] = vals[rp[r]:rp[r + 1]]
        rng = np.random.default_rng(4)
        for _ in range(2):
            b = rng.normal(size=n)
            x, it, rr = m.solve(b)
            assert relerr(x, np.linalg.solve(A, b)) < 1e-10


def test_pcg_against_dense_solve(gpu_mod):
    fx = load("quad_8x4")
    desc, _ = model_of(fx)
    with gpu_mod.DeviceModel(desc) as m:
        m.set_system(gpu_mod.XG_SYSTEM_BJPCG)
        m.set_trial_disp(fx["cap_U"][1])
        vals, resid, _ = m.update()
        rp, ci = m.pattern()
        n = m.neq
        A = np.zeros((n, n))
        for r in range(n):
            A[r, ci[rp[r]:rp[r + 1]]] = vals[rp[r]:rp[r + 1]]
        b = np.random.default_rng(3).normal(size=n)
        x, it, rr = m.solve(b, rtol=1e-13)
    xd = np.linalg.solve(A, b)
    assert rr <= 1e-13
    assert relerr(x, xd) < 1e-9


def test_pipelined_sweeps_two_rhs_displacement_control(gpu_mod):
    """DisplacementControl solves two right-hand sides per factorisation; on
    8,128 equations (254 tile rows) they run through the pipelined
    substitutions at distance two: four steps against the oracle."""
    from oracle import port
    from xara_gb300 import configs
    desc, phases = configs.quad_block(128, 32, steps=4)
    o = port.OracleModel(desc)
    Uo, lo, _ = o.run(phases)
    o.close()
    with gpu_mod.DeviceModel(desc) as m:
        m.set_system(gpu_mod.XG_SYSTEM_PROFILE_SPD)
        assert m.neq >= 128 * 32
        U, lam, _ = m.run(phases)
    assert relerr(U, Uo) < RTOL_HISTORY
    assert relerr(lam, lo) < RTOL_HISTORY


def test_pcg_long_constraint_row(gpu_mod):
    """Block-Jacobi PCG on a brick block whose top face is tied in z to one
    node: that node's row (1,446 entries) is summed in chunks of 512 entries
    by separate warps, the other rows one thread each from the sliced copy of
    the matrix.  The solution against the device LDL' and the residual."""
    sp = pytest.importorskip("scipy.sparse")
    from xara_gb300 import configs
    desc, _ = configs.brick_block(nx=16, ny=16, nz=4, steps=1)
    with gpu_mod.DeviceModel(desc) as m:
        u = np.zeros(m.nu)
        u[2::3] = -1e-4 * desc.node_crd.reshape(-1, 3)[:, 2]    # uniform compression
        m.set_trial_disp(u)
        vals, _, _ = m.update()
        rp, ci = m.pattern()
        assert np.diff(rp).max() > 1024
        A = sp.csr_matrix((vals, ci, rp), shape=(m.neq, m.neq))
        b = np.random.default_rng(5).normal(size=m.neq)
        m.set_system(gpu_mod.XG_SYSTEM_BJPCG)
        x, it, rr = m.solve(b, rtol=1e-13)
        assert rr <= 1e-13 and it > 0
        assert np.linalg.norm(A @ x - b) / np.linalg.norm(b) < 1e-11
        m.set_system(gpu_mod.XG_SYSTEM_PROFILE_SPD)
        xl, _, _ = m.solve(b)
    assert relerr(x, xl) < 1e-9


def test_oracle_full_size_quad_against_device(gpu_mod):
    """C0 at full size through the oracle restatement and the device."""
    from oracle import port
    from xara_gb300 import configs
    desc, phases = configs.quad_block(64, 16, steps=20)
    o = port.OracleModel(desc)
    Uo, lo, _ = o.run(phases)
    with gpu_mod.DeviceModel(desc) as m:
        U, lam, _ = m.run(phases)
    assert relerr(U, Uo) < RTOL_HISTORY
    assert relerr(lam, lo) < RTOL_HISTORY


def test_round_trip_history_checkpoint(gpu_mod):
    """The committed history read back and written again reproduces the
    same element state (the SoA store is the checkpoint)."""
    fx = load("quad_8x4")
    desc, phases = model_of(fx)
    with gpu_mod.DeviceModel(desc) as m:
        m.run(phases)
        h = m.history()
        u, _ = m.disp()
        m.set_trial_disp(u)
        v1, r1, _ = m.update()
        m.set_history(h)
        v2, r2, _ = m.update()
    assert np.array_equal(v1, v2) and np.array_equal(r1, r2)


FRAMES = ["frame2d_2x3", "frame3d_1x1x2", "frame3d_2x1x3", "frame2d_eq_2x3", "frame2d_pd_2x3",
          "frame2d_settle_2x3", "frame2d_s01_2x3", "frame2d_s01_eq_2x3",
          "frame2d_rc01_2x3"]


@pytest.mark.parametrize("name", FRAMES)
def test_frame_numbering_pattern_and_history(gpu_mod, name):
    """forceBeamColumn frames (Steel02 / Concrete02 fibers): bit-exact
    numbering and pattern, then the whole gravity + pushover analysis on the
    device against the reference's converged displacements."""
    fx = load(name)
    desc, phases = model_of(fx)
    with gpu_mod.DeviceModel(desc) as m:
        assert np.array_equal(m.numbering(), fx["eqn"])
        rp, ci = m.pattern()
        assert np.array_equal(rp, fx["colstart"]) and np.array_equal(ci, fx["rowidx"])
        U, lam, stats = m.run(phases)
    assert relerr(U, fx["step_u"]) < RTOL_HISTORY
    assert relerr(lam, fx["step_lambda"]) < RTOL_HISTORY
    iters = np.array([s[0] for s in stats])
    assert np.mean(iters == fx["step_iters"]) >= 0.8, (iters, fx["step_iters"])


@pytest.mark.parametrize("name", ["frame2d_2x3", "frame3d_1x1x2", "frame2d_pd_2x3",
                                  "frame2d_settle_2x3", "frame2d_s01_2x3",
                                  "frame2d_rc01_2x3"])
def test_frame_replay_first_step(gpu_mod, name):
    """Every Newton iteration of the first gravity step, replayed in the
    reference's order (the element state is incremental): resisting force
    and tangent of each trial displacement."""
    fx = load(name)
    desc, _ = model_of(fx)
    eqn = fx["eqn"]
    with gpu_mod.DeviceModel(desc) as m:
        for k in range(len(fx["cap_step"])):
            m.set_trial_disp(fx["cap_U"][k])
            vals, resid, st = m.update()
            fext = external_load(fx, desc, k, eqn)
            assert relerr(resid, fext - fx["cap_B"][k]) < RTOL_STATE
            ref = csc_to_csr_values(fx, fx["cap_A"][k])
            assert relerr(vals, ref) < RTOL_STATE
            assert row_relerr(fx, vals, ref) < RTOL_STATE


@pytest.mark.parametrize("name", ["revert_frame2d_2x3", "revert_frame3d_1x1x2",
                                  "revert_quad_8x4"])
def test_revert_to_last_commit(gpu_mod, name):
    """Element state at U + dU, then xg_elemset_revert (Domain::
    revertToLastCommit) and the state at U + dU/2, against the reference's
    element responses: initialFlag, the sections re-evaluated at their
    committed deformations and the fiber records all return as the
    reference's do."""
    fx = load(name)
    desc, phases = model_of(fx)
    rp, ci = fx["colstart"], fx["rowidx"]
    u = fx["u"]
    with gpu_mod.DeviceModel(desc) as m:
        m.run(phases[:1], record=False)
        uc, _ = m.disp()
        assert relerr(uc, u) < RTOL_HISTORY
        for key, trial, revert in (("1", u + fx["du"], False), ("2", u + 0.5 * fx["du"], True)):
            if revert:
                m.revert()
            m.set_trial_disp(trial)
            vals, resid, st = m.update()
            v_ref, r_ref = assemble_elements(desc, fx["eqn"], rp, ci, fx["K" + key],
                                             fx["P" + key])
            assert relerr(resid, r_ref) < RTOL_STATE, key
            assert relerr(vals, v_ref) < RTOL_STATE, key
            assert row_relerr(fx, vals, v_ref) < RTOL_STATE, key


@pytest.mark.parametrize("system", ["profile", "pcg"])
def test_frame_batch_parts_match_separate_runs(gpu_mod, system):
    """Six frames under their own records in one device model (Newmark,
    per-frame Rayleigh factors, per-node ground-motion records, per-part
    convergence) against every frame run alone through the oracle: each
    frame's displacement history within 1e-8."""
    from oracle import port
    from xara_gb300 import configs
    desc, phases, parts = configs.frame_batch(6, steps=60, seed=3, return_parts=True)
    with gpu_mod.DeviceModel(desc) as m:
        m.set_system(gpu_mod.XG_SYSTEM_PROFILE_SPD if system == "profile"
                     else gpu_mod.XG_SYSTEM_BJPCG)
        U, _, stats = m.run(phases)
    off = 0
    for d, p in parts:
        o = port.OracleModel(d)
        Uf, _, its = o.run(p)
        o.close()
        nu = d.num_nodes * d.ndf
        assert relerr(U[:, off:off + nu], Uf) < RTOL_HISTORY, off
        off += nu
    assert off == U.shape[1]


def test_autotuned_element_shape_gives_identical_results(gpu_mod):
    """The element kernel's block shape (chosen by the autotuner) does not
    change a single bit of the analysis."""
    from xara_gb300 import configs
    desc, phases = configs.frame_batch(3, steps=30, seed=5)
    runs = []
    for tune in (False, True):
        with gpu_mod.DeviceModel(desc) as m:
            m.set_system(gpu_mod.XG_SYSTEM_PROFILE_SPD)
            if tune:
                gpu_mod.autotune(m, element=True, pcg=False)
            U, _, _ = m.run(phases)
            runs.append(U)
            if tune:
                warps, _, pending = gpu_mod.autotune_result(m)
                assert warps in (1, 2, 4, 8) and pending == 0
    assert np.array_equal(runs[0], runs[1])


def test_profile_pipelined_sweeps_residual(gpu_mod):
    """A system with enough tile rows (8,514 equations, 267 tile rows) for
    the substitutions to run pipelined over many blocks: the LDL' solution's
    relative residual, and agreement with a tightly converged PCG."""
    sp = pytest.importorskip("scipy.sparse")
    from xara_gb300 import configs
    desc, _ = configs.quad_block(128, 32)
    with gpu_mod.DeviceModel(desc) as m:
        u = np.zeros(m.nu)
        crd = desc.node_crd.reshape(-1, 2)
        u[1::2] = -2e-3 * crd[:, 1] * (1 + 0.3 * np.sin(crd[:, 0] / 9.0))
        m.set_trial_disp(u)
        vals, _, _ = m.update()
        rp, ci = m.pattern()
        assert m.neq >= 128 * 32
        A = sp.csr_matrix((vals, ci, rp), shape=(m.neq, m.neq))
        b = np.random.default_rng(9).normal(size=m.neq)
        m.set_system(gpu_mod.XG_SYSTEM_PROFILE_SPD)
        x, _, _ = m.solve(b)
        assert np.linalg.norm(A @ x - b) / np.linalg.norm(b) < 1e-12
        m.set_system(gpu_mod.XG_SYSTEM_BJPCG)
        xp, _, rr = m.solve(b, rtol=1e-14)
        assert relerr(x, xp) < 1e-9


def test_brick_tangent_outside_the_split_range(gpu_mod):
    """A brick block whose coordinates (and displacements) are scaled by
    1e-35: the strains are unchanged but dN/dx reaches 1e35, past the range
    a float pair holds, so the model forms the tangent with its FP64 kernel
    (and gathers doubles).  Element matrices and resisting forces against
    the oracle's within 1e-12, as at ordinary scales."""
    from oracle import port
    from xara_gb300._abi import ModelDesc
    fx = load("brick_4x3x2")
    desc, _ = model_of(fx)
    s = 1e-35
    kw = {k: v for k, v in desc.arrays.items() if v is not None}
    kw["node_crd"] = np.asarray(desc.arrays["node_crd"]) * s
    small = ModelDesc(ndm=desc.ndm, ndf=desc.ndf, elem_type=desc.elem_type,
                      handler=desc.handler, **kw)
    U = fx["step_u"][3] * s
    o = port.OracleModel(small)
    Ko, Po = o.element_matrices(U)
    o.close()
    with gpu_mod.DeviceModel(small) as m:
        m.set_trial_disp(U)
        m.update()
        K, P = m.element_matrices()
    kscale = np.abs(Ko).reshape(len(Ko), -1).max(axis=1)[:, None, None]
    pscale = np.abs(Po).max(axis=1)[:, None]
    assert np.abs(Ko).max() < 1e-20                      # the model's own units
    assert np.max(np.abs(K - Ko) / kscale) < RTOL_STATE
    assert np.max(np.abs(P - Po) / pscale) < RTOL_STATE


@pytest.mark.parametrize("name", ["quad_8x4", "brick_4x3x2", "frame2d_2x3", "frame3d_1x1x2"])
def test_element_matrices_match_the_oracle(gpu_mod, name):
    """xg_elemset_element_matrices (what the element-set shim hands the
    reference's FE_Elements): every element's tangent and resisting force
    after an update at a trial displacement of the reference's record,
    against the oracle's element by element, entry-wise against the
    element's largest entry within 1e-12."""
    from oracle import port
    fx = load(name)
    desc, _ = model_of(fx)
    U = fx["step_u"][min(3, len(fx["step_u"]) - 1)]
    o = port.OracleModel(desc)
    Ko, Po = o.element_matrices(U)
    o.close()
    with gpu_mod.DeviceModel(desc) as m:
        m.set_trial_disp(U)
        m.update()
        K, P = m.element_matrices()
    kscale = np.abs(Ko).reshape(len(Ko), -1).max(axis=1)[:, None, None]
    pscale = np.maximum(np.abs(Po).max(axis=1)[:, None], 1e-300)
    assert np.max(np.abs(K - Ko) / kscale) < RTOL_STATE
    assert np.max(np.abs(P - Po) / pscale) < RTOL_STATE
