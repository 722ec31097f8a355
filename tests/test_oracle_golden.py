"""The oracle (oracle/xara_oracle.c) against fixtures produced by the
reference's own CPU classes (tests/golden/make_golden.py).  CPU only."""
import numpy as np
import pytest

from oracle import port
from golden_util import (RTOL_HISTORY, RTOL_STATE, assemble_elements, csc_to_csr_values,
                         external_load, load, model_of, relerr, row_relerr, unbalance_solves)

MODELS = ["quad_8x4", "quad_64x16", "brick_4x3x2", "brick_8x8x4"]


def test_j2_material_paths():
    fx = load("j2_paths")
    for dim in (2, 3):
        s, t = port.j2_path(dim, fx[f"d{dim}_param"], fx[f"d{dim}_strain"], fx[f"d{dim}_commit"])
        for k in range(len(s)):
            assert relerr(s[k], fx[f"d{dim}_stress"][k]) < RTOL_STATE
            assert relerr(t[k], fx[f"d{dim}_tangent"][k]) < RTOL_STATE


@pytest.mark.parametrize("name", MODELS)
def test_numbering_and_pattern_bit_exact(name):
    fx = load(name)
    desc, phases = model_of(fx)
    o = port.OracleModel(desc)
    assert np.array_equal(o.numbering(), fx["eqn"])
    rp, ci = o.pattern()
    assert np.array_equal(rp, fx["colstart"])
    assert np.array_equal(ci, fx["rowidx"])


@pytest.mark.parametrize("name", MODELS)
def test_history(name):
    fx = load(name)
    desc, phases = model_of(fx)
    o = port.OracleModel(desc)
    U, lam, its = o.run(phases)
    assert relerr(U, fx["step_u"]) < RTOL_HISTORY
    assert relerr(lam, fx["step_lambda"]) < RTOL_HISTORY
    assert np.array_equal(its, fx["step_iters"])


@pytest.mark.parametrize("name", ["quad_8x4", "brick_4x3x2"])
def test_replay_element_state(name):
    """Resisting force and tangent of every captured Newton iteration."""
    fx = load(name)
    desc, phases = model_of(fx)
    eqn = fx["eqn"]
    for si, step in enumerate(fx["hist_steps"]):
        o = port.OracleModel(desc)
        ep = fx["hist_ep"][si]
        full = np.zeros((ep.shape[0], 9))
        full[:, [0, 4, 8, 1, 5, 6]] = ep
        full[:, [3, 7, 2]] = ep[:, [3, 4, 5]]
        o.set_history(full, fx["hist_xi"][si])
        for k in unbalance_solves(fx, desc, phases[0]):
            if fx["cap_step"][k] != step:
                continue
            vals, resid = o.elem_state(fx["cap_U"][k])
            fext = external_load(fx, desc, k, eqn)
            assert relerr(resid, fext - fx["cap_B"][k]) < RTOL_STATE
            ref = csc_to_csr_values(fx, fx["cap_A"][k])
            assert relerr(vals, ref) < RTOL_STATE
            assert row_relerr(fx, vals, ref) < RTOL_STATE
        o.close()


FRAMES = ["frame2d_2x3", "frame3d_1x1x2", "frame3d_2x1x3", "frame2d_eq_2x3", "frame2d_pd_2x3",
          "frame2d_settle_2x3", "frame2d_s01_2x3", "frame2d_s01_eq_2x3",
          "frame2d_rc01_2x3"]


def test_uniaxial_paths():
    fx = load("uniaxial_paths")
    for kind in (1, 2, 4, 5):      # Steel02, Concrete02, Steel01, Concrete01
        s, t = port.uniaxial_path(kind, fx[f"k{kind}_param"], fx[f"k{kind}_strain"],
                                  fx[f"k{kind}_commit"])
        assert relerr(s, fx[f"k{kind}_stress"]) < RTOL_STATE
        assert relerr(t, fx[f"k{kind}_tangent"]) < RTOL_STATE


@pytest.mark.parametrize("name", FRAMES)
def test_frame_numbering_and_history(name):
    fx = load(name)
    desc, phases = model_of(fx)
    o = port.OracleModel(desc)
    assert np.array_equal(o.numbering(), fx["eqn"])
    rp, ci = o.pattern()
    assert np.array_equal(rp, fx["colstart"]) and np.array_equal(ci, fx["rowidx"])
    U, lam, its = o.run(phases)
    assert relerr(U, fx["step_u"]) < RTOL_HISTORY
    assert relerr(lam, fx["step_lambda"]) < RTOL_HISTORY
    assert np.array_equal(its, fx["step_iters"])


@pytest.mark.parametrize("name", ["frame2d_2x3", "frame3d_1x1x2", "frame2d_pd_2x3",
                                  "frame2d_settle_2x3", "frame2d_s01_2x3",
                                  "frame2d_rc01_2x3"])
def test_frame_replay_first_step(name):
    """Every Newton iteration of the first gravity step, replayed in order
    (the force-based element state is incremental, so the trial displacements
    are applied in the reference's sequence)."""
    fx = load(name)
    desc, phases = model_of(fx)
    o = port.OracleModel(desc)
    eqn = fx["eqn"]
    for k in range(len(fx["cap_step"])):
        vals, resid = o.elem_state(fx["cap_U"][k])
        fext = external_load(fx, desc, k, eqn)
        assert relerr(resid, fext - fx["cap_B"][k]) < RTOL_STATE
        ref = csc_to_csr_values(fx, fx["cap_A"][k])
        assert relerr(vals, ref) < RTOL_STATE
        assert row_relerr(fx, vals, ref) < RTOL_STATE


REVERTS = ["revert_frame2d_2x3", "revert_frame3d_1x1x2", "revert_quad_8x4"]


@pytest.mark.parametrize("name", REVERTS)
def test_revert_to_last_commit(name):
    """Element state at U + dU, then Domain::revertToLastCommit and the state
    at U + dU/2, against the reference's element responses."""
    fx = load(name)
    desc, phases = model_of(fx)
    rp, ci = fx["colstart"], fx["rowidx"]
    o = port.OracleModel(desc)
    U, _, _ = o.run(phases[:1])
    assert relerr(U[-1], fx["u"]) < RTOL_HISTORY
    u = fx["u"]
    for key, trial, revert in (("1", u + fx["du"], False), ("2", u + 0.5 * fx["du"], True)):
        if revert:
            o.revert()
        vals, resid = o.elem_state(trial)
        v_ref, r_ref = assemble_elements(desc, fx["eqn"], rp, ci, fx["K" + key], fx["P" + key])
        assert relerr(resid, r_ref) < RTOL_STATE, key
        assert relerr(vals, v_ref) < RTOL_STATE, key
        assert row_relerr(fx, vals, v_ref) < RTOL_STATE, key
    o.close()
