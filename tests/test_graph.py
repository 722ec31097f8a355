"""Newmark steps of a batch of frames as CUDA graphs: the captured step
(predictor, conditional Newton loop with the device-side per-part
convergence check) against the host-driven step, bit for bit."""
import numpy as np
import pytest

from xara_gb300 import configs


@pytest.mark.gpu
def test_graph_steps_equal_host_steps(need_gpu):
    from xara_gb300 import gpu
    desc, phases = configs.frame_batch(6, steps=40, seed=3)
    runs = {}
    for graph in (False, True):
        with gpu.DeviceModel(desc) as m:
            m.set_system(gpu.XG_SYSTEM_PROFILE_SPD)
            gpu.set_graph(m, graph)
            U, lam, stats = m.run(phases)
            runs[graph] = (U, [s[0] for s in stats], gpu.graph_steps(m))
    assert runs[False][2] == 0 and runs[True][2] == 40
    np.testing.assert_array_equal(runs[True][0], runs[False][0])
    assert runs[True][1] == runs[False][1]


@pytest.mark.gpu
def test_graph_step_failure_reverts(need_gpu):
    """A step that cannot converge within max_iter fails, and the model keeps
    its last committed state, as in the host-driven loop."""
    from xara_gb300 import gpu
    from xara_gb300._abi import PhaseDesc
    desc, phases = configs.frame_batch(3, steps=10, seed=4)
    kw = dict(phases[0].kw)
    kw.update(num_steps=10, max_iter=1, tol=1e-300)
    ph = PhaseDesc(**kw, gm_accel=phases[0].gm_accel, gm_node_record=phases[0].gm_node_record,
                   alpha_m_node=phases[0].alpha_m_node,
                   beta_k_init_elem=phases[0].beta_k_init_elem)
    with gpu.DeviceModel(desc) as m:
        m.set_system(gpu.XG_SYSTEM_PROFILE_SPD)
        gpu.set_graph(m, True)
        m.set_phase(ph)
        u0, _ = m.disp()
        with pytest.raises(gpu.XaraGpuError):
            m.analyze(1)
        u1, _ = m.disp()
        assert gpu.graph_steps(m) == 1
    np.testing.assert_array_equal(u0, u1)
