"""The allocation-free solve (xg_pcg_solve_noalloc) against the allocating one.

Callers that cannot allocate device memory when they solve -- a framework
whose device memory belongs to its own pool, or a latency-bound loop that
cannot pay for cudaMalloc's device-wide synchronisation -- use
xg_pcg_solve_noalloc, which keeps its scratch in a fixed device array.  This
test hands it device arrays that PyTorch allocated (the caller's memory),
calls it twice in a row, and checks both solutions against xg_soe_solve on
the same system, within the tolerance the other PCG tests use.  The file is
named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL_SOLVE = 1e-9     # same bound as test_gpu_parity.test_pcg_against_dense_solve


def _node_blocks(desc, eqn):
    """Diagonal blocks of the library's preconditioner: the equations each
    node numbered for itself (equalDOF-constrained dofs belong to the
    retained node's block), in equation order."""
    nn, ndf = desc.num_nodes, desc.ndf
    own = eqn.reshape(nn, ndf).copy()
    if desc.mp_constrained is not None:
        for c, dof in zip(desc.mp_constrained, desc.mp_dof):
            own[np.searchsorted(desc.node_tag, c), dof] = -1
    starts = sorted(int(r[r >= 0].min()) for r in own if np.any(r >= 0))
    return np.asarray(starts + [int(eqn.max()) + 1], np.int32)


def test_noalloc_solve_matches_soe_solve(need_gpu):
    import torch
    from xara_gb300 import configs, gpu

    L = gpu.lib()
    L.xg_pcg_solve_noalloc.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                       C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_int,
                                       C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double)]
    desc, _ = configs.quad_block(64, 16)
    with gpu.DeviceModel(desc) as m:
        m.set_system(gpu.XG_SYSTEM_BJPCG)
        u = np.zeros(m.nu)
        u[1::2] = -1e-4 * desc.node_crd.reshape(-1, 2)[:, 1]     # a uniform compression
        m.set_trial_disp(u)
        vals, _, _ = m.update()
        rowptr, colidx = m.pattern()
        blk = _node_blocks(desc, m.numbering())
        assert np.all(np.diff(blk) >= 1) and np.all(np.diff(blk) <= 6)
        rng = np.random.default_rng(11)
        rhs = [rng.normal(size=m.neq), rng.normal(size=m.neq)]
        expect = [m.solve(b, rtol=1e-12)[0] for b in rhs]

    dev = torch.device("cuda")
    d_rowptr = torch.from_numpy(rowptr).to(dev)
    d_colidx = torch.from_numpy(colidx).to(dev)
    d_vals = torch.from_numpy(vals).to(dev)
    d_blk = torch.from_numpy(blk).to(dev)
    n, nblk = len(rowptr) - 1, len(blk) - 1
    ptr = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    for b, x_ref in zip(rhs, expect):          # two calls in a row
        d_b = torch.from_numpy(b).to(dev)
        d_x = torch.full((n,), float("nan"), dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        it, rr = C.c_int(), C.c_double()
        r = L.xg_pcg_solve_noalloc(n, ptr(d_rowptr), ptr(d_colidx), ptr(d_vals), nblk,
                                   ptr(d_blk), ptr(d_b), ptr(d_x), 1e-12, 20000, None,
                                   C.byref(it), C.byref(rr))
        assert r == 0, L.xg_last_error()
        x = d_x.cpu().numpy()
        assert rr.value <= 1e-12 and it.value > 0
        err = np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref)
        assert err < RTOL_SOLVE, err

    # a system beyond the fixed scratch is refused before any device access
    it, rr = C.c_int(), C.c_double()
    r = L.xg_pcg_solve_noalloc(5_000_000, ptr(d_rowptr), ptr(d_colidx), ptr(d_vals),
                               5_000_000, ptr(d_blk), ptr(d_b), ptr(d_x), 1e-12, 100, None,
                               C.byref(it), C.byref(rr))
    assert r < 0 and b"scratch" in L.xg_last_error()
