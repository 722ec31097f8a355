"""The C-ABI library loads, exports every declared entry point, and its
host-side integer pipeline (DOF numbering, CSR pattern) is bit-exact against
the reference fixtures.  CPU only: no compute call needs a GPU here."""
import ctypes as C

import numpy as np
import pytest

from golden_util import load, model_of
from xara_gb300 import configs, gpu

MODELS = ["quad_8x4", "quad_64x16", "brick_4x3x2", "brick_8x8x4", "frame2d_2x3",
          "frame3d_1x1x2", "frame3d_2x1x3", "frame2d_settle_2x3"]


def test_exports_every_declared_symbol():
    L = gpu.lib()
    names = gpu.declared_symbols()
    assert "xg_model_create" in names and "xg_soe_solve" in names
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_version_and_error_text():
    L = gpu.lib()
    assert L.xg_version() >= 1
    h = C.c_void_p()
    assert L.xg_model_create(None, C.byref(h)) < 0
    assert b"null" in L.xg_last_error()


@pytest.mark.parametrize("name", MODELS)
def test_plan_bit_exact(name):
    fx = load(name)
    desc, _ = model_of(fx)
    eqn, rp, ci = gpu.plan(desc)
    assert np.array_equal(eqn, fx["eqn"])
    assert np.array_equal(rp, fx["colstart"])
    assert np.array_equal(ci, fx["rowidx"])


def test_plan_rejects_bad_models():
    desc, _ = configs.quad_block(4, 2)
    bad = desc.arrays["elem_conn"].copy()
    bad[0] = 10_000
    desc.arrays["elem_conn"] = bad
    with pytest.raises(gpu.XaraGpuError):
        gpu.plan(desc)
    desc, _ = configs.quad_block(4, 2)
    desc.arrays["node_tag"] = desc.arrays["node_tag"][::-1].copy()
    with pytest.raises(gpu.XaraGpuError):
        gpu.plan(desc)


def test_plan_disconnected_and_empty_rows():
    """Two separate blocks (a disconnected node graph) and an unattached node."""
    d1, _ = configs.quad_block(3, 2)
    d2, _ = configs.quad_block(2, 2)
    from xara_gb300._abi import ModelDesc, XG_ELE_QUAD
    off = 100
    crd = np.concatenate([d1.node_crd.reshape(-1, 2), d2.node_crd.reshape(-1, 2) + [10, 0],
                          [[50.0, 50.0]]])
    tags = np.concatenate([d1.node_tag, d2.node_tag + off, [999]])
    conn = np.concatenate([d1.elem_conn.reshape(-1, 4), d2.elem_conn.reshape(-1, 4) + off])
    desc = ModelDesc(ndm=2, ndf=2, elem_type=XG_ELE_QUAD, node_tag=tags, node_crd=crd,
                     elem_tag=np.arange(1, len(conn) + 1), elem_conn=conn,
                     elem_mat=np.zeros(len(conn)), j2_param=configs.J2_STEEL,
                     sp_node=[1, 1, 101, 101], sp_dof=[0, 1, 0, 1], sp_pattern=[-1] * 4,
                     sp_value=[0.0] * 4)
    eqn, rp, ci = gpu.plan(desc)
    neq = len(rp) - 1
    assert sorted(eqn[eqn >= 0]) == list(range(neq))
    assert np.all(np.diff(rp) >= 1)
    for r in range(neq):
        row = ci[rp[r]:rp[r + 1]]
        assert np.all(np.diff(row) > 0) and r in row
    # the oracle restatement numbers the same way
    from oracle import port
    o = port.OracleModel(desc)
    assert np.array_equal(o.numbering(), eqn)
    orp, oci = o.pattern()
    assert np.array_equal(orp, rp) and np.array_equal(oci, ci)


@pytest.mark.gpu
def test_chain_reciprocal_error_bound(need_gpu):
    """The LDL' pivot chains' reciprocal (single-precision seed, one cubic
    refinement step) against the correctly rounded __drcp_rn over a
    log-uniform sweep of both signs: within one unit in the last place, and
    equal to it outside 2^-100 .. 2^100 where it falls back to it."""
    L = gpu.lib()
    rng = np.random.default_rng(17)
    mag = np.exp2(rng.uniform(-110.0, 110.0, size=200_000))
    d = mag * np.where(rng.random(mag.size) < 0.5, -1.0, 1.0)
    d = np.concatenate([d, [1.0, -1.0, 3.0, 0.1, 2.0 ** -100, 2.0 ** 100, np.nextafter(2.0, 0)]])
    y, yrn = np.zeros_like(d), np.zeros_like(d)
    vp = C.c_void_p
    L.xg_chain_reciprocal_check.argtypes = [C.c_int, vp, vp, vp]
    assert L.xg_chain_reciprocal_check(d.size, d.ctypes.data_as(vp), y.ctypes.data_as(vp),
                                       yrn.ctypes.data_as(vp)) == 0
    assert np.array_equal(yrn, 1.0 / d)                 # __drcp_rn is the IEEE quotient
    ulps = np.abs(y - yrn) / np.spacing(np.abs(yrn))
    assert ulps.max() <= 1.0, ulps.max()
    outside = (np.abs(d) < 2.0 ** -100) | (np.abs(d) >= 2.0 ** 100)
    assert outside.sum() > 1000 and np.array_equal(y[outside], yrn[outside])
