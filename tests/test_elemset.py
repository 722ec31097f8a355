"""The element-set shim (include/CudaElementSet.h) inside the reference's
own analysis loop.

The shim is compiled against the reference's headers and claims the
elements of a Domain built by the reference harness (oracle/_ref): every
quad, brick or force-based frame element is replaced by a proxy, and the
reference's Domain::update / commit / revertToLastCommit reach the element
set once per call instead of once per element.  Behind the element-set C ABI
sits here the C oracle (tests/shim/oracle_elemset.c), so the whole loop runs
on the host: the reference's NewtonRaphson, integrators, DOF numbering and
ProfileSPD assemble the proxies' tangents and forces.  Checked: the claim's
refusals, the order of the forwarded calls, and the converged displacement
histories against the reference's own run (the fixtures), within 1e-12.
The same entry points on the device are covered by
tests/test_gpu_parity.py::test_element_matrices_match_the_oracle.
"""
import ctypes as C
import os
import subprocess
import sys

import numpy as np
import pytest

from golden_util import load, model_of, relerr

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import build_ref  # noqa: E402
import ref  # noqa: E402

MODELS = ["quad_8x4", "brick_4x3x2", "frame2d_2x3", "frame3d_1x1x2", "frame2d_pd_2x3",
          "frame2d_eq_2x3", "frame2d_rc01_2x3"]


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    if not (ref.available() and os.path.isdir(build_ref.source_dir())):
        pytest.skip("reference sources or oracle/_ref/libxara_ref.so absent")
    out_dir = tmp_path_factory.mktemp("elemset")
    out = str(out_dir / "libelemset_driver.so")
    objs = []
    for src in (os.path.join(ROOT, "oracle", "xara_oracle.c"),
                os.path.join(ROOT, "tests", "shim", "oracle_elemset.c")):
        obj = str(out_dir / (os.path.basename(src) + ".o"))
        r = subprocess.run(["gcc", "-O2", "-fPIC", "-std=c11", "-ffp-contract=off",
                            "-I" + os.path.join(ROOT, "include"), "-c", src, "-o", obj],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-3000:]
        objs.append(obj)
    refdir = os.path.dirname(ref.LIB)
    cmd = (["g++", "-std=c++17", "-fconcepts", "-O1", "-fPIC", "-shared", "-w",
            "-I" + os.path.join(ROOT, "include")]
           + build_ref.include_flags(build_ref.source_dir())
           + [os.path.join(ROOT, "tests", "shim", "elemset_driver.cpp")] + objs
           + ["-o", out, ref.LIB, "-lm", "-Wl,-rpath," + refdir])
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    ref.lib()
    D = C.CDLL(out)
    D.elemset_claim.argtypes = [C.c_void_p, C.c_void_p]
    D.elemset_counts.argtypes = [C.c_void_p] * 3
    D.elemset_class_of.argtypes = [C.c_void_p, C.c_int, C.c_char_p, C.c_int]
    D.oelem_log.restype = C.c_char_p
    return D


def run_claimed(D, desc, phases, claim_desc=None):
    """Run the phases through the reference's loop on the Domain built from
    desc, with the elements claimed by the shim for claim_desc (desc by
    default); returns (RefRun, claim status, call log)."""
    st = (claim_desc or desc).struct()
    status = {}
    D.oelem_log_reset()

    def attach(h):
        status["claim"] = D.elemset_claim(C.c_void_p(h), C.byref(st))
        status["class"] = C.create_string_buffer(64)
        D.elemset_class_of(C.c_void_p(h), int(desc.elem_tag[0]), status["class"], 64)

    run = ref.RefRun(desc, phases, attach=attach)
    return run, status, D.oelem_log().decode()


@pytest.mark.parametrize("name", MODELS)
def test_claimed_elements_reproduce_the_reference(driver, name):
    """The reference's loop on the proxies gives the reference's own
    converged displacements and load factors, step by step."""
    fx = load(name)
    desc, phases = model_of(fx)
    run, st, log = run_claimed(driver, desc, phases)
    assert st["claim"] == 0
    assert st["class"].value == b"CudaElementProxy"
    assert relerr(run.step_u, fx["step_u"]) < 1e-12
    assert relerr(run.step_lambda, fx["step_lambda"]) < 1e-12
    assert np.array_equal(run.step_iters, fx["step_iters"])
    # one device update per Domain::update (every update reads the element
    # matrices back), one commit per step, nothing per element
    u, c, r = C.c_long(), C.c_long(), C.c_long()
    driver.elemset_counts(C.byref(u), C.byref(c), C.byref(r))
    assert log.startswith("MTUK")
    assert log.count("TUK") == log.count("U") == u.value
    assert log.count("C") == c.value == len(fx["step_u"])
    assert log.count("R") == r.value == 0
    assert u.value < desc.num_elems * len(fx["step_u"])


def test_claim_refuses_a_description_that_differs(driver):
    """A node moved, an element on other nodes, or the wrong element class:
    the claim is refused and the Domain keeps its own elements."""
    from xara_gb300._abi import PhaseDesc
    fx = load("frame2d_2x3")
    desc, phases = model_of(fx)
    one = [PhaseDesc(**{**phases[0].kw, "num_steps": 1})]
    crd = np.asarray(desc.arrays["node_crd"]).copy()
    crd[-1] += 1e-3
    moved, _ = model_of(fx)
    moved.arrays["node_crd"] = crd
    _, st, _ = run_claimed(driver, desc, one, claim_desc=moved)
    assert st["claim"] == -2 and st["class"].value == b"ForceBeamColumn2d"
    conn = np.asarray(desc.arrays["elem_conn"]).copy()
    conn[[0, 1]] = conn[[1, 0]]
    swapped, _ = model_of(fx)
    swapped.arrays["elem_conn"] = conn
    _, st, _ = run_claimed(driver, desc, one, claim_desc=swapped)
    assert st["claim"] == -3 and st["class"].value == b"ForceBeamColumn2d"
