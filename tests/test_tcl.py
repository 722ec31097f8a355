"""The Tcl subset (xara_gb300.tcl): the reference's kind of model script --
variables, expr, loops, procs, section and pattern bodies -- builds the
same model description as the library's builder or the equivalent
OpenSeesPy-style calls (CPU), and (GPU) runs the same analysis."""
import numpy as np
import pytest

from xara_gb300 import configs
from xara_gb300 import openseespy as ops
from xara_gb300 import tcl

QUAD = """
wipe
model BasicBuilder -ndm 2 -ndf 2
set nx 8; set ny 4
# nodes row by row
for {set j 0} {$j <= $ny} {incr j} {
    for {set i 0} {$i <= $nx} {incr i} {
        node [expr $j*($nx+1) + $i + 1] [expr 1.0*$i] [expr 1.0*$j]
    }
}
nDMaterial J2Plasticity 1 %s
set t 1
for {set j 0} {$j < $ny} {incr j} {
    for {set i 0} {$i < $nx} {incr i} {
        set n1 [expr $j*($nx+1) + $i + 1]
        element quad $t $n1 [expr $n1+1] [expr $n1+$nx+2] [expr $n1+$nx+1] 1.0 PlaneStrain 1
        incr t
    }
}
for {set i 1} {$i <= $nx+1} {incr i} { fix $i 1 1 }
set master [expr $ny*($nx+1) + 1]
for {set i 1} {$i <= $nx} {incr i} { equalDOF $master [expr $master+$i] 2 }
pattern Plain 1 Linear {
    load $master 0.0 -1.0
}
constraints Plain
numberer RCM
system ProfileSPD
test NormDispIncr 1.0e-10 25
algorithm Newton
integrator DisplacementControl $master 2 [expr -0.005*$ny/4]
analysis Static
""" % " ".join(repr(v) for v in configs.J2_STEEL[:6])

FRAME = """
wipe
model basic -ndm 2 -ndf 3
proc column_line {x base} {
    node $base $x 0.0
    node [expr $base+1] $x 3.5
}
column_line 0.0 1
column_line 6.0 3
fix 1 1 1 1; fix 3 1 1 1
uniaxialMaterial Concrete02 1 -30e6 -0.002 -6e6 -0.006 0.1 3e6 1.5e9
uniaxialMaterial Steel02 2 420e6 200e9 0.01 18.0 0.925 0.15
section Fiber 1 {
    patch rect 1 8 1 -0.25 -0.2 0.25 0.2
    layer straight 2 3 491e-6 -0.2 0.15 -0.2 -0.15
    layer straight 2 3 491e-6 0.2 0.15 0.2 -0.15
}
geomTransf Linear 1
beamIntegration Lobatto 1 1 5
element forceBeamColumn 1 1 2 1 1
element forceBeamColumn 2 3 4 1 1
element forceBeamColumn 3 2 4 1 1
mass 2 1e4 1e4 0.0; mass 4 1e4 1e4 0.0
timeSeries Path 2 -dt 0.01 -values {0.0 0.5 1.0 0.5 0.0 -0.5 -1.0} -factor 9.81
pattern UniformExcitation 3 1 -accel 2
rayleigh 0.1 0.0 0.002 0.0
integrator Newmark 0.5 0.25
analysis Transient
"""


def _frame_python():
    ops.wipe()
    ops.model("basic", "-ndm", 2, "-ndf", 3)
    for base, x in ((1, 0.0), (3, 6.0)):
        ops.node(base, x, 0.0)
        ops.node(base + 1, x, 3.5)
    ops.fix(1, 1, 1, 1)
    ops.fix(3, 1, 1, 1)
    ops.uniaxialMaterial("Concrete02", 1, -30e6, -0.002, -6e6, -0.006, 0.1, 3e6, 1.5e9)
    ops.uniaxialMaterial("Steel02", 2, 420e6, 200e9, 0.01, 18.0, 0.925, 0.15)
    ops.section("Fiber", 1)
    ops.patch("rect", 1, 8, 1, -0.25, -0.2, 0.25, 0.2)
    ops.layer("straight", 2, 3, 491e-6, -0.2, 0.15, -0.2, -0.15)
    ops.layer("straight", 2, 3, 491e-6, 0.2, 0.15, 0.2, -0.15)
    ops.geomTransf("Linear", 1)
    ops.beamIntegration("Lobatto", 1, 1, 5)
    ops.element("forceBeamColumn", 1, 1, 2, 1, 1)
    ops.element("forceBeamColumn", 2, 3, 4, 1, 1)
    ops.element("forceBeamColumn", 3, 2, 4, 1, 1)
    ops.mass(2, 1e4, 1e4, 0.0)
    ops.mass(4, 1e4, 1e4, 0.0)
    ops.timeSeries("Path", 2, "-dt", 0.01, "-values", 0.0, 0.5, 1.0, 0.5, 0.0, -0.5, -1.0,
                   "-factor", 9.81)
    ops.pattern("UniformExcitation", 3, 1, "-accel", 2)
    ops.rayleigh(0.1, 0.0, 0.002, 0.0)
    ops.integrator("Newmark", 0.5, 0.25)
    ops.analysis("Transient")


def _same(a, b):
    for k, v in b.arrays.items():
        if v is None:
            assert a.arrays[k] is None, k
        else:
            np.testing.assert_array_equal(a.arrays[k], v, err_msg=k)


def test_quad_script_gives_the_builders_model():
    tcl.eval_script(QUAD, fresh=True)
    d, _ = configs.quad_block(8, 4, steps=4)
    _same(ops.build_desc(), d)
    ops.wipe()


def test_frame_script_matches_the_python_calls():
    tcl.eval_script(FRAME, fresh=True)
    d_tcl, ph_tcl = ops.build_desc(), ops._phase(7, 0.01)
    _frame_python()
    d_py, ph_py = ops.build_desc(), ops._phase(7, 0.01)
    _same(d_tcl, d_py)
    assert ph_tcl.keys() == ph_py.keys()
    for k in ph_py:
        np.testing.assert_array_equal(ph_tcl[k], ph_py[k], err_msg=k)
    assert len(d_py.fib_y) == 8 + 6 and np.isclose(d_py.fib_area[:8].sum(), 0.5 * 0.4)
    ops.wipe()


def test_tcl_language_pieces():
    it = tcl.Interp()
    assert it.eval("expr 7/2") == 3 and it.eval("expr 7.0/2") == 3.5
    assert it.eval("set x 4; expr {$x > 3 && !($x == 5) ? 10 : 20}") == 10
    assert it.eval("proc f {a {b 2}} { return [expr $a*$b] }; f 3") == 6
    it.eval("set s 0; foreach v {1 2 3 4} { if {$v == 3} continue; set s [expr $s+$v] }")
    assert it.eval("set s") == 7
    assert it.eval("set L [list a {b c} d]; llength $L") == 3
    assert it.eval('set n 5; set msg "n = $n"') == "n = 5"
    with pytest.raises(tcl.TclError, match="invalid command"):
        it.eval("no_such_command 1 2")


def test_one_line_bodies():
    tcl.eval_script("""wipe
model basic -ndm 2 -ndf 3
uniaxialMaterial Elastic 1 2.0e11
section Fiber 1 { fiber 0.1 0.0 0.01 1; fiber -0.1 0.0 0.01 1 }
timeSeries Linear 1
pattern Plain 1 1 { load 2 1.0 0.0 0.0 }
""", fresh=True)
    assert len(ops._S.sections[1]["fibers"]) == 2
    assert ops._S.patterns[0]["loads"] == [(2, [1.0, 0.0, 0.0])]
    ops.wipe()


@pytest.mark.gpu
def test_quad_script_runs_like_the_builders(need_gpu):
    from xara_gb300 import gpu
    tcl.eval_script(QUAD + "\nset ok [analyze 4]\n", fresh=True)
    assert tcl._INTERP.vars["ok"] == 0
    u = tcl.eval_script("nodeDisp 37 2")
    ops.wipe()
    desc, phases = configs.quad_block(8, 4, steps=4)
    with gpu.DeviceModel(desc) as m:
        U, _, _ = m.run(phases)
    i = list(desc.node_tag).index(37)
    assert u == U[-1, 2 * i + 1]
