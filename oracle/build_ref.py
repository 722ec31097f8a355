#!/usr/bin/env python3
"""Build the reference's own CPU hot-path classes into ``oracle/_ref/libxara_ref.so``.

Test infrastructure only.  The reference sources are compiled unchanged where
they lie (``--src``, default ``/root/reference/SRC``); nothing is copied into
this repository.  The output goes to ``oracle/_ref/`` (git-ignored).

Link closure: the listed translation units reference many classes that the
hot path never executes (recorders, parameters, databases, Tcl glue).  After a
first link, every symbol that is still undefined and is not provided by the C
or C++ runtime gets a generated stub in ``_ref/stubs.c``: functions print their
mangled name and abort, data symbols are zero-filled blocks.  A stub that is
ever reached therefore fails loudly instead of giving a wrong answer.

Our own harness (``ref_harness.cpp``) builds models through the reference's C++
API (the pattern of ``tests/Other/UnitTests/Example1/main.cpp``) and exports a
small ``extern "C"`` surface for ctypes.

Usage: python oracle/build_ref.py [--src SRC] [-j N]   (SRC defaults to
$XARA_REFERENCE_SRC, else /root/reference/SRC)
"""
import argparse
import concurrent.futures as cf
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
DEFAULT_SRC = "/root/reference/SRC"


def source_dir():
    """The reference's SRC folder: $XARA_REFERENCE_SRC when set, else the
    default location of the read-only reference checkout."""
    return os.environ.get("XARA_REFERENCE_SRC") or DEFAULT_SRC

# Reference translation units (paths relative to SRC).
SOURCES = """
matrix/Matrix.cpp matrix/Vector.cpp matrix/ID.cpp
matrix/routines/invGL2.c matrix/routines/invGL3.c matrix/routines/invGL4.c
matrix/routines/invGL5.c matrix/routines/invGL6.c
tagged/TaggedObject.cpp tagged/storage/MapOfTaggedObjects.cpp
tagged/storage/MapOfTaggedObjectsIter.cpp tagged/storage/ArrayOfTaggedObjects.cpp
tagged/storage/ArrayOfTaggedObjectsIter.cpp
actor/actor/MovableObject.cpp
handler/OPS_Stream.cpp handler/StandardStream.cpp handler/DummyStream.cpp
handler/DataFileStream.cpp recorder/Recorder.cpp recorder/NodeRecorder.cpp
recorder/EnvelopeNodeRecorder.cpp
domain/domain/Domain.cpp domain/node/Node.cpp domain/node/NodalLoad.cpp
domain/component/DomainComponent.cpp domain/component/Parameter.cpp
domain/constraints/SP_Constraint.cpp domain/constraints/MP_Constraint.cpp
domain/load/Load.cpp element/ElementalLoad.cpp
domain/pattern/LoadPattern.cpp domain/pattern/LoadPatternIter.cpp
domain/pattern/series/TimeSeries.cpp domain/pattern/series/LinearSeries.cpp
domain/pattern/series/PathSeries.cpp domain/pattern/series/TimeSeriesIntegrator.cpp
domain/pattern/series/TrapezoidalTimeSeriesIntegrator.cpp
domain/pattern/UniformExcitation.cpp domain/pattern/EarthquakePattern.cpp
domain/groundMotion/GroundMotion.cpp
domain/domain/single/SingleDomEleIter.cpp domain/domain/single/SingleDomNodIter.cpp
domain/domain/single/SingleDomSP_Iter.cpp domain/domain/single/SingleDomMP_Iter.cpp
domain/domain/single/SingleDomAllSP_Iter.cpp domain/domain/single/SingleDomPC_Iter.cpp
domain/domain/single/SingleDomParamIter.cpp
domain/load/ElementalLoadIter.cpp
element/Element.cpp element/Information.cpp
recorder/response/Response.cpp recorder/response/ElementResponse.cpp
element/Plane/FourNodeQuad.cpp element/Brick/Brick.cpp interpolate/shp3d.cpp
element/Frame/Other/Force/ForceBeamColumn2d.cpp
element/Frame/Other/Force/ForceBeamColumn3d.cpp
material/nD/NDMaterial.cpp
material/uniaxial/UniaxialMaterial.cpp
material/plastic/J2Plasticity.cpp material/Plane/J2PlaneStrain.cpp
material/plastic/J2ThreeDimensional.cpp
material/uniaxial/steel/Steel02.cpp material/uniaxial/concrete/Concrete02.cpp
material/uniaxial/steel/Steel01.cpp material/uniaxial/concrete/Concrete01.cpp
material/uniaxial/ElasticMaterial.cpp
material/section/SectionForceDeformation.cpp
material/section/FiberSection2d.cpp material/section/FiberSection3d.cpp
quadrature/Frame/BeamIntegration.cpp quadrature/Frame/LobattoBeamIntegration.cpp
coordTransformation/CrdTransf.cpp coordTransformation/PDeltaCrdTransf2d.cpp
coordTransformation/LinearCrdTransf2d.cpp
coordTransformation/Frame/BasicFrameTransf.cpp
analysis/model/AnalysisModel.cpp analysis/model/FE_EleIter.cpp
analysis/model/DOF_GrpIter.cpp
analysis/fe_ele/FE_Element.cpp analysis/dof_grp/DOF_Group.cpp
analysis/handler/ConstraintHandler.cpp analysis/handler/PlainHandler.cpp
analysis/handler/TransformationConstraintHandler.cpp
analysis/fe_ele/transformation/TransformationFE.cpp
analysis/dof_grp/TransformationDOF_Group.cpp
analysis/numberer/DOF_Numberer.cpp
graph/numberer/GraphNumberer.cpp graph/numberer/RCM.cpp
graph/graph/Graph.cpp graph/graph/Vertex.cpp graph/graph/VertexIter.cpp
analysis/integrator/Integrator.cpp analysis/integrator/IncrementalIntegrator.cpp
analysis/integrator/StaticIntegrator.cpp analysis/integrator/TransientIntegrator.cpp
analysis/integrator/Static/LoadControl.cpp
analysis/integrator/Static/DisplacementControl.cpp
analysis/integrator/Dynamic/Newmark.cpp
analysis/algorithm/SolutionAlgorithm.cpp
analysis/algorithm/equiSolnAlgo/EquiSolnAlgo.cpp
analysis/algorithm/equiSolnAlgo/NewtonRaphson.cpp
analysis/criteria/ConvergenceTest.cpp analysis/criteria/CTestNormDispIncr.cpp
analysis/criteria/CTestNormUnbalance.cpp
system_of_eqn/linearSOE/LinearSOE.cpp system_of_eqn/linearSOE/LinearSOESolver.cpp
system_of_eqn/linearSOE/profileSPD/ProfileSPDLinSOE.cpp
system_of_eqn/linearSOE/profileSPD/ProfileSPDLinSolver.cpp
system_of_eqn/linearSOE/profileSPD/ProfileSPDLinDirectSolver.cpp
system_of_eqn/linearSOE/sparseGEN/SparseGenColLinSOE.cpp
system_of_eqn/linearSOE/sparseGEN/SparseGenColLinSolver.cpp
""".split()

HARNESS = ["ref_harness.cpp", "ref_blas.c"]


def sh(cmd, **kw):
    r = subprocess.run(cmd, capture_output=True, text=True, **kw)
    if r.returncode != 0:
        raise RuntimeError(f"command failed: {' '.join(cmd[:3])} ...\n{r.stderr[-3000:]}")
    return r


def include_flags(src):
    dirs = []
    for root, subdirs, _ in os.walk(src):
        if "/opensees" in root[len(src):]:
            continue
        dirs.append(root)
    dirs.sort()
    return ["-I" + d for d in dirs]


def compile_one(args):
    path, obj, incs, opt = args
    if os.path.exists(obj) and os.path.getmtime(obj) > os.path.getmtime(path):
        return obj, None
    if path.endswith(".c"):
        cmd = ["gcc", opt, "-fPIC", "-w", "-ffp-contract=off"] + incs + ["-c", path, "-o", obj]
    else:
        cmd = ["g++", "-std=c++17", "-fconcepts", opt, "-fPIC", "-w", "-ffp-contract=off"] + incs + ["-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return obj, r.stderr[-4000:]
    return obj, None


def runtime_symbols():
    """Symbols exported by libc, libm and libstdc++ (never stubbed)."""
    libs = []
    for name in ("libstdc++.so.6", "libm.so.6", "libc.so.6", "libgcc_s.so.1"):
        r = subprocess.run(["g++", "-print-file-name=" + name], capture_output=True, text=True)
        p = r.stdout.strip()
        if os.path.exists(p):
            libs.append(os.path.realpath(p))
    syms = set()
    for lib in libs:
        out = sh(["nm", "-D", "--defined-only", lib]).stdout
        for line in out.splitlines():
            parts = line.split()
            if len(parts) >= 3:
                syms.add(parts[2].split("@")[0])
    return syms


def undefined_in(objs):
    defined, undefined = set(), set()
    for o in objs:
        out = sh(["nm", o]).stdout
        for line in out.splitlines():
            parts = line.split()
            if len(parts) == 2 and parts[0] in ("U", "w"):
                if parts[0] == "U":
                    undefined.add(parts[1])
            elif len(parts) == 3 and parts[1] not in ("U", "w"):
                defined.add(parts[2])
    return undefined - defined


def classify(symbols):
    """Return {symbol: 'func'|'data'} using the demangled form."""
    syms = sorted(symbols)
    out = sh(["c++filt"], input="\n".join(syms)).stdout.splitlines()
    kinds = {}
    for s, d in zip(syms, out):
        if d.startswith(("vtable for", "typeinfo for", "typeinfo name for", "VTT for",
                         "construction vtable", "guard variable")):
            kinds[s] = "data"
        elif s.startswith("_Z"):
            kinds[s] = "func" if "(" in d else "data"
        else:
            kinds[s] = "func"
    return kinds


def write_stubs(kinds, path):
    lines = ["/* generated by build_ref.py: unreachable reference symbols */",
             "#include <stdio.h>", "#include <stdlib.h>"]
    for s, k in sorted(kinds.items()):
        if k == "func":
            lines.append(f'void {s}(void) {{ fprintf(stderr, "xara_ref stub reached: {s}\\n"); abort(); }}')
        else:
            lines.append(f"__attribute__((aligned(64))) char {s}[4096];")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--src", default=source_dir())
    ap.add_argument("-j", type=int, default=os.cpu_count() or 4)
    ap.add_argument("--opt", default="-O2")
    a = ap.parse_args()
    if not os.path.isdir(a.src):
        print(f"reference sources not found at {a.src}; oracle/_ref not built", file=sys.stderr)
        return 2
    objdir = os.path.join(OUT, "obj")
    os.makedirs(objdir, exist_ok=True)
    incs = include_flags(a.src)
    jobs = []
    for rel in SOURCES:
        path = os.path.join(a.src, rel)
        obj = os.path.join(objdir, rel.replace("/", "__") + ".o")
        jobs.append((path, obj, incs, a.opt))
    for rel in HARNESS:
        path = os.path.join(HERE, rel)
        obj = os.path.join(objdir, "harness__" + rel + ".o")
        jobs.append((path, obj, incs, a.opt))
    errors = []
    with cf.ThreadPoolExecutor(a.j) as ex:
        for obj, err in ex.map(compile_one, jobs):
            if err:
                errors.append((obj, err))
    if errors:
        for obj, err in errors:
            print("FAILED", obj, "\n", err, file=sys.stderr)
        return 1
    objs = [j[1] for j in jobs]
    undef = {u for u in undefined_in(objs) - runtime_symbols()
             if not u.startswith(("_GLOBAL_OFFSET_TABLE_", "__dso_handle", "__cxa_", "__gxx_"))}
    kinds = classify(undef)
    stub_c = os.path.join(OUT, "stubs.c")
    write_stubs(kinds, stub_c)
    stub_o = os.path.join(objdir, "stubs.o")
    sh(["gcc", "-O0", "-fPIC", "-w", "-c", stub_c, "-o", stub_o])
    lib = os.path.join(OUT, "libxara_ref.so")
    # link beside it, then rename: a process that has the old library loaded
    # keeps its mapping
    sh(["g++", "-shared", "-o", lib + ".tmp"] + objs + [stub_o, "-Wl,--no-undefined", "-lm"])
    os.replace(lib + ".tmp", lib)
    print(f"built {lib}: {len(objs)} objects, {len(kinds)} stubbed symbols")
    return 0


if __name__ == "__main__":
    sys.exit(main())
