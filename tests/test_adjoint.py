"""Adjoint of a Newmark run of force-based frames.

CPU: the material point's vector-Jacobian product (the library's host entry)
against central finite differences of the oracle's Steel02 on every branch
(first loading, same branch, reversals with and without a new extreme
strain, zero increments, isotropic shift).  GPU: gradients of the roof-drift
objective with respect to per-member Steel02 parameters against central
finite differences of the device forward run (2D steel and RC frames, 2D
frames under P-Delta, a 3D RC frame), and the checkpoint interval changing
nothing.
"""
import numpy as np
import pytest

from oracle import port
from xara_gb300 import configs
from xara_gb300._abi import (XG_UNI_CONCRETE01, XG_UNI_CONCRETE02, XG_UNI_ELASTIC,
                             XG_UNI_STEEL01, XG_UNI_STEEL02)

FIELDS = (0, 1, 2, 3, 4, 5, 6, 9, 10)            # continuous record fields


def _gpu():
    from xara_gb300 import gpu
    return gpu


def _path_states(q, strains):
    """(committed record, trial strain) at every point of a committed path."""
    hc = port.uniaxial_init(XG_UNI_STEEL02, q)
    out = []
    for e in strains:
        out.append((hc.copy(), float(e)))
        hc = port.uniaxial_trial(XG_UNI_STEEL02, q, hc, e)
    return out


def _scales(q):
    ey = q[0] / q[1]
    s = np.full(12, ey)
    s[4] = s[6] = s[9] = q[0]
    return s


def _fd_check(q, hc, eps, rng, rel=1e-7):
    gpu = _gpu()
    sc = _scales(q)
    yb = np.zeros(12)
    yb[list(FIELDS)] = rng.normal(size=len(FIELDS)) / sc[list(FIELDS)]
    hb, sb, qb = gpu.uniaxial_vjp(XG_UNI_STEEL02, q, hc, eps, yb)

    def J(hc_, eps_, q_):
        return float(yb @ port.uniaxial_trial(XG_UNI_STEEL02, q_, hc_, eps_))

    checks = []
    h = rel * sc[10]
    checks.append(("strain", sb, (J(hc, eps + h, q) - J(hc, eps - h, q)) / (2 * h), sc[10]))
    # on the first loading branch epspl == epss0 and the law's R has a kink
    # in epspl - epss0: there the two move together (both are +-Fy/E0), so
    # only their sum is checked
    kink = int(hc[7]) in (1, 2) and hc[2] == hc[3]
    groups = [(f,) for f in FIELDS if not (kink and f in (2, 3))]
    if kink:
        groups.append((2, 3))
    for g in groups:
        h = rel * sc[g[0]]
        hp, hm = hc.copy(), hc.copy()
        hp[list(g)] += h
        hm[list(g)] -= h
        checks.append((f"record{g}", sum(hb[f] for f in g),
                       (J(hp, eps, q) - J(hm, eps, q)) / (2 * h), sc[g[0]]))
    for k, s in enumerate((q[0], q[1], q[2])):
        h = rel * s
        qp, qm = q.copy(), q.copy()
        qp[k] += h
        qm[k] -= h
        checks.append((f"param[{k}]", qb[k], (J(hc, eps, qp) - J(hc, eps, qm)) / (2 * h), s))
    total = sum(abs(a) * s for _, a, _, s in checks) + 1e-12
    for name, a, b, s in checks:
        assert abs(a - b) * s <= 2e-6 * total, (name, a, b)


@pytest.mark.parametrize("shift", [False, True])
def test_steel02_vjp_against_finite_differences(shift):
    q = configs.steel02_row(fy=350e6, E=200e9, b=0.015, R0=18.0)
    if shift:                                    # Filippou isotropic shift a1..a4
        q[6:10] = [0.04, 1.0, 0.04, 1.0]
    ey = q[0] / q[1]
    t = np.linspace(0.0, 6.0 * np.pi, 240)
    strains = ey * (0.5 + 0.05 * t) * np.sin(t) * 3.0
    rng = np.random.default_rng(3)
    states = _path_states(q, strains)
    kinds = set()
    for hc, eps in states[1:]:
        deps = eps - hc[10]
        if abs(deps) < 1e-4 * ey:
            continue                             # too close to a branch switch for FD
        kon = int(hc[7])
        kinds.add((kon, deps > 0))
        _fd_check(q, hc, eps, rng)
    # every branch of the law was visited: first loading from kon 0, same
    # branch and reversal from kon 1 and 2
    assert {(1, True), (1, False), (2, True), (2, False)} <= kinds
    # first loading from the fresh record, both directions
    for e in (0.3 * ey, -0.7 * ey, 2.5 * ey):
        _fd_check(q, port.uniaxial_init(XG_UNI_STEEL02, q), e, rng)


@pytest.mark.parametrize("shift", [False, True])
def test_steel02_jvp_against_the_vjp_and_finite_differences(shift):
    """Steel02 in forward mode (the DDM's law, written step by step from the
    primal) along the VJP test's path: equal to the reverse mode through
    y.(Jt) = (J'y).t at every point, and to central differences of the
    oracle's law in random directions of (strain, record, parameters) --
    where the record sits on a first-loading branch (epspl = epss0, the kink
    of R in their difference) the two move together."""
    gpu = _gpu()
    q = configs.steel02_row(fy=350e6, E=200e9, b=0.015, R0=18.0)
    if shift:
        q[6:10] = [0.04, 1.0, 0.04, 1.0]
    ey = q[0] / q[1]
    t = np.linspace(0.0, 6.0 * np.pi, 240)
    strains = ey * (0.5 + 0.05 * t) * np.sin(t) * 3.0
    rng = np.random.default_rng(17)
    sc = _scales(q)
    fields = list(FIELDS)
    checked = 0
    for hc, eps in _path_states(q, strains)[1:]:
        de = rng.normal() * ey
        dhc = np.zeros(12)
        dhc[fields] = rng.normal(size=len(fields)) * sc[fields]
        if int(hc[7]) in (1, 2) and hc[2] == hc[3]:
            dhc[3] = dhc[2]
        dq = rng.normal(size=3) * q[:3]
        dht = gpu.uniaxial_jvp(XG_UNI_STEEL02, q, hc, eps, de, dhc, dq)
        yb = np.zeros(12)
        yb[fields] = rng.normal(size=len(fields)) / sc[fields]
        hb, sb, qb = gpu.uniaxial_vjp(XG_UNI_STEEL02, q, hc, eps, yb)
        terms = [sb * de, *(hb[f] * dhc[f] for f in fields), *(qb * dq)]
        assert abs(float(yb @ dht) - sum(terms)) <= 1e-11 * sum(abs(x) for x in terms), eps
        if abs(eps - hc[10]) < 1e-4 * ey:
            continue
        rel = 1e-7
        hp, hm = hc + rel * dhc, hc - rel * dhc
        hp[7] = hm[7] = hc[7]
        qp, qm = q.copy(), q.copy()
        qp[:3] += rel * dq
        qm[:3] -= rel * dq
        qp[11] = qp[0] / qp[1]
        qm[11] = qm[0] / qm[1]
        fd = (port.uniaxial_trial(XG_UNI_STEEL02, qp, hp, eps + rel * de) -
              port.uniaxial_trial(XG_UNI_STEEL02, qm, hm, eps - rel * de)) / (2 * rel)
        for f in (0, 1, 2, 3, 4, 5, 6, 9, 10):
            assert abs(dht[f] - fd[f]) <= 1e-7 * sc[f], (eps, f, dht[f], fd[f])
        checked += 1
    assert checked > 200


def test_steel02_vjp_zero_increment_and_elastic():
    gpu = _gpu()
    q = configs.steel02_row()
    hc = port.uniaxial_init(XG_UNI_STEEL02, q)
    yb = np.arange(12, dtype=float)
    hb, sb, qb = gpu.uniaxial_vjp(XG_UNI_STEEL02, q, hc, 0.0, yb)
    assert np.array_equal(hb[:7], yb[:7]) and sb == yb[10] and not qb.any()
    qe = np.zeros(12)
    qe[0] = 2.0e11
    hb, sb, qb = gpu.uniaxial_vjp(XG_UNI_ELASTIC, qe, np.zeros(12), 1e-3, yb)
    assert sb == pytest.approx(2.0e11 * yb[9] + yb[10]) and qb[0] == pytest.approx(1e-3 * yb[9])
    with pytest.raises(gpu.XaraGpuError):
        q2 = q.copy()
        q2[10] = 1e6                             # initial stress: not covered
        gpu.uniaxial_vjp(XG_UNI_STEEL02, q2, hc, 1e-3, yb)


S01_FIELDS = (0, 1, 2, 3, 9, 10)     # minStrain, maxStrain, shiftP, shiftN, sig, eps


@pytest.mark.parametrize("shift", [False, True])
def test_steel01_vjp_against_finite_differences(shift):
    """Steel01's vector-Jacobian product (the library's host entry) against
    central differences of the oracle's law, along a cyclic path of growing
    amplitude: the elastic predictor, both hardening bounds, reversals with
    and without a new extreme strain, with and without the isotropic shifts."""
    gpu = _gpu()
    q = configs.steel01_row(350e6, 200e9, 0.015, *((0.04, 1.0, 0.03, 1.5) if shift
                                                    else (0.0, 1.0, 0.0, 1.0)))
    ey = q[0] / q[1]
    t = np.linspace(0.0, 6.0 * np.pi, 240)
    strains = ey * (0.5 + 0.05 * t) * np.sin(t) * 3.0
    rng = np.random.default_rng(5)
    sc = np.full(12, ey)
    sc[2] = sc[3] = 1.0
    sc[9] = q[0]
    hc = port.uniaxial_init(XG_UNI_STEEL01, q)
    branches = set()
    checked = 0
    for e in strains:
        deps = e - hc[10]
        ht = port.uniaxial_trial(XG_UNI_STEEL01, q, hc, float(e))
        if abs(deps) > 1e-4 * ey and abs(abs(ht[9]) - abs(hc[9] + q[1] * deps)) > 1e-6 * q[0]:
            branches.add("bound")
        elif abs(deps) > 1e-4 * ey:
            branches.add("elastic")
        if abs(deps) > 1e-4 * ey and int(hc[4]) * deps < 0:
            branches.add("reversal")
        yb = np.zeros(12)
        yb[list(S01_FIELDS)] = rng.normal(size=len(S01_FIELDS)) / sc[list(S01_FIELDS)]
        hb, sb, qb = gpu.uniaxial_vjp(XG_UNI_STEEL01, q, hc, float(e), yb)

        def J(hc_, eps_, q_):
            return float(yb @ port.uniaxial_trial(XG_UNI_STEEL01, q_, hc_, eps_))

        rel = 1e-7
        checks = [("strain", sb, (J(hc, e + rel * ey, q) - J(hc, e - rel * ey, q)) /
                   (2 * rel * ey), ey)]
        for f in S01_FIELDS:
            hp, hm = hc.copy(), hc.copy()
            hp[f] += rel * sc[f]
            hm[f] -= rel * sc[f]
            checks.append((f"record[{f}]", hb[f], (J(hp, e, q) - J(hm, e, q)) /
                           (2 * rel * sc[f]), sc[f]))
        for k in range(3):
            qp, qm = q.copy(), q.copy()
            qp[k] += rel * q[k]
            qm[k] -= rel * q[k]
            checks.append((f"param[{k}]", qb[k], (J(hc, e, qp) - J(hc, e, qm)) / (2 * rel * q[k]),
                           q[k]))
        total = sum(abs(a) * s_ for _, a, _, s_ in checks) + 1e-12
        # the kinks of the law: the elastic predictor at a hardening bound
        c = hc[9] + q[1] * deps
        c1, fyomb = q[2] * q[1] * e, q[0] * (1 - q[2])
        kink = min(abs(c - (c1 + hc[2] * fyomb)), abs(c - (c1 - hc[3] * fyomb))) < 1e-3 * q[0]
        if abs(deps) > 1e-4 * ey and not kink:
            for name, a, b, s_ in checks:
                assert abs(a - b) * s_ <= 2e-6 * total, (name, a, b)
            checked += 1
        hc = ht
    assert {"bound", "elastic", "reversal"} <= branches
    assert checked > 200


@pytest.mark.parametrize("shift", [False, True])
def test_steel01_jvp_against_finite_differences_and_the_vjp(shift):
    """Steel01's Jacobian-vector product (the DDM's law in forward mode)
    along the cyclic path of the VJP test: against central differences of the
    oracle's law in a random direction of (strain, record, parameters), and
    equal to the vector-Jacobian product through y . (J t) = (J' y) . t."""
    gpu = _gpu()
    q = configs.steel01_row(350e6, 200e9, 0.015, *((0.04, 1.0, 0.03, 1.5) if shift
                                                    else (0.0, 1.0, 0.0, 1.0)))
    ey = q[0] / q[1]
    t = np.linspace(0.0, 6.0 * np.pi, 240)
    strains = ey * (0.5 + 0.05 * t) * np.sin(t) * 3.0
    rng = np.random.default_rng(7)
    sc = np.full(12, ey)
    sc[2] = sc[3] = 1.0
    sc[9] = q[0]
    hc = port.uniaxial_init(XG_UNI_STEEL01, q)
    checked = 0
    for e in strains:
        deps = e - hc[10]
        ht = port.uniaxial_trial(XG_UNI_STEEL01, q, hc, float(e))
        de = rng.normal() * ey
        dhc = np.zeros(12)
        dhc[list(S01_FIELDS)] = rng.normal(size=len(S01_FIELDS)) * sc[list(S01_FIELDS)]
        dq = rng.normal(size=3) * q[:3]
        dht = gpu.uniaxial_jvp(XG_UNI_STEEL01, q, hc, float(e), de, dhc, dq)
        # forward against reverse mode: exact up to rounding
        yb = np.zeros(12)
        yb[list(S01_FIELDS)] = rng.normal(size=len(S01_FIELDS)) / sc[list(S01_FIELDS)]
        hb, sb, qb = gpu.uniaxial_vjp(XG_UNI_STEEL01, q, hc, float(e), yb)
        lhs = float(yb @ dht)
        terms = [sb * de, *(hb[f] * dhc[f] for f in S01_FIELDS), *(qb * dq)]
        rhs = float(sum(terms))
        assert abs(lhs - rhs) <= 1e-12 * sum(abs(x) for x in terms) + 1e-300, (e, lhs, rhs)
        # against central differences, away from the law's kinks
        rel = 1e-7
        hp, hm = hc + rel * dhc, hc - rel * dhc
        hp[4] = hm[4] = hc[4]
        qp, qm = q.copy(), q.copy()
        qp[:3] += rel * dq
        qm[:3] -= rel * dq
        fd = (port.uniaxial_trial(XG_UNI_STEEL01, qp, hp, float(e + rel * de)) -
              port.uniaxial_trial(XG_UNI_STEEL01, qm, hm, float(e - rel * de))) / (2 * rel)
        c = hc[9] + q[1] * deps
        c1, fyomb = q[2] * q[1] * e, q[0] * (1 - q[2])
        kink = min(abs(c - (c1 + hc[2] * fyomb)), abs(c - (c1 - hc[3] * fyomb))) < 1e-3 * q[0]
        if abs(deps) > 1e-4 * ey and not kink:
            for f in S01_FIELDS:
                assert abs(dht[f] - fd[f]) <= 1e-7 * sc[f], (f, dht[f], fd[f])
            checked += 1
        hc = ht
    assert checked > 200
    # the elastic law and a refused case
    de, dq = 1e-4, np.array([2e9, 0.0, 0.0])
    dht = gpu.uniaxial_jvp(XG_UNI_ELASTIC, np.r_[200e9, np.zeros(11)], np.zeros(12), 1e-3, de,
                           np.zeros(12), dq)
    assert dht[9] == pytest.approx(2e9 * 1e-3 + 200e9 * 1e-4) and dht[10] == de
    q2 = configs.steel02_row()
    q2[10] = 1e6                                 # Steel02 initial stress: not covered
    with pytest.raises(_gpu().XaraGpuError):
        gpu.uniaxial_jvp(XG_UNI_STEEL02, q2, np.zeros(12), 1e-3, de, np.zeros(12), dq)


C01_FIELDS = (0, 1, 2, 9, 10)          # minStrain, endStrain, unloadSlope, sig, eps


def test_concrete01_derivatives_against_finite_differences():
    """Concrete01 in forward mode (the DDM's law) against central differences
    of the oracle's law in random directions of (strain, record, fpc, epsc0,
    fpcu), along a compression path of growing amplitude with excursions
    into tension: the parabola, the linear descent and the crushed plateau
    of the envelope, unloading, reloading, the return line and tension; the
    reverse mode (the adjoint's) equal to it through y.(Jt) = (J'y).t.
    Finite differences skip the points where the return line and the
    reloading line coincide (the committed point lies on the unloading line
    and the law takes the larger of two equal stresses) and strains at the
    committed one (the law keeps the committed state there)."""
    gpu = _gpu()
    q = configs.concrete01_row(30e6)
    e0 = 0.002
    t = np.linspace(0.0, 8.0 * np.pi, 400)
    strains = -e0 * (0.2 + 0.5 * t / np.pi) * np.abs(np.sin(t)) * 1.2 + 0.0004 * np.sin(3 * t)
    rng = np.random.default_rng(3)
    sc = np.zeros(12)
    sc[[0, 1, 10]] = e0
    sc[2] = 15e9
    sc[9] = 30e6
    hc = port.uniaxial_init(XG_UNI_CONCRETE01, q)
    labels, checked = set(), 0
    for e in strains:
        e = float(e)
        ht = port.uniaxial_trial(XG_UNI_CONCRETE01, q, hc, e)
        de = rng.normal() * e0
        dhc = np.zeros(12)
        dhc[list(C01_FIELDS)] = rng.normal(size=len(C01_FIELDS)) * sc[list(C01_FIELDS)]
        dq = rng.normal(size=3) * np.abs(q[:3])
        dht = gpu.uniaxial_jvp(XG_UNI_CONCRETE01, q, hc, e, de, dhc, dq)
        yb = np.zeros(12)
        yb[list(C01_FIELDS)] = rng.normal(size=len(C01_FIELDS)) / sc[list(C01_FIELDS)]
        hb, sb, qb = gpu.uniaxial_vjp(XG_UNI_CONCRETE01, q, hc, e, yb)
        terms = [sb * de, *(hb[f] * dhc[f] for f in C01_FIELDS), *(qb * dq)]
        assert abs(float(yb @ dht) - sum(terms)) <= 1e-12 * sum(abs(x) for x in terms) + 1e-300
        # branch labels and the coincident-lines kink
        temp = hc[9] + hc[2] * (e - hc[10])
        kink = False
        if e > 0:
            labels.add("tension")
        elif e <= hc[10] and e <= hc[0]:
            labels.add("parabola" if e > -e0 else "descent" if e > -0.006 else "crushed")
        elif e <= hc[10] and e <= hc[1]:
            labels.add("reload")
            kink = abs(temp - hc[2] * (e - hc[1])) < 1e-6 * 30e6
        elif e > hc[10] and temp <= 0:
            labels.add("return")
        rel = 1e-7
        qp, qm = q.copy(), q.copy()
        qp[:3] += rel * dq
        qm[:3] -= rel * dq
        fd = (port.uniaxial_trial(XG_UNI_CONCRETE01, qp, hc + rel * dhc, e + rel * de) -
              port.uniaxial_trial(XG_UNI_CONCRETE01, qm, hc - rel * dhc, e - rel * de)) / (2 * rel)
        if not kink and abs(e - hc[10]) > 1e-4 * e0:
            for f in C01_FIELDS:
                assert abs(dht[f] - fd[f]) <= 1e-7 * sc[f], (e, f, dht[f], fd[f])
            checked += 1
        hc = ht
    assert {"tension", "parabola", "descent", "crushed", "reload", "return"} <= labels, labels
    assert checked > 300


C02_FIELDS = (0, 1, 9, 10)                       # ecmin, dept, sig, eps


def _c02_branch(q, hc, eps):
    """Which piece of Concrete02's law a trial strain lands on (a label;
    finite differences are taken only where every perturbation stays on
    it)."""
    fc, e0, fcu, ecu = (-abs(v) for v in q[:4])
    rat, ft, Ets = q[4], q[5], q[6]

    def compr(x):
        if x >= e0:
            return "c0", fc * (x / e0) * (2 - x / e0)
        if x > ecu:
            return "c1", (fcu - fc) * (x - e0) / (ecu - e0) + fc
        return "c2", fcu

    def tens(x):
        Ec0 = 2 * fc / e0
        if x <= ft / Ec0:
            return "t0"
        return "t1" if x <= ft * (1 / Ets + 1 / Ec0) else "t2"

    if abs(eps - hc[10]) < np.finfo(float).eps:
        return "zero"
    if eps < hc[0]:
        return "env-" + compr(eps)[0]
    ec0 = 2 * fc / e0
    epsr = (fcu - rat * ec0 * ecu) / (ec0 * (1 - rat))
    _, sigmm = compr(hc[0])
    er = (sigmm - ec0 * epsr) / (hc[0] - epsr)
    ept = hc[0] - sigmm / er
    if eps <= ept:
        sig = hc[9] + ec0 * (eps - hc[10])
        which = "elastic"
        if sig <= sigmm + er * (eps - hc[0]):
            sig, which = sigmm + er * (eps - hc[0]), "lower"
        if sig >= er * 0.5 * (eps - ept):
            which = "upper"
        return "unload-" + which
    if eps <= ept + hc[1]:
        return "reload-" + tens(hc[1])
    return "tension-" + tens(eps - ept)


def _c02_fd_check(q, hc, eps, rng, rel=1e-7):
    gpu = _gpu()
    sc = np.full(12, abs(q[1]))
    sc[9] = abs(q[0])
    yb = np.zeros(12)
    yb[list(C02_FIELDS)] = rng.normal(size=len(C02_FIELDS)) / sc[list(C02_FIELDS)]
    hb, sb, qb = gpu.uniaxial_vjp(XG_UNI_CONCRETE02, q, hc, eps, yb)
    label = _c02_branch(q, hc, eps)

    def J(hc_, eps_, q_):
        return float(yb @ port.uniaxial_trial(XG_UNI_CONCRETE02, q_, hc_, eps_))

    checks = []
    h = rel * sc[10]
    if _c02_branch(q, hc, eps + h) == label == _c02_branch(q, hc, eps - h):
        checks.append(("strain", sb, (J(hc, eps + h, q) - J(hc, eps - h, q)) / (2 * h), sc[10]))
    for f in C02_FIELDS:
        h = rel * sc[f]
        hp, hm = hc.copy(), hc.copy()
        hp[f] += h
        hm[f] -= h
        if _c02_branch(q, hp, eps) == label == _c02_branch(q, hm, eps):
            checks.append((f"record{f}", hb[f], (J(hp, eps, q) - J(hm, eps, q)) / (2 * h), sc[f]))
    for k in range(3):
        h = rel * abs(q[k])
        qp, qm = q.copy(), q.copy()
        qp[k] += h
        qm[k] -= h
        if _c02_branch(qp, hc, eps) == label == _c02_branch(qm, hc, eps):
            checks.append((f"param[{k}]", qb[k], (J(hc, eps, qp) - J(hc, eps, qm)) / (2 * h),
                           abs(q[k])))
    total = sum(abs(a) * s for _, a, _, s in checks) + 1e-30
    for name, a, b, s in checks:
        assert abs(a - b) * s <= 2e-6 * total, (label, name, a, b)
    return label


def test_concrete02_vjp_against_finite_differences():
    """Concrete02's vector-Jacobian product against central differences of
    the oracle's law along a path through every piece of it: the compression
    envelope's three regions, unloading (elastic step, lower and upper
    bound), reloading towards the tension point and along the tension
    envelope and its softening branch."""
    q = configs.concrete02_row(fc=30e6)
    segs = [np.linspace(0, -0.003, 25), np.linspace(-0.003, -0.0012, 12),
            np.linspace(-0.0012, -0.0045, 20), np.linspace(-0.0045, 0.0004, 40),
            np.linspace(0.0004, -0.0005, 12), np.linspace(-0.0005, 0.0012, 25),
            np.linspace(0.0012, -0.0075, 50), np.linspace(-0.0075, -0.004, 10)]
    strains = np.concatenate(segs)
    hc = port.uniaxial_init(XG_UNI_CONCRETE02, q)
    rng = np.random.default_rng(7)
    labels = set()
    for e in strains[1:]:
        if abs(e - hc[10]) > 1e-9:
            labels.add(_c02_fd_check(q, hc, float(e), rng))
        hc = port.uniaxial_trial(XG_UNI_CONCRETE02, q, hc, float(e))
    need = {"env-c0", "env-c1", "env-c2", "unload-elastic", "unload-lower", "unload-upper",
            "tension-t0", "tension-t1"}
    assert need <= labels, labels


def test_concrete02_jvp_against_the_vjp_and_finite_differences():
    """Concrete02 in forward mode (the DDM's law) along the VJP test's path:
    equal to the reverse mode through y.(Jt) = (J'y).t at every point, and to
    central differences of the oracle's law in random directions of
    (strain, ecmin, dept, stress, strain, fc, epsc0, fcu) wherever the
    perturbed inputs stay on the same piece of the law."""
    gpu = _gpu()
    q = configs.concrete02_row(fc=30e6)
    segs = [np.linspace(0, -0.003, 25), np.linspace(-0.003, -0.0012, 12),
            np.linspace(-0.0012, -0.0045, 20), np.linspace(-0.0045, 0.0004, 40),
            np.linspace(0.0004, -0.0005, 12), np.linspace(-0.0005, 0.0012, 25),
            np.linspace(0.0012, -0.0075, 50), np.linspace(-0.0075, -0.004, 10)]
    strains = np.concatenate(segs)
    hc = port.uniaxial_init(XG_UNI_CONCRETE02, q)
    rng = np.random.default_rng(41)
    sc = np.full(12, abs(q[1]))
    sc[9] = abs(q[0])
    fields = list(C02_FIELDS)
    labels = set()
    for e in strains[1:]:
        e = float(e)
        de = rng.normal() * abs(q[1])
        dhc = np.zeros(12)
        dhc[fields] = rng.normal(size=len(fields)) * sc[fields]
        dq = rng.normal(size=3) * np.abs(q[:3])
        dht = gpu.uniaxial_jvp(XG_UNI_CONCRETE02, q, hc, e, de, dhc, dq)
        yb = np.zeros(12)
        yb[fields] = rng.normal(size=len(fields)) / sc[fields]
        hb, sb, qb = gpu.uniaxial_vjp(XG_UNI_CONCRETE02, q, hc, e, yb)
        terms = [sb * de, *(hb[f] * dhc[f] for f in fields), *(qb * dq)]
        assert abs(float(yb @ dht) - sum(terms)) <= 1e-11 * sum(abs(x) for x in terms), e
        rel = 1e-7
        qp, qm = q.copy(), q.copy()
        qp[:3] += rel * dq
        qm[:3] -= rel * dq
        hp, hm = hc + rel * dhc, hc - rel * dhc
        label = _c02_branch(q, hc, e)
        if abs(e - hc[10]) > 1e-9 and \
                _c02_branch(qp, hp, e + rel * de) == label == _c02_branch(qm, hm, e - rel * de):
            fd = (port.uniaxial_trial(XG_UNI_CONCRETE02, qp, hp, e + rel * de) -
                  port.uniaxial_trial(XG_UNI_CONCRETE02, qm, hm, e - rel * de)) / (2 * rel)
            for f in fields:
                assert abs(dht[f] - fd[f]) <= 1e-6 * sc[f], (label, f, dht[f], fd[f])
            labels.add(label)
        hc = port.uniaxial_trial(XG_UNI_CONCRETE02, q, hc, e)
    need = {"env-c0", "env-c1", "env-c2", "unload-elastic", "unload-lower", "unload-upper",
            "tension-t0", "tension-t1"}
    assert need <= labels, labels


# ---------------------------------------------------------------------------
# GPU: gradients of a transient run
# ---------------------------------------------------------------------------
def _adjoint_model(n_frames=2, steps=40, seed=5, pga_scale=1.0):
    """Small frames of the batched-frames workload, one Steel02 per member."""
    desc, phases = configs.adjoint_frames(n_frames=n_frames, steps=steps, seed=seed,
                                          pga_scale=pga_scale)
    return desc, phases[0]


def _objective(desc):
    return desc.meta["obj_node"], desc.meta["obj_dof"], desc.meta["obj_weight"]


@pytest.mark.gpu
@pytest.mark.parametrize("pga_scale,steps", [(1.0, 40), (6.0, 120)])
def test_adjoint_gradient_matches_finite_differences(need_gpu, pga_scale, steps):
    gpu = _gpu()
    desc, ph = _adjoint_model(steps=steps, pga_scale=pga_scale)
    node, dof, w = _objective(desc)
    q0 = desc.uni_param.reshape(-1, 12).copy()
    with gpu.DeviceModel(desc) as m:
        J0 = gpu.adjoint_forward(m, ph, steps, 10, node, dof, w)
        rec = m.fiber_records()
        g = gpu.adjoint_backward(m)
        assert J0 > 0 and np.isfinite(g).all()
        if pga_scale > 1.0:
            # the strong case runs through yielding and load reversals
            ey = q0[0, 0] / q0[0, 1]
            assert (np.abs(rec[:, 10]) > ey).mean() > 0.01
            assert (rec[:, 5] != 0.0).mean() > 0.05

        def J(q):
            gpu.set_uniaxial_params(m, q)
            return gpu.adjoint_forward(m, ph, steps, 10, node, dof, w)

        rng = np.random.default_rng(11)
        scale = np.abs(q0[:, :3])
        # directional derivative along a random direction over all parameters
        d = rng.normal(size=q0[:, :3].shape) * scale
        h = 1e-6
        qp, qm = q0.copy(), q0.copy()
        qp[:, :3] += h * d
        qm[:, :3] -= h * d
        fd = (J(qp) - J(qm)) / (2 * h)
        ad = float((g * d).sum())
        assert ad == pytest.approx(fd, rel=1e-4), (ad, fd)
        # a few single parameters: the members with the largest sensitivities
        gs = np.abs(g) * scale
        for idx in np.argsort(gs.ravel())[-4:]:
            u, k = divmod(int(idx), 3)
            qp, qm = q0.copy(), q0.copy()
            qp[u, k] *= 1 + h
            qm[u, k] *= 1 - h
            fd = (J(qp) - J(qm)) / (2 * h * q0[u, k])
            assert g[u, k] == pytest.approx(fd, rel=1e-3, abs=1e-4 * gs.max() / q0[u, k]), (u, k)


@pytest.mark.gpu
@pytest.mark.parametrize("pga_scale,steps", [(1.0, 40), (3.0, 80)])
def test_adjoint_rc_frames_match_finite_differences(need_gpu, pga_scale, steps):
    """Reinforced-concrete members (Concrete02 layers and Steel02 bars, two
    materials per member): gradients with respect to every member's fc,
    epsc0, fcu and Fy, E0, b against central differences of the device
    forward run, through cracking, crushing and yielding at the stronger
    record; betaK0 damping on such members is refused."""
    gpu = _gpu()
    desc, phases = configs.adjoint_rc_frames(n_frames=2, steps=steps, seed=5,
                                             pga_scale=pga_scale)
    ph = phases[0]
    node, dof, w = _objective(desc)
    q0 = desc.uni_param.reshape(-1, 12).copy()
    conc = np.asarray(desc.uni_type) == XG_UNI_CONCRETE02
    with gpu.DeviceModel(desc) as m:
        J0 = gpu.adjoint_forward(m, ph, steps, 10, node, dof, w)
        rec = m.fiber_records()
        g = gpu.adjoint_backward(m)
        assert J0 > 0 and np.isfinite(g).all()
        assert np.abs(g[conc]).max() > 0 and np.abs(g[~conc]).max() > 0
        if pga_scale > 1.0:
            # cracked concrete (a tension excursion recorded) and yielded bars
            ss, fm = desc.arrays["sec_fiber_start"], desc.arrays["fib_mat"]
            kinds = np.concatenate([np.tile(np.asarray(desc.uni_type)[fm[ss[s_]:ss[s_ + 1]]],
                                            desc.fbc_num_ip)
                                    for s_ in desc.arrays["elem_mat"]])
            c_rec, s_rec = rec[kinds == XG_UNI_CONCRETE02], rec[kinds == XG_UNI_STEEL02]
            assert (c_rec[:, 1] > 0).mean() > 0.05
            assert (np.abs(s_rec[:, 10]) > 420e6 / 200e9).mean() > 0.001

        def J(q):
            gpu.set_uniaxial_params(m, q)
            return gpu.adjoint_forward(m, ph, steps, 10, node, dof, w)

        rng = np.random.default_rng(13)
        scale = np.abs(q0[:, :3])
        d = rng.normal(size=scale.shape) * scale
        h = 1e-6
        qp, qm = q0.copy(), q0.copy()
        qp[:, :3] += h * d
        qm[:, :3] -= h * d
        fd = (J(qp) - J(qm)) / (2 * h)
        ad = float((g * d).sum())
        assert ad == pytest.approx(fd, rel=1e-4), (ad, fd)
        gs = np.abs(g) * scale
        for sel in (conc, ~conc):
            idx = np.nonzero(sel)[0]
            top = idx[np.argsort(gs[idx].max(axis=1))[-2:]]
            for u in top:
                k = int(np.argmax(gs[u]))
                qp, qm = q0.copy(), q0.copy()
                qp[u, k] *= 1 + h
                qm[u, k] *= 1 - h
                fd = (J(qp) - J(qm)) / (2 * h * q0[u, k])
                assert g[u, k] == pytest.approx(fd, rel=1e-3, abs=1e-4 * gs.max() / abs(q0[u, k])), \
                    (u, k)
        # betaK0 Rayleigh damping is covered for single-material members only
        gpu.set_uniaxial_params(m, q0)
        phk = configs.adjoint_frames(n_frames=2, steps=steps, seed=5)[1][0]
        with pytest.raises(gpu.XaraGpuError, match="betaK0"):
            gpu.adjoint_forward(m, phk, steps, 10, node, dof, w)


def _fd_gradient_checks(m, desc, ph, steps, g, seed, nsingle=4):
    """The adjoint gradient ``g`` against central differences of the device
    forward run: along a seeded direction over every parameter (relative
    1e-4) and for the ``nsingle`` parameters with the largest scaled
    sensitivities (relative 1e-3)."""
    gpu = _gpu()
    node, dof, w = _objective(desc)
    q0 = desc.uni_param.reshape(-1, 12).copy()

    def J(q):
        gpu.set_uniaxial_params(m, q)
        return gpu.adjoint_forward(m, ph, steps, 10, node, dof, w)

    rng = np.random.default_rng(seed)
    scale = np.abs(q0[:, :3])
    d = rng.normal(size=scale.shape) * scale
    h = 1e-6
    qp, qm = q0.copy(), q0.copy()
    qp[:, :3] += h * d
    qm[:, :3] -= h * d
    fd = (J(qp) - J(qm)) / (2 * h)
    ad = float((g * d).sum())
    assert ad == pytest.approx(fd, rel=1e-4), (ad, fd)
    gs = np.abs(g) * scale
    for idx in np.argsort(gs.ravel())[len(gs.ravel()) - nsingle:]:
        u, k = divmod(int(idx), 3)
        qp, qm = q0.copy(), q0.copy()
        qp[u, k] *= 1 + h
        qm[u, k] *= 1 - h
        fd = (J(qp) - J(qm)) / (2 * h * q0[u, k])
        assert g[u, k] == pytest.approx(fd, rel=1e-3, abs=1e-4 * gs.max() / abs(q0[u, k])), (u, k)
    gpu.set_uniaxial_params(m, q0)


@pytest.mark.gpu
@pytest.mark.parametrize("pga_scale,steps", [(1.0, 40), (3.0, 80)])
def test_adjoint_pdelta_frames_match_finite_differences(need_gpu, pga_scale, steps):
    """2D frames under `geomTransf PDelta` with growing floor weights: the
    adjoint carries the transformation's force term (N / L) ul14 g into the
    basic-force adjoint and its tangent's non-symmetric part by a fixed
    point on the factored tangent.  Gradients against central differences
    of the device forward run; the P-Delta terms move the gradients well
    past the tolerance (the same frames with linear transformations)."""
    gpu = _gpu()
    desc, phases = configs.adjoint_pdelta_frames(steps=steps, pga_scale=pga_scale, seed=5)
    lin, lphases = configs.adjoint_pdelta_frames(steps=steps, pga_scale=pga_scale, seed=5,
                                                 pdelta=0)
    assert desc.geom_transf == 1 and lin.geom_transf == 0
    node, dof, w = _objective(desc)
    with gpu.DeviceModel(lin) as m:
        gpu.adjoint_forward(m, lphases[0], steps, 10, node, dof, w)
        g_lin = gpu.adjoint_backward(m)
    with gpu.DeviceModel(desc) as m:
        J0 = gpu.adjoint_forward(m, phases[0], steps, 10, node, dof, w)
        g = gpu.adjoint_backward(m)
        assert J0 > 0 and np.isfinite(g).all()
        assert np.abs(g - g_lin).max() > 1e-3 * np.abs(g).max()
        _fd_gradient_checks(m, desc, phases[0], steps, g, seed=17)


@pytest.mark.gpu
@pytest.mark.parametrize("pga_scale,steps", [(1.0, 40), (3.0, 80)])
def test_adjoint_rc_frame_3d_matches_finite_differences(need_gpu, pga_scale, steps):
    """A 3D RC frame (Concrete02 cover and core, Steel02 bars, elastic
    torsion, `geomTransf PDelta`, whose 3D terms cancel in the reference's
    transformation) under a ground motion in x: gradients with respect to
    every material's first three parameters against central differences of
    the device forward run, through cracking at both records."""
    gpu = _gpu()
    desc, phases = configs.adjoint_rc_frame_3d(steps=steps, pga_scale=pga_scale)
    node, dof, w = _objective(desc)
    conc = np.asarray(desc.uni_type) == XG_UNI_CONCRETE02
    with gpu.DeviceModel(desc) as m:
        J0 = gpu.adjoint_forward(m, phases[0], steps, 10, node, dof, w)
        rec = m.fiber_records()
        g = gpu.adjoint_backward(m)
        assert J0 > 0 and np.isfinite(g).all()
        assert np.abs(g[conc]).max() > 0 and np.abs(g[~conc]).max() > 0
        ss, fm = desc.arrays["sec_fiber_start"], desc.arrays["fib_mat"]
        kinds = np.concatenate([np.tile(np.asarray(desc.uni_type)[fm[ss[s_]:ss[s_ + 1]]],
                                        desc.fbc_num_ip)
                                for s_ in desc.arrays["elem_mat"]])
        assert (rec[kinds == XG_UNI_CONCRETE02, 1] > 0).mean() > 0.05    # cracked
        _fd_gradient_checks(m, desc, phases[0], steps, g, seed=19)


@pytest.mark.gpu
def test_adjoint_checkpoint_interval_and_end_state(need_gpu):
    gpu = _gpu()
    desc, ph = _adjoint_model(n_frames=3, steps=30, seed=9)
    node, dof, w = _objective(desc)
    with gpu.DeviceModel(desc) as m:
        Ja = gpu.adjoint_forward(m, ph, 30, 7, node, dof, w)
        ua, _ = m.disp()
        ga = gpu.adjoint_backward(m)
        ub, _ = m.disp()
        np.testing.assert_array_equal(ua, ub)   # left at the run's last state
        m.reset()
        Jb = gpu.adjoint_forward(m, ph, 30, 30, node, dof, w)
        gb = gpu.adjoint_backward(m)
    assert Ja == Jb
    np.testing.assert_allclose(ga, gb, rtol=1e-12, atol=1e-12 * np.abs(ga).max())


@pytest.mark.gpu
def test_adjoint_through_torch_autograd(need_gpu):
    import torch
    gpu = _gpu()
    from xara_gb300.adjoint import frame_response
    desc, ph = _adjoint_model(n_frames=2, steps=20, seed=2)
    obj = _objective(desc)
    q0 = desc.uni_param.reshape(-1, 12)
    with gpu.DeviceModel(desc) as m:
        theta = torch.tensor(q0[:, :3], dtype=torch.float64, requires_grad=True)
        J = frame_response(theta, m, ph, 20, 5, obj)
        (2.0 * J).backward()
        m.reset()
        J2 = gpu.adjoint_forward(m, ph, 20, 5, *obj)
        g = gpu.adjoint_backward(m)
    assert float(J.detach()) == J2
    np.testing.assert_allclose(theta.grad.numpy(), 2.0 * g, rtol=1e-13, atol=0)


DDM_CASES = ["ddm_steel01_frame", "ddm_rc01_frame"]


def _kinds(desc):
    """(material rows of one law, parameter index): the parameter kinds the
    gradient checks scale separately."""
    ut = np.asarray(desc.uni_type)
    return [(np.nonzero(ut == t)[0], k) for t in np.unique(ut) for k in range(3)]


@pytest.mark.gpu
def test_forward_mode_through_torch(need_gpu):
    """torch's forward-mode AD (a dual tensor through frame_response) runs
    the DDM: its tangent equals the reverse-mode gradient projected on the
    tangent direction (1e-9), and the primal equals the plain run's J."""
    import torch
    import torch.autograd.forward_ad as fwAD
    gpu = _gpu()
    from xara_gb300.adjoint import frame_response
    desc, ph = _adjoint_model(n_frames=2, steps=30, seed=2)
    obj = _objective(desc)
    q0 = desc.uni_param.reshape(-1, 12)
    d = np.random.default_rng(53).normal(size=q0[:, :3].shape) * np.abs(q0[:, :3])
    with gpu.DeviceModel(desc) as m:
        theta = torch.tensor(q0[:, :3], dtype=torch.float64)
        with fwAD.dual_level():
            J = frame_response(fwAD.make_dual(theta, torch.tensor(d)), m, ph, 30, 10, obj)
            Jp, dJ = fwAD.unpack_dual(J)
        m.reset()
        J2 = gpu.adjoint_forward(m, ph, 30, 10, *obj)
        g = gpu.adjoint_backward(m)
    assert float(Jp) == J2
    assert float(dJ) == pytest.approx(float((g * d).sum()), rel=1e-9)


def _ddm_case(name="ddm_steel01_frame"):
    from golden_util import load, model_of
    fx = load(name)
    desc, phases = model_of(fx)
    obj = (desc.meta["obj_node"], desc.meta["obj_dof"], desc.meta["obj_weight"])
    return fx, desc, phases, obj


@pytest.mark.parametrize("name", DDM_CASES)
def test_ddm_surrogate_forward_matches_the_reference(name):
    """The massless ramps the reference's DDM runs on (Steel01 members; RC
    members of Concrete01 and Steel01): the oracle's history and objective
    equal the reference's (the fixture), and the fixture's gradient passed
    central differences of the oracle when it was made."""
    fx, desc, phases, obj = _ddm_case(name)
    if "fd_check" in fx:
        assert fx["fd_check"][0] < 1e-7
    o = port.OracleModel(desc)
    U, _, its = o.run(phases)
    o.close()
    assert np.array_equal(its, fx["step_iters"])
    assert np.linalg.norm(U - fx["step_u"]) <= 1e-12 * np.linalg.norm(fx["step_u"])
    roof = list(desc.node_tag).index(int(obj[0][0]))
    J = obj[2][0] * np.sum(U[:, 3 * roof] ** 2)
    assert abs(J - fx["J"][0]) <= 1e-12 * fx["J"][0]


@pytest.mark.gpu
@pytest.mark.parametrize("name", DDM_CASES)
def test_adjoint_matches_the_reference_ddm(need_gpu, name):
    """The device adjoint against the reference's own DDM sensitivity
    (Newmark::computeSensitivities after every step, the gradient of the
    summed squared roof drift accumulated from Node::getDispSensitivity) on
    the massless ramps: every member's d/d(fy, E0, b) of Steel01 and
    d/d(fpc, epsc0, fpcu) of Concrete01, each parameter kind within 1e-6
    relative of its largest entry, and the objective within 1e-12."""
    gpu = _gpu()
    fx, desc, phases, obj = _ddm_case(name)
    ph = phases[0]
    with gpu.DeviceModel(desc) as m:
        m.set_system(gpu.XG_SYSTEM_PROFILE_SPD)
        J = gpu.adjoint_forward(m, ph, ph.num_steps, 25, *obj)
        g = gpu.adjoint_backward(m)
    ref = fx["grad"]
    assert abs(J - fx["J"][0]) <= 1e-12 * fx["J"][0]
    assert g.shape == ref.shape
    for rows, k in _kinds(desc):
        scale = np.abs(ref[rows, k]).max()
        assert np.max(np.abs(g[rows, k] - ref[rows, k])) <= 1e-6 * scale, (k, g[rows, k],
                                                                           ref[rows, k])


# ---------------------------------------------------------------------------
# GPU: direct differentiation (DDM), forward mode
# ---------------------------------------------------------------------------
def _unit_directions(nu):
    """One direction per (material, parameter 0..2)."""
    return np.eye(nu * 3).reshape(nu * 3, nu, 3)


@pytest.mark.gpu
@pytest.mark.parametrize("name", DDM_CASES)
def test_ddm_matches_the_reference_ddm_and_the_adjoint(need_gpu, name):
    """The device DDM on the massless ramps (Steel01 members; Concrete01 and
    Steel01 members), one direction per material and parameter: against the
    reference's own DDM (each parameter kind
    within 1e-6 of its largest entry; the reference solves with the last
    Newton iteration's factors, the device at the converged state) and
    against the device adjoint (1e-10: both are exact derivatives of the
    same discrete path, by independent code)."""
    gpu = _gpu()
    fx, desc, phases, obj = _ddm_case(name)
    ph = phases[0]
    nu = len(desc.uni_type)
    with gpu.DeviceModel(desc) as m:
        m.set_system(gpu.XG_SYSTEM_PROFILE_SPD)
        J, dJ = gpu.ddm_forward(m, ph, ph.num_steps, _unit_directions(nu), *obj)
        m.reset()
        Ja = gpu.adjoint_forward(m, ph, ph.num_steps, 25, *obj)
        ga = gpu.adjoint_backward(m)
    g = dJ.reshape(nu, 3)
    ref = fx["grad"]
    assert J == Ja
    assert abs(J - fx["J"][0]) <= 1e-12 * fx["J"][0]
    for rows, k in _kinds(desc):
        scale = np.abs(ref[rows, k]).max()
        assert np.max(np.abs(g[rows, k] - ref[rows, k])) <= 1e-6 * scale, (k, g[rows, k],
                                                                           ref[rows, k])
        assert np.max(np.abs(g[rows, k] - ga[rows, k])) <= 1e-10 * scale, (k, g[rows, k],
                                                                            ga[rows, k])


@pytest.mark.gpu
@pytest.mark.parametrize("pga_scale,steps", [(1.0, 40), (6.0, 120)])
def test_ddm_under_ground_motion_matches_the_adjoint(need_gpu, pga_scale, steps):
    """Two Steel01 frames with floor masses under their records (the second
    at six times the record, through yielding and reversals): the DDM along
    seeded directions equals the adjoint's gradient projected on them (1e-9)
    and central differences of the forward run (1e-4); at the unscaled
    record the displacement tangent after the last step against central
    differences of the final displacements (at six times the record a
    single displacement sees a fiber change branch within h)."""
    gpu = _gpu()
    desc, phases = configs.ddm_steel01_frames_eq(steps=steps, pga_scale=pga_scale, seed=5)
    ph = phases[0]
    node, dof, w = _objective(desc)
    q0 = desc.uni_param.reshape(-1, 12).copy()
    nu = len(q0)
    rng = np.random.default_rng(23)
    dirs = rng.normal(size=(3, nu, 3)) * np.abs(q0[:, :3])
    with gpu.DeviceModel(desc) as m:
        J, dJ = gpu.ddm_forward(m, ph, steps, dirs, node, dof, w)
        du = gpu.ddm_disp_sensitivity(m, 0)
        rec = m.fiber_records()
        m.reset()
        Ja = gpu.adjoint_forward(m, ph, steps, 10, node, dof, w)
        ga = gpu.adjoint_backward(m)
        assert J == Ja and np.abs(dJ).min() > 0
        if pga_scale > 1.0:
            ey = q0[0, 0] / q0[0, 1]
            assert (np.abs(rec[:, 10]) > ey).mean() > 0.01
        for k in range(3):
            assert dJ[k] == pytest.approx(float((ga * dirs[k]).sum()), rel=1e-9), k
        h = 1e-6
        m.reset()
        gpu.set_uniaxial_params(m, np.c_[q0[:, :3] + h * dirs[0], q0[:, 3:]])
        Jp = gpu.adjoint_forward(m, ph, steps, steps, node, dof, w)
        up, _ = m.disp()
        m.reset()
        gpu.set_uniaxial_params(m, np.c_[q0[:, :3] - h * dirs[0], q0[:, 3:]])
        Jm = gpu.adjoint_forward(m, ph, steps, steps, node, dof, w)
        um, _ = m.disp()
    assert dJ[0] == pytest.approx((Jp - Jm) / (2 * h), rel=1e-4)
    fdu = (np.asarray(up) - np.asarray(um)).reshape(du.shape) / (2 * h)
    if pga_scale == 1.0:
        assert np.abs(du - fdu).max() <= 1e-4 * np.abs(fdu).max()


@pytest.mark.gpu
@pytest.mark.parametrize("pga_scale,steps", [(1.0, 40), (3.0, 80)])
def test_ddm_rc01_frames_under_ground_motion(need_gpu, pga_scale, steps):
    """Two RC frames with Concrete01 layers and Steel01 bars, floor masses,
    under their records (the second at three times the record, through
    cracking and crushing): the DDM along seeded directions against the
    adjoint (1e-9) and central differences of the forward run (1e-4)."""
    gpu = _gpu()
    desc, phases = configs.adjoint_rc_frames(n_frames=2, steps=steps, seed=5,
                                             pga_scale=pga_scale, laws="01")
    ph = phases[0]
    node, dof, w = _objective(desc)
    q0 = desc.uni_param.reshape(-1, 12).copy()
    nu = len(q0)
    rng = np.random.default_rng(31)
    dirs = rng.normal(size=(3, nu, 3)) * np.abs(q0[:, :3])
    with gpu.DeviceModel(desc) as m:
        J, dJ = gpu.ddm_forward(m, ph, steps, dirs, node, dof, w)
        rec = m.fiber_records()
        m.reset()
        Ja = gpu.adjoint_forward(m, ph, steps, 10, node, dof, w)
        ga = gpu.adjoint_backward(m)
        assert J == Ja and np.abs(dJ).min() > 0
        ss, fm = desc.arrays["sec_fiber_start"], desc.arrays["fib_mat"]
        kinds = np.concatenate([np.tile(np.asarray(desc.uni_type)[fm[ss[s_]:ss[s_ + 1]]],
                                        desc.fbc_num_ip)
                                for s_ in desc.arrays["elem_mat"]])
        c_rec = rec[kinds == XG_UNI_CONCRETE01]
        assert (c_rec[:, 0] < -1e-4).mean() > 0.01               # compressed beyond 1e-4
        for k in range(3):
            assert dJ[k] == pytest.approx(float((ga * dirs[k]).sum()), rel=1e-9), k
        h = 1e-6
        qp, qm = q0.copy(), q0.copy()
        qp[:, :3] += h * dirs[0]
        qm[:, :3] -= h * dirs[0]
        gpu.set_uniaxial_params(m, qp)
        Jp = gpu.adjoint_forward(m, ph, steps, steps, node, dof, w)
        gpu.set_uniaxial_params(m, qm)
        Jm = gpu.adjoint_forward(m, ph, steps, steps, node, dof, w)
    assert dJ[0] == pytest.approx((Jp - Jm) / (2 * h), rel=1e-4)


@pytest.mark.gpu
def test_ddm_3d_frame_and_refusals(need_gpu):
    """A 3D frame (the RC frame's sections with Steel01 fibers) under a
    ground motion: DDM against the adjoint along seeded directions (1e-9);
    Steel02 with an initial stress and betaK0 damping on mixed members are
    refused."""
    gpu = _gpu()
    base, phases = configs.adjoint_rc_frame_3d(steps=40, pga_scale=3.0)
    nu = len(base.uni_type)
    rows = np.stack([configs.steel01_row(fy=30e6, E=30e9, b=0.01)] * nu)
    rows[-1] = configs.steel01_row(fy=420e6, E=200e9, b=0.01)
    desc = configs._with_geometry(base, uni_type=np.full(nu, XG_UNI_STEEL01), uni_param=rows)
    ph = phases[0]
    node, dof, w = _objective(base)
    rng = np.random.default_rng(29)
    dirs = rng.normal(size=(2, nu, 3)) * np.abs(rows[:, :3])
    with gpu.DeviceModel(desc) as m:
        J, dJ = gpu.ddm_forward(m, ph, 40, dirs, node, dof, w)
        rec = m.fiber_records()
        m.reset()
        Ja = gpu.adjoint_forward(m, ph, 40, 10, node, dof, w)
        ga = gpu.adjoint_backward(m)
    assert J == Ja
    assert (np.abs(rec[:, 10]) > 1e-3).mean() > 0.01          # some fibers yield
    for k in range(2):
        assert dJ[k] == pytest.approx(float((ga * dirs[k]).sum()), rel=1e-9), k
    d2, p2 = configs.adjoint_frames(n_frames=1, steps=5, seed=3)
    q2 = d2.uni_param.reshape(-1, 12).copy()
    q2[:, 10] = 1e6                                     # Steel02 initial stress
    d2 = configs._with_geometry(d2, uni_param=q2)
    with gpu.DeviceModel(d2) as m:
        with pytest.raises(gpu.XaraGpuError, match="initial stress"):
            gpu.ddm_forward(m, p2[0], 5, np.zeros((1, len(d2.uni_type), 3)),
                            *_objective(d2))
    d3, p3 = configs.adjoint_rc_frames(n_frames=1, steps=5, seed=3, laws="01")
    p3[0].beta_k_init_elem = np.full(len(d3.arrays["elem_tag"]), 1e-3)
    with gpu.DeviceModel(d3) as m:
        with pytest.raises(gpu.XaraGpuError, match="betaK0"):
            gpu.ddm_forward(m, p3[0], 5, np.zeros((1, len(d3.uni_type), 3)), *_objective(d3))


@pytest.mark.gpu
@pytest.mark.parametrize("pga_scale,steps", [(1.0, 40), (3.0, 80)])
def test_ddm_of_rc_frames_matches_the_adjoint(need_gpu, pga_scale, steps):
    """The adjoint's RC frames (Concrete02 layers and Steel02 bars, the second
    record through cracking, crushing and yielding): the DDM along seeded
    directions equals the adjoint's gradient projected on them (1e-9)."""
    gpu = _gpu()
    desc, phases = configs.adjoint_rc_frames(n_frames=2, steps=steps, seed=5,
                                             pga_scale=pga_scale)
    ph = phases[0]
    node, dof, w = _objective(desc)
    q0 = desc.uni_param.reshape(-1, 12)
    rng = np.random.default_rng(43)
    dirs = rng.normal(size=(3, len(q0), 3)) * np.abs(q0[:, :3])
    with gpu.DeviceModel(desc) as m:
        J, dJ = gpu.ddm_forward(m, ph, steps, dirs, node, dof, w)
        m.reset()
        Ja = gpu.adjoint_forward(m, ph, steps, 10, node, dof, w)
        ga = gpu.adjoint_backward(m)
    assert J == Ja and np.abs(dJ).min() > 0
    for k in range(3):
        assert dJ[k] == pytest.approx(float((ga * dirs[k]).sum()), rel=1e-9), k


@pytest.mark.gpu
@pytest.mark.parametrize("pga_scale,steps", [(1.0, 40), (3.0, 80)])
def test_ddm_of_pdelta_frames_matches_the_adjoint(need_gpu, pga_scale, steps):
    """2D frames under `geomTransf PDelta` with growing floor weights and
    betaK0 damping: the DDM (the P-Delta force's axial term at fixed
    displacements, the tangent's non-symmetric term by a fixed point on the
    factored tangent) along seeded directions equals the adjoint's gradient
    projected on them (1e-9)."""
    gpu = _gpu()
    desc, phases = configs.adjoint_pdelta_frames(steps=steps, pga_scale=pga_scale, seed=5)
    ph = phases[0]
    node, dof, w = _objective(desc)
    q0 = desc.uni_param.reshape(-1, 12)
    rng = np.random.default_rng(47)
    dirs = rng.normal(size=(2, len(q0), 3)) * np.abs(q0[:, :3])
    with gpu.DeviceModel(desc) as m:
        J, dJ = gpu.ddm_forward(m, ph, steps, dirs, node, dof, w)
        m.reset()
        Ja = gpu.adjoint_forward(m, ph, steps, 10, node, dof, w)
        ga = gpu.adjoint_backward(m)
    assert J == Ja and np.abs(dJ).min() > 0
    for k in range(2):
        assert dJ[k] == pytest.approx(float((ga * dirs[k]).sum()), rel=1e-9), k


@pytest.mark.gpu
@pytest.mark.parametrize("pga_scale,steps", [(1.0, 40), (6.0, 120)])
def test_ddm_of_the_adjoint_frames_frame_by_frame(need_gpu, pga_scale, steps):
    """The adjoint's own frames (Steel02 members, 2 % Rayleigh with betaK0 per
    frame; the second case through yielding and reversals): one DDM
    direction over every member gives each frame's directional derivative
    through that frame's objective term, equal to the adjoint's gradient
    projected on the frame's members (1e-9 of the frame's value)."""
    gpu = _gpu()
    desc, ph = _adjoint_model(n_frames=3, steps=steps, pga_scale=pga_scale, seed=7)
    node, dof, w = _objective(desc)
    q0 = desc.uni_param.reshape(-1, 12)
    frame = np.asarray(desc.meta["member_frame"])
    rng = np.random.default_rng(37)
    d = rng.normal(size=(1, len(q0), 3)) * np.abs(q0[:, :3])
    with gpu.DeviceModel(desc) as m:
        J, dJ = gpu.ddm_forward(m, ph, steps, d, node, dof, w)
        per_frame = gpu.ddm_objective_terms(m, 0, len(node))
        m.reset()
        Ja = gpu.adjoint_forward(m, ph, steps, 10, node, dof, w)
        ga = gpu.adjoint_backward(m)
    assert J == Ja
    assert dJ[0] == pytest.approx(per_frame.sum(), rel=1e-12)
    for f in range(len(node)):
        proj = float((ga[frame == f] * d[0][frame == f]).sum())
        assert per_frame[f] == pytest.approx(proj, rel=1e-9), f


@pytest.mark.gpu
def test_ddm_of_a_static_pushover(need_gpu):
    """LoadControl (the reference's LoadControl::computeSensitivities: no
    inertia, K dU = -dP at fixed U): a 2D steel frame pushed laterally into
    Steel02's nonlinear transition, the DDM of the summed squared roof drift
    along seeded directions against central differences of the device run
    (1e-5)."""
    from xara_gb300._abi import PhaseDesc, XG_INT_LOAD_CONTROL
    gpu = _gpu()
    desc, _ = configs.steel_frame_2d(2, 3, gravity=0.0)
    ph = PhaseDesc(integrator=XG_INT_LOAD_CONTROL, pattern=1, num_steps=20, d_lambda=25e3,
                   tol=1e-10, max_iter=50)
    roof = int(desc.meta["roof"])
    obj = (np.array([roof], np.int32), np.zeros(1, np.int32), np.array([1.0 / 10.5 ** 2]))
    q0 = desc.uni_param.reshape(-1, 12).copy()
    rng = np.random.default_rng(59)
    dirs = rng.normal(size=(2, len(q0), 3)) * np.abs(q0[:, :3])
    none = np.zeros((1, len(q0), 3))

    def J(m, q):
        gpu.set_uniaxial_params(m, q)
        m.reset()
        return gpu.ddm_forward(m, ph, 20, none, *obj)[0]

    with gpu.DeviceModel(desc) as m:
        J0, dJ = gpu.ddm_forward(m, ph, 20, dirs, *obj)
        rec = m.fiber_records()
        # the extreme fibers well into Steel02's curved transition
        assert np.abs(rec[:, 10]).max() > 0.7 * q0[0, 0] / q0[0, 1]
        assert J(m, q0) == J0
        h = 1e-6
        for k in range(2):
            fd = (J(m, q0 + np.c_[h * dirs[k], np.zeros((len(q0), 9))]) -
                  J(m, q0 - np.c_[h * dirs[k], np.zeros((len(q0), 9))])) / (2 * h)
            assert dJ[k] == pytest.approx(fd, rel=1e-5), k


@pytest.mark.gpu
def test_ddm_argument_checks(need_gpu):
    """The DDM entry points refuse what they cannot serve: reads before a
    run, a direction out of range, a term count that is not the run's, no
    directions, a run that does not start from the initial state."""
    gpu = _gpu()
    desc, ph = _adjoint_model(n_frames=1, steps=5, seed=3)
    node, dof, w = _objective(desc)
    nu = len(desc.uni_type)
    with gpu.DeviceModel(desc) as m:
        with pytest.raises(gpu.XaraGpuError, match="no DDM run"):
            gpu.ddm_objective_terms(m, 0, len(node))
        with pytest.raises(gpu.XaraGpuError):
            gpu.ddm_forward(m, ph, 5, np.zeros((0, nu, 3)), node, dof, w)
        J, dJ = gpu.ddm_forward(m, ph, 5, np.ones((1, nu, 3)), node, dof, w)
        assert np.isfinite(J) and np.isfinite(dJ).all()
        with pytest.raises(gpu.XaraGpuError, match="bad direction"):
            gpu.ddm_objective_terms(m, 1, len(node))
        with pytest.raises(gpu.XaraGpuError, match="terms"):
            gpu.ddm_objective_terms(m, 0, len(node) + 1)
        with pytest.raises(gpu.XaraGpuError, match="bad direction"):
            gpu.ddm_disp_sensitivity(m, 2)
        with pytest.raises(gpu.XaraGpuError, match="initial state"):
            gpu.ddm_forward(m, ph, 5, np.ones((1, nu, 3)), node, dof, w)


@pytest.mark.parametrize("kind", [XG_UNI_STEEL02, XG_UNI_CONCRETE02, XG_UNI_STEEL01,
                                  XG_UNI_CONCRETE01])
def test_jvp_at_the_committed_strain(kind):
    """A trial strain equal to the committed one keeps the committed state
    in every law; its forward mode passes the record's tangents through
    (the strain's own tangent for the strain field) and agrees with the
    reverse mode there too."""
    gpu = _gpu()
    q = {XG_UNI_STEEL02: configs.steel02_row(), XG_UNI_CONCRETE02: configs.concrete02_row(30e6),
         XG_UNI_STEEL01: configs.steel01_row(), XG_UNI_CONCRETE01: configs.concrete01_row(30e6)}[kind]
    hc = port.uniaxial_trial(kind, q, port.uniaxial_init(kind, q), -1e-3)   # a committed state
    rng = np.random.default_rng(61)
    dhc = rng.normal(size=12)
    dhc[[7, 8, 11]] = 0.0
    dq = rng.normal(size=3)
    de = rng.normal()
    eps = float(hc[10])
    dht = gpu.uniaxial_jvp(kind, q, hc, eps, de, dhc, dq)
    fields = {XG_UNI_STEEL02: list(range(7)), XG_UNI_CONCRETE02: [0, 1],
              XG_UNI_STEEL01: [0, 1, 2, 3], XG_UNI_CONCRETE01: [0, 1, 2]}[kind]
    np.testing.assert_array_equal(dht[fields], dhc[fields])
    yb = rng.normal(size=12)
    yb[[7, 8, 11]] = 0.0
    hb, sb, qb = gpu.uniaxial_vjp(kind, q, hc, eps, yb)
    keep = fields + [9, 10]
    lhs = float(yb[keep] @ dht[keep])
    rhs = sb * de + float(hb[keep] @ dhc[keep]) + float(qb @ dq)
    assert lhs == pytest.approx(rhs, rel=1e-12, abs=1e-300)
