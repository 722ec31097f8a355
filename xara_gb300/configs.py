"""Seeded synthetic models for the workloads the hot path is measured on.

Each builder returns ``(ModelDesc, [PhaseDesc, ...])``.  The models are the
ones the reference's modelling commands would build (`node`, `fix`,
`equalDOF`, `element quad|stdBrick`, `nDMaterial J2Plasticity`,
`pattern Plain` with a reference `load`, `integrator DisplacementControl`,
`test NormDispIncr`, `algorithm Newton`, the default PlainHandler), generated
from a seed; no data set is involved.

The loaded edge/face is tied to a master node with `equalDOF` in the loaded
direction and driven by DisplacementControl on that node.  (Imposing the
displacement as `sp` values through the Transformation handler puts the
whole first increment into the loaded element layer, which yields, and the
reference's own Newton iteration then diverges on these models.)

Workloads (all FP64):
  * plane-strain block of 4-node quads with J2 plasticity, top edge pushed
    down to a nominal strain in equal increments (64 x 16 elements, 20
    increments to 0.5 %);
  * 8-node brick block with J2 plasticity, per-element yield stress drawn
    uniformly from a seed, top face compressed (128 x 128 x 64 elements,
    50 increments to 1 %).
"""
import numpy as np

from ._abi import (ModelDesc, PhaseDesc, XG_ELE_BRICK, XG_ELE_QUAD,
                   XG_HANDLER_PLAIN, XG_HANDLER_TRANSFORMATION, XG_INT_DISP_CONTROL,
                   XG_INT_NEWMARK,
                   XG_TEST_NORM_DISP_INCR)

# nDMaterial J2Plasticity K G sigma0 sigma_inf delta H eta rho
J2_STEEL = (166.7e9, 76.9e9, 250e6, 250e6, 0.0, 1e9, 0.0, 0.0)


def quad_block(nx=64, ny=16, lx=None, ly=None, strain=0.005, steps=20,
               j2=J2_STEEL, thickness=1.0, tol=1e-10, max_iter=25):
    """`element quad` block, bottom edge fixed, top edge displaced downwards.

    Node tags run row by row from 1; element tags from 1.  The top edge is
    tied in y to its left node, which DisplacementControl drives down by
    strain*H/steps per step, so after the last step the nominal vertical
    strain equals ``strain``.
    """
    lx = float(nx) if lx is None else lx
    ly = float(ny) if ly is None else ly
    xs = np.linspace(0.0, lx, nx + 1)
    ys = np.linspace(0.0, ly, ny + 1)
    X, Y = np.meshgrid(xs, ys)             # rows = y
    crd = np.stack([X.ravel(), Y.ravel()], axis=1)
    nn = (nx + 1) * (ny + 1)
    tags = np.arange(1, nn + 1, dtype=np.int32)

    def nid(i, j):
        return j * (nx + 1) + i + 1

    conn = []
    for j in range(ny):
        for i in range(nx):
            conn.append([nid(i, j), nid(i + 1, j), nid(i + 1, j + 1), nid(i, j + 1)])
    conn = np.asarray(conn, np.int32)
    ne = len(conn)
    sp_node, sp_dof = [], []
    for i in range(nx + 1):                  # bottom edge: fix i 1 1
        sp_node += [nid(i, 0), nid(i, 0)]
        sp_dof += [0, 1]
    master = nid(0, ny)                      # top edge: equalDOF master i 2
    mp_c = [nid(i, ny) for i in range(1, nx + 1)]
    desc = ModelDesc(
        ndm=2, ndf=2, elem_type=XG_ELE_QUAD, thickness=thickness,
        handler=XG_HANDLER_PLAIN,
        node_tag=tags, node_crd=crd,
        elem_tag=np.arange(1, ne + 1), elem_conn=conn, elem_mat=np.zeros(ne),
        j2_param=np.asarray(j2, np.float64),
        sp_node=sp_node, sp_dof=sp_dof, sp_pattern=np.full(len(sp_node), -1),
        sp_value=np.zeros(len(sp_node)),
        mp_retained=np.full(len(mp_c), master), mp_constrained=mp_c,
        mp_dof=np.ones(len(mp_c)),
        load_node=[master], load_pattern=[0], load_value=[[0.0, -1.0]],
    )
    desc.meta = dict(workload=f"quad J2 plane strain {nx}x{ny}", nx=nx, ny=ny,
                     nip=4 * ne, master=master)
    phase = PhaseDesc(integrator=XG_INT_DISP_CONTROL, pattern=0, num_steps=steps,
                      dc_node=master, dc_dof=1, dc_incr=-strain * ly / steps,
                      test=XG_TEST_NORM_DISP_INCR, tol=tol, max_iter=max_iter)
    return desc, [phase]


def brick_block(nx=128, ny=128, nz=64, strain=0.01, steps=50, j2=J2_STEEL,
                sig_range=(200e6, 300e6), seed=0, tol=1e-10, max_iter=25):
    """`element stdBrick` block of unit cubes, base fixed, top face compressed.

    Each element gets its own J2 row with sigma0 = sigma_inf drawn uniformly
    from ``sig_range`` (seeded).  Node tags run x fastest, then y, then z.
    The top face is tied in z to its first node, which DisplacementControl
    drives down by strain*H/steps per step.
    """
    rng = np.random.default_rng(seed)
    xs = np.arange(nx + 1, dtype=np.float64)
    ys = np.arange(ny + 1, dtype=np.float64)
    zs = np.arange(nz + 1, dtype=np.float64)
    Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
    crd = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    nn = crd.shape[0]
    tags = np.arange(1, nn + 1, dtype=np.int32)
    sx, sy = 1, nx + 1
    sz = (nx + 1) * (ny + 1)
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    base = (k * sz + j * sy + i * sx).ravel() + 1
    # stdBrick node order: bottom face counter-clockwise, then top face
    offs = np.array([0, sx, sx + sy, sy, sz, sz + sx, sz + sx + sy, sz + sy])
    conn = (base[:, None] + offs[None, :]).astype(np.int32)
    ne = conn.shape[0]
    sig = rng.uniform(sig_range[0], sig_range[1], size=ne)
    j2rows = np.tile(np.asarray(j2, np.float64), (ne, 1))
    j2rows[:, 2] = sig
    j2rows[:, 3] = sig
    bot = np.arange(1, sz + 1)
    top = np.arange(nz * sz + 1, nn + 1)
    master = int(top[0])
    sp_node = np.repeat(bot, 3)
    sp_dof = np.tile([0, 1, 2], len(bot))
    desc = ModelDesc(
        ndm=3, ndf=3, elem_type=XG_ELE_BRICK, handler=XG_HANDLER_PLAIN,
        node_tag=tags, node_crd=crd,
        elem_tag=np.arange(1, ne + 1), elem_conn=conn, elem_mat=np.arange(ne),
        j2_param=j2rows,
        sp_node=sp_node, sp_dof=sp_dof, sp_pattern=np.full(len(sp_node), -1),
        sp_value=np.zeros(len(sp_node)),
        mp_retained=np.full(len(top) - 1, master), mp_constrained=top[1:],
        mp_dof=np.full(len(top) - 1, 2),
        load_node=[master], load_pattern=[0], load_value=[[0.0, 0.0, -1.0]],
    )
    desc.meta = dict(workload=f"brick J2 {nx}x{ny}x{nz}", nx=nx, ny=ny, nz=nz,
                     nip=8 * ne, master=master)
    phase = PhaseDesc(integrator=XG_INT_DISP_CONTROL, pattern=0, num_steps=steps,
                      dc_node=master, dc_dof=2, dc_incr=-strain * nz / steps,
                      test=XG_TEST_NORM_DISP_INCR, tol=tol, max_iter=max_iter)
    return desc, [phase]


# ---------------------------------------------------------------------------
# frames: `element forceBeamColumn` with Lobatto points and fiber sections
# ---------------------------------------------------------------------------
from ._abi import (XG_ELE_FBC2D, XG_ELE_FBC3D, XG_INT_LOAD_CONTROL,  # noqa: E402
                   XG_UNI_CONCRETE01, XG_UNI_CONCRETE02, XG_UNI_ELASTIC, XG_UNI_STEEL01,
                   XG_UNI_STEEL02, XG_UNI_NPARAM)


def steel02_row(fy=350e6, E=200e9, b=0.01, R0=18.0, cR1=0.925, cR2=0.15):
    """`uniaxialMaterial Steel02 tag fy E b R0 cR1 cR2` (a1..a4 = 0 1 0 1)."""
    r = np.zeros(XG_UNI_NPARAM)
    r[:11] = [fy, E, b, R0, cR1, cR2, 0.0, 1.0, 0.0, 1.0, 0.0]
    return r


def steel01_row(fy=350e6, E=200e9, b=0.01, a1=0.0, a2=1.0, a3=0.0, a4=1.0):
    """`uniaxialMaterial Steel01 tag fy E b a1 a2 a3 a4` (no isotropic
    hardening by default)."""
    r = np.zeros(XG_UNI_NPARAM)
    r[:7] = [fy, E, b, a1, a2, a3, a4]
    return r


def steel_row(law, fy, E, b):
    """The steel row of a frame section: Steel02 (R0 18, cR1 0.925, cR2
    0.15) or Steel01."""
    if law == "Steel01":
        return steel01_row(fy, E, b)
    return steel02_row(fy, E, b)


def steel_type(law):
    return XG_UNI_STEEL01 if law == "Steel01" else XG_UNI_STEEL02


def concrete01_row(fc, epsc0=0.002, fcu_ratio=0.2, epscu=0.006):
    """`uniaxialMaterial Concrete01 tag fpc epsc0 fpcu epscu` with the
    compressive values negative, as the command takes them: fpc = -fc,
    fpcu = -fcu_ratio fc."""
    r = np.zeros(XG_UNI_NPARAM)
    r[:4] = (-abs(fc), -abs(epsc0), -abs(fcu_ratio * fc), -abs(epscu))
    return r


def concrete02_row(fc, epsc0=0.002, fcu_ratio=0.2, epscu=0.006, rat=0.1, ft_ratio=0.1):
    """`uniaxialMaterial Concrete02 tag fc epsc0 fcu epscu lambda ft Ets` with
    ft = ft_ratio*fc and Ets = ft_ratio*fc/epsc0 (magnitudes; signs forced
    negative by the material for the compressive values)."""
    r = np.zeros(XG_UNI_NPARAM)
    r[:7] = [-fc, -epsc0, -fcu_ratio * fc, -epscu, rat, ft_ratio * fc, ft_ratio * fc / epsc0]
    return r


def wide_flange_fibers(d=0.4, bf=0.2, tf=0.015, tw=0.01, nf=40):
    """Fibers (y, A) of a wide-flange section about its strong axis: nf/4 per
    flange, nf/2 in the web."""
    nfl, nw = nf // 4, nf - 2 * (nf // 4)
    ys, As = [], []
    hw = d - 2 * tf
    for k in range(nfl):                       # top flange
        ys.append(d / 2 - tf * (k + 0.5) / nfl)
        As.append(bf * tf / nfl)
    for k in range(nw):                        # web
        ys.append(hw / 2 - hw * (k + 0.5) / nw)
        As.append(tw * hw / nw)
    for k in range(nfl):                       # bottom flange
        ys.append(-d / 2 + tf * (k + 0.5) / nfl)
        As.append(bf * tf / nfl)
    return np.array(ys), np.array(As)


def steel_frame_2d(bays=2, stories=3, bay=6.0, story=3.5, nfib=40, fy=350e6, E=200e9,
                   b=0.01, pdelta=0, gravity=-150e3, drift=0.02, steps=20, grav_steps=10,
                   max_iter=50, tol=1e-10, seed=None, law="Steel02"):
    """2D steel moment frame: `forceBeamColumn` columns and beams with 5
    Lobatto points and Steel02 (or, with law="Steel01", Steel01)
    wide-flange fiber sections, base fixed,
    gravity at every floor node (LoadControl, then `loadConst -time 0`), and a
    lateral pushover of the roof-left node by DisplacementControl against a
    triangular reference load pattern."""
    rng = np.random.default_rng(seed) if seed is not None else None
    nx = bays + 1
    tags, crd = [], []
    for j in range(stories + 1):
        for i in range(nx):
            tags.append(j * nx + i + 1)
            crd.append([i * bay, j * story])
    crd = np.asarray(crd)
    conn, sec = [], []
    for j in range(stories):                   # columns
        for i in range(nx):
            conn.append([j * nx + i + 1, (j + 1) * nx + i + 1])
            sec.append(0)
    for j in range(1, stories + 1):            # beams
        for i in range(bays):
            conn.append([j * nx + i + 1, j * nx + i + 2])
            sec.append(1)
    ne = len(conn)
    if rng is not None:
        fy = float(np.exp(rng.normal(np.log(fy), 0.1)))
        b = float(rng.uniform(0.005, 0.02))
    yc, Ac = wide_flange_fibers(0.45, 0.3, 0.022, 0.014, nfib)
    yb, Ab = wide_flange_fibers(0.5, 0.2, 0.016, 0.010, nfib)
    uni = np.stack([steel_row(law, fy, E, b)])
    fib_y = np.concatenate([yc, yb])
    fib_A = np.concatenate([Ac, Ab])
    fib_m = np.zeros(len(fib_y), np.int32)
    sp_node = np.repeat(np.arange(1, nx + 1), 3)
    sp_dof = np.tile([0, 1, 2], nx)
    floors = np.arange(nx + 1, (stories + 1) * nx + 1)
    roof_left = stories * nx + 1
    load_node = list(floors) + [j * nx + 1 for j in range(1, stories + 1)]
    load_pat = [0] * len(floors) + [1] * stories
    load_val = [[0.0, gravity, 0.0]] * len(floors) + \
               [[float(j) / stories, 0.0, 0.0] for j in range(1, stories + 1)]
    desc = ModelDesc(
        ndm=2, ndf=3, elem_type=XG_ELE_FBC2D, geom_transf=pdelta, fbc_num_ip=5,
        node_tag=tags, node_crd=crd,
        elem_tag=np.arange(1, ne + 1), elem_conn=conn, elem_mat=sec,
        uni_type=[steel_type(law)], uni_param=uni,
        sec_fiber_start=[0, nfib, 2 * nfib], fib_y=fib_y, fib_area=fib_A, fib_mat=fib_m,
        sp_node=sp_node, sp_dof=sp_dof, sp_pattern=np.full(len(sp_node), -1),
        sp_value=np.zeros(len(sp_node)),
        load_node=load_node, load_pattern=load_pat, load_value=load_val,
    )
    H = stories * story
    desc.meta = dict(workload=f"2D steel frame {bays}x{stories}", fibers=ne * 5 * nfib,
                     roof=roof_left)
    phases = [
        PhaseDesc(integrator=XG_INT_LOAD_CONTROL, pattern=0, num_steps=grav_steps,
                  d_lambda=1.0 / grav_steps, tol=tol, max_iter=max_iter, load_const=1),
        PhaseDesc(integrator=XG_INT_DISP_CONTROL, pattern=1, num_steps=steps,
                  dc_node=roof_left, dc_dof=0, dc_incr=drift * H / steps, tol=tol,
                  max_iter=max_iter),
    ]
    return desc, phases


def settlement_frame_2d(bays=2, stories=3, settlement=-0.03, steps=12, grav_steps=10,
                        **kw):
    """The 2D steel frame of ``steel_frame_2d`` under `constraints
    Transformation`: its middle (or second) base node settles vertically by
    ``settlement`` metres, imposed as an `sp` in the gravity pattern and so
    applied with the gravity load by LoadControl; after `loadConst` the
    settled support holds while the pushover runs."""
    desc, phases = steel_frame_2d(bays, stories, steps=steps, grav_steps=grav_steps, **kw)
    a = desc.arrays
    settle_node = bays // 2 + 1
    sp_node = np.asarray(a["sp_node"]).copy()
    sp_dof = np.asarray(a["sp_dof"]).copy()
    sp_pat = np.asarray(a["sp_pattern"]).copy()
    sp_val = np.asarray(a["sp_value"]).copy()
    k = int(np.nonzero((sp_node == settle_node) & (sp_dof == 1))[0][0])
    sp_pat[k] = 0
    sp_val[k] = settlement
    kw_ = {key: v for key, v in a.items() if v is not None}
    kw_.update(sp_pattern=sp_pat, sp_value=sp_val)
    out = ModelDesc(ndm=desc.ndm, ndf=desc.ndf, elem_type=desc.elem_type,
                    geom_transf=desc.geom_transf, fbc_num_ip=desc.fbc_num_ip,
                    handler=XG_HANDLER_TRANSFORMATION, **kw_)
    out.meta = dict(desc.meta, workload=f"2D steel frame {bays}x{stories}, support settlement "
                                        f"{settlement} m (Transformation handler)")
    return out, phases


def rc_section_fibers(b, h, cover, n_core_y, n_core_z, n_cover, n_bars, bar_area):
    """Fibers (y, z, A, kind) of a rectangular RC section: a core patch
    n_core_y x n_core_z, a cover ring of n_cover fibers, and n_bars bars on
    the core perimeter.  kind 0 core concrete, 1 cover concrete, 2 steel."""
    ys, zs, As, kind = [], [], [], []
    bc, hc = b - 2 * cover, h - 2 * cover
    for i in range(n_core_y):
        for k in range(n_core_z):
            ys.append(-hc / 2 + hc * (i + 0.5) / n_core_y)
            zs.append(-bc / 2 + bc * (k + 0.5) / n_core_z)
            As.append(bc * hc / (n_core_y * n_core_z))
            kind.append(0)
    per_side = n_cover // 4
    sides = [((-h / 2 + cover / 2, -b / 2), (-h / 2 + cover / 2, b / 2), b * cover),
             ((h / 2 - cover / 2, -b / 2), (h / 2 - cover / 2, b / 2), b * cover),
             ((-hc / 2, -b / 2 + cover / 2), (hc / 2, -b / 2 + cover / 2), hc * cover),
             ((-hc / 2, b / 2 - cover / 2), (hc / 2, b / 2 - cover / 2), hc * cover)]
    for (p0, p1, area) in sides:
        for k in range(per_side):
            t = (k + 0.5) / per_side
            ys.append(p0[0] + t * (p1[0] - p0[0]))
            zs.append(p0[1] + t * (p1[1] - p0[1]))
            As.append(area / per_side)
            kind.append(1)
    per = n_bars // 4
    corners = [(-hc / 2, -bc / 2), (-hc / 2, bc / 2), (hc / 2, bc / 2), (hc / 2, -bc / 2)]
    for s in range(4):
        a, c = corners[s], corners[(s + 1) % 4]
        for k in range(per):
            t = k / per
            ys.append(a[0] + t * (c[0] - a[0]))
            zs.append(a[1] + t * (c[1] - a[1]))
            As.append(bar_area)
            kind.append(2)
    return np.array(ys), np.array(zs), np.array(As), np.array(kind)


def rc_frame_3d(bays_x=10, bays_y=10, stories=20, bay=6.0, story=3.5, col_fibers=120,
                beam_fibers=64, pdelta=1, drift=0.02, steps=200, grav_steps=10, seed=0,
                gravity=-250e3, max_iter=50, tol=1e-10):
    """3D RC frame of `forceBeamColumn` elements (5 Lobatto points) with
    Concrete02 (cover fc 28 MPa, core fc 45 MPa at the base falling linearly
    to 28 MPa at the roof) and Steel02 (fy 420 MPa, E 200 GPa, b 0.01, R0 18)
    fiber sections and elastic torsion, `geomTransf PDelta`; gravity at every
    floor node by LoadControl then `loadConst`; pushover of a roof corner in x
    by DisplacementControl to ``drift`` of the height against a triangular
    reference pattern.  Column sections have ``col_fibers`` fibers, beams
    ``beam_fibers``."""
    rng = np.random.default_rng(seed)
    nxn, nyn = bays_x + 1, bays_y + 1
    per_floor = nxn * nyn

    def nid(i, j, k):
        return k * per_floor + j * nxn + i + 1

    tags, crd = [], []
    for k in range(stories + 1):
        for j in range(nyn):
            for i in range(nxn):
                tags.append(nid(i, j, k))
                crd.append([i * bay, j * bay, k * story])
    crd = np.asarray(crd)
    # materials: 0 cover, 1..stories core by story, last steel
    core_fc = 45e6 - (45e6 - 28e6) * np.arange(stories) / max(stories - 1, 1)
    core_fc *= 1.0 + 0.02 * rng.uniform(-1, 1, size=stories)
    uni_rows = [concrete02_row(28e6, 0.002, 0.2, 0.006)]
    for fc in core_fc:
        uni_rows.append(concrete02_row(fc, 0.002, 0.2, 0.02))
    uni_rows.append(steel02_row(420e6, 200e9, 0.01, 18.0))
    steel = len(uni_rows) - 1
    uni_type = [XG_UNI_CONCRETE02] * (stories + 1) + [XG_UNI_STEEL02]
    # sections: columns per story, beams per story
    def fibers_for(total, b, h):
        n_bars = 16 if total >= 100 else (8 if total >= 40 else 4)
        n_cover = 40 if total >= 100 else (16 if total >= 40 else 8)
        rest = total - n_bars - n_cover
        ny = int(np.floor(np.sqrt(rest)))
        while rest % ny:
            ny -= 1
        return rc_section_fibers(b, h, 0.04, ny, rest // ny, n_cover, n_bars,
                                 0.0005 if total >= 100 else 0.0004)
    sec_start, fy_, fz_, fA_, fm_, GJ = [0], [], [], [], [], []
    Gc = 12e9
    for k in range(stories):
        for (total, b, h) in ((col_fibers, 0.6, 0.6), (beam_fibers, 0.4, 0.6)):
            y, z, A, kind = fibers_for(total, b, h)
            mat = np.where(kind == 0, 1 + k, np.where(kind == 1, 0, steel))
            fy_.append(y); fz_.append(z); fA_.append(A); fm_.append(mat)
            sec_start.append(sec_start[-1] + len(y))
            J = 0.141 * max(b, h) * min(b, h) ** 3
            GJ.append(Gc * J)
    conn, sec, vecxz = [], [], []
    for k in range(stories):                    # columns
        for j in range(nyn):
            for i in range(nxn):
                conn.append([nid(i, j, k), nid(i, j, k + 1)])
                sec.append(2 * k)
                vecxz.append([1.0, 0.0, 0.0])
    for k in range(1, stories + 1):             # beams in x, then in y
        for j in range(nyn):
            for i in range(bays_x):
                conn.append([nid(i, j, k), nid(i + 1, j, k)])
                sec.append(2 * (k - 1) + 1)
                vecxz.append([0.0, 0.0, 1.0])
        for j in range(bays_y):
            for i in range(nxn):
                conn.append([nid(i, j, k), nid(i, j + 1, k)])
                sec.append(2 * (k - 1) + 1)
                vecxz.append([0.0, 0.0, 1.0])
    ne = len(conn)
    base = [nid(i, j, 0) for j in range(nyn) for i in range(nxn)]
    sp_node = np.repeat(base, 6)
    sp_dof = np.tile(np.arange(6), len(base))
    floors = [nid(i, j, k) for k in range(1, stories + 1) for j in range(nyn) for i in range(nxn)]
    roof = nid(0, 0, stories)
    lat_nodes = [nid(0, 0, k) for k in range(1, stories + 1)]
    load_node = floors + lat_nodes
    load_pat = [0] * len(floors) + [1] * len(lat_nodes)
    load_val = [[0.0, 0.0, gravity, 0.0, 0.0, 0.0]] * len(floors) + \
               [[float(k) / stories, 0, 0, 0, 0, 0] for k in range(1, stories + 1)]
    desc = ModelDesc(
        ndm=3, ndf=6, elem_type=XG_ELE_FBC3D, geom_transf=pdelta, fbc_num_ip=5,
        node_tag=tags, node_crd=crd,
        elem_tag=np.arange(1, ne + 1), elem_conn=conn, elem_mat=sec, elem_vecxz=vecxz,
        uni_type=uni_type, uni_param=np.stack(uni_rows),
        sec_fiber_start=sec_start, fib_y=np.concatenate(fy_), fib_z=np.concatenate(fz_),
        fib_area=np.concatenate(fA_), fib_mat=np.concatenate(fm_), sec_GJ=GJ,
        sp_node=sp_node, sp_dof=sp_dof, sp_pattern=np.full(len(sp_node), -1),
        sp_value=np.zeros(len(sp_node)),
        load_node=load_node, load_pattern=load_pat, load_value=load_val,
    )
    H = stories * story
    nfib = sum(np.diff(sec_start)[sec[e]] for e in range(ne)) * 5
    desc.meta = dict(workload=f"3D RC frame {bays_x}x{bays_y}x{stories}", roof=roof,
                     fiber_points=int(nfib), elements=ne)
    phases = [
        PhaseDesc(integrator=XG_INT_LOAD_CONTROL, pattern=0, num_steps=grav_steps,
                  d_lambda=1.0 / grav_steps, tol=tol, max_iter=max_iter, load_const=1),
        PhaseDesc(integrator=XG_INT_DISP_CONTROL, pattern=1, num_steps=steps,
                  dc_node=roof, dc_dof=0, dc_incr=drift * H / steps, tol=tol,
                  max_iter=max_iter),
    ]
    return desc, phases


# ---------------------------------------------------------------------------
# transient: synthetic ground motions and frames under them
# ---------------------------------------------------------------------------
G = 9.81


def kanai_tajimi(npts, dt, pga, seed, wg=15.6, zg=0.6, t_rise=2.0, t_decay=None):
    """Seeded Kanai-Tajimi filtered white noise (ground filter frequency wg,
    damping zg) under a trapezoidal envelope, scaled to peak ground
    acceleration ``pga`` (m/s^2).  The filter is integrated exactly for a
    piecewise-constant input over each sample interval."""
    rng = np.random.default_rng(seed)
    w = rng.normal(size=npts)
    A = np.array([[0.0, 1.0], [-wg * wg, -2.0 * zg * wg]])
    lam, V = np.linalg.eig(A)
    Ad = np.real(V @ np.diag(np.exp(lam * dt)) @ np.linalg.inv(V))
    Bd = np.real(np.linalg.solve(A, (Ad - np.eye(2)) @ np.array([0.0, -1.0])))
    x = np.zeros(2)
    ag = np.zeros(npts)
    for k in range(npts):
        x = Ad @ x + Bd * w[k]
        ag[k] = -(2.0 * zg * wg * x[1] + wg * wg * x[0])
    t = np.arange(npts) * dt
    T = npts * dt
    t_decay = 0.3 * T if t_decay is None else t_decay
    env = np.minimum(1.0, t / t_rise) * np.minimum(1.0, np.maximum(0.0, (T - t) / t_decay))
    ag *= env
    peak = np.abs(ag).max()
    return ag * (pga / peak) if peak > 0 else ag


def rayleigh_2pct(stories, zeta=0.02):
    """Rayleigh factors (alphaM, betaK0) giving ``zeta`` at the first and third
    modes, with the periods estimated as T1 = 0.1 s per story and T3 = T1/5
    (a uniform shear building's third mode), so no eigen-solution is needed
    for thousands of frames; betaK multiplies the initial stiffness."""
    w1 = 2.0 * np.pi / (0.1 * stories)
    w3 = 5.0 * w1
    return 2.0 * zeta * w1 * w3 / (w1 + w3), 2.0 * zeta / (w1 + w3)


def steel_frame_2d_eq(bays=2, stories=3, steps=200, dt=0.01, pga=0.4 * G, seed=1,
                      grav_steps=10, floor_mass=None, with_gravity=True, record=None,
                      **frame_kw):
    """The 2D steel frame of ``steel_frame_2d`` with lumped floor masses (the
    gravity load over g at every floor node, horizontal and vertical),
    gravity by LoadControl then `loadConst`, and a transient phase:
    `integrator Newmark 0.5 0.25`, 2 % Rayleigh on the initial stiffness,
    `pattern UniformExcitation` in x with a Kanai-Tajimi record."""
    kw = dict(frame_kw)
    kw.setdefault("seed", seed)
    desc, phases = steel_frame_2d(bays, stories, steps=1, grav_steps=grav_steps, **kw)
    gravity = kw.get("gravity", -150e3)
    m = abs(gravity) / G if floor_mass is None else floor_mass
    nn = desc.num_nodes
    mass = np.zeros((nn, 3))
    tags = np.asarray(desc.node_tag)
    crd = desc.node_crd.reshape(-1, 2)
    mass[crd[:, 1] > 0, 0] = m
    mass[crd[:, 1] > 0, 1] = m
    desc.arrays["node_mass"] = mass.ravel()
    am, bk0 = rayleigh_2pct(stories)
    rec = kanai_tajimi(steps + 2, dt, pga, seed + 1000) if record is None else record
    quake = PhaseDesc(integrator=XG_INT_NEWMARK, pattern=2, num_steps=steps, dt=dt,
                      gamma=0.5, beta=0.25, alpha_m=am, beta_k_init=bk0, gm_dof=0,
                      gm_accel=rec, gm_dt=dt, tol=1e-10, max_iter=50)
    phases = [phases[0], quake] if with_gravity else [quake]
    desc.meta = dict(desc.meta, record_pga=pga, alpha_m=am, beta_k0=bk0)
    del tags
    return desc, phases


def kanai_tajimi_batch(n, npts, dt, pgas, seed, wg=15.6, zg=0.6, t_rise=2.0):
    """``n`` Kanai-Tajimi records at once (the filter of ``kanai_tajimi``
    stepped over all records together), record r scaled to ``pgas[r]``."""
    rng = np.random.default_rng(seed)
    w = rng.normal(size=(n, npts))
    A = np.array([[0.0, 1.0], [-wg * wg, -2.0 * zg * wg]])
    lam, V = np.linalg.eig(A)
    Ad = np.real(V @ np.diag(np.exp(lam * dt)) @ np.linalg.inv(V))
    Bd = np.real(np.linalg.solve(A, (Ad - np.eye(2)) @ np.array([0.0, -1.0])))
    x = np.zeros((2, n))
    ag = np.zeros((n, npts))
    for k in range(npts):
        x = Ad @ x + Bd[:, None] * w[:, k][None, :]
        ag[:, k] = -(2.0 * zg * wg * x[1] + wg * wg * x[0])
    t = np.arange(npts) * dt
    T = npts * dt
    env = np.minimum(1.0, t / t_rise) * np.minimum(1.0, np.maximum(0.0, (T - t) / (0.3 * T)))
    ag *= env[None, :]
    peak = np.abs(ag).max(axis=1)
    return ag * (np.asarray(pgas) / np.where(peak > 0, peak, 1.0))[:, None]


def frame_batch(n_frames=4096, steps=2000, dt=0.01, seed=0, nfib=40, return_parts=False):
    """``n_frames`` independent 2D steel moment frames in one model: bays
    uniform in 1..12 and stories in 2..20, 40-fiber Steel02 wide-flange
    sections with fy lognormal (median 350 MPa, CoV 0.1) and b uniform in
    [0.005, 0.02] per frame, lumped floor masses, each under its own seeded
    Kanai-Tajimi record (PGA uniform in [0.1, 0.8] g, dt 0.01 s), Newmark
    (0.5, 0.25), 2 % Rayleigh on the initial stiffness with every frame's
    own factors.  The frames share no node, so the model's parts converge
    one by one; ``return_parts`` also returns every frame's own (desc,
    phases) for comparisons."""
    rng = np.random.default_rng(seed)
    bays = rng.integers(1, 13, size=n_frames)
    stories = rng.integers(2, 21, size=n_frames)
    pgas = rng.uniform(0.1, 0.8, size=n_frames) * G
    recs = kanai_tajimi_batch(n_frames, steps + 2, dt, pgas, seed + 7)
    keys = ("node_tag", "node_crd", "node_mass", "elem_tag", "elem_conn", "elem_mat",
            "uni_param", "fib_y", "fib_area", "fib_mat", "sp_node", "sp_dof", "sp_pattern",
            "sp_value")
    acc = {k: [] for k in keys}
    uni_type, sec_start, node_rec, am_node, bk0_elem = [], [0], [], [], []
    parts = []
    node_off = elem_off = sec_off = uni_off = fib_off = 0
    for f in range(n_frames):
        d, ph = steel_frame_2d_eq(int(bays[f]), int(stories[f]), steps=steps, dt=dt,
                                  seed=seed * 100003 + f + 1, with_gravity=False,
                                  record=recs[f], nfib=nfib)
        a = d.arrays
        if return_parts:
            parts.append((d, ph))
        nn, ne = len(a["node_tag"]), len(a["elem_tag"])
        acc["node_tag"].append(np.asarray(a["node_tag"]) + node_off)
        acc["node_crd"].append(np.asarray(a["node_crd"]).reshape(-1, 2))
        acc["node_mass"].append(np.asarray(a["node_mass"]))
        acc["elem_tag"].append(np.asarray(a["elem_tag"]) + elem_off)
        acc["elem_conn"].append(np.asarray(a["elem_conn"]).reshape(-1, 2) + node_off)
        acc["elem_mat"].append(np.asarray(a["elem_mat"]) + sec_off)
        acc["uni_param"].append(np.asarray(a["uni_param"]).reshape(-1, XG_UNI_NPARAM))
        acc["fib_y"].append(np.asarray(a["fib_y"]))
        acc["fib_area"].append(np.asarray(a["fib_area"]))
        acc["fib_mat"].append(np.asarray(a["fib_mat"]) + uni_off)
        acc["sp_node"].append(np.asarray(a["sp_node"]) + node_off)
        acc["sp_dof"].append(np.asarray(a["sp_dof"]))
        acc["sp_pattern"].append(np.asarray(a["sp_pattern"]))
        acc["sp_value"].append(np.asarray(a["sp_value"]))
        uni_type.extend(list(np.asarray(a["uni_type"])))
        ss = np.asarray(a["sec_fiber_start"])
        sec_start.extend(list(ss[1:] + fib_off))
        node_rec.extend([f] * nn)
        am_node.extend([ph[0].alpha_m] * nn)
        bk0_elem.extend([ph[0].beta_k_init] * ne)
        node_off = int(acc["node_tag"][-1].max())
        elem_off = int(acc["elem_tag"][-1].max())
        sec_off += len(ss) - 1
        uni_off += len(a["uni_type"])
        fib_off += int(ss[-1])
    cat = {k: np.concatenate(v) for k, v in acc.items()}
    desc = ModelDesc(
        ndm=2, ndf=3, elem_type=XG_ELE_FBC2D, geom_transf=0, fbc_num_ip=5,
        node_tag=cat["node_tag"], node_crd=cat["node_crd"], node_mass=cat["node_mass"],
        elem_tag=cat["elem_tag"], elem_conn=cat["elem_conn"], elem_mat=cat["elem_mat"],
        uni_type=uni_type, uni_param=cat["uni_param"], sec_fiber_start=sec_start,
        fib_y=cat["fib_y"], fib_area=cat["fib_area"], fib_mat=cat["fib_mat"],
        sp_node=cat["sp_node"], sp_dof=cat["sp_dof"], sp_pattern=cat["sp_pattern"],
        sp_value=cat["sp_value"])
    nfp = int(np.diff(np.asarray(sec_start))[cat["elem_mat"]].sum() * 5)
    desc.meta = dict(workload=f"{n_frames} 2D steel frames", frames=n_frames,
                     fiber_points=nfp, elements=len(cat["elem_tag"]),
                     nodes=len(cat["node_tag"]))
    quake = PhaseDesc(integrator=XG_INT_NEWMARK, pattern=2, num_steps=steps, dt=dt,
                      gamma=0.5, beta=0.25, gm_dof=0, gm_accel=recs, gm_dt=dt,
                      gm_node_record=np.asarray(node_rec, np.int32),
                      alpha_m_node=np.asarray(am_node), beta_k_init_elem=np.asarray(bk0_elem),
                      tol=1e-10, max_iter=50)
    if return_parts:
        return desc, [quake], parts
    return desc, [quake]


def adjoint_frames(n_frames=64, steps=2000, dt=0.01, seed=0, nfib=40, member_cov=0.05,
                   pga_scale=1.0):
    """Frames of the batched-frames workload with one Steel02 material per
    member (fy and b varied per member by a lognormal factor of CoV
    ``member_cov``), for gradients with respect to per-member parameters.
    The objective terms in ``desc.meta`` are every frame's roof drift: the
    roof-left node's horizontal displacement over the frame height, squared
    and summed over the steps (node tags, dof 0, weight 1/H^2)."""
    desc, phases = frame_batch(n_frames=n_frames, steps=steps, dt=dt, seed=seed, nfib=nfib)
    a = desc.arrays
    ss, em, fmat = a["sec_fiber_start"], a["elem_mat"], a["fib_mat"]
    uni = a["uni_param"].reshape(-1, XG_UNI_NPARAM)
    rng = np.random.default_rng(seed + 11)
    ne = len(em)
    lo, hi = ss[em], ss[em + 1]
    counts = hi - lo
    idx = np.concatenate([np.arange(l, h) for l, h in zip(lo, hi)])
    rows = uni[fmat[lo]].copy()
    rows[:, 0] *= np.exp(rng.normal(0.0, member_cov, ne))
    rows[:, 2] *= np.exp(rng.normal(0.0, member_cov, ne))
    kw = {k: v for k, v in a.items() if v is not None}
    kw.update(elem_mat=np.arange(ne), sec_fiber_start=np.concatenate([[0], np.cumsum(counts)]),
              fib_y=a["fib_y"][idx], fib_area=a["fib_area"][idx],
              fib_mat=np.repeat(np.arange(ne), counts), uni_type=np.full(ne, XG_UNI_STEEL02),
              uni_param=rows)
    out = ModelDesc(ndm=desc.ndm, ndf=desc.ndf, elem_type=desc.elem_type,
                    geom_transf=desc.geom_transf, fbc_num_ip=desc.fbc_num_ip, **kw)
    ph = phases[0]
    rec = np.asarray(ph.gm_node_record)
    crd = a["node_crd"].reshape(-1, 2)
    tags = a["node_tag"]
    obj_node, obj_w = [], []
    for f in range(n_frames):
        nodes = np.nonzero(rec == f)[0]
        top = crd[nodes, 1].max()
        roof = nodes[crd[nodes, 1] == top]
        obj_node.append(int(tags[roof[np.argmin(crd[roof, 0])]]))
        obj_w.append(1.0 / (top * top))
    if pga_scale != 1.0:
        ph.gm_accel = np.ascontiguousarray(ph.gm_accel * pga_scale)
    node_idx = {int(t): i for i, t in enumerate(tags)}
    member_frame = rec[[node_idx[int(n_)] for n_ in a["elem_conn"].reshape(-1, 2)[:, 0]]]
    out.meta = dict(desc.meta, workload=f"{n_frames} 2D steel frames, one Steel02 per member",
                    member_frame=np.asarray(member_frame),
                    obj_node=np.asarray(obj_node, np.int32),
                    obj_dof=np.zeros(n_frames, np.int32), obj_weight=np.asarray(obj_w),
                    members=ne)
    return out, [ph]



def ddm_steel01_frame(bays=2, stories=3, steps=100, dt=0.01, base_shear=720e3, seed=3,
                      member_cov=0.05, nfib=40):
    """One 2D steel frame for comparing gradients with the reference's DDM
    sensitivity (its Steel01 has stress sensitivities, its Steel02 has
    none).  The reference's transient DDM cannot run with nodal mass
    (Node::getMassSensitivity, domain/node/Node.cpp:1445-1469, returns a
    local Matrix through the move constructor, which throws,
    matrix/Matrix.cpp:130-141), so the frame carries no mass and no
    damping: `integrator Newmark 0.5 0.25` with a triangular lateral load
    pattern on a Linear series, ramped to ``base_shear`` at the last step (1.5 %
    roof drift for the default frame) -- a path-dependent, quasi-static
    response through yielding.  One Steel01 material per member (fy and b
    varied by a lognormal factor of CoV ``member_cov``, E 200 GPa).  The
    objective is the summed squared roof drift, as in
    :func:`adjoint_frames`."""
    desc, _ = steel_frame_2d(bays, stories, steps=1, grav_steps=1, law="Steel01", gravity=0.0,
                             nfib=nfib)
    a = desc.arrays
    ss, em = a["sec_fiber_start"], a["elem_mat"]
    uni = a["uni_param"].reshape(-1, XG_UNI_NPARAM)
    rng = np.random.default_rng(seed + 13)
    ne = len(em)
    lo, hi = ss[em], ss[em + 1]
    counts = hi - lo
    idx = np.concatenate([np.arange(l_, h_) for l_, h_ in zip(lo, hi)])
    rows = np.repeat(uni[:1], ne, axis=0)
    rows[:, 0] *= np.exp(rng.normal(0.0, member_cov, ne))
    rows[:, 2] *= np.exp(rng.normal(0.0, member_cov, ne))
    # the lateral pattern only (pattern 0), scaled so that lambda = t reaches
    # the base shear at t = steps * dt
    lat = np.asarray(a["load_pattern"]) == 1
    load_val = np.asarray(a["load_value"]).reshape(-1, 3)[lat] * base_shear / (steps * dt)
    kw = {k: v for k, v in a.items() if v is not None}
    kw.update(elem_mat=np.arange(ne), sec_fiber_start=np.concatenate([[0], np.cumsum(counts)]),
              fib_y=a["fib_y"][idx], fib_area=a["fib_area"][idx],
              fib_mat=np.repeat(np.arange(ne), counts), uni_type=np.full(ne, XG_UNI_STEEL01),
              uni_param=rows, load_node=np.asarray(a["load_node"])[lat],
              load_pattern=np.zeros(int(lat.sum()), np.int32), load_value=load_val)
    out = ModelDesc(ndm=desc.ndm, ndf=desc.ndf, elem_type=desc.elem_type,
                    geom_transf=desc.geom_transf, fbc_num_ip=desc.fbc_num_ip, **kw)
    ramp = PhaseDesc(integrator=XG_INT_NEWMARK, pattern=0, num_steps=steps, dt=dt,
                     gamma=0.5, beta=0.25, tol=1e-10, max_iter=50)
    H = stories * 3.5
    roof = stories * (bays + 1) + 1
    out.meta = dict(desc.meta, workload=f"2D steel frame {bays}x{stories}, one Steel01 per "
                                        f"member, massless Newmark ramp",
                    obj_node=np.array([roof], np.int32), obj_dof=np.zeros(1, np.int32),
                    obj_weight=np.array([1.0 / (H * H)]), members=ne)
    return out, [ramp]


def adjoint_rc_frames(n_frames=2, steps=2000, dt=0.01, seed=0, member_cov=0.05, pga_scale=1.0,
                      ncl=12, laws="02"):
    """The frames of :func:`adjoint_frames` with reinforced-concrete members:
    every member a 0.4 x 0.5 m section of ``ncl`` Concrete02 layers (fc
    30 MPa, epsc0 0.002, fcu 0.2 fc, epscu 0.006, ft 0.1 fc) and two layers of
    Steel02 bars (4 x 491 mm^2 each, 50 mm cover; fy 420 MPa, E 200 GPa,
    b 0.01), one concrete and one steel material per member with fc and fy
    varied by a lognormal factor of CoV ``member_cov``; mass-proportional
    Rayleigh damping only.  Same objective terms as :func:`adjoint_frames`.
    ``laws="01"`` gives the Concrete01 / Steel01 surrogate of the same
    members (fc and fy as above, b 0.01)."""
    desc, phases = adjoint_frames(n_frames=n_frames, steps=steps, dt=dt, seed=seed,
                                  member_cov=member_cov, pga_scale=pga_scale)
    a = desc.arrays
    ne = len(a["elem_tag"])
    rng = np.random.default_rng(seed + 23)
    b, h, cover, bar = 0.4, 0.5, 0.05, 4 * 491e-6
    yc = (np.arange(ncl) + 0.5) * h / ncl - h / 2
    ys = np.array([h / 2 - cover, -(h / 2 - cover)])
    fy_sec = np.concatenate([yc, ys])
    fa_sec = np.concatenate([np.full(ncl, b * h / ncl), np.full(2, bar)])
    nf = ncl + 2
    rows, types = [], []
    fc = 30e6 * np.exp(rng.normal(0.0, member_cov, ne))
    fy = 420e6 * np.exp(rng.normal(0.0, member_cov, ne))
    for e in range(ne):
        if laws == "01":
            rows.append(concrete01_row(fc=fc[e]))
            rows.append(steel01_row(fy=fy[e], E=200e9, b=0.01))
            types += [XG_UNI_CONCRETE01, XG_UNI_STEEL01]
        else:
            rows.append(concrete02_row(fc=fc[e]))
            rows.append(steel02_row(fy=fy[e], E=200e9, b=0.01, R0=18.0))
            types += [XG_UNI_CONCRETE02, XG_UNI_STEEL02]
    fib_mat = np.concatenate([np.r_[np.full(ncl, 2 * e), np.full(2, 2 * e + 1)]
                              for e in range(ne)])
    kw = {k: v for k, v in a.items() if v is not None}
    kw.update(elem_mat=np.arange(ne), sec_fiber_start=np.arange(ne + 1) * nf,
              fib_y=np.tile(fy_sec, ne), fib_area=np.tile(fa_sec, ne), fib_mat=fib_mat,
              uni_type=np.asarray(types), uni_param=np.asarray(rows))
    out = ModelDesc(ndm=desc.ndm, ndf=desc.ndf, elem_type=desc.elem_type,
                    geom_transf=desc.geom_transf, fbc_num_ip=desc.fbc_num_ip, **kw)
    ph = phases[0]
    ph.beta_k_init_elem = np.zeros(ne)
    ph.kw["beta_k_init"] = 0.0
    out.meta = dict(desc.meta, workload=f"{n_frames} 2D RC frames, Concrete02 and Steel02 per "
                    "member")
    return out, [ph]

def _with_geometry(desc, geom_transf=None, **arrays):
    """A copy of ``desc`` with some arrays (and the transformation) replaced."""
    kw = {k: v for k, v in desc.arrays.items() if v is not None}
    kw.update(arrays)
    out = ModelDesc(ndm=desc.ndm, ndf=desc.ndf, elem_type=desc.elem_type,
                    geom_transf=desc.geom_transf if geom_transf is None else geom_transf,
                    fbc_num_ip=desc.fbc_num_ip, **kw)
    out.meta = dict(desc.meta)
    return out


def adjoint_pdelta_frames(n_frames=2, steps=40, dt=0.01, seed=0, pga_scale=1.0,
                          weight_factor=1.0, pdelta=1):
    """The frames of :func:`adjoint_frames` under `geomTransf PDelta` with the
    floor weights as vertical nodal loads in the transient phase's pattern
    (a Linear series, so the loads grow with time to ``weight_factor`` times
    every floor node's weight at the last step): columns carry axial loads
    while the record sways them.  ``pdelta=0`` gives the same model with
    linear transformations."""
    desc, phases = adjoint_frames(n_frames=n_frames, steps=steps, dt=dt, seed=seed,
                                  pga_scale=pga_scale)
    a = desc.arrays
    mass = a["node_mass"].reshape(-1, 3)
    floor = np.nonzero(mass[:, 0] > 0)[0]
    val = np.zeros((len(floor), 3))
    val[:, 1] = -weight_factor * mass[floor, 0] * G / (steps * dt)
    ph = phases[0]
    out = _with_geometry(desc, geom_transf=pdelta, load_node=a["node_tag"][floor],
                         load_pattern=np.full(len(floor), ph.pattern), load_value=val)
    out.meta["workload"] = (f"{n_frames} 2D steel frames under P-Delta, one Steel02 per member, "
                            "growing floor weights")
    return out, [ph]


def adjoint_rc_frame_3d(bays_x=1, bays_y=1, stories=2, steps=40, dt=0.01, seed=0,
                        pga=0.4 * G, pga_scale=1.0, col_fibers=40, beam_fibers=24, pdelta=1,
                        gravity=-250e3):
    """A small 3D RC frame of :func:`rc_frame_3d` (Concrete02 cover and core,
    Steel02 bars, elastic torsion) for gradients of the transient run: floor
    masses (the gravity load over g at every floor node in x, y and z), the
    gravity loads in the transient phase's pattern growing with time to their
    full value at the last step, `integrator Newmark 0.5 0.25`, mass-
    proportional 2 % Rayleigh damping, `pattern UniformExcitation` in x with a
    Kanai-Tajimi record.  The objective terms are the roof corner's x
    displacement over the height, squared and summed over the steps."""
    desc, _ = rc_frame_3d(bays_x, bays_y, stories, col_fibers=col_fibers,
                          beam_fibers=beam_fibers, pdelta=pdelta, steps=1, grav_steps=1,
                          seed=seed, gravity=gravity)
    a = desc.arrays
    crd = a["node_crd"].reshape(-1, 3)
    floor = np.nonzero(crd[:, 2] > 0)[0]
    m = abs(gravity) / G
    mass = np.zeros((len(crd), 6))
    mass[floor, :3] = m
    val = np.zeros((len(floor), 6))
    val[:, 2] = gravity / (steps * dt)
    am, _ = rayleigh_2pct(stories)
    rec = kanai_tajimi(steps + 2, dt, pga * pga_scale, seed + 1000)
    out = _with_geometry(desc, node_mass=mass, load_node=a["node_tag"][floor],
                         load_pattern=np.full(len(floor), 2), load_value=val)
    quake = PhaseDesc(integrator=XG_INT_NEWMARK, pattern=2, num_steps=steps, dt=dt,
                      gamma=0.5, beta=0.25, alpha_m=am, gm_dof=0, gm_accel=rec, gm_dt=dt,
                      tol=1e-10, max_iter=50)
    H = stories * 3.5
    out.meta = dict(desc.meta, workload=f"3D RC frame {bays_x}x{bays_y}x{stories} under a "
                    "ground motion", obj_node=np.array([desc.meta["roof"]], np.int32),
                    obj_dof=np.zeros(1, np.int32), obj_weight=np.array([1.0 / (H * H)]))
    return out, [quake]


def ddm_steel01_frames_eq(n_frames=2, steps=40, dt=0.01, seed=0, pga_scale=1.0):
    """The frames of :func:`adjoint_frames` with their members' Steel02
    replaced by Steel01 of the same fy, E and b (the law whose stress
    sensitivity the reference's DDM has) and mass-proportional Rayleigh
    damping only: a transient, path-dependent case for the direct
    differentiation.  Same objective terms."""
    desc, phases = adjoint_frames(n_frames=n_frames, steps=steps, dt=dt, seed=seed,
                                  pga_scale=pga_scale)
    uni = desc.uni_param.reshape(-1, XG_UNI_NPARAM)
    rows = np.stack([steel01_row(fy=r[0], E=r[1], b=r[2]) for r in uni])
    out = _with_geometry(desc, uni_type=np.full(len(rows), XG_UNI_STEEL01), uni_param=rows)
    ph = phases[0]
    ph.beta_k_init_elem = np.zeros(len(desc.arrays["elem_tag"]))
    ph.kw["beta_k_init"] = 0.0
    out.meta["workload"] = f"{n_frames} 2D steel frames, one Steel01 per member"
    return out, [ph]


def rc_frame_2d(bays=2, stories=3, bay=6.0, story=3.5, ncl=10, fc=30e6, fy=420e6, E=200e9,
                b=0.01, gravity=-100e3, drift=0.015, steps=20, grav_steps=10, max_iter=50,
                tol=1e-10):
    """2D reinforced-concrete frame of `forceBeamColumn` members (5 Lobatto
    points) with layered fiber sections: ``ncl`` Concrete01 layers (fc,
    epsc0 0.002, fcu 0.2 fc, epscu 0.006) and two layers of Steel01 bars
    (fy, E, b; 50 mm cover); columns 0.5 x 0.5 m with 3 x 491 mm^2 per layer,
    beams 0.4 x 0.6 m with 4 x 491 mm^2 per layer.  Gravity at every floor
    node (LoadControl, then `loadConst -time 0`) and a pushover of the
    roof-left node by DisplacementControl against a triangular pattern --
    the Steel01 / Concrete01 surrogate of the reinforced-concrete frames."""
    nx = bays + 1
    tags, crd = [], []
    for j in range(stories + 1):
        for i in range(nx):
            tags.append(j * nx + i + 1)
            crd.append([i * bay, j * story])
    conn, sec = [], []
    for j in range(stories):
        for i in range(nx):
            conn.append([j * nx + i + 1, (j + 1) * nx + i + 1])
            sec.append(0)
    for j in range(1, stories + 1):
        for i in range(bays):
            conn.append([j * nx + i + 1, j * nx + i + 2])
            sec.append(1)
    fib_y, fib_A, fib_m, sec_start = [], [], [], [0]
    for (bw, h, nbar) in ((0.5, 0.5, 3), (0.4, 0.6, 4)):
        yc = (np.arange(ncl) + 0.5) * h / ncl - h / 2
        ys = np.array([h / 2 - 0.05, -(h / 2 - 0.05)])
        fib_y += [yc, ys]
        fib_A += [np.full(ncl, bw * h / ncl), np.full(2, nbar * 491e-6)]
        fib_m += [np.zeros(ncl, np.int32), np.ones(2, np.int32)]
        sec_start.append(sec_start[-1] + ncl + 2)
    uni = np.stack([concrete01_row(fc), steel01_row(fy, E, b)])
    sp_node = np.repeat(np.arange(1, nx + 1), 3)
    sp_dof = np.tile([0, 1, 2], nx)
    floors = np.arange(nx + 1, (stories + 1) * nx + 1)
    load_node = list(floors) + [j * nx + 1 for j in range(1, stories + 1)]
    load_pat = [0] * len(floors) + [1] * stories
    load_val = [[0.0, gravity, 0.0]] * len(floors) + \
               [[float(j) / stories, 0.0, 0.0] for j in range(1, stories + 1)]
    desc = ModelDesc(
        ndm=2, ndf=3, elem_type=XG_ELE_FBC2D, geom_transf=0, fbc_num_ip=5,
        node_tag=tags, node_crd=np.asarray(crd), elem_tag=np.arange(1, len(conn) + 1),
        elem_conn=conn, elem_mat=sec, uni_type=[XG_UNI_CONCRETE01, XG_UNI_STEEL01],
        uni_param=uni, sec_fiber_start=sec_start, fib_y=np.concatenate(fib_y),
        fib_area=np.concatenate(fib_A), fib_mat=np.concatenate(fib_m),
        sp_node=sp_node, sp_dof=sp_dof, sp_pattern=np.full(len(sp_node), -1),
        sp_value=np.zeros(len(sp_node)), load_node=load_node, load_pattern=load_pat,
        load_value=load_val)
    roof = stories * nx + 1
    H = stories * story
    desc.meta = dict(workload=f"2D RC frame {bays}x{stories} (Steel01, Concrete01)",
                     roof=roof, elements=len(conn))
    phases = [
        PhaseDesc(integrator=XG_INT_LOAD_CONTROL, pattern=0, num_steps=grav_steps,
                  d_lambda=1.0 / grav_steps, tol=tol, max_iter=max_iter, load_const=1),
        PhaseDesc(integrator=XG_INT_DISP_CONTROL, pattern=1, num_steps=steps,
                  dc_node=roof, dc_dof=0, dc_incr=drift * H / steps, tol=tol,
                  max_iter=max_iter),
    ]
    return desc, phases


def ddm_rc01_frame(bays=2, stories=3, steps=100, dt=0.01, base_shear=230e3, seed=4,
                   member_cov=0.05, ncl=10):
    """The frame of :func:`rc_frame_2d` as the reference's DDM can run it
    (massless, undamped `integrator Newmark 0.5 0.25` under a triangular
    lateral pattern on a Linear series ramped to ``base_shear`` at the last
    step, no gravity) with one Concrete01 and one Steel01 material per
    member (fc and fy varied by a lognormal factor of CoV ``member_cov``):
    the Steel01 / Concrete01 surrogate frame for comparing gradients with the
    reference's DDM.  Objective: the summed squared roof drift."""
    desc, _ = rc_frame_2d(bays, stories, ncl=ncl, gravity=0.0)
    a = desc.arrays
    ss, em = a["sec_fiber_start"], a["elem_mat"]
    rng = np.random.default_rng(seed)
    ne = len(em)
    lo, hi = ss[em], ss[em + 1]
    counts = hi - lo
    idx = np.concatenate([np.arange(l_, h_) for l_, h_ in zip(lo, hi)])
    fm = a["fib_mat"][idx] + 2 * np.repeat(np.arange(ne), counts)
    fcs = 30e6 * np.exp(rng.normal(0.0, member_cov, ne))
    fys = 420e6 * np.exp(rng.normal(0.0, member_cov, ne))
    rows, types = [], []
    for e in range(ne):
        rows += [concrete01_row(fcs[e]), steel01_row(fys[e], 200e9, 0.01)]
        types += [XG_UNI_CONCRETE01, XG_UNI_STEEL01]
    lat = np.asarray(a["load_pattern"]) == 1
    load_val = np.asarray(a["load_value"]).reshape(-1, 3)[lat] * base_shear / (steps * dt)
    kw = {k: v for k, v in a.items() if v is not None}
    kw.update(elem_mat=np.arange(ne), sec_fiber_start=np.concatenate([[0], np.cumsum(counts)]),
              fib_y=a["fib_y"][idx], fib_area=a["fib_area"][idx], fib_mat=fm,
              uni_type=np.asarray(types), uni_param=np.stack(rows),
              load_node=np.asarray(a["load_node"])[lat],
              load_pattern=np.zeros(int(lat.sum()), np.int32), load_value=load_val)
    out = ModelDesc(ndm=2, ndf=3, elem_type=desc.elem_type, geom_transf=0,
                    fbc_num_ip=desc.fbc_num_ip, **kw)
    ramp = PhaseDesc(integrator=XG_INT_NEWMARK, pattern=0, num_steps=steps, dt=dt,
                     gamma=0.5, beta=0.25, tol=1e-10, max_iter=50)
    H = stories * 3.5
    out.meta = dict(workload=f"2D RC frame {bays}x{stories}, one Concrete01 and one Steel01 "
                             "per member, massless Newmark ramp",
                    obj_node=np.array([desc.meta["roof"]], np.int32),
                    obj_dof=np.zeros(1, np.int32), obj_weight=np.array([1.0 / (H * H)]),
                    members=ne)
    return out, [ramp]
