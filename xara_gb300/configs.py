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
                   XG_HANDLER_PLAIN, XG_INT_DISP_CONTROL, XG_TEST_NORM_DISP_INCR)

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
