/*
 * xara_gpu.h -- C ABI of libxara_gpu.so, the GB300 implementation of the
 * xara/OpenSees Newton-iteration hot path (element state determination,
 * material updates, global assembly and the linear solve of one load or
 * time step).
 *
 * Conventions (all entry points):
 *   - return 0 on success, a negative XG_E* code on failure; the last error
 *     text is available from xg_last_error();
 *   - host arrays are borrowed for the duration of the call only;
 *   - device memory never crosses the boundary: every handle owns its device
 *     buffers and one CUDA stream, and calls on one handle are synchronous
 *     and not reentrant (the reference path is single threaded as well);
 *   - all arithmetic is IEEE FP64, all counts and indices are int32.
 *
 * Each entry point names the reference interface it replaces
 * (paths are relative to the reference's SRC/ directory).
 */
#ifndef XARA_GPU_H
#define XARA_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

/* ----------------------------------------------------------------------- */
/* error codes                                                               */
/* ----------------------------------------------------------------------- */
#define XG_OK              0
#define XG_EINVAL         -1   /* bad argument or model description        */
#define XG_ECUDA          -2   /* CUDA runtime error                       */
#define XG_ENOMEM         -3   /* device allocation failed                 */
#define XG_ESOLVE         -4   /* linear solve failed (breakdown / maxit)  */
#define XG_ENOCONV        -5   /* Newton test failed (TestFailed)          */
#define XG_EELEMENT       -6   /* element state determination failed       */
#define XG_ESTATE         -7   /* call out of sequence                     */

/* element families (one family per model) */
#define XG_ELE_QUAD        1   /* element/Plane/FourNodeQuad.cpp           */
#define XG_ELE_BRICK       2   /* element/Brick/Brick.cpp                  */
#define XG_ELE_FBC2D       3   /* element/Frame/Other/Force/ForceBeamColumn2d.cpp */
#define XG_ELE_FBC3D       4   /* element/Frame/Other/Force/ForceBeamColumn3d.cpp */

/* uniaxial material laws (fiber sections) */
#define XG_UNI_STEEL02     1   /* material/uniaxial/steel/Steel02.cpp      */
#define XG_UNI_CONCRETE02  2   /* material/uniaxial/concrete/Concrete02.cpp */
#define XG_UNI_ELASTIC     3   /* linear elastic fiber (known-answer tests) */
#define XG_UNI_STEEL01     4   /* material/uniaxial/steel/Steel01.cpp      */
#define XG_UNI_CONCRETE01  5   /* material/uniaxial/concrete/Concrete01.cpp */

/* constraint handlers (analysis/handler) */
#define XG_HANDLER_PLAIN           0  /* PlainHandler.cpp                   */
#define XG_HANDLER_TRANSFORMATION  1  /* TransformationConstraintHandler.cpp */

/* integrators */
#define XG_INT_LOAD_CONTROL   0  /* analysis/integrator/Static/LoadControl.cpp          */
#define XG_INT_DISP_CONTROL   1  /* analysis/integrator/Static/DisplacementControl.cpp  */
#define XG_INT_NEWMARK        2  /* analysis/integrator/Dynamic/Newmark.cpp              */

/* convergence tests */
#define XG_TEST_NORM_DISP_INCR  0  /* analysis/criteria/CTestNormDispIncr.cpp */
#define XG_TEST_NORM_UNBALANCE  1  /* analysis/criteria/CTestNormUnbalance.cpp */

/* linear systems */
#define XG_SYSTEM_BJPCG    0   /* block-Jacobi PCG on the device (new `system CudaBJPCG`) */
#define XG_SYSTEM_PROFILE_SPD 1 /* skyline LDL' on the device (`system ProfileSPD`,
                                  system_of_eqn/linearSOE/profileSPD/ProfileSPDLinDirectSolver.cpp) */

/* J2 parameter row (nDMaterial J2Plasticity, material/plastic/J2Plasticity.cpp:84-111) */
#define XG_J2_NPARAM 8         /* K G sigma0 sigma_inf delta H eta rho */
/* uniaxial parameter row, Steel02: fy E0 b R0 cR1 cR2 a1 a2 a3 a4 sigInit
   (material/uniaxial/steel/Steel02.h:47-50); Concrete02: fc epsc0 fcu epscu
   rat ft Ets (material/uniaxial/concrete/Concrete02.h:48-49); Steel01: fy
   E0 b a1 a2 a3 a4 (material/uniaxial/steel/Steel01.h:48-49); Elastic: E */
#define XG_UNI_NPARAM 12

/*
 * Model description: the data the reference's modelling commands
 * (`node`, `fix`, `element quad|stdBrick|forceBeamColumn`, `nDMaterial
 * J2Plasticity`, `uniaxialMaterial Steel02|Concrete02`, `section Fiber`,
 * `geomTransf`, `pattern Plain`/`load`/`sp`, `mass`) put into a Domain,
 * flattened into structure-of-arrays form.  Node and element tags must be
 * strictly ascending: the reference iterates its MapOfTaggedObjects storage
 * in ascending tag order (tagged/storage/MapOfTaggedObjects.cpp), which fixes
 * both the DOF numbering and the assembly order.
 */
typedef struct xg_model_desc {
  int ndm, ndf;                 /* 2/2 quad, 3/3 brick, 2/3 frame2d, 3/6 frame3d */

  int num_nodes;
  const int    *node_tag;       /* [num_nodes] ascending                     */
  const double *node_crd;       /* [num_nodes*ndm]                           */
  const double *node_mass;      /* [num_nodes*ndf] lumped mass or NULL       */

  int elem_type;                /* XG_ELE_*                                  */
  int num_elems;
  const int    *elem_tag;       /* [num_elems] ascending                     */
  const int    *elem_conn;      /* [num_elems*nen] node tags                 */
  const int    *elem_mat;       /* [num_elems] J2 row (quad/brick) or section row (frames) */
  double        thickness;      /* quad thickness                            */

  /* frames */
  const double *elem_vecxz;     /* [num_elems*3] frame3d orientation (geomTransf vecxz) */
  int geom_transf;              /* 0 Linear, 1 PDelta                        */
  int fbc_num_ip;               /* Lobatto points per element (reference default 5) */
  int fbc_max_iters;            /* element compatibility iterations (default 10) */
  double fbc_tol;               /* element energy tolerance (default 1e-12)   */

  /* material tables */
  int num_j2;
  const double *j2_param;       /* [num_j2*XG_J2_NPARAM]                     */
  int num_uni;
  const int    *uni_type;       /* [num_uni] XG_UNI_*                        */
  const double *uni_param;      /* [num_uni*XG_UNI_NPARAM]                   */

  /* fiber sections: fibers of section s are [sec_fiber_start[s], sec_fiber_start[s+1]) */
  int num_sec;
  const int    *sec_fiber_start;/* [num_sec+1]                               */
  const double *fib_y;          /* [total fibers]                            */
  const double *fib_z;          /* [total fibers] (frame3d)                  */
  const double *fib_area;       /* [total fibers]                            */
  const int    *fib_mat;        /* [total fibers] uniaxial row               */
  const double *sec_GJ;         /* [num_sec] elastic torsion (frame3d)       */

  /* single-point constraints: pattern < 0 is a fixed homogeneous `fix`;
     pattern p >= 0 imposes value*lambda_p (an `sp` inside `pattern Plain p`) */
  int num_sp;
  const int    *sp_node;        /* node tag                                  */
  const int    *sp_dof;         /* 0-based dof                               */
  const int    *sp_pattern;
  const double *sp_value;
  int handler;                  /* XG_HANDLER_*                              */

  /* `equalDOF rNode cNode dof`: MP_Constraint with an identity constraint
     matrix (domain/constraints/MP_Constraint.h:62-66).  PlainHandler gives the
     constrained dof the retained dof's equation number
     (analysis/handler/PlainHandler.cpp:128-180, DOF_Numberer.cpp:155-185). */
  int num_mp;
  const int    *mp_retained;    /* retained node tag                         */
  const int    *mp_constrained; /* constrained node tag                      */
  const int    *mp_dof;         /* 0-based dof, same on both nodes           */

  /* nodal loads of `pattern Plain p { load ... }`, linear time series */
  int num_loads;
  const int    *load_node;      /* node tag                                  */
  const int    *load_pattern;
  const double *load_value;     /* [num_loads*ndf]                           */
} xg_model_desc;

/*
 * One analysis phase (`integrator ...; test ...; algorithm Newton;
 * analysis Static|Transient; analyze num_steps [dt]`).  Phase p drives load
 * pattern p.  After a phase with load_const != 0 has run all of its steps,
 * setting the next phase first holds every pattern constant and resets the
 * domain time to 0 (`loadConst -time 0.0` between the two `analyze`
 * commands), so xg_get_disp still reports the phase's last load factor.
 */
typedef struct xg_phase_desc {
  int integrator;               /* XG_INT_*                                  */
  int pattern;                  /* pattern driven by this phase              */
  int num_steps;
  double d_lambda;              /* LoadControl increment                     */
  int dc_node, dc_dof;          /* DisplacementControl node tag, 0-based dof */
  double dc_incr;               /* DisplacementControl increment             */
  double dt, gamma, beta;       /* Newmark                                   */
  double alpha_m, beta_k, beta_k_init, beta_k_comm;  /* rayleigh           */
  const double *alpha_m_node;   /* [num_nodes] alphaM per node or NULL       */
  const double *beta_k_init_elem; /* [num_elems] betaK0 per element or NULL:
                                   disconnected parts of one model with their
                                   own `rayleigh` factors                    */
  int gm_dof;                   /* UniformExcitation direction (0-based)     */
  int gm_npts;                  /* ground acceleration samples per record    */
  double gm_dt;
  const double *gm_accel;       /* [gm_count*gm_npts] PathSeries values      */
  int gm_count;                 /* records (0 or 1: one for every node)      */
  const int *gm_node_record;    /* [num_nodes] record of each node, or NULL:
                                   a separate UniformExcitation per group of
                                   nodes, e.g. disconnected frames batched
                                   into one model                            */
  int test;                     /* XG_TEST_*                                 */
  double tol;
  int max_iter;
  int load_const;
} xg_phase_desc;

/* per-step statistics written by xg_analyze */
typedef struct xg_step_stats {
  int newton_iters;             /* Newton iterations of the step             */
  int solver_iters;             /* total PCG iterations of the step          */
  int elem_iters;               /* total element (compatibility) iterations  */
  int status;                   /* 0 ok, < 0 XG_E*                           */
} xg_step_stats;

typedef struct xg_model xg_model;   /* opaque handle */

const char *xg_last_error(void);
int xg_version(void);

/* ------------------------------------------------------------------------ */
/* Domain + handler + numberer (analysis/handler/PlainHandler.cpp:60-260,   */
/* analysis/numberer/DOF_Numberer.cpp:93-205, graph/numberer/RCM.cpp:67-277,*/
/* analysis/model/AnalysisModel.cpp:286-400) and the device element set.     */
/* ------------------------------------------------------------------------ */

/* Build the device model: SoA element/material store, DOF numbering, the
   sparsity pattern and the element-to-slot map.  Replaces
   BasicAnalysisBuilder::domainChanged (runtime/runtime/BasicAnalysisBuilder.cpp:225-300). */
int xg_model_create(const xg_model_desc *desc, xg_model **out);
int xg_model_destroy(xg_model *m);

/* Host-only planning (no device work): the equation number of every
   (node, dof) and the scalar CSR pattern, exactly as DOF_Numberer::numberDOF
   and SparseGenColLinSOE::setSize produce them.  Any output may be NULL;
   call once with NULL arrays to learn num_eqn and nnz. */
int xg_model_plan(const xg_model_desc *desc, int *eqn, int *rowptr, int *colidx,
                  int *num_eqn, int *nnz);

/* Number of equations and scalar non-zeros of the system (the CSR/CSC
   pattern of sparseGEN/SparseGenColLinSOE.cpp:161-261, symmetric). */
int xg_model_sizes(const xg_model *m, int *num_eqn, int *nnz);

/* Equation number of every (node, dof) as DOF_Group::getID() holds it after
   numbering: >= 0 equation, -1 constrained.  eqn[num_nodes*ndf]. */
int xg_model_numbering(const xg_model *m, int *eqn);

/* Scalar CSR pattern in equation order: rowptr[num_eqn+1], colidx[nnz],
   columns ascending within a row (identical to the reference's CSC since
   the pattern is symmetric). */
int xg_model_pattern(const xg_model *m, int *rowptr, int *colidx);

/* ---- element set: Element::update / getTangentStiff / getResistingForce,
        commitState / revertToLastCommit (element/Element.h:51-103) ---- */

/* Copy trial nodal displacements (host, [num_nodes*ndf]) to the device. */
int xg_elemset_set_trial_disp(xg_model *m, const double *u);

/* Domain::update (domain/domain/Domain.cpp:1988-2006): state determination
   of every element from its committed state and the trial displacements,
   then deterministic assembly of the tangent and the resisting force.
   csr_vals[nnz] (may be NULL) receives the assembled tangent in the order
   of xg_model_pattern; resid[num_eqn] (may be NULL) receives the assembled
   resisting force P_int (no external load).  Returns the number of
   elements whose state determination failed as a negative code. */
int xg_elemset_update(xg_model *m, double *csr_vals, double *resid);

/* Per-element results of the last xg_elemset_update, in element order, for
   callers that assemble through their own loop (FE_Element::addKtToTang /
   addRtoResidual, analysis/fe_ele/FE_Element.cpp:266-430): K[num_elems *
   ned * ned] the element tangent (Element::getTangentStiff), P[num_elems *
   ned] the resisting force (Element::getResistingForce), row-major in the
   element's dof order (node by node, then dof).  Either may be NULL. */
int xg_elemset_element_matrices(const xg_model *m, double *K, double *P);

int xg_elemset_commit(xg_model *m);             /* Domain::commit          */
int xg_elemset_revert(xg_model *m);             /* revertToLastCommit      */
int xg_elemset_revert_to_start(xg_model *m);    /* revertToStart           */

/* Committed material history, SoA, for checkpoints and tests.
   which = 0: J2 plastic strain (ncomp x nip) + xi.  Force-based frames:
   1 = fiber records, 12 doubles per fiber and section in element order
   (Steel02: epsmin epsmax epspl epss0 sigs0 epsr sigr kon e sig eps),
   2 = element states (Se, kv, section deformations, flexibilities, forces).
   Writes at most cap doubles, returns the count written (or < 0). */
int xg_elemset_get_history(const xg_model *m, int which, double *out, long cap);
int xg_elemset_set_history(xg_model *m, int which, const double *in, long n);

/* ---- LinearSOE (system_of_eqn/linearSOE/LinearSOE.h) on the model's
        pattern: skyline LDL' (`system ProfileSPD`, the reference default,
        runtime/runtime/BasicAnalysisBuilder.cpp:820) or block-Jacobi PCG,
        both on the device ---- */

/* `loadConst -time t`: every load pattern applied so far keeps its current
   factor from now on and the domain time becomes t (the same happens at the
   next xg_analysis_set_phase when a finished phase has load_const set). */
int xg_analysis_load_const(xg_model *m, double time);

/* Choose the system (XG_SYSTEM_*); the default is XG_SYSTEM_PROFILE_SPD.
   Choosing the profile allocates its envelope tiles and fails with
   XG_ENOMEM when they would take more than half the free device memory. */
int xg_analysis_set_system(xg_model *m, int system);

/* Solve K x = b with the tangent assembled by the last xg_elemset_update.
   b, x are host arrays [num_eqn].  ProfileSPD: factors once per tangent
   (the reference's isAfactored) and returns XG_ESOLVE when a pivot fails
   the reference's checks (first pivot <= 0, a pivot == 0 or |pivot| <=
   1e-12); rtol and maxit are unused and iters = relres = 0.  PCG: returns
   XG_ESOLVE on breakdown or when maxit is reached; iters/relres report the
   final state. */
int xg_soe_solve(xg_model *m, const double *b, double *x,
                 double rtol, int maxit, int *iters, double *relres);

/* Device-pointer forms for callers whose vectors already live on the GPU
   (no host copies, ordered on the model's stream): u_dev [num_nodes*ndf];
   b_dev, x_dev [num_eqn]. */
int xg_elemset_set_trial_disp_device(xg_model *m, const double *u_dev);
int xg_soe_solve_device(xg_model *m, const double *b_dev, double *x_dev,
                        double rtol, int maxit, int *iters, double *relres);

/* ---- NewtonRaphson::solveCurrentStep (analysis/algorithm/equiSolnAlgo/
        NewtonRaphson.cpp:125-222) with its integrator and convergence test,
        all resident on the device ---- */
int xg_analysis_set_phase(xg_model *m, const xg_phase_desc *ph);
int xg_analysis_set_solver(xg_model *m, double rtol, int maxit);
/* Run num_steps steps of the current phase; stats[num_steps] may be NULL. */
int xg_analyze(xg_model *m, int num_steps, xg_step_stats *stats);
/* Committed nodal displacements [num_nodes*ndf] and the load factor. */
int xg_get_disp(const xg_model *m, double *u, double *lambda);
/* Reset displacements, time and material state to the start. */
int xg_reset(xg_model *m);

/* ---- tracing: CUDA-event timing of every kernel group on the model's
        stream (the reference times phases with its Timer class,
        utility/Timer.cpp, and the `totalCPU`/`solveCPU` commands) ---- */
/* Enable (1) or disable (0) and reset the per-kernel counters. */
int xg_profile_enable(xg_model *m, int enable);
/* Slot k (0..): name, accumulated milliseconds and launch count.  The slot
   after the last kernel reports the number of return maps that hit their
   iteration cap in the last update (in `launches`).  Returns XG_EINVAL past
   the end. */
int xg_profile_get(const xg_model *m, int k, char *name, int cap, double *ms, long *launches);

/* Autotuner (no counterpart in the reference).  what = XG_TUNE_ELEMENT:
   elements per block of the force-based element kernel (1, 2, 4, 8);
   XG_TUNE_PCG: rows per block of the PCG launch (32..256).  The next
   launches of the analysis try the candidates in turn (three timed samples
   each, CUDA events, normalised by fiber state determinations or PCG
   iterations) and keep the cheapest.  Element shapes give bit-identical
   results; PCG grids change the reduction tree (rounding only). */
#define XG_TUNE_ELEMENT 1
#define XG_TUNE_PCG     2
int xg_analysis_autotune(xg_model *m, int what);
/* The current choices and the number of tunings still sampling. */
int xg_autotune_result(const xg_model *m, int *elem_warps, int *pcg_rows_per_block,
                       int *pending);

/* Newmark steps as CUDA graphs (no counterpart in the reference): with
   enable = 1, a transient step of a model made of several parts (a batch of
   frames, per-part band LDL') whose external loads are constant runs as one
   graph launch -- the predictor, then a conditional loop whose body is one
   Newton iteration ending in a device-side per-part convergence check --
   and the host reads the outcome once per step.  Other steps, and steps
   while per-kernel timing or the autotuner is active, keep the host-driven
   loop; results are the same bit for bit.  xg_analysis_graph_steps counts
   the steps that ran as graphs. */
int xg_analysis_set_graph(xg_model *m, int enable);
int xg_analysis_graph_steps(const xg_model *m, long *steps);

/* The CUDA stream (a cudaStream_t) every kernel of the model runs on, for
   callers that time or order their own work against it. */
int xg_model_stream(const xg_model *m, void **stream);

/* Layout of the PCG's node-block copy of the tangent (built at the first
   PCG solve): its block order (2, 3 or 6: the largest number of free dofs
   of a node; 0 while no copy exists, the solve then reading the CSR arrays),
   the number of node-pair blocks held and the rows left to the CSR chunks
   (those of nodes coupled to more than 96 nodes). */
int xg_model_pcg_layout(const xg_model *m, int *block_order, long long *blocks,
                        long long *chunked_rows);

/* Work counters since xg_profile_enable: material-point state
   determinations (J2 points; for frames every fiber of every section in
   every compatibility iteration), section state determinations (frames)
   and element state determinations. */
int xg_profile_counters(xg_model *m, long long *point_updates, long long *section_updates,
                        long long *element_updates);

/* ---- A standalone linear system on the device: LinearSOE
        (system_of_eqn/linearSOE/LinearSOE.h: setSize, zeroA, zeroB, addA,
        addB, setB, solve, getX, getB) for callers that keep the
        reference's own element loop (FE_Element::addAtoSOE feeding addA).
        The pattern is CSR with sorted columns (SparseGenColLinSOE::setSize
        order); addA / addB / setB follow SparseGenColLinSOE.cpp:214-350 (an
        equation number outside 0..n-1 and an entry outside the pattern are
        skipped, as the reference skips them) and accumulate on the host; solve runs block-Jacobi PCG on
        the device (blocks of 1-6 equations, or point Jacobi when nblk is
        0) and copies X back.  Not reentrant per handle. ---- */
typedef struct xg_linsoe xg_linsoe;
int xg_linsoe_create(int num_eqn, const int *rowptr, const int *colidx, const int *blk_start,
                     int nblk, xg_linsoe **out);
void xg_linsoe_destroy(xg_linsoe *s);
int xg_linsoe_zero_a(xg_linsoe *s);                               /* zeroA */
int xg_linsoe_zero_b(xg_linsoe *s);                               /* zeroB */
/* A(id[i], id[j]) += fact * m[i*ndof + j] (addA, m row-major ndof x ndof) */
int xg_linsoe_add_a(xg_linsoe *s, const double *m, const int *id, int ndof, double fact);
int xg_linsoe_add_b(xg_linsoe *s, const double *v, const int *id, int ndof, double fact);
/* B = fact * v; fact == 0 leaves B unchanged (SparseGenColLinSOE::setB) */
int xg_linsoe_set_b(xg_linsoe *s, const double *v, double fact);
int xg_linsoe_get_a(const xg_linsoe *s, double *vals);            /* CSR values */
int xg_linsoe_get_b(const xg_linsoe *s, double *b);
/* The solver behind solve(): XG_SYSTEM_BJPCG (the default, `system
   CudaBJPCG`) or XG_SYSTEM_PROFILE_SPD (`system ProfileSPD`,
   profileSPD/ProfileSPDLinSOE.cpp and ProfileSPDLinDirectSolver.cpp: addA
   keeps only the terms with row <= col, as ProfileSPDLinSOE::addA, stored
   in the lower triangle's slot (col, row); get_a returns that lower
   triangle, the upper is zero).  Switching the system zeroes A. */
int xg_linsoe_set_system(xg_linsoe *s, int system);
/* BJPCG: PCG to ||r|| <= rtol ||b||; XG_ESOLVE on breakdown or maxit (X
   holds the last iterate).  PROFILE_SPD: the device LDL' (factored once per
   matrix: again only after zeroA or addA) and its substitutions; rtol and
   maxit unused, iters = relres = 0; XG_ESOLVE when a pivot fails the
   reference's checks (a first pivot <= 0, a pivot == 0 or |pivot| <=
   1e-12).  The device copy of the pattern is made at the first call. */
int xg_linsoe_solve(xg_linsoe *s, double rtol, int maxit, int *iters, double *relres);
int xg_linsoe_get_x(const xg_linsoe *s, double *x);

/* ---- Recorders (recorder/NodeRecorder.cpp, EnvelopeNodeRecorder.cpp; the
        `recorder Node|EnvelopeNode -file f <-time> <-dT dt> -node ... -dof
        ... disp|vel|accel` commands).  Values are gathered on the device
        after every committed step of xg_analyze (no host traffic per step);
        dofs are 0-based here (the command's are 1-based), a dof a node does
        not have records 0. ---- */
#define XG_REC_NODE     0   /* one row per recorded step: [time] values */
#define XG_REC_ENVELOPE 1   /* three rows: min, max, max |.| ([time value] pairs with echo_time) */
#define XG_REC_DISP     0
#define XG_REC_VEL      1
#define XG_REC_ACCEL    2
/* The committed displacements, velocities or accelerations (XG_REC_DISP /
   VEL / ACCEL) of every node, [num_nodes * ndf] in node-tag order
   (Node::getDisp / getVel / getAccel). */
int xg_get_response(const xg_model *m, int response, double *out);
int xg_recorder_add(xg_model *m, int kind, int response, const int *node_tags, int num_nodes,
                    const int *dofs, int num_dofs, int echo_time, double dT, int *id);
/* Rows recorded so far (3 for an envelope once it has a record) and columns. */
int xg_recorder_size(const xg_model *m, int id, int *rows, int *cols);
/* Copy up to max_rows rows (row-major); returns the number of rows copied. */
int xg_recorder_read(const xg_model *m, int id, double *out, int max_rows);
/* Write the rows as the reference's DataFileStream does (values separated by
   blanks, %g with the given number of significant digits, 6 by default in
   the reference). */
int xg_recorder_write(const xg_model *m, int id, const char *path, int precision);

/* FP64 FMA throughput of the current device in TFLOP/s (a short probe
   kernel with no memory traffic), the ceiling of the FP64 element kernels. */
int xg_measure_fp64_peak(double *tflops);

/* The reciprocal the LDL' kernels use on their pivot chains (a single-
   precision seed refined by one cubically convergent step) and the
   correctly rounded __drcp_rn, both evaluated on the device for the n host
   values d: y[i] and y_rn[i].  For testing its error bound; no counterpart
   in the reference (ProfileSPDLinDirectSolver divides). */
int xg_chain_reciprocal_check(int n, const double *d, double *y, double *y_rn);

/* ---- Adjoint of a transient run (no counterpart in the reference; its
        DDM sensitivity, `computeGradients` (runtime/commands/analysis/
        sensitivity.cpp:22-41, Newmark.cpp:904-959), has no Steel02 stress
        sensitivity).  Gradients of J = sum over the steps n = 1..N and the
        terms k of weight_k * u(node_k, dof_k, t_n)^2 with respect to the
        first three parameters of every uniaxial material (Steel02: Fy, E0,
        b; Steel01: fy, E0, b; Concrete02: fc, epsc0, fcu; Concrete01: fpc,
        epsc0, fpcu; elastic: E).  Covers 2D and 3D force-based frames
        (Linear or PDelta transformations) whose sections use at most four
        materials (Steel02 without initial stress, Steel01, Concrete02,
        Concrete01, elastic), Newmark with alphaM Rayleigh damping (betaK0
        as well where an element has a single Steel02, Steel01 or elastic
        material), UniformExcitation and nodal load patterns, from the
        model's initial state. ---- */
typedef struct xg_objective_desc {
  int num_terms;
  const int *node;            /* node tags */
  const int *dof;             /* 0-based dof */
  const double *weight;
} xg_objective_desc;
/* Replace the uniaxial parameters (num_uni x XG_UNI_NPARAM, the model
   description's layout) and reset the model to its initial state. */
int xg_model_set_uniaxial_params(xg_model *m, const double *uni_param, int num_uni);
/* Run num_steps steps of the Newmark phase ph from the initial state, keep
   the committed state every ckpt_every steps, and return J. */
int xg_adjoint_forward(xg_model *m, const xg_phase_desc *ph, int num_steps, int ckpt_every,
                       const xg_objective_desc *obj, double *J);
/* The last run's objective term by term (J_k summed over the steps; J is
   their sum in term order). */
int xg_adjoint_objective_terms(const xg_model *m, double *Jk, int num_terms);
/* Reverse sweep of the last xg_adjoint_forward: each segment between
   checkpoints is run again and swept backwards.  grad[u*3 + k] = scale *
   dJ/d uni_param[u][k], k = 0, 1, 2, for the num_uni materials.  The model
   is left at the state after the run's last step. */
int xg_adjoint_backward(xg_model *m, double scale, double *grad, int num_uni);
/* ---- Direct differentiation (DDM) of a transient run: the reference's
        `sensitivityAlgorithm -computeAtEachStep` with one `parameter` per
        direction (runtime/commands/analysis/sensitivity.cpp:22-41;
        Newmark::computeSensitivities, Newmark.cpp:904-959;
        ForceBeamColumn2d's basic-force sensitivity and commitSensitivity,
        ForceBeamColumn2d.cpp:2890-3007; Steel01::getStressSensitivity and
        commitSensitivity, Steel01.cpp:552-660; Concrete01's, Concrete01.cpp:
        655-775), a forward-mode path independent of the adjoint above.
        Covers 2D and 3D force-based frames (Linear or PDelta
        transformations) with Steel02 (no initial stress) and
        Concrete02 (the reference has no sensitivity for either), Steel01,
        Concrete01 and elastic fibers, Newmark with alphaM Rayleigh damping
        (betaK0 as well on elements of one Steel02, Steel01 or elastic
        material) or LoadControl (LoadControl::computeSensitivities),
        UniformExcitation and nodal load patterns, from the model's initial
        state.  After each converged step the effective tangent is formed
        again at the converged state (the reference solves with the last
        Newton iteration's factors). ---- */
/* Newmark or LoadControl run of num_steps from the initial state carrying num_dir
   directions: dtheta[(k*num_uni + u)*3 + j] is direction k's tangent of
   parameter j (0..2) of material u (Steel02 and Steel01: fy, E0, b;
   Concrete02: fc, epsc0, fcu; Concrete01: fpc, epsc0, fpcu; elastic: E).
   J as xg_adjoint_forward; dJ[k] = the derivative of J along direction k. */
int xg_ddm_forward(xg_model *m, const xg_phase_desc *ph, int num_steps, int num_dir,
                   const double *dtheta, const xg_objective_desc *obj, double *J, double *dJ);
/* The last DDM run's dJ along direction dir term by term (dJ[dir] is their
   sum in term order); for separate models batched into one, each term
   gives its own model's directional derivative. */
int xg_ddm_objective_terms(const xg_model *m, int dir, double *dJk, int num_terms);
/* The last DDM run's displacement tangent of direction dir after its last
   step, out[num_nodes*ndf] (zero on constrained dofs; `sensNodeDisp`). */
int xg_ddm_disp_sensitivity(const xg_model *m, int dir, double *out);
/* Jacobian-vector product of one material point's trial record (host only;
   Steel02, Concrete02, Steel01, Concrete01 or elastic): given the tangents
   of the strain, of the committed record dhc[12] and of parameters 0-2
   dq[3], the tangent of the trial record dht[12] (Steel02 fields 0-6,
   Concrete02 0-1, Steel01 0-3, Concrete01 0-2, 9 stress, 10 strain). */
int xg_uniaxial_jvp(int type, const double *q, const double *hc, double strain,
                    double dstrain, const double *dhc, const double *dq, double *dht);
/* Vector-Jacobian product of one material point's trial record (host only;
   Steel02, Concrete02, Steel01, Concrete01 or elastic): given the adjoint
   yb[12] of the trial record (history fields: Steel02 0-6, Concrete02 0-1,
   Steel01 0-3, Concrete01 0-2; 9 stress, 10 strain), the adjoints of the
   committed record hb[12], of the strain *sb and of parameters 0-2 qb[3]. */
int xg_uniaxial_vjp(int type, const double *q, const double *hc, double strain,
                    const double *yb, double *hb, double *sb, double *qb);

/* ---- Allocation-free solve.  No counterpart in the reference: it exists
        for callers that cannot allocate device memory when they solve -- a
        host application or framework whose device memory is owned by its own
        pool (PyTorch's caching allocator, say), or a latency-bound loop that
        cannot pay for cudaMalloc/cudaFree, which synchronise the whole device.
   Solves A x = b by the same block-Jacobi PCG as xg_soe_solve, on CSR arrays
   and vectors the caller already holds on the device: rowptr[n+1],
   colidx[nnz], vals[nnz], blk_start[nblk+1] (diagonal blocks of 1..6
   consecutive equations), b[n], x[n] (output; zeroed first).  stream may be
   NULL; the call returns when the solve is done.  Its scratch is a fixed
   device array of XG_NOALLOC_MAX_DOUBLES doubles (32 MiB) that every GPU
   using the library holds until the process exits; a system needing more
   than 36*nblk + 4*n + 3*(cooperative blocks) + 24 doubles of it (about
   260,000 equations with 3x3 node blocks, 100,000 with 1x1 blocks) is
   rejected with XG_EINVAL.  Every call looks up the array's device address
   in the current context.  The call waits on its stream before it returns.  All
   calls share the one array: calls that overlap on the GPU race and must be
   serialised by the caller.  Allocates no device memory. ---- */
#define XG_NOALLOC_MAX_DOUBLES 4194304
int xg_pcg_solve_noalloc(int n, const int *rowptr, const int *colidx, const double *vals,
                         int nblk, const int *blk_start, const double *b, double *x,
                         double rtol, int maxit, void *stream, int *iters, double *relres);

#ifdef __cplusplus
}
#endif
#endif /* XARA_GPU_H */
