#!/usr/bin/env python3
"""Benchmark of the Newton-iteration hot path on one GB300.

Workload `frame3d` (default): the 3D RC frame of 10 x 10 bays x 20 stories
(6,820 forceBeamColumn elements, 5 Lobatto sections each, 120-fiber columns
and 64-fiber beams with Concrete02 / Steel02, 14,520 equations), FP64, under
its BASELINE analysis: gravity by LoadControl, loadConst, then the
DisplacementControl pushover of a roof corner to 2 % drift in 200 steps.  A
step is one pushover load step through the device Newton driver: per Newton
iteration the state determination of every element (the force-based
compatibility iteration over every fiber of every section), assembly of the
tangent and the resisting force, the `system ProfileSPD` LDL' factorisation
and two right-hand sides (DisplacementControl), and the NormDispIncr test.
Gravity and the first W pushover steps are untimed; the next K are timed.
The rest of the pushover then runs to 2 % drift and its roof history is
compared with the reference's own record (tests/golden/frame3d_c1.npz).
`e2e` runs the same K steps with the reference's Newton loop on the host
calling the reference-facing C ABI with host buffers.  The line also carries
the brick, batch and adjoint workloads below as sub-blocks (`workloads`).

Metric: IP updates/s -- fiber state determinations per second, every fiber
counted once per inner compatibility iteration of its element; Newton
iterations/s is reported beside it.

Workload `brick`: the element phase of the stdBrick J2 block 128 x 128 x 64
(1,048,576 bricks, 8,388,608 integration points), one pass per step.

Workload `batch`: 4,096 independent 2D steel frames (1-12 bays, 2-20
stories, 40-fiber Steel02 sections), each under its own Kanai-Tajimi record,
in one device model; a step is one Newmark time step of every frame (its
Newton iterations, each frame converging on its own).  Metric: frame time
steps/s, beside the same kernels run one frame per model.

Workload `adjoint`: gradients of the summed squared roof drift of 64 such
frames (one Steel02 material per member) over 2,000 Newmark steps with
respect to every member's Fy, E0 and b, checkpoints every 100 steps.
Metric: reverse-sweep time / forward-run time (lower is better), with a
central finite-difference check of one directional derivative.

  python bench.py [--workload frame3d|brick|batch|adjoint] [--gpus N] [--steps K]
                  [--warmup W] [--impl xara|reference]

--impl reference times the reference algorithm's CPU path (the C oracle, a
restatement of the reference's classes compiled on this host) on every host
core, one model per process, on the same workload and metric.
"""
import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "IP updates/s"
UNIT = "material-point updates/s"
FRAME = dict(bays_x=10, bays_y=10, stories=20)
BRICK = dict(nx=128, ny=128, nz=64)
BRICK_SAMPLE = dict(nx=24, ny=24, nz=12)


# ---------------------------------------------------------------------------
# shared helpers
# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.id = gpu_smi_id()
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.id}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=5)
        sm = [float(r[1]) for r in self.rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            if len(r) < 9:
                continue
            for name, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def gpu_smi_id():
    """nvidia-smi's name for the GPU this process computes on: its UUID.
    nvidia-smi numbers GPUs physically and ignores CUDA_VISIBLE_DEVICES, so
    an index could name another process's GPU."""
    try:
        import torch
        uuid = str(torch.cuda.get_device_properties(torch.cuda.current_device()).uuid)
        return uuid if uuid.startswith("GPU-") else "GPU-" + uuid
    except Exception:
        return "0"


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs"), "of measured"
    return 6800.0, "of fallback"


def fp64_peak_probe():
    from xara_gb300 import gpu
    L = gpu.lib()
    v = C.c_double()
    L.xg_measure_fp64_peak.argtypes = [C.POINTER(C.c_double)]
    if L.xg_measure_fp64_peak(C.byref(v)) != 0:
        return None
    return v.value


def ncu_traffic(workload, kernel):
    """DRAM bytes per launch of the kernel from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "dram_traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        d = json.load(f)
    return d.get(workload, {}).get(kernel)


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        # one replica per GPU: one model's Newton iteration does not shard.
        # The rank takes the local-rank-th GPU of the list it was given and
        # never widens that list.
        visible = os.environ.get("CUDA_VISIBLE_DEVICES")
        if visible:
            devices = [d for d in visible.split(",") if d.strip()]
            if local >= len(devices):
                raise RuntimeError(f"local rank {local} has no GPU in "
                                   f"CUDA_VISIBLE_DEVICES={visible}")
            os.environ["CUDA_VISIBLE_DEVICES"] = devices[local]
        else:
            os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    import torch
    import torch.distributed as dist
    if world > 1:
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        if torch.cuda.is_available():
            torch.cuda.set_device(0)
    return world, rank, local, torch, dist


def _over_ranks(x, world, torch, dist, op):
    if world == 1:
        return x
    # NCCL reduces device tensors only; gloo (the host-side runs) host ones
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=op)
    return float(t.item())


def max_over_ranks(x, world, torch, dist):
    """The slowest rank's time: the whole job ends when it does."""
    return _over_ranks(x, world, torch, dist, dist.ReduceOp.MAX if world > 1 else None)


def sum_over_ranks(x, world, torch, dist):
    """Units processed by all ranks together."""
    return _over_ranks(x, world, torch, dist, dist.ReduceOp.SUM if world > 1 else None)


def job_rate(units, dt, world, torch, dist):
    """Whole-job throughput: the units of every replica over the slowest
    replica's time (each rank passes its own units and its own time)."""
    return sum_over_ranks(units, world, torch, dist) / max_over_ranks(dt, world, torch, dist)


# ---------------------------------------------------------------------------
# frame3d: one Newton iteration of the 3D RC frame per step
# ---------------------------------------------------------------------------
def frame_model():
    from xara_gb300 import configs
    desc, phases = configs.rc_frame_3d(**FRAME)
    return desc, phases


C1_FIXTURE = os.path.join(ROOT, "tests", "golden", "frame3d_c1.npz")
C1_PARITY_TESTS = ["tests/test_full_size.py::test_c1_first_pushover_step_entrywise",
                   "tests/test_full_size.py::test_c1_pushover_history"]


def c1_reference():
    """The reference's own C1 pushover record (roof history every step,
    snapshots of every free displacement every 10 steps), made by
    tests/golden/make_golden.py from the reference's classes."""
    if not os.path.exists(C1_FIXTURE):
        return None
    z = np.load(C1_FIXTURE)
    return {k: z[k] for k in ("roof_u", "step_lambda", "step_iters", "snap_steps", "snap_u",
                              "free")}


def relerr(a, b):
    a, b = np.ravel(a), np.ravel(b)
    d = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (d if d > 0 else 1.0))


def profile_stats(rowptr, colidx):
    """Envelope entries (the ProfileSPD storage) and FP64 FMAs of its LDL'."""
    first = colidx[rowptr[:-1]]
    h = np.arange(len(first)) - first + 1
    return int(h.sum()), float((h.astype(np.float64) ** 2).sum() / 2.0)


def frame_alg_bytes(desc, nnz, neq):
    """Algorithmic bytes of the kernels of one Newton iteration, from the
    per-unit figures: fiber history (Steel02 80 B, Concrete02 32 B) read
    committed and written trial once per element update; element state
    (Se, kv, 5 x (vs, fs, Ssr)) 1.3 KB read and written; nodal
    displacements; CSR values and residual written; the LDL' reads the
    envelope of the tangent and writes its factor."""
    from xara_gb300._abi import XG_UNI_STEEL02
    sec_start = np.asarray(desc.arrays["sec_fiber_start"])
    fmat = np.asarray(desc.arrays["fib_mat"])
    utype = np.asarray(desc.arrays["uni_type"])
    per_fiber = np.where(utype[fmat] == XG_UNI_STEEL02, 160, 64)
    sec_bytes = np.array([per_fiber[sec_start[s]:sec_start[s + 1]].sum()
                          for s in range(len(sec_start) - 1)])
    emat = np.asarray(desc.arrays["elem_mat"])
    ne = len(emat)
    fib = float(sec_bytes[emat].sum()) * 5
    update = fib + ne * 2 * 1300 + desc.num_nodes * 48
    return {"fbc_update": update, "fbc_assemble": ne * (1300 + 144 * 8 + 12 * 8),
            "gather_tangent": nnz * 8.0, "gather_resid": neq * 8.0}


def pattern_loads(desc, eqn, neq, pattern):
    """Reference load vector of one load pattern, per equation."""
    f = np.zeros(neq)
    tags = np.asarray(desc.node_tag)
    vals = np.asarray(desc.load_value).reshape(-1, desc.ndf)
    for i, n in enumerate(desc.load_node):
        if desc.load_pattern[i] != pattern:
            continue
        idx = int(np.searchsorted(tags, n))
        for j in range(desc.ndf):
            r = eqn[idx * desc.ndf + j]
            if r >= 0:
                f[r] += vals[i, j]
    return f


class HostDisplacementControl:
    """The reference's own analysis loop driving the library through its
    reference-facing C ABI, as the element-set and LinearSOE shims do:
    NewtonRaphson::solveCurrentStep (NewtonRaphson.cpp:125-222) with
    DisplacementControl::newStep / update (DisplacementControl.cpp:121-281)
    and CTestNormDispIncr on the host, every element update
    (xg_elemset_set_trial_disp + xg_elemset_update) and every solve
    (xg_soe_solve, the device LDL') through host buffers in pinned memory."""

    def __init__(self, m, desc, phase, const_factor, torch):
        from xara_gb300 import gpu
        self.gpu, self.L, self.m = gpu, gpu.lib(), m
        eqn = m.numbering()
        self.map = np.nonzero(eqn >= 0)[0]
        self.eq = eqn[self.map]
        nd = int(np.searchsorted(np.asarray(desc.node_tag), phase.dc_node))
        self.ceq = int(eqn[nd * desc.ndf + phase.dc_dof])
        self.incr, self.tol, self.maxit = phase.dc_incr, phase.tol, phase.max_iter
        # gravity, held at its last factor by loadConst
        self.fconst = const_factor * pattern_loads(desc, eqn, m.neq, 0)
        self.phat = pattern_loads(desc, eqn, m.neq, phase.pattern)
        pin = lambda n: torch.zeros(n, dtype=torch.float64).pin_memory()  # noqa: E731
        self.Uh, self.Rh = pin(m.nu), pin(m.neq)
        self.bh, self.xh = pin(m.neq), pin(m.neq)
        self.U, self.R = self.Uh.numpy(), self.Rh.numpy()
        self.b, self.x = self.bh.numpy(), self.xh.numpy()
        u, lam = m.disp()
        self.U[:] = u
        self.lam = lam
        self.h2d = self.d2h = 0
        self.ptr = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731

    def _update(self):
        g, L, m = self.gpu, self.L, self.m
        g._check(L.xg_elemset_set_trial_disp(m.h, self.ptr(self.Uh)))
        r = L.xg_elemset_update(m.h, None, self.ptr(self.Rh))
        if r < 0:
            raise RuntimeError(f"element state determination failed ({r})")
        self.h2d += self.U.nbytes
        self.d2h += self.R.nbytes

    def _solve(self, rhs):
        g, L, m = self.gpu, self.L, self.m
        self.b[:] = rhs
        it_, rr_ = C.c_int(), C.c_double()
        g._check(L.xg_soe_solve(m.h, self.ptr(self.bh), self.ptr(self.xh), 1e-12, 20000,
                                C.byref(it_), C.byref(rr_)))
        self.h2d += self.b.nbytes
        self.d2h += self.x.nbytes
        return self.x.copy()

    def _incr(self, dU):
        np.add.at(self.U, self.map, dU[self.eq])

    def step(self):
        """One load step; returns the Newton iterations."""
        dUhat = self._solve(self.phat)                   # newStep: tangent of the last update
        dlam = self.incr / dUhat[self.ceq]
        self.lam += dlam
        self._incr(dlam * dUhat)
        self._update()
        it = 0
        while True:
            dUbar = self._solve(self.fconst + self.lam * self.phat - self.R)
            dUhat = self._solve(self.phat)
            dl = -dUbar[self.ceq] / dUhat[self.ceq]
            dU = dUbar + dl * dUhat
            self.lam += dl
            self._incr(dU)
            self._update()
            it += 1
            if np.linalg.norm(dU) <= self.tol:
                break
            if it >= self.maxit:
                raise RuntimeError("host DisplacementControl step did not converge")
        self.gpu._check(self.L.xg_elemset_commit(self.m.h))
        return it


def run_frame(args):
    world, rank, local, torch, dist = dist_setup()
    from xara_gb300 import gpu
    desc, phases = frame_model()
    grav, push = phases
    W, K = args.warmup, args.steps
    t_setup = time.perf_counter()
    m = gpu.DeviceModel(desc)
    m.set_system(gpu.XG_SYSTEM_PROFILE_SPD)
    t_setup = time.perf_counter() - t_setup
    rowptr, colidx = m.pattern()
    envelope, ldl_fma = profile_stats(rowptr, colidx)
    stream = torch.cuda.ExternalStream(gpu.model_stream(m))
    fp64_peak = fp64_peak_probe()
    rid = m.add_recorder([desc.meta["roof"]], dofs=list(range(6)))

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    # gravity (LoadControl, loadConst), then W pushover steps: untimed
    m.set_phase(grav)
    it_lead = sum(s[0] for s in m.analyze(grav.num_steps))
    grav_factor = m.disp()[1]          # the gravity pattern's factor from now on
    m.set_phase(push)
    it_lead += sum(s[0] for s in m.analyze(W))
    # the timed steps: K DisplacementControl steps of the pushover through the
    # device Newton driver (element state, assembly, LDL' factor, two
    # right-hand sides per iteration, the norm test), inputs resident
    gpu.profile_enable(m, True)
    sampler = ClockSampler()
    sampler.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    barrier()
    ev0.record(stream)
    stats = m.analyze(K)
    ev1.record(stream)
    barrier()
    clocks = sampler.stop()
    dt = ev0.elapsed_time(ev1) * 1e-3
    points, sections, elems = gpu.profile_counters(m)
    prof = gpu.profile_read(m)
    gpu.profile_enable(m, False)
    newton = sum(s[0] for s in stats)
    value = job_rate(points, dt, world, torch, dist)
    newton_rate = job_rate(newton, dt, world, torch, dist)
    dt = max_over_ranks(dt, world, torch, dist)
    u_dev, lam_dev = m.disp()

    # the rest of the pushover to 2 % roof drift, in chunks of ten steps
    # (the snapshots' spacing), against the reference's record
    ref = c1_reference()
    full = None
    if not args.no_analysis:
        done = grav.num_steps + W + K
        total = grav.num_steps + push.num_steps
        snaps = {}
        t0 = time.perf_counter()
        it_rest = 0
        while done < total:
            n = min(10 - done % 10 if done % 10 else 10, total - done)
            it_rest += sum(s[0] for s in m.analyze(n))
            done += n
            if done % 10 == 0:
                snaps[done - 1] = m.disp()[0]
        t_rest = time.perf_counter() - t0
        hist = m.recorder(rid)
        full = {"steps": push.num_steps, "drift": 0.02,
                "rest_seconds": t_rest, "rest_newton_iterations": it_rest,
                "note": f"pushover steps {W + K + 1}..{push.num_steps} after the timed ones, "
                        "host clock, displacements read every 10 steps"}
        if ref is not None:
            nrec = hist.shape[0]
            full.update({
                "roof_relerr": relerr(hist[:, -6:], ref["roof_u"][:nrec]),
                "lambda_relerr": relerr(np.asarray([lam_dev]),
                                        ref["step_lambda"][grav.num_steps + W + K - 1]),
                "snapshot_relerr": max(relerr(snaps[s][ref["free"]],
                                              ref["snap_u"][i])
                                       for i, s in enumerate(ref["snap_steps"]) if s in snaps),
                "snapshots": len(snaps), "recorded_steps": int(nrec),
                "reference_newton_iterations": int(ref["step_iters"].sum()),
                "device_newton_iterations": int(it_lead + newton + it_rest),
            })

    # end to end: the same timed window again through the reference-facing C
    # ABI (the reference's own Newton loop on the host, host buffers)
    m.reset()
    m.set_phase(grav)
    m.analyze(grav.num_steps)
    m.set_phase(push)
    m.analyze(W)
    host = HostDisplacementControl(m, desc, push, grav_factor, torch)
    gpu.profile_enable(m, True)
    barrier()
    t0 = time.perf_counter()
    it_e2e = sum(host.step() for _ in range(K))
    barrier()
    dt_e2e = time.perf_counter() - t0
    points_e2e, _, _ = gpu.profile_counters(m)
    gpu.profile_enable(m, False)
    e2e_value = job_rate(points_e2e, dt_e2e, world, torch, dist)
    e2e_vs_device = relerr(host.U, u_dev)

    if rank != 0:
        dist.destroy_process_group()
        return None

    kernels = {k: v for k, v in prof.items() if v[1] > 0 and k != "return_map_cap_hits"}
    gpu_launches = sum(v[1] for v in kernels.values())
    dominant = max(kernels, key=lambda k: kernels[k][0])
    peak, peak_kind = measured_peaks()
    alg = frame_alg_bytes(desc, m.nnz, m.neq)
    alg["ldl_factor"] = envelope * 16.0        # envelope read, factor written
    alg["ldl_solve"] = envelope * 16.0         # forward and backward sweeps
    ldl_ms, ldl_n = kernels.get("ldl_factor", (0.0, 0))
    factorisations = max(ldl_n // 2, 1)        # two timed kernel groups per factorisation
    ldl_s = ldl_ms * 1e-3 / factorisations
    ldl_flops = 2.0 * ldl_fma
    if dominant == "ldl_factor":
        tf = ldl_flops / ldl_s / 1e12
        gbs = alg["ldl_factor"] / ldl_s / 1e9
        roof_line = {"bound": "fp64", "kernel": dominant, "achieved": tf,
                     "peak": fp64_peak, "unit": "TFLOP/s",
                     "frac": tf / fp64_peak if fp64_peak else None,
                     "peak_source": "of the FP64 probe (xg_measure_fp64_peak, this run): "
                                    "MEASURED_PEAKS.json holds no FP64 figure",
                     "flops_per_launch": ldl_flops,
                     "traffic": ncu_traffic("frame3d", dominant),
                     "hbm": {"achieved": gbs, "peak": peak, "unit": "GB/s",
                             "frac": gbs / peak if peak else None, "peak_source": peak_kind,
                             "algorithmic_bytes_per_launch": alg["ldl_factor"]}}
    else:
        dom_ms, dom_n = kernels[dominant]
        per = dom_ms * 1e-3 / max(dom_n, 1)
        gbs = alg.get(dominant, 0.0) / per / 1e9
        roof_line = {"bound": "hbm", "kernel": dominant, "achieved": gbs, "peak": peak,
                     "unit": "GB/s", "frac": gbs / peak if peak else None,
                     "peak_source": peak_kind, "traffic": ncu_traffic("frame3d", dominant),
                     "algorithmic_bytes_per_launch": alg.get(dominant)}
    window = f"pushover steps {W + 1}..{W + K} of 200 (after gravity and loadConst)"
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": K, "warmup": W, "ms_per_step": 1e3 * dt / K,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded RC frame model; the BASELINE pushover)",
        "config": {"workload": "3D RC frame 10x10x20 (6,820 force-based elements), "
                               "DisplacementControl pushover: one load step per step -- "
                               "forceBeamColumn state determination, assembly, ProfileSPD "
                               "LDL' factor, two right-hand sides per Newton iteration, "
                               "NormDispIncr 1e-10",
                   "timed_window": window, "elements": desc.num_elems, "equations": m.neq,
                   "nnz": m.nnz, "fiber_points": desc.meta["fiber_points"],
                   "envelope": envelope, "system": "ProfileSPD (device LDL')",
                   "parallelism": f"replicas x{world}",
                   "l2": "per-step working set (factor tiles 89 MB rewritten, fiber records "
                         "275 MB) exceeds L2; no flush"},
        "newton_iters_per_s": newton_rate,
        "newton_iters_per_step": newton / K,
        "point_updates_per_step": points / K,
        "section_updates_per_step": sections / K,
        "e2e": {"value": e2e_value, "unit": UNIT,
                "h2d_bytes_per_step": int(host.h2d / K), "d2h_bytes_per_step": int(host.d2h / K),
                "newton_iterations": it_e2e, "relerr_vs_device_driver": e2e_vs_device,
                "path": "the reference's NewtonRaphson + DisplacementControl on the host over "
                        "xg_elemset_set_trial_disp + xg_elemset_update + xg_soe_solve (two "
                        "right-hand sides per iteration) + xg_elemset_commit, pinned host "
                        "buffers"},
        "gpu_launches": int(gpu_launches),
        "roofline": roof_line,
        "ldl": {"factorisations_per_step": factorisations / K, "ms_per_factorisation": 1e3 * ldl_s,
                "flops_per_factorisation": ldl_flops},
        "kernels_ms_per_step": {k: v[0] / K for k, v in kernels.items()},
        "parity": {"tests": C1_PARITY_TESTS, "fixture": "tests/golden/frame3d_c1.npz",
                   "full_pushover": full},
        "clocks": clocks,
        "setup_s": t_setup,
    }
    if not args.no_cpu_baseline:
        rate, its, sample = frame_cpu_sample(W, seconds=args.cpu_seconds)
        line["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": 1, "kind": "port",
                                "sample": sample, "newton_iters_per_s": its}
    m.close()
    return line


class FrameCpu:
    """The oracle's path (element state, assembly, ProfileSPD) on one model,
    brought through gravity and the first pushover steps."""

    def __init__(self, lead):
        from oracle import port
        from xara_gb300._abi import PhaseDesc
        self.desc, (grav, push) = frame_model()
        self.o = port.OracleModel(self.desc)
        self.o.run([grav, PhaseDesc(**{**push.kw, "num_steps": lead})])
        self.push = push
        self.PhaseDesc = PhaseDesc

    def steps(self, n):
        """n pushover steps; returns (point updates, Newton iterations)."""
        p0, _ = self.o.work()
        _, _, its = self.o.run([self.PhaseDesc(**{**self.push.kw, "num_steps": n})])
        return self.o.work()[0] - p0, int(its.sum())


def frame_cpu_sample(lead, seconds=12.0):
    t0 = time.perf_counter()
    cpu = FrameCpu(lead)
    pts, its, n, t1 = 0, 0, 0, time.perf_counter()
    while n < 1 or time.perf_counter() - t1 < seconds:
        p, i = cpu.steps(1)
        pts, its, n = pts + p, its + i, n + 1
    dt = time.perf_counter() - t1
    sample = (f"3D RC frame 10x10x20 at full size, pushover steps {lead + 1}..{lead + n} "
              f"({its} Newton iterations: element state, assembly, ProfileSPD factor and "
              f"two right-hand sides each), 1 thread; model set-up, gravity and the first "
              f"{lead} pushover steps ({t1 - t0:.0f} s) untimed")
    return pts / dt, its / dt, sample


_CPU = None


def _frame_worker(args):
    global _CPU
    kind, n = args
    if kind == "init":
        _CPU = FrameCpu(n)
        return 0
    t0 = time.perf_counter()
    pts, its = _CPU.steps(n)
    return pts, its, time.perf_counter() - t0


def run_reference_frame(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return None
    import multiprocessing as mp
    cores = os.cpu_count() or 1
    W, K = args.warmup, args.steps
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        pool.map(_frame_worker, [("init", W)] * cores, chunksize=1)
        t0 = time.perf_counter()
        res = pool.map(_frame_worker, [("steps", K)] * cores, chunksize=1)
        wall = time.perf_counter() - t0
    pts = sum(r[0] for r in res)
    its = sum(r[1] for r in res)
    value = pts / wall
    sample = (f"3D RC frame 10x10x20 at full size, one model per process on {cores} "
              f"processes: gravity and pushover steps 1..{W} untimed, then steps "
              f"{W + 1}..{W + K} timed (element state, assembly, ProfileSPD factor and two "
              f"right-hand sides per Newton iteration)")
    desc, _ = frame_model()
    return {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": K, "warmup": W,
        "ms_per_step": 1e3 * wall / K, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded RC frame model; the BASELINE pushover)",
        "config": {"workload": "3D RC frame 10x10x20 (6,820 force-based elements), "
                               "DisplacementControl pushover: one load step per step -- "
                               "forceBeamColumn state determination, assembly, ProfileSPD "
                               "LDL' factor, two right-hand sides per Newton iteration, "
                               "NormDispIncr 1e-10",
                   "timed_window": f"pushover steps {W + 1}..{W + K} of 200 (after gravity "
                                   f"and loadConst)",
                   "elements": desc.num_elems, "fiber_points": desc.meta["fiber_points"],
                   "system": "ProfileSPD (the oracle's skyline LDL')",
                   "parallelism": f"{cores} processes, one model each"},
        "newton_iters_per_s": its / wall,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "wall_s": wall,
    }


# ---------------------------------------------------------------------------
# batch: thousands of independent 2D frames under their own ground motions
# ---------------------------------------------------------------------------
BATCH_FRAMES = 4096
BATCH_SAMPLE = 32          # frames of the per-model GPU loop
BATCH_CPU_FRAMES = 8       # frames of the one-core CPU sample


def batch_model(nframes, steps):
    from xara_gb300 import configs
    return configs.frame_batch(nframes, steps=steps, seed=0, return_parts=True)


def run_batch(args):
    world, rank, local, torch, dist = dist_setup()
    from xara_gb300 import gpu
    lead, nsteps = args.batch_lead, args.batch_lead + args.warmup + args.steps
    desc, phases, parts = batch_model(args.frames, nsteps)
    t_setup = time.perf_counter()
    m = gpu.DeviceModel(desc)
    m.set_system(gpu.XG_SYSTEM_PROFILE_SPD)      # one band per frame, one launch
    m.set_phase(phases[0])
    gpu.autotune(m, element=True, pcg=False)
    t_setup = time.perf_counter() - t_setup
    stream = torch.cuda.ExternalStream(gpu.model_stream(m))

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    m.analyze(lead + args.warmup)                 # into the strong motion, untimed
    tuned = gpu.autotune_result(m)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    # host-driven steps with per-kernel timing (the breakdown)
    gpu.profile_enable(m, True)
    barrier()
    ev0.record(stream)
    stats_h = m.analyze(args.steps)
    ev1.record(stream)
    barrier()
    dt_host = max_over_ranks(ev0.elapsed_time(ev1) * 1e-3, world, torch, dist)
    points, sections, elems = gpu.profile_counters(m)
    prof = gpu.profile_read(m)
    gpu.profile_enable(m, False)
    # the timed steps: every time step one CUDA graph (predictor, conditional
    # Newton loop with the device-side convergence check)
    gpu.set_graph(m, True)
    m.analyze(1)                                   # builds the graph, untimed
    sampler = ClockSampler()
    sampler.start()
    barrier()
    ev0.record(stream)
    stats = m.analyze(args.steps)
    ev1.record(stream)
    barrier()
    clocks = sampler.stop()
    dt = max_over_ranks(ev0.elapsed_time(ev1) * 1e-3, world, torch, dist)
    graph_steps = gpu.graph_steps(m)
    frame_steps = args.frames * args.steps * world
    value = frame_steps / dt
    newton = sum(s_[0] for s_ in stats)

    # end to end through the C ABI: every step xg_analyze, then the committed
    # displacements of all frames copied to pinned host memory (a recorder)
    uh = torch.empty(m.nu, dtype=torch.float64).pin_memory()
    L = gpu.lib()
    lam = C.c_double()
    st_buf = (gpu.xg_step_stats * 1)()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        gpu._check(L.xg_analyze(m.h, 1, st_buf))
        gpu._check(L.xg_get_disp(m.h, C.c_void_p(uh.data_ptr()), C.byref(lam)))
    barrier()
    dt_e2e = max_over_ranks(time.perf_counter() - t0, world, torch, dist)
    e2e_value = args.frames * args.e2e_steps * world / dt_e2e
    m.close()

    # the per-model GPU loop: the same kernels, one frame per model, on a
    # sample of the batch's frames over the same window of their records
    t_loop, n_loop = 0.0, 0
    for d, p in parts[:BATCH_SAMPLE]:
        mm = gpu.DeviceModel(d)
        mm.set_system(gpu.XG_SYSTEM_PROFILE_SPD)
        mm.set_phase(p[0])
        mm.analyze(lead + args.warmup)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        mm.analyze(args.steps)
        torch.cuda.synchronize()
        t_loop += time.perf_counter() - t0
        n_loop += args.steps
        mm.close()
    loop_value = n_loop / t_loop
    if rank != 0:
        dist.destroy_process_group()
        return None
    kernels = {k: v for k, v in prof.items() if v[1] > 0 and k != "return_map_cap_hits"}
    dominant = max(kernels, key=lambda k: kernels[k][0])
    dom_ms, dom_launches = kernels[dominant]
    peak, peak_kind = measured_peaks()
    alg = frame_alg_bytes(desc, 0, 0)["fbc_update"]
    achieved = alg / (dom_ms * 1e-3 / max(dom_launches, 1)) / 1e9 if dominant == "fbc_update" \
        else None
    line = {
        "metric": "frame-steps/s (batched)", "value": value, "unit": "frame time steps/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded frames and Kanai-Tajimi records)",
        "config": {"workload": f"{args.frames} independent 2D steel frames under their own ground motions: "
                               "Newmark time steps, each frame under its own record",
                   "frames": args.frames, "elements": desc.meta["elements"],
                   "fiber_points": desc.meta["fiber_points"], "equations": m.neq,
                   "timed_window": f"steps {lead + args.warmup + args.steps + 1}.."
                                   f"{lead + args.warmup + 2 * args.steps + 1} of the records "
                                   f"(dt 0.01 s)",
                   "step": "one CUDA graph per time step (conditional Newton loop)",
                   "system": "ProfileSPD: every frame's LDL' in its own band, one launch",
                   "parallelism": f"replicas x{world}"},
        "newton_iters_per_step": newton / args.steps,
        "graph_steps": graph_steps,
        "host_loop": {"value": args.frames * args.steps * world / dt_host,
                      "unit": "frame time steps/s",
                      "newton_iters_per_step": sum(s_[0] for s_ in stats_h) / args.steps,
                      "ip_updates_per_s": points / dt_host,
                      "note": "the preceding steps, host-driven Newton loop with per-kernel "
                              "timing (kernels_ms_per_step)"},
        "per_model_gpu_loop": {"value": loop_value, "unit": "frame time steps/s",
                               "frames": min(BATCH_SAMPLE, len(parts)),
                               "note": "the same kernels, one frame per model, same steps"},
        "batched_over_per_model": value / loop_value,
        "autotuned": {"elements_per_block": tuned[0], "pcg_rows_per_block": tuned[1],
                      "still_sampling": tuned[2]},
        "e2e": {"value": e2e_value, "unit": "frame time steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": int(uh.numel() * 8),
                "path": "xg_analyze + xg_get_disp into pinned host memory every step; the "
                        "records are resident"},
        "gpu_launches": int(sum(v[1] for v in kernels.values())),
        "roofline": {"bound": "hbm", "kernel": dominant,
                     "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak if achieved and peak else None,
                     "peak_source": peak_kind, "traffic": ncu_traffic("batch", dominant),
                     "algorithmic_bytes_per_launch": alg,
                     "limit": "the FP64 pipe, not HBM: 78.6 % active under ncu "
                              "(profiles/k_fbc_update_batch_c3.md); the fraction above is the "
                              "kernel's HBM view"},
        "kernels_ms_per_step": {k: v[0] / args.steps for k, v in kernels.items()},
        "clocks": clocks,
        "setup_s": t_setup,
    }
    if not args.no_cpu_baseline:
        rate, sample = batch_cpu_sample(parts[:BATCH_CPU_FRAMES], lead + args.warmup,
                                        args.steps)
        line["cpu_baseline"] = {"value": rate, "unit": "frame time steps/s", "cores": 1,
                                "kind": "port", "sample": sample}
    if world > 1:
        dist.destroy_process_group()
    return line


def _batch_cpu(parts, lead, steps):
    from oracle import port
    from xara_gb300._abi import PhaseDesc
    t, n = 0.0, 0
    for d, p in parts:
        o = port.OracleModel(d)
        kw = dict(p[0].kw)
        a = PhaseDesc(**{**kw, "num_steps": lead}, gm_accel=p[0].gm_accel)
        o.run([a])
        b = PhaseDesc(**{**kw, "num_steps": steps}, gm_accel=p[0].gm_accel)
        t0 = time.perf_counter()
        o.run([b])
        t += time.perf_counter() - t0
        n += steps
        o.close()
    return n, t


def batch_cpu_sample(parts, lead, steps):
    n, t = _batch_cpu(parts, lead, steps)
    return n / t, (f"{len(parts)} frames of the batch, steps {lead}..{lead + steps} each "
                   f"(Newmark, Newton, ProfileSPD), 1 thread")


def _batch_worker(args):
    idx, lead, steps, nframes = args
    _, _, parts = batch_model(nframes, lead + steps + 2)
    return _batch_cpu([parts[i] for i in idx], lead, steps)


def run_reference_batch(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return None
    import multiprocessing as mp
    cores = os.cpu_count() or 1
    lead = args.batch_lead + args.warmup
    per = 2
    jobs = [(list(range(c * per, (c + 1) * per)), lead, args.steps, args.frames)
            for c in range(cores)]
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(cores) as pool:
        res = pool.map(_batch_worker, jobs, chunksize=1)
    wall = time.perf_counter() - t0
    n = sum(r[0] for r in res)
    tmax = max(r[1] for r in res)
    value = n / tmax
    line = {
        "impl": "reference", "metric": "frame-steps/s (batched)", "value": value,
        "unit": "frame time steps/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * tmax / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded frames and Kanai-Tajimi records)",
        "config": {"workload": f"{args.frames} independent 2D steel frames under their own ground motions"},
        "cpu_baseline": {"value": value, "unit": "frame time steps/s", "cores": cores,
                         "kind": "port",
                         "sample": f"{cores} processes x {per} frames, steps {lead}.."
                                   f"{lead + args.steps}"},
        "e2e": {"value": value, "unit": "frame time steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "wall_s": wall,
    }
    return line


# ---------------------------------------------------------------------------
# adjoint: gradients of a transient response (64 frames, 2,000 steps)
# ---------------------------------------------------------------------------
def run_adjoint(args):
    world, rank, local, torch, dist = dist_setup()
    from xara_gb300 import configs, gpu
    from xara_gb300.adjoint import frame_response
    N, K = args.adj_steps, args.ckpt_every
    desc, phases = configs.adjoint_frames(n_frames=args.adj_frames, steps=N, seed=0)
    ph = phases[0]
    obj = (desc.meta["obj_node"], desc.meta["obj_dof"], desc.meta["obj_weight"])
    q0 = desc.uni_param.reshape(-1, 12).copy()
    m = gpu.DeviceModel(desc)
    m.set_system(gpu.XG_SYSTEM_PROFILE_SPD)
    stream = torch.cuda.ExternalStream(gpu.model_stream(m))

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    def timed(fn):
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        barrier()
        ev0.record(stream)
        out = fn()
        ev1.record(stream)
        barrier()
        return out, max_over_ranks(ev0.elapsed_time(ev1) * 1e-3, world, torch, dist)

    # warm-up: a short run forward and backward
    w = min(N, 10 * args.warmup)
    gpu.adjoint_forward(m, ph, w, max(1, w // 3), *obj)
    gpu.adjoint_backward(m)
    # the plain forward run (xg_analyze)
    m.reset()
    m.set_phase(ph)
    sampler = ClockSampler()
    sampler.start()
    gpu.profile_enable(m, True)
    stats, t_fwd = timed(lambda: m.analyze(N))
    prof = gpu.profile_read(m)
    gpu.profile_enable(m, False)
    # the same run with checkpoints, then the reverse sweep
    m.reset()
    J, t_fwd_ck = timed(lambda: gpu.adjoint_forward(m, ph, N, K, *obj))
    g, t_bwd = timed(lambda: gpu.adjoint_backward(m))
    clocks = sampler.stop()
    # end to end through the autograd function: parameters from and the
    # gradient to host memory
    theta = torch.tensor(q0[:, :3], dtype=torch.float64, requires_grad=True)
    barrier()
    t0 = time.perf_counter()
    Jt = frame_response(theta, m, ph, N, K, obj)
    Jt.backward()
    barrier()
    t_e2e = max_over_ranks(time.perf_counter() - t0, world, torch, dist)
    # central finite differences (h = 1e-6 relative) of one directional
    # derivative, frame by frame: every frame's objective term against the
    # adjoint restricted to its members.  The hysteretic response is only
    # piecewise smooth (a fiber's load reversal can move by a step under a
    # perturbation), so a few frames' difference quotients do not converge
    # in h; the check reports how many frames agree.
    nf = args.adj_frames
    efr = desc.meta["member_frame"]
    rng = np.random.default_rng(1)
    d = rng.normal(size=q0[:, :3].shape) * np.abs(q0[:, :3])
    h = 1e-6
    Jt = {}
    for sgn in (1, -1):
        q = q0.copy()
        q[:, :3] += sgn * h * d
        gpu.set_uniaxial_params(m, q)
        gpu.adjoint_forward(m, ph, N, K, *obj)
        Jt[sgn] = gpu.adjoint_objective_terms(m, nf)
    fd_f = (Jt[1] - Jt[-1]) / (2 * h)
    ad_f = np.array([(g[efr == f] * d[efr == f]).sum() for f in range(nf)])
    rel = np.abs(ad_f - fd_f) / np.maximum(np.abs(fd_f), 1e-300)
    ad, fd = float(ad_f.sum()), float(fd_f.sum())
    m.close()
    if rank != 0:
        dist.destroy_process_group()
        return None
    kernels = {k: v for k, v in prof.items() if v[1] > 0 and k != "return_map_cap_hits"}
    newton = sum(s_[0] for s_ in stats)
    line = {
        "metric": "adjoint/forward time", "value": t_bwd / t_fwd, "unit": "ratio",
        "n_gpus": world, "steps": N, "warmup": w, "ms_per_step": 1e3 * t_bwd / N,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded frames and Kanai-Tajimi records)",
        "config": {"workload": f"gradient of the summed squared roof drift of {args.adj_frames} "
                               f"2D steel frames over {N} Newmark steps "
                               f"w.r.t. every member's Steel02 Fy, E0, b",
                   "frames": args.adj_frames, "members": int(desc.num_elems),
                   "parameters": int(3 * desc.num_elems), "checkpoint_every": K,
                   "system": "ProfileSPD (a band per frame)",
                   "parallelism": f"replicas x{world}"},
        "forward_s": t_fwd, "forward_with_checkpoints_s": t_fwd_ck, "reverse_sweep_s": t_bwd,
        "gradient_over_forward": (t_fwd_ck + t_bwd) / t_fwd,
        "newton_iters_per_step": newton / N,
        "J": J,
        "fd_check": {"h": h, "frames": nf,
                     "median_relative_difference": float(np.median(rel)),
                     "frames_within_1e-6": int((rel < 1e-6).sum()),
                     "frames_within_1e-3": int((rel < 1e-3).sum()),
                     "directional_adjoint_all_frames": ad, "central_fd_all_frames": fd},
        "e2e": {"value": t_e2e / t_fwd, "unit": "ratio (autograd forward+backward / forward)",
                "seconds": t_e2e, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0,
                "path": "xara_gb300.adjoint.frame_response(theta on the host) then backward()"},
        "gpu_launches": int(sum(v[1] for v in kernels.values())),
        "kernels_ms_forward": {k: v[0] for k, v in kernels.items()},
        "clocks": clocks,
    }
    if not args.no_cpu_baseline:
        _, _, parts = configs.frame_batch(2, steps=60, seed=0, return_parts=True)
        rate, sample = batch_cpu_sample(parts, 0, 50)
        line["cpu_baseline"] = {
            "value": rate, "unit": "frame time steps/s (forward)", "cores": 1, "kind": "port",
            "sample": sample + "; the reference has no Steel02 sensitivity, so a CPU gradient "
                      f"by central differences costs {2 * 3 * int(desc.num_elems)} forward runs"}
    if world > 1:
        dist.destroy_process_group()
    return line


def run_adjoint_fd(args):
    """Where central differences and the adjoint of the 2,000-step gradient
    disagree, and why.  For the frames of the adjoint workload (64 frames,
    one Steel02 per member, the same random direction of every member's Fy,
    E0, b as the adjoint workload's check):

    * the per-frame relative difference of the adjoint directional
      derivative and h = 1e-6 central differences over the whole record;
    * for every frame, the first step at which the +h and -h runs put a
      Steel02 fiber of the frame on different branches (the Menegotto-Pinto
      state kon of any fiber differs between the two runs' committed
      records): past it the response is not differentiable along the
      perturbation, and the difference quotient measures a branch switch;
    * for the frames that disagree, adjoint and central differences again,
      over the record up to the step before that switch;
    * the adjoint and central differences at h = 1e-4 ... 1e-8 over 300,
      1,000 and 2,000 steps;
    * the direct differentiation (DDM, forward mode, independent code) along
      the same direction, frame by frame through each frame's objective
      term, against the adjoint over the whole record.

    ``--fd-parts ddm`` stops after the whole-record comparison of the three."""
    world, rank, local, torch, dist = dist_setup()
    if rank != 0:
        return None
    from xara_gb300 import configs, gpu
    N, K = args.adj_steps, args.ckpt_every
    desc, phases = configs.adjoint_frames(n_frames=args.adj_frames, steps=N, seed=0)
    ph = phases[0]
    obj = (desc.meta["obj_node"], desc.meta["obj_dof"], desc.meta["obj_weight"])
    q0 = desc.uni_param.reshape(-1, 12).copy()
    nf = args.adj_frames
    efr = np.asarray(desc.meta["member_frame"])
    d = np.random.default_rng(1).normal(size=q0[:, :3].shape) * np.abs(q0[:, :3])
    m = gpu.DeviceModel(desc)
    m.set_system(gpu.XG_SYSTEM_PROFILE_SPD)
    t0 = time.perf_counter()

    def adjoint(H):
        gpu.set_uniaxial_params(m, q0)
        gpu.adjoint_forward(m, ph, H, K, *obj)
        g = gpu.adjoint_backward(m)
        return np.array([(g[efr == f] * d[efr == f]).sum() for f in range(nf)])

    def central(H, h):
        J = {}
        for sgn in (1, -1):
            q = q0.copy()
            q[:, :3] += sgn * h * d
            gpu.set_uniaxial_params(m, q)
            gpu.adjoint_forward(m, ph, H, K, *obj)
            J[sgn] = gpu.adjoint_objective_terms(m, nf)
        gpu.set_uniaxial_params(m, q0)
        return (J[1] - J[-1]) / (2 * h)

    def rel(a, b):
        return np.abs(a - b) / np.maximum(np.abs(b), 1e-300)

    h0 = 1e-6
    ta = time.perf_counter()
    ad_full = adjoint(N)
    t_adjoint = time.perf_counter() - ta
    fd_full = central(N, h0)
    rel_full = rel(ad_full, fd_full)
    bad = [int(f) for f in np.nonzero(rel_full > 1e-3)[0]]
    # the DDM along d: every frame's directional derivative from its term
    m.reset()
    gpu.set_uniaxial_params(m, q0)
    td = time.perf_counter()
    gpu.ddm_forward(m, ph, N, d[None], *obj)
    t_ddm = time.perf_counter() - td
    ddm_full = gpu.ddm_objective_terms(m, 0, nf)
    m.reset()
    rel_ddm = rel(ad_full, ddm_full)
    ddm = {"median_relative_difference_to_adjoint": float(np.median(rel_ddm)),
           "max_relative_difference_to_adjoint": float(rel_ddm.max()),
           "frames_within_1e-9": int((rel_ddm < 1e-9).sum()),
           "disagreeing_frames": {str(f): {"adjoint": float(ad_full[f]), "ddm": float(ddm_full[f]),
                                           "central": float(fd_full[f])} for f in bad},
           "adjoint_s": t_adjoint, "ddm_s": t_ddm}
    if getattr(args, "fd_parts", "all") == "ddm":
        m.close()
        return {
            "metric": "adjoint vs DDM vs central differences, frame by frame",
            "unit": "relative difference",
            "config": {"workload": f"gradient of the summed squared roof drift of {nf} 2D steel "
                                   f"frames over {N} Newmark steps w.r.t. every member's Steel02 "
                                   f"Fy, E0, b; one random direction", "frames": nf,
                       "members": int(desc.num_elems), "checkpoint_every": K},
            "whole_record": {"h": h0, "median": float(np.median(rel_full)),
                             "within_1e-6": int((rel_full < 1e-6).sum()),
                             "within_1e-3": int((rel_full < 1e-3).sum()),
                             "disagreeing_frames": bad},
            "ddm": ddm, "wall_s": time.perf_counter() - t0}

    # the first step at which the +h and -h runs take different branches
    runs = []
    for sgn in (1, -1):
        mm = gpu.DeviceModel(desc)
        mm.set_system(gpu.XG_SYSTEM_PROFILE_SPD)
        q = q0.copy()
        q[:, :3] += sgn * h0 * d
        gpu.set_uniaxial_params(mm, q)
        mm.set_phase(ph)
        runs.append(mm)
    first = np.full(nf, -1)
    ne = desc.num_elems
    for n in range(N):
        kons = []
        for mm in runs:
            mm.analyze(1)
            kons.append(mm.fiber_records()[:, 7].reshape(ne, -1))
        switched = np.unique(efr[(kons[0] != kons[1]).any(axis=1)])
        new = switched[first[switched] < 0]
        first[new] = n + 1
        if (first >= 0).all():
            break
    for mm in runs:
        mm.close()

    # the disagreeing frames before their first branch switch
    before = {}
    for H in sorted({int(first[f]) - 1 for f in bad if first[f] > 1}):
        ad_h, fd_h = adjoint(H), central(H, h0)
        for f in bad:
            if int(first[f]) - 1 == H:
                before[f] = {"steps": H, "adjoint": float(ad_h[f]), "central": float(fd_h[f]),
                             "relative_difference": float(rel(ad_h[f], fd_h[f]))}
    # h sweeps over three horizons
    sweep = {}
    for H in (300, 1000, N):
        ad_h = adjoint(H)
        rows = {}
        for h in (1e-4, 1e-5, 1e-6, 1e-7, 1e-8):
            fd_h = central(H, h)
            r = rel(ad_h, fd_h)
            rows[f"{h:g}"] = {"median": float(np.median(r)), "within_1e-6": int((r < 1e-6).sum()),
                              "within_1e-3": int((r < 1e-3).sum()),
                              "disagreeing_frames_central": [float(fd_h[f]) for f in bad]}
        sweep[str(H)] = {"adjoint_of_disagreeing_frames": [float(ad_h[f]) for f in bad],
                         "h": rows}
    m.close()
    return {
        "metric": "adjoint vs central differences, frame by frame", "unit": "relative difference",
        "config": {"workload": f"gradient of the summed squared roof drift of {nf} 2D steel "
                               f"frames over {N} Newmark steps w.r.t. every member's Steel02 Fy, "
                               f"E0, b; one random direction",
                   "frames": nf, "members": int(ne), "checkpoint_every": K},
        "whole_record": {"h": h0, "median": float(np.median(rel_full)),
                         "within_1e-6": int((rel_full < 1e-6).sum()),
                         "within_1e-3": int((rel_full < 1e-3).sum()),
                         "disagreeing_frames": bad,
                         "relative_difference": [float(rel_full[f]) for f in bad]},
        "first_branch_switch_step": {str(f): int(first[f]) for f in range(nf)},
        "disagreeing_frames_before_their_switch": {str(f): v for f, v in before.items()},
        "h_sweep": sweep,
        "ddm": ddm,
        "wall_s": time.perf_counter() - t0,
    }


def run_reference_adjoint(args):
    if int(os.environ.get("RANK", "0")) != 0:
        return None
    return {"impl": "reference", "unavailable":
            "the reference has no Steel02 stress sensitivity (its DDM, computeGradients, "
            "covers Steel01/Concrete01), so it has no gradient path for this workload; its "
            "CPU forward is timed by --workload batch"}


# ---------------------------------------------------------------------------
# brick: the element phase of the stdBrick J2 block
# ---------------------------------------------------------------------------
def brick_trial_field(desc, nx, ny, nz, eps=2.5e-3):
    """A seeded, spatially varying compression field that leaves part of the
    block elastic and part plastic (sigma0 is U[200, 300] MPa per element)."""
    rng = np.random.default_rng(7)
    crd = desc.node_crd.reshape(-1, 3)
    x, y, z = crd[:, 0] / nx, crd[:, 1] / ny, crd[:, 2] / nz
    shape = 1.0 + 0.6 * np.sin(2 * np.pi * x) * np.cos(np.pi * y)
    u = np.zeros((len(crd), 3))
    u[:, 2] = -eps * nz * z * shape
    u[:, 0] = 0.3 * eps * nx * (x - 0.5) * z
    u[:, 1] = 0.3 * eps * ny * (y - 0.5) * z
    u += rng.normal(0.0, 1e-6, size=u.shape) * (z[:, None] > 0)
    return u.ravel()


def brick_alg_bytes(npts, ne, nn, nnz, neq):
    """Bytes the element phase must move, per the per-unit figures: per
    integration point 56 B of committed history read (plastic strain 6 + xi)
    and 56 B of trial history written; per node 48 B (coordinates and trial
    displacements); 8 B per CSR value written; 8 B per residual entry."""
    return {
        "phase": npts * 112 + nn * 48 + nnz * 8 + neq * 8,
        "brick_update": npts * (112 + 48 + 72) + nn * 48,
        "brick_assemble": npts * (48 + 72) + ne * (576 + 24) * 8 + nn * 24,
        "gather_tangent": nnz * 8,
        "gather_resid": neq * 8,
    }


def pcg_iteration_bytes(kb, blocks, nnz, neq):
    """Bytes one PCG iteration must move.  With the node-block copy (block
    order kb > 0): per block its kb*kb values as float pairs (8 B each, the
    zero padding of nodes with fewer free dofs included) and a 4 B column
    index; without it: per CSR entry an 8 B value and a 4 B column.  Per
    equation 131 B of vectors: q written and p read by the SpMV (16), x and r
    read and written, p and q read, z written (56), the inverted diagonal
    block (24 for 3 x 3 blocks), z and p read, p written and its split copy
    (35)."""
    matrix = blocks * (8 * kb * kb + 4) if kb > 0 else 12 * nnz
    return matrix + 131 * neq


def brick_cpu_sample(seconds=12.0):
    from oracle import port
    from xara_gb300 import configs
    desc, _ = configs.brick_block(**BRICK_SAMPLE, steps=1)
    o = port.OracleModel(desc)
    U = brick_trial_field(desc, **BRICK_SAMPLE)
    npts = desc.num_elems * 8
    o.elem_state(U)
    n, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        o.elem_state(U)
        n += 1
    dt = time.perf_counter() - t0
    s = BRICK_SAMPLE
    return npts * n / dt, (f"brick J2 {s['nx']}x{s['ny']}x{s['nz']} ({desc.num_elems} "
                           f"elements, {npts} points), {n} element phases")


def _brick_worker(args):
    seconds, = args
    rate, _ = brick_cpu_sample(seconds)
    return rate


def run_reference_brick(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return None
    import multiprocessing as mp
    cores = os.cpu_count() or 1
    per_step = 4.0
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        for _ in range(args.warmup):
            pool.map(_brick_worker, [(0.5,)] * cores)
        t0 = time.perf_counter()
        rates = []
        for _ in range(args.steps):
            rates.append(sum(pool.map(_brick_worker, [(per_step,)] * cores)))
        wall = time.perf_counter() - t0
    value = float(np.mean(rates))
    npts = int(np.prod(args.brick_dims)) * 8
    s = BRICK_SAMPLE
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * npts / value, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": "stdBrick J2 128x128x64 element phase (one Newton iteration)",
                   "elements": npts // 8, "points": npts},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"brick J2 {s['nx']}x{s['ny']}x{s['nz']} element phase, "
                                   f"{cores} processes x {per_step:.0f} s per step"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "wall_s": wall,
    }
    return line


def run_brick(args):
    world, rank, local, torch, dist = dist_setup()
    from xara_gb300 import configs, gpu
    dims = dict(zip(("nx", "ny", "nz"), args.brick_dims))
    desc, _ = configs.brick_block(**dims, steps=1)
    npts = desc.num_elems * 8
    t_setup = time.perf_counter()
    m = gpu.DeviceModel(desc)
    m.set_system(gpu.XG_SYSTEM_BJPCG)
    t_setup = time.perf_counter() - t_setup
    U = brick_trial_field(desc, **dims)
    m.set_trial_disp(U)
    fp64_peak = fp64_peak_probe()
    stream = torch.cuda.ExternalStream(gpu.model_stream(m))

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        m.update(False, False)
    gpu.profile_enable(m, True)
    sampler = ClockSampler()
    sampler.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    barrier()
    ev0.record(stream)
    for _ in range(args.steps):
        m.update(False, False)
    ev1.record(stream)
    barrier()
    clocks = sampler.stop()
    dt = ev0.elapsed_time(ev1) * 1e-3
    prof = gpu.profile_read(m)
    gpu.profile_enable(m, False)
    value = job_rate(npts * args.steps, dt, world, torch, dist)
    dt = max_over_ranks(dt, world, torch, dist)

    # a whole Newton iteration: the element phase, then the block-Jacobi PCG
    # solve of the assembled tangent to rtol 1e-10 (the configuration's
    # `system CudaBJPCG`), the right-hand side the assembled residual
    L = gpu.lib()
    L.xg_soe_solve_device.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_int,
                                      C.POINTER(C.c_int), C.POINTER(C.c_double)]
    bdev = torch.empty(m.neq, dtype=torch.float64, device="cuda")
    xdev = torch.empty(m.neq, dtype=torch.float64, device="cuda")
    newton = None
    if not args.no_analysis:
        gen = torch.Generator(device="cpu").manual_seed(3)
        bdev.copy_(torch.randn(m.neq, generator=gen, dtype=torch.float64))
        it_c, rr_c = C.c_int(), C.c_double()
        gpu.profile_enable(m, True)
        t_it = []
        for k in range(2):
            barrier()
            ev0.record(stream)
            m.update(False, False)
            gpu._check(L.xg_soe_solve_device(m.h, C.c_void_p(bdev.data_ptr()),
                                             C.c_void_p(xdev.data_ptr()), 1e-10, 20000,
                                             C.byref(it_c), C.byref(rr_c)))
            ev1.record(stream)
            barrier()
            t_it.append(ev0.elapsed_time(ev1) * 1e-3)
        gpu.profile_enable(m, False)
        pcg_it = it_c.value
        kb, nblocks, nchunked = C.c_int(), C.c_longlong(), C.c_longlong()
        gpu._check(L.xg_model_pcg_layout(m.h, C.byref(kb), C.byref(nblocks), C.byref(nchunked)))
        pcg_bytes = pcg_iteration_bytes(kb.value, nblocks.value, m.nnz, m.neq)
        pcg_s = t_it[-1] - dt / args.steps         # the iteration less its element phase
        newton = {"newton_iters_per_s": 1.0 / t_it[-1], "ms_per_newton_iteration": 1e3 * t_it[-1],
                  "pcg_iterations": pcg_it, "pcg_relative_residual": rr_c.value,
                  "pcg_ms": 1e3 * pcg_s, "pcg_ms_per_iteration": 1e3 * pcg_s / max(pcg_it, 1),
                  "pcg_GBps": pcg_bytes * pcg_it / pcg_s / 1e9 if pcg_s > 0 else None,
                  "pcg_bytes_per_iteration": pcg_bytes,
                  "pcg_block_order": kb.value, "pcg_blocks": nblocks.value,
                  "pcg_chunked_rows": nchunked.value,
                  "rhs": "seeded random right-hand side, x0 = 0, rtol 1e-10",
                  "arithmetic": "vectors, inner products and preconditioner in FP64; the SpMV's "
                                "products in float-float (2^-46 of each product); the "
                                "relative residual above is the recurrence's",
                  "ip_updates_per_s": npts / t_it[-1]}

    Uh = torch.from_numpy(U).pin_memory()
    resid = torch.empty(m.neq, dtype=torch.float64).pin_memory()
    ph = C.c_void_p(Uh.data_ptr())
    pr = C.c_void_p(resid.data_ptr())
    for _ in range(2):
        L.xg_elemset_set_trial_disp(m.h, ph)
        L.xg_elemset_update(m.h, None, pr)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        gpu._check(L.xg_elemset_set_trial_disp(m.h, ph))
        gpu._check(L.xg_elemset_update(m.h, None, pr))
    barrier()
    e2e_value = job_rate(npts * args.steps, time.perf_counter() - t0, world, torch, dist)
    if rank != 0:
        dist.destroy_process_group()
        return None
    alg = brick_alg_bytes(npts, desc.num_elems, desc.num_nodes, m.nnz, m.neq)
    kernels = {k: v for k, v in prof.items() if v[1] > 0 and k != "return_map_cap_hits"}
    dominant = max(kernels, key=lambda k: kernels[k][0])
    dom_ms, dom_launches = kernels[dominant]
    per_launch_s = dom_ms * 1e-3 / max(dom_launches, 1)
    if dominant.startswith("gather"):
        per_launch_s *= 2   # two kernels per gather launch group
    peak, peak_kind = measured_peaks()
    achieved = alg.get(dominant, alg["phase"]) / per_launch_s / 1e9
    phase_s = dt / args.steps
    flops = npts * 700 + desc.num_elems * 36 * 8 * 64
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * phase_s,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded trial displacement field)",
        "config": {"workload": f"stdBrick J2 {dims['nx']}x{dims['ny']}x{dims['nz']} "
                               "element phase (one Newton iteration)",
                   "elements": desc.num_elems, "points": npts, "equations": m.neq,
                   "nnz": m.nnz, "parallelism": f"replicas x{world}",
                   "l2": "inputs larger than L2 (no flush needed)",
                   "arithmetic": "J2 state, resisting force and assembled values in FP64; the "
                                 "tangent's node-pair sums in float-float (pairs of floats, "
                                 "2^-46 of each product), within 1e-12 of each row's largest "
                                 "entry of the FP64 oracle"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(U.nbytes),
                "d2h_bytes_per_step": int(resid.numel() * 8)},
        "gpu_launches": int(sum(v[1] for v in kernels.values())),
        "roofline": {"bound": "hbm", "kernel": dominant, "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak if peak else None,
                     "peak_source": peak_kind, "traffic": ncu_traffic("brick", dominant),
                     "algorithmic_bytes_per_launch": alg.get(dominant, alg["phase"]),
                     "limit": "instruction issue on the single-precision pipes, not HBM: the "
                              "tangent's float-float sums (IPC 2.3 of 4, FMA pipe 42 % under "
                              "ncu: profiles/k_brick_assemble_brick_c2_small.md)"},
        "fp64": {"est_flops_per_step": flops, "achieved_tflops": flops / phase_s / 1e12,
                 "peak_tflops_probe": fp64_peak,
                 "frac": (flops / phase_s / 1e12) / fp64_peak if fp64_peak else None},
        "kernels_ms_per_step": {k: v[0] / args.steps for k, v in kernels.items()},
        "clocks": clocks,
        "setup_s": t_setup,
        "newton_iteration": newton,
    }
    if newton and newton.get("pcg_GBps") and peak:
        newton["pcg_roofline_frac"] = newton["pcg_GBps"] / peak
    if not args.no_cpu_baseline:
        rate, sample = brick_cpu_sample()
        line["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": 1, "kind": "port",
                                "sample": sample}
    if world > 1:
        dist.destroy_process_group()
    return line


SUB_WORKLOADS = (("brick", "run_brick", dict(steps=10, warmup=3)),
                 ("batch", "run_batch", dict(steps=20, warmup=3)),
                 ("adjoint", "run_adjoint", dict(warmup=3)))


def sub_workloads(args):
    """The other BASELINE configurations, each measured as its own workload
    would measure it (own clocks, own CPU sample): the stdBrick J2 block
    128x128x64 (config 2), 4,096 batched frames (config 3) and the adjoint
    of 64 frames over 2,000 steps (config 4)."""
    import torch
    out = {}
    for name, fn, over in SUB_WORKLOADS:
        a = argparse.Namespace(**{**vars(args), **over, "workload": name})
        t0 = time.perf_counter()
        try:
            out[name] = globals()[fn](a)
        except Exception as e:            # one failing block must not lose the others
            out[name] = {"error": f"{type(e).__name__}: {e}"}
        out[name]["wall_s"] = time.perf_counter() - t0
        torch.cuda.empty_cache()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="frame3d",
                    choices=["frame3d", "brick", "batch", "adjoint", "adjoint-fd"])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="xara", choices=["xara", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-analysis", action="store_true",
                    help="frame3d: skip the rest of the pushover after the timed steps")
    ap.add_argument("--no-sub", action="store_true",
                    help="frame3d: skip the brick, batch and adjoint blocks")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--frames", type=int, default=BATCH_FRAMES)
    ap.add_argument("--batch-lead", type=int, default=150)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--adj-frames", type=int, default=64)
    ap.add_argument("--adj-steps", type=int, default=2000)
    ap.add_argument("--ckpt-every", type=int, default=100)
    ap.add_argument("--fd-parts", default="all", choices=["all", "ddm"],
                    help="adjoint-fd: the whole study, or only the adjoint / DDM / central "
                         "difference comparison over the whole record")
    ap.add_argument("--brick-dims", type=int, nargs=3, default=[BRICK["nx"], BRICK["ny"], BRICK["nz"]],
                    metavar=("NX", "NY", "NZ"), help="brick workload mesh (a smaller case for profiling)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        line = {"frame3d": run_reference_frame, "brick": run_reference_brick,
                "batch": run_reference_batch, "adjoint": run_reference_adjoint,
                "adjoint-fd": run_reference_adjoint}[args.workload](args)
    else:
        line = {"frame3d": run_frame, "brick": run_brick, "batch": run_batch,
                "adjoint": run_adjoint, "adjoint-fd": run_adjoint_fd}[args.workload](args)
        if (line is not None and args.workload == "frame3d" and not args.no_sub
                and line["n_gpus"] == 1):
            line["workloads"] = sub_workloads(args)
    if line is not None:
        print(json.dumps(line))
    return 0


if __name__ == "__main__":
    sys.exit(main())
