#!/usr/bin/env python3
"""Benchmark of the Newton-iteration hot path on one GB300.

Workload (default): the element phase of one Newton iteration of the
stdBrick J2 block, 128 x 128 x 64 elements (1,048,576 bricks, 8,388,608
integration points, 3,178,432 equations, 252,000,686 CSR non-zeros), FP64:
material state determination of every integration point (J2 radial return),
element tangents and resisting forces, and the deterministic assembly of the
CSR tangent and the residual (Domain::update + formTangent + formUnbalance).
A step is one such pass over all elements.  Inputs (model, history, trial
displacements) are resident in HBM when the timed region starts; every array
is far larger than the 129 MB L2, so no flush is needed between steps.

Metric: integration-point updates per second (higher is better).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl xara|reference]

--impl reference times the reference algorithm's CPU path (the C oracle,
a restatement of the reference's classes, compiled on this host) on the
host's cores, on a bounded sample of the same workload.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

WORKLOAD = dict(nx=128, ny=128, nz=64)
SAMPLE = dict(nx=24, ny=24, nz=12)   # CPU baseline sample (6,912 bricks)
METRIC = "IP updates/s"
UNIT = "integration-point updates/s"


def trial_field(desc, nx, ny, nz, eps=2.5e-3):
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


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
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


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs"), "of measured"
    return 6800.0, "of fallback"


def algorithmic_bytes(npts, ne, nn, nnz, neq):
    """Bytes the element phase must move, per the per-unit figures:
    per integration point 56 B of committed history read (plastic strain 6 +
    xi), 56 B of trial history written; per node 48 B (coordinates and trial
    displacements); 8 B per CSR value written; 8 B per residual entry."""
    return {
        "phase": npts * 112 + nn * 48 + nnz * 8 + neq * 8,
        # the material-update kernel: history in/out plus the trial stress
        # (6 doubles) and tangent parameters (9 doubles) it hands to the
        # element kernel, and the nodal data
        "brick_update": npts * (112 + 48 + 72) + nn * 48,
        # element kernel: point stress + tangent parameters in, node-pair
        # blocks (324 doubles) and element forces (24) out per element
        "brick_assemble": npts * (48 + 72) + ne * (324 + 24) * 8 + nn * 24,
        # gather of the tangent: every CSR value written once
        "gather_tangent": nnz * 8,
        "gather_resid": neq * 8,
    }


def flops_estimate(npts, ne):
    """FP64 flops of the element phase (counted from the kernels' source):
    J2 return map + strain + shape functions ~ 700 per point; node-pair
    stiffness blocks 36 pairs x 8 points x 64 flops per element."""
    return npts * 700 + ne * 36 * 8 * 64


def cpu_baseline_sample(seconds=12.0):
    """The oracle's element phase (single thread) on a sample of the workload."""
    from oracle import port
    from xara_gb300 import configs
    desc, _ = configs.brick_block(**SAMPLE, steps=1)
    o = port.OracleModel(desc)
    U = trial_field(desc, **SAMPLE)
    npts = desc.num_elems * 8
    o.elem_state(U)
    n, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        o.elem_state(U)
        n += 1
    dt = time.perf_counter() - t0
    return npts * n / dt, f"brick J2 {SAMPLE['nx']}x{SAMPLE['ny']}x{SAMPLE['nz']} " \
                          f"({desc.num_elems} elements, {npts} points), {n} element phases"


def _ref_worker(args):
    seconds, = args
    rate, _ = cpu_baseline_sample(seconds)
    return rate


def run_reference(args):
    """CPU path of the reference algorithm on all host cores (processes)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    import multiprocessing as mp
    cores = os.cpu_count() or 1
    per_step = 4.0
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        for _ in range(args.warmup):
            pool.map(_ref_worker, [(0.5,)] * cores)
        t0 = time.perf_counter()
        rates = []
        for _ in range(args.steps):
            rates.append(sum(pool.map(_ref_worker, [(per_step,)] * cores)))
        wall = time.perf_counter() - t0
    value = float(np.mean(rates))
    npts = WORKLOAD["nx"] * WORKLOAD["ny"] * WORKLOAD["nz"] * 8
    sample = (f"brick J2 {SAMPLE['nx']}x{SAMPLE['ny']}x{SAMPLE['nz']} element phase, "
              f"{cores} processes x {per_step:.0f} s per step")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * npts / value, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": "stdBrick J2 128x128x64 element phase (one Newton iteration)",
                   "elements": npts // 8, "points": npts, "l2": "inputs larger than L2"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "wall_s": wall,
    }
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="xara", choices=["xara", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--nx", type=int, default=WORKLOAD["nx"])
    ap.add_argument("--ny", type=int, default=WORKLOAD["ny"])
    ap.add_argument("--nz", type=int, default=WORKLOAD["nz"])
    args = ap.parse_args()
    WORKLOAD.update(nx=args.nx, ny=args.ny, nz=args.nz)
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        # one replica per GPU: the element phase of one model does not shard
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    import torch
    import torch.distributed as dist
    if world > 1:
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        torch.cuda.set_device(0)

    from xara_gb300 import configs, gpu
    desc, _ = configs.brick_block(**WORKLOAD, steps=1)
    npts = desc.num_elems * 8
    t_setup = time.perf_counter()
    m = gpu.DeviceModel(desc)
    t_setup = time.perf_counter() - t_setup
    U = trial_field(desc, **WORKLOAD)
    m.set_trial_disp(U)
    fp64_peak = C_double_probe()

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        m.update(False, False)
    gpu.profile_enable(m, True)
    sampler = ClockSampler(local if world == 1 else 0)
    sampler.start()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        m.update(False, False)
    barrier()
    dt = time.perf_counter() - t0
    clocks = sampler.stop()
    prof = gpu.profile_read(m)
    gpu.profile_enable(m, False)
    # max over ranks
    if world > 1:
        t = torch.tensor([dt], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dt = float(t.item())
    value = npts * args.steps * world / dt

    # end to end through the C ABI with host buffers: trial displacements in
    # from pinned host memory, the assembled resisting force back out
    Uh = torch.from_numpy(U).pin_memory().numpy()
    resid = torch.empty(m.neq, dtype=torch.float64).pin_memory().numpy()
    L = gpu.lib()
    import ctypes as C
    ph = Uh.ctypes.data_as(C.c_void_p)
    pr = resid.ctypes.data_as(C.c_void_p)
    for _ in range(2):
        L.xg_elemset_set_trial_disp(m.h, ph)
        L.xg_elemset_update(m.h, None, pr)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        gpu._check(L.xg_elemset_set_trial_disp(m.h, ph))
        gpu._check(L.xg_elemset_update(m.h, None, pr))
    barrier()
    dt_e2e = time.perf_counter() - t0
    if world > 1:
        t = torch.tensor([dt_e2e], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dt_e2e = float(t.item())
    e2e_value = npts * args.steps * world / dt_e2e

    if rank != 0:
        dist.destroy_process_group()
        return 0

    nn = desc.num_nodes
    alg = algorithmic_bytes(npts, desc.num_elems, nn, m.nnz, m.neq)
    kernels = {k: v for k, v in prof.items() if v[1] > 0 and k != "return_map_cap_hits"}
    dominant = max(kernels, key=lambda k: kernels[k][0])
    dom_ms, dom_launches = kernels[dominant]
    per_launch_s = dom_ms * 1e-3 / max(dom_launches, 1)
    if dominant.startswith("gather"):
        per_launch_s *= 2   # two kernels per gather launch group
    peak, peak_kind = measured_peaks()
    achieved = alg.get(dominant, alg["phase"]) / per_launch_s / 1e9
    traffic = _ncu_traffic(dominant)
    phase_s = dt / args.steps
    gpu_launches = sum(v[1] for v in kernels.values())
    flops = flops_estimate(npts, desc.num_elems)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * phase_s,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded trial displacement field)",
        "config": {"workload": f"stdBrick J2 {WORKLOAD['nx']}x{WORKLOAD['ny']}x{WORKLOAD['nz']} "
                               "element phase (one Newton iteration)",
                   "elements": desc.num_elems, "points": npts, "equations": m.neq,
                   "nnz": m.nnz, "parallelism": f"replicas x{world}",
                   "l2": "inputs larger than L2 (no flush needed)"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(U.nbytes),
                "d2h_bytes_per_step": int(resid.nbytes)},
        "gpu_launches": int(gpu_launches),
        "roofline": {"bound": "hbm", "kernel": dominant, "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak if peak else None,
                     "peak_source": peak_kind, "traffic": traffic,
                     "algorithmic_bytes_per_launch": alg.get(dominant, alg["phase"])},
        "phase_roofline": {"algorithmic_bytes": alg["phase"],
                           "achieved_gbs": alg["phase"] / phase_s / 1e9},
        "fp64": {"est_flops_per_step": flops, "achieved_tflops": flops / phase_s / 1e12,
                 "peak_tflops_probe": fp64_peak,
                 "frac": (flops / phase_s / 1e12) / fp64_peak if fp64_peak else None},
        "kernels_ms_per_step": {k: v[0] / args.steps for k, v in kernels.items()},
        "return_map_cap_hits": prof.get("return_map_cap_hits", (0, 0))[1],
        "clocks": clocks,
        "setup_s": t_setup,
    }
    if not args.no_cpu_baseline:
        rate, sample = cpu_baseline_sample()
        line["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": 1, "kind": "port",
                                "sample": sample}
    print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()
    return 0


def C_double_probe():
    import ctypes as C
    from xara_gb300 import gpu
    L = gpu.lib()
    v = C.c_double()
    L.xg_measure_fp64_peak.argtypes = [C.POINTER(C.c_double)]
    if L.xg_measure_fp64_peak(C.byref(v)) != 0:
        return None
    return v.value


def _ncu_traffic(kernel):
    """DRAM bytes per launch of the kernel from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "dram_traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        d = json.load(f)
    return d.get(kernel)


if __name__ == "__main__":
    sys.exit(main())
