#!/usr/bin/env python
"""Benchmark of the batched point-vs-SDF contact evaluation on GB300.

Workload (the batched BFS direction sweep on the peg-in-hole): 1024 pair
instances, each a 50k-point peg (cylinder r=0.49, length 2) against a socket
(cube [-1,1]^3 minus a z bore of r=0.5) stored as a 128^3 FP32 SDF grid; each
instance is pushed 0.0201 sideways along the lateral part of its Fibonacci-
sphere pull direction (a penetration of 1e-4 beyond the 0.01 collision
threshold) and moves along it.  Seeded synthetic inputs stand in for the
reference's download-only assembly datasets.

A step is one force evaluation with derivatives of the whole batch: detection
over every point of every instance, then force, dF/dq and dF/dqdot of every
active contact (ForceGeneralSDFContact::computeForceWithDerivative,
simulation/redmax/Force/ForceGeneralSDFContact.cpp:69-105), reduced per
instance in FP64.  The metric is contact-point evaluations per second of the
batched mixed-precision path (FP64 penetration depth and sums, FP32
per-contact algebra); the line also carries the plain per-instance FP64 GPU
path on the same inputs and the mixed path's error against it.

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]

--impl reference times the CPU restatement of the reference path (oracle/) on
the host cores on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import importlib
import json
import multiprocessing as mp
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
PKG = "assemble-them-all_gb300"
W = importlib.import_module(f"{PKG}.workloads")

METRIC = "SDF contact pts/s (batched force+Jacobian evaluation)"
UNIT = "contact-pts/s"
COL_TH = 0.01
PARAMS = (1e5, 1e3, 0.3, 1e3, 1.0, 1.0)  # kn, kt, mu, damping, scale, contact_scale
L2_BYTES = 129 * 2 ** 20
SIM_H = float(np.float32(5e-3))  # the reference reads the time step as FP32
SIM_GRAVITY = (0.0, 0.0, -9.8)
SIM_PULL = 1.0  # pull force magnitude along each direction (scaled by the mass, Body.cpp:267-268)


def instance_states(n, rank=0, world=1):
    """Pose / twist of each instance from its pull direction (workloads.direction_sweep_states):
    replica `rank` of `world` takes its own block of n directions of one shared sweep."""
    return W.direction_sweep_states(n, rank, world)


def build_workload(n_inst, n_pts, grid_n, rank=0, world=1):
    grid = W.socket_grid(grid_n, dtype=np.float32)
    pts = W.peg_points(n_pts, seed=0)
    return grid, pts, instance_states(n_inst, rank, world)


# --------------------------------------------------------------------------- CPU baseline (oracle)
_G = {}


def _cpu_init(grid_vals, mn, mx, dx, pts):
    from oracle import oracle as O
    _G["O"] = O
    _G["grid"] = O.Grid(grid_vals, mn, mx, dx, COL_TH)
    _G["pts"] = pts
    _G["prm"] = O.Params(*PARAMS)


def _cpu_eval(args):
    EA, phiA, EB, phiB = args
    O = _G["O"]
    t = time.perf_counter()
    O.pair_eval(_G["grid"], _G["pts"], EA, phiA, EB, phiB, _G["prm"], True)
    return time.perf_counter() - t


def _cpu_result(args):
    EA, phiA, EB, phiB = args
    fm, Km, Dm, _ = _G["O"].pair_eval(_G["grid"], _G["pts"], EA, phiA, EB, phiB, _G["prm"], True)
    return fm, Km, Dm


def _cpu_norm_sum(args):
    """Sum of |fm_i| over one instance's active contacts (the error scale of fm where the contacts'
    forces cancel), by the oracle."""
    EA, phiA, EB, phiB = args
    return _G["O"].pair_force_norm_sum(_G["grid"], _G["pts"], EA, phiA, EB, phiB, _G["prm"])


def _cpu_sim(args):
    """One scene of the direction sweep stepped by the oracle's BDF1 restatement."""
    d, steps = args
    O = _G["O"]
    m, inertia = W.cylinder_mass_props()
    mover = O.Mover(m, inertia, np.eye(4), np.eye(4), SIM_GRAVITY, SIM_H, np.concatenate([np.zeros(3), d]))
    pair = O.ScenePair(_G["grid"], _G["pts"], True, np.eye(4), _G["prm"])
    t = time.perf_counter()
    qs, qds, conv, its, evs = O.bdf1_steps(mover, [pair], np.zeros(3), np.zeros(3), steps)
    t_fwd = time.perf_counter() - t
    w = np.zeros((steps, 3))
    w[-1] = d  # L = displacement along the pull after the last step
    t = time.perf_counter()
    O.bdf1_backward(mover, [pair], qs, np.zeros(3), w)
    return t_fwd, int(evs.sum()), time.perf_counter() - t


# The reference's own ForceGeneralSDFContact (oracle/_ref, compiled from the reference's sources
# where they are staged) in the same kind of worker pool.
def _ref_init(grid_vals, mn, mx, dx, pts):
    from oracle import refsim
    sim, _ = refsim.make_pair_sim()
    sim.set_sdf("B", grid_vals, mn, mx, dx, COL_TH)
    sim.set_contact_points("A", pts)
    sim.set_contact_scale("A", PARAMS[5])
    _G["ref"] = sim


def _ref_eval(args):
    EA, phiA, EB, phiB = args
    sim = _G["ref"]
    sim.set_pose("A", EA, phiA)
    sim.set_pose("B", EB, phiB)
    t = time.perf_counter()
    sim.pair_force("A", "B", *PARAMS[:5], want_deriv=True)
    return time.perf_counter() - t


def _ref_result(args):
    EA, phiA, EB, phiB = args
    sim = _G["ref"]
    sim.set_pose("A", EA, phiA)
    sim.set_pose("B", EB, phiB)
    return sim.pair_force("A", "B", *PARAMS[:5], want_deriv=True)


def reference_library():
    """Whether oracle/_ref (the reference compiled from its own sources) is there, building it
    from the staged sources when they are present; the reason when it is not."""
    try:
        from oracle import refsim
    except Exception as e:  # pragma: no cover
        return False, f"oracle.refsim: {e}"
    if refsim.available():
        return True, ""
    if refsim.reference_root() is None:
        return False, "the reference's sources are not staged (baseline/_ref/src)"
    try:
        return refsim.build(), "build finished without the library"
    except Exception as e:
        return False, f"building the reference failed: {e}"


def ref_pool(grid, pts, procs):
    ctx = mp.get_context("spawn")
    return ctx.Pool(procs, initializer=_ref_init, initargs=(grid.values, grid.min_box, grid.max_box, grid.dx, pts))


def cpu_pool(grid, pts, procs):
    from oracle import oracle as O
    O.build()
    ctx = mp.get_context("spawn")
    return ctx.Pool(procs, initializer=_cpu_init, initargs=(grid.values, grid.min_box, grid.max_box, grid.dx, pts))


def ref_time(pool, states, idx):
    EA, phiA, EB, phiB = states
    t = time.perf_counter()
    pool.map(_ref_eval, [(EA[k], phiA[k], EB[k], phiB[k]) for k in idx], chunksize=1)
    return time.perf_counter() - t


def cpu_time(pool, states, idx):
    EA, phiA, EB, phiB = states
    t = time.perf_counter()
    pool.map(_cpu_eval, [(EA[k], phiA[k], EB[k], phiB[k]) for k in idx], chunksize=1)
    return time.perf_counter() - t


# --------------------------------------------------------------------------- helpers
def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if os.environ.get("SDFC_BENCH_BACKEND") != "gloo" else "gloo")
    return world, rank


def dist_max(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_sum(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def whole_job_rate(units_per_rank, seconds, world):
    """Weak-scaling aggregate: every replica processes `units_per_rank` units; the job's time is
    the slowest replica's.  Returns (units per second over all replicas, the max-over-ranks time)."""
    s = dist_max(seconds, world)
    return world * units_per_rank / s, s


def gather_rows(x, world):
    """Per-instance results of every rank, in rank order, on every rank (a host-side gather of
    the replicas' results; no device collective)."""
    if world == 1:
        return np.asarray(x)
    import torch.distributed as dist
    out = [None] * world
    dist.all_gather_object(out, np.asarray(x))
    return np.concatenate(out)


def rank_block(total, n, rank, world):
    """Replica `rank`'s block of n items of a workload of n * world items (`total` gives them all)."""
    return total[rank * n:(rank + 1) * n]


def dist_barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


class ClockSampler:
    """SM clock and clock-event (throttle) reasons sampled during the timed region: read-only
    NVML queries every 2 ms from a thread, or nvidia-smi every 100 ms where NVML cannot be
    loaded."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    # NVML clock-event reason bits (nvml.h: nvmlClocksEventReason*)
    REASON_BITS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
                   0x40: "hw_thermal_slowdown"}

    def __init__(self, device_index=0, uuid=None):
        self.proc = None
        self.thread = None
        self.samples, self.mask, self.mx = [], 0, 0.0
        try:
            self._start_nvml(device_index, uuid)
            return
        except Exception:
            self.thread = None
        # raw samples (the JSON line carries their summary); SDFC_CLOCKS_DIR keeps them elsewhere
        import tempfile
        self.out = os.path.join(os.environ.get("SDFC_CLOCKS_DIR", tempfile.gettempdir()), f"clocks_{os.getpid()}.csv")
        try:
            os.makedirs(os.path.dirname(self.out), exist_ok=True)
            self.fh = open(self.out, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={device_index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.fh,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def _start_nvml(self, device_index, uuid):
        import ctypes
        import threading
        lib = ctypes.CDLL("libnvidia-ml.so.1")
        if lib.nvmlInit_v2() != 0:
            raise OSError("nvmlInit")
        h = ctypes.c_void_p()
        rc = 1
        if uuid:
            rc = lib.nvmlDeviceGetHandleByUUID(uuid.encode(), ctypes.byref(h))
        if rc != 0:
            rc = lib.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(device_index), ctypes.byref(h))
        if rc != 0:
            raise OSError("nvml handle")
        try:
            reasons = lib.nvmlDeviceGetCurrentClocksEventReasons
        except AttributeError:
            reasons = lib.nvmlDeviceGetCurrentClocksThrottleReasons
        mx = ctypes.c_uint()
        if lib.nvmlDeviceGetMaxClockInfo(h, ctypes.c_int(1), ctypes.byref(mx)) == 0:  # NVML_CLOCK_SM
            self.mx = float(mx.value)
        self.stop_flag = threading.Event()

        def run():
            c, r = ctypes.c_uint(), ctypes.c_ulonglong()
            while not self.stop_flag.is_set():
                if lib.nvmlDeviceGetClockInfo(h, ctypes.c_int(1), ctypes.byref(c)) == 0:
                    self.samples.append(float(c.value))
                if reasons(h, ctypes.byref(r)) == 0:
                    self.mask |= r.value
                time.sleep(0.002)

        self.thread = threading.Thread(target=run, daemon=True)
        self.thread.start()
        time.sleep(0.01)  # the first samples precede the timed region

    def stop(self):
        if self.thread is not None:
            self.stop_flag.set()
            self.thread.join(timeout=5)
            if not self.samples:
                return None
            reasons = sorted(nm for bit, nm in self.REASON_BITS.items() if self.mask & bit)
            return {"sm_mhz": float(np.median(self.samples)), "sm_max_mhz": self.mx, "reasons": reasons,
                    "samples": len(self.samples), "source": "nvml"}
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, mx, reasons = [], 0.0, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in open(self.out):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm),
                "source": "nvidia-smi"}


def load_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return None


def profile_figures(fname):
    """name -> value pairs of a committed ncu summary under profiles/ (empty if absent)."""
    path = os.path.join(ROOT, "profiles", fname)
    out = {}
    if os.path.exists(path):
        for line in open(path):
            parts = line.split()
            if len(parts) >= 2 and not parts[0].startswith("#"):
                try:
                    out[parts[0]] = float(parts[1])
                except ValueError:
                    pass
    return out


def profile_traffic(name):
    """DRAM bytes per launch of `name` from the committed ncu summary, if one exists."""
    path = os.path.join(ROOT, "profiles", "ncu_dram_per_launch.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        parts = line.split()
        if len(parts) >= 2 and parts[0] == name:
            try:
                return float(parts[1])
            except ValueError:
                return None
    return None


# --------------------------------------------------------------------------- arms
def run_reference(args, world, rank):
    """The reference path's CPU cost on the host cores, on a bounded sample: the reference's own
    ForceGeneralSDFContact (oracle/_ref) one process per core where it can be built from the
    staged sources, else the oracle's C port of it."""
    if rank != 0:
        return
    grid, pts, states = build_workload(args.instances, args.points, args.grid)
    procs = os.cpu_count() or 1
    have_ref, why = reference_library() if not args.ref_port else (False, "--ref-port given")
    kind = "reference" if have_ref else "port"
    pool = ref_pool(grid, pts, procs) if have_ref else cpu_pool(grid, pts, procs)
    sample = min(args.instances, max(procs, args.ref_sample if have_ref else args.cpu_sample))
    rng = np.random.default_rng(0)
    timer = (lambda idx: ref_time(pool, states, idx)) if have_ref else (lambda idx: cpu_time(pool, states, idx))
    for _ in range(args.warmup):
        timer(rng.choice(args.instances, min(procs, args.instances), replace=False))
    times = []
    for _ in range(args.steps):
        times.append(timer(rng.choice(args.instances, sample, replace=False)))
    agreement = None
    if have_ref:  # the reference against the oracle port on two instances of the workload
        ref_out = pool.map(_ref_result, [tuple(x[k] for x in states) for k in (0, 1)])
        pool.close()
        port = cpu_pool(grid, pts, 2)
        port_out = port.map(_cpu_result, [tuple(x[k] for x in states) for k in (0, 1)])
        port.close()
        agreement = max(float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / max(np.linalg.norm(np.ravel(b)), 1e-300))
                        for r, p in zip(ref_out, port_out) for a, b in zip(r, p))
        pool = cpu_pool(grid, pts, procs) if args.sim_steps > 0 else None
    sim = cpu_sim_rate(pool, args.cpu_sim_scenes, min(args.sim_early, 25), procs) if args.sim_steps > 0 else None
    if pool is not None:
        pool.close()
    per_step = float(np.mean(times))
    value = sample * args.points / per_step
    sample_desc = f"{sample} of {args.instances} instances per step, derivative evaluation, one process per core"
    if have_ref:
        sample_desc += (f"; the reference's ForceGeneralSDFContact::computeForceWithDerivative (oracle/_ref); "
                        f"fm/Km/Dm against the oracle port {agreement:.1e} relative")
    else:
        sample_desc += f"; the oracle's C port ({why})"
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": per_step * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(args),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": procs, "kind": kind, "sample": sample_desc},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    if sim is not None:
        sim["kind"] = "port"  # the simulation sample always steps the oracle's BDF1 restatement
        line["sim"] = sim
    print(json.dumps(line), flush=True)


def workload_config(args):
    return {"workload": "batched BFS direction sweep, peg-in-hole (force+Jacobian evaluation)",
            "instances": args.instances, "points_per_instance": args.points, "grid": f"{args.grid}^3 fp32",
            "directions": "fibonacci sphere", "active_set": "peg pressed 1e-4 into the bore wall",
            "l2": "flushed between timed steps (256 MiB write)", "parallelism": "instances per GPU (replicas)"}


def rel_err(a, b):
    """|a - b| / max(min(|a|, |b|), 1e-4) (simulation/redmax/Utils.h:362-381), worst over instances."""
    a = a.reshape(len(a), -1)
    b = b.reshape(len(b), -1)
    e = np.linalg.norm(a - b, axis=1)
    d = np.maximum(np.minimum(np.linalg.norm(a, axis=1), np.linalg.norm(b, axis=1)), 1e-4)
    return float(np.max(e / d))


def run_gpu(args, world, rank):
    grid, pts, states = build_workload(args.instances, args.points, args.grid, rank, world)
    pool = None
    if rank == 0 and not args.no_cpu_baseline:
        pool = cpu_pool(grid, pts, os.cpu_count() or 1)  # spawned before the first CUDA call
    import torch

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    sdfc = importlib.import_module(f"{PKG}.sdfc")
    dev = torch.cuda.current_device()
    ctx = sdfc.Context(dev)
    g = ctx.upload_grid(grid.values, grid.min_box, grid.max_box, grid.dx, COL_TH, sdfc.STORAGE_F32)
    p = ctx.upload_points(pts, sdfc.STORAGE_F32)
    n = args.instances
    batch = ctx.batch([p] * n, [g] * n)
    batch.set_precision(sdfc.PRECISION_MIXED if args.precision == "mixed" else sdfc.PRECISION_FP64)
    EA, phiA, EB, phiB = states
    prm_rows = np.tile(np.array(PARAMS), (n, 1))
    cuda = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()  # noqa: E731
    dEA, dphiA, dEB, dphiB, dprm = cuda(EA), cuda(phiA), cuda(EB), cuda(phiB), cuda(prm_rows)
    fm = torch.zeros(n, 12, dtype=torch.float64, device="cuda")
    Km = torch.zeros(n, 144, dtype=torch.float64, device="cuda")
    Dm = torch.zeros(n, 144, dtype=torch.float64, device="cuda")
    nact = torch.zeros(n, dtype=torch.int32, device="cuda")
    st = torch.zeros(n, dtype=torch.int32, device="cuda")
    flush = torch.empty(2 * L2_BYTES, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.Stream()
    torch.cuda.synchronize()

    def step(b=batch):
        b.evaluate_device(dEA.data_ptr(), dphiA.data_ptr(), dEB.data_ptr(), dphiB.data_ptr(), dprm.data_ptr(),
                          fm.data_ptr(), Km.data_ptr(), Dm.data_ptr(), nact.data_ptr(), st.data_ptr(),
                          want_deriv=True, stream=stream.cuda_stream)

    tuning = None
    if args.tuning:  # a given launch configuration: form, slots, chunks per slot
        form, slots, per = args.tuning.split(",")
        batch.set_tuning(int(slots), {"ctas": 0, "workers": 1, "grid": 2}[form], chunks_per_slot=int(per))
    elif not args.no_autotune:  # the batch's launch configuration, timed once on these inputs
        tuning = batch.autotune(dEA.data_ptr(), dphiA.data_ptr(), dEB.data_ptr(), dphiB.data_ptr(), dprm.data_ptr(),
                                fm.data_ptr(), Km.data_ptr(), Dm.data_ptr(), nact.data_ptr(), st.data_ptr(),
                                want_deriv=True, stream=stream.cuda_stream)
    tuning_used = batch.tuning()
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            step()
        stream.synchronize()
        assert not st.any().item(), "non-finite contact output"
        n_active = int(nact.sum().item())
        nact_rows = nact.cpu().numpy().astype(np.int64)
        out_fast = (fm.cpu().numpy().copy(), Km.cpu().numpy().copy(), Dm.cpu().numpy().copy())

        # timed region: K steps, each bracketed by CUDA events on the launching stream, L2 flushed between
        dist_barrier(world)
        torch.cuda.synchronize()
        try:
            uuid = "GPU-" + str(torch.cuda.get_device_properties(dev).uuid)
        except Exception:
            uuid = None
        clocks = ClockSampler(dev, uuid)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        t0 = time.perf_counter()
        for a, b in ev:
            flush.zero_()
            a.record(stream)
            step()
            b.record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        clk = clocks.stop()
        dist_barrier(world)
        pts_per_step = n * args.points
        value, step_s = whole_job_rate(pts_per_step, float(np.mean([a.elapsed_time(b) for a, b in ev])) / 1e3, world)
        step_ms = step_s * 1e3

        # per-phase device times (separate pass with events between the launches)
        batch.set_timing(True)
        phases = []
        for _ in range(max(3, args.steps // 2)):
            flush.zero_()
            stream.synchronize()
            batch.evaluate_device(dEA.data_ptr(), dphiA.data_ptr(), dEB.data_ptr(), dphiB.data_ptr(),
                                  dprm.data_ptr(), fm.data_ptr(), Km.data_ptr(), Dm.data_ptr(), nact.data_ptr(),
                                  st.data_ptr(), want_deriv=True, stream=stream.cuda_stream)
            phases.append(batch.last_timing())
        batch.set_timing(False)
        det_ms, frc_ms, red_ms = (float(np.mean([x[i] for x in phases])) for i in range(3))
        rechecked = batch.recheck_count(reset=True) / (args.warmup + args.steps + len(phases))

    # the plain per-instance FP64 GPU path on the same inputs: a one-instance FP64 batch evaluated
    # once per instance on device arrays, the instances' launches back to back on the stream (no
    # host round trip per instance), CUDA events around the run
    plain = ctx.batch([p], [g])
    plain.set_precision(sdfc.PRECISION_FP64)
    params_rows = np.tile(np.array(PARAMS, dtype=np.float64), (n, 1))  # sdfc_params rows, as a C caller holds them
    m = n if args.full_error else min(n, args.plain_sample)
    pfm = torch.zeros(n, 12, dtype=torch.float64, device="cuda")
    pKm = torch.zeros(n, 144, dtype=torch.float64, device="cuda")
    pDm = torch.zeros(n, 144, dtype=torch.float64, device="cuda")
    off = lambda t, k, w: t.data_ptr() + 8 * w * k  # noqa: E731  (row k of an FP64 tensor of width w)
    ioff = lambda t, k: t.data_ptr() + 4 * k  # noqa: E731

    def plain_eval(k):
        plain.evaluate_device(off(dEA, k, 16), off(dphiA, k, 6), off(dEB, k, 16), off(dphiB, k, 6), off(dprm, k, 6),
                              off(pfm, k, 12), off(pKm, k, 144), off(pDm, k, 144), ioff(nact, k), ioff(st, k),
                              want_deriv=True, stream=stream.cuda_stream)

    with torch.cuda.stream(stream):
        for k in range(3):  # warm-up
            plain_eval(k)
        flush.zero_()
        pa, pb = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        pa.record(stream)
        for k in range(m):
            plain_eval(k)
        pb.record(stream)
        stream.synchronize()
    plain_rate = m * args.points / (pa.elapsed_time(pb) / 1e3)
    ref = (pfm.cpu().numpy()[:m], pKm.cpu().numpy().reshape(n, 12, 12)[:m], pDm.cpu().numpy().reshape(n, 12, 12)[:m])
    err = {"fm": rel_err(out_fast[0][:m], ref[0]), "Km": rel_err(out_fast[1][:m], ref[1]),
           "Dm": rel_err(out_fast[2][:m], ref[2]), "instances": m}

    # the batched path with FP64 per-contact algebra on the same batch (same launches, FP64 kernels)
    batch.set_precision(sdfc.PRECISION_FP64)
    with torch.cuda.stream(stream):
        for _ in range(2):
            step()
        f64_ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                  for _ in range(max(3, args.steps // 2))]
        for a, b in f64_ev:
            flush.zero_()
            a.record(stream)
            step()
            b.record(stream)
        stream.synchronize()
    f64_ms = float(np.mean([a.elapsed_time(b) for a, b in f64_ev]))
    batch.set_precision(sdfc.PRECISION_MIXED if args.precision == "mixed" else sdfc.PRECISION_FP64)

    # e2e through the C ABI with host buffers (H2D of the instance states, D2H of fm/Km/Dm into
    # result arrays the caller keeps across calls, as a simulator's force assembly does)
    e2e_out = (np.zeros((n, 12)), np.zeros((n, 12, 12)), np.zeros((n, 12, 12)), np.zeros(n, np.int32),
               np.zeros(n, np.int32))
    e2e_t = []
    for k in range(max(3, args.steps // 2) + 1):
        flush.zero_()
        torch.cuda.synchronize()
        t = time.perf_counter()
        batch.evaluate(EA, phiA, EB, phiB, params_rows, want_deriv=True, out=e2e_out)
        if k:
            e2e_t.append(time.perf_counter() - t)
    e2e_value, e2e_s = whole_job_rate(pts_per_step, float(np.mean(e2e_t)), world)
    h2d = n * 50 * 8
    d2h = n * (300 * 8 + 2 * 4)

    # the simulation, rollout and multi-part legs shard their scenes over the replicas too; the
    # single-GPU studies (FP16 bricks, SDF construction, planner queries) run on rank 0
    sim_res = run_sim(args, sdfc, ctx, g, p, n, world, rank) if args.sim_steps > 0 else None
    c5_res = run_c5(args, sdfc, ctx, torch) if args.c5_points > 0 and rank == 0 else None
    c4_res = run_c4(args, sdfc, ctx, g, torch, world, rank) if args.c4_instances > 0 else None
    ls_res = run_levelset(args, sdfc, ctx, torch) if args.ls_segments > 0 and rank == 0 else None
    pl_res = run_planner(args, sdfc, ctx, torch) if args.planner_states > 0 and rank == 0 else None
    c3_res = run_c3(args, sdfc, ctx, torch, world, rank) if args.c3_assemblies > 0 else None
    if sim_res is not None and rank == 0:
        plain = run_sim_plain(args, sdfc, ctx, g, p, n)
        # per GPU: the batched rate of one replica against the per-instance path on one GPU
        plain["speedup_of_batched"] = sim_res["first_steps"]["scene_steps_per_s"] / world / plain["scene_steps_per_s"]
        sim_res["plain_fp64_per_instance"] = plain

    if rank != 0:
        return
    peaks = load_peaks()
    hbm_peak = peaks["hbm_gbs"] if peaks else 6800.0
    # algorithmic bytes: detection reads 12 B per point and 8 FP32 corners (32 B) per query
    det_bytes = pts_per_step * (12 + 8 * 4)
    # forces: per active contact its id (4 B), point (12 B) and 8 FP32 corners; per (instance, share) 300 FP64
    # partials, the shares of each instance as the tuning cuts its active contacts
    chunk = 32 if tuning_used["force_variant"] == "workers" else 128
    shares = np.minimum(tuning_used["slots"],
                        -(-(-(-nact_rows // chunk)) // tuning_used["chunks_per_slot"]))
    rows = int(shares.sum())
    frc_bytes = n_active * (4 + 12 + 32) + rows * 300 * 8
    kernels = {
        "detect": {"ms": det_ms, "bytes": det_bytes},
        "force_kernel": {"ms": frc_ms, "bytes": frc_bytes},
        "finalize_kernel": {"ms": red_ms, "bytes": rows * 300 * 8 + n * 300 * 8},
    }
    dom = max(kernels, key=lambda k: kernels[k]["ms"])
    ach = kernels[dom]["bytes"] / (kernels[dom]["ms"] / 1e3) / 1e9
    traffic = profile_traffic(dom)
    # the force kernel's own limit (issue slots, with the FP64 pipe beside it): its warp
    # instructions per contact from the committed ncu capture x this run's active contacts over the
    # live force time, against 4 warp instructions per SM per clock
    issue = profile_figures("ncu_force_kernel_issue.txt")
    force_issue = None
    if issue.get("warp_inst_per_contact") and frc_ms > 0:
        sm_mhz = (clk or {}).get("sm_mhz") or 2070.0
        sms = torch.cuda.get_device_properties(dev).multi_processor_count
        ach_i = issue["warp_inst_per_contact"] * n_active / (frc_ms / 1e3)
        peak_i = 4.0 * sms * sm_mhz * 1e6
        force_issue = {"kernel": "force_kernel", "bound": "issue", "achieved": ach_i, "peak": peak_i,
                       "unit": "warp-inst/s", "frac": ach_i / peak_i,
                       "warp_inst_per_contact": issue["warp_inst_per_contact"],
                       "ncu_issue_active": issue.get("issue_active"),
                       "ncu_fp64_pipe_active": issue.get("fp64_pipe_active"),
                       "ncu_warps_active": issue.get("warps_active"),
                       "note": "instructions per contact and pipe fractions from the 512-instance ncu capture "
                               "(profiles/force_kernel_direction_sweep_512x50k.md); the rate from this run"}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        "dtype": ("f32 per-contact algebra and 32-contact warp sums; f64 depth; warp totals TwoSum-compensated "
                  "f32 within a force CTA, f64 across CTAs") if args.precision == "mixed" else "f64",
        "data": "synthetic",
        "config": workload_config(args),
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": e2e_s * 1e3},
        "roofline": {"kernel": dom, "bound": "hbm", "achieved": ach, "peak": hbm_peak, "unit": "GB/s",
                     "frac": ach / hbm_peak, "traffic": traffic,
                     "peak_source": "measured" if peaks else "fallback"},
        # the whole evaluation against the same peak, with the per-point algorithmic bytes of a
        # contact-point evaluation (12 B point + 8 FP32 corners), plus the active contacts' force
        # reads and the partial rows
        "roofline_force_issue": force_issue,
        "roofline_evaluation": {"bound": "hbm", "bytes_per_step": det_bytes + frc_bytes,
                                "achieved": (det_bytes + frc_bytes) / (step_ms / 1e3) / 1e9, "peak": hbm_peak,
                                "unit": "GB/s", "frac": (det_bytes + frc_bytes) / (step_ms / 1e3) / 1e9 / hbm_peak,
                                "note": "points and grid are shared by all instances, so these bytes are L2 reads; "
                                        "DRAM traffic per step is ~35 MB (profiles/)"},
        "phases_ms": {"detect": det_ms, "force": frc_ms, "reduce": red_ms},
        "plain_fp64_per_instance": {"value": plain_rate, "unit": UNIT, "instances_timed": m,
                                    "how": "one-instance FP64 batch per instance, device arrays, launches back to "
                                           "back on one stream, CUDA events",
                                    "speedup_of_batched": value / plain_rate},
        "batched_fp64": {"value": n * args.points / (f64_ms / 1e3), "unit": UNIT, "ms_per_step": f64_ms,
                         "how": "the same batch and launch configuration with FP64 per-contact algebra",
                         "speedup_of_mixed": f64_ms / step_ms},
        "error_vs_fp64_path": err,
        "tuning": {"chosen": tuning_used, "autotuned": tuning is not None,
                   "partial_rows": rows,
                   "candidates": "force pass on persistent 128-thread CTAs or one-warp workers over (instance, share) "
                                 "items x 1-32 chunks per share (at most 128 shares per instance, fewer above 2048 "
                                 "instances), or a grid of one CTA "
                                 "per item x 1-16 shares per instance; each timed on one evaluation"},
        "active_contacts_per_step": n_active, "fp64_rechecked_points_per_step": rechecked,
        # prep, detect, recheck, (plan, for the queue forms), force, finalize
        "gpu_launches": (5 if tuning_used["force_variant"] == "grid" else 6) * args.steps,
        "clocks": clk,
        "wall_s": wall,
    }
    if pool is not None:
        procs = os.cpu_count() or 1
        sample = max(procs, args.cpu_sample)
        rng = np.random.default_rng(0)
        cpu_time(pool, states, rng.choice(n, procs, replace=False))
        # the best of three timings of one sample: the host's cores are shared with other jobs
        idx = rng.choice(n, sample, replace=False)
        ct = min(cpu_time(pool, states, idx) for _ in range(3))
        line["cpu_baseline"] = {"value": sample * args.points / ct, "unit": UNIT, "cores": procs, "kind": "port",
                                "sample": f"{sample} of {n} instances, derivative evaluation, one process per core, "
                                          "best of 3 timings"}
        # the error of fm relative to the sum of the contacts' own force norms (where radial forces
        # cancel, |fm| understates the scale of the sum)
        m_err = err["instances"]
        sums = np.array(pool.map(_cpu_norm_sum, [(EA[k], phiA[k], EB[k], phiB[k]) for k in range(m_err)]))
        dev_fm = np.linalg.norm(out_fast[0][:m_err] - ref[0][:m_err], axis=1)
        line["error_vs_fp64_path"]["fm_over_sum_of_contact_norms"] = float(np.max(dev_fm / sums))
        if sim_res is not None:
            line["cpu_baseline"]["sim"] = cpu_sim_rate(pool, args.cpu_sim_scenes, min(args.sim_early, 25), procs)
        pool.close()
    if sim_res is not None:
        line["sim"] = sim_res
    if c5_res is not None:
        line["fp16_bricks"] = c5_res
    if c4_res is not None:
        line["differentiable_rollout"] = c4_res
    if ls_res is not None:
        line["sdf_construction"] = ls_res
    if pl_res is not None:
        line["planner_queries"] = pl_res
    if c3_res is not None:
        line["uneven_assemblies"] = c3_res
    print(json.dumps(line), flush=True)


def run_sim(args, sdfc, ctx, g, p, n, world=1, rank=0):
    """The direction sweep stepped: n scenes (peg on a translational joint, fixed socket), each pulled along
    its Fibonacci direction, args.sim_steps BDF1 steps through sdfc_sim_step (host state in and out).
    With world replicas the sweep has n * world directions and replica rank steps its block; rates are
    over all replicas' scenes and the slowest replica's time, and the final states are gathered."""
    dirs = rank_block(W.fibonacci_directions(n * world), n, rank, world)
    m, inertia = W.cylinder_mass_props()
    mover = sdfc.Mover.make(m, inertia, np.eye(4), SIM_H, SIM_GRAVITY)
    prm = sdfc.Params(*PARAMS)
    pairs = [sdfc.ScenePair.make(i, p, g, True, np.eye(4), prm) for i in range(n)]
    sim = ctx.sim([mover] * n, pairs)
    sim.set_precision(sdfc.PRECISION_MIXED if args.precision == "mixed" else sdfc.PRECISION_FP64)
    F = np.zeros((n, 6))
    F[:, 3:] = SIM_PULL * dirs
    sim.set_state(np.zeros((n, 3)), np.zeros((n, 3)))
    sim.set_external_force(F)
    sim.step(1)  # warm-up step
    sim.set_state(np.zeros((n, 3)), np.zeros((n, 3)))
    sim.record(args.sim_steps)  # the trajectory for the adjoint (one device copy per step)
    r0, e0 = sim.stats()
    dist_barrier(world)
    t0 = time.perf_counter()
    early = min(args.sim_steps, args.sim_early)
    conv = sim.step(early)
    t_early = time.perf_counter() - t0
    r1, e1 = sim.stats()
    if args.sim_steps > early:
        conv = sim.step(args.sim_steps - early)
    q, qd = sim.get_state()
    wall = time.perf_counter() - t0
    r2, e2 = sim.stats()
    # adjoint of the whole rollout for L_i = d_i . q_T (displacement along the pull):
    # dL/dq0, dL/dqdot0 and dL/d(pull force) of every scene
    w = np.zeros((n, args.sim_steps, 3))
    w[:, -1] = dirs
    dist_barrier(world)
    t1 = time.perf_counter()
    g0, gd0, gf = sim.backward(w)
    t_bwd = time.perf_counter() - t1
    sim.close()
    rate, wall_job = whole_job_rate(n * args.sim_steps, wall, world)
    early_rate, _ = whole_job_rate(n * early, t_early, world)
    bwd_rate, t_bwd_job = whole_job_rate(n * args.sim_steps, t_bwd, world)
    evals = int(dist_sum(e2 - e0, world))
    q_all = gather_rows(q, world)  # every replica's final states, on every rank
    conv_all = gather_rows(conv, world)
    finite = bool(gather_rows([np.isfinite(gf).all() and np.isfinite(g0).all()], world).all())
    return {"scenes": n * world, "steps": args.sim_steps, "wall_s": wall_job,
            "scene_steps_per_s": rate,
            "contact_pts_per_s": evals * args.points / wall_job,
            "rounds": r2 - r0, "scene_evaluations": evals,
            "first_steps": {"steps": early, "wall_s": t_early, "scene_steps_per_s": early_rate,
                            "scene_evaluations": int(dist_sum(e1 - e0, world))},
            "converged_last_step": float(np.mean(conv_all)),
            "final_z_mean": float(q_all[:, 2].mean()),
            "adjoint": {"steps": args.sim_steps, "wall_s": t_bwd_job, "scene_steps_per_s": bwd_rate,
                        "finite": finite}}


def run_sim_plain(args, sdfc, ctx, g, p, n_dirs, instances=4):
    """The plain per-instance FP64 GPU path of the same scenes: one scene per sdfc_sim, FP64
    force evaluations, over the same first steps as the batched run's first_steps figure."""
    dirs = W.fibonacci_directions(n_dirs)
    idx = np.linspace(0, n_dirs - 1, instances).astype(int)
    m, inertia = W.cylinder_mass_props()
    mover = sdfc.Mover.make(m, inertia, np.eye(4), SIM_H, SIM_GRAVITY)
    prm = sdfc.Params(*PARAMS)
    steps = min(args.sim_steps, args.sim_early)
    total = 0.0
    for k in idx:
        sim = ctx.sim([mover], [sdfc.ScenePair.make(0, p, g, True, np.eye(4), prm)])
        sim.set_precision(sdfc.PRECISION_FP64)
        F = np.zeros((1, 6))
        F[0, 3:] = SIM_PULL * dirs[k]
        sim.set_external_force(F)
        sim.set_state(np.zeros((1, 3)), np.zeros((1, 3)))
        sim.step(1)  # warm-up (graph capture)
        sim.set_state(np.zeros((1, 3)), np.zeros((1, 3)))
        t0 = time.perf_counter()
        sim.step(steps)
        total += time.perf_counter() - t0
        sim.close()
    return {"scene_steps_per_s": instances * steps / total, "instances": int(instances), "steps": steps,
            "precision": "fp64", "scenes_per_sim": 1}


def run_c5(args, sdfc, ctx, torch):
    """Precision scaling: a two-part tab-in-slot assembly whose slotted part is a 512^3 SDF stored
    as FP16 bricks (8^3 nodes, FP32 scale/offset per brick), the other part's 1M surface points
    against it, 256 pull directions.  Batched derivative evaluations (mixed precision) are timed;
    then 200 BDF1 steps of all directions.  Errors are reported against the same scenes on the
    FP64 grid with FP64 evaluations: forces on a sample of instances, poses after the steps on a
    sample of scenes, and the grid values themselves."""
    asm = W.procedural_assembly(5, n_parts=2, points=(args.c5_points, args.c5_points), grids=(args.c5_grid,))
    mover, still = 0, 1  # part 0's tab sits in part 1's slot
    t = time.perf_counter()
    grid = asm.parts[still].grid(args.c5_grid)
    gen_s = time.perf_counter() - t
    pts = asm.parts[mover].surface_points(args.c5_points, 55).astype(np.float32).astype(np.float64)
    t = time.perf_counter()
    g16 = ctx.upload_grid(grid.values, grid.min_box, grid.max_box, grid.dx, 0.0, sdfc.STORAGE_F16_BRICKS)
    up_s = time.perf_counter() - t
    g64 = ctx.upload_grid(grid.values, grid.min_box, grid.max_box, grid.dx, 0.0, sdfc.STORAGE_F64)
    dec = ctx.grid_values(g16)
    near = np.abs(grid.values) < 0.05
    dist_err = {"max_abs": float(np.abs(dec - grid.values).max()),
                "max_abs_within_0.05_of_surface": float(np.abs(dec - grid.values)[near].max()),
                "max_rel": float((np.abs(dec - grid.values) / np.maximum(np.abs(grid.values), 1e-12)).max())}
    ph = ctx.upload_points(pts, sdfc.STORAGE_F32)
    n = args.c5_dirs
    dirs = W.fibonacci_directions(n)
    E_still = W.pose(None, asm.parts[still].position)
    EA = np.stack([W.pose(None, asm.parts[mover].position + 0.0105 * d) for d in dirs])
    EB = np.broadcast_to(E_still, (n, 4, 4)).copy()
    phiA = np.zeros((n, 6))
    phiA[:, 3:] = 0.01 * dirs
    phiB = np.zeros((n, 6))
    prm = [sdfc.Params(*PARAMS)] * n
    b16 = ctx.batch([ph] * n, [g16] * n)
    b16.set_precision(sdfc.PRECISION_MIXED)
    cuda = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()  # noqa: E731
    dEA, dphiA, dEB, dphiB = cuda(EA), cuda(phiA), cuda(EB), cuda(phiB)
    dprm = cuda(np.tile(np.array(PARAMS), (n, 1)))
    fm = torch.zeros(n, 12, dtype=torch.float64, device="cuda")
    Km = torch.zeros(n, 144, dtype=torch.float64, device="cuda")
    Dm = torch.zeros(n, 144, dtype=torch.float64, device="cuda")
    nact = torch.zeros(n, dtype=torch.int32, device="cuda")
    st = torch.zeros(n, dtype=torch.int32, device="cuda")
    flush = torch.empty(2 * L2_BYTES, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.Stream()
    torch.cuda.synchronize()

    def step():
        b16.evaluate_device(dEA.data_ptr(), dphiA.data_ptr(), dEB.data_ptr(), dphiB.data_ptr(), dprm.data_ptr(),
                            fm.data_ptr(), Km.data_ptr(), Dm.data_ptr(), nact.data_ptr(), st.data_ptr(),
                            want_deriv=True, stream=stream.cuda_stream)

    if not args.no_autotune:  # the batch's launch configuration, timed once on these inputs
        b16.autotune(dEA.data_ptr(), dphiA.data_ptr(), dEB.data_ptr(), dphiB.data_ptr(), dprm.data_ptr(),
                     fm.data_ptr(), Km.data_ptr(), Dm.data_ptr(), nact.data_ptr(), st.data_ptr(), want_deriv=True,
                     stream=stream.cuda_stream)
    c5_tuning = b16.tuning()

    with torch.cuda.stream(stream):
        for _ in range(3):
            step()
        stream.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(10)]
        for a, b in ev:
            flush.zero_()
            a.record(stream)
            step()
            b.record(stream)
        torch.cuda.synchronize()
    ms = float(np.mean([a.elapsed_time(b) for a, b in ev]))
    # per-phase device times (separate pass with events between the launches)
    b16.set_timing(True)
    phases = []
    with torch.cuda.stream(stream):
        for _ in range(5):
            flush.zero_()
            stream.synchronize()
            step()
            phases.append(b16.last_timing())
    b16.set_timing(False)
    c5_phases = {k: float(np.mean([x[i] for x in phases])) for i, k in enumerate(("detect", "force", "reduce"))}
    act = nact.cpu().numpy()
    n_active = int(act.sum())
    m = min(n, args.c5_check)
    idx = np.sort(np.argsort(-act, kind="stable")[:m])  # the instances with the most contacts
    f16 = (fm.cpu().numpy()[idx], Km.cpu().numpy()[idx].reshape(m, 12, 12), Dm.cpu().numpy()[idx].reshape(m, 12, 12))
    b64 = ctx.batch([ph] * m, [g64] * m)
    b64.set_precision(sdfc.PRECISION_FP64)
    r = b64.evaluate(EA[idx], phiA[idx], EB[idx], phiB[idx], prm[:m], want_deriv=True)
    force_err = {"fm": rel_err(f16[0], r[0]), "Km": rel_err(f16[1], r[1]), "Dm": rel_err(f16[2], r[2]),
                 "fm_norm_rel": float(np.max(np.linalg.norm(f16[0] - r[0], axis=1) /
                                             np.maximum(np.linalg.norm(r[0], axis=1), 1e-12))),
                 "instances": m, "active_contacts_checked": int(act[idx].sum())}
    b16.close()
    b64.close()
    out = {"grid": f"{args.c5_grid}^3 fp16 bricks", "grid_bytes": int(((args.c5_grid + 7) // 8) ** 3 * (512 * 2 + 8)),
           "fp64_grid_bytes": int(args.c5_grid ** 3 * 8), "points": args.c5_points, "instances": n,
           "ms_per_eval": ms, "phases_ms": c5_phases, "tuning": c5_tuning,
           "contact_pts_per_s": n * args.c5_points / (ms / 1e3),
           "active_contacts_per_eval": n_active, "grid_sample_s": gen_s, "grid_encode_upload_s": up_s,
           "distance_error_vs_fp64_grid": dist_err, "force_error_vs_fp64_grid": force_err}
    if args.c5_steps > 0:
        m_, inertia = asm.parts[mover].mass_props()
        E_pj0 = W.pose(None, asm.parts[mover].position)
        mv = sdfc.Mover.make(m_, inertia, np.eye(4), SIM_H, SIM_GRAVITY, E_pj0=E_pj0)
        F = np.zeros((n, 6))
        F[:, 3:] = SIM_PULL * dirs

        def sim_run(grid_h, which, precision):
            scenes = len(which)
            sim = ctx.sim([mv] * scenes, [sdfc.ScenePair.make(i, ph, grid_h, True, E_still, sdfc.Params(*PARAMS))
                                          for i in range(scenes)])
            sim.set_precision(precision)
            sim.set_state(np.zeros((scenes, 3)), np.zeros((scenes, 3)))
            sim.set_external_force(F[which])
            if not args.no_autotune and precision == sdfc.PRECISION_MIXED:
                sim.autotune()
            t0 = time.perf_counter()
            conv = sim.step(args.c5_steps)
            wall = time.perf_counter() - t0
            q, _ = sim.get_state()
            r_, e_ = sim.stats()
            sim.close()
            return q, wall, conv, r_, e_

        q16, wall, conv, rounds, evals = sim_run(g16, np.arange(n), sdfc.PRECISION_MIXED)
        q64, _, _, _, _ = sim_run(g64, idx, sdfc.PRECISION_FP64)
        # the planner's decision per direction (PhysicsPlanner.is_disassembled,
        # examples/run_joint_plan.py:291-302) after the steps, on the FP16-brick grid and on the
        # FP64 grid (both with the same mixed-precision evaluations): does the storage change it?
        q64m, _, _, _, _ = sim_run(g64, np.arange(n), sdfc.PRECISION_MIXED)
        M = importlib.import_module(f"{PKG}.mesh")
        still_pts = asm.parts[still].surface_points(20000, 56) + asm.parts[still].position
        check = M.DisassemblyCheck(ctx, pts[::max(1, len(pts) // 20000)], still_pts)
        at = lambda q: np.stack([W.pose(None, asm.parts[mover].position + x) for x in q])  # noqa: E731
        d16, d64 = check(at(q16)), check(at(q64m))
        out["sim"] = {"scenes": n, "steps": args.c5_steps, "wall_s": wall, "scene_steps_per_s": n * args.c5_steps / wall,
                      "rounds": rounds, "scene_evaluations": evals, "converged_last_step": float(np.mean(conv)),
                      "pose_error_vs_fp64_grid": {"max_abs": float(np.abs(q16[idx] - q64).max()),
                                                   "max_displacement": float(np.abs(q64).max()), "scenes": m},
                      "planner_decision_vs_fp64_grid": {
                          "directions": n, "disassembled_fp16_bricks": int(d16.sum()),
                          "disassembled_fp64_grid": int(d64.sum()), "same_decision": int((d16 == d64).sum()),
                          "rule": "is_disassembled after the steps (convex hulls of 20k surface points each), "
                                  "mixed-precision evaluations on both grids"}}
    return out


def run_levelset(args, sdfc, ctx, torch):
    """Mesh -> SDF grid (sdfgen::make_level_set3, the work of BodySDFObj::precompute_SDF): a seeded
    bumpy torus of args.ls_segments x args.ls_segments/2 quads (2 triangles each) on a grid of
    spacing args.ls_dx with 2 cells of margin, exact band 1.  Device arrays in and out (value) and
    host arrays through sdfc_make_level_set3 (e2e); the oracle's sequential restatement of the
    reference times a smaller grid of the same mesh on one host core.  The GPU result on that
    grid is compared bit for bit with the oracle's."""
    from oracle import oracle
    n, m = args.ls_segments, args.ls_segments // 2
    V, F = W.torus_mesh(0.6, 0.25, n, m)
    V = V * (1 + 0.03 * np.random.default_rng(n).standard_normal((len(V), 1)))
    origin, shape = W.level_set_grid(V, args.ls_dx)
    nodes = int(np.prod(shape))
    Vd = torch.tensor(np.asarray(V, np.float32), device="cuda")
    Fd = torch.tensor(np.asarray(F, np.int32), device="cuda")
    st = torch.cuda.Stream()
    torch.cuda.synchronize()
    ctx.make_level_set3_device(Vd, Fd, origin, args.ls_dx, shape, stream=st)  # warm-up
    times = []
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        ctx.make_level_set3_device(Vd, Fd, origin, args.ls_dx, shape, stream=st)
        e1.record(st)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    ms = float(np.median(times))
    t = time.perf_counter()
    ctx.make_level_set3(V, F, origin, args.ls_dx, shape)
    e2e_ms = (time.perf_counter() - t) * 1e3
    A, B, C = shape[0] - 2, shape[1] - 2, shape[2] - 2
    out = {"mesh": f"bumpy torus, {len(F)} triangles", "grid": list(shape), "nodes": nodes, "exact_band": 1,
           "ms": ms, "nodes_per_s": nodes / (ms / 1e3),
           "e2e": {"ms": e2e_ms, "nodes_per_s": nodes / (e2e_ms / 1e3),
                   "h2d_bytes": int(V.size * 4 + F.size * 4), "d2h_bytes": nodes * 4},
           "sweep_diagonals": 16 * (A + B + C + 1), "us_per_sweep_diagonal": ms * 1e3 / (16 * (A + B + C + 1))}
    if args.ls_cpu_dx > 0:
        o2, s2 = W.level_set_grid(V, args.ls_cpu_dx)
        t = time.perf_counter()
        want = oracle.make_level_set3(V, F, o2, args.ls_cpu_dx, s2)
        ct = time.perf_counter() - t
        got = ctx.make_level_set3(V, F, o2, args.ls_cpu_dx, s2)
        out["bit_exact_vs_oracle"] = bool(np.array_equal(got.view(np.uint32), want.view(np.uint32)))
        out["cpu_baseline"] = {"value": int(np.prod(s2)) / ct, "unit": "nodes/s", "cores": 1, "kind": "port",
                               "sample": f"same mesh on a {s2[0]}x{s2[1]}x{s2[2]} grid (spacing {args.ls_cpu_dx})"}
        out["speedup_vs_cpu"] = out["nodes_per_s"] / out["cpu_baseline"]["value"]
    return out


def run_planner(args, sdfc, ctx, torch):
    """Planner-side queries, batched: get_body_distance of a moving part's mesh vertices against a
    still part's grid (the planner's collision_th set-up and body_in_contact) and the disassembly
    check, for args.planner_states poses of a procedural assembly's mover.  Device arrays in and
    out, CUDA events; the oracle's restatements timed on one core on a sample of poses."""
    from oracle import disassembly as D
    from oracle import oracle
    mesh = importlib.import_module(f"{PKG}.mesh")
    n = args.planner_states
    asm = W.procedural_assembly(11, n_parts=6, points=(args.planner_vertices, args.planner_vertices), grids=(128,))
    mover, still = asm.parts[0], asm.parts[1]
    verts = mover.surface_points(args.planner_vertices, 21)
    grid = still.grid(128)
    gB = ctx.upload_grid(grid.values, grid.min_box, grid.max_box, grid.dx, 0.01, sdfc.STORAGE_F32)
    rng = np.random.default_rng(12)
    E = np.zeros((n, 4, 4))
    for k in range(n):
        # the mover around its assembled place (the parts' frames are translations)
        E[k] = W.pose(W.rotvec_to_matrix(rng.normal(size=3) * 0.05), mover.position + rng.normal(size=3) * 0.3)
    EB = np.tile(W.pose(np.eye(3), still.position), (n, 1, 1))
    bd = mesh.BodyDistance(ctx, verts, gB, n)
    dE = torch.tensor(E.reshape(n, 16), device="cuda")
    dEB = torch.tensor(EB.reshape(n, 16), device="cuda")
    dmin = torch.empty(n, dtype=torch.float64, device="cuda")
    st = torch.cuda.Stream()
    torch.cuda.synchronize()
    L = sdfc.lib()

    def dist_call():
        rc = L.sdfc_batch_distance_device(bd.batch._h, dE.data_ptr(), dEB.data_ptr(), dmin.data_ptr(), None,
                                          st.cuda_stream)
        assert rc == 0

    still_verts = np.concatenate([p.surface_points(args.planner_vertices // 2, 30 + k) + p.position
                                  for k, p in enumerate(asm.parts[1:])])
    chk = mesh.DisassemblyCheck(ctx, verts, still_verts)
    dout = torch.empty(n, dtype=torch.int32, device="cuda")
    Ew = E
    dEw = dE

    def dis_call():
        rc = L.sdfc_disassembled_device(ctx._h, chk.hull_move, chk.hull_still, dEw.data_ptr(), n, dout.data_ptr(),
                                        None, st.cuda_stream)
        assert rc == 0

    def timed(fn, reps=5):
        fn()
        ts = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            fn()
            e1.record(st)
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        return float(np.median(ts))

    dist_ms, dis_ms = timed(dist_call), timed(dis_call)
    # the oracle on a sample of poses, one core
    og = oracle.Grid(grid.values.astype(np.float32).astype(np.float64), grid.min_box, grid.max_box, grid.dx, 0.01)
    m = min(n, args.planner_cpu_sample)
    t = time.perf_counter()
    ref_min = np.array([oracle.body_distance(og, E[k], EB[k], verts) for k in range(m)])
    cpu_dist = m / (time.perf_counter() - t)
    got_min = dmin.cpu().numpy()
    oc = D.Checker(verts, still_verts)
    md = min(n, max(8, args.planner_cpu_sample // 8))
    t = time.perf_counter()
    want = np.array([oc(Ew[k]) for k in range(md)])
    cpu_dis = md / (time.perf_counter() - t)
    got = dout.cpu().numpy().astype(bool)
    return {"states": n, "mover_vertices": len(verts), "grid": "128^3 fp32",
            "hull_vertices": {"move": int(len(oc.VA0)), "still": int(len(oc.VB))},
            "body_distance": {"ms": dist_ms, "states_per_s": n / (dist_ms / 1e3),
                              "vertex_queries_per_s": n * len(verts) / (dist_ms / 1e3),
                              "bit_exact_vs_oracle_sample": bool(np.array_equal(got_min[:m], ref_min)),
                              "cpu_baseline": {"value": cpu_dist, "unit": "states/s", "cores": 1, "kind": "port",
                                               "sample": f"{m} poses"}},
            "disassembly_check": {"ms": dis_ms, "states_per_s": n / (dis_ms / 1e3), "disassembled": int(got.sum()),
                                  "agree_with_oracle_sample": int((got[:md] == want).sum()), "sample": md,
                                  "cpu_baseline": {"value": cpu_dis, "unit": "states/s", "cores": 1, "kind": "port",
                                                   "sample": f"{md} poses, LP feasibility (HiGHS)"}}}


def run_c4(args, sdfc, ctx, g, torch, world=1, rank=0):
    """Differentiable rollout: args.c4_instances pegs on free3d-exp joints in the socket, initial
    pose perturbed (sigma 0.01 translation, sigma 1 degree rotation), pulled along directions in a
    30 degree cone about +z, args.c4_steps BDF1 steps.  Loss per instance: the steps' summed
    penetration energy plus |q_T - target|^2 (target: the peg extracted 0.25 along +z).  The
    gradients wrt the initial pose and the pull direction come from the adjoint
    (sdfc_sim_backward_energy); the joint trajectory, recorded every step, is the checkpoint from
    which each step's matrices are recomputed."""
    n, T = args.c4_instances, args.c4_steps
    rng = np.random.default_rng(4)
    pts = W.peg_points(args.c4_points, seed=9)
    ph = ctx.upload_points(pts, sdfc.STORAGE_F32)
    # with world replicas: n * world instances, replica rank takes its block
    dirs = rank_block(W.cone_directions(n * world, 30.0, seed=4), n, rank, world)
    m, inertia = W.cylinder_mass_props()
    mv = sdfc.Mover.make(m, inertia, np.eye(4), SIM_H, SIM_GRAVITY, joint=sdfc.JOINT_FREE3D_EXP)
    sim = ctx.sim([mv] * n, [sdfc.ScenePair.make(i, ph, g, True, np.eye(4), sdfc.Params(*PARAMS)) for i in range(n)])
    sim.set_precision(sdfc.PRECISION_MIXED if args.c4_precision == "mixed" else sdfc.PRECISION_FP64)
    q0_all = np.zeros((n * world, 6))
    q0_all[:, :3] = rng.normal(size=(n * world, 3)) * 0.01
    q0_all[:, 3:] = rng.normal(size=(n * world, 3)) * np.deg2rad(1.0)
    q0 = rank_block(q0_all, n, rank, world)
    F = np.zeros((n, 6))
    F[:, 3:] = SIM_PULL * dirs
    target = np.array([0.0, 0.0, 0.25, 0.0, 0.0, 0.0])
    # warm-up (graph capture of the rounds and the reverse step)
    sim.record_energy(True)
    sim.set_state(q0, np.zeros((n, 6)))
    sim.set_external_force(F)
    sim.record(2)
    sim.step(2)
    sim.backward(np.zeros((n, 2, 6)), np.ones(n))
    sim.record(T)
    sim.set_state(q0, np.zeros((n, 6)))
    torch.cuda.synchronize()
    r0, e0 = sim.stats()
    dist_barrier(world)
    t0 = time.perf_counter()
    conv = sim.step(T)
    qh = sim.history()
    _, E = sim.energy()
    t_fwd = time.perf_counter() - t0
    r1, e1 = sim.stats()
    L = E + ((qh[:, T] - target) ** 2).sum(1)
    df_dq = np.zeros((n, T, 6))
    df_dq[:, T - 1] = 2.0 * (qh[:, T] - target)
    dist_barrier(world)
    t1 = time.perf_counter()
    g0, gd0, gf = sim.backward(df_dq, np.ones(n))
    t_bwd = time.perf_counter() - t1
    r, e = sim.stats()
    sim.close()
    check = None
    if args.c4_check > 0 and rank == 0:
        check = c4_gradient_check(sdfc, ctx, g, ph, mv, q0, dirs, T, target, g0, gf, args.c4_check)
    fwd_rate, t_fwd_job = whole_job_rate(n * T, t_fwd, world)
    bwd_rate, t_bwd_job = whole_job_rate(n * T, t_bwd, world)
    # every replica's per-instance results, gathered
    L, E, conv = gather_rows(L, world), gather_rows(E, world), gather_rows(conv, world)
    g0, gf = gather_rows(g0, world), gather_rows(gf, world)
    g_dir = SIM_PULL * gf[:, 3:]  # F = pull * direction
    out = {"instances": n * world, "steps": T, "points": args.c4_points, "joint": "free3d-exp",
            "precision": args.c4_precision, "rounds": r1 - r0, "scene_evaluations": int(dist_sum(e1 - e0, world)),
            "converged_last_step": float(np.mean(conv)),
            "forward_wall_s": t_fwd_job, "backward_wall_s": t_bwd_job,
            "forward_scene_steps_per_s": fwd_rate, "backward_scene_steps_per_s": bwd_rate,
            "loss_mean": float(L.mean()), "penetration_energy_mean": float(E.mean()),
            "grad_q0_norm_mean": float(np.linalg.norm(g0, axis=1).mean()),
            "grad_direction_norm_mean": float(np.linalg.norm(g_dir, axis=1).mean()),
            "finite": bool(np.isfinite(g0).all() and np.isfinite(gf).all()),
            "checkpoint": "joint trajectory every step (48 B per scene-step); step matrices recomputed in reverse"}
    if check is not None:
        out["gradient_check"] = check
    return out


def c4_gradient_check(sdfc, ctx, g, ph, mv, q0, dirs, T, target, g0_mixed, gf_mixed, k):
    """Adjoint gradients of k instances spread over the rollout against central differences of
    rollouts with FP64 evaluations and Newton solved to |g| < 1e-13, at the workload's step 1e-6
    and at 1e-8 and 3e-9: dL/dq0 (6) and dL/d(direction) on the tangent plane of the unit sphere
    at the direction (2).  The loss is piecewise smooth (contact points entering the active set
    are kinks), so differences at 1e-6 straddle kinks; at 1e-8 they resolve the derivative except
    for components whose +- rollouts still straddle a kink, which the 3e-9 differences reveal
    (they disagree with the 1e-8 ones), or that have a kink at the base point itself, whose
    one-sided slopes keep their gap at both 1e-8 and 3e-9: those are reported apart, as the GPU
    test of this check does.  An instance with a step that did not converge (its loss is not
    differentiable there), or whose rotation vector was reparameterised between steps (a map the
    adjoint does not differentiate, as the reference's does not), is marked and left out of the
    summary.  The FP64 adjoint comes from the tightly solved base scene; the mixed one is the
    timed rollout's (FP32 per-contact algebra, the reference's Newton tolerance 1e-8)."""
    n = len(q0)
    idx = np.linspace(0, n - 1, k).astype(int)
    steps = (1e-6, 1e-8, 3e-9)
    q0s, Fs, bases = [], [], []
    for i in idx:
        a = np.array([1.0, 0.0, 0.0]) if abs(dirs[i][0]) < 0.9 else np.array([0.0, 1.0, 0.0])
        t1 = np.cross(dirs[i], a)
        t1 /= np.linalg.norm(t1)
        t2 = np.cross(dirs[i], t1)
        bases.append((t1, t2))
        var = [(q0[i], dirs[i])]
        for h in steps:
            for j in range(6):
                for sgn in (1.0, -1.0):
                    q = q0[i].copy()
                    q[j] += sgn * h
                    var.append((q, dirs[i]))
            for t in (t1, t2):
                for sgn in (1.0, -1.0):
                    var.append((q0[i], dirs[i] + sgn * h * t))
        for q, d in var:
            q0s.append(q)
            Fs.append(np.concatenate([np.zeros(3), SIM_PULL * d]))
    m = len(q0s)
    sim = ctx.sim([mv] * m, [sdfc.ScenePair.make(j, ph, g, True, np.eye(4), sdfc.Params(*PARAMS)) for j in range(m)])
    sim.set_precision(sdfc.PRECISION_FP64)
    sim.set_tolerance(1e-13)
    sim.record_energy(True)
    sim.set_state(np.array(q0s), np.zeros((m, 6)))
    sim.set_external_force(np.array(Fs))
    sim.record(T)
    t0 = time.perf_counter()
    conv = np.ones(m, bool)
    for _ in range(T):
        conv &= sim.step(1)
    qh = sim.history()
    _, E = sim.energy()
    L = E + ((qh[:, T] - target) ** 2).sum(1)
    df_dq = np.zeros((m, T, 6))
    df_dq[:, T - 1] = 2.0 * (qh[:, T] - target)
    g0, _, gf = sim.backward(df_dq, np.ones(m))
    wall = time.perf_counter() - t0
    sim.close()
    # scenes whose rotation vector was reparameterised (a jump of about 2 pi between steps): the
    # adjoint, like the reference's, does not differentiate that map
    reparam = (np.linalg.norm(np.diff(qh[:, :, 3:6], axis=1), axis=2) > np.pi).any(axis=1)
    per = 1 + 16 * len(steps)
    rows = []
    for s_, i in enumerate(idx):
        o = per * s_
        t1, t2 = bases[s_]
        gd = SIM_PULL * gf[o, 3:]
        a64 = np.concatenate([g0[o], [gd @ t1, gd @ t2]])
        gm = SIM_PULL * gf_mixed[i, 3:]
        amx = np.concatenate([g0_mixed[i], [gm @ t1, gm @ t2]])
        row = {"instance": int(i), "mixed_vs_fp64_adjoint": float(np.linalg.norm(amx - a64) / np.linalg.norm(a64)),
               "rotation_reparameterised": bool(reparam[o])}
        fds = {}
        for mm, h in enumerate(steps):
            r = L[o + 1 + 16 * mm:o + 1 + 16 * (mm + 1)]
            fd = (r[0::2] - r[1::2]) / (2 * h)
            fds[h] = fd
            row[f"fp64_adjoint_vs_fd_{h:g}"] = float(np.linalg.norm(a64 - fd) / np.linalg.norm(fd))
            row[f"all_steps_converged_{h:g}"] = bool(conv[o] and conv[o + 1 + 16 * mm:o + 1 + 16 * (mm + 1)].all())
        # components whose 1e-8 and 3e-9 central differences agree and that show no kink at the
        # base point (where both central differences average the two one-sided slopes): the
        # adjoint against the 1e-8 difference there, relative to the gradient's norm
        scale = np.linalg.norm(fds[1e-8])
        gap = {}  # one-sided slope gaps: shrink with the step under curvature, stay at a kink
        for mm in (1, 2):
            r = L[o + 1 + 16 * mm:o + 1 + 16 * (mm + 1)]
            gap[mm] = np.abs((r[0::2] - L[o]) - (L[o] - r[1::2])) / steps[mm]
        kink_at_base = (gap[1] > 1e-5 * scale) & (gap[2] > 0.6 * gap[1])
        smooth = (np.abs(fds[1e-8] - fds[3e-9]) <= 1e-5 * scale) & ~kink_at_base
        row["smooth_components"] = int(smooth.sum())
        row["fp64_adjoint_vs_fd_1e-08_smooth"] = float(np.abs(a64 - fds[1e-8])[smooth].max() / scale) if smooth.any() else None
        rows.append(row)
    ok = [r for r in rows if r["all_steps_converged_1e-08"] and r["all_steps_converged_3e-09"]
          and not r["rotation_reparameterised"]]
    sm = [r["fp64_adjoint_vs_fd_1e-08_smooth"] for r in ok if r["fp64_adjoint_vs_fd_1e-08_smooth"] is not None]
    return {"fd_steps": list(steps), "newton_tol": 1e-13, "per_instance": rows, "scenes": m, "wall_s": wall,
            "components": "dL/dq0 (6) and dL/d(direction) along two tangent directions (2)",
            "converged_instances": len(ok),
            "smooth_components_of_converged": int(sum(r["smooth_components"] for r in ok)),
            "max_fp64_adjoint_vs_fd_smooth": max(sm) if sm else None}


# --------------------------------------------------------------------------- uneven multi-part batch
# The planner's scene parameters (examples/run_joint_plan.py:147-153, 192-216): h = 1e-3 (read as
# FP32), gravity 1e-12 along +z, kn = 1e6, kt = 1e3, mu = 0, damping = 0, pull 100, and
# col_th = max(-min distance, 0) + 0.01 = 0.01 for these assemblies (parts 0.005 apart).
C3_H = float(np.float32(1e-3))
C3_GRAVITY = (0.0, 0.0, 1e-12)
C3_PULL = 100.0
C3_PRM = (1e6, 1e3, 0.0, 0.0, 1.0, 1.0)
C3_COL_TH = 0.01


def _c3_cpu_scene(args):
    """Steps of one assembly scene by the oracle (spawned worker): (seconds, scene evaluations)."""
    from oracle import oracle as O
    mover, pairs, steps = args
    grids, opairs = {}, []
    for (gkey, gv, mn, mx, dx), pts, is_contact, E_fixed in pairs:
        if gkey not in grids:
            grids[gkey] = O.Grid(gv, mn, mx, dx, C3_COL_TH)
        opairs.append(O.ScenePair(grids[gkey], pts, is_contact, E_fixed, O.Params(*C3_PRM)))
    t = time.perf_counter()
    _, _, _, _, evs = O.bdf1_steps(O.Mover(*mover), opairs, np.zeros(3), np.zeros(3), steps)
    return time.perf_counter() - t, int(evs.sum())


def run_c3(args, sdfc, ctx, torch, world=1, rank=0):
    """Uneven multi-part batch: args.c3_assemblies seeded procedural assemblies (2-12 parts, per
    part log-uniform 2k-200k contact points and a grid of 64^3, 128^3 or 256^3 FP32 nodes), one
    part of each pulled along a random axis for args.c3_steps BDF1 steps, all scenes in one
    sdfc_sim (the pulled part against every other part both ways, as the planner declares it).
    Grids are sampled on the GPU and kept as FP32 node values (4 B per node)."""
    S = importlib.import_module(f"{PKG}.scenes")
    t0 = time.perf_counter()
    # with world replicas: assemblies (seeds) rank * n .. (rank + 1) * n - 1
    seeds = list(range(rank * args.c3_assemblies, (rank + 1) * args.c3_assemblies))
    asms = [W.procedural_assembly(s) for s in seeds]
    scenes = [S.AssemblyScene.make_device(ctx, a, s, col_th=C3_COL_TH) for s, a in zip(seeds, asms)]
    sim = S.build_sim(ctx, scenes, C3_H, C3_GRAVITY, sdfc.Params(*C3_PRM), col_th=C3_COL_TH,
                      storage=sdfc.STORAGE_F32_NODES)
    setup_s = time.perf_counter() - t0
    sim.set_precision(sdfc.PRECISION_MIXED if args.precision == "mixed" else sdfc.PRECISION_FP64)
    n = len(scenes)
    F = S.pull_forces(scenes, C3_PULL)
    zero = np.zeros((n, 3))
    sim.set_state(zero, zero)
    sim.set_external_force(F)
    tuning = sim.autotune() if not args.no_autotune else sim.tuning()
    sim.step(1)  # warm-up: the round graphs are captured here
    sim.set_state(zero, zero)
    e0 = sim.scene_evaluations()
    r0, _ = sim.stats()
    torch.cuda.synchronize()
    dist_barrier(world)
    t = time.perf_counter()
    conv = sim.step(args.c3_steps)
    wall_rank = time.perf_counter() - t
    r1, _ = sim.stats()
    evals = sim.scene_evaluations() - e0
    q, _ = sim.get_state()
    # contact points one evaluation of a scene evaluates: its pairs' contact-body points
    pts_scene = np.array([sum(len(sc.points[a]) for a, _ in sc.contact_pairs()) for sc in scenes], dtype=np.int64)
    _, wall = whole_job_rate(1, wall_rank, world)
    # every replica's per-scene results, gathered
    evals, pts_scene = gather_rows(evals, world), gather_rows(pts_scene, world)
    q, conv = gather_rows(q, world), gather_rows(conv, world)
    n = len(evals)
    cpe = int((evals * pts_scene).sum())
    disp = np.linalg.norm(q, axis=1)
    parts = gather_rows([len(a.parts) for a in asms], world).tolist()
    grid_n = gather_rows([g for a in asms for g in a.grid_n], world).tolist()
    npts = gather_rows([x for a in asms for x in a.n_points], world)
    out = {
        "assemblies": n, "parts": int(sum(parts)), "parts_per_assembly": [int(min(parts)), int(max(parts))],
        "pairs": int(sum(2 * (k - 1) for k in parts)), "contact_points_total": int(npts.sum()),
        "points_per_part": [int(npts.min()), int(npts.max())],
        "grids": {f"{g}^3": int(sum(1 for x in grid_n if x == g)) for g in (64, 128, 256)},
        "grid_storage": "fp32 nodes", "grid_bytes": int(sum(4 * g ** 3 for g in grid_n)),
        "grid_bytes_cell_corner_layout": int(sum(40 * g ** 3 for g in grid_n)),
        "precision": args.precision, "tuning": tuning, "setup_s": setup_s, "steps": args.c3_steps, "wall_s": wall,
        "scene_steps_per_s": n * args.c3_steps / wall, "rounds": r1 - r0,
        "scene_evaluations": int(evals.sum()),
        "evaluations_per_scene_step": float(evals.sum()) / (n * args.c3_steps),
        "contact_point_evaluations": cpe, "contact_pts_per_s": cpe / wall,
        "work_spread": {
            "points_per_scene_evaluation": {"min": int(pts_scene.min()), "median": float(np.median(pts_scene)),
                                            "max": int(pts_scene.max())},
            "evaluations_per_scene": {"min": int(evals.min()), "median": float(np.median(evals)),
                                      "max": int(evals.max())},
            "contact_points_per_scene": {"min": int((evals * pts_scene).min()),
                                         "median": float(np.median(evals * pts_scene)),
                                         "max": int((evals * pts_scene).max())}},
        "converged_last_step": float(np.mean(conv)),
        "displacement": {"escaped_over_1": int((disp > 1.0).sum()), "held_under_0.1": int((disp < 0.1).sum())},
    }
    if args.c3_cpu_scenes > 0 and rank == 0:
        # the oracle on the first scenes, a few steps each, one process per scene
        k = min(args.c3_cpu_scenes, len(scenes))
        jobs = []
        for sc in scenes[:k]:
            m = sc.asm.mover
            Fm = np.zeros(6)
            Fm[3:] = C3_PULL * sc.asm.direction
            mover = (sc.mass, sc.inertia, np.eye(4), sc.placement(m), C3_GRAVITY, C3_H, Fm)
            pairs = []
            for a, b in sc.contact_pairs():
                lo, hi, dx = sc.grid_boxes[b]
                pairs.append(((b, ctx.grid_values(sc.grid_handles[b]), lo, hi, dx), sc.points[a], a == m,
                              sc.placement(b if a == m else a)))
            jobs.append((mover, pairs, args.c3_cpu_steps))
        procs = min(k, os.cpu_count() or 1)
        t = time.perf_counter()
        with mp.get_context("spawn").Pool(procs) as pool:
            res = pool.map(_c3_cpu_scene, jobs, chunksize=1)
        cwall = time.perf_counter() - t
        ev = np.array([r[1] for r in res])
        out["cpu_baseline"] = {
            "value": k * args.c3_cpu_steps / cwall, "unit": "scene-steps/s", "cores": procs, "kind": "port",
            "contact_pts_per_s": float((ev * pts_scene[:k]).sum()) / cwall,
            "sample": f"scenes 0-{k - 1}, {args.c3_cpu_steps} steps each from rest, one process per scene "
                      "(wall time includes sending each scene's grids to its process)"}
    sim.close()
    return out


def cpu_sim_rate(pool, n_scenes, steps, procs):
    dirs = W.fibonacci_directions(1024)
    idx = np.linspace(0, len(dirs) - 1, n_scenes).astype(int)
    t = time.perf_counter()
    res = pool.map(_cpu_sim, [(dirs[k], steps) for k in idx], chunksize=1)
    wall = time.perf_counter() - t
    evals = sum(r[1] for r in res)
    t_fwd, t_bwd = sum(r[0] for r in res), sum(r[2] for r in res)
    return {"scene_steps_per_s": n_scenes * steps / wall, "steps": steps, "scenes": n_scenes, "cores": procs,
            "scene_evaluations": evals, "wall_s": wall,
            # forward and adjoint share the wall time; split it by their single-core times
            "adjoint_scene_steps_per_s": n_scenes * steps / (wall * t_bwd / max(t_fwd + t_bwd, 1e-12))}


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=("gb300", "reference"), default="gb300")
    ap.add_argument("--instances", type=int, default=1024)
    ap.add_argument("--points", type=int, default=50000)
    ap.add_argument("--grid", type=int, default=128)
    ap.add_argument("--cpu-sample", type=int, default=512, help="instances per CPU-baseline step")
    ap.add_argument("--ref-sample", type=int, default=128,
                    help="--impl reference: instances per step when the reference itself is timed")
    ap.add_argument("--ref-port", action="store_true",
                    help="--impl reference: time the oracle's C port even where the reference can be built")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="keep the batches' default launch configuration")
    ap.add_argument("--precision", choices=("mixed", "fp64"), default="mixed")
    ap.add_argument("--plain-sample", type=int, default=64, help="instances timed on the per-instance FP64 path")
    ap.add_argument("--full-error", action="store_true", help="compare every instance against the FP64 path")
    ap.add_argument("--sim-steps", type=int, default=500, help="BDF1 steps of the direction sweep (0: skip)")
    ap.add_argument("--sim-early", type=int, default=25, help="steps also timed alone (compared with the CPU)")
    ap.add_argument("--cpu-sim-scenes", type=int, default=32, help="scenes stepped by the CPU baseline")
    ap.add_argument("--c4-instances", type=int, default=4096, help="differentiable-rollout leg: instances (0: skip)")
    ap.add_argument("--c4-steps", type=int, default=200, help="differentiable-rollout leg: BDF1 steps")
    ap.add_argument("--c4-points", type=int, default=10000, help="differentiable-rollout leg: peg points")
    ap.add_argument("--c4-check", type=int, default=8,
                    help="differentiable-rollout leg: instances whose gradients are checked by central differences")
    ap.add_argument("--c4-precision", choices=("mixed", "fp64"), default="mixed",
                    help="differentiable-rollout leg: precision of the force evaluations")
    ap.add_argument("--planner-states", type=int, default=4096, help="planner-query leg: poses (0: skip the leg)")
    ap.add_argument("--planner-vertices", type=int, default=20000, help="planner-query leg: mover mesh vertices")
    ap.add_argument("--planner-cpu-sample", type=int, default=64, help="planner-query leg: poses timed on the CPU")
    ap.add_argument("--ls-segments", type=int, default=512,
                    help="SDF-construction leg: torus segments (x segments/2 quads; 0: skip the leg)")
    ap.add_argument("--ls-dx", type=float, default=0.0068, help="SDF-construction leg: grid spacing")
    ap.add_argument("--ls-cpu-dx", type=float, default=0.02, help="SDF-construction leg: spacing of the CPU sample")
    ap.add_argument("--tuning", default="",
                    help="headline batch: launch configuration FORM,SLOTS,CHUNKS_PER_SLOT (FORM ctas, workers or "
                         "grid) instead of the autotuner's")
    ap.add_argument("--c5-grid", type=int, default=512, help="FP16-brick leg: grid nodes per axis")
    ap.add_argument("--c5-points", type=int, default=1000000, help="FP16-brick leg: points (0: skip the leg)")
    ap.add_argument("--c5-dirs", type=int, default=256, help="FP16-brick leg: pull directions")
    ap.add_argument("--c5-steps", type=int, default=200, help="FP16-brick leg: BDF1 steps (0: skip)")
    ap.add_argument("--c5-check", type=int, default=8, help="FP16-brick leg: instances checked on the FP64 grid")
    ap.add_argument("--c3-assemblies", type=int, default=256,
                    help="uneven multi-part leg: procedural assemblies (0: skip the leg)")
    ap.add_argument("--c3-steps", type=int, default=300, help="uneven multi-part leg: BDF1 steps")
    ap.add_argument("--c3-cpu-scenes", type=int, default=8, help="uneven multi-part leg: scenes stepped on the CPU")
    ap.add_argument("--c3-cpu-steps", type=int, default=3, help="uneven multi-part leg: CPU steps per scene")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    world, rank = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_gpu(args, world, rank)


if __name__ == "__main__":
    main()
