#!/usr/bin/env python
"""Throughput of the Multall time-marching loop on GB300, in Gnode-iter/s.

Workload: the single-stage axial turbine, 65 x 242 x 49 nodes (121 J-points
per row), 48-vane nozzle + 60-blade rotor at 9000 rpm with 1 % tip gap,
mixing plane, 3-level multigrid (blocks 3 and 9), SCREE, mixing-length LOSS
every 5 steps, the 5-step monitor tail and STEPUP -- synthetic seeded
geometry (no public benchmark suite exists for this solver).  One "step" is
one full LOOP iteration.  Gnode-iter/s = IM*JM*KM*steps/seconds/1e9.

GPU arm (default): steps are CUDA-graph replays timed with CUDA events on
the library's stream, with an L2-sized buffer rewritten between steps
(outside the timed events).  e2e: the same steps through the C ABI call a
Fortran LOOP replacement would make, mgpu_step() per iteration (host->device
control word, device->host monitors, synchronous), plus the upload of the
flow state from host buffers before and the download after, all inside the
wall-clock region.  Multi-GPU (torchrun): one independent instance per GPU
(replicas, weak scaling), host-side barrier and max-over-ranks time.

Reference arm (--impl reference): the CPU oracle -- the serial C++
restatement of the reference's LOOP -- on the same workload, on the box's
host cores; the reference program is serial, so it uses one thread.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "multall-open-18.3_gb300"))

METRIC = "Gnode-iter/s"
WORKLOADS = {
    "stage": ("turbine_stage",
              "single-stage axial turbine 65x242x49 (121 J per row), nozzle 48 vanes + rotor 60 blades "
              "9000 rpm, 1% tip gap, mixing plane, 3-level multigrid, SCREE, mixing-length LOSS/5 steps"),
    "compressor": ("compressor_4stage",
                   "4-stage axial compressor 73x752x57, 8 rows (36..64 blades) 12000 rpm, mixing planes "
                   "between all rows, 3-level multigrid, SCREE, mixing-length LOSS/5 steps"),
    "deck_stage": ("deck:Single-stage-turbine-17.1",
                   "the reference's own single-stage turbine test deck (Single-stage-turbine-17.1.dat) 46x282x46, "
                   "nozzle 71 vanes + rotor 83 blades 3000 rpm, mixing plane, 3-level multigrid, SCREE, "
                   "mixing-length LOSS/5 steps, read by mgpu.deck (tests/golden/decks)"),
    "nozzle": ("nozzle_row",
               "axial turbine nozzle row 37x97x33, 48 vanes, 3-level multigrid (level 2 off), SCREE, "
               "mixing-length LOSS/5 steps"),
    "adjoint": ("turbine_stage",
                "discrete adjoint (frozen mixing length) of the single-stage turbine 65x242x49, SFXIN=SFTIN=0.02: "
                "gradients of eta_tt and inlet mass flow w.r.t. 30 blade-angle design variables "
                "(stagger, inlet and exit metal angle at 5 span sections x 2 rows)"),
    "converge": ("turbine_stage",
                 "single-stage axial turbine 65x242x49 as the headline workload with SFXIN=SFTIN=0.02, marched "
                 "from SETUP's initial guess to the reference's end test (EAVG or |EMAX| below CONLIM=1e-5 with "
                 "ECONT < 1%): default precision split against the plain FP32 path"),
    "batch64": ("batch_instance",
                "64 single-stage turbines in one batch graph: I in {33,49,65}, K in {33,49}, J in [97,161], "
                "exit P/P0 in [0.45,0.70], 7000-10000 rpm (seeded), SCREE, mixing-length LOSS/5 steps"),
}
BATCH = 64
# The default precision split (REDUCE_ORDER=0), as the JSON line names it
REDUCTIONS = ("precision split (REDUCE_ORDER=0): FP32 field arithmetic; the long sums (multigrid blocks, row means, "
              "mixing-plane averages, monitors) formed wide and rounded once: double-float FP32 pairs in the "
              "TSTEP kernels, FP64 elsewhere")

# Compulsory traffic of one LOOP iteration per node (FP32), every array read
# once and written once: 5 state arrays r+w (40 B), 5 SCREE histories r+w
# (40 B), 9 geometry arrays r (36 B), 4 body forces r (16 B).
B_ALG_STEP = 132
# Per kernel: (compulsory bytes per node for one unit of its work, units per
# step).  A TSTEP kernel's unit is one variable (5 per step, batched 2 + 3 per
# launch); LOSS runs every NLOS = 5 steps.
#   cells   XFLUX, TFLUX, RFLUX, SOURCE, DIFF read; DIFF, STORE written
#   prolong STORE, STEP, RSTEP read; STORE written
#   update  STORE, D read; TMP written
#   smooth  TMP read; D written
KERNEL_BYTES = {
    # mass and energy fluxes: ROVX, ROVR, RO, ROVT, 6 areas, HO, PEFF, QSOURCE read (13 arrays); FLOWX, FLOWT,
    # FLOWR, ROWT, WT and ROE's XFLUX, TFLUX, RFLUX, SOURCE written (9)
    "k_prim": (48, 1), "k_flux_mass_energy": (88, 1),
    # momentum fluxes: 19 arrays read (P, V*, ROVT, FLOW*, 6 areas, VOLOR, 3 forces, RO for the
    # density-limiter flags), 13 written (9 fluxes, 3 sources, PEFF)
    "k_flux_mom": (128, 1),
    "k_mach_limiter": (24, 1),
    "k_ts_cells": (28, 5), "k_ts_prolong": (16, 5), "k_ts_update": (12, 5), "k_ts_update_pair": (12, 5),
    "k_ts_smooth": (8, 5),
    "k_loss_kfaces": (72, 0.2), "k_loss_ifaces": (84, 0.2),
}
PROFILE_STEPS = 10
ARGS_WORKLOAD = "stage"


def env_int(name, default):
    try:
        return int(os.environ.get(name, default))
    except ValueError:
        return default


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


def ncu_traffic_per_launch():
    """Per-kernel (DRAM bytes per launch, threads per CTA) from the committed
    ncu summary of the stage workload (profiles/ncu_stage_traffic.md), if
    present: one-kernel captures of an untuned run, not of this run."""
    p = os.path.join(ROOT, "profiles", "ncu_stage_traffic.md")
    out = {}
    if not os.path.exists(p):
        return out
    for line in open(p):
        cols = [c.strip() for c in line.strip().strip("|").split("|")]
        if len(cols) >= 6 and cols[0].startswith("k_"):
            try:
                out[cols[0]] = (float(cols[2]), cols[5])
            except ValueError:
                pass
    return out


class NvmlSampler:
    """SM clock and clock-event reasons read through NVML (the driver's
    libnvidia-ml, bound with ctypes) every ~2 ms on a thread, so that a timed
    region of a few milliseconds still holds samples.  Reads only."""
    SM_CLOCK = 1
    REASONS = {0x8: "hw_slowdown", 0x40: "hw_thermal_slowdown", 0x20: "sw_thermal_slowdown", 0x4: "sw_power_cap"}

    def __init__(self, gpu_index=0):
        import ctypes
        self.ct = ctypes
        self.nv = ctypes.CDLL("libnvidia-ml.so.1")
        if self.nv.nvmlInit_v2() != 0:
            raise OSError("nvmlInit failed")
        self.h = ctypes.c_void_p()
        if self.nv.nvmlDeviceGetHandleByIndex_v2(gpu_index, ctypes.byref(self.h)) != 0:
            raise OSError("no NVML device")
        try:
            self.reasons_fn = self.nv.nvmlDeviceGetCurrentClocksEventReasons
        except AttributeError:
            self.reasons_fn = self.nv.nvmlDeviceGetCurrentClocksThrottleReasons
        mx = ctypes.c_uint()
        self.nv.nvmlDeviceGetMaxClockInfo(self.h, self.SM_CLOCK, ctypes.byref(mx))
        self.max_mhz = float(mx.value)
        self.rows = []
        self.stop = threading.Event()

    def _read(self):
        ct = self.ct
        mhz, rs = ct.c_uint(), ct.c_ulonglong()
        while not self.stop.is_set():
            if self.nv.nvmlDeviceGetClockInfo(self.h, self.SM_CLOCK, ct.byref(mhz)) == 0:
                r = rs.value if self.reasons_fn(self.h, ct.byref(rs)) == 0 else 0
                self.rows.append((float(mhz.value), int(r)))
            time.sleep(0.002)

    def __enter__(self):
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()
        return self

    def __exit__(self, *a):
        self.stop.set()
        self.t.join(timeout=2)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": self.max_mhz, "reasons": [], "samples": 0, "source": "nvml"}
        reasons = set()
        for _, r in self.rows:
            for bit, name in self.REASONS.items():
                if r & bit:
                    reasons.add(name)
        return {"sm_mhz": statistics.median(m for m, _ in self.rows), "sm_max_mhz": self.max_mhz,
                "reasons": sorted(reasons), "samples": len(self.rows), "source": "nvml, every ~2 ms"}


def clock_sampler(gpu_index=0):
    """NVML sampler when the driver's library loads, else nvidia-smi."""
    try:
        return NvmlSampler(gpu_index)
    except (OSError, AttributeError):
        return ClockSampler(gpu_index)


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during a region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.rows = []
        self.proc = None
        self.gpu = gpu_index

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for n, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def pinned_like(a):
    """A page-locked host copy of a (torch's pinned allocator), as a numpy
    view; a plain copy when pinning is unavailable."""
    try:
        import torch
        t = torch.empty(a.shape, dtype=getattr(torch, a.dtype.name), pin_memory=True)
        out = t.numpy()            # shares t's storage and keeps it alive
        out[...] = a
        return out
    except Exception:
        return a.copy()


def dist_setup(world, rank):
    if world <= 1:
        return None
    import torch.distributed as dist
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group("gloo", rank=rank, world_size=world)
    return dist


def replica_setup(world, rank, local_rank):
    """One process per GPU: rank r sees only GPU local_rank, and the ranks
    join one gloo group for the host-side barrier and the max-over-ranks
    time (there is no data-path collective: each rank marches its own
    instance)."""
    if world > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local_rank)
    return dist_setup(world, rank)


def replica_value(dist, world, nodes_per_rank, steps, ms_local):
    """(slowest rank's ms, whole-job Gnode-iter/s): every rank marched
    nodes_per_rank nodes for `steps` steps; the job took the slowest rank's
    time."""
    ms_max = dist_max(dist, ms_local)
    return ms_max, nodes_per_rank * steps * world / (ms_max / 1e3) / 1e9


def dist_max(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_barrier(dist):
    if dist is not None:
        dist.barrier()


def build_case():
    from mgpu import case, common_setup
    if ARGS_WORKLOAD == "batch64":          # one member stands for the batch on the CPU
        return common_setup.build_common(case.batch_instance(0))
    src = WORKLOADS[ARGS_WORKLOAD][0]
    if src.startswith("deck:"):             # a reference deck, as the reader left it
        from mgpu import deck
        spec, geo = deck.load_fixture(os.path.join(ROOT, "tests", "golden", "decks", src[5:] + ".npz"))
        return common_setup.build_common(spec, geo)
    spec = getattr(case, src)()
    return common_setup.build_common(spec)


def host_cpu():
    """nproc and the CPU model of the host the CPU baseline runs on."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                model = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.TimeoutExpired):
        pass
    if model is None and os.path.exists("/proc/cpuinfo"):
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith("model name"):
                model = line.split(":", 1)[1].strip()
                break
    return {"nproc": os.cpu_count(), "model": model}


def cpu_oracle_rate(cd, seconds, max_steps, warmup=1):
    """Serial CPU oracle (FP32) on the workload, the process pinned to one
    core for the timed steps (as `taskset -c <core>` would): a dict with
    Gnode-iter/s, steps, seconds, the core, the host and the reference's own
    figure, CPU time per point per step (multall-open-18.3.f:5404-5414)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    o = O.Oracle(cd)
    o.setup_calls()
    for _ in range(warmup):
        o.step()
    old = os.sched_getaffinity(0) if hasattr(os, "sched_getaffinity") else None
    core = min(old) if old else None
    if core is not None:
        os.sched_setaffinity(0, {core})
    try:
        t0 = time.perf_counter()
        n = 0
        while n < max_steps and (n == 0 or time.perf_counter() - t0 < seconds):
            o.step()
            n += 1
        dt = time.perf_counter() - t0
    finally:
        if old is not None:
            os.sched_setaffinity(0, old)
    o.close()
    return {"rate": cd.nodes() * n / dt / 1e9, "steps": n, "seconds": dt, "warmup": warmup, "core": core,
            "host": host_cpu(), "cpu_time_per_point_per_step_s": dt / n / cd.nodes()}


def cpu_baseline_entry(r, what):
    return {"value": r["rate"], "unit": METRIC, "cores": 1, "kind": "port",
            "pinned_core": r["core"], "host": r["host"],
            "cpu_time_per_point_per_step_s": r["cpu_time_per_point_per_step_s"],
            "sample": f"{r['steps']} LOOP iterations of {what} after {r['warmup']} warm-up, serial C++ "
                      f"restatement of LOOP (oracle) built -O2 -ffp-contract=off, one thread pinned to core "
                      f"{r['core']}, {r['seconds']:.1f} s"}


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    cd = build_case()
    budget = float(os.environ.get("MGPU_REF_SECONDS", "120"))
    r = cpu_oracle_rate(cd, budget, max(1, args.steps), warmup=max(1, min(args.warmup, 3)))
    rate, n, dt = r["rate"], r["steps"], r["seconds"]
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": METRIC, "n_gpus": args.gpus,
        "steps": n, "warmup": r["warmup"], "ms_per_step": dt / n * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOADS[ARGS_WORKLOAD][1], "nodes": cd.nodes(),
                   "parallelism": "serial CPU: the reference is a serial program, so one thread is all it uses"},
        "cpu_baseline": cpu_baseline_entry(r, "the workload"),
        "e2e": {"value": rate, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def _build_instance(seed):
    from mgpu import case, common_setup
    return common_setup.build_common(case.batch_instance(seed))


def run_batch(args, rank, world, local_rank):
    """The 64-instance batch: one graph launch steps every instance."""
    if world > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local_rank)
    import multiprocessing as mp
    from concurrent.futures import ProcessPoolExecutor
    # host-side set-up of the 64 decks in a spawn pool, before any GPU call
    with ProcessPoolExecutor(max_workers=min(16, os.cpu_count() or 1), mp_context=mp.get_context("spawn")) as ex:
        cds = list(ex.map(_build_instance, range(BATCH)))
    dist = dist_setup(world, rank)
    from mgpu import lib
    nodes = sum(cd.nodes() for cd in cds)
    probs = [lib.Problem(cd) for cd in cds]
    # The members keep the default TSTEP size (256 threads per J-plane CTA).
    # mgpu_autotune times a member alone, where 512-thread CTAs win for the
    # small grids; inside the batch the members share the SMs, and the tuned
    # batch ran 6 % slower than the untuned one.  MGPU_AUTOTUNE=1 tunes them.
    if os.environ.get("MGPU_AUTOTUNE", "0") == "1":
        tuned = [p.autotune()[0] for p in probs]
    else:
        tuned = [(256, 256)] * len(probs)
    batch = lib.Batch(probs)
    batch.run(max(args.warmup, 3))
    dist_barrier(dist)
    with clock_sampler(0) as clk:
        ms = batch.bench_steps(args.steps, flush_l2=True)
    dist_barrier(dist)
    ms_max = dist_max(dist, ms)
    value = nodes * args.steps * world / (ms_max / 1e3) / 1e9
    # the same instances one after another, each from its own step graph
    nseq = max(5, args.steps // 10)
    seq_ms = sum(p.bench_steps(nseq, flush_l2=True) for p in probs)
    seq_value = nodes * nseq / (seq_ms / 1e3) / 1e9
    # end to end: flow state of every instance in from host buffers, batch
    # steps with the control blocks read back, state out
    state = ["RO", "ROVX", "ROVR", "RORVT", "ROE"]
    host = [{n: p.get(n) for n in state} for p in probs]
    ne = max(1, args.steps // 2)
    dist_barrier(dist)
    t0 = time.perf_counter()
    for p, hd in zip(probs, host):
        for n in state:
            p.set(n, hd[n])
    batch.run(ne)
    for p in probs:
        for n in state:
            p.get(n)
    t1 = time.perf_counter()
    e2e_s = dist_max(dist, t1 - t0)
    state_bytes = sum(a.nbytes for hd in host for a in hd.values())
    peak, peak_kind = load_peaks()
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOADS["batch64"][1], "instances": BATCH, "nodes": nodes,
                       "autotune": {"tstep_threads_per_cta": {
                           p: {str(b): [t[q] for t in tuned].count(b) for b in (128, 192, 256, 512)}
                           for q, p in enumerate(("ro_roe_pass", "momentum_pass"))}},
                       "l2": "flushed between timed steps", "parallelism": f"replicas: one batch per GPU x{world}",
                       "reductions": REDUCTIONS},
            "roofline": {"bound": "hbm", "kernel": None, "peak": peak, "unit": "GB/s", "peak_source": peak_kind,
                         "step": {"alg_bytes_per_node_iter": B_ALG_STEP, "achieved": value / world * B_ALG_STEP,
                                  "frac": value / world * B_ALG_STEP / peak}},
            "sequential": {"value": seq_value, "unit": METRIC, "steps": nseq,
                           "how": "the same 64 instances stepped one after another, each from its own graph"},
            "cpu_baseline": None,
            "clocks": clk.summary(),
            "e2e": {"value": nodes * ne * world / e2e_s / 1e9, "unit": METRIC,
                    "h2d_bytes_per_step": state_bytes / ne, "d2h_bytes_per_step": state_bytes / ne,
                    "steps": ne, "how": "mgpu_batch_run over all steps (control blocks read back every 50), "
                                        "every instance's flow state uploaded before and downloaded after"},
        }
        print(json.dumps(line), flush=True)
    batch.close()
    for p in probs:
        p.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


# reverse-step kernels: seeds, mixing plane (when there is one), 2 limiters,
# 2 x 4 TSTEP kernels, momentum, energy and mass fluxes (a coefficient and a
# gather pass each), inlet/exit, exit sums, primitives; PEFF's own reverse
# only when F_PDOWN != 0
def adj_kernels_per_step(cd) -> int:
    n = 20
    if cd.ints.get("IFMIX", 0) > 0 and cd.reals.get("RFMIX", 0.0) > 1e-3 and cd.nrows > 1:
        n += 1
    if cd.reals.get("F_PDOWN", 0.0) != 0.0:
        n += 1
    return n


def run_adjoint(args, rank, world, local_rank):
    """Config 2: adjoint against finite-difference gradient time.  The time
    of one primal solve (LOSS on, from the initial guess to the FP32
    convergence floor), of the adjoint gradient of two objectives with
    respect to 30 design variables (recording, GMRES on the transposed step,
    geometry gradients and the chain to the variables), and of one
    perturbed primal solve, which 60 central differences need each."""
    if world > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local_rank)
        if rank != 0:
            return 0            # replicas only: one problem per GPU, reported by rank 0
    import numpy as np
    from mgpu import case, lib, design

    def make():
        sp = case.turbine_stage()
        sp.sfxin = sp.sftin = 0.02
        return sp

    ds = design.DesignSpace.seeded(make)
    alpha = ds.alpha0
    cd = ds.deck(alpha)
    cd.ints["NSTEPS_MAX"] = 10 ** 9
    cd.reals["CONLIM"] = 1e-9
    # GMRES stops at tol, at max_steps, or when a restart cycle lowers the
    # residual by less than 1 % (stagnation: on this frozen-turbulence stage
    # the residual levels off at 0.09 for eta_tt and 0.20 for the mass flow)
    n_primal, inner, restart, max_steps, stall, n_fd = 16000, 50, 30, 30000, 0.01, 10000
    if os.environ.get("MGPU_ADJ_PROFILE") == "1":
        # a short run for kernel profiles: 200 primal steps, then 20 transposed
        # steps with an objective and the geometry pass, no solve and no FD
        p = lib.Problem(cd)
        p.run(200)
        p.adjoint_prepare()
        p.adjoint_objective("eta_tt")
        p.adjoint_iterate(5)
        t0 = time.perf_counter()
        rel = p.adjoint_iterate(20)
        ms = (time.perf_counter() - t0) / 20 * 1e3
        p.adjoint_gradient()
        print(json.dumps({"workload": "adjoint profile run", "transposed_steps": 26, "rel_change": rel,
                          "ms_per_transposed_step": ms}), flush=True)
        p.close()
        return 0
    p = lib.Problem(cd)
    p.run(max(args.warmup, 3))
    p.close()
    p = lib.Problem(cd)
    p.autotune()
    t0 = time.perf_counter()
    _, m = p.run(n_primal)
    t_primal = time.perf_counter() - t0
    state = {n: p.get(n) for n, a in cd.arrays.items() if a.dtype == np.float32}
    integ = p.integrals()
    # dTHETA/d(alpha) of the generator; the device turns dJ/dA into dJ/dTHETA
    # (transposed SETUP metrics), so the host differences the node angles only
    t0 = time.perf_counter()
    sens = ds.theta_sensitivities(alpha)
    t_sens = time.perf_counter() - t0
    g64 = ds.geometry64(alpha)
    grads, solves = {}, {}
    t_adj = 0.0
    d2h = 0
    with clock_sampler(0) as clk:
        for obj in ("eta_tt", "mass_flow_in"):
            t0 = time.perf_counter()
            p.adjoint_prepare()
            val = p.adjoint_objective(obj)
            ok, steps, res = p.adjoint_solve_krylov(inner=inner, restart=restart, max_steps=max_steps, tol=1e-6,
                                                    stall=stall)
            p.adjoint_gradient(read=False)
            gth = p.adjoint_gradient_theta()
            t_adj += time.perf_counter() - t0
            d2h += gth.nbytes
            grads[obj] = ds.chain_theta(gth, sens)
            solves[obj] = {"value": val, "converged": ok, "transposed_steps": steps, "rel_residual": res}
    # finite differences: restarts of the primal (LOSS on) from the converged
    # state with the geometry moved by +-h
    h = 0.2
    checks = []
    t_fd_one = None
    for i in (ds.index(1, "stagger", 2), ds.index(0, "stagger", 0)):
        js = []
        for sgn in (1.0, -1.0):
            a = alpha.copy()
            a[i] += sgn * h
            gp = ds.geometry64(a)
            cdp = design.perturbed_state(cd, state, {n: gp[n] - g64[n] for n in design.GEOM})
            cdp.ints["NSTEP"] = cd.ints["NCHANGE"] - 1
            pp = lib.Problem(cdp, setup_calls=False)
            t0 = time.perf_counter()
            pp.run(n_fd)
            dt = time.perf_counter() - t0
            t_fd_one = dt if t_fd_one is None else min(t_fd_one, dt)
            r = pp.integrals()
            js.append((r.eta_tt, r.mass_flow_in))
            pp.close()
        checks.append({"variable": ds.names()[i],
                       "eta_tt": {"adjoint": float(grads["eta_tt"][i]), "fd": (js[0][0] - js[1][0]) / (2 * h)},
                       "mass_flow_in": {"adjoint": float(grads["mass_flow_in"][i]),
                                        "fd": (js[0][1] - js[1][1]) / (2 * h)}})
    t_fd = 2 * ds.size * t_fd_one
    t_adj_total = t_adj + t_sens
    steps_total = sum(v["transposed_steps"] for v in solves.values()) + 2 * 2
    line = {
        "metric": "FD / adjoint gradient time", "value": t_fd / t_adj_total, "unit": "x", "n_gpus": world,
        "steps": steps_total, "warmup": max(args.warmup, 3), "ms_per_step": t_adj / max(steps_total, 1) * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOADS["adjoint"][1], "nodes": cd.nodes(), "design_variables": ds.size,
                   "objectives": ["eta_tt", "mass_flow_in"], "primal_steps": n_primal,
                   "krylov": {"inner": inner, "restart": restart, "max_steps": max_steps, "stall": stall},
                   "fd": {"h_deg": h, "steps_per_solve": n_fd, "solves": 2 * ds.size}},
        "adjoint_time_s": t_adj_total, "adjoint_device_s": t_adj, "sensitivities_host_s": t_sens,
        "primal_solve_s": t_primal, "adjoint_over_primal": t_adj_total / t_primal,
        "fd_gradient_time_s": t_fd, "fd_solve_s": t_fd_one,
        "primal": {"eavg": float(m.eavg), "eta_tt": integ.eta_tt, "mass_flow_in": integ.mass_flow_in},
        "solves": solves, "checks": checks,
        "cpu_baseline": None, "clocks": clk.summary(),
        "e2e": {"value": t_fd / t_adj_total, "unit": "x", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": d2h / max(steps_total, 1),
                "how": "mgpu_adjoint_* through the C ABI; dJ/dTHETA read back to the host for the chain"},
        "gpu_launches": adj_kernels_per_step(cd) * steps_total,
    }
    print(json.dumps(line), flush=True)
    p.close()
    return 0


CONVERGE_SMOOTHING = 0.02      # SFXIN = SFTIN: with the default 0.005 the stage does not settle
CONVERGE_MAXSTEPS = 40000
CONVERGE_CHUNK = 500


def run_converge(args, rank, world, local_rank):
    """Time to convergence on the stage, each path from SETUP's initial guess
    through mgpu_run in chunks of CONVERGE_CHUNK steps.  After each chunk the
    monitors of the last tail and the integrals are read, and two times are
    recorded: when the EAVG clause of the reference's end test holds (EAVG <
    CONLIM, multall-open-18.3.f:3763), and when mass flow and total-to-total
    efficiency first sit within 1e-4 (relative, absolute) of the FP64
    oracle's converged values (tests/golden/stage_converged_fp64.json, made
    by tests/golden/make_converged_fp64.py).  The time to convergence is the
    later of the two.  The full end test also asks ECONT < 1 %; on this
    synthetic stage the continuity error settles at 1.2 % one plane ahead
    of the stator trailing edge, in the oracle as on the GPU, so it never
    holds and is reported, not waited for.  Paths: the default precision
    split (FP64 long sums) and the plain FP32 path (REDUCE_ORDER=2)."""
    if world > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local_rank)
        if rank != 0:
            return 0            # replicas only: one problem per GPU, reported by rank 0
    from mgpu import case, common_setup, lib
    fx_path = os.path.join(ROOT, "tests", "golden", "stage_converged_fp64.json")
    fx = json.load(open(fx_path)) if os.path.exists(fx_path) else None

    def spec():
        sp = case.turbine_stage()
        sp.sfxin = sp.sftin = CONVERGE_SMOOTHING
        return sp

    # warm-up: one short run builds the library's graph and loads the kernels
    w = lib.Problem(common_setup.build_common(spec()))
    w.run(max(args.warmup, 3))
    w.close()
    res = {}
    conlim = None
    with clock_sampler(0) as clk:
        for name, order in (("chosen", 0), ("plain_fp32", 2)):
            cd = common_setup.build_common(spec())
            conlim = cd.reals["CONLIM"]
            cd.ints["NSTEPS_MAX"] = 10 ** 9
            cd.ints["REDUCE_ORDER"] = order
            p = lib.Problem(cd)
            tuned, _ = p.autotune()       # restores the state it times on
            p.run(0)                      # builds the step graph outside the timed region
            p.sync()
            t_eavg = t_close = None
            s_eavg = s_close = None
            hist = []
            t0 = time.perf_counter()
            steps = 0
            while steps < CONVERGE_MAXSTEPS:
                _, m = p.run(CONVERGE_CHUNK)
                steps += CONVERGE_CHUNK
                it = p.integrals()
                t = time.perf_counter() - t0
                e_eta = abs(it.eta_tt - fx["eta_tt"]) if fx else None
                e_m = abs(it.mass_flow_in - fx["mass_flow_in"]) / abs(fx["mass_flow_in"]) if fx else None
                hist.append([steps, round(t, 4), float(m.eavg), float(m.econt), it.eta_tt, it.mass_flow_in])
                if t_eavg is None and m.eavg < conlim:
                    t_eavg, s_eavg = t, steps
                if fx and t_close is None and e_eta <= 1e-4 and e_m <= 1e-4:
                    t_close, s_close = t, steps
                if t_eavg is not None and (fx is None or t_close is not None):
                    break
            r = {"steps_to_eavg_below_conlim": s_eavg, "seconds_to_eavg_below_conlim": t_eavg,
                 "steps_to_within_1e-4_of_fp64": s_close, "seconds_to_within_1e-4_of_fp64": t_close,
                 "converged_seconds": None if (t_eavg is None or (fx and t_close is None)) else
                 max(t_eavg, t_close or 0.0),
                 "final": {"steps": steps, "eavg": float(m.eavg), "emax": float(m.emax), "econt": float(m.econt),
                           "jcont": int(m.jcont), "eta_tt": it.eta_tt, "mass_flow_in": it.mass_flow_in},
                 "tstep_threads_per_cta": list(tuned), "history": hist}
            if fx is not None:
                r["final"]["eta_err_vs_fp64"] = abs(it.eta_tt - fx["eta_tt"])
                r["final"]["mass_flow_rel_err_vs_fp64"] = abs(it.mass_flow_in - fx["mass_flow_in"]) / abs(
                    fx["mass_flow_in"])
            r["kernels_per_step"] = [p.kernels_per_step(), p.kernels_per_step(loss=True, tail=True)]
            res[name] = r
            p.close()
    c, pl = res["chosen"], res["plain_fp32"]
    nodes = 65 * 242 * 49
    value = c["converged_seconds"]
    steps = c["final"]["steps"]
    line = {
        "metric": "time to convergence", "value": value, "unit": "s", "n_gpus": world, "steps": steps,
        "warmup": max(args.warmup, 3), "ms_per_step": c["history"][-1][1] / steps * 1e3,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOADS["converge"][1], "nodes": nodes, "chunk_steps": CONVERGE_CHUNK,
                   "conlim": conlim, "max_steps": CONVERGE_MAXSTEPS,
                   "l2": "inputs (216 MB working set) larger than L2, no flush inside a run",
                   "fp64_oracle": None if fx is None else {k: fx.get(k) for k in ("nstep", "eta_tt", "mass_flow_in",
                                                                                  "eavg", "econt")}},
        "chosen": c, "plain_fp32": pl,
        "plain_over_chosen_time": (pl["converged_seconds"] / value) if (value and pl["converged_seconds"]) else None,
        "cpu_baseline": None, "clocks": clk.summary(),
        "e2e": {"value": value, "unit": "s", "h2d_bytes_per_step": 4,
                "d2h_bytes_per_step": (200 * steps / 5 + 64 * steps / CONVERGE_CHUNK) / max(steps, 1),
                "how": "mgpu_run through the C ABI in chunks (control block read back every fifth step), "
                       "mgpu_integrals_compute after each chunk"},
        "gpu_launches": c["kernels_per_step"][0] * steps
        + (c["kernels_per_step"][1] - c["kernels_per_step"][0]) * (steps // 5),
    }
    print(json.dumps(line), flush=True)
    return 0


def run_gpu(args, rank, world, local_rank):
    dist = replica_setup(world, rank, local_rank)
    from mgpu import lib
    import numpy as np
    cd = build_case()
    N = cd.nodes()
    prob = lib.Problem(cd)
    kps = prob.kernels_per_step()
    kps_loss, kps_tail = prob.kernels_per_step(loss=True) - kps, prob.kernels_per_step(tail=True) - kps
    prob.run(max(args.warmup, 3))
    tuned, tune_ms = (256, 256), None
    if os.environ.get("MGPU_AUTOTUNE", "1") != "0":
        tuned, tune_ms = prob.autotune()    # threads per J-plane CTA of the TSTEP kernels
        prob.run(3)
    dist_barrier(dist)
    with clock_sampler(0) as clk:
        t_wall0 = time.perf_counter()
        ms = prob.bench_steps(args.steps, flush_l2=True)
        t_wall1 = time.perf_counter()
    dist_barrier(dist)
    ms_max, value = replica_value(dist, world, N, args.steps, ms)
    ms_per_step = ms_max / args.steps

    # per-kernel device times (events around each launch, no graph); LOSS
    # and tail kernels are launched every step here and return at once on
    # the steps that do not need them
    prof = prob.profile_steps(PROFILE_STEPS)
    step_kernels = [p for p in prof if p[0] in KERNEL_BYTES]
    dom_name, dom_launches, dom_ms = max(step_kernels, key=lambda p: p[2])
    bpn, units = KERNEL_BYTES[dom_name]
    step_s = dom_ms / PROFILE_STEPS / 1e3                    # this kernel's device time per step
    alg_step = bpn * N * units                               # its compulsory bytes per step
    launches_step = dom_launches / PROFILE_STEPS
    achieved = alg_step / step_s / 1e9
    peak, peak_kind = load_peaks()
    # DRAM traffic of the dominant kernel: measured by ncu on the stage
    # workload only, in its own capture (profiles/ncu_stage_traffic.md)
    traffic = traffic_source = None
    if ARGS_WORKLOAD == "stage" and dom_name in ncu_traffic_per_launch():
        traffic, cta = ncu_traffic_per_launch()[dom_name]
        traffic_source = (f"profile: profiles/ncu_stage_traffic.md, ncu dram__bytes_read.sum+dram__bytes_write.sum "
                          f"of a one-kernel capture (-c 4, cold L2) of an untuned run at {cta} threads per CTA, "
                          f"not of this run")
    total_prof = sum(p[2] for p in prof)

    # end to end through the C ABI, as a Fortran LOOP replacement drives it:
    # the flow state (the COMMON arrays RO, ROVX, ROVR, RORVT, ROE) uploaded
    # from pinned host buffers, then every one of the K steps through
    # mgpu_step() (control word in, monitors out, synchronous), then the
    # state downloaded into the pinned buffers, all inside the wall clock
    state = ["RO", "ROVX", "ROVR", "RORVT", "ROE"]
    host = {n: pinned_like(prob.get(n)) for n in state}
    h2d_step, d2h_step = lib.step_io_bytes()
    ne = max(1, args.steps)
    dist_barrier(dist)
    t0 = time.perf_counter()
    for n in state:
        prob.set(n, host[n])
    for _ in range(ne):
        prob.step()
    for n in state:
        prob.get_into(n, host[n])
    t1 = time.perf_counter()
    dist_barrier(dist)
    e2e_s = dist_max(dist, t1 - t0)
    state_bytes = sum(host[n].nbytes for n in state)
    e2e = {"value": N * ne * world / e2e_s / 1e9, "unit": METRIC,
           "h2d_bytes_per_step": (state_bytes + h2d_step * ne) / ne,
           "d2h_bytes_per_step": (state_bytes + d2h_step * ne) / ne,
           "steps": ne, "wall_s": e2e_s,
           "how": f"the flow state ({state_bytes} B) uploaded from pinned host buffers, then {ne} x mgpu_step() "
                  f"(graph launch, {h2d_step} B control word in, {d2h_step} B monitors out, synchronous), then "
                  f"the state downloaded; bytes per step include the state copies spread over the {ne} steps"}

    # the plain FP32 path (REDUCE_ORDER=2: the same parallel trees with FP32
    # adds) and the reference-order path (REDUCE_ORDER=1: the long sums
    # formed by single threads in the reference's sequential REAL*4 order,
    # the parity mode), each on the same workload with the same CTA sizes
    plain = ref_order = None
    if os.environ.get("MGPU_BENCH_PLAIN", "1") != "0":
        for order in (2, 1):
            cdp = build_case()
            cdp.ints["REDUCE_ORDER"] = order
            cdp.ints["TS_THREADS"] = 0
            pp = lib.Problem(cdp)
            pp.run(max(args.warmup, 3))
            if order == 2:
                pp.autotune()
                pp.run(3)
            npl = max(20, min(200, args.steps)) if order == 2 else 10
            ms_pl = pp.bench_steps(npl, flush_l2=True)
            pp.close()
            v_pl = N * npl / (ms_pl / 1e3) / 1e9
            entry = {"value": v_pl, "unit": METRIC, "steps": npl, "ms_per_step": ms_pl / npl,
                     "chosen_over_this": value / world / v_pl}
            if order == 2:
                entry["how"] = ("REDUCE_ORDER=2: the default path's parallel reduction trees (multigrid superblock, "
                                "row-mean, monitor sums) with FP32 adds, mixing-plane line sums in REAL*4; "
                                "time to convergence and errors against the FP64 oracle: bench.py --workload "
                                "converge")
                plain = entry
            else:
                entry["how"] = ("REDUCE_ORDER=1: the long sums formed by single threads in the reference's "
                                "sequential REAL*4 order (the parity mode)")
                ref_order = entry

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        r = cpu_oracle_rate(cd, float(os.environ.get("MGPU_CPU_SECONDS", "15")), 10 ** 6)
        cpu = cpu_baseline_entry(r, "the same workload")
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOADS[ARGS_WORKLOAD][1], "nodes": N, "l2": "flushed between timed steps",
                       "parallelism": f"replicas: one instance per GPU x{world}",
                       "reductions": REDUCTIONS,
                       "autotune": {"tstep_threads_per_cta": {"ro_roe_pass": tuned[0], "momentum_pass": tuned[1]},
                                    "tstep_pass_ms": None if tune_ms is None else
                                    {p: dict(zip(("128", "192", "256", "512"), v)) for p, v in tune_ms.items()}}},
            "roofline": {"bound": "hbm", "kernel": dom_name, "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "traffic_source": traffic_source,
                         "peak_source": peak_kind,
                         "alg_bytes_per_launch": alg_step / launches_step,
                         "avg_launch_ms": step_s * 1e3 / launches_step,
                         "alg_bytes_per_node_unit": bpn, "units_per_step": units,
                         "share_of_step": dom_ms / total_prof,
                         "step": {"alg_bytes_per_node_iter": B_ALG_STEP,
                                  "achieved": value / world * B_ALG_STEP, "frac": value / world * B_ALG_STEP / peak}},
            "plain_fp32": plain,
            "reference_order": ref_order,
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
            "e2e": e2e,
            # NSTEP runs on from the warm-up; over a whole number of 5-step
            # cycles every 5th step runs LOSS (NLOS = 5) and the tail
            "gpu_launches": kps * args.steps + (kps_loss + kps_tail) * (args.steps // 5),
            "kernels_per_step": {"plain": kps, "loss_extra": kps_loss, "tail_extra": kps_tail},
            "wall_s_timed_region": t_wall1 - t_wall0,
        }
        print(json.dumps(line), flush=True)
        if args.profile_out:
            with open(args.profile_out, "w") as f:
                for name, launches, tot in sorted(prof, key=lambda p: -p[2]):
                    f.write(f"{name} {launches} {tot:.4f}\n")
    prob.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", choices=["gpu", "reference"], default="gpu")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile-out", default=None)
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="stage",
                    help="the headline workload is the single-stage turbine; the others are extra lines")
    args = ap.parse_args()
    global ARGS_WORKLOAD
    ARGS_WORKLOAD = args.workload
    rank = env_int("RANK", 0)
    world = env_int("WORLD_SIZE", 1)
    local_rank = env_int("LOCAL_RANK", 0)
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if args.workload == "batch64":
        return run_batch(args, rank, world, local_rank)
    if args.workload == "adjoint":
        return run_adjoint(args, rank, world, local_rank)
    if args.workload == "converge":
        return run_converge(args, rank, world, local_rank)
    return run_gpu(args, rank, world, local_rank)


if __name__ == "__main__":
    sys.exit(main())
