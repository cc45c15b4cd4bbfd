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
    "nozzle": ("nozzle_row",
               "axial turbine nozzle row 37x97x33, 48 vanes, 3-level multigrid (level 2 off), SCREE, "
               "mixing-length LOSS/5 steps"),
    "adjoint": ("turbine_stage",
                "discrete adjoint (frozen mixing length) of the single-stage turbine 65x242x49, SFXIN=SFTIN=0.02: "
                "gradients of eta_tt and inlet mass flow w.r.t. 30 blade-angle design variables "
                "(stagger, inlet and exit metal angle at 5 span sections x 2 rows)"),
    "batch64": ("batch_instance",
                "64 single-stage turbines in one batch graph: I in {33,49,65}, K in {33,49}, J in [97,161], "
                "exit P/P0 in [0.45,0.70], 7000-10000 rpm (seeded), SCREE, mixing-length LOSS/5 steps"),
}
BATCH = 64
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
    "k_prim": (48, 1), "k_flux_mass": (60, 1), "k_flux_energy": (40, 1),
    # momentum fluxes: 19 arrays read (P, V*, ROVT, FLOW*, 6 areas, VOLOR, 3 forces, RO for the
    # density-limiter flags), 13 written (9 fluxes, 3 sources, PEFF)
    "k_flux_mom": (128, 1),
    "k_mach_limiter": (24, 1),
    "k_ts_cells": (28, 5), "k_ts_prolong": (16, 5), "k_ts_update": (12, 5), "k_ts_smooth": (8, 5),
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
    """Per-kernel DRAM bytes per launch from the committed ncu summary of
    this workload (profiles/ncu_stage_traffic.md), if present."""
    p = os.path.join(ROOT, "profiles", "ncu_stage_traffic.md")
    out = {}
    if not os.path.exists(p):
        return out
    for line in open(p):
        cols = [c.strip() for c in line.strip().strip("|").split("|")]
        if len(cols) >= 3 and cols[0].startswith("k_"):
            try:
                out[cols[0]] = float(cols[2])
            except ValueError:
                pass
    return out


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


def dist_setup(world, rank):
    if world <= 1:
        return None
    import torch.distributed as dist
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group("gloo", rank=rank, world_size=world)
    return dist


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
    spec = getattr(case, WORKLOADS[ARGS_WORKLOAD][0])()
    return common_setup.build_common(spec)


def cpu_oracle_rate(cd, seconds, max_steps):
    """Serial CPU oracle (FP32) on the workload: (Gnode-iter/s, steps, s)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    o = O.Oracle(cd)
    o.setup_calls()
    o.step()                                  # warm-up step
    t0 = time.perf_counter()
    n = 0
    while n < max_steps and (n == 0 or time.perf_counter() - t0 < seconds):
        o.step()
        n += 1
    dt = time.perf_counter() - t0
    o.close()
    return cd.nodes() * n / dt / 1e9, n, dt


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    cd = build_case()
    budget = float(os.environ.get("MGPU_REF_SECONDS", "120"))
    rate, n, dt = cpu_oracle_rate(cd, budget, max(1, args.steps))
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": METRIC, "n_gpus": args.gpus,
        "steps": n, "warmup": 1, "ms_per_step": dt / n * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOADS[ARGS_WORKLOAD][1], "nodes": cd.nodes(),
                   "parallelism": "serial CPU (the reference is serial)"},
        "cpu_baseline": {"value": rate, "unit": METRIC, "cores": 1, "kind": "port",
                         "sample": f"{n} LOOP iterations of the workload after 1 warm-up, serial C++ restatement "
                                   f"(oracle) built -O2 -ffp-contract=off, {dt:.1f} s"},
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
    with ClockSampler(0) as clk:
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
                       "reductions": "FP64 tree sums (REDUCE_ORDER=0)"},
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
    with ClockSampler(0) as clk:
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


def run_gpu(args, rank, world, local_rank):
    if world > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local_rank)
    dist = dist_setup(world, rank)
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
    with ClockSampler(0) as clk:
        t_wall0 = time.perf_counter()
        ms = prob.bench_steps(args.steps, flush_l2=True)
        t_wall1 = time.perf_counter()
    dist_barrier(dist)
    ms_max = dist_max(dist, ms)
    value = N * args.steps * world / (ms_max / 1e3) / 1e9
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
    traffic = ncu_traffic_per_launch().get(dom_name)
    total_prof = sum(p[2] for p in prof)

    # end to end through the C ABI with host buffers
    state = ["RO", "ROVX", "ROVR", "RORVT", "ROE"]
    host = {n: prob.get(n) for n in state}
    h2d_step, d2h_step = lib.step_io_bytes()
    ne = max(1, args.steps // 2)
    dist_barrier(dist)
    t0 = time.perf_counter()
    for n in state:
        prob.set(n, host[n])
    for _ in range(ne):
        prob.step()
    out = {n: prob.get(n) for n in state}
    t1 = time.perf_counter()
    dist_barrier(dist)
    e2e_s = dist_max(dist, t1 - t0)
    state_bytes = sum(host[n].nbytes for n in state)
    e2e = {"value": N * ne * world / e2e_s / 1e9, "unit": METRIC,
           "h2d_bytes_per_step": (state_bytes + h2d_step * ne) / ne,
           "d2h_bytes_per_step": (state_bytes + d2h_step * ne) / ne,
           "steps": ne, "how": "per step mgpu_step() (graph launch, control word in, monitors out, sync); "
                               "flow state uploaded before and downloaded after from pageable host buffers"}

    # the plain FP32 path: the same workload with the long sums formed in the
    # reference's sequential REAL*4 order (REDUCE_ORDER=1, the parity mode)
    plain = None
    if os.environ.get("MGPU_BENCH_PLAIN", "1") != "0":
        cdp = build_case()
        cdp.ints["REDUCE_ORDER"] = 1
        pp = lib.Problem(cdp)
        pp.run(max(args.warmup, 3))
        npl = max(10, min(60, args.steps // 10))
        ms_pl = pp.bench_steps(npl, flush_l2=True)
        pp.close()
        v_pl = N * npl / (ms_pl / 1e3) / 1e9
        plain = {"value": v_pl, "unit": METRIC, "steps": npl, "ms_per_step": ms_pl / npl,
                 "chosen_over_plain": value / world / v_pl,
                 "how": "REDUCE_ORDER=1: multigrid, row-mean, mixing-plane and monitor sums in the reference's "
                        "sequential REAL*4 order; accuracy of both paths against the FP64 oracle is checked in "
                        "tests/test_gpu_parity.py (small stage, 1500 steps)"}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        rate, n, dt = cpu_oracle_rate(cd, float(os.environ.get("MGPU_CPU_SECONDS", "15")), 10 ** 6)
        cpu = {"value": rate, "unit": METRIC, "cores": 1, "kind": "port",
               "sample": f"{n} LOOP iterations of the same workload after 1 warm-up, serial C++ restatement of "
                         f"LOOP (oracle), {dt:.1f} s"}
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOADS[ARGS_WORKLOAD][1], "nodes": N, "l2": "flushed between timed steps",
                       "parallelism": f"replicas: one instance per GPU x{world}",
                       "reductions": "FP64 tree sums (REDUCE_ORDER=0)",
                       "autotune": {"tstep_threads_per_cta": {"ro_roe_pass": tuned[0], "momentum_pass": tuned[1]},
                                    "tstep_pass_ms": None if tune_ms is None else
                                    {p: dict(zip(("128", "192", "256", "512"), v)) for p, v in tune_ms.items()}}},
            "roofline": {"bound": "hbm", "kernel": dom_name, "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                         "alg_bytes_per_launch": alg_step / launches_step,
                         "avg_launch_ms": step_s * 1e3 / launches_step,
                         "alg_bytes_per_node_unit": bpn, "units_per_step": units,
                         "share_of_step": dom_ms / total_prof,
                         "step": {"alg_bytes_per_node_iter": B_ALG_STEP,
                                  "achieved": value / world * B_ALG_STEP, "frac": value / world * B_ALG_STEP / peak}},
            "plain_fp32": plain,
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
    return run_gpu(args, rank, world, local_rank)


if __name__ == "__main__":
    sys.exit(main())
