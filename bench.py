"""Benchmark of the explicit r-z step on GB300.

Workload (the metric of the reference's target): the axisymmetric blast at
4096 x 2048 cells (z in [-1,1], r in [0,1], gamma 5/3, CFL 0.4, rho=1, v=0,
p=10 inside radius 0.2, 0.1 outside; reflecting axis, outflow elsewhere) with
the exact-Godunov flux and minmod reconstruction.  A step is one time step
over the whole grid; the metric is cell-updates/s = N*M*steps / time.

Forms measured (each from the same initial state, warm-up steps first):
  fp64_godunov   plain FP64 path (the reference's solver; the oracle-comparable form)
  fp32_pvrs      FP32 form, Newton for p* from the acoustic (PVRS-type) start value
  fp32_learned   FP32 form, Newton from the learned start value (the headline)
  fp32_learned_skip  the same with skip_uniform = 1: tiles whose staged cells are
                 all bit-identical skip the face pass (identical results, checked
                 bit for bit against fp32_learned; not the headline)
  fp64_hll, fp32_hll  the HLL flux in FP64 and in the FP32 form
  fp32_hll_skip  fp32_hll with skip_uniform = 1 (uniform tiles skip the face
                 pass; face pairs of undisturbed gas skip the reconstruction),
                 checked bit for bit against fp32_hll
The FP32 forms report their density and pressure L1 error against the FP64
run after the same steps, and Newton statistics (mean/max iterations,
fallback rate).  The headline `value` is the form named in config.form.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun (N > 1) each rank advances an independent replica (the path
is not decomposed across GPUs); value is the sum over ranks of the work over
the slowest rank's time.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_Z, M_R = 4096, 2048   # overridable with --grid for profiling runs
PERSISTENT = 1          # FP32 kernel: 1 persistent tile kernel (bulk-tensor staging), 0 one CTA per tile, 2 strips
BYTES_PER_CELL = {"fp64": 64, "fp32": 32}   # one read + one write of 4 state values
REF_BUDGET_S = 150.0    # reference arm: seconds of timed host work
# DRAM bytes (read + write) per launch of the FP32 persistent kernel at
# 4096x2048 from the state at step 1000, from one ncu capture of
#   bench.py --steps 2 --warmup 1 --no-forms --no-stats --no-cpu --accuracy-steps 0 --batch-steps 0 [--form F]
# (dram__bytes_read.sum + dram__bytes_write.sum); the default grid only
MEASURED_TRAFFIC = {"fp32_learned": 134.40e6 + 94.28e6, "fp32_hll": 134.29e6 + 93.31e6}
MEASURED_TRAFFIC_SOURCE = ("a constant, not measured in this run: ncu dram__bytes_read.sum + dram__bytes_write.sum "
                           "of one launch (profiles/step_kernel_tma_fp32_learned_godunov_4096x2048.md, the capture "
                           "of the current kernel)")


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during a region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index, interval_ms=20):
        self.index = index
        self.interval_ms = interval_ms
        self.proc = None
        self.lines = []          # (host time, line)
        self.window = None       # (begin, end) host times of the timed region

    def start(self, ready_timeout=10.0):
        """Starts nvidia-smi and waits for its first sample, so that the
        timed region that follows is sampled from its beginning."""
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", str(self.interval_ms)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (FileNotFoundError, OSError):
            self.proc = None
            return
        t0 = time.perf_counter()
        while not self.lines and time.perf_counter() - t0 < ready_timeout:
            time.sleep(0.01)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))

    def begin(self):
        self.window = (time.perf_counter(), None)

    def end(self):
        self.window = (self.window[0], time.perf_counter())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        lines = self.lines
        if self.window and self.window[1] is not None:
            # the samples taken while the timed region ran (each sample
            # reports the state over the interval before it is printed)
            b, e = self.window
            inside = [x for x in lines if b <= x[0] <= e + self.interval_ms / 1e3]
            lines = inside if inside else lines
        for _, ln in lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for name, val in zip(names, parts[4:8]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm), "interval_ms": self.interval_ms}


# the measured forms: FP64 plain (the reference's solver), and the FP32 form
# started from the acoustic value or from the learned network, both at the
# Newton tolerance 1e-8 (clamped to 4 ulps of FP32)
# (the HLL pair is the precision form of the small config's flux at full
# size, timed for its own rate and %HBM)
# profiling builds (--phase-clocks): per form, the persistent kernel's SM
# cycles per phase
PHASES = None

FORMS = ("fp64_godunov", "fp32_pvrs", "fp32_learned", "fp32_learned_skip", "fp64_hll", "fp32_hll", "fp32_hll_skip")


def make_config(form):
    from asteriy_2d_gb300 import abi as A
    from asteriy_2d_gb300 import problems
    prec = A.PREC_FP64 if form.startswith("fp64") else A.PREC_FP32
    flux = A.FLUX_HLL if "_hll" in form else A.FLUX_GODUNOV
    cfg = problems.blast_config(N_Z, M_R, flux=flux, precision=prec)
    cfg.persistent = PERSISTENT
    if prec == A.PREC_FP32:
        cfg.riemann_tol = 1e-8
        cfg.guess = A.GUESS_MLP if form.startswith("fp32_learned") else A.GUESS_PVRS
        cfg.skip_uniform = 1 if form.endswith("_skip") else 0
    return cfg


def time_config(cfg, s0, u0, steps, warmup, torch):
    """Device-timed steps of one configuration from (s0, u0) at t = 0
    (CUDA events on the solver's stream).  Returns seconds."""
    from asteriy_2d_gb300 import solver
    stream = torch.cuda.Stream()
    with solver.Solver(cfg, stream=stream.cuda_stream) as S:
        S.set_state(s0, u0)
        S.step(warmup)
        S.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        S.step(steps, sync=False)
        e1.record(stream)
        S.synchronize()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1e3


def time_configs(warmup, torch):
    """The other configurations of the scope table, each timed from t = 0
    as its own run: C1, the blast at 256x128 with HLL + minmod in FP64 (the
    small case, 500 steps; launch-bound at this size), and C2, the
    wind-counterflow at 2048x1024 with HLLC + minmod (seeded density noise,
    the wind sphere held fixed) in FP64 and in the FP32 form."""
    from asteriy_2d_gb300 import abi as A
    from asteriy_2d_gb300 import problems, solver
    out = {}
    runs = [("C1_blast_256x128_hll_fp64", problems.blast_config(256, 128, flux=A.FLUX_HLL), "blast", 500)]
    for prec, tag in ((A.PREC_FP64, "fp64"), (A.PREC_FP32, "fp32")):
        runs.append((f"C2_wind_2048x1024_hllc_{tag}", problems.wind_config(2048, 1024, precision=prec), "wind",
                     200 if prec == A.PREC_FP64 else 1000))
    for name, cfg, setup, steps in runs:
        s0, u0 = solver.fill_blast(cfg) if setup == "blast" else solver.fill_wind(cfg)
        sec = time_config(cfg, s0, u0, steps, warmup, torch)
        out[name] = {"value": cfg.N * cfg.M * steps / sec, "unit": "cell-updates/s",
                     "ms_per_step": sec * 1e3 / steps, "steps": steps}
    return out


def learned_params(s0, u0):
    """Trained parameters of the start-value network: the committed ones
    (asteriy_2d_gb300/train_guess.py) or, when absent, a quick training on
    faces recorded from 200 FP64 steps of this workload."""
    from asteriy_2d_gb300 import learned
    path = os.path.join(ROOT, "asteriy_2d_gb300", "data", "guess_blast.npy")
    if os.path.exists(path):
        return np.load(path), "asteriy_2d_gb300/data/guess_blast.npy"
    rec, _ = learned.record_faces(make_config("fp64_godunov"), s0, u0, 200, every=20, capacity=1 << 24)
    params, _ = learned.train_guess(learned.sample_records(rec, 1 << 20), epochs=10, batch=16384)
    return params, "trained in this run on faces of 200 FP64 steps"


def phase_breakdown(phases):
    """Per form: each phase's share of the CTAs' cycles and its cycles per
    tile, from ast_get_phase_clocks counters."""
    out = {}
    for form, p in phases.items():
        names = ("arrival", "ghost", "faces", "queue", "update", "report")
        total = sum(p[k] for k in names)
        if not total or not p["tiles"]:
            continue
        out[form] = {"share": {k: round(p[k] / total, 4) for k in names},
                     "cycles_per_tile": {k: round(p[k] / p["tiles"], 1) for k in names},
                     "tiles": p["tiles"], "ctas": p["ctas"],
                     "note": "thread 0 of each CTA: SM cycles between the barriers that end each phase, summed over "
                             "CTAs, warm-up and timed steps"}
    return out


def time_form(form, start, steps, warmup, torch, params=None, stats_steps=0, sampler=None):
    """Device-timed steps of one form from the start state `start` = (s, u,
    (T_do, TT, step)): inputs resident in HBM, CUDA events on the solver's
    stream.  Returns (seconds, final s, final u, stats)."""
    from asteriy_2d_gb300 import solver
    s0, u0, clock = start
    cfg = make_config(form)
    stream = torch.cuda.Stream()
    with solver.Solver(cfg, stream=stream.cuda_stream) as S:
        if params is not None:
            S.set_mlp(params)
        S.set_state(s0, u0)
        S.set_clock(*clock)
        S.step(warmup)
        S.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        if sampler:
            sampler.begin()
        e0.record(stream)
        S.step(steps, sync=False)
        e1.record(stream)
        S.synchronize()
        torch.cuda.synchronize()
        if sampler:
            sampler.end()
        ms = e0.elapsed_time(e1)
        s, u = S.get_state()
        if PHASES is not None:
            # profiling build: this form's cycles per phase over warm-up and
            # timed steps (the counters start at zero with the solver)
            PHASES[form] = S.phase_clocks()
    st = None
    if stats_steps:
        # Newton statistics from a separate run with the counters on
        c = cfg.copy()
        c.collect_stats = 1
        with solver.Solver(c) as S:
            if params is not None:
                S.set_mlp(params)
            S.set_state(s0, u0)
            S.set_clock(*clock)
            S.step(warmup + stats_steps)
            st = S.stats()
    return ms / 1e3, s, u, st


def advance(form, s0, u0, nsteps, params=None):
    """The blast advanced nsteps from t = 0 with one form: (s, u, clock)."""
    from asteriy_2d_gb300 import solver
    with solver.Solver(make_config(form)) as S:
        if params is not None:
            S.set_mlp(params)
        S.set_state(s0, u0)
        S.step(nsteps)
        s, u = S.get_state()
        clock = S.clock()
    return s, u, clock


def axis_shock_z(s):
    """z of the largest density jump along the axis row (m = 0), z > 0."""
    rho = s[:N_Z, 0]
    jump = np.abs(np.diff(rho))
    h = N_Z // 2
    i = h + int(np.argmax(jump[h:]))
    dx = 2.0 / (N_Z - 1)
    return -1.0 + (i + 0.5) * dx


def _errs(r32, r64):
    d = np.abs(r32 - r64)
    return {"l1_rho": float(d[:, 0].sum() / np.abs(r64[:, 0]).sum()),
            "l1_p": float(d[:, 1].sum() / np.abs(r64[:, 1]).sum()),
            "linf_rho": float(d[:, 0].max() / np.abs(r64[:, 0]).max()),
            "linf_p": float(d[:, 1].max() / np.abs(r64[:, 1]).max())}


def _timed_steps(S, n, stream, torch):
    """n steps of solver S in one call, device-timed on its stream: seconds."""
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    S.step(n, sync=False)
    e1.record(stream)
    S.synchronize()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / 1e3


def run_from_t0(flux, nsteps, params, torch, fp32_forms):
    """The blast from t = 0 over nsteps steps: the FP64 run and the given
    FP32 forms ((name, guess) pairs), each form's average rate over the run
    (device-timed, one call of all its steps: the FP64 run over its first
    nsteps - 16 steps, after which it continues step by step), and each FP32
    form's error against the FP64 run at the same step count and at the same
    simulated time (the FP64 solution linearly interpolated in time to the
    FP32 run's final time: the runs' lagged time steps drift apart, which
    moves every shock by a fraction of a cell)."""
    from asteriy_2d_gb300 import abi as A
    from asteriy_2d_gb300 import problems, solver
    cells = N_Z * M_R
    cfg64 = problems.blast_config(N_Z, M_R, flux=flux, precision=A.PREC_FP64)
    s0, u0 = solver.fill_blast(cfg64)
    stream = torch.cuda.Stream()
    out, finals = {}, {}
    for name, guess in fp32_forms:
        cfg32 = problems.blast_config(N_Z, M_R, flux=flux, precision=A.PREC_FP32)
        if flux == A.FLUX_GODUNOV:
            cfg32.riemann_tol = 1e-8
            cfg32.guess = guess
        with solver.Solver(cfg32, stream=stream.cuda_stream) as S:
            if guess == A.GUESS_MLP:
                S.set_mlp(params)
            S.set_state(s0, u0)
            sec = _timed_steps(S, nsteps, stream, torch)
            finals[name] = (S.get_state()[0], S.clock()[1])
        out[name] = {"rate": cells * nsteps / sec, "ms_per_step": sec * 1e3 / nsteps}
    # FP64: nsteps - 16 steps in one timed call, then single steps to
    # nsteps + 8, keeping the states around the FP32 runs' final times
    k0 = nsteps - 16
    with solver.Solver(cfg64, stream=stream.cuda_stream) as S:
        S.set_state(s0, u0)
        sec = _timed_steps(S, k0, stream, torch)
        out["fp64"] = {"rate": cells * k0 / sec, "ms_per_step": sec * 1e3 / k0, "timed_steps": k0}
        hist = [(S.clock()[1], S.get_state()[0])]
        for _ in range(24):
            S.step(1)
            hist.append((S.clock()[1], S.get_state()[0]))
    r64, tt64 = hist[16][1], hist[16][0]
    out["fp64"]["tt"] = tt64
    out["fp64"]["axis_shock_z"] = axis_shock_z(r64)
    for name, (r32, tt32) in finals.items():
        res = out[name]
        res.update({"steps": nsteps, "same_step": _errs(r32, r64), "tt": tt32,
                    "tt_rel_drift": (tt32 - tt64) / tt64, "axis_shock_z": axis_shock_z(r32)})
        for (ta, sa), (tb, sb) in zip(hist[:-1], hist[1:]):
            if ta <= tt32 <= tb:
                w = (tt32 - ta) / (tb - ta) if tb > ta else 0.0
                res["same_time"] = _errs(r32, (1.0 - w) * sa + w * sb)
                break
    return out


def accuracy(nsteps, params, torch):
    """Error of the FP32 forms against the FP64 path after nsteps from t = 0,
    and every form's average rate over that run: the precision form (HLL +
    minmod) and, on the exact solver's problem (the learned form's run), the
    FP32 form from the acoustic start value and from the learned one."""
    from asteriy_2d_gb300 import abi as A
    from asteriy_2d_gb300 import problems, solver
    out = {"precision_hll": run_from_t0(A.FLUX_HLL, nsteps, None, torch, [("fp32_hll", A.GUESS_PVRS)]),
           "godunov": run_from_t0(A.FLUX_GODUNOV, nsteps, params, torch,
                                  [("fp32_pvrs", A.GUESS_PVRS), ("fp32_learned", A.GUESS_MLP)])}
    # the flow's own sensitivity: FP64 from an initial density perturbed by
    # 1e-12 relative, against the unperturbed FP64 run (HLL, nsteps)
    cfg64 = problems.blast_config(N_Z, M_R, flux=A.FLUX_HLL, precision=A.PREC_FP64)
    s0, u0 = solver.fill_blast(cfg64)
    sp = s0.copy()
    sp[:, 0] *= 1.0 + 1e-12 * np.random.default_rng(1).uniform(-1.0, 1.0, len(sp))
    with solver.Solver(cfg64) as S:
        S.set_state(s0, u0)
        S.step(nsteps)
        r64 = S.get_state()[0]
        S.set_state(sp, u0)
        S.set_clock(cfg64.dt_first, 0.0, 0)
        S.step(nsteps)
        rp = S.get_state()[0]
    d = np.abs(rp - r64)
    out["fp64_sensitivity_1e-12"] = {"steps": nsteps, "l1_rho": float(d[:, 0].sum() / np.abs(r64[:, 0]).sum()),
                                     "linf_rho": float(d[:, 0].max() / np.abs(r64[:, 0]).max())}
    return out


def time_e2e(form, start, steps, torch, params=None, mode="chain"):
    """Through the public API with host buffers: every step copies the state
    in from pinned host memory, steps once and writes the result back to
    pinned host memory (ping-pong between two pairs of host arrays).
    mode "chain": one ast_step_host_n call for all the steps (the copies in,
    the step and the copies out pipelined over bands of rows, and the bands
    of consecutive steps overlapping); "per_step": one ast_step_host call
    per step; "three_calls": ast_set_state, ast_step(1), ast_get_state."""
    from asteriy_2d_gb300 import solver
    s0, u0, clock = start
    cfg = make_config(form)
    K = cfg.N * cfg.M
    hs, hu, hs2, hu2 = (torch.empty((K, 2), dtype=torch.float64, pin_memory=True) for _ in range(4))
    lib = solver.load()
    with solver.Solver(cfg) as S:
        if params is not None:
            S.set_mlp(params)
        S.set_clock(*clock)
        bufs = [(hs, hu), (hs2, hu2)]

        def run(n):
            if mode == "chain":
                (a_s, a_u), (b_s, b_u) = bufs
                S.step_host_n(n, a_s.data_ptr(), a_u.data_ptr(), b_s.data_ptr(), b_u.data_ptr())
                return
            for _ in range(n):
                (a_s, a_u), (b_s, b_u) = bufs
                if mode == "per_step":
                    S.step_host(a_s.data_ptr(), a_u.data_ptr(), b_s.data_ptr(), b_u.data_ptr())
                else:
                    solver.check(lib.ast_set_state(S.h, a_s.data_ptr(), a_u.data_ptr(), 0), "set_state")
                    S.step(1, sync=False)
                    solver.check(lib.ast_get_state(S.h, b_s.data_ptr(), b_u.data_ptr(), 0), "get_state")
                bufs.reverse()
        hs.numpy()[:] = s0
        hu.numpy()[:] = u0
        run(1)   # warm-up (streams, events, graph-free launch path)
        hs.numpy()[:] = s0
        hu.numpy()[:] = u0
        bufs[:] = [(hs, hu), (hs2, hu2)]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        run(steps)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
    return dt, 2 * K * 16, 2 * K * 16


def batch_modes(torch, nprob=64, seed=64, steps=96, pre=16):
    """The batch's schedules side by side, each from the initial states after
    `pre` steps, CUDA events over `steps` steps: each class's problems alone
    with one CTA per 32x16 tile, with the persistent class kernel and with the
    persistent one-launch kernel; all problems as two launches (both
    schedules) and as one launch (modes 1 and 2).  ms per step."""
    from asteriy_2d_gb300 import abi as A
    from asteriy_2d_gb300 import solver
    probs = solver.problem_set(seed, nprob, A.PREC_FP32)
    init = [solver.problem_fill(p) for p in probs]

    def run(idx, sched=None, mixed=0):
        stream = torch.cuda.Stream()
        with solver.Batch([probs[i].cfg for i in idx], stream=stream.cuda_stream) as B:
            for k, i in enumerate(idx):
                B.set_state(k, *init[i])
            if mixed:
                B.set_mixed(mixed)
            else:
                for c in range(B.info()["launches_per_step"]):
                    B.set_schedule(c, sched)
            B.step(pre)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            B.step(steps, sync=False)
            e1.record(stream)
            B.synchronize()
            return round(e0.elapsed_time(e1) / steps, 4)

    out = {}
    for name, flux in (("hllc", A.FLUX_HLLC), ("godunov", A.FLUX_GODUNOV)):
        idx = [i for i, p in enumerate(probs) if p.cfg.flux == flux]
        out[name] = {"problems": len(idx), "cells": sum(probs[i].cfg.N * probs[i].cfg.M for i in idx),
                     "per_tile_32x16_ms": run(idx, sched=0), "persistent_ms": run(idx, sched=solver.PERSISTENT),
                     "one_launch_persistent_ms": run(idx, mixed=2)}
    idx = list(range(nprob))
    out["all"] = {"two_launches_per_tile_32x16_ms": run(idx, sched=0),
                  "two_launches_persistent_ms": run(idx, sched=solver.PERSISTENT),
                  "one_launch_per_tile_ms": run(idx, mixed=1), "one_launch_persistent_ms": run(idx, mixed=2)}
    out["note"] = "ms per step over %d steps after %d, from the seeded initial states" % (steps, pre)
    return out


def time_batch(steps, warmup, torch, nprob=64, seed=64, solo_steps=32, tune_at=200, mixed=None):
    """The batched form: the seeded set of nprob problems (ast_problem_set:
    128x64 .. 1024x512, blast or wind, HLLC or exact Godunov, gamma 5/3 or
    1.4, Mach 1.5-6), FP32, all advanced together by ast_batch_step.  The
    schedules are tuned after `tune_at` steps (the initial states are cheaper
    than the run's: the blasts have not spread yet), then timed with CUDA
    events over `steps` steps after `warmup`; the same problems
    stepped one solver after another (each its own graph) for solo_steps
    steps give the unbatched rate; every problem's density L1 error against
    the FP64 run of the same steps (an FP64 batch: bitwise the FP64 solo
    runs) is reported."""
    from asteriy_2d_gb300 import abi as A
    from asteriy_2d_gb300 import solver
    probs = solver.problem_set(seed, nprob, A.PREC_FP32)
    init = [solver.problem_fill(p) for p in probs]
    cells = sum(p.cfg.N * p.cfg.M for p in probs)
    stream = torch.cuda.Stream()
    with solver.Batch([p.cfg for p in probs], stream=stream.cuda_stream) as B:
        for i, (s0, u0) in enumerate(init):
            B.set_state(i, s0, u0)
        # schedule per class and one-launch mode, timed on the states after
        # tune_at steps (the tuner leaves the state and clocks as they were)
        B.step(tune_at)
        classes = B.autotune(10)
        if mixed is not None:
            # a one-launch mode forced over the tuner's choice (profiling)
            B.set_mixed(mixed)
        one_launch = B.mixed()
        info = B.info()
        B.step(warmup)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        # events between windows of whole 16-step graph blocks: the step's
        # cost as the run goes on (the tuner sees only the initial states)
        win = 16 * max(1, steps // 160)
        marks = []
        torch.cuda.synchronize()
        e0.record(stream)
        done = 0
        while done < steps:
            k = min(win, steps - done)
            B.step(k, sync=False)
            done += k
            ev = torch.cuda.Event(enable_timing=True)
            ev.record(stream)
            marks.append((done, ev))
        e1.record(stream)
        B.synchronize()
        torch.cuda.synchronize()
        sec = e0.elapsed_time(e1) / 1e3
        windows, prev, prev_ev = [], 0, e0
        for d, ev in marks:
            windows.append([prev, d, round(prev_ev.elapsed_time(ev) / (d - prev), 4)])
            prev, prev_ev = d, ev
        fp32 = [B.get_state(i)[0] for i in range(nprob)]
        tt32 = [B.clock(i)[1] for i in range(nprob)]
    # unbatched: one solver per problem, stepped in turn on one stream
    solos = []
    for p, (s0, u0) in zip(probs, init):
        S = solver.Solver(p.cfg, stream=stream.cuda_stream)
        S.set_state(s0, u0)
        S.step(16)   # captures its graph
        solos.append(S)
    torch.cuda.synchronize()
    e0.record(stream)
    for S in solos:
        S.step(solo_steps, sync=False)
    e1.record(stream)
    torch.cuda.synchronize()
    solo_sec = e0.elapsed_time(e1) / 1e3
    for S in solos:
        S.close()
    # FP64 runs of the same problems and steps
    cfg64 = []
    for p in probs:
        c = p.cfg.copy()
        c.precision = A.PREC_FP64
        cfg64.append(c)
    # at the same step count, and at the same simulated time (the FP64
    # density linearly interpolated in time to each FP32 problem's final
    # time, from single FP64 steps around it)
    def rel_l1(a, ref):
        return float(np.sum(np.abs(a - ref)) / np.sum(np.abs(ref)))
    l1, l1t, drift = [], [None] * nprob, []
    total = tune_at + warmup + steps
    with solver.Batch(cfg64) as B:
        for i, (s0, u0) in enumerate(init):
            B.set_state(i, s0, u0)
        B.step(total - 8)
        prev = [(B.clock(i)[1], B.get_state(i)[0][:, 0]) for i in range(nprob)]
        for k in range(16):
            B.step(1)
            for i in range(nprob):
                tb, rb = B.clock(i)[1], B.get_state(i)[0][:, 0]
                ta, ra = prev[i]
                if k == 7:
                    l1.append(rel_l1(fp32[i][:, 0], rb))
                    drift.append((tt32[i] - tb) / tb)
                if l1t[i] is None and ta <= tt32[i] <= tb:
                    w = (tt32[i] - ta) / (tb - ta) if tb > ta else 0.0
                    l1t[i] = rel_l1(fp32[i][:, 0], (1.0 - w) * ra + w * rb)
                prev[i] = (tb, rb)
    l1 = np.array(l1)
    found = np.array([v for v in l1t if v is not None])
    kinds = [("godunov" if p.cfg.flux == A.FLUX_GODUNOV else "hllc") + "/" +
             ("wind" if p.setup == A.SETUP_WIND else "blast") for p in probs]
    return {
        "value": cells * steps / sec, "unit": "cell-updates/s", "ms_per_step": sec * 1e3 / steps,
        "steps": steps, "warmup": warmup, "tuned_after_steps": tune_at, "problems": nprob, "seed": seed,
        "cells": cells,
        "tiles": info["tiles"], "launches_per_step": info["launches_per_step"],
        "classes": [{"flux": ["hll", "hllc", "godunov", "hllc_a"][c["flux"]], "problems": c["problems"],
                     "schedule": solver.SCHEDULES[c["schedule"]], "tile": "%dx%d" % c["tile"],
                     "tuner_ms": {name: round(m, 4) for name, m in zip(solver.SCHEDULES, c["ms_per_schedule"])}}
                    for c in classes],
        "one_launch": {"in_use": ["no", "a CTA per tile", "persistent"][one_launch[0]],
                       "tuner_ms": round(one_launch[1], 4),
                       "tuner_ms_per_class_launches": round(one_launch[2], 4),
                       "note": "every problem in one launch (32x16 tiles, each tile the code of its problem's "
                               "flux), a CTA per tile or the persistent kernel, against one launch per class; "
                               "tuner_ms is the faster one-launch mode's; the tuner keeps the fastest"},
        "ms_per_step_by_window": {"windows": windows,
                                  "note": "[first step, end step, ms per step] of the timed run, counted from "
                                          "the end of the warm-up; the tuner timed the states after "
                                          "tuned_after_steps steps"},
        "mix": {k: kinds.count(k) for k in sorted(set(kinds))},
        "solo_value": cells * solo_steps / solo_sec, "solo_steps": solo_steps,
        "l1_rho_vs_fp64": {"median": float(np.median(l1)), "max": float(l1.max()),
                           "above_1e-4": int(np.sum(l1 > 1e-4)),
                           "per_problem": [float("%.3g" % v) for v in l1]},
        "l1_rho_vs_fp64_same_time": {"median": float(np.median(found)) if found.size else None,
                                     "max": float(found.max()) if found.size else None,
                                     "above_1e-4": int(np.sum(found > 1e-4)), "problems": int(found.size),
                                     "tt_rel_drift_median": float(np.median(drift)),
                                     "tt_rel_drift_max_abs": float(np.max(np.abs(drift))),
                                     "note": "each FP32 problem against its FP64 run interpolated in time to the "
                                             "FP32 run's final time (problems whose time lies within 8 steps "
                                             "of the FP64 run's)"},
        "dtype": "f32",
    }


def cpu_baseline(cfg, s0, u0, nsteps, clock, where):
    """The reference's face functions compiled for the host (oracle/_ref) in
    the oracle's step loop, on all host threads; the oracle port if the
    reference build is absent."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as O
    nt = os.cpu_count() or 1
    T_do, TT, step = clock
    if O.have_ref():
        kind = "reference"
        fn = lambda: O.ref_run_composed(cfg, s0, u0, nsteps, nthreads=nt, T_do=T_do, TT=TT, step_no=step)  # noqa: E731
    else:
        kind = "port"
        fn = lambda: O.run(cfg, s0, u0, nsteps, T_do=T_do, TT=TT, step_no=step, nthreads=nt)  # noqa: E731
    t0 = time.perf_counter()
    fn()
    dt = time.perf_counter() - t0
    cells = cfg.N * cfg.M * nsteps
    return {"value": cells / dt, "unit": "cell-updates/s", "cores": nt, "kind": kind,
            "sample": f"{nsteps} step(s) of the full {cfg.N}x{cfg.M} grid from {where}, FP64"}


def blast_host(cfg, p_in=10.0, p_out=0.1, radius=0.2):
    """The blast's initial state by numpy, the values ast_fill_blast writes
    (the reference arm does not load the CUDA library)."""
    x = cfg.x_min + np.arange(cfg.N) * ((cfg.x_max - cfg.x_min) / (cfg.N - 1))
    y = (cfg.y_max / (2.0 * cfg.M)) + np.arange(cfg.M) * (cfg.y_max / cfg.M)
    dist = np.sqrt(x[None, :] * x[None, :] + y[:, None] * y[:, None])
    s = np.empty((cfg.M * cfg.N, 2))
    s[:, 0] = 1.0
    s[:, 1] = np.where(dist < radius, p_in, p_out).reshape(-1)
    return s, np.zeros((cfg.M * cfg.N, 2))


def blast_host_advanced(cfg, nsteps, run, margin=64, radius=0.2):
    """The blast advanced nsteps steps from t = 0 on the host: `run(sub, s, u,
    n)` (the reference's functions or the oracle port) steps only the part of
    the grid the solution can have reached, and the rest keeps the ambient
    state.  That part is the half z >= 0 (the blast is symmetric about z = 0,
    the face between the two middle columns, which a reflecting side
    reproduces) and the rows and columns within the blast radius plus the
    distance a wave travels in nsteps steps (at most cfl cells per step)
    plus `margin` cells.  The sub-grid keeps the cell size and positions of
    the full grid (its dx may differ from the full grid's in the last bit).
    Returns (s, u, (T_do, TT, step))."""
    from asteriy_2d_gb300 import abi as A
    N, M = cfg.N, cfg.M
    assert N % 2 == 0 and cfg.x_min == -cfg.x_max
    dx = (cfg.x_max - cfg.x_min) / (N - 1)
    dy = cfg.y_max / M
    reach = cfg.cfl * nsteps + margin
    nz = min(N // 2, int(np.ceil(radius / dx + reach)))
    mr = min(M, int(np.ceil(radius / dy + reach)))
    s, u = blast_host(cfg)
    if nsteps == 0:
        return s, u, (cfg.dt_first, 0.0, 0)
    sub = cfg.copy()
    sub.N, sub.M = nz, mr
    sub.x_min = cfg.x_min + (N // 2) * dx
    sub.x_max = cfg.x_min + (N // 2 + nz - 1) * dx
    sub.y_max = cfg.y_max * mr / M
    A.set_bc(sub, A.Z_LO, A.BC_REFLECT)
    g = s.reshape(M, N, 2)
    h = u.reshape(M, N, 2)
    ss = np.ascontiguousarray(g[:mr, N // 2:N // 2 + nz]).reshape(-1, 2)
    us = np.ascontiguousarray(h[:mr, N // 2:N // 2 + nz]).reshape(-1, 2)
    ss, us, T_do, TT, step, _ = run(sub, ss, us, nsteps)
    ss, us = ss.reshape(mr, nz, 2), us.reshape(mr, nz, 2)
    g[:mr, N // 2:N // 2 + nz] = ss
    h[:mr, N // 2:N // 2 + nz] = us
    g[:mr, N // 2 - nz:N // 2] = ss[:, ::-1]
    h[:mr, N // 2 - nz:N // 2] = us[:, ::-1] * np.array([-1.0, 1.0])
    return s, u, (T_do, TT, step)


def reduce_max(value, torch):
    """The largest of the ranks' values, on every rank (the value itself
    without a process group): the slowest rank's time."""
    if not (torch.distributed.is_available() and torch.distributed.is_initialized()):
        return value
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return t.item()


def job_rate(ws, units_per_rank, sec):
    """Whole-job throughput: the units all ranks processed (each rank an
    independent replica of the same work) over the slowest rank's time."""
    return ws * units_per_rank / sec


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def shared_config(args):
    """The workload, identical in both arms' lines."""
    return {"workload": f"blast {N_Z}x{M_R}, exact Godunov + minmod, axisymmetric, CFL 0.4",
            "start_step": args.start_step,
            "l2": "state larger than L2 (ping-pong of 2x134 MB in FP32, 2x268 MB in FP64)"}


def reference_arm(args):
    """The reference's own functions compiled for the host (oracle/_ref; the
    oracle port when they are absent) on all host threads, FP64, from the
    same start as the GPU arm: the blast advanced args.start_step steps,
    computed here on the host (blast_host_advanced), so that this process
    never loads the CUDA library.  One full-grid step first (warm-up, and
    the time of a full step), then the remaining warm-up steps and the
    timed steps on a band of the grid's first rows (the blast's centre and
    the axis, all columns) sized so the timed steps take about REF_BUDGET_S
    seconds, or the full grid when that fits."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as O
    nt = os.cpu_count() or 1
    kind = "reference" if O.have_ref() else "port"

    def run(c, s, u, n, clock=None):
        T_do, TT, step = clock if clock else (None, 0.0, 0)
        if kind == "reference":
            return O.ref_run_composed(c, s, u, n, nthreads=nt, T_do=T_do, TT=TT, step_no=step)
        return O.run(c, s, u, n, T_do=T_do, TT=TT, step_no=step, nthreads=nt)

    cfg = make_config("fp64_godunov")
    t0 = time.perf_counter()
    s0, u0, clock = blast_host_advanced(cfg, args.start_step, run)
    t_prep = time.perf_counter() - t0
    t0 = time.perf_counter()
    s1, u1, T_do, TT, step, _ = run(cfg, s0, u0, 1, clock)
    t_full = time.perf_counter() - t0
    rows = cfg.M
    if args.steps * t_full > REF_BUDGET_S:
        rows = max(16, int(cfg.M * REF_BUDGET_S / (args.steps * t_full)))
    band = cfg.copy()
    band.M = rows
    band.y_max = cfg.y_max * rows / cfg.M
    sb, ub = s1[:rows * cfg.N], u1[:rows * cfg.N]
    bclock = (T_do, TT, step)
    if args.warmup > 1:
        sb, ub, T_do, TT, step, _ = run(band, sb, ub, args.warmup - 1, bclock)
        bclock = (T_do, TT, step)
    t0 = time.perf_counter()
    run(band, sb, ub, args.steps, bclock)
    dt = time.perf_counter() - t0
    v = band.N * band.M * args.steps / dt
    sample = (f"{args.steps} steps of rows 0..{rows - 1} of the {N_Z}x{M_R} grid ({N_Z}x{rows} cells per step) "
              f"from the blast advanced {args.start_step} steps (computed on the host by the same functions in "
              f"{t_prep:.0f} s on the part of the grid the blast can reach), after {args.warmup} warm-up "
              f"step(s), the first on the full grid ({t_full:.2f} s)")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "cell-updates/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": dt * 1e3 / args.steps, "higher_is_better": True, "dtype": "f64",
            "data": "synthetic", "scaling": "weak", "vs_baseline": None,
            "config": shared_config(args), "form": "fp64_godunov", "parallelism": "host threads",
            "cpu_baseline": {"value": v, "unit": "cell-updates/s", "cores": nt, "kind": kind, "sample": sample},
            "e2e": {"value": v, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


METRIC = "cell-updates/s at 4096x2048 (exact Godunov + minmod)"


def newton_summary(st):
    return {"mean_iters": st["newton_iters"] / st["newton_calls"], "max_iters": st["newton_max_iters"],
            "fallback_rate": st["mlp_fallback"] / max(1, st["strong_calls"]), "gated_faces": st["strong_calls"],
            "gated_mean_iters": st["strong_iters"] / max(1, st["strong_calls"])}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--form", default="fp32_learned", choices=list(FORMS))
    ap.add_argument("--no-stats", action="store_true", help="skip the Newton-statistics runs")
    ap.add_argument("--no-cpu", action="store_true", help="skip the cpu_baseline leg")
    ap.add_argument("--no-forms", action="store_true", help="time only --form")
    ap.add_argument("--grid", default=None, help="NxM instead of 4096x2048 (profiling runs)")
    ap.add_argument("--start-step", type=int, default=1000, help="timed window starts at this step of the run")
    ap.add_argument("--accuracy-steps", type=int, default=2000,
                    help="whole runs from t = 0 of this many steps: rates and FP32 error vs FP64 (0: skip)")
    ap.add_argument("--batch-steps", type=int, default=1000, help="steps of the 64-problem batch (0: skip)")
    ap.add_argument("--per-tile", action="store_true", help="FP32 forms with one CTA per tile, not the persistent kernel")
    ap.add_argument("--fp32-kernel", type=int, default=1, choices=[0, 1, 2],
                    help="FP32 step kernel: 1 persistent tile kernel, 0 one CTA per tile, 2 strip kernel")
    ap.add_argument("--batch-modes", action="store_true",
                    help="time the batch's schedules and one-launch modes side by side")
    ap.add_argument("--batch-mixed", type=int, default=None, choices=[0, 1, 2],
                    help="force the batch leg's one-launch mode (0 two launches, 1 a CTA per tile, 2 persistent)")
    ap.add_argument("--phase-clocks", action="store_true",
                    help="report the persistent kernel's cycles per phase (library built with AST_PHASE_CLOCKS=1)")
    args = ap.parse_args()
    global N_Z, M_R, PERSISTENT, PHASES
    if args.phase_clocks:
        PHASES = {}
    PERSISTENT = 0 if args.per_tile else args.fp32_kernel
    if args.grid:
        N_Z, M_R = (int(v) for v in args.grid.lower().split("x"))
    ws, rank, local = dist_setup()

    if args.impl == "reference":
        if rank != 0:
            return 0
        return reference_arm(args)

    import torch
    from asteriy_2d_gb300 import solver
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    cfg = make_config(args.form)
    s0, u0 = solver.fill_blast(cfg)
    cells = cfg.N * cfg.M
    params, params_src = (None, None)
    if any(f.startswith("fp32_learned") for f in ((args.form,) if args.no_forms else FORMS)) or args.accuracy_steps:
        params, params_src = learned_params(s0, u0)
    # the timing window starts mid-run: the blast advanced start_step steps
    # from t = 0 by the FP64 path (the reference arm computes the same start
    # with the reference's functions on the host), the same start for all
    # forms
    start = advance("fp64_godunov", s0, u0, args.start_step) if args.start_step else (s0, u0, (cfg.dt_first, 0.0, 0))

    # side-by-side forms (same start state, same step count); the headline
    # form is timed last, under the clock sampler and the rank barrier
    forms, finals = {}, {}
    for form in FORMS:
        if form == args.form or args.no_forms:
            continue
        sec, s, u, st = time_form(form, start, args.steps, args.warmup, torch,
                                  params if form.startswith("fp32_learned") else None,
                                  stats_steps=0 if args.no_stats else 5)
        forms[form] = {"value": cells * args.steps / sec, "ms_per_step": sec * 1e3 / args.steps}
        pf = "fp64" if form.startswith("fp64") else "fp32"
        forms[form]["hbm_frac"] = BYTES_PER_CELL[pf] * cells / (sec / args.steps) / 1e9 / peaks()[0]
        finals[form] = s
        if st and st["newton_calls"]:
            forms[form]["newton"] = newton_summary(st)
    if ws > 1:
        torch.distributed.barrier()
    sampler = ClockSampler(local)
    sampler.start()
    sec, s, u, st = time_form(args.form, start, args.steps, args.warmup, torch,
                              params if args.form.startswith("fp32_learned") else None,
                              stats_steps=0 if args.no_stats else 5, sampler=sampler)
    clocks = sampler.stop()
    sec = reduce_max(sec, torch)
    value = job_rate(ws, cells * args.steps, sec)
    forms[args.form] = {"value": cells * args.steps / sec, "ms_per_step": sec * 1e3 / args.steps}
    finals[args.form] = s
    if st and st["newton_calls"]:
        forms[args.form]["newton"] = newton_summary(st)
    # density / pressure L1 error of the FP32 forms against the FP64 run over
    # the timed window (same start, same steps)
    for ref_form, pair in (("fp64_godunov", ("fp32_pvrs", "fp32_learned", "fp32_learned_skip")),
                           ("fp64_hll", ("fp32_hll", "fp32_hll_skip"))):
        if ref_form not in finals:
            continue
        ref = finals[ref_form]
        for form, sf in finals.items():
            if form not in pair:
                continue
            forms[form]["l1_rho_vs_fp64"] = float(np.sum(np.abs(sf[:, 0] - ref[:, 0])) / np.sum(np.abs(ref[:, 0])))
            forms[form]["l1_p_vs_fp64"] = float(np.sum(np.abs(sf[:, 1] - ref[:, 1])) / np.sum(np.abs(ref[:, 1])))
    if "fp64_godunov" in forms and args.form != "fp64_godunov":
        forms[args.form]["speedup_vs_fp64"] = forms[args.form]["value"] / forms["fp64_godunov"]["value"]
    if "fp32_pvrs" in forms and args.form == "fp32_learned":
        forms["fp32_learned"]["speedup_vs_fp32_pvrs"] = forms["fp32_learned"]["value"] / forms["fp32_pvrs"]["value"]

    # the host-array legs: at least 10 steps per timed call (one call of a
    # few milliseconds is at the mercy of a single host hiccup), the median
    # of three calls
    e2e_steps = max(10, min(args.steps, 50))
    for skip_form, plain in (("fp32_learned_skip", "fp32_learned"), ("fp32_hll_skip", "fp32_hll")):
        if skip_form in finals and plain in finals:
            forms[skip_form]["bitwise_equal_to_" + plain] = bool(np.array_equal(finals[skip_form], finals[plain]))
    eparams = params if args.form.startswith("fp32_learned") else None
    def median_e2e(mode):
        runs = [time_e2e(args.form, start, e2e_steps, torch, eparams, mode=mode) for _ in range(3)]
        return sorted(r[0] for r in runs)[1], runs[0][1], runs[0][2]

    esec, bi, bo = median_e2e("chain")
    esec1, _, _ = median_e2e("per_step")
    esec3, _, _ = median_e2e("three_calls")
    hbm, src = peaks()
    prec = "fp64" if args.form.startswith("fp64") else "fp32"
    achieved = BYTES_PER_CELL[prec] * cells / (sec / args.steps) / 1e9
    traffic = MEASURED_TRAFFIC.get(args.form) if (N_Z, M_R) == (4096, 2048) and PERSISTENT == 1 else None
    line = {
        "metric": METRIC,
        "value": value, "unit": "cell-updates/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": sec * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if prec == "fp64" else "f32", "data": "synthetic",
        "config": shared_config(args),
        "form": args.form, "parallelism": "replicas" if ws > 1 else "single GPU",
        "fp32_kernel": {0: "one CTA per tile", 1: "persistent, bulk-tensor staged", 2: "strips swept by warps"}[PERSISTENT],
        "mlp_params": params_src,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "peak_source": src, "traffic": traffic,
                     "traffic_source": (MEASURED_TRAFFIC_SOURCE if traffic is not None else None),
                     "note": "algorithmic bytes = %d B/cell-update (one state read + one write)" % BYTES_PER_CELL[prec]},
        "forms": forms,
        "e2e": {"value": cells * e2e_steps / esec, "unit": "cell-updates/s", "h2d_bytes_per_step": bi,
                "d2h_bytes_per_step": bo,
                "steps": e2e_steps,
                "note": "the median of three timed calls; one ast_step_host_n call for all the steps; every step "
                        "copies its whole input in from pinned host arrays and its whole result out to pinned host "
                        "arrays (pipelined over 4 bands of rows, the bands of consecutive steps overlapping)",
                "per_step": {"value": cells * e2e_steps / esec1, "unit": "cell-updates/s",
                             "note": "one ast_step_host call per step (16 bands)"},
                "three_calls": {"value": cells * e2e_steps / esec3, "unit": "cell-updates/s",
                                "note": "per step: ast_set_state from pinned host, ast_step(1), "
                                        "ast_get_state to pinned host"}},
        "gpu_launches": args.steps,
        "clocks": clocks,
    }
    if rank == 0 and not args.no_forms:
        line["configs"] = time_configs(args.warmup, torch)
    if PHASES:
        line["phase_clocks"] = phase_breakdown(PHASES)
    if rank == 0 and args.batch_steps:
        line["batch"] = time_batch(args.batch_steps, args.warmup, torch, mixed=args.batch_mixed)
        line["gpu_launches_batch_step"] = line["batch"]["launches_per_step"]
    if rank == 0 and args.batch_modes:
        line["batch_modes"] = batch_modes(torch)
    if rank == 0 and args.accuracy_steps:
        acc = accuracy(args.accuracy_steps, params, torch)
        line["accuracy_vs_fp64"] = acc
        g = acc["godunov"]
        line["run_average"] = {
            "steps": args.accuracy_steps, "unit": "cell-updates/s",
            "fp32_learned": g["fp32_learned"]["rate"], "fp32_pvrs": g["fp32_pvrs"]["rate"],
            "fp64_godunov": g["fp64"]["rate"],
            "fp32_learned_over_fp64": g["fp32_learned"]["rate"] / g["fp64"]["rate"],
            "note": "the whole run of the learned form's workload from t = 0, one timed call per form (FP64 over "
                    "its first %d steps)" % (args.accuracy_steps - 16)}
    if rank == 0 and not args.no_cpu:
        cb = cpu_baseline(make_config("fp64_godunov"), start[0], start[1], 1, start[2],
                          where=f"the blast advanced {args.start_step} steps")
        line["cpu_baseline"] = cb
        if "fp64_godunov" in forms:
            # the same-precision comparison: the FP64 GPU path against the
            # reference's functions on the host cores, same state, FP64
            line["fp64_vs_cpu_reference"] = {"gpu_fp64": forms["fp64_godunov"]["value"], "cpu_fp64": cb["value"],
                                             "ratio": forms["fp64_godunov"]["value"] / cb["value"]}
    if rank == 0:
        print(json.dumps(line))
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
