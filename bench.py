"""Benchmark of the TVDLF/Hancock path on GB300.

Workload (one "step" = one VAC time step, i.e. three split sweeps of the
twostep Hancock/TVDLF scheme): 3-D ideal MHD, 256^3 periodic unit cube,
woodward limiter, gamma=5/3, divbfix (Powell), courantpar=0.8, seeded
random-mode initial state (rho, v and a divergence-free B from 8 Fourier
modes each, uniform low-beta p=0.05).  The state (8 FP32 fields x 256^3 =
537 MB, 1.07 GB in FP64) is larger than the 129 MB L2, so no flush is needed
between steps.

Default: mixed precision (FP32 state, double-precision pressure recovery).
The same run in plain FP64 is measured alongside, and the mixed result is
compared with it (relative L1 / Linf per variable).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Under torchrun (N>1) every rank advances its own independent solve (replicas
only: the path has no cross-GPU exchange); value = all cells updated by all
ranks / max-over-ranks time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "MHD TVDLF cell-updates/s on 1 GB300, mixed vs FP64 (L1 err); served p50/p99"
UNIT = "cell-updates/s"
N = 256
NW = 8


def workload_config(prec_name):
    mb = NW * 4 * N ** 3 / 1e6
    return {"workload": "3D ideal MHD TVDLF+woodward %d^3 periodic, random modes "
                        "(seeded), 100-step run timed per step" % N,
            "grid": [N, N, N], "nw": NW, "limiter": "woodward",
            "precision": prec_name,
            "l2": "state > L2 (%.0f MB FP32), no flush needed" % mb if mb > 129
                  else "state fits L2 (%.0f MB FP32)" % mb}


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.p = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        time.sleep(0.2)
        self.rows = []
        if self.p:
            self.p.terminate()
            out, _ = self.p.communicate(timeout=5)
            for ln in out.strip().splitlines():
                f = [x.strip() for x in ln.split(",")]
                if len(f) >= 7:
                    self.rows.append(f)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for n, v in zip(names, r[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    lrank = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if os.environ.get("VACGPU_BENCH_GLOO") is None
                                else "gloo")
    return ws, rank, lrank


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(ws, v):
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job(ws, units_per_rank, seconds):
    """Replicas: every rank advanced units_per_rank cell-updates in its own
    seconds; the job's rate is all ranks' units over the slowest rank."""
    el = max_over_ranks(ws, seconds)
    return units_per_rank * ws / el, el


def make_params(snap, prec):
    from vac_gb300 import inistate
    return inistate.params_for(snap, limiter="woodward", bc="periodic", precision=prec)


def cpu_sample(snap, steps, threads):
    """The FP64 oracle port on the host cores (OpenMP, `threads`)."""
    os.environ["OMP_NUM_THREADS"] = str(threads)
    from oracle.oracle import Oracle
    p = make_params(snap, 0)
    o = Oracle(p, snap.x, snap.w)
    o.step(1)  # first step includes the cell-centred CFL pass; not timed
    t0 = time.perf_counter()
    o.step(steps)
    dt = time.perf_counter() - t0
    return N ** 3 * steps / dt, dt


def cpu_serial_ot200():
    """Orszag-Tang 200^2 in full (FP64, minmod, 200 steps) by the
    FP64 oracle port on one core: VAC itself is serial.  Runs in a child
    process started with OMP_NUM_THREADS=1 (the OpenMP runtime reads it
    once per process)."""
    from oracle.oracle import Oracle
    from vac_gb300 import abi, inistate
    snap = inistate.orszag_tang(200)
    p = inistate.params_for(snap, limiter="minmod", bc="periodic", precision=abi.PREC_FP64)
    o = Oracle(p, snap.x, snap.w)
    t0 = time.perf_counter()
    o.step(200)
    el = time.perf_counter() - t0
    return {"value": 200 * 200 * 200 / el, "seconds": el}


def cpu_serial_subprocess():
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run([sys.executable, os.path.abspath(__file__), "--cpu-serial-only"],
                       capture_output=True, text=True, env=env, timeout=600)
    if r.returncode != 0:
        return {"unavailable": r.stderr.strip().splitlines()[-1] if r.stderr else "failed"}
    d = json.loads(r.stdout.strip().splitlines()[-1])
    return {"value": d["value"], "unit": UNIT, "cores": 1, "kind": "port",
            "sample": "Orszag-Tang 200^2 in full: FP64, minmod, 200 steps, "
                      "FP64 oracle port on 1 core, %.1f s (VAC is serial)" % d["seconds"]}


def sweep_traffic(ncell):
    """DRAM bytes (read + write) of one fused-sweep launch at the bench's
    256^3 size, from the committed ncu record of that launch
    (profiles/k_sweep_pair_mhd_256.md, mean of the x, y and z sweeps);
    (None, reason) if the record is absent."""
    f = os.path.join(ROOT, "profiles", "k_sweep_pair_mhd_256.md")
    if os.path.exists(f):
        for ln in open(f):
            if ln.startswith("dram_bytes_per_launch_256="):
                v = float(ln.split("=")[1])
                return v * ncell / 256 ** 3, ("ncu dram__bytes_read.sum + dram__bytes_write.sum "
                                              "of 256^3 launches, profiles/k_sweep_pair_mhd_256.md")
    return None, "no committed 256^3 ncu record"


def run_batched(args):
    """The batched workload: 64 2-D gamma=1.4 Riemann problems, sides log-uniform in
    [64, 1024], outflow, minmod, mixed precision; all grids advance 50 steps
    in one replay of a CUDA graph of batched persistent-kernel launches."""
    import torch
    from vac_gb300 import inistate
    from vac_gb300.engine import Batch
    grids = inistate.riemann_batch(n=64, seed=0)
    cells = sum(int(np.prod([g[0].nx[d] for d in range(2)])) for g in grids)
    b = Batch(grids)
    ctas, order, rows, one, ms = b.tune()
    b.step(50)  # capture + first replay
    torch.cuda.synchronize()
    if args.profile_range:
        torch.cuda.profiler.start()
    t0 = time.perf_counter()
    b.step(50)
    el = time.perf_counter() - t0
    if args.profile_range:
        torch.cuda.profiler.stop()
    one = b.tune()[3]  # 2: the one launch was captured into a CUDA graph
    b.close()
    return {"workload": "64 grids 2D HD Riemann, sides log-uniform [64,1024] (seeded), "
                        "cont, minmod, mixed, 50 steps per grid in one call (graph replay "
                        "or one cooperative launch, as tuned)",
            "grids": 64, "cells": cells, "steps": 50, "seconds": el,
            "value": cells * 50 / el, "unit": UNIT,
            "tuned": {"persistent_ctas": ctas, "order": ["round-robin", "grid-major"][order],
                      "rows_per_item": rows, "one_launch": one, "trial_ms": ms}}


def _errors(wm, w64):
    """Per variable: relative L1 sum|a-b|/sum|b| and relative Linf
    max|a-b|/max|b| of the mixed state against the FP64 state."""
    l1, linf = [], []
    for i in range(w64.shape[0]):
        d = np.abs(wm[i] - w64[i])
        l1.append(float(d.sum() / max(np.abs(w64[i]).sum(), 1e-300)))
        linf.append(float(d.max() / max(np.abs(w64[i]).max(), 1e-300)))
    return l1, linf


def _physical(w, gamma, mhd):
    """Minimum density and thermal pressure of an FP64 state."""
    nd = w.shape[0] - 2 if not mhd else (w.shape[0] - 2) // 2
    rho = w[0]
    m2 = sum(w[1 + c] ** 2 for c in range(nd))
    b2 = sum(w[2 + nd + c] ** 2 for c in range(nd)) if mhd else 0.0
    p = (gamma - 1.0) * (w[1 + nd] - 0.5 * m2 / rho - 0.5 * b2)
    return {"min_rho": float(rho.min()), "min_p": float(p.min())}


def _fresh_timed(params, snap, k, stream, warm):
    """A new engine on the seeded state: `warm` untimed steps (graph capture,
    z-chunk tuning), the state uploaded again (it=0, t=0), then k steps timed
    with CUDA events on its stream.  Returns (seconds, state after k steps)."""
    from vac_gb300.engine import Engine
    e = Engine(params, snap.x, snap.w)
    e.set_stream(stream.cuda_stream)
    if warm:
        e.step(warm)
        e.upload(snap.w)
    el = _timed_steps(e, k, stream)
    w = e.state()
    e.close()
    return el, w


def fp64_per_cell_update(key):
    """FP64 operations (key fp64_flops_per_cell_update, DFMA = 2) or FP64
    pipe instructions (fp64_inst_per_cell_update) per cell-update of the
    plain path (the 256^3 3-D MHD step), from the committed ncu record of
    its FP64 instruction counts (profiles/fp64_step_mhd_128.md); None if
    absent."""
    f = os.path.join(ROOT, "profiles", "fp64_step_mhd_128.md")
    if os.path.exists(f):
        for ln in open(f):
            if ln.startswith(key + "="):
                return float(ln.split("=")[1])
    return None


def run_fp64_c2(args, snap, stream, mixed_value):
    """The 256^3 3-D MHD run in plain FP64, and the mixed path's error against it: both
    precisions advance exactly --acc-steps (the run's 100) steps from the
    same seeded state; the FP64 run is timed over those steps.  The FP64
    path's own roofline: FP64 FLOP/s against the FP64 pipe's measured
    throughput, and its HBM fraction."""
    from vac_gb300 import abi
    from vac_gb300.engine import measure_fp64_peak
    k = args.acc_steps
    ncell = N ** 3
    el64, w64 = _fresh_timed(make_params(snap, abi.PREC_FP64), snap, k, stream, 1)
    _, wm = _fresh_timed(make_params(snap, abi.PREC_MIXED), snap, k, stream, 3)
    l1, linf = _errors(wm, w64)
    v64 = ncell * k / el64
    peak = measure_fp64_peak(stream.cuda_stream)
    fpc = fp64_per_cell_update("fp64_flops_per_cell_update")
    ipc = fp64_per_cell_update("fp64_inst_per_cell_update")
    hbm = _hbm_peak()
    roof = {"bound": "fp64", "unit": "TFLOP/s", "peak": peak / 1e12,
            "peak_source": "measured: vacgpu_measure_fp64_peak (DFMA chains on every SM, "
                           "CUDA events)",
            "flops_per_cell_update": fpc,
            "flops_source": "ncu FP64 instruction counts of one step "
                            "(profiles/fp64_step_mhd_128.md)",
            "hbm_frac": 2 * 3 * NW * 8 * v64 / (hbm * 1e9),
            "hbm_alg_bytes_per_cell_update": 2 * 3 * NW * 8}
    if fpc:
        roof["achieved"] = fpc * v64 / 1e12
        roof["frac"] = fpc * v64 / peak
    if ipc:
        # DADD and DMUL occupy the pipe like a DFMA: instruction rate against
        # the DFMA rate (half the flop peak)
        roof["inst_per_cell_update"] = ipc
        roof["pipe_frac"] = ipc * v64 / (peak / 2)
    return {"value": v64, "unit": UNIT, "ms_per_step": el64 / k * 1e3, "steps": k,
            "mixed_over_fp64": mixed_value / v64,
            "steps_compared": k, "rel_l1_mixed_vs_fp64": l1, "rel_linf_mixed_vs_fp64": linf,
            "max_rel_l1": max(l1),
            "fp64_state_after_steps": _physical(w64, float(snap.eqpar[0]), True),
            "roofline": roof}


def _hbm_peak():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"]
    except Exception:
        return 6800.0


def _timed_steps(eng, k, stream):
    """k steps on the engine's stream between CUDA events; seconds."""
    import torch
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    eng.step(k)
    b.record(stream)
    torch.cuda.synchronize()
    return a.elapsed_time(b) / 1e3


def run_plain(args):
    """The plain FP64 method, 2-D ideal MHD Orszag-Tang on
    200^2 periodic cells, minmod, 200 steps (state resident, 2 MB: an L2
    resident latency case, not a roofline case), with the FP64 oracle port
    on the host cores timed on the same run."""
    import torch
    from vac_gb300 import abi, inistate
    from vac_gb300.engine import Engine
    snap = inistate.orszag_tang(200)
    p = inistate.params_for(snap, limiter="minmod", bc="periodic", precision=abi.PREC_FP64)
    stream = torch.cuda.Stream()
    e = Engine(p, snap.x, snap.w)
    e.set_stream(stream.cuda_stream)
    e.step(3)
    e.upload(snap.w)
    el = _timed_steps(e, 200, stream)
    e.close()
    out = {"workload": "2D ideal MHD Orszag-Tang 200^2 periodic, minmod, FP64, 200 steps",
           "steps": 200, "seconds": el, "ms_per_step": el / 200 * 1e3,
           "value": 200 * 200 * 200 / el, "unit": UNIT}
    if args.cpu_steps > 0:
        os.environ["OMP_NUM_THREADS"] = str(os.cpu_count() or 1)
        from oracle.oracle import Oracle
        o = Oracle(p, snap.x, snap.w)
        t0 = time.perf_counter()
        o.step(200)
        ct = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": 200 * 200 * 200 / ct, "unit": UNIT,
                               "cores": os.cpu_count() or 1, "kind": "port",
                               "sample": "the same 200 steps, FP64 oracle port (OpenMP)"}
    return out


def run_blast(args):
    """3-D ideal MHD blast on 512^3 cells, outflow ('cont'),
    woodward, B=(1,1,0)/sqrt2, p from 10 to 0.1 across r=0.1.  Mixed and
    FP64 each advance --blast-steps (the run's 100) steps from the same
    initial state, timed over those steps; the mixed state's relative L1
    and Linf per variable against the FP64 state after them."""
    from vac_gb300 import abi, inistate
    import torch
    n = args.blast_side
    k = args.blast_steps
    snap = inistate.blast_3d(n)
    ncell = n ** 3
    stream = torch.cuda.Stream()
    pm = inistate.params_for(snap, limiter="woodward", bc="cont", precision=abi.PREC_MIXED)
    p64 = inistate.params_for(snap, limiter="woodward", bc="cont", precision=abi.PREC_FP64)
    elm, wm = _fresh_timed(pm, snap, k, stream, 3)
    el64, w64 = _fresh_timed(p64, snap, k, stream, 1)
    l1, linf = _errors(wm, w64)
    del wm
    out = {"workload": "3D ideal MHD blast %d^3, cont, woodward, %d steps per precision "
                       "from the same initial state" % (n, k),
           "mixed": {"steps": k, "ms_per_step": elm / k * 1e3, "value": ncell * k / elm,
                     "unit": UNIT},
           "fp64": {"steps": k, "ms_per_step": el64 / k * 1e3, "value": ncell * k / el64,
                    "unit": UNIT},
           "steps_compared": k, "rel_l1_mixed_vs_fp64": l1, "rel_linf_mixed_vs_fp64": linf,
           "max_rel_l1": max(l1),
           "fp64_state_after_steps": _physical(w64, float(snap.eqpar[0]), True)}
    out["mixed_over_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    return out


def run_tvdmu(args):
    """The TVD-MUSCL/Roe corrector ('tvdmu', src/vactvd.t:86-243) on the
    3-D random-mode MHD state at --tvdmu-side^3, woodward, periodic: mixed
    and FP64 timed over --tvdmu-steps steps each, the Roe kernel's share of
    the step, and the mixed-vs-FP64 relative L1 after those steps."""
    import torch
    from vac_gb300 import abi, inistate
    from vac_gb300.engine import Engine
    n = args.tvdmu_side
    snap = inistate.random_modes(n, seed=0)
    ncell = n ** 3
    k = args.tvdmu_steps
    stream = torch.cuda.Stream()
    out = {"workload": "3D ideal MHD random modes %d^3 periodic, woodward, typefull='tvdmu' "
                       "(Roe, 8 waves), %d steps timed per precision" % (n, k)}
    res = {}
    for name, prec in (("mixed", abi.PREC_MIXED), ("fp64", abi.PREC_FP64)):
        p = make_params(snap, prec)
        p.typefull = abi.TVDMU
        e = Engine(p, snap.x, snap.w)
        e.set_stream(stream.cuda_stream)
        e.step(3)
        e.upload(snap.w)
        el = _timed_steps(e, k, stream)
        e.timing(True)
        e.step(1)
        kst = e.kernel_stats()
        e.timing(False)
        tot = sum(v[1] for v in kst.values())
        share = {kk: round(v[1] / tot, 4) for kk, v in kst.items() if v[0]}
        res[name] = e.state()
        e.close()
        out[name] = {"steps": k, "ms_per_step": el / k * 1e3, "value": ncell * k / el,
                     "unit": UNIT, "kernel_share": share}
    out["mixed_over_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    out["rel_l1_mixed_vs_fp64"], out["rel_linf_mixed_vs_fp64"] = _errors(res["mixed"],
                                                                         res["fp64"])
    return out


def random_modes_dev(n, seed, ndim, device, packed=False):
    """vac_gb300.inistate.random_modes (p0=0.05, beta ~ 0.1, 8 modes per
    field) with the fields evaluated by torch on `device`: the same seeded
    draws in the same order, the same formulas; the result differs from the
    NumPy evaluation by rounding only.  Returns (x, w) as NumPy arrays in
    the (ndim|nw, *nx) layout of a snapshot.  The served stream's requests
    are drawn with it (a NumPy evaluation of a 256^3 state takes tens of
    seconds of host time).  packed: (x, w) as flat arrays in the C ABI's
    layout instead (each component in Fortran order, permuted on the
    device)."""
    import torch
    from vac_gb300 import inistate
    rng = np.random.default_rng(seed)
    nmodes, gamma = 8, 5.0 / 3.0
    nx = (n,) * ndim
    x = inistate.domain_grid(nx, (0.0,) * ndim, (1.0,) * ndim)
    xd = [torch.as_tensor(x[d], device=device) for d in range(ndim)]

    def phase_fields(ks, phis):
        out = []
        for k, ph in zip(ks, phis):
            z = torch.full(nx, complex(np.cos(ph), np.sin(ph)), dtype=torch.complex128,
                           device=device)
            for d in range(ndim):
                z = z * torch.exp(2j * np.pi * float(k[d]) * xd[d])
            out.append(z.real)
        return out

    ks = inistate._modes(rng, nmodes, ndim)
    a = rng.uniform(0.5, 1.0, nmodes)
    a *= 0.2 / a.sum()
    cs = phase_fields(ks, rng.uniform(0, 2 * np.pi, nmodes))
    rho = torch.ones(nx, dtype=torch.float64, device=device)
    for ak, c in zip(a, cs):
        rho += float(ak) * c
    ks = inistate._modes(rng, nmodes, ndim)
    dirs = rng.normal(size=(nmodes, 3))
    if ndim == 2:
        dirs[:, 2] = 0.0
    cs = phase_fields(ks, rng.uniform(0, 2 * np.pi, nmodes))
    v = [torch.zeros(nx, dtype=torch.float64, device=device) for _ in range(ndim)]
    for dvec, c in zip(dirs, cs):
        for d in range(ndim):
            v[d] += float(dvec[d]) * c
    vr = torch.sqrt(torch.mean(sum(vc * vc for vc in v)))
    v = [vc * (0.3 / vr) for vc in v]
    ks = inistate._modes(rng, nmodes, ndim)
    es = rng.normal(size=(nmodes, 3))
    cs = phase_fields(ks, rng.uniform(0, 2 * np.pi, nmodes))
    bp = [torch.zeros(nx, dtype=torch.float64, device=device) for _ in range(ndim)]
    for k, e, c in zip(ks, es, cs):
        pol = np.cross(e, k)
        for d in range(ndim):
            bp[d] += float(pol[d]) * c
    br = torch.sqrt(torch.mean(sum(bc * bc for bc in bp)))
    b = [bc * (0.1 / br) for bc in bp]
    b[0] = b[0] + 1.0
    v2 = sum(vc * vc for vc in v)
    b2 = sum(bc * bc for bc in b)
    e = 0.05 / (gamma - 1) + 0.5 * rho * v2 + 0.5 * b2
    w = torch.stack([rho] + [rho * vc for vc in v] + [e] + b)
    if packed:
        perm = (0,) + tuple(range(ndim, 0, -1))
        xt = torch.as_tensor(np.ascontiguousarray(x), device=device)
        return (xt.permute(*perm).contiguous().reshape(-1).cpu().numpy(),
                w.permute(*perm).contiguous().reshape(-1).cpu().numpy())
    return x, w.cpu().numpy()


def _served_requests(args):
    """The served request stream (seeded): kind, side, step count."""
    rng = np.random.default_rng(7)
    reqs = []
    for i in range(args.served):
        if rng.uniform() < 0.5:
            n, nd = int(round(np.exp(rng.uniform(np.log(128), np.log(2048))))), 2
        else:
            n, nd = int(round(np.exp(rng.uniform(np.log(64), np.log(256))))), 3
        reqs.append((nd, n, int(rng.integers(20, 501)), 100 + i))
    return reqs


def run_served_rate(args, reqs, rate, arrivals_seed):
    """One served run: the requests arrive as a Poisson stream of the given
    mean rate.  A producer thread draws them on the device, in the ABI's
    packed layout, and hands them to the submitting thread, at most 8 GB
    ahead; the submitting thread submits each at its arrival time (the
    server copies it, and back to the device on admission).  Per request:
    time to solution, its queue part (submission to admission) and its
    service part (admission to result); max_submit_lag_s is how far the
    latest submission fell behind its arrival time."""
    import queue
    import threading
    from vac_gb300 import abi, inistate
    from vac_gb300.engine import Server
    rng = np.random.default_rng(arrivals_seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, len(reqs)))
    srv = Server(hbm_budget_bytes=150e9, max_active=args.served_slots,
                 steps_per_chunk=args.served_chunk)
    ids = [None] * len(reqs)
    late = [0.0] * len(reqs)
    ready = queue.Queue()
    cv = threading.Condition()
    ahead = [0]  # bytes drawn and not yet submitted
    cap = 8e9

    def produce():
        for nd, n, steps, seed in reqs:
            nw = 2 + 2 * nd
            nbytes = 8 * (nw + nd) * n ** nd
            with cv:
                cv.wait_for(lambda: ahead[0] == 0 or ahead[0] + nbytes <= cap)
                ahead[0] += nbytes
            xf, wf = random_modes_dev(n, seed, nd, "cuda", packed=True)
            shape = np.broadcast_to(np.float64(0.0), (nw,) + (n,) * nd)
            snap = inistate._snap(None, shape, 5.0 / 3.0, True, nd, "served")
            p = inistate.params_for(snap, limiter="woodward", precision=abi.PREC_MIXED)
            ready.put((p, xf, wf, steps, nbytes))

    prod = threading.Thread(target=produce)
    prod.start()
    while ready.qsize() < min(16, len(reqs)) and prod.is_alive():
        time.sleep(0.01)
    t0 = time.perf_counter()
    for i in range(len(reqs)):
        p, xf, wf, steps, nbytes = ready.get()
        dt = arrivals[i] - (time.perf_counter() - t0)
        if dt > 0:
            time.sleep(dt)
        late[i] = max(0.0, -dt)
        ids[i] = srv.submit(p, xf, wf, steps)
        del xf, wf
        with cv:
            ahead[0] -= nbytes
            cv.notify_all()
    prod.join()
    tts, qs, svs = [], [], []
    for rid in ids:
        res = srv.result(rid, wait=1200.0, fetch=False)
        tts.append(res[3])
        q, sv = srv.timing(rid)
        qs.append(q)
        svs.append(sv)
    st = srv.stats()
    srv.close()

    def pct(a):
        return {"p50": float(np.percentile(a, 50)), "p99": float(np.percentile(a, 99)),
                "mean": float(np.mean(a))}
    return {"offered_rate_per_s": rate, "requests": len(reqs),
            "time_to_solution_s": pct(tts), "queue_s": pct(qs), "service_s": pct(svs),
            "value": st["cell_updates"] / st["span_s"] if st["span_s"] > 0 else None,
            "unit": UNIT, "peak_concurrent": st["peak_active"],
            "cell_updates": st["cell_updates"], "span_s": st["span_s"],
            "max_submit_lag_s": float(max(late))}


def run_served(args, capacity):
    """The served workload: a Poisson stream of 2-D (128^2..2048^2) and 3-D
    (64^3..256^3) random-mode MHD solves, 20..500 steps each, mixed
    precision, admitted against a 150 GB HBM budget, at offered loads of
    --served-loads times the single-grid capacity (cell-updates/s of the
    256^3 bench divided by the stream's mean work per request); per load
    p50/p99 of the time to solution, split into queue and service time,
    and the aggregate cell-updates/s."""
    reqs = _served_requests(args)
    work = np.mean([(n ** nd) * steps for nd, n, steps, _ in reqs])
    loads = [float(v) for v in args.served_loads.split(",")]
    runs = []
    for i, ld in enumerate(loads):
        runs.append(dict(run_served_rate(args, reqs, ld * capacity / work, 11 + i), load=ld))
    return {"workload": "Poisson stream of %d MHD solves per load: 2D 128^2-2048^2 / "
                        "3D 64^3-256^3, 20-500 steps, random modes, mixed, 150 GB budget, "
                        "%d slots" % (len(reqs), args.served_slots),
            "loads": runs, "slots": args.served_slots,
            "mean_cell_updates_per_request": float(work),
            "capacity_cell_updates_per_s": capacity}


def run_snapshots(args, snap, hin):
    """Save events every --snap-every steps on the 256^3 mixed run, 40 steps:
    the state leaves the device synchronously (vacgpu_download into a pinned
    buffer, then the next steps) or as an asynchronous snapshot
    (vacgpu_snapshot_begin; a second host thread waits for it and takes it in
    place from the library's page-locked copy, as the vacgb host program's
    writer thread does, while the next steps run).  Wall-clock time of each
    against the same steps without saves."""
    import threading as th
    import torch
    from vac_gb300 import abi
    from vac_gb300.engine import Engine
    k, n = args.snap_every, 40
    out = torch.empty_like(hin).pin_memory()
    res = {}
    for mode in ("none", "sync", "async"):
        e = Engine(make_params(snap, abi.PREC_MIXED), snap.x, snap.w)
        e.step(3)
        e.upload(snap.w)
        if mode == "async":  # first use of the slot allocates its buffers
            e.snapshot_begin(0)
            e.snapshot_view(0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        writer = None
        for _ in range(n // k):
            e.step(k)
            if mode == "sync":
                e.download_flat(out.data_ptr())
            elif mode == "async":
                if writer:
                    writer.join()
                e.snapshot_begin(0)
                writer = th.Thread(target=e.snapshot_view, args=(0,))
                writer.start()
        if writer:
            writer.join()
        torch.cuda.synchronize()
        res[mode] = time.perf_counter() - t0
        e.close()
    return {"workload": "3D MHD random modes %d^3 mixed, %d steps, a save event every %d "
                        "steps (%d MB FP64 state per save)" % (N, n, k, hin.numel() * 8 // 10**6),
            "seconds_no_saves": res["none"], "seconds_sync_saves": res["sync"],
            "seconds_async_saves": res["async"],
            "save_cost_sync_ms": (res["sync"] - res["none"]) / (n // k) * 1e3,
            "save_cost_async_ms": (res["async"] - res["none"]) / (n // k) * 1e3}


def run_reference(args, ws, rank):
    if rank != 0:
        return
    from vac_gb300 import inistate
    threads = os.cpu_count() or 1
    snap = inistate.random_modes(N, seed=0)
    os.environ["OMP_NUM_THREADS"] = str(threads)
    from oracle.oracle import Oracle
    p = make_params(snap, 0)
    o = Oracle(p, snap.x, snap.w)
    o.step(max(args.warmup, 1))
    t0 = time.perf_counter()
    o.step(args.steps)
    el = time.perf_counter() - t0
    v = N ** 3 * args.steps / el
    line = {"metric": METRIC, "value": v, "unit": UNIT, "impl": "reference",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": el / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": workload_config(args.precision),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": "%d full 256^3 steps of the FP64 oracle port "
                                       "(OpenMP, %d threads)" % (args.steps, threads)},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    global N
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=2)
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--served", type=int, default=200,
                    help="requests per offered load in the served stream (0: skip)")
    ap.add_argument("--served-slots", type=int, default=8,
                    help="solves the served run keeps in flight at most")
    ap.add_argument("--served-chunk", type=int, default=16,
                    help="steps the server issues per solve at a time")
    ap.add_argument("--served-loads", default="0.5,0.9,1.2",
                    help="offered loads of the served stream, in units of the capacity")
    ap.add_argument("--acc-steps", type=int, default=100,
                    help="steps of the 256^3 mixed-vs-FP64 accuracy run")
    ap.add_argument("--no-serial", action="store_true",
                    help="skip the 1-core CPU baseline (Orszag-Tang 200^2 in full)")
    ap.add_argument("--cpu-serial-only", action="store_true", help=argparse.SUPPRESS)
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--batched-only", action="store_true",
                    help="run the batched workload alone and print its JSON object (profiling)")
    ap.add_argument("--no-plain", action="store_true", help="skip the Orszag-Tang 200^2 FP64 run")
    ap.add_argument("--blast-side", type=int, default=512,
                    help="blast run cells per side (0: skip)")
    ap.add_argument("--blast-steps", type=int, default=100)
    ap.add_argument("--tvdmu-side", type=int, default=128,
                    help="cells per side of the tvdmu/Roe case (0: skip)")
    ap.add_argument("--tvdmu-steps", type=int, default=10)
    ap.add_argument("--snap-every", type=int, default=4,
                    help="steps between save events of the snapshot run (0: skip)")
    ap.add_argument("--side", type=int, default=N,
                    help="cells per side of the cube (smaller cases for profiling)")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"],
                    help="precision of the timed 256^3 run (the headline is mixed)")
    ap.add_argument("--profile-range", action="store_true",
                    help="bracket the timed steps with cudaProfilerStart/Stop (for ncu "
                         "--profile-from-start off)")
    args = ap.parse_args()
    N = args.side
    if args.cpu_serial_only:
        print(json.dumps(cpu_serial_ot200()), flush=True)
        return
    ws, rank, lrank = dist_setup()
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return
    if args.batched_only:
        import torch
        torch.cuda.set_device(lrank)
        print(json.dumps(run_batched(args)), flush=True)
        return

    import torch
    torch.cuda.set_device(lrank)
    from vac_gb300 import abi, inistate
    from vac_gb300.engine import Engine

    snap = inistate.random_modes(N, seed=rank)
    ncell = N ** 3
    K, W = args.steps, max(args.warmup, 3)

    prec = abi.PREC_MIXED if args.precision == "mixed" else abi.PREC_FP64
    elem = 4 if args.precision == "mixed" else 8
    stream = torch.cuda.Stream()
    eng = Engine(make_params(snap, prec), snap.x, snap.w)
    eng.set_stream(stream.cuda_stream)
    eng.step(W)
    # ---- device-resident timed region: K steps, CUDA events on the stream
    eng.timing(True)
    eng.timing(False)  # launch counters reset; no per-kernel events here
    barrier(ws)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(lrank) as clk:
        if args.profile_range:
            torch.cuda.profiler.start()
        ev0.record(stream)
        eng.step(K)
        ev1.record(stream)
        torch.cuda.synchronize()
        if args.profile_range:
            torch.cuda.profiler.stop()
    el = ev0.elapsed_time(ev1) / 1e3
    barrier(ws)
    value, el = whole_job(ws, ncell * K, el)
    stats = eng.kernel_stats()
    launches = sum(v[0] for v in stats.values())

    # ---- roofline of the dominant kernel: a second pass with per-launch events
    eng.timing(True)
    eng.step(K)
    kst = eng.kernel_stats()
    eng.timing(False)
    dom = max((k for k in kst if kst[k][0]), key=lambda k: kst[k][1])
    n_l, ms_l = kst[dom]
    avg_s = ms_l / n_l / 1e3
    alg_bytes = 2 * NW * elem * ncell  # one read + one write of the state per sweep
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    achieved = alg_bytes / avg_s / 1e9
    traffic, traffic_src = sweep_traffic(ncell)
    shares = {k: round(v[1] / sum(x[1] for x in kst.values()), 4) for k, v in kst.items() if v[0]}

    # ---- end to end through the C ABI with host buffers
    hin = torch.from_numpy(np.concatenate([snap.w[i].ravel(order="F") for i in range(NW)])).pin_memory()
    hout = torch.empty_like(hin).pin_memory()
    eng2 = Engine(make_params(snap, prec), snap.x, snap.w)
    eng2.set_stream(stream.cuda_stream)
    eng2.step(W)
    # warm-up of the transfer path too: the first DMA over freshly pinned
    # buffers runs several times slower than the steady state
    for _ in range(2):
        eng2.upload_flat(hin.data_ptr())
        eng2.step(1)
        eng2.download_flat(hout.data_ptr())
    torch.cuda.synchronize()
    barrier(ws)
    t0 = time.perf_counter()
    eng2.upload_flat(hin.data_ptr())
    eng2.step(K)
    eng2.download_flat(hout.data_ptr())
    torch.cuda.synchronize()
    e2e_value, e2e_el = whole_job(ws, ncell * K, time.perf_counter() - t0)
    eng2.close()

    # ---- plain FP64 run and the mixed-vs-FP64 error after the run's steps
    fp64 = None
    if not args.no_fp64 and rank == 0:
        fp64 = run_fp64_c2(args, snap, stream, value / ws)

    batched = served = plain = blast = tvdmu = snaps = None
    if rank == 0 and args.snap_every > 0:
        snaps = run_snapshots(args, snap, hin)
    if rank == 0 and not args.no_plain:
        plain = run_plain(args)
    if rank == 0 and args.blast_side > 0:
        blast = run_blast(args)
    if rank == 0 and args.tvdmu_side > 0:
        tvdmu = run_tvdmu(args)
    if rank == 0 and not args.no_batched:
        batched = run_batched(args)
    if rank == 0 and args.served > 0:
        served = run_served(args, value / ws)

    cpu = serial = None
    if rank == 0 and ws == 1 and not args.no_serial:
        serial = cpu_serial_subprocess()
    if rank == 0 and ws == 1 and args.cpu_steps > 0:
        threads = os.cpu_count() or 1
        v, t = cpu_sample(snap, args.cpu_steps, threads)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": "%d full %d^3 steps of the FP64 oracle port (OpenMP, %d threads), "
                         "%.1f s" % (args.cpu_steps, N, threads, t)}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
                "steps": K, "warmup": W, "ms_per_step": el / K * 1e3,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32 (FP64 pressure recovery via double-float, FP64 sums and t)"
                         if elem == 4 else "f64",
                "data": "synthetic", "config": workload_config(args.precision),
                "parallelism": "replicas" if ws > 1 else "single",
                "e2e": {"value": e2e_value, "unit": UNIT,
                        "h2d_bytes_per_step": hin.numel() * 8 / K,
                        "d2h_bytes_per_step": hout.numel() * 8 / K,
                        "note": "vacgpu_upload of the FP64 .ini state + %d steps + "
                                "vacgpu_download, host pinned buffers" % K},
                "gpu_launches": launches,
                "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved,
                             "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                             "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)",
                             "traffic": traffic, "traffic_source": traffic_src,
                             "avg_launch_ms": avg_s * 1e3,
                             "alg_bytes_per_launch": alg_bytes,
                             "kernel_share": shares},
                "fp64": fp64, "plain_fp64_ot200": plain, "blast_512": blast,
                "tvdmu_roe": tvdmu, "snapshots": snaps,
                "batched": batched, "served": served,
                "cpu_baseline": cpu, "cpu_baseline_serial": serial,
                "clocks": clk.summary()}
        print(json.dumps(line), flush=True)
    eng.close()
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
