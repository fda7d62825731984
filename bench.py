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
                        "(seeded), 100-step config timed per step" % N,
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


def run_batched(args):
    """Config 3: 64 2-D gamma=1.4 Riemann problems, sides log-uniform in
    [64, 1024], outflow, minmod, mixed precision; all grids advance 50 steps
    in one replay of a CUDA graph of batched persistent-kernel launches."""
    import torch
    from vac_gb300 import inistate
    from vac_gb300.engine import Batch
    grids = inistate.riemann_batch(n=64, seed=0)
    cells = sum(int(np.prod([g[0].nx[d] for d in range(2)])) for g in grids)
    b = Batch(grids)
    ctas, order, ms = b.tune()
    b.step(50)  # capture + first replay
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    b.step(50)
    el = time.perf_counter() - t0
    b.close()
    return {"workload": "64 grids 2D HD Riemann, sides log-uniform [64,1024] (seeded), "
                        "cont, minmod, mixed, 50 steps per grid in one graph launch",
            "grids": 64, "cells": cells, "steps": 50, "seconds": el,
            "value": cells * 50 / el, "unit": UNIT,
            "tuned": {"persistent_ctas": ctas, "order": ["round-robin", "grid-major"][order],
                      "trial_ms": ms}}


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
    """Config 1: the plain FP64 method, 2-D ideal MHD Orszag-Tang on
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
    """Config 5: 3-D ideal MHD blast on 512^3 cells, outflow ('cont'),
    woodward, B=(1,1,0)/sqrt2, p from 10 to 0.1 across r=0.1: mixed
    precision timed over --blast-steps steps (the fused sweep), FP64 over 2
    steps, and the mixed-vs-FP64 relative L1 after those 2 steps from the
    same initial state."""
    import torch
    from vac_gb300 import abi, inistate
    from vac_gb300.engine import Engine
    n = args.blast_side
    snap = inistate.blast_3d(n)
    ncell = n ** 3
    stream = torch.cuda.Stream()
    out = {"workload": "3D ideal MHD blast %d^3, cont, woodward, mixed %d steps timed, "
                       "FP64 2 steps timed" % (n, args.blast_steps)}
    pm = inistate.params_for(snap, limiter="woodward", bc="cont", precision=abi.PREC_MIXED)
    em = Engine(pm, snap.x, snap.w)
    em.set_stream(stream.cuda_stream)
    em.step(2)
    wm2 = em.state()
    em.step(3)
    el = _timed_steps(em, args.blast_steps, stream)
    em.close()
    out["mixed"] = {"steps": args.blast_steps, "ms_per_step": el / args.blast_steps * 1e3,
                    "value": ncell * args.blast_steps / el, "unit": UNIT}
    p64 = inistate.params_for(snap, limiter="woodward", bc="cont", precision=abi.PREC_FP64)
    e64 = Engine(p64, snap.x, snap.w)
    e64.set_stream(stream.cuda_stream)
    el64 = _timed_steps(e64, 2, stream)
    w64 = e64.state()
    e64.close()
    out["fp64"] = {"steps": 2, "ms_per_step": el64 / 2 * 1e3, "value": ncell * 2 / el64,
                   "unit": UNIT}
    out["mixed_over_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    out["rel_l1_mixed_vs_fp64_after_2_steps"] = [
        float(np.abs(wm2[i] - w64[i]).sum() / max(np.abs(w64[i]).sum(), 1e-300))
        for i in range(w64.shape[0])]
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
    wm, w64 = res["mixed"], res["fp64"]
    out["rel_l1_mixed_vs_fp64"] = [
        float(np.abs(wm[i] - w64[i]).sum() / max(np.abs(w64[i]).sum(), 1e-300))
        for i in range(w64.shape[0])]
    return out


def run_served(args, capacity):
    """Config 4: a Poisson stream of 2-D (128^2..2048^2) and 3-D (64^3..256^3)
    random-mode MHD solves, 20..500 steps each, mixed precision, admitted
    against a 150 GB HBM budget; p50/p99 time to solution."""
    import threading
    from vac_gb300 import abi, inistate
    from vac_gb300.engine import Server
    rng = np.random.default_rng(7)
    reqs = []
    for i in range(args.served):
        if rng.uniform() < 0.5:
            n = int(round(np.exp(rng.uniform(np.log(128), np.log(2048)))))
            s = inistate.random_modes(n, seed=100 + i, ndim=2)
        else:
            n = int(round(np.exp(rng.uniform(np.log(64), np.log(256)))))
            s = inistate.random_modes(n, seed=100 + i, ndim=3)
        steps = int(rng.integers(20, 501))
        p = inistate.params_for(s, limiter="woodward", precision=abi.PREC_MIXED)
        reqs.append((p, s.x, s.w, steps, int(np.prod(s.w.shape[1:]))))
    work = [r[4] * r[3] for r in reqs]
    rate = 0.9 * capacity / np.mean(work)  # offered load ~0.9 of capacity
    arrivals = np.cumsum(rng.exponential(1.0 / rate, len(reqs)))
    srv = Server(hbm_budget_bytes=150e9, max_active=8, steps_per_chunk=16)
    ids = [None] * len(reqs)
    t0 = time.perf_counter()

    def feed():
        for i, r in enumerate(reqs):
            dt = arrivals[i] - (time.perf_counter() - t0)
            if dt > 0:
                time.sleep(dt)
            ids[i] = srv.submit(r[0], r[1], r[2], r[3])

    th = threading.Thread(target=feed)
    th.start()
    th.join()
    tts = []
    for rid in ids:
        res = srv.result(rid, wait=600.0, fetch=False)
        tts.append(res[3])
    st = srv.stats()
    srv.close()
    return {"workload": "Poisson stream of %d MHD solves: 2D 128^2-2048^2 / 3D 64^3-256^3, "
                        "20-500 steps, random modes, mixed, 150 GB budget" % len(reqs),
            "requests": len(reqs), "offered_rate_per_s": rate,
            "p50_s": float(np.percentile(tts, 50)), "p99_s": float(np.percentile(tts, 99)),
            "value": st["cell_updates"] / st["span_s"] if st["span_s"] > 0 else None,
            "unit": UNIT, "peak_concurrent": st["peak_active"],
            "cell_updates": st["cell_updates"], "span_s": st["span_s"]}


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
            "data": "synthetic", "config": workload_config("fp64"),
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
    ap.add_argument("--served", type=int, default=12, help="requests in the served stream (0: skip)")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-plain", action="store_true", help="skip config 1")
    ap.add_argument("--blast-side", type=int, default=512,
                    help="config 5 cells per side (0: skip)")
    ap.add_argument("--blast-steps", type=int, default=20)
    ap.add_argument("--tvdmu-side", type=int, default=128,
                    help="cells per side of the tvdmu/Roe case (0: skip)")
    ap.add_argument("--tvdmu-steps", type=int, default=10)
    ap.add_argument("--side", type=int, default=N,
                    help="cells per side of the cube (smaller cases for profiling)")
    args = ap.parse_args()
    N = args.side
    ws, rank, lrank = dist_setup()
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return

    import torch
    torch.cuda.set_device(lrank)
    from vac_gb300 import abi, inistate
    from vac_gb300.engine import Engine

    snap = inistate.random_modes(N, seed=rank)
    ncell = N ** 3
    K, W = args.steps, max(args.warmup, 3)

    stream = torch.cuda.Stream()
    eng = Engine(make_params(snap, abi.PREC_MIXED), snap.x, snap.w)
    eng.set_stream(stream.cuda_stream)
    eng.step(W)
    # ---- device-resident timed region: K steps, CUDA events on the stream
    eng.timing(True)
    eng.timing(False)  # launch counters reset; no per-kernel events here
    barrier(ws)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(lrank) as clk:
        ev0.record(stream)
        eng.step(K)
        ev1.record(stream)
        torch.cuda.synchronize()
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
    alg_bytes = 2 * NW * 4 * ncell  # one read + one write of the state per sweep
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    achieved = alg_bytes / avg_s / 1e9
    traffic = None
    tf = os.path.join(ROOT, "profiles", "traffic_%s.txt" % dom)
    if os.path.exists(tf):
        for ln in open(tf):
            if ln.startswith("bytes_per_cell="):
                traffic = float(ln.split("=")[1]) * ncell
    shares = {k: round(v[1] / sum(x[1] for x in kst.values()), 4) for k, v in kst.items() if v[0]}

    # ---- end to end through the C ABI with host buffers
    hin = torch.from_numpy(np.concatenate([snap.w[i].ravel(order="F") for i in range(NW)])).pin_memory()
    hout = torch.empty_like(hin).pin_memory()
    eng2 = Engine(make_params(snap, abi.PREC_MIXED), snap.x, snap.w)
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

    # ---- plain FP64 run of the same steps and the mixed-vs-FP64 error
    fp64 = None
    if not args.no_fp64:
        wm = eng.state()  # mixed state after W + 2K steps
        e64 = Engine(make_params(snap, abi.PREC_FP64), snap.x, snap.w)
        e64.set_stream(stream.cuda_stream)
        e64.step(W)
        torch.cuda.synchronize()
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a0.record(stream)
        e64.step(K)
        a1.record(stream)
        torch.cuda.synchronize()
        el64 = a0.elapsed_time(a1) / 1e3
        e64.step(K)
        w64 = e64.state()
        rel_l1 = [float(np.abs(wm[i] - w64[i]).sum() / max(np.abs(w64[i]).sum(), 1e-300))
                  for i in range(NW)]
        linf = [float(np.abs(wm[i] - w64[i]).max() / max(np.abs(w64[i]).max(), 1e-300))
                for i in range(NW)]
        fp64 = {"value": ncell * K / el64, "unit": UNIT, "ms_per_step": el64 / K * 1e3,
                "mixed_over_fp64": (ncell * K / el) / (ncell * K / el64),
                "steps_compared": W + 2 * K,
                "rel_l1_mixed_vs_fp64": rel_l1, "rel_linf_mixed_vs_fp64": linf}
        e64.close()

    batched = served = plain = blast = tvdmu = None
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

    cpu = None
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
                "dtype": "f32 (FP64 pressure recovery via double-float, FP64 sums and t)",
                "data": "synthetic", "config": workload_config("mixed"),
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
                             "traffic": traffic, "avg_launch_ms": avg_s * 1e3,
                             "alg_bytes_per_launch": alg_bytes,
                             "kernel_share": shares},
                "fp64": fp64, "plain_fp64_config1": plain, "blast_config5": blast,
                "tvdmu_roe": tvdmu,
                "batched": batched, "served": served,
                "cpu_baseline": cpu, "clocks": clk.summary()}
        print(json.dumps(line), flush=True)
    eng.close()
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
