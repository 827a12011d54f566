#!/usr/bin/env python
"""Benchmark: full single-shot RTM on the 512 x 512 x 400 grid (dx 12.5 m,
dt 1 ms, 4000 steps; padded to 560 x 560 x 496) -- Born data generation
(rtm_forward), random-boundary source propagation (source_prop) and the RTM
adjoint with source reconstruction and zero-lag imaging (rtm_adjoint).

One "step" = those three time loops for one shot.  Metric: Gcell-updates/s
(updated interior cells x field-steps / time).  ``value`` is timed with the
inputs resident in HBM (CUDA events on the library's stream); ``e2e`` runs the
same step through the reference-named C ABI with pinned host buffers and all
host<->device copies inside the timed region.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

HBM_FALLBACK_GBS = 6800.0


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=2)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--nt", type=int, default=4000, help="propagation steps (the workload's 4000)")
    p.add_argument("--grid", default="512x512x400")
    # a 100-step window of each loop on the full grid
    p.add_argument("--cpu-sample-steps", type=int, default=100)
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--e2e-clock-ms", type=int, default=1000,
                   help="nvidia-smi sampling interval during the e2e region (0: none)")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--workload", default="rtm", choices=["rtm", "batch"],
                   help="rtm: the single-shot RTM line; batch: 16 batched shots")
    p.add_argument("--batch-nt", type=int, default=1000)
    return p.parse_args()


# ------------------------------------------------------------------ distributed
def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def dist_init(ws, local):
    if ws > 1:
        # one visible GPU per rank: every rank runs an independent shot
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo")
        return dist
    return None


def max_over_ranks(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


# ------------------------------------------------------------------ clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, interval_ms=200):
        self.proc = None
        self.lines = []
        self.interval_ms = interval_ms

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", str(self.interval_ms)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = max(mx, float(parts[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if parts[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        loaded = [v for v in sm if v > 0.5 * mx] or sm
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------------ workload
def build_workload(args):
    """The survey and the product's own shot set-up (GPU arm)."""
    from sep_code_gb300 import model as M
    from sep_code_gb300 import surveys as S
    n1, n2, n3 = (int(v) for v in args.grid.split("x"))
    s = S.layered_survey(n1, n2, n3, nt=args.nt)
    return s, M.prepare_shot(s)


def build_workload_oracle(args, orc):
    """The same survey and shot set-up from the oracle alone (CPU arm): no
    product library is loaded on this path."""
    from oracle.shot_setup import prepare_shot
    from sep_code_gb300 import surveys as S
    n1, n2, n3 = (int(v) for v in args.grid.split("x"))
    s = S.layered_survey(n1, n2, n3, nt=args.nt)
    return s, prepare_shot(orc, s)


def workload_config(args, st, ws):
    """The ``config`` object of both arms' JSON lines (identical keys)."""
    n1, n2, n3 = st.n
    cells, fsteps = cell_updates(st)
    return {"workload": f"rtm_single_shot_{args.grid}_nt{st.nt}",
            "model_grid": args.grid, "padded_grid": f"{n1}x{n2}x{n3}", "dx_m": st.d[0],
            "dt_s": st.dt, "nt": st.nt, "receivers": st.rnx * st.rny,
            "cells_per_field_step": cells, "field_steps_per_step": fsteps,
            "l2": "inputs larger than L2 (each volume "
                  f"{4 * n1 * n2 * n3 / 1e6:.0f} MB > 129 MB)",
            "parallelism": f"{ws} independent shot(s), one per GPU"}


def cell_updates(st):
    n1, n2, n3 = st.n
    cells = (16 * ((n1 - 8) // 16)) * (16 * ((n2 - 8) // 16)) * max(0, n3 - 12)
    nt = st.nt
    field_steps = {"source_prop": nt + 1, "rtm_forward": 2 * nt, "rtm_adjoint": 2 * nt - 1}
    return cells, field_steps


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d.get("hbm_gbs", HBM_FALLBACK_GBS)), "measured"
    return HBM_FALLBACK_GBS, "fallback"


def profiled_traffic(kernel_key: str):
    """dram bytes per launch recorded in profiles/ (from an ncu capture)."""
    for f in sorted((ROOT / "profiles").glob("*.md")):
        txt = f.read_text()
        m = re.search(rf"traffic_bytes_per_launch\[{re.escape(kernel_key)}\]:\s*([0-9.eE+]+)", txt)
        if m:
            return float(m.group(1)), f.name
    return None, None


# ------------------------------------------------------------------ CPU baseline (oracle)
def cpu_baseline(s, st, steps, orc=None):
    """The reference path's CPU restatement (oracle/) on a bounded sample: the
    three time loops of the workload, ``steps`` time steps each, full grid,
    all host threads.  Inputs come from the oracle's own set-up routines."""
    from oracle.bindings import Oracle
    from oracle.shot_setup import make_ctx, source_vals
    orc = orc or Oracle()
    n1, n2, n3 = st.n
    keep = []
    locs, vals = source_vals(orc, s, st, 9)
    ctx = make_ctx(orc, s, st, locs, vals, keep)
    nrec = st.rnx * st.rny
    dat = np.zeros((nrec, vals.shape[1]), np.float32)
    img = np.ascontiguousarray(st.img_lap, np.float32)
    cells, _ = cell_updates(st)
    t0 = time.perf_counter()
    p0, p1 = orc.source_prop(ctx, st.vel2dt2, st.jts, 9, steps - 1)
    orc.rtm_forward(ctx, st.vel2dt2, st.jtd, img, dat, 9, steps)
    orc.rtm_adjoint(ctx, st.vel2dt2, st.jtd, p1, p0, dat, 9, steps)
    el = time.perf_counter() - t0
    updates = cells * (steps + 2 * steps + (2 * steps - 1))
    return {"value": updates / el / 1e9, "unit": "Gcell/s", "cores": orc.num_threads(),
            "kind": "port", "seconds": el,
            "sample": f"oracle (C/OpenMP restatement), {steps} time steps of each of the three "
                      f"loops on the full {n1}x{n2}x{n3} padded grid"}


# ------------------------------------------------------------------ GPU arm
def run_ours(args, ws, rank, dist):
    import torch
    from sep_code_gb300 import gpu_funcs as gf
    from sep_code_gb300._lib import lib

    s, st = build_workload(args)
    n1, n2, n3 = st.n
    nrec = st.rnx * st.rny
    wd = gf.wavelet_deriv(s.wavelet, s.dtw)
    sx, sy, sz = s.shots[0]
    locs9, vals9 = gf.source_func(wd, sx, sy, sz, n1, n2, st.o, st.d, s.data_nt + 9)
    locs8, vals8 = gf.source_func(wd, sx, sy, sz, n1, n2, st.o, st.d, s.data_nt + 8)

    gf.setup_cuda(1)
    gf.create_gpu_space(st.d[0], st.d[1], st.d[2], s.bc_a, s.bc_b, s.bc_b, n1, n2, n3)
    gf.transfer_sinc_table_s(st.sinc_s)
    gf.transfer_sinc_table_d(st.sinc_d)
    gf.transfer_vel_func1(st.vel2dt2)
    zeros_tr = np.zeros((nrec, st.nt_big), np.float32)
    gf.transfer_receiver_func(st.rnx, st.rny, st.rec_locs, zeros_tr)
    gf.transfer_source_func(locs9, vals9)
    lib.sepx_set_image(np.ascontiguousarray(st.img_lap, np.float32))
    gf.synchronize()

    stream = torch.cuda.ExternalStream(lib.sepx_get_stream())

    def chk(rc):
        if rc != 0:
            raise gf.SepxError(lib.sepx_last_error().decode())

    def step(events=None):
        if events:
            events[0].record(stream)
        chk(lib.sepx_source_prop_resident(st.jts, 9, st.nt))
        if events:
            events[1].record(stream)
        chk(lib.sepx_zero_traces())
        chk(lib.sepx_rtm_forward_resident(st.jtd, 9, st.nt))
        if events:
            events[2].record(stream)
        chk(lib.sepx_rtm_adjoint_resident(st.jtd, 9, st.nt, 1))
        if events:
            events[3].record(stream)

    for _ in range(args.warmup):
        step()
    gf.synchronize()

    cells, fsteps = cell_updates(st)
    updates_per_step = cells * sum(fsteps.values())
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(args.steps)]
    clocks = ClockSampler()
    barrier(dist)
    torch.cuda.synchronize()
    gf.synchronize()
    clocks.start()
    launches0 = gf.kernel_launches()
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    t_start.record(stream)
    for k in range(args.steps):
        step(evs[k])
    t_end.record(stream)
    gf.synchronize()
    torch.cuda.synchronize()
    clk = clocks.stop()
    barrier(dist)
    launches = gf.kernel_launches() - launches0
    elapsed = t_start.elapsed_time(t_end) / 1e3
    elapsed_max = max_over_ranks(dist, elapsed)
    per_loop = {"source_prop": 0.0, "rtm_forward": 0.0, "rtm_adjoint": 0.0}
    for e in evs:
        per_loop["source_prop"] += e[0].elapsed_time(e[1]) / 1e3
        per_loop["rtm_forward"] += e[1].elapsed_time(e[2]) / 1e3
        per_loop["rtm_adjoint"] += e[2].elapsed_time(e[3]) / 1e3
    value = ws * updates_per_step * args.steps / elapsed_max / 1e9

    # roofline of the dominant kernel (the loop with the largest share)
    bytes_per_cell = {"source_prop": 16, "rtm_forward": 32, "rtm_adjoint": 36}
    launches_per_loop = {"source_prop": st.nt + 1, "rtm_forward": st.nt, "rtm_adjoint": st.nt}
    kernel_name = {"source_prop": "prop_step_kernel<kSrcProp>", "rtm_forward": "prop_step_kernel<kBornFwd>",
                   "rtm_adjoint": "prop_step_kernel<kRtmAdj>"}
    dom = max(per_loop, key=per_loop.get)
    avg_launch = per_loop[dom] / (launches_per_loop[dom] * args.steps)
    alg_bytes = cells * bytes_per_cell[dom]
    achieved = alg_bytes / avg_launch / 1e9
    peak, peak_kind = peaks()
    traffic, traffic_src = profiled_traffic(dom)
    roof = {"bound": "hbm", "kernel": kernel_name[dom], "achieved": round(achieved, 1),
            "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
            "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
            else "fallback 6.8 TB/s",
            "algorithmic_bytes_per_launch": alg_bytes,
            "avg_launch_ms": round(avg_launch * 1e3, 4),
            "traffic": traffic, "traffic_source": traffic_src,
            "loop_seconds": {k: round(v / args.steps, 4) for k, v in per_loop.items()},
            # every loop's kernel against the same peak (the dominant one is above)
            "per_kernel": {kernel_name[k]: {
                "achieved_gbs": round(cells * bytes_per_cell[k] /
                                      (per_loop[k] / (launches_per_loop[k] * args.steps)) / 1e9, 1),
                "frac": round(cells * bytes_per_cell[k] /
                              (per_loop[k] / (launches_per_loop[k] * args.steps)) / 1e9 / peak, 4),
                "bytes_per_cell": bytes_per_cell[k]} for k in per_loop},
            "loop_gcells": {k: round(cells * fsteps[k] / (per_loop[k] / args.steps) / 1e9, 2)
                            for k in per_loop}}

    # ---------------- e2e through the reference-named C ABI, pinned host buffers
    e2e = None
    if not args.no_e2e:
        def pinned(shape):
            return torch.empty(shape, dtype=torch.float32, pin_memory=True).numpy()
        vol = (n3, n2, n1)
        h_vel, h_img = pinned(vol), pinned(vol)
        h_vel[...] = st.vel2dt2
        h_img[...] = st.img_lap
        h_p0, h_p1, h_im = pinned(vol), pinned(vol), pinned(vol)
        h_zero, h_dat = pinned((nrec, st.nt_big)), pinned((nrec, st.nt_big))
        h_zero[...] = 0
        h_v9, h_v8 = pinned(vals9.shape), pinned(vals8.shape)
        h_v9[...] = vals9
        h_v8[...] = vals8
        L = lib
        i32 = lambda a: np.ascontiguousarray(a, np.int32)

        def e2e_step():
            # create_source_fields (Born/rtm_zero_op_3d.cpp:52-77)
            chk(L.sepx_transfer_source_func(9, h_v9.shape[1], i32(locs9), h_v9))
            chk(L.sepx_transfer_vel_func1(n1, n2, n3, h_vel))
            chk(L.sepx_source_prop(n1, n2, n3, False, True, h_p0, h_p1, st.jts, 9, st.nt))
            # forward (:126-157)
            chk(L.sepx_transfer_source_func(9, h_v8.shape[1], i32(locs8), h_v8))
            chk(L.sepx_transfer_vel_func1(n1, n2, n3, h_vel))
            chk(L.sepx_transfer_vel_func2(n1, n2, n3, h_vel))
            chk(L.sepx_transfer_receiver_func(st.rnx, st.rny, st.nt_big, i32(st.rec_locs), h_zero))
            chk(L.sepx_rtm_forward(n1, n2, n3, st.jtd, h_img, h_dat, 9, st.nt, st.nt_big, st.rnx,
                                   st.rny))
            # adjoint (:228-262): source fields read back swapped
            chk(L.sepx_transfer_source_func(9, h_v8.shape[1], i32(locs8), h_v8))
            chk(L.sepx_transfer_vel_func1(n1, n2, n3, h_vel))
            chk(L.sepx_transfer_receiver_func(st.rnx, st.rny, st.nt_big, i32(st.rec_locs), h_dat))
            chk(L.sepx_rtm_adjoint(n1, n2, n3, st.jtd, h_p1, h_p0, h_im, 9, st.nt))

        e2e_step()   # warm
        barrier(dist)
        # one sample a second here: polling every 200 ms slowed the host-buffer
        # Born forward of this step by 0.4-0.5 s (8.50 -> 8.95-9.15 s per step,
        # the device-resident loops were unaffected)
        e2e_clocks = ClockSampler(interval_ms=args.e2e_clock_ms) if args.e2e_clock_ms > 0 else None
        if e2e_clocks:
            e2e_clocks.start()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e2e_step()
        e_el = max_over_ranks(dist, time.perf_counter() - t0)
        e2e_clk = e2e_clocks.stop() if e2e_clocks else None
        vb = 4 * n1 * n2 * n3
        tb = 4 * nrec * st.nt_big
        h2d = 3 * vb + vb + 2 * vb + 2 * tb + 4 * (h_v9.size + 2 * h_v8.size)
        d2h = 2 * vb + tb + vb
        e2e = {"value": round(ws * updates_per_step * args.steps / e_el / 1e9, 3), "unit": "Gcell/s",
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
               "ms_per_step": round(e_el / args.steps * 1e3, 2),
               "path": "reference-named C ABI (sepx_source_prop / sepx_rtm_forward / "
                       "sepx_rtm_adjoint) with pinned host buffers",
               "clocks": e2e_clk}

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        cpu = cpu_baseline(s, st, args.cpu_sample_steps)
        cpu["value"] = round(cpu["value"], 4)

    out = {
        "metric": "Gcell-updates/s (full single-shot RTM: Born forward + source propagation + "
                  "RTM adjoint)",
        "value": round(value, 3), "unit": "Gcell/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(elapsed_max / args.steps * 1e3, 2),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded layered 1500-4500 m/s model, 8 dipping interfaces, 20 Hz Ricker)",
        "config": workload_config(args, st, ws),
        "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "clocks": clk,
        "gpu_launches": int(launches),
    }
    if rank == 0:
        print(json.dumps(out))


# ------------------------------------------------------------------ batched shots
def run_batch(args):
    """16 uneven-window shots on a 1024 x 1024 x 400 model: source_prop, Born
    forward and RTM adjoint of every shot, shot after shot (the reference's
    shot loops) against one launch per step for all shots, with and without a
    captured CUDA graph, after the autotuner picked the Born forward's launch
    style, z-chunk and ring depth."""
    import torch
    from sep_code_gb300 import batch as Bt
    nt = args.batch_nt
    t0 = time.perf_counter()
    surveys = Bt.windowed_surveys(nt=nt)
    b = Bt.BatchRTM(surveys)
    t_setup = time.perf_counter() - t0
    stream = torch.cuda.ExternalStream(Bt.lib.sepx_get_stream())
    loops = ("source_prop", "forward", "adjoint")
    updates = b.cell_updates(loops)
    out = {"metric": "Gcell-updates/s (batched RTM, 16 shots: source_prop + Born forward + adjoint)",
           "unit": "Gcell/s", "n_gpus": 1, "higher_is_better": True, "dtype": "f32",
           "data": "synthetic",
           "config": {"workload": "batch_16_shots_1024x1024x400", "nt": nt,
                      "windows": [list(s.vel.shape[::-1]) for s in surveys],
                      "padded": ["x".join(map(str, st.n)) for st in b.setups],
                      "cells_per_field_step": int(sum(b.cells))},
           "setup_seconds": round(t_setup, 1)}
    z, st_, sty, ms = b.autotune(nsteps=8)
    out["autotune"] = {"zchunk": z, "stages": st_, "style": ["all-tiles", "persistent"][sty],
                       "ms_per_step": round(ms, 4)}
    res = {}
    clocks = ClockSampler()
    clocks.start()
    for how in ("sequential", "persistent", "graph", "graph"):
        b.set_images()   # the previous adjoint wrote its image into the forward's input
        torch.cuda.synchronize()
        evs = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        evs[0].record(stream)
        b.source_prop(how)
        evs[1].record(stream)
        b.zero_traces()
        b.forward(how)
        evs[2].record(stream)
        b.adjoint(how)
        evs[3].record(stream)
        evs[3].synchronize()
        sec = evs[0].elapsed_time(evs[3]) / 1e3
        key = how if how not in res else how + "_replay"
        res[key] = {"seconds": round(sec, 4), "gcells": round(updates / sec / 1e9, 2),
                    "loop_seconds": {k: round(evs[i].elapsed_time(evs[i + 1]) / 1e3, 4)
                                     for i, k in enumerate(loops)}}
    out["clocks"] = clocks.stop()
    b.close()
    out["runs"] = res
    out["value"] = res["graph_replay"]["gcells"]
    out["speedup_vs_sequential"] = round(res["sequential"]["seconds"] / res["graph_replay"]["seconds"], 3)
    print(json.dumps(out))


# ------------------------------------------------------------------ reference arm
def run_reference(args, ws, rank):
    """The reference has no CPU propagation; its CPU path is the oracle's
    restatement (oracle/), timed on the host cores with all threads.  Survey,
    random boundary, sinc tables and source stencil come from the oracle's
    own set-up routines: this arm loads no product library."""
    if rank != 0:
        return
    from oracle.bindings import Oracle
    orc = Oracle()
    s, st = build_workload_oracle(args, orc)
    for _ in range(args.warmup):
        cpu_baseline(s, st, max(1, args.cpu_sample_steps // 10), orc)
    vals = []
    secs = 0.0
    for _ in range(args.steps):
        r = cpu_baseline(s, st, args.cpu_sample_steps, orc)
        vals.append(r["value"])
        secs += r["seconds"]
    v = float(np.mean(vals))
    out = {
        "impl": "reference",
        "metric": "Gcell-updates/s (full single-shot RTM: Born forward + source propagation + "
                  "RTM adjoint)",
        "value": round(v, 4), "unit": "Gcell/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(secs / args.steps * 1e3, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded layered 1500-4500 m/s model, 8 dipping interfaces, 20 Hz Ricker)",
        "config": workload_config(args, st, ws),
        "cpu_baseline": {"value": round(v, 4), "unit": "Gcell/s", "cores": r["cores"],
                         "kind": "port", "sample": r["sample"] + " per step"},
        "e2e": {"value": round(v, 4), "unit": "Gcell/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


def main():
    args = parse_args()
    ws, rank, local = dist_env()
    dist = dist_init(ws, local)
    if args.workload == "batch" and args.impl == "ours":
        if rank == 0:
            run_batch(args)
    elif args.impl == "reference":
        run_reference(args, ws, rank)
    else:
        run_ours(args, ws, rank, dist)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
