"""Benchmark of the shallow-water step on the conformal cubed sphere (GB300).

Workload (one "step" = one RK4 time step): C384 (6 x 384 x 384 interior cells,
halo 3) from the seeded state with orography (spherical harmonics, h = 8000 m +
200 m RMS perturbation, 40 m/s non-divergent wind, orography clipped to
0-2000 m), CFL 0.5.  Metric: interior cell-steps per second of the mixed
FP32/FP64 lane; the FP64 parity lane is measured beside it on the same state.

  value      device-timed throughput, inputs resident in HBM, L2 flushed between
             timed steps (CUDA events on the library's own stream around each
             step: one graph of four stage launches)
  e2e        the same metric through the C ABI with host buffers: every step is
             ccs_set_state_async of its input (pinned host -> device) +
             ccs_step_async(1) + ccs_get_state_async of its result (device ->
             pinned host), one ccs_sync at the end, so one step's copies overlap
             the neighbouring steps; the synchronous calls are reported beside it,
             and the host link's own rates for the same bytes (link_*_gbs)
  roofline   the mixed stage kernel (a quarter of the timed step) against the
             measured HBM copy bandwidth; roofline.issue puts it against the bound
             the kernel actually has, instruction issue
  ensemble   64 x C96 members in one launch per RK stage (graph-captured) against
             the same members stepped one after another
  uneven     16 x C48 + 8 x C96 + 4 x C192 + 1 x C384, FP64 and mixed members in one
             batch (one launch per lane and RK stage)
  cpu_baseline  the CPU FP64 oracle (a restatement of the reference step) on the
             host cores, on a bounded sample of the workload

--impl reference times only the reference CPU step (the oracle) on the same
workload and prints its own line; its inputs come from oracle/case_setup.py, so that
process maps no file of the CUDA library.  Under torchrun (N > 1) every rank
advances its own C384 replica (the single-member step does not shard): value is
the total over ranks divided by the slowest rank's time; the ensemble shards by
member.  --workload ensemble and --workload uneven print only those lines.  Tile
shapes come from the autotuner (--tile-variant pins the mixed one for profiling
runs).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402

N_BENCH = 384
HALO = 3
SEED = 1
# Algorithmic bytes per interior cell-step (RK4, four stages): mixed lane 396 B
# (FP32 state and accumulator, FP64 metric streamed), FP64 lane 600 B.
ALG_BYTES_MIXED = 396.0
ALG_BYTES_FP64 = 600.0


def _dist():
    """(world_size, rank, local_rank) from the torchrun environment (read here, so
    that the reference arm imports nothing of the package)."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.rows = []
        self._stop = threading.Event()
        self._t = None

    def __enter__(self):
        def run():
            while not self._stop.is_set():
                try:
                    out = subprocess.run(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits"], capture_output=True, text=True,
                                         timeout=5).stdout.strip()
                    if out:
                        self.rows.append([x.strip() for x in out.split(",")])
                except Exception:
                    pass
                self._stop.wait(0.2)
        self._t = threading.Thread(target=run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = []
        for k, n in enumerate(names):
            if any(len(r) > 5 + k and r[5 + k].lower() == "active" for r in self.rows):
                reasons.append(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# the sources of the stage kernels whose ncu counters profiles/roofline_traffic.json holds
KERNEL_SOURCES = ("ccs_mixed.cu", "ccs_fp64.cu", "ccs_kernels.h", "ccs_internal.h")


def kernel_sources_hash() -> str:
    """First 16 hex digits of the SHA-256 of the stage kernels' sources."""
    import hashlib
    h = hashlib.sha256()
    for name in KERNEL_SOURCES:
        h.update((ROOT / "conformal_cubed_sphere_gb300" / "csrc" / name).read_bytes())
    return h.hexdigest()[:16]


def profiled_counters() -> dict:
    """The ncu counters of profiles/roofline_traffic.json, only when they were taken on
    this build of the stage kernels (its sources_sha16 equals kernel_sources_hash());
    {} otherwise, so that a kernel edit never leaves stale counters on the line."""
    p = ROOT / "profiles" / "roofline_traffic.json"
    if not p.exists():
        return {}
    try:
        d = json.loads(p.read_text())
    except Exception:
        return {}
    return d if d.get("sources_sha16") == kernel_sources_hash() else {}


def fp64_roofline(avg_ms, fp64_inst, sms, clocks):
    """The FP64 lane's stage kernel against its bound, the FP64 pipe: FP64 thread
    instructions per launch (ncu, committed summary) over the launch time, against
    two FP64 lanes per SM per cycle at the SM clock sampled during the timed region
    (DFMA counted once; 1.26 TFLOP/s counting it as two flops at 2070 MHz)."""
    mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz")
    if not fp64_inst or not mhz:
        return None
    achieved = fp64_inst / (avg_ms * 1e-3)
    peak = 2 * sms * mhz * 1e6
    return {"bound": "fp64 pipe", "achieved": achieved, "peak": peak, "unit": "FP64 thread inst/s",
            "frac": achieved / peak, "fp64_inst_per_launch": fp64_inst}


def issue_roofline(avg_ms, warp_inst, sms, clocks):
    """The stage kernel against its actual bound, instruction issue: warp instructions
    per launch (ncu, committed summary) over the launch time, against one warp
    instruction per cycle on each of the four schedulers of every SM at the SM clock
    sampled during the timed region."""
    mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz")
    if not warp_inst or not mhz:
        return None
    achieved = warp_inst / (avg_ms * 1e-3)
    peak = 4 * sms * mhz * 1e6
    return {"achieved": achieved, "peak": peak, "unit": "warp inst/s", "frac": achieved / peak,
            "warp_inst_per_launch": warp_inst}


def build_case(N=N_BENCH, seed=SEED, oro=True):
    from conformal_cubed_sphere_gb300 import _lib as L
    from conformal_cubed_sphere_gb300 import model as M
    mesh = M.Mesh(N, HALO)
    s = M.initial_state(mesh, kind=L.CCS_IC_SEEDED, seed=seed, lmax_oro=8 if oro else 0)
    dt = M.cfl_dt(mesh, s, 0.5)
    return mesh, s, dt


def time_device_steps(stepper, torch, steps: int, flush: "torch.Tensor"):
    """Per-step CUDA-event timing on the library's stream, L2 flushed in between."""
    st = torch.cuda.ExternalStream(stepper.stream_ptr)
    total = 0.0
    for _ in range(steps):
        with torch.cuda.stream(st):
            flush.add_(1.0)  # writes > L2 bytes
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(st)
        stepper.step_async(1)
        ev1.record(st)
        ev1.synchronize()
        total += ev0.elapsed_time(ev1)
    return total / 1e3  # seconds


def pinned_state(M, mesh, torch, order, fill=None):
    """A model.State whose fields are consecutive slices of one page-locked block, in
    `order` first (then the remaining fields), optionally filled from `fill`."""
    names = list(order) + [k for k in M.STATE_FIELDS if k not in order]
    block = torch.empty(len(names) * mesh.ncell, dtype=torch.float64).pin_memory().numpy()
    arrays = {}
    for q, k in enumerate(names):
        arrays[k] = block[q * mesh.ncell:(q + 1) * mesh.ncell]
        if fill is not None:
            arrays[k][:] = fill[k]
    return M.State(arrays)


def e2e_rate(stepper, mesh, state, steps: int, torch):
    """Per step: ccs_set_state of the step's input (pinned host -> device), ccs_step(1)
    and ccs_get_state of its result (device -> pinned host).  The host fields of a
    state are slices of one page-locked block in the order the lane moves them
    (phi, u, v up; the eight output fields down), so each direction is one copy.
    Three loops: the async entry points (upload of step k+1 and download of result k
    overlap the steps; two result buffers in turn), the same with every field in its
    own pinned array (eleven copies per step), and the synchronous calls one after
    another.  Returns the three loops' wall times and the bytes moved per step each
    way."""
    from conformal_cubed_sphere_gb300 import model as M
    sin = pinned_state(M, mesh, torch, ("phi", "u", "v"), fill=state)
    outs = [pinned_state(M, mesh, torch, M.STATE_FIELDS) for _ in range(2)]
    sep_in = M.State({k: torch.from_numpy(state[k].copy()).pin_memory().numpy() for k in M.STATE_FIELDS})
    sep_outs = [M.State({k: torch.empty(mesh.ncell, dtype=torch.float64).pin_memory().numpy()
                         for k in M.STATE_FIELDS}) for _ in range(2)]
    # inputs the lane uploads / outputs it downloads
    lane_mixed = stepper._cfg.precision == 1
    n_in = 3 if lane_mixed else 8
    n_out = 8

    def run_async(si, so):
        for _ in range(2):  # warm-up
            stepper.set_state_async(si)
            stepper.step_async(1)
            stepper.get_state_async(so[0])
        stepper.sync()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k in range(steps):
            stepper.set_state_async(si)
            stepper.step_async(1)
            stepper.get_state_async(so[k % 2])
        stepper.sync()
        return time.perf_counter() - t0

    el_async = run_async(sin, outs)
    el_sep = run_async(sep_in, sep_outs)
    t0 = time.perf_counter()
    for _ in range(steps):
        stepper.set_state(sin)
        stepper.step(1)
        stepper.get_state(outs[0])
    el_sync = time.perf_counter() - t0
    nb = mesh.ncell * 8
    return el_async, el_sep, el_sync, n_in * nb, n_out * nb


def link_rates(torch, dev: int, h2d_bytes: int, d2h_bytes: int, reps: int = 10) -> dict:
    """The host link alone, for one step's bytes: `reps` pinned uploads of h2d_bytes
    back to back, `reps` pinned downloads of d2h_bytes, and both streams at once (the
    e2e loop's pattern); CUDA events around each run after a warm-up run, per copy.
    The e2e loop cannot move its bytes faster than `both_ms` per step."""
    hin = torch.empty(h2d_bytes, dtype=torch.uint8).pin_memory()
    hout = torch.empty(d2h_bytes, dtype=torch.uint8).pin_memory()
    din = torch.empty(h2d_bytes, dtype=torch.uint8, device=dev)
    dout = torch.empty(d2h_bytes, dtype=torch.uint8, device=dev)
    s_up, s_down = torch.cuda.Stream(dev), torch.cuda.Stream(dev)

    def timed(up: bool, down: bool) -> float:
        ms = 0.0
        for r in range(2):  # the first run warms up
            torch.cuda.synchronize(dev)
            e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
            e0.record(s_up)
            s_down.wait_event(e0)
            for _ in range(reps):
                if up:
                    with torch.cuda.stream(s_up):
                        din.copy_(hin, non_blocking=True)
                if down:
                    with torch.cuda.stream(s_down):
                        hout.copy_(dout, non_blocking=True)
            e1.record(s_up)
            e2.record(s_down)
            torch.cuda.synchronize(dev)
            ms = max(e0.elapsed_time(e1), e0.elapsed_time(e2)) / reps
        return ms

    t_up, t_down, t_both = timed(True, False), timed(False, True), timed(True, True)
    return {"link_h2d_gbs": h2d_bytes / t_up / 1e6, "link_d2h_gbs": d2h_bytes / t_down / 1e6,
            "link_both_ms": t_both, "link_how": "%d pinned copies of the e2e step's bytes back to back per "
                                               "direction, CUDA events, per copy; both = the two directions at "
                                               "once on two streams" % reps}


def cpu_baseline(mesh, state, dt, seconds=10.0):
    """The oracle on all host cores, on a sample of about `seconds` of CPU work:
    as many C384 RK4 steps as one warm-up step says fit (at most 300)."""
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    orc = O.Oracle.from_mesh(mesh, threads=threads)
    orc.set_state(state.arrays)
    t0 = time.perf_counter()
    orc.run(dt, 1)  # warm-up (first touch of the work arrays)
    steps = max(1, min(300, int(seconds / max(time.perf_counter() - t0, 1e-3))))
    t0 = time.perf_counter()
    orc.run(dt, steps)
    el = time.perf_counter() - t0
    cells = 6 * mesh.N * mesh.N
    return {"value": cells * steps / el, "unit": "cell-steps/s", "cores": O.lib().orc_get_threads(),
            "kind": "port",
            "sample": f"{steps} RK4 step(s) of C{mesh.N} FP64 (CPU restatement of the reference step), "
                      f"{el:.1f} s"}


def run_reference(args):
    """The reference CPU step (the oracle) on all host cores.  Its inputs come from
    oracle/case_setup.py (the host set-up code built for the CPU alone), so this
    process maps no file of the CUDA library; they equal the GPU arm's bit for bit."""
    ws, rank, _ = _dist()
    if rank != 0:
        return
    from oracle import case_setup as CS
    from oracle import oracle as O
    mesh, s, dt = CS.seeded_case(N_BENCH, HALO, seed=SEED, lmax_oro=8)
    threads = os.cpu_count() or 1
    orc = O.Oracle.from_mesh(mesh, threads=threads)
    orc.set_state(s)
    # one step = one RK4 step of C384 on all host cores (about 0.1 s on 16 Grace
    # cores); K and W are honoured up to 600 and 5
    steps = max(1, min(args.steps, 600))
    warm = max(1, min(args.warmup, 5))
    orc.run(dt, warm)
    t0 = time.perf_counter()
    orc.run(dt, steps)
    el = time.perf_counter() - t0
    cells = 6 * mesh.N * mesh.N
    v = cells * steps / el
    line = {
        "impl": "reference", "metric": "C384 cell-steps/s", "value": v, "unit": "cell-steps/s",
        "n_gpus": args.gpus, "steps": steps, "warmup": warm, "ms_per_step": 1e3 * el / steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "C384 seeded state with orography, RK4, CFL 0.5", "N": mesh.N, "halo": HALO,
                   "inputs": "oracle/case_setup.py (CPU-only set-up library; no CUDA library mapped)"},
        "cpu_baseline": {"value": v, "unit": "cell-steps/s", "cores": O.lib().orc_get_threads(), "kind": "port",
                         "sample": f"{steps} RK4 steps of C384 after {warm} warm-up step(s)"},
        "e2e": {"value": v, "unit": "cell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def variant_name(lane: str, var: int) -> str:
    """A stage-kernel variant as "<tile> <halo-staging schedule>" (mixed lane) or
    "<tile>" (FP64 lane)."""
    from conformal_cubed_sphere_gb300 import _lib as L
    if lane == "mixed":
        tx, ty, staging = L.MIXED_VARIANTS[var]
        return f"{tx}x{ty} {staging}"
    return ("32x8", "16x16", "64x4")[var]


def _batch_time(batch, torch, steps: int):
    st = torch.cuda.ExternalStream(batch.stream_ptr)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(st)
    batch.step_async(steps)
    ev1.record(st)
    ev1.synchronize()
    return ev0.elapsed_time(ev1) / 1e3


def run_ensemble(torch, members_per_gpu: int, steps: int, warmup: int) -> dict:
    """`members_per_gpu` members at C96 per GPU (seed + k, RMS 150-250 m, wind 30-50
    m/s), mixed lane, one launch per RK stage for all of a rank's members,
    graph-captured; against the same members advanced one after another through
    their own handles.  Under torchrun the ensemble is members x ranks, sharded round
    robin by member with no collective on the data path (weak scaling)."""
    from conformal_cubed_sphere_gb300 import model as M
    from conformal_cubed_sphere_gb300.parallel import shard_members, slowest_rank_seconds
    ws, rank, _ = _dist()
    N = 96
    total = members_per_gpu * ws
    mine = shard_members(total, rank, ws)
    n = len(mine)
    mesh = M.Mesh(N, HALO)
    states = [M.ensemble_member_state(mesh, k, seed=SEED) for k in mine]
    dts = [M.cfl_dt(mesh, st, 0.5) for st in states]
    phibar = 8000.0 * mesh.gravity
    owner = M.Stepper(mesh, dts[0], precision="mixed", phi_mean=phibar)
    members = [owner] + [M.Stepper(mesh, dts[k], precision="mixed", phi_mean=phibar, share_with=owner)
                         for k in range(1, n)]
    for st, m in zip(states, members):
        m.set_state(st)
        m.autotune(reps=5)  # timed once for the grid, then the cached choice
    batch = M.Batch(members)
    batch.autotune(reps=3)
    batch.step(max(warmup, 3))
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    t_batch = slowest_rank_seconds(_batch_time(batch, torch, steps))
    # sequential: the same members, one handle after another
    for m in members:
        m.step(1)
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    for m in members:
        m.step(steps)
    t_seq = slowest_rank_seconds(time.perf_counter() - t0)
    cells = 6 * N * N * total
    launches, groups = batch.info()
    alg = ALG_BYTES_MIXED * cells * steps / t_batch / 1e9
    hbm = _peaks()[0] * ws
    return {
        "member_steps_per_s": total * steps / t_batch, "cell_steps_per_s": cells * steps / t_batch,
        "members": total, "N": N, "steps": steps, "warmup": max(warmup, 3), "ms_per_step": 1e3 * t_batch / steps,
        "sequential_member_steps_per_s": total * steps / t_seq, "batch_over_sequential": t_seq / t_batch,
        "hbm_frac": alg / hbm, "alg_GBs": alg, "launches_per_stage": launches,
        "tile_variant": groups[0][1] if groups else None,
        "variant": variant_name("mixed", groups[0][1]) if groups else None,
        "how": "one graph per step, one persistent launch per RK stage over all members' tiles, CUDA events on "
               "the batch stream; sequential = each member's own handle (graph per step) one after another, "
               "host-timed; inputs larger than L2",
    }


def run_uneven(torch, steps: int, warmup: int) -> dict:
    """16 x C48 + 8 x C96 + 4 x C192 + 1 x C384, per-instance CFL dt; one member of
    each resolution below C384 on the FP64 lane, the others mixed; one batch, one
    launch per lane and RK stage, each lane's tile variant chosen by the batch
    autotuner on its own work list.  Under torchrun every rank advances its own copy."""
    from conformal_cubed_sphere_gb300 import model as M
    from conformal_cubed_sphere_gb300.parallel import slowest_rank_seconds
    ws, rank, _ = _dist()
    groups = [(48, 16), (96, 8), (192, 4), (384, 1)]
    members, cells64, cells32, k = [], 0, 0, 0
    for N, cnt in groups:
        mesh = M.Mesh(N, HALO)
        for c in range(cnt):
            lane = "fp64" if (c == 0 and N < 384) else "mixed"
            st = M.ensemble_member_state(mesh, k, seed=SEED, lmax_oro=8)
            dt = M.cfl_dt(mesh, st, 0.5)
            m = M.Stepper(mesh, dt, precision=lane, phi_mean=8000.0 * mesh.gravity)
            m.set_state(st)
            members.append(m)
            if lane == "fp64":
                cells64 += 6 * N * N
            else:
                cells32 += 6 * N * N
            k += 1
    batch = M.Batch(members)
    batch.autotune(reps=3)
    batch.step(max(warmup, 3))
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    t = slowest_rank_seconds(_batch_time(batch, torch, steps))
    cells = cells64 + cells32
    alg = (ALG_BYTES_FP64 * cells64 + ALG_BYTES_MIXED * cells32) * steps / t / 1e9
    launches, info = batch.info()
    tiles = {"fp64" if lane == 0 else "mixed": var for lane, var, _ in info}
    names = {k: variant_name(k, v) for k, v in tiles.items()}
    # the same mixed members batched without the FP64 ones: the FP64 lane's stages
    # (FP64-pipe bound) pace the mixed batch above
    batch.close()
    mixed_only = M.Batch([m for m in members if m.precision == "mixed"])
    mixed_only.autotune(reps=3)
    mixed_only.step(max(warmup, 3))
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    t32 = slowest_rank_seconds(_batch_time(mixed_only, torch, steps))
    alg32 = ALG_BYTES_MIXED * cells32 * steps / t32 / 1e9
    n32, info32 = mixed_only.info()
    mixed_only.close()
    return {
        "cell_steps_per_s": ws * cells * steps / t, "steps": steps, "warmup": max(warmup, 3),
        "ms_per_step": 1e3 * t / steps, "hbm_frac": ws * alg / (_peaks()[0] * ws), "alg_GBs": ws * alg,
        "launches_per_stage": launches, "tile_variants": tiles, "variants": names, "fp64_cells": cells64,
        "mixed_cells": cells32,
        "instances": len(members),
        "how": "29 instances with per-instance CFL dt, one FP64 member per resolution below C384; one graph per "
               "step, each lane's stages on its own stream; CUDA events on the batch stream",
        "mixed_members_alone": {
            "cell_steps_per_s": ws * cells32 * steps / t32, "ms_per_step": 1e3 * t32 / steps,
            "hbm_frac": alg32 / _peaks()[0], "alg_GBs": ws * alg32, "launches_per_stage": n32,
            "variant": variant_name("mixed", info32[0][1]) if info32 else None,
            "how": "the 26 mixed instances in a batch of their own, same timing"},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="c384", choices=["c384", "ensemble", "uneven"])
    ap.add_argument("--members", type=int, default=64)
    ap.add_argument("--tile-variant", type=int, default=-1,
                    help="mixed-lane tile variant of the C384 run (-1: autotuner)")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--N", type=int, default=N_BENCH)
    ap.add_argument("--fp64-steps", type=int, default=8)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batches", action="store_true", help="skip the ensemble and uneven measurements")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
        return
    ws, rank, local = _dist()
    import torch
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    batch_steps = max(5, min(args.steps, 50))
    if args.workload == "ensemble":
        e = run_ensemble(torch, args.members, args.steps, args.warmup)
        if rank == 0:
            print(json.dumps({
                "metric": f"ensemble member-steps/s ({args.members} x C96 per GPU, mixed lane)",
                "value": e["member_steps_per_s"], "unit": "member-steps/s", "n_gpus": ws, "steps": e["steps"],
                "warmup": e["warmup"], "ms_per_step": e["ms_per_step"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32 (f64 metric transforms)",
                "data": "synthetic (seeded spherical harmonics)",
                "config": {"workload": f"{e['members']} members at C96 ({args.members} per GPU, sharded by member), "
                                       "seed+k, RMS U[150,250] m, wind U[30,50] m/s, RK4, CFL 0.5",
                           "l2": "inputs larger than L2 (all members' state)"},
                "ensemble": e}))
        return
    if args.workload == "uneven":
        u = run_uneven(torch, args.steps, args.warmup)
        if rank == 0:
            print(json.dumps({
                "metric": "uneven batch cell-steps/s (16xC48 + 8xC96 + 4xC192 + 1xC384)",
                "value": u["cell_steps_per_s"], "unit": "cell-steps/s", "n_gpus": ws, "steps": u["steps"],
                "warmup": u["warmup"], "ms_per_step": u["ms_per_step"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32 mixed + f64",
                "data": "synthetic (seeded spherical harmonics)",
                "config": {"workload": "29 instances, per-instance CFL dt, one FP64 member per resolution below "
                                       "C384", "l2": "inputs larger than L2"},
                "uneven": u}))
        return
    from conformal_cubed_sphere_gb300 import model as M

    mesh, s, dt = build_case(args.N)
    cells = 6 * mesh.N * mesh.N
    phibar = 8000.0 * mesh.gravity
    mixed = M.Stepper(mesh, dt, precision="mixed", device=local, phi_mean=phibar)
    mixed.set_state(s)
    if args.tile_variant >= 0:  # fixed (profiling runs: timing under a profiler is not representative)
        mixed.set_variant(args.tile_variant)
        tuned = {"mixed": (args.tile_variant, [])}
    else:
        tuned = {"mixed": mixed.autotune(reps=5)}
    flush = torch.zeros(64 * 1024 * 1024, dtype=torch.float32, device=f"cuda:{local}")  # 256 MB > L2
    mixed.step(max(args.warmup, 3))
    torch.cuda.synchronize()

    def barrier():
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    sampler = ClockSampler(local)
    barrier()
    with sampler:
        t_mixed = time_device_steps(mixed, torch, args.steps, flush)
    barrier()
    from conformal_cubed_sphere_gb300.parallel import slowest_rank_seconds
    t_mixed = slowest_rank_seconds(t_mixed)
    value = ws * cells * args.steps / t_mixed
    ms_step = 1e3 * t_mixed / args.steps
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    counters = profiled_counters()

    # roofline of the dominant kernel (the mixed stage kernel): a quarter of the timed
    # step (events around each step's graph of four launches, so the launch gaps count
    # against the kernel and 4 x kernel time equals the step time)
    avg_ms = ms_step / 4.0
    hbm, peak_kind = _peaks()
    bytes_per_launch = ALG_BYTES_MIXED / 4.0 * cells
    achieved = bytes_per_launch / (avg_ms * 1e-3) / 1e9
    # ncu counters of the variant the autotuner chose (taken at C384 for each mixed variant)
    prof = counters.get("mixed_C384", {}).get(str(mixed.variant[0]), {}) if mesh.N == 384 else {}
    traffic = prof.get("dram_bytes")

    # FP64 parity lane on the same state
    f64 = M.Stepper(mesh, dt, precision="fp64", device=local)
    f64.set_state(s)
    tuned["fp64"] = f64.autotune(reps=2)
    f64.step(1)
    torch.cuda.synchronize()
    t_f64 = time_device_steps(f64, torch, args.fp64_steps, flush)
    fp64_value = cells * args.fp64_steps / t_f64
    ms64 = 1e3 * t_f64 / args.fp64_steps

    # end to end through the C ABI
    e2e_steps = max(3, min(50, args.steps))
    mixed2 = M.Stepper(mesh, dt, precision="mixed", device=local, phi_mean=phibar)
    mixed2.set_state(s)
    mixed2.set_variant(mixed.variant[0])
    if ws > 1:
        torch.distributed.barrier()
    el_async, el_sep, el_sync, h2d, d2h = e2e_rate(mixed2, mesh, s, e2e_steps, torch)
    # every rank moves its own replica's data over its own host link: whole-job rate
    e2e = ws * cells * e2e_steps / slowest_rank_seconds(el_async)
    e2e_sep = ws * cells * e2e_steps / slowest_rank_seconds(el_sep)
    e2e_sync = ws * cells * e2e_steps / slowest_rank_seconds(el_sync)
    link = link_rates(torch, local, h2d, d2h)
    link["link_bound_cell_steps_per_s"] = ws * cells / (link["link_both_ms"] * 1e-3)
    for m in (mixed2,):
        m.close()

    ens = unv = None
    if not args.no_batches:
        ens = run_ensemble(torch, args.members, batch_steps, args.warmup)
        unv = run_uneven(torch, batch_steps, args.warmup)

    if rank != 0:
        return
    clocks = sampler.summary()
    cpu = None if args.no_cpu else cpu_baseline(mesh, s, dt)
    fp64_inst = counters.get("f64_stage_C384_fp64_thread_inst") if (
        mesh.N == 384 and f64.variant[0] == counters.get("f64_variant", 1)) else None
    line = {
        "metric": "C384 cell-steps/s", "value": value, "unit": "cell-steps/s", "n_gpus": ws,
        "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": ms_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32 (f64 metric transforms)",
        "data": "synthetic (seeded spherical harmonics)",
        "config": {"workload": f"C{mesh.N} seeded state with orography, RK4, CFL 0.5, mixed FP32/FP64 lane",
                   "N": mesh.N, "halo": HALO, "dt_s": dt, "l2": "flushed (256 MB write) between timed steps",
                   "parallelism": "replicas" if ws > 1 else "single",
                   "tile_variants": {lane: {"chosen": v, "variant": variant_name(lane, v), "launch_us": t}
                                     for lane, (v, t) in tuned.items()}},
        "fp64_lane": {"value": fp64_value, "unit": "cell-steps/s", "ms_per_step": ms64,
                      "kernel_ms_avg": ms64 / 4.0, "mixed_over_fp64": value / ws / fp64_value,
                      "over_cpu_baseline": (fp64_value / cpu["value"]) if cpu else None,
                      "roofline": fp64_roofline(ms64 / 4.0, fp64_inst, sms, clocks)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": traffic, "kernel": "mixed_stage_kernel", "kernel_ms_avg": avg_ms,
                     "kernel_ms_how": "timed step / 4 (events around each step's graph of four launches)",
                     "alg_bytes_per_launch": bytes_per_launch, "peak_source": peak_kind,
                     "counters_sha16": counters.get("sources_sha16"),
                     "issue": issue_roofline(avg_ms, prof.get("warp_inst"), sms, clocks)},
        "e2e": {"value": e2e, "unit": "cell-steps/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "how": "ccs_set_state_async + ccs_step_async(1) + ccs_get_state_async per step, each state's "
                       "fields in one pinned host block (one copy per direction), one ccs_sync at the end",
                "separate_field_arrays": e2e_sep, "synchronous_calls": e2e_sync, **link},
        "ensemble": ens,
        "uneven": unv,
        "gpu_launches": 4 * args.steps,
        "clocks": clocks,
        "cpu_baseline": cpu,
    }
    print(json.dumps(line))


if __name__ == "__main__":
    main()
