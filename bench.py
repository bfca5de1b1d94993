#!/usr/bin/env python3
"""Benchmark of the Metropolis trial-move energy path on GB300.

Headline (``value``): aggregate MC moves/s of the batched device-resident
form on 512 independent water chains (N log-uniform in [64, 2048] at
1.0 g/cc, T uniform in [280, 360] K, cutoff min(9, L/2), FP32 pair terms,
FP64 per-move dE and running totals).  One bench step = ``STEPS_PER_BENCH``
Metropolis steps of every chain (one CUDA-graph replay).  Beside it, the
plain single-chain GPU drop-in (the SimulationStep contract driven from the
host with the C library's rand(), one launch per contract call) on the
256-water box, so the batched/plain ratio of the metric is on the line, and
the same plain path with intramolecular moves on a flexible-molecule box
(``flexible``), the single large chains (``single_chain``: 4000 x 16-atom
molecules; ``large_system``: 32,768 waters, NPT, the precision sweep) one
step at a time and in windows of 8 and 16 steps over a thread-block
cluster, and the served request loop (``served``).

``--impl reference`` times the reference's CPU implementation of the path
(the FP64 restatement in oracle/, bit-identical to the compiled reference)
on the host cores with the same workload, metric and unit.

Multi-GPU: replicas only (chains are independent; no collective); each
rank runs its own seeded replica and value = all ranks' moves / max time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = ("MC moves/s: batched+served vs plain 1-chain on same GB300 at \u0394E rel err"
          "\u22641e-5; p99 job")
N_CHAINS = 512
STEPS_PER_BENCH = 64
CHAIN_STEPS = 20000        # steps of each chain of the batched workload
E2E_BENCH_STEPS = 40
WORKLOAD = ("512 independent NVT water chains (3-site TIP3P-like, rigid), N log-uniform in "
            "[64, 2048] at 1.0 g/cc, T uniform in [280, 360] K, cutoff min(9, L/2) A, "
            "+-0.15 A / +-15 deg random-axis moves, Philox proposals, on-device accept")
FP32_FLOPS_PER_PAIR = 38   # per atom pair, fixed by convention from the reference's arithmetic
# DRAM bytes (read + write) per launch of k_chain_steps on this workload,
# measured with ncu (dram__bytes_read.sum + dram__bytes_write.sum, mean of six
# launches after the untimed steps, L2 flushed between bench steps), by tile
# (threads, chains per CTA, steps per launch, lanes per molecule), each with
# the version of the chain kernel it was captured on.  A capture is reported
# only for its own tile and kernel version; otherwise the line's traffic is
# null and says why (a launch reads the chains' rows about once whatever the
# tile, ~34 MB, but a figure from another tile or kernel is not this run's).
CHAIN_KERNEL_VERSION = ("pair code shared by both placements, LJ mask in the header, FP32-only "
                        "step, FP64 re-takes from per-atom blending rows and one rsqrt")
# (the re-take's screen reusing the step's FP32 screen changed no row a launch
# reads outside the rare re-takes; the capture above stands for it)
CHAIN_TRAFFIC_BYTES = {(160, 1, 64, 1): (33.97e6, CHAIN_KERNEL_VERSION)}


def chain_traffic(tile):
    """(bytes per launch, note): the capture of this tile on the current
    kernel version, else (None, why not)."""
    hit = CHAIN_TRAFFIC_BYTES.get(tuple(tile))
    if hit is None:
        return None, "no ncu capture of this tile"
    if hit[1] != CHAIN_KERNEL_VERSION:
        return None, "the capture of this tile predates the current chain kernel"
    return hit[0], "ncu capture of this tile and kernel version"
# L2 sector throughput peak implied by the same captures: lts__t_sectors.sum.per_second
# (32 B sectors) over lts__t_sectors.sum.pct_of_peak_sustained_elapsed (36.25 and 36.37
# TB/s on the two tiles); MEASURED_PEAKS.json holds no L2 figure
L2_PEAK_GBS = 36300.0
ATOMS_PER_WATER = 3


def fp32_peak_tflops(sm_count: int = 152, mhz: float = 2070.0) -> float:
    """Nominal FP32 CUDA-core peak: SMs x 128 lanes x 2 flop x clock
    (MEASURED_PEAKS.json holds no FP32 figure)."""
    return sm_count * 128 * 2 * mhz * 1e6 / 1e12


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def dist_init(ws):
    if ws <= 1:
        return None
    import torch.distributed as dist
    dist.init_process_group("gloo")
    return dist


def dist_max(dist, v: float) -> float:
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_sum(dist, v: float) -> float:
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


# ---- CPU baseline -------------------------------------------------------------

CPU_STEPS_PER_CALL = 200   # MC steps of every chain per timed call of the CPU path


def cpu_baseline(boxes, seeds, target_s: float = 12.0, threads: int | None = None) -> dict:
    """The reference's algorithm (FP64 restatement, oracle/) on the host
    cores: every chain of the workload advanced by the same Philox moves,
    chains spread over all threads, CPU_STEPS_PER_CALL steps of every chain
    per call; calls repeated until about target_s seconds (a bounded
    sample)."""
    from oracle.pyoracle import OracleBox, chains_run_mt
    threads = threads or os.cpu_count() or 1
    obs = [OracleBox(b) for b in boxes]
    chains_run_mt(obs, seeds, 1, 1, threads, step0=0)    # warm-up: one step per chain
    step, moves, calls = 1, 0, 0
    t0 = time.perf_counter()
    while True:
        moves += chains_run_mt(obs, seeds, CPU_STEPS_PER_CALL, 1, threads, step0=step)
        step += CPU_STEPS_PER_CALL
        calls += 1
        dt = time.perf_counter() - t0
        if dt >= target_s:
            break
    return {"value": moves / dt, "unit": "moves/s", "cores": threads, "kind": "port",
            "sample": f"{len(boxes)} chains x {calls} x {CPU_STEPS_PER_CALL} steps "
                      f"({moves} moves) in {dt:.2f} s"}


def _product_library_mapped() -> bool:
    """True if this process has the product's CUDA library mapped."""
    try:
        return "libmcgpu_gb300" in Path("/proc/self/maps").read_text()
    except OSError:
        return False


def run_reference(args, ws, rank):
    """--impl reference: rank 0 times the reference's CPU path on the host:
    the FP64 restatement (oracle/, bit-identical to the reference compiled
    from its sources) on the same 512-chain workload, every bench step one
    call advancing every chain by CPU_STEPS_PER_CALL steps on all host
    threads.  The workload is built with the oracle's own centre builder, so
    this arm never loads the product library (checked)."""
    if rank != 0:
        return
    from mcgpu_gb300 import workloads as W
    from oracle.pyoracle import OracleBox, build_centres, chains_run_mt
    boxes, seeds = W.batch_water_512(seed=2024, centres=build_centres)
    if _product_library_mapped():
        raise RuntimeError("the reference arm must not load the product library")
    threads = os.cpu_count() or 1
    obs = [OracleBox(b) for b in boxes]
    per_step = CPU_STEPS_PER_CALL
    step = 0
    for _ in range(args.warmup):
        chains_run_mt(obs, seeds, per_step, 1, threads, step0=step)
        step += per_step
    t0 = time.perf_counter()
    moves = 0
    for _ in range(args.steps):
        moves += chains_run_mt(obs, seeds, per_step, 1, threads, step0=step)
        step += per_step
    dt = time.perf_counter() - t0
    v = moves / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "moves/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000 * dt / max(1, args.steps), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "chains": N_CHAINS,
                   "steps_per_bench_step": per_step,
                   "note": "reference CPU path as its FP64 restatement (oracle/mcgpu_oracle.c, "
                           "bit-identical to the compiled reference, which is built only where "
                           "the reference sources are); chains over all host threads; workload "
                           "built without the product library"},
        "cpu_baseline": {"value": v, "unit": "moves/s", "cores": threads, "kind": "port",
                         "sample": f"{N_CHAINS} chains x {args.steps} x {per_step} steps "
                                   f"({moves} moves) in {dt:.2f} s"},
        "e2e": {"value": v, "unit": "moves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---- plain single-chain drop-in ---------------------------------------------------

FP64_PEAK_TFLOPS = 1.25    # nominal GB300 FP64 (no measured FP64 figure in MEASURED_PEAKS.json)


def bench_plain(ctx, n_steps: int = 2000) -> dict:
    """The SimulationStep contract on the GPU driven from the host, as
    metrosim's loop drives it: one launch (and one D2H scalar) per energy
    call, one launch per move and per rollback; 256 waters (the CPU-runnable
    reference configuration).  Two hosts of the loop: the library's C++
    (mcgpu_run_plain, the calls a GpuBruteForceStep makes under the
    reference's own loop) and the Python mirror (step.py), both with the
    C library's rand() draws.  The C++ entries carry the device-counted pair
    work and its roofline (FP64 pairs against the nominal FP64 peak, FP32
    pairs against the nominal FP32 peak)."""
    import mcgpu_gb300 as M
    box = M.water_box(256, L=19.71, seed=12345)
    out = {"cpp": {}, "python": {}}
    for name, prec, fused in (("fp64", M.PREC_FP64, False), ("fp64_fused", M.PREC_FP64, True),
                              ("mixed", M.PREC_MIXED, False),
                              ("mixed_fused", M.PREC_MIXED, True)):
        g = M.GpuBox(ctx, box, prec)
        g.run_plain_native(41, 50, fused=fused)            # warm-up
        t0 = time.perf_counter()
        st = g.run_plain_native(42, n_steps, fused=fused)
        dt = time.perf_counter() - t0
        g.close()
        peak = FP64_PEAK_TFLOPS if prec == M.PREC_FP64 else fp32_peak_tflops()
        achieved = st.pairs * FP32_FLOPS_PER_PAIR / dt / 1e12
        out["cpp"][name] = {"moves_per_s": n_steps / dt, "accepted": st.accepted,
                            "steps": n_steps, "pairs_per_move": st.pairs / n_steps,
                            "roofline": {"bound": "fp64" if prec == M.PREC_FP64 else "fp32",
                                         "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                                         "frac": achieved / peak}}
    out["device"] = {}
    for name, prec in (("fp64", M.PREC_FP64), ("mixed", M.PREC_MIXED)):
        g = M.GpuBox(ctx, box, prec)
        g.run_plain_device(41, 200)                          # warm-up
        n_dev = 10 * n_steps
        t0 = time.perf_counter()
        st = g.run_plain_device(42, n_dev)
        dt = time.perf_counter() - t0
        g.close()
        out["device"][name] = {"moves_per_s": n_dev / dt, "accepted": st.accepted,
                               "steps": n_dev, "pairs_per_move": st.pairs / n_dev}
    # an ensemble of the same box, one per CTA, two CTAs per SM, own seeds
    n_boxes = 2 * ctx_sm_count()
    for name, prec, n_ens in (("ensemble_mixed", M.PREC_MIXED, 2000),
                              ("ensemble_fp64", M.PREC_FP64, 500)):
        gs = [M.GpuBox(ctx, box, prec) for _ in range(n_boxes)]
        M.run_plain_device_many(gs, range(1, n_boxes + 1), 20)      # warm-up
        t0 = time.perf_counter()
        res = M.run_plain_device_many(gs, range(101, n_boxes + 101), n_ens)
        dt = time.perf_counter() - t0
        out["device"][name] = {"moves_per_s": n_boxes * n_ens / dt, "boxes": n_boxes,
                               "steps": n_ens,
                               "pairs_per_move": sum(r.pairs for r in res) / (n_boxes * n_ens)}
        for g in gs:
            g.close()
    for name, prec, fused in (("fp64", M.PREC_FP64, False), ("mixed", M.PREC_MIXED, False),
                              ("mixed_fused", M.PREC_MIXED, True)):
        g = M.GpuBox(ctx, box, prec)
        step = M.GpuSimulationStep(g, M.LibcRand(42))
        M.run_plain(step, 50, fused=fused)      # warm-up
        t0 = time.perf_counter()
        res = M.run_plain(step, n_steps, fused=fused)
        dt = time.perf_counter() - t0
        out["python"][name] = {"moves_per_s": n_steps / dt, "accepted": res.accepted,
                               "steps": n_steps}
        g.close()
    out["note"] = ("roofline peaks are nominal (FP64 1.25 TFLOP/s, FP32 152 SMs x 128 x 2 x "
                   "2.07 GHz); the plain form is launch- and sync-bound by design: one launch "
                   "and one D2H sync per contract call; 'device' runs the same loop (same "
                   "rand() stream, restated on the device) on one CTA with no host round trip")
    return out


def ctx_sm_count() -> int:
    import torch
    return torch.cuda.get_device_properties(0).multi_processor_count


def bench_flex(ctx, n_steps: int = 3000, cpu_target_s: float = 3.0) -> dict:
    """Flexible molecules: the plain path with intramolecular moves on (the
    reference's code behind ENABLE_INTRA), 512 molecules (256 amine chains
    with every bond and angle variable, 256 rigid waters; the synthetic
    stand-in for the reference's flexible example, 500 methanols).  Every
    step: molecule energies with the intramolecular term, the rigid move,
    a random set of bond stretches and of angle expansions with their MC
    tests, the width tuning every 1000 steps, accept or roll back (lengths
    and sizes too); rand() draws in the reference's order.  GPU: the
    library's C++ loop (two waits a step), FP64 and FP32 intermolecular
    pairs (intramolecular terms FP64), and the Python mirror making the
    contract calls one by one.  CPU baseline: the oracle's loop (the
    reference's arithmetic, one core) on the same box, a bounded sample."""
    import mcgpu_gb300 as M
    box, topo = M.workloads.flex_amine_water(512)
    out = {"workload": f"{box.n_mol} molecules (256 flexible 9-atom amine chains, 256 rigid "
                       f"waters), {topo.n_bond} bonds, {topo.n_angle} angles, L = "
                       f"{box.size[0]:.2f} A, rc {box.cutoff} A, {box.temperature} K",
           "unit": "moves/s"}
    for name, prec in (("cpp_fp64", M.PREC_FP64), ("cpp_mixed", M.PREC_MIXED)):
        g = M.GpuBox(ctx, box, prec)
        g.set_topology(topo)
        g.set_intra(True)
        g.run_plain_native(41, 100)                          # warm-up
        t0 = time.perf_counter()
        st = g.run_plain_native(42, n_steps)
        dt = time.perf_counter() - t0
        s = g.intra_state()
        out[name] = {"moves_per_s": n_steps / dt, "accepted": st.accepted, "steps": n_steps,
                     "pairs_per_move": st.pairs / n_steps,
                     "bond_width": s["max_bond_delta"], "angle_width": s["max_angle_delta"]}
        g.close()
    for name, prec in (("device_fp64", M.PREC_FP64), ("device_mixed", M.PREC_MIXED)):
        g = M.GpuBox(ctx, box, prec)
        g.set_topology(topo)
        g.set_intra(True)
        g.run_plain_device(41, 100)                          # warm-up
        n_dev = 5 * n_steps
        t0 = time.perf_counter()
        st = g.run_plain_device(42, n_dev)
        dt = time.perf_counter() - t0
        s = g.intra_state()
        out[name] = {"moves_per_s": n_dev / dt, "accepted": st.accepted, "steps": n_dev,
                     "pairs_per_move": st.pairs / n_dev,
                     "bond_width": s["max_bond_delta"], "angle_width": s["max_angle_delta"]}
        g.close()
    # an ensemble: one box per CTA, two CTAs per SM, each its own seed
    n_boxes = 2 * ctx_sm_count()
    for name, prec in (("device_ensemble_mixed", M.PREC_MIXED),
                       ("device_ensemble_fp64", M.PREC_FP64)):
        gs = []
        for _ in range(n_boxes):
            g = M.GpuBox(ctx, box, prec)
            g.set_topology(topo)
            g.set_intra(True)
            gs.append(g)
        n_ens = 1000 if prec == M.PREC_MIXED else 300
        M.run_plain_device_many(gs, range(1, n_boxes + 1), 20)      # warm-up
        t0 = time.perf_counter()
        res = M.run_plain_device_many(gs, range(101, n_boxes + 101), n_ens)
        dt = time.perf_counter() - t0
        out[name] = {"moves_per_s": n_boxes * n_ens / dt, "boxes": n_boxes, "steps": n_ens,
                     "accepted": int(sum(r.accepted for r in res))}
        for g in gs:
            g.close()
    g = M.GpuBox(ctx, box, M.PREC_FP64)
    g.set_topology(topo)
    g.set_intra(True)
    step = M.GpuSimulationStep(g, M.LibcRand(42))
    M.run_plain(step, 50)
    n_py = max(200, n_steps // 3)
    t0 = time.perf_counter()
    res = M.run_plain(step, n_py)
    out["python_fp64"] = {"moves_per_s": n_py / (time.perf_counter() - t0),
                          "accepted": res.accepted, "steps": n_py}
    g.close()
    from oracle.pyoracle import OracleFlex
    o = OracleFlex(box, topo)
    e0 = o.system_energy()
    M.LibcRand(42)
    done, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < cpu_target_s:
        o.run_plain(200, e0)
        done += 200
    out["cpu_baseline"] = {"moves_per_s": done / (time.perf_counter() - t0), "kind": "port",
                           "cores": 1, "sample": f"{done} steps of the oracle's loop"}
    cpu_v = out["cpu_baseline"]["moves_per_s"]
    cores = os.cpu_count() or 1
    out["cpu_ensemble_bound"] = {"moves_per_s": cpu_v * cores, "cores": cores,
                                 "note": "the one-core rate times the host's cores (ideal "
                                         "scaling of independent boxes)"}
    out["gpu_over_cpu"] = {k: out[k]["moves_per_s"] / cpu_v
                           for k in ("cpp_fp64", "cpp_mixed", "device_fp64", "device_mixed")}
    out["ensemble_over_cpu_cores"] = {
        k: out[k]["moves_per_s"] / (cpu_v * cores)
        for k in ("device_ensemble_mixed", "device_ensemble_fp64")}
    out["note"] = ("cpp_*: the host loop over the contract calls, two device waits per step "
                   "(the bond and angle MC tests decide whether rand() is drawn again before "
                   "the next draws); device_*: the same loop on one CTA with the C library's "
                   "generator restated on the device, no host round trip")
    return out


# ---- single chain (4000 x 16-atom bicyclic) and large system (32768 waters) ----------

def timed_chain(g, seed: int, n_steps: int):
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    st, _ = g.chain_run(seed=seed, n_steps=n_steps)
    torch.cuda.synchronize()
    return n_steps / (time.perf_counter() - t0), st


def bench_single(ctx, plain_steps: int = 150, chain_steps: int = 4000) -> dict:
    """4000 rigid 16-atom bicyclic molecules, L = 86.1 A, rc 12 A, 298 K,
    +-0.2 A / +-10 deg: the plain GPU drop-in (host loop over the
    SimulationStep contract, FP64 and FP32 pairs) against the device-resident
    chain (FP32 pairs, FP64 sums, on-device RNG and accept), with and without
    the Verlet list (skin 1.5 A), one step at a time and in windows of 8 and
    16 steps (a thread-block cluster per chain).  Start: FCC lattice (10^3 cells hold the
    4000 centres exactly), one common orientation, as the reference builds
    its boxes; random centres at this density put atoms of neighbours on top
    of each other (energies ~1e19 kcal/mol)."""
    import mcgpu_gb300 as M
    box = M.workloads.bicyclic_4000()
    out = {"workload": "4000 x 16-atom bicyclic, L=86.1 A, rc 12 A, NVT 298 K, single chain"}
    for name, prec in (("plain_fp64", M.PREC_FP64), ("plain_mixed", M.PREC_MIXED)):
        g = M.GpuBox(ctx, box, prec)
        g.run_plain_native(6, 10, fused=True)
        t0 = time.perf_counter()
        g.run_plain_native(7, plain_steps, fused=True)
        out[name] = plain_steps / (time.perf_counter() - t0)
        g.close()
    for name, skin, window in (("chain_full_scan", 0.0, 1), ("chain_verlet", 1.5, 1),
                               ("chain_verlet_w8", 1.5, 8), ("chain_verlet_w16", 1.5, 16)):
        g = M.GpuBox(ctx, box, M.PREC_MIXED)
        if skin > 0:
            g.set_verlet(skin)
        try:
            g.set_window(window)
        except M.MCGPUError as e:
            out[name] = None
            out[name + "_refused"] = str(e)
            g.close()
            continue
        g.chain_run(seed=11, n_steps=64)
        out[name], st = timed_chain(g, 11, chain_steps)
        out[name + "_fp64_retakes"] = st.ties
        if window > 1:
            out[name + "_redo"] = st.window_redo
        g.close()
    win = {k: out.get(f"chain_verlet_w{k}") for k in (8, 16)}
    best = max((k for k in win if win[k]), key=lambda k: win[k], default=None)
    out["chain_verlet_window"] = win[best] if best else None
    out["chain_verlet_window_steps"] = best
    out["window_note"] = ("windows of K steps: one thread-block cluster of K CTAs per chain, "
                          "the K moves evaluated at once against the window's start state and "
                          "decided in step order (a step re-evaluated when an earlier accepted "
                          "step of its window moved its molecule or one within range of it); "
                          "the same decisions and coordinates as one step at a time")
    out["chain_over_plain_fp64"] = (out["chain_verlet_window"] or out["chain_verlet"]) / out["plain_fp64"]
    out["unit"] = "moves/s"
    return out


def bench_large(ctx, steps: int = 200000, interval: int = 500, max_dlnv: float = 0.0015,
                recompute_every: int = 1000) -> dict:
    """32768 waters (98,304 atoms), L = 99.3 A, rc 12 A, NPT 298 K and
    1 atm, Verlet list (skin 1.5 A) rebuilt on the skin/2 trigger, a volume
    move every `interval` steps, `steps` steps from a liquid start (512
    relaxed waters replicated 4 x 4 x 4): the precision sweep.  Two arms
    from the same start with the same Philox streams: FP32 pair terms
    (volume energies FP32 with the threshold re-takes) and FP64 pair terms
    (every step and volume move).  Their decisions are the FP64 ones in
    both, so they follow one trajectory and differ only in the rounding of
    the running energy.  The FP32 arm runs in windows of 8 steps and the
    FP64 arm in windows of 16 (a thread-block cluster of as many CTAs, the
    same decisions as one step at a time); beside them the FP32 arm one step
    at a time for 20,000 steps.  Every `recompute_every` steps a full FP64 system
    energy gives the drift of the running energy, U/N and the density;
    block averages (10 blocks) give <U>/N and <rho> with their standard
    errors.  Beside it the plain FP64 drop-in for a few steps."""
    import numpy as np
    import torch
    import mcgpu_gb300 as M
    from mcgpu_gb300.prepare import relaxed_water_32768
    t0 = time.perf_counter()
    box = relaxed_water_32768(ctx)
    t_relax = time.perf_counter() - t0
    n = box.n_mol
    out = {"workload": f"32768 waters, L=99.3 A, rc 12 A, NPT 298 K / 1 atm, Verlet skin 1.5 A, "
                       f"volume move every {interval} steps (ln V step +-{max_dlnv}), {steps} steps",
           "start": "512 waters relaxed by the chain kernel (400 sweeps, NVT 298 K, rc 9 A) at "
                    "the same density, replicated 4 x 4 x 4",
           "relax_s": t_relax, "unit": "moves/s"}

    def block(x, nb=10):
        x = np.asarray(x, np.float64)
        b = x[: len(x) - len(x) % nb].reshape(nb, -1).mean(axis=1)
        return float(b.mean()), float(b.std(ddof=1) / math.sqrt(nb))

    # one step at a time (one group of 16 warps), FP32 pairs, for comparison
    bt = M.ChainBatch(ctx, [box], [0x5EED], rotation=M.ROT_AXIS)
    bt.set_tile(512, 1, 64)
    bt.set_verlet(1.5)
    bt.set_npt(interval, 1.0, max_dlnv, M.PREC_MIXED)
    n1 = min(steps, 20000)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    bt.run(n1)
    torch.cuda.synchronize()
    out["fp32_pairs_one_step_moves_per_s"] = n1 / (time.perf_counter() - t1)
    out["fp32_pairs_one_step_steps"] = n1
    bt.close()

    def windowed(bt, k):
        """Windows of k steps (a cluster of k CTAs), else the largest that fits."""
        for w in (k, 8, 4, 2, 1):
            if w > k:
                continue
            try:
                bt.set_window(w)
                return w
            except M.MCGPUError:
                pass
        return 1

    coords = {}
    for name, prec, want in (("fp32_pairs", M.PREC_MIXED, 8), ("fp64_pairs", M.PREC_FP64, 16)):
        bt = M.ChainBatch(ctx, [box], [0x5EED], rotation=M.ROT_AXIS)
        bt.set_tile(512, 1, 64)          # one chain: groups of 16 warps
        window = windowed(bt, want)
        bt.set_verlet(1.5)
        bt.set_npt(interval, 1.0, max_dlnv, prec)
        bt.set_precision(prec)
        run_s, drift, u, rho = 0.0, [], [], []
        for _ in range(steps // recompute_every):
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            bt.run(recompute_every)
            torch.cuda.synchronize()
            run_s += time.perf_counter() - t1
            st = bt.stats()[0]
            full = float(bt.system_energies()[0])
            vol = st.box[0] * st.box[1] * st.box[2]
            drift.append((st.energy - full) / abs(full))
            u.append(full / n)
            rho.append(n / vol)
        st = bt.stats()[0]
        coords[name] = bt.download_all()[0]
        bt.close()
        mu, su = block(u)
        mr, sr = block(rho)
        out[name] = {"moves_per_s": steps / run_s, "run_s": run_s, "window_steps": window,
                     "window_redo": st.window_redo,
                     "drift_rel_final": drift[-1], "drift_rel_max": max(abs(d) for d in drift),
                     "drift_series_every_steps": recompute_every,
                     "drift_rel_series": [float(f"{d:.3e}") for d in drift[:: max(1, len(drift) // 20)]],
                     "U_per_molecule": mu, "U_per_molecule_se": su,
                     "density_mol_per_A3": mr, "density_se": sr,
                     "acceptance": st.accepted / steps,
                     "volume_moves": st.vol_tried, "volume_accepted": st.vol_accepted,
                     "edge_A": st.box[0], "nl_builds": st.nl_builds,
                     "nl_full_scan_steps": st.nl_full_scans, "fp64_steps": st.ties,
                     "error": st.error}
    a, b = out["fp32_pairs"], out["fp64_pairs"]
    out["same_trajectory"] = all(np.array_equal(p, q) for p, q in
                                 zip(coords["fp32_pairs"], coords["fp64_pairs"]))
    out["U_z"] = abs(a["U_per_molecule"] - b["U_per_molecule"]) / max(
        math.hypot(a["U_per_molecule_se"], b["U_per_molecule_se"]), 1e-300)
    out["density_z"] = abs(a["density_mol_per_A3"] - b["density_mol_per_A3"]) / max(
        math.hypot(a["density_se"], b["density_se"]), 1e-300)
    out["chain_verlet_npt"] = a["moves_per_s"]
    g = M.GpuBox(ctx, box, M.PREC_FP64)
    g.run_plain_native(2, 5, fused=True)
    t0 = time.perf_counter()
    g.run_plain_native(3, 60, fused=True)
    out["plain_fp64"] = 60 / (time.perf_counter() - t0)
    g.close()
    return out


# ---- served request loop ---------------------------------------------------------------

def bench_served(ctx, rate: float = 200.0, window_s: float = 60.0, steps_per_job: int = 20000,
                 tile=(256, 1, 0),
                 pool_each: int = 32, seed: int = 77) -> dict:
    """Jobs arrive as a Poisson stream (rate jobs/s over window_s seconds),
    50/50 water and 16-atom bicyclic, N log-uniform in [128, 8192], NPT at
    1 atm with T uniform in [280, 360] K, a ln V move (+-0.01) every 100
    steps, steps_per_job steps each; admitted against a 120 GB budget and
    advanced by the server's rounds.  Boxes come from a pre-built pool
    (pool_each per species; water from random centres, the 16-atom molecule
    on an FCC lattice) with per-job temperature and Philox key."""
    import numpy as np
    import mcgpu_gb300 as M
    rng = np.random.default_rng(seed)
    pool = []
    for k in range(pool_each):
        n = int(round(math.exp(rng.uniform(math.log(128), math.log(8192)))))
        pool.append(M.water_box(n, cutoff=9.0, seed=1000 + k))
        n = int(round(math.exp(rng.uniform(math.log(128), math.log(8192)))))
        pool.append(M.bicyclic_box(n, seed=2000 + k, lattice=True))
    for b in pool:
        b.cutoff = min(b.cutoff, 0.5 * float(b.size[0]))
    arrivals = []
    t = 0.0
    while True:
        t += rng.exponential(1.0 / rate)
        if t > window_s:
            break
        arrivals.append(t)
    srv = M.JobServer(ctx, hbm_budget_bytes=120 << 30, max_slots=512, round_steps=100,
                      max_mol_atoms=16, max_atoms=24_000_000, max_molecules=4_000_000,
                      tile=tile)
    jobs = []
    for i, ta in enumerate(arrivals):
        b = pool[int(rng.integers(len(pool)))].copy()
        b.temperature = float(rng.uniform(280.0, 360.0))
        jobs.append((ta, b, int(rng.integers(1, 2 ** 63)), i))
    done = {}
    t0 = srv.clock()
    nxt = 0
    while len(done) < len(jobs):
        now = srv.clock() - t0
        while nxt < len(jobs) and jobs[nxt][0] <= now:
            ta, b, sd, i = jobs[nxt]
            srv.submit(b, sd, steps_per_job, chain_id=i, npt=True, pressure_atm=1.0,
                       max_dlnv=0.01, want_coords=False, vol_precision=M.PREC_MIXED)
            nxt += 1
        st = srv.status()
        if st["running"] == 0 and st["queued"] == 0 and nxt < len(jobs):
            time.sleep(max(0.0, jobs[nxt][0] - (srv.clock() - t0)))
            continue
        srv.step()
        done.update(srv.results())
    lat = sorted(r.result.t_done - r.result.t_submit for r in done.values())
    t_first = min(r.result.t_submit for r in done.values())
    t_last = max(r.result.t_done for r in done.values())
    moves = sum(r.result.steps for r in done.values())
    errors = sum(1 for r in done.values() if r.result.error)
    ties = sum(r.result.ties for r in done.values())
    cnt = srv.counters()
    srv.close()
    pct = lambda q: lat[min(len(lat) - 1, int(q * len(lat)))]
    makespan = t_last - t_first
    capacity = moves / makespan                       # moves/s the server delivered
    demand = rate * steps_per_job                     # moves/s the arrivals ask for
    # achieved pair arithmetic over the GPU time of the rounds (chain kernel +
    # volume phase; the volume phase's pair terms are not in the count, so
    # this understates the work)
    achieved = cnt["pairs"] * FP32_FLOPS_PER_PAIR / max(cnt["gpu_seconds"], 1e-12) / 1e12
    peak = fp32_peak_tflops()
    return {"workload": f"Poisson {rate:.0f} jobs/s for {window_s:.0f} s ({len(jobs)} jobs), 50/50 "
                        "water / 16-atom bicyclic, N log-uniform [128, 8192], NPT 1 atm, "
                        f"T U[280,360] K, ln V move every 100 steps, {steps_per_job} steps/job",
            "window_s": window_s, "arrival_rate_jobs_per_s": rate,
            "jobs": len(jobs), "moves_per_s": capacity, "unit": "moves/s",
            "p50_s": pct(0.50), "p99_s": pct(0.99), "max_s": lat[-1],
            "makespan_s": makespan, "errors": errors, "fp64_retakes": ties,
            "demand_moves_per_s": demand,
            "capacity_jobs_per_s": capacity / steps_per_job,
            "load": demand / capacity,
            "load_note": ("demand above capacity: the queue grows through the window, so p50/p99 "
                          "include the backlog" if demand > capacity else
                          "demand within capacity: p50/p99 are steady-state times"),
            "gpu_seconds": cnt["gpu_seconds"], "rounds": cnt["rounds"],
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak,
                         "unit": "TFLOP/s", "frac": achieved / peak,
                         "work": f"{FP32_FLOPS_PER_PAIR} flop x {cnt['pairs']} device-counted atom "
                                 "pairs of the chain steps over the GPU time of the rounds "
                                 "(volume-phase pairs not counted)"},
            "tile": {"threads": tile[0], "chains_per_cta": tile[1], "lanes_per_molecule": tile[2]},
            "note": f"boxes from a pool of {2 * pool_each} pre-built configurations; "
                    "volume-move energies FP32 pairs with FP64 re-take near the threshold"}


# ---- batched ------------------------------------------------------------------------

def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=4)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--no-single", action="store_true", help="skip the 4000 x 16-atom chain")
    ap.add_argument("--no-large", action="store_true", help="skip the 32768-water system")
    ap.add_argument("--no-served", action="store_true", help="skip the served request loop")
    ap.add_argument("--no-flex", action="store_true",
                    help="skip the flexible-molecule plain path (intramolecular moves)")
    ap.add_argument("--served-window", type=float, default=60.0,
                    help="Poisson arrival window in seconds (60 in the served workload)")
    ap.add_argument("--served-steps", type=int, default=20000)
    ap.add_argument("--served-tile", default="256,1,0",
                    help="threads,chains_per_cta,lanes of the serving loop's chain kernel")
    ap.add_argument("--tile", default=None,
                    help="threads,chains_per_cta,steps_per_launch,lanes (skips the autotuner)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    ws, rank, local = dist_info()
    dist = dist_init(ws)

    if args.impl == "reference":
        run_reference(args, ws, rank)
        return

    import torch
    import mcgpu_gb300 as M
    torch.cuda.set_device(local)
    ctx = M.Context(local)

    boxes, seeds = M.workloads.batch_water_512(seed=2024 + 7919 * rank)
    bt = M.ChainBatch(ctx, boxes, seeds, rotation=M.ROT_AXIS)
    # Each chain runs CHAIN_STEPS steps: the untimed steps before the warm-up
    # and timed ones come first, so the timed steps are the last of every
    # chain's run (relaxed from its random start), not its first.
    pre_steps = max(0, CHAIN_STEPS - (args.warmup + args.steps) * STEPS_PER_BENCH)
    pre_steps -= pre_steps % STEPS_PER_BENCH
    bt.set_tile(160, 1, STEPS_PER_BENCH, 0)
    bt.run(pre_steps, sync=True)
    if args.tile:
        bt.set_tile(*[int(v) for v in args.tile.split(",")])
        tile = bt.tile
    else:
        tile = bt.autotune(128) if not args.no_autotune else bt.tile
    threads, cpc, spl, lanes = tile
    launches_per_step = math.ceil(STEPS_PER_BENCH / spl)

    # The library launches on a torch stream, so CUDA events recorded on that
    # stream bracket exactly the chain kernels of each bench step.
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    # L2 flush buffer (> 129 MB L2), written between timed steps
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            bt.run(STEPS_PER_BENCH, sync=False)
        torch.cuda.synchronize()
        st0 = bt.stats()
        pairs0 = sum(s.pairs for s in st0)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(args.steps)]
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        with ClockSampler(local) as clk:
            wall0 = time.perf_counter()
            for k in range(args.steps):
                flush.fill_(float(k))
                ev[k][0].record(stream)
                bt.run(STEPS_PER_BENCH, sync=False)
                ev[k][1].record(stream)
            torch.cuda.synchronize()
            wall = time.perf_counter() - wall0
        if dist:
            dist.barrier()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    st1 = bt.stats()
    acc_rate = (sum(s.accepted for s in st1) - sum(s.accepted for s in st0)) / (
        N_CHAINS * STEPS_PER_BENCH * args.steps)
    pairs = sum(s.pairs for s in st1) - pairs0
    t_local = sum(step_ms) / 1000.0
    t_max = dist_max(dist, t_local)
    moves_local = N_CHAINS * STEPS_PER_BENCH * args.steps
    moves_all = dist_sum(dist, moves_local)
    value = moves_all / t_max
    kernel_s_per_launch = t_local / (args.steps * launches_per_step)
    flops_per_launch = pairs * FP32_FLOPS_PER_PAIR / (args.steps * launches_per_step)
    pk, src = peaks()
    sm_count = torch.cuda.get_device_properties(local).multi_processor_count
    fp32_peak = sm_count * 128 * 2 * 2.07e9 / 1e12
    achieved = flops_per_launch / kernel_s_per_launch / 1e12
    mean_pairs_per_move = pairs / moves_local
    traffic, traffic_note = chain_traffic((threads, cpc, spl, lanes))
    # 2 n_in a^2 pairs per move (a = 3 on water): 2 n_in a = pairs / a atom rows
    l2_bytes_move = (mean_pairs_per_move / ATOMS_PER_WATER + 2 * ATOMS_PER_WATER) * 16

    ctx.set_stream(None)
    # end to end through the public API: boxes from host memory, run, results back
    e2e = None
    if True:
        torch.cuda.synchronize()
        h2d = sum(b.n_atom * (6 * 8) + b.n_mol * 16 + b.n_pidx * 4 for b in boxes)
        d2h = sum(b.n_atom * 24 for b in boxes) + N_CHAINS * 40
        # a set length (40 bench steps: 2560 moves a chain) whatever --steps
        # is, so the batch creation weighs the same in every run
        e2e_steps = E2E_BENCH_STEPS
        t0 = time.perf_counter()
        b2 = M.ChainBatch(ctx, boxes, seeds, rotation=M.ROT_AXIS)
        b2.set_tile(threads, cpc, spl, lanes)
        b2.run(STEPS_PER_BENCH * e2e_steps, sync=True)
        st_e2e = b2.stats()
        b2.download_all()
        dt_e2e = time.perf_counter() - t0
        b2.close()
        e2e = {"value": N_CHAINS * STEPS_PER_BENCH * e2e_steps / dt_e2e, "unit": "moves/s",
               "h2d_bytes_per_step": h2d / e2e_steps, "d2h_bytes_per_step": d2h / e2e_steps,
               "steps": e2e_steps,
               "note": "create batch from host boxes (incl. initial FP32-pair system energies), "
                       f"{STEPS_PER_BENCH * e2e_steps} steps per chain, all coordinates and "
                       "stats back"}

    plain = None
    if rank == 0 and not args.no_plain:
        plain = bench_plain(ctx)
    single = large = served = flex = None
    if rank == 0 and not args.no_flex:
        flex = bench_flex(ctx)
    if rank == 0 and not args.no_single:
        single = bench_single(ctx)
    if rank == 0 and not args.no_large:
        large = bench_large(ctx)
    if rank == 0 and not args.no_served:
        served = bench_served(ctx, window_s=args.served_window, steps_per_job=args.served_steps,
                              tile=tuple(int(v) for v in args.served_tile.split(",")))
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(boxes, seeds)
    if rank != 0:
        return
    clocks = clk.summary()
    line = {
        "metric": METRIC, "value": value, "unit": "moves/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000 * t_max / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "chains": N_CHAINS,
                   "molecules": sum(b.n_mol for b in boxes),
                   "steps_per_bench_step": STEPS_PER_BENCH,
                   "steps_before_timing": pre_steps + args.warmup * STEPS_PER_BENCH,
                   "chain_steps": CHAIN_STEPS,
                   "acceptance": acc_rate,
                   "tile": {"threads": threads, "chains_per_cta": cpc, "steps_per_launch": spl,
                            "lanes_per_molecule": lanes},
                   "precision": "FP32 pair terms with double-float sums; FP32 decision "
                                "outside a guard band around the threshold, FP64 re-take "
                                "inside it; FP64 running energies",
                   "l2": "flushed between timed steps (256 MiB write); the rows a launch "
                         "reads (anchors, offsets, screen positions: 22.5 MB) come from "
                         "HBM at each step start",
                   "parallelism": "replicas" if ws > 1 else "single GPU"},
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": fp32_peak,
                     "unit": "TFLOP/s", "frac": achieved / fp32_peak,
                     "traffic": traffic,
                     "traffic_unit": "bytes per launch (ncu capture)",
                     "traffic_note": traffic_note,
                     "kernel": "k_chain_steps",
                     "work": f"{FP32_FLOPS_PER_PAIR} flop x {mean_pairs_per_move:.1f} atom pairs "
                             "per move (device-counted, old+new)",
                     "peak_source": "nominal FP32 CUDA-core peak at 2070 MHz "
                                    "(no measured FP32 figure in MEASURED_PEAKS.json)",
                     "hbm_peak_gbs": pk.get("hbm_gbs"), "hbm_peak_source": src,
                     "l2": {"bytes_per_move": l2_bytes_move,
                            "achieved_gbs": value * l2_bytes_move / 1e9,
                            "peak_gbs": L2_PEAK_GBS,
                            "frac": value * l2_bytes_move / 1e9 / L2_PEAK_GBS,
                            "work": "2 n_in a 16 + 2 a 16 bytes per move (float4 rows of the "
                                    "in-range neighbours' atoms and of the moved molecule, "
                                    "both placements)",
                            "peak_source": "ncu L2 sector throughput peak of the k_chain_steps "
                                           "captures"}},
        "gpu_launches": args.steps * launches_per_step,
        "clocks": clocks,
        "e2e": e2e,
        "plain_1chain": plain,
        "batched_over_plain": (value / plain["cpp"]["fp64"]["moves_per_s"]) if plain else None,
        "served": served,
        "served_over_plain": (served["moves_per_s"] / plain["cpp"]["fp64"]["moves_per_s"])
                             if (served and plain) else None,
        "single_chain": single,
        "large_system": large,
        "flexible": flex,
        "cpu_baseline": cpu,
        "wall_s_timed": wall,
    }
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
