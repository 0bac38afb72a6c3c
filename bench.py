"""Throughput of the ideal-MHD Godunov step on GB300: zone-cycles/s.

Workload (one "step" = one RK2 TimeIntegrator cycle): 3-D decaying MHD
turbulence, 256^3 periodic unit box, HLLD + PLM (van Leer) + CT
(uct_contact), RK2, CFL 0.6, FP64 — seeded synthetic initial state (Gaussian
velocity and vector-potential fields, k^-2 on 1 <= |k| <= 8, rms Mach 1,
B = (0.1,0,0) + curl A, beta ~ 10).  The state (1.5 GB) is far larger than
the 129 MB L2, so no flush is needed between cycles.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun (N > 1) every rank advances its own 256^3 box (replicas: the
single-GPU path has no data exchange), value = sum over ranks.  The
reference arm times the CPU implementation of the same path on the host
cores on the same 256^3 workload: the C restatement of the reference's
stage (OpenMP, every host core), pinned bit for bit to the reference's own
kernels - the reference itself needs Kokkos, which its tree does not carry,
and its sources are not present where the bench runs.  Run serially on one
x86 host, the reference's own kernels (compiled against a serial shim of the
Kokkos subset) take 1.18x the time of this restatement per zone-cycle, so
the CPU figure is, if anything, favourable to the CPU.

vs_baseline: value / the reference's published FP64 figure on one H100
(3.08e8 zone-cycles/s, 3-D Orszag-Tang 128^3, doc/source/bench.json:84-90);
that problem and this workload count the same FP64 operations per
zone-cycle to within 2 %.
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

METRIC = "zone-cycles/s (256^3 MHD)"
UNIT = "zone-cycles/s"
H100_PUBLISHED = 3.079643e8  # doc/source/bench.json:84-90 (128^3 per GPU, FP64, H100)
BYTES_PER_ZONE_CYCLE = 320.0  # 8 FP64 state values x 5 transfers per RK2 cycle
# FP64 thread instructions (dadd + dmul + dfma + the rest of the FP64 pipe,
# predicated on) per active cell of one sweep launch, and DRAM bytes per
# active cell of one sweep launch, with the march segment of this workload at
# 256^3 (64 cells): ncu on the 128^3 case with segments 64 (stage 0, the
# three sweep launches of the first cycle), scaled to 256^3 by the columns a
# sweep processes (the CT-extension columns add 1.6 % of the cells at 256^3
# against 3.1 % at 128^3; per processed column-cell the counts are the same
# at one segment length).  Shorter segments reconstruct more cells twice:
# at 128^3 with segments 8 the same sweeps take 526-539 instructions per cell.
FP64_INST_PER_CELL = {"sweep_x": 473.7, "sweep_y": 463.0, "sweep_z": 466.1}
DRAM_BYTES_PER_CELL = {"sweep_x": 224.3, "sweep_y": 176.9, "sweep_z": 177.1}
# FP64 operations per active zone and RK2 cycle of the reference algorithm on
# this workload at 256^3, each add/sub, mul, div and sqrt counted once
# (1465.5 + 1662.8 + 215.5 + 35.8): the operation-counting build of the CPU
# oracle, `python -m oracle.opcount --n 256`.
FP64_FLOP_PER_ZONE_CYCLE = 3379.6


def fp64_flop_roof(value, peak_gops):
    """The algorithmic FP64 rate of one GPU running `value` zone-cycles/s,
    against the FP64 issue rate measured on it (Gop/s), and the zone-cycle
    rate that issue rate allows if every counted operation took a single FP64
    instruction (an upper bound: a correctly rounded division or square root
    takes several)."""
    if not peak_gops or peak_gops <= 0.0:
        return None
    ach = value * FP64_FLOP_PER_ZONE_CYCLE / 1e9
    return {"flop_per_zone_cycle": FP64_FLOP_PER_ZONE_CYCLE, "achieved": ach, "unit": "G FP64 FLOP/s",
            "peak": peak_gops, "frac": ach / peak_gops,
            "ceiling_zone_cycles_per_gpu": peak_gops * 1e9 / FP64_FLOP_PER_ZONE_CYCLE,
            "count_source": "operation-counting build of the CPU oracle on this workload, 256^3"}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--size", type=int, default=256)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-mixed", action="store_true", help="skip the mixed-precision side measurement")
    p.add_argument("--precision", default="fp64", choices=["fp64", "mixed"],
                   help="mixed: FP32 reconstruction + Riemann (profiling runs; the headline is fp64)")
    return p.parse_args()


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region"""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        sm.sort()
        med = sm[len(sm) // 2] if sm else None
        return {"sm_mhz": med, "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(values, world, device="cuda"):
    """element-wise maximum of per-rank timings over the process group (the
    slowest rank sets the whole job's time); identity on one rank"""
    if world <= 1:
        return [float(v) for v in values]
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t.tolist()]


def whole_job_rate(cells_per_rank, steps, world, seconds):
    """zone-cycles/s of the whole job: every rank advances its own box
    (replicas, weak scaling), timed by the slowest rank"""
    return cells_per_rank * steps * world / seconds


def cpu_baseline(size=256, cycles=8, seed=1):
    """the CPU path (oracle restatement, OpenMP on every host core) on a
    bounded sample: the same size^3 workload for `cycles` cycles"""
    from idefix_gb300 import build, ic
    from oracle.pyofx import Oracle

    build.build_oracle()
    threads = os.cpu_count() or 1
    Vc, Vs = ic.turbulence_3d(size, seed=seed)
    o = Oracle(3, (size,) * 3, order="plm", solver="hlld", emf="uct_contact", cfl=0.6,
               first_dt=1e-4, threads=threads, log_period=100, check_nan_period=100)
    o.set_prim(Vc, Vs)
    o.run(max_cycles=1)  # warm-up
    t0 = time.perf_counter()
    o.run(max_cycles=cycles)
    el = time.perf_counter() - t0
    return {"value": size**3 * cycles / el, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"the same {size}^3 workload, {cycles} RK2 cycles after 1 warm-up cycle, "
                      f"{el:.2f} s wall on {threads} threads (C restatement of the reference's stage, "
                      "bit-identical to it)"}


def state_bytes_of(size):
    """bytes of one 256^3-style state in the reference layout: Vc (8 variables,
    2 ghosts a side) and Vs (3 components, one more face per direction)"""
    return 8 * (8 * (size + 4) ** 3 + 3 * (size + 5) ** 3)


def workload_config(size, precision, state_bytes):
    """the `config` of both arms' lines: the workload the metric is quoted on"""
    return {"workload": f"3-D MHD decaying turbulence {size}^3 periodic, HLLD+PLM "
                        "(van Leer)+CT uct_contact, RK2, CFL 0.6, "
                        + ("FP64 bit-identical to the reference" if precision == "fp64"
                           else "mixed precision (FP32 reconstruction, Riemann and EMF averaging, "
                                "FP64 state, ConsToPrim and face update)"),
            "cells_per_gpu": size**3,
            "l2": f"inputs larger than L2 ({state_bytes / 1e9:.2f} GB state), no flush",
            "ic": "seeded Gaussian k^-2, Mach 1, beta 10"}


def run_reference(args, world, rank):
    if rank != 0:
        return
    from idefix_gb300 import build, ic
    from oracle.pyofx import Oracle

    build.build_oracle()
    threads = os.cpu_count() or 1
    size = args.size
    Vc, Vs = ic.turbulence_3d(size, seed=1)
    o = Oracle(3, (size,) * 3, order="plm", solver="hlld", emf="uct_contact", cfl=0.6,
               first_dt=1e-4, threads=threads, log_period=100, check_nan_period=100)
    o.set_prim(Vc, Vs)
    o.run(max_cycles=args.warmup)
    t0 = time.perf_counter()
    o.run(max_cycles=args.steps)
    el = time.perf_counter() - t0
    value = size**3 * args.steps / el
    sample = (f"each step = one RK2 cycle of the {size}^3 workload on the host CPU ({threads} threads; "
              "C restatement of the reference's stage, pinned bit for bit to the reference's kernels)")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": value / H100_PUBLISHED,
            "dtype": "f64", "data": "synthetic",
            "config": workload_config(args.size, "fp64", state_bytes_of(args.size)),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, world, rank, local):
    import torch

    import idefix_gb300 as ig
    from idefix_gb300 import build, ic

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    build.build_library()
    n = (args.size,) * 3
    Vc, Vs = ic.turbulence_3d(args.size, seed=1 + rank)
    stream = torch.cuda.Stream()
    blk = ig.GpuBlock(3, n, order="plm", solver="hlld", emf="uct_contact", nstages=2, cfl=0.6,
                      first_dt=1e-4, log_period=100, check_nan_period=100,
                      precision=args.precision, stream=stream.cuda_stream)
    blk.upload(Vc, Vs)
    blk.autotune(3)  # march segment length per direction (results do not depend on it)
    blk.run(max_cycles=args.warmup)
    cells = args.size**3

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    # ---- device-resident throughput --------------------------------------
    barrier()
    sampler = ClockSampler(local)
    sampler.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    blk.run(max_cycles=args.steps)
    e1.record(stream)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    ms = max_over_ranks([e0.elapsed_time(e1)], world)[0]
    value = whole_job_rate(cells, args.steps, world, ms * 1e-3)
    ms_step = ms / args.steps

    # ---- end to end through the C ABI with host buffers ------------------
    # (a) pipelined: every step takes its own input state from pinned host
    # memory and returns its result state to pinned host memory; the copies
    # run on side streams, double-buffered through device staging arrays, so
    # the host->device copy of step k+1 and the device->host copy of step
    # k-1 overlap the cycle of step k.  Every byte of every step crosses the
    # host link inside the timed region.
    e2e_steps = max(3, min(args.steps, 20))
    h_in, h_out, d_in, d_out = [], [], [], []
    first = blk.download()
    for b in range(2):
        pair = [torch.empty(sh, dtype=torch.float64, pin_memory=True) for sh in (blk.vc_shape, blk.vs_shape)]
        pair[0].numpy()[...] = first[0]
        pair[1].numpy()[...] = first[1]
        h_in.append(pair)
        h_out.append([torch.empty(sh, dtype=torch.float64, pin_memory=True) for sh in (blk.vc_shape, blk.vs_shape)])
        d_in.append([torch.empty(sh, dtype=torch.float64, device="cuda") for sh in (blk.vc_shape, blk.vs_shape)])
        d_out.append([torch.empty(sh, dtype=torch.float64, device="cuda") for sh in (blk.vc_shape, blk.vs_shape)])
    s_h2d, s_d2h = torch.cuda.Stream(), torch.cuda.Stream()
    ev_h2d = [torch.cuda.Event(), torch.cuda.Event()]
    ev_d2h = [torch.cuda.Event(), torch.cuda.Event()]

    def h2d(b):
        with torch.cuda.stream(s_h2d):
            d_in[b][0].copy_(h_in[b][0], non_blocking=True)
            d_in[b][1].copy_(h_in[b][1], non_blocking=True)
            ev_h2d[b].record(s_h2d)

    barrier()
    t0 = time.perf_counter()
    h2d(0)
    for k in range(e2e_steps):
        b = k % 2
        ev_h2d[b].synchronize()                                       # step k's input is on the device
        blk.upload_device(d_in[b][0].data_ptr(), d_in[b][1].data_ptr())
        if k + 1 < e2e_steps:
            h2d((k + 1) % 2)                                          # next input, during this cycle
        blk.cycle()                                                   # one TimeIntegrator::Cycle
        ev_d2h[b].synchronize()                                       # staging b free again
        blk.download_device(d_out[b][0].data_ptr(), d_out[b][1].data_ptr())
        with torch.cuda.stream(s_d2h):                                # result, during the next cycle
            h_out[b][0].copy_(d_out[b][0], non_blocking=True)
            h_out[b][1].copy_(d_out[b][1], non_blocking=True)
            ev_d2h[b].record(s_d2h)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    # (b) synchronous chain: upload, cycle, download, the result fed back
    blk.upload(first[0], first[1])
    hVc, hVs = h_out[0][0].numpy(), h_out[0][1].numpy()
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        blk.upload(hVc, hVs)   # host -> device (pinned), synchronous
        blk.cycle()            # one TimeIntegrator::Cycle (synchronous)
        blk.download((hVc, hVs))  # device -> host
    torch.cuda.synchronize()
    sync_s = time.perf_counter() - t0
    e2e_s, sync_s = max_over_ranks([e2e_s, sync_s], world)
    e2e_value = whole_job_rate(cells, e2e_steps, world, e2e_s)
    e2e_sync_value = whole_job_rate(cells, e2e_steps, world, sync_s)
    state_bytes = hVc.nbytes + hVs.nbytes
    del h_in, h_out, d_in, d_out

    # ---- per-kernel timing (separate run, events around each launch) -----
    blk.profile(True)
    blk.run(max_cycles=3)
    prof = blk.profile_read()
    blk.profile(False)
    prof_cycles = 3
    sweep_classes = ["sweep_x", "sweep_y", "sweep_z"]
    dom = max(prof, key=lambda k: prof[k][0])
    # kernels of the timed cycles: cycle begin/end + per stage: face ghosts,
    # stage begin, 3 sweeps, CT corner, CT faces, stage end; diagnostics on
    # cycles that are multiples of 100 (divB: 2 kernels, NaN: 2 per stage)
    first = args.warmup
    checks = sum(1 for c in range(first, first + args.steps) if c % 100 == 0)
    gpu_launches = args.steps * (2 + 2 * 8) + checks * (2 + 2 * 2)

    hbm_peak, peak_kind = measured_peaks()
    # algorithmic bytes of one launch of a sweep kernel: per active cell it
    # must read the 7 transverse-reconstructed primitives and the normal face
    # field, read and write the 5 conserved hydro variables, and write the
    # two face EMFs and the upwind flag (InvDt is stage-0 only)
    sweep_bytes_per_cell = 8.0 * (7 + 1 + 2 * 5 + 3)
    dom_ms, dom_n = prof[dom]
    dom_avg_s = dom_ms / max(dom_n, 1) * 1e-3
    achieved_gbs = sweep_bytes_per_cell * cells / dom_avg_s / 1e9 if dom in sweep_classes else None
    cycle_gbs = BYTES_PER_ZONE_CYCLE * cells / (ms_step * 1e-3) / 1e9
    traffic = DRAM_BYTES_PER_CELL[dom] * cells if dom in DRAM_BYTES_PER_CELL else None
    # the binding roof: FP64 issue of the dominant sweep against the DFMA
    # throughput measured on this GPU in this run
    fp64_peak = ig.measure_fp64_peak(stream.cuda_stream)
    fp64_roof = None
    if dom in FP64_INST_PER_CELL and args.precision == "fp64":
        ach = FP64_INST_PER_CELL[dom] * cells / dom_avg_s / 1e9
        fp64_roof = {"achieved": ach, "peak": fp64_peak, "unit": "G FP64 thread-op/s", "frac": ach / fp64_peak,
                     "kernel": dom, "inst_per_cell": FP64_INST_PER_CELL[dom],
                     "peak_kind": "measured in this run (DFMA, idfx_measure_fp64_peak)",
                     "inst_source": "ncu FP64-pipe thread instructions per active cell, 128^3 stage-0 sweep "
                                    "with segments 64, scaled to 256^3 by the processed columns"}

    # the same workload in the mixed precision mode (FP32 reconstruction and
    # Riemann solve, FP64 state), for reference beside the FP64 headline
    mixed = None
    if args.precision == "fp64" and not args.no_mixed:
        mblk = ig.GpuBlock(3, n, order="plm", solver="hlld", emf="uct_contact", nstages=2, cfl=0.6,
                           first_dt=1e-4, log_period=100, check_nan_period=100, precision="mixed",
                           stream=stream.cuda_stream)
        mblk.upload(Vc, Vs)
        mblk.autotune(3)
        mblk.run(max_cycles=args.warmup)
        barrier()
        e0.record(stream)
        mblk.run(max_cycles=args.steps)
        e1.record(stream)
        torch.cuda.synchronize()
        mms = max_over_ranks([e0.elapsed_time(e1)], world)[0]
        mixed = {"value": whole_job_rate(cells, args.steps, world, mms * 1e-3), "unit": UNIT,
                 "ms_per_step": mms / args.steps,
                 "dtype": "f32 recon+Riemann / f64 state", "segments": mblk.segments(),
                 "sweep_kernels": mblk.sweep_kernels()}
        # per-kernel time of the mixed cycle (separate run, events around each launch)
        mblk.profile(True)
        mblk.run(max_cycles=3)
        mprof = mblk.profile_read()
        mblk.profile(False)
        mixed["kernel_ms_per_cycle"] = {k: v[0] / 3 for k, v in mprof.items() if v[1]}
        mblk.close()

    out = None
    if rank == 0:
        cpu = None if args.no_cpu_baseline else cpu_baseline(size=args.size)
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": value / world / H100_PUBLISHED,
            "vs_baseline_of": "the reference's published FP64 zone-cycles/s on one H100 (3-D Orszag-Tang 128^3, "
                              "doc/source/bench.json:84-90), per GPU",
            "dtype": "f64" if args.precision == "fp64" else "f32 recon+Riemann / f64 state", "data": "synthetic",
            "config": workload_config(args.size, args.precision, state_bytes),
            "clocks": clocks,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": state_bytes,
                    "d2h_bytes_per_step": state_bytes, "steps": e2e_steps,
                    "how": "per step: its input Vc+Vs from pinned host to the device, "
                           "idfx_gpu_upload_prim_device, one idfx_gpu_cycle, idfx_gpu_download_prim_device, "
                           "its result Vc+Vs to pinned host; copies on side streams, double-buffered, "
                           "overlapping the neighbouring steps' cycles",
                    "sync_chain": {"value": e2e_sync_value,
                                   "how": "upload (pinned, synchronous), one cycle, download, result fed back"}},
            "gpu_launches": gpu_launches,
            "roofline": {"bound": "hbm", "achieved": achieved_gbs, "peak": hbm_peak, "unit": "GB/s",
                         "frac": (achieved_gbs / hbm_peak) if achieved_gbs else None,
                         "traffic": traffic, "kernel": dom, "peak_kind": peak_kind,
                         "bytes_per_cell": sweep_bytes_per_cell,
                         "traffic_note": "ncu dram read+write per active cell of the 128^3 sweep (segments 64), "
                                         "scaled to 256^3 by the processed columns, x 256^3 cells",
                         "note": "FP64-issue bound (GB300 FP64 ~1.2 TFLOP/s): see fp64_roofline"},
            "fp64_roofline": fp64_roof,
            "fp64_flop": fp64_flop_roof(value / world, fp64_peak) if args.precision == "fp64" else None,
            "segments": blk.segments(),
            "cycle_hbm": {"achieved": cycle_gbs, "unit": "GB/s", "frac": cycle_gbs / hbm_peak,
                          "bytes_per_zone_cycle": BYTES_PER_ZONE_CYCLE},
            "kernel_ms_per_cycle": {k: v[0] / prof_cycles for k, v in prof.items() if v[1]},
            "reference_h100_published": H100_PUBLISHED,
            "mixed_precision": mixed,
        }
        if cpu:
            out["cpu_baseline"] = cpu
        print(json.dumps(out), flush=True)
    blk.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return out


def main():
    args = parse()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
        return
    run_ours(args, world, rank, local)


if __name__ == "__main__":
    main()
