"""Benchmark: navigation steps per second on one GB300.

A step is one ComputeStepAndNextVolume (DistanceToOut of the current volume, BVH daughter
intersection, boundary relocation) for every track of the batch. Inputs (points,
directions, located states) are resident in HBM when the timed region starts; `e2e`
repeats the measurement through the host-array C-ABI entry point with the host<->device
copies inside the timed region. The CPU baseline is the oracle (a scalar restatement of
the reference's CPU path) on the host cores over a bounded sample of the same tracks.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
For N > 1 (torchrun) every rank runs an independent replica of the workload (the path has
no exchange step) and rank 0 reports the aggregate.
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

STEP_BYTES = 24 + 24 + 12 + 12 + 8  # p, d, state in, state out, step (FP64 SoA + 12 B states)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="barrel", choices=["barrel"])
    ap.add_argument("--tracks", type=int, default=1 << 22)
    ap.add_argument("--seed", type=int, default=0xC0FFEE)
    ap.add_argument("--cpu-sample", type=int, default=1 << 18)
    return ap.parse_args()


def dist_setup(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        backend = "nccl" if args.impl == "ours" else "gloo"
        dist.init_process_group(backend)
    return ws, rank, local


class ClockSampler:
    """nvidia-smi samples (200 ms) during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": mx, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def make_workload(args, geo_factory):
    from vecgeom_gb300 import workloads as W
    geo = geo_factory()
    W.build_barrel(geo)
    pts, dirs = W.tracks_in_cylinder(args.tracks, seed=args.seed)
    cfg = {"workload": "barrel nav step (1e4 placed volumes, depth 4)", "geometry": "10 tube layers x 64..640 box "
           "modules + sensors, world 4x4x6 m", "tracks": args.tracks, "track_start": "r<30 mm, |z|<500 mm, isotropic",
           "seed": args.seed}
    return geo, pts, dirs, cfg


def cpu_baseline(args, pts, dirs, nthreads):
    """Oracle port on the host cores over a bounded sample of the same tracks."""
    from oracle.oracle import OracleGeometry
    from vecgeom_gb300 import workloads as W
    o = OracleGeometry()
    W.build_barrel(o)
    m = min(args.cpu_sample, len(pts[0]))
    sub = [np.ascontiguousarray(a[:m]) for a in (*pts, *dirs)]
    st, _ = o.locate(*sub[:3], nthreads=nthreads)
    best = None
    for _ in range(3):
        _, _, _, t = o.step(*sub, st, nthreads=nthreads)
        best = t if best is None else min(best, t)
    return {"value": m / best, "unit": "nav steps/s", "cores": nthreads, "kind": "port",
            "sample": "%d of the %d tracks, one step each, best of 3" % (m, len(pts[0]))}


def run_reference(args, ws, rank):
    """CPU implementation of the path (the oracle port; the reference itself needs VecCore,
    which is not available) on all host cores, same metric/config, bounded per step."""
    if rank != 0:
        return
    from oracle.oracle import OracleGeometry
    from vecgeom_gb300 import workloads as W
    nthreads = os.cpu_count() or 1
    o = OracleGeometry()
    W.build_barrel(o)
    pts, dirs = W.tracks_in_cylinder(args.tracks, seed=args.seed)
    m = min(args.cpu_sample, args.tracks)
    sub = [np.ascontiguousarray(a[:m]) for a in (*pts, *dirs)]
    st, _ = o.locate(*sub[:3], nthreads=nthreads)
    for _ in range(args.warmup):
        o.step(*sub, st, nthreads=nthreads)
    times = []
    for _ in range(args.steps):
        _, _, _, t = o.step(*sub, st, nthreads=nthreads)
        times.append(t)
    tot = sum(times)
    value = m * args.steps / tot
    _, _, _, cfg = None, None, None, {"workload": "barrel nav step (1e4 placed volumes, depth 4)",
                                       "tracks": args.tracks, "seed": args.seed}
    line = {"metric": "nav steps/s", "value": value, "unit": "nav steps/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * tot / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)", "config": cfg,
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": "nav steps/s", "cores": nthreads, "kind": "port",
                             "sample": "%d tracks per step of the %d-track batch" % (m, args.tracks)},
            "e2e": {"value": value, "unit": "nav steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    ws, rank, local = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return
    import torch
    import __graft_entry__
    __graft_entry__.build()
    import vecgeom_gb300 as vg

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    geo, pts, dirs, cfg = make_workload(args, vg.Geometry)
    n = args.tracks
    t = [torch.from_numpy(a).to(dev) for a in (*pts, *dirs)]
    st = torch.empty(n * 12, dtype=torch.uint8, device=dev)
    geo.locate_point(t[0], t[1], t[2], st)
    out = torch.empty_like(st)
    step = torch.empty(n, dtype=torch.float64, device=dev)
    status = torch.empty(n, dtype=torch.int32, device=dev)
    torch.cuda.synchronize()

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()

    def timed(flags):
        for _ in range(args.warmup):
            geo.compute_step_and_next_volume(*t, st, out, step, status=status, flags=flags)
        torch.cuda.synchronize()
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(args.steps):
            geo.compute_step_and_next_volume(*t, st, out, step, status=status, flags=flags)
        e1.record()
        torch.cuda.synchronize()
        barrier()
        ms = e0.elapsed_time(e1)
        if ws > 1:
            import torch.distributed as dist
            v = torch.tensor([ms], device=dev)
            dist.all_reduce(v, op=dist.ReduceOp.MAX)
            ms = float(v.item())
        return ms / args.steps

    with ClockSampler(local) as clocks:
        ms_fp64 = timed(vg.PREC_FP64)
    n_err = int((status != 0).sum().item())

    # e2e: host arrays through the C-ABI host entry point (pinned), copies inside the timed region
    hp = [torch.from_numpy(a).pin_memory() for a in (*pts, *dirs)]
    hst = st.cpu().pin_memory()
    hout = torch.empty_like(hst).pin_memory()
    hstep = torch.empty(n, dtype=torch.float64).pin_memory()
    for _ in range(2):
        geo.compute_step_and_next_volume_host(*hp, hst, hout, hstep)
    barrier()
    t0 = time.perf_counter()
    ke = max(3, args.steps // 4)
    for _ in range(ke):
        geo.compute_step_and_next_volume_host(*hp, hst, hout, hstep)
    torch.cuda.synchronize()
    barrier()
    e2e_s = (time.perf_counter() - t0) / ke

    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    value = ws * n / (ms_fp64 * 1e-3)
    achieved = STEP_BYTES * n / (ms_fp64 * 1e-3) / 1e9
    line = {
        "metric": "nav steps/s", "value": value, "unit": "nav steps/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_fp64, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded, generated on the host)",
        "config": dict(cfg, precision="plain FP64", l2="inputs 240 MB > L2 (129 MB); geometry L2-resident by design",
                       parallelism="replicas" if ws > 1 else "single GPU"),
        "e2e": {"value": ws * n / e2e_s, "unit": "nav steps/s", "h2d_bytes_per_step": n * (48 + 12),
                "d2h_bytes_per_step": n * (12 + 8)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "traffic": None,
                     "note": "algorithmic bytes %d B/step; FP64-issue bound kernel (GB300 FP64 ~1.2 TF/s), "
                             "peak %s" % (STEP_BYTES, "of measured" if peaks else "of fallback")},
        "gpu_launches": args.steps,
        "track_errors": n_err,
        "clocks": clocks.summary(),
    }
    if rank == 0:
        line["cpu_baseline"] = cpu_baseline(args, pts, dirs, os.cpu_count() or 1)
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
