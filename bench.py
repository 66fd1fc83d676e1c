"""Benchmark: navigation steps per second on one GB300.

A step is one ComputeStepAndNextVolume (DistanceToOut of the current volume, BVH daughter
intersection, boundary relocation) for every track of the batch. The default workload is
the config-4 detector (150k box modules in a 20-layer barrel + two endcaps of Polycone
holders with Trd wedges); the 2^22 step inputs are drawn from straight-track transport
histories generated on the GPU, so they cover every kind of volume. Inputs are resident in
HBM when the timed region starts; `e2e` repeats the measurement through the host-array
C-ABI entry point with the host<->device copies inside the timed region. The CPU baseline
is the oracle (a scalar restatement of the reference's CPU path) on the host cores over a
bounded sample of the same step inputs.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                       [--workload detector|barrel]
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

METRIC = "nav steps/s on 1 GB300, plain FP64 vs mixed-prec+learned order, ids identical"
UNIT = "nav steps/s"
STEP_BYTES = 24 + 24 + 12 + 12 + 8  # p, d, state in, state out, step (FP64 SoA + 12 B states)
# FP64-pipe thread instructions per scheduled detector step, counted by ncu
# (sm__thread_inst_executed_pipe_fp64_pred_on over the launches of one scheduled step on 2^20
# detector step inputs; the summaries are under profiles/): sort keys 3.0 + proposal 10.2 +
# the step kernel(s): 289.4 fused (work-queue configurations 1-4); 279.1 + 14.5 split into
# the step kernel, which also writes each track's relocation point, and the relocation
# kernel that reads it (configurations 5-8). Per-thread counts do not depend on how lanes
# group into warps, so they hold at 2^22. Counted before the candidate buffer kept its
# lowest bounds when full; the kernels now evaluate fewer candidates per step, so these
# counts, and the FP64 fraction computed from them, are upper bounds.
# What the CPU figures are: the oracle port stands in for the reference's CPU code, whose
# sources are not on the GPU machine.
PORT_NOTE = ("oracle port; bit-identical to the reference's own code compiled in the development container, "
             "where that code ran 1.07-1.23x as fast on the same inputs")
FP64_OPS_PER_STEP = {"fused": 3.0 + 10.2 + 289.4, "split": 3.0 + 10.2 + 279.1 + 14.5}
# DRAM bytes per step of the step kernel launch(es) by work-queue configuration, from one ncu
# capture each on 2^20 steps (spills included), scaled to the bench launch by its steps:
# fused 128 x 5: read 727.3 MB + write 297.5 MB; split 256 x 2: step kernel 464.5 + 141.1 MB,
# relocation kernel 122.1 + 5.5 MB. Configurations not captured report null.
STEP_TRAFFIC_PER_STEP = {4: (727.3e6 + 297.5e6) / (1 << 20),
                         6: (464.5e6 + 141.1e6 + 122.1e6 + 5.5e6) / (1 << 20)}
# name -> (precision | scheduling flags): 1 = VG_PREC_MIXED, 2 = VG_NAV_SORT, 4 = VG_NAV_QUEUE
# 8 = VG_NAV_LEARNED (explore the BVH subtree proposed by the trained model first)
SCHEDULES = {"fp64": 0, "fp64_sort": 2, "mixed": 1, "mixed_sort": 3, "mixed_queue": 5, "mixed_sort_queue": 7,
             "mixed_sort_queue_learned": 15}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="detector", choices=["detector", "barrel"])
    ap.add_argument("--tracks", type=int, default=1 << 22)
    ap.add_argument("--primaries", type=int, default=1 << 20)
    ap.add_argument("--seed", type=int, default=0xC0FFEE)
    ap.add_argument("--cpu-sample", type=int, default=1 << 17)
    ap.add_argument("--schedule", default="mixed_sort_queue_learned", choices=sorted(SCHEDULES),
                    help="precision and scheduling of the headline measurement")
    ap.add_argument("--variants", type=int, default=1, help="also time the other schedules (1/0)")
    ap.add_argument("--train-samples", type=int, default=10_000_000,
                    help="plain-navigator steps sampled to train the learned proposal")
    ap.add_argument("--train-epochs", type=int, default=3)
    ap.add_argument("--stream", type=int, default=1, help="also run the config-5 transport stream (1/0)")
    ap.add_argument("--stream-tracks", type=int, default=1 << 20)
    ap.add_argument("--shapes", type=int, default=1, help="also time the config-1/2 shape queries (1/0)")
    ap.add_argument("--shape-reps", type=int, default=20, help="graph-captured calls per shape-query timing")
    ap.add_argument("--section", default="all", choices=["all", "shapes"],
                    help="'shapes': only the shape-query rows (one JSON line), e.g. for profiling")
    ap.add_argument("--graph", type=int, default=1,
                    help="time the headline step as replays of a captured CUDA graph (1/0)")
    ap.add_argument("--tune", type=int, default=1,
                    help="autotune sort-key bits / queue occupancy before timing (untimed; 1/0)")
    ap.add_argument("--cell-bits", type=int, default=0, help="sort-key Morton bits per axis without --tune (0: default)")
    ap.add_argument("--queue-blocks", type=int, default=0,
                    help="work-queue configuration without --tune (1: 256x1, 2: 256x2, 3: 128x3, 4: 128x5; "
                         "5-8: the same with the step split into step and relocation kernels; 0: default)")
    return ap.parse_args()


def dist_setup(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if args.impl == "ours" else "gloo")
    return ws, rank, local


def max_over_ranks(value, ws, device):
    """The largest `value` over all ranks (timings are reported as the slowest rank's)."""
    if ws <= 1:
        return value
    import torch
    import torch.distributed as dist
    v = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(v, op=dist.ReduceOp.MAX)
    return float(v.item())


class ClockSampler:
    """nvidia-smi samples (every 50 ms) during the timed region."""

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
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self.proc = None
        # the first sample marks the end of nvidia-smi's start-up, which then overlaps no timing
        t0 = time.perf_counter()
        while self.proc and not self.lines and self.proc.poll() is None and time.perf_counter() - t0 < 5.0:
            time.sleep(0.01)
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


def builder(name):
    from vecgeom_gb300 import workloads as W
    return W.build_detector if name == "detector" else W.build_barrel


def config_of(args, total_pool=None):
    if args.workload == "detector":
        cfg = {"workload": "detector nav step (config 4 geometry: 150k box modules in 20 barrel layers, "
                           "2x12 Polycone holders x 167 Trd wedges; 150,213 placed volumes, depth 4)",
               "tracks": args.tracks,
               "track_sample": "uniform draw from straight-track transport histories of %d primaries "
                               "(eta in [-3,3], phi uniform, from the origin)" % args.primaries}
    else:
        cfg = {"workload": "barrel nav step (config 3: 1e4 placed volumes, depth 4)", "tracks": args.tracks,
               "track_sample": "r<30 mm, |z|<500 mm, isotropic"}
    cfg["seed"] = args.seed
    if total_pool:
        cfg["sample_pool"] = total_pool
    return cfg


def make_inputs(args, geo, torch, dev):
    from vecgeom_gb300 import workloads as W
    if args.workload == "detector":
        t, st, total = W.sample_transport_steps(geo, args.tracks, args.seed, torch, dev, n_primaries=args.primaries)
        return t, st, total
    pts, dirs = W.tracks_in_cylinder(args.tracks, seed=args.seed)
    t = [torch.from_numpy(a).to(dev) for a in (*pts, *dirs)]
    st = torch.empty(args.tracks * 12, dtype=torch.uint8, device=dev)
    geo.locate_point(t[0], t[1], t[2], st)
    return t, st, None


def train_proposer(args, geo, torch, dev):
    """Train the learned proposal on steps of the plain FP64 navigator (a separate sample of
    the same transport histories, other seed), keep 10% of the hits for a held-out check,
    attach the model. Untimed setup; its figures go into the result line."""
    from vecgeom_gb300 import learned as L
    from vecgeom_gb300 import workloads as W
    t0 = time.perf_counter()
    tt, tst, _ = W.sample_transport_steps(geo, args.train_samples, args.seed ^ 0x5EED5EED, torch, dev,
                                          n_primaries=args.primaries)
    feat, lv, lab = L.features(geo, *tt, tst)
    del tt, tst
    hits = ((lv >= 0) & (lab >= 0) & (lab <= 7)).nonzero().flatten()
    gen = torch.Generator(device="cpu").manual_seed(args.seed & 0x7FFFFFFF)
    hits = hits[torch.randperm(hits.numel(), generator=gen).to(dev)]
    ntr = hits.numel() * 9 // 10
    tr, te = hits[:ntr], hits[ntr:]
    model = L.Proposer(geo, seed=args.seed)
    losses = model.train(feat[tr].contiguous(), lv[tr].contiguous(), lab[tr].contiguous(), epochs=args.train_epochs,
                         batch=8192, lr=3e-3, seed=args.seed)
    pred = model.infer(feat[te].contiguous(), lv[te].contiguous())
    acc = float((pred.to(torch.int64) == lab[te].to(torch.int64)).float().mean().item())
    model.attach(geo)
    info = {"train_steps_sampled": args.train_samples, "train_hit_samples": int(ntr), "epochs": args.train_epochs,
            "epoch_loss": [round(x, 4) for x in losses], "holdout_top1": round(acc, 4),
            "train_s": round(time.perf_counter() - t0, 2)}
    del feat, lv, lab
    torch.cuda.empty_cache()
    return model, info


def run_stream(args, geo, torch, dev, head, clocks_cls, local):
    """Config 5: 2^20 tracks (80% primaries from the origin, 20% restarting at random points
    of the world) transported until they leave the world, plain FP64 vs the headline
    schedule; steps/s over all steps, identity of every track's step count, final state and
    position; the oracle's transport loop on a bounded sample on the host cores."""
    import vecgeom_gb300 as vg
    from vecgeom_gb300 import workloads as W
    n = args.stream_tracks
    pts, dirs, restart = W.stream_tracks(n, args.seed)
    res = {}
    for name, flags in (("fp64", vg.PREC_FP64), ("headline", head)):
        dv = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in (*pts, *dirs)]
        st = torch.empty(n * 12, dtype=torch.uint8, device=dev)
        geo.locate_point(*dv[:3], st)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        nsteps, status, iters, _, _ = geo.transport(*dv, st, max_steps=400, flags=flags)
        torch.cuda.synchronize()
        sec = time.perf_counter() - t0
        total = int(nsteps.to(torch.int64).sum().item())
        res[name] = dict(seconds=sec, steps=total, iterations=iters, nsteps=nsteps.cpu().numpy(),
                         final=st.cpu().numpy(), pos=[a.cpu().numpy() for a in dv[:3]],
                         errors=int((status != 0).sum().item()))
    a, b = res["fp64"], res["headline"]
    identical = (np.array_equal(a["nsteps"], b["nsteps"]) and np.array_equal(a["final"], b["final"])
                 and all(np.array_equal(p, q) for p, q in zip(a["pos"], b["pos"])))
    out = {"tracks": n, "restart_fraction": round(float(restart.mean()), 4), "max_steps": 400,
           "total_steps": a["steps"], "steps_per_track_max": int(a["nsteps"].max()),
           "fp64": {"steps_per_s": a["steps"] / a["seconds"], "seconds": round(a["seconds"], 4)},
           "headline": {"steps_per_s": b["steps"] / b["seconds"], "seconds": round(b["seconds"], 4),
                        "iterations": b["iterations"]},
           "speedup": a["seconds"] / b["seconds"], "identical_to_fp64": bool(identical),
           "track_errors": a["errors"] + b["errors"]}
    # the oracle's transport loop on the host cores over a bounded sample of the same tracks
    from oracle.oracle import OracleGeometry
    o = OracleGeometry()
    builder(args.workload)(o)
    m = min(4096, n)
    sx = [np.ascontiguousarray(v[:m]) for v in (*pts, *dirs)]
    ost, _ = o.locate(*sx[:3], nthreads=os.cpu_count() or 1)
    ons, ofin, _, _, osec = o.transport(*sx, ost, 400, nthreads=os.cpu_count() or 1)
    out["cpu_oracle"] = {"steps_per_s": float(ons.sum()) / osec, "cores": os.cpu_count() or 1,
                         "sample_tracks": m, "steps_match_gpu": bool(np.array_equal(ons, a["nsteps"][:m]))}
    return out


def timed_graph(torch, call, reps):
    """Device time per call: `reps` calls captured in one CUDA graph and replayed between
    CUDA events, so host launch overhead is not timed (falls back to an eager loop if the
    capture is refused)."""
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        for _ in range(2):
            call()
    torch.cuda.current_stream().wait_stream(side)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    try:
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            for _ in range(reps):
                call()
        graph.replay()
        torch.cuda.synchronize()
        e0.record()
        graph.replay()
        e1.record()
    except RuntimeError:
        torch.cuda.synchronize()
        e0.record()
        for _ in range(reps):
            call()
        e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


QUERY_BYTES = {"inside": 28, "contains": 25, "distance_to_in": 56, "distance_to_out": 56, "safety_to_in": 32,
               "safety_to_out": 32}  # FP64 SoA inputs + output per query (step_max not passed)


# Parity bar of distances and safeties against the FP64 oracle (the tests' bar)
ABS_TOL, REL_TOL = 1e-9, 1e-12
INF = np.finfo(np.float64).max


def compare_to_oracle(gpu, ref):
    """Parity figures of one GPU output array against the oracle's on the same inputs:
    integer outputs must be equal; distances and safeties within 1e-9 mm + 1e-12 relative,
    with the kInfLength sentinel matching exactly."""
    gpu, ref = np.asarray(gpu), np.asarray(ref)
    if gpu.dtype != np.float64:
        return {"mismatch_vs_oracle": int((gpu.astype(np.int64) != ref.astype(np.int64)).sum())}
    inf_g, inf_r = gpu == INF, ref == INF
    fin = ~inf_g & ~inf_r
    d = np.abs(gpu - ref)[fin]
    tol = ABS_TOL + REL_TOL * np.abs(ref[fin])
    return {"max_abs_err_vs_oracle": float(d.max()) if d.size else 0.0,
            "beyond_tol_vs_oracle": int((d > tol).sum()) + int((inf_g != inf_r).sum()),
            "bit_identical_to_oracle": int((gpu.view(np.int64) == ref.view(np.int64)).sum())}


QUERY_INDEX = {"inside": 0, "contains": 1, "distance_to_in": 2, "distance_to_out": 3, "safety_to_in": 4,
               "safety_to_out": 5}


def shape_rows(args, torch, dev, hbm_peak, oracle=True):
    """Config 1 (Box, Tube, Cone; 2^20 points uniform in the 1.2x extent box) and config 2
    (2^22 points: thirds inside, outside, within 1e-6 mm of the surface) shape queries per
    precision: queries/s, algorithmic GB/s and its fraction of the HBM peak; every output of
    both precisions is compared with the FP64 oracle run over the same points on the host
    cores (untimed), and the mixed path also with the FP64 kernel."""
    import vecgeom_gb300 as vg
    from vecgeom_gb300 import workloads as W
    if oracle:
        from oracle.oracle import OracleGeometry
    nthreads = os.cpu_count() or 1
    rows = []
    cases = [(k, v, 1 << 20, "cfg1") for k, v in W.SHAPES_CFG1.items()] + \
            [(k, v, 1 << 22, "cfg2") for k, v in W.SHAPES_CFG2.items()]
    for name, (kind, params), n, cfg in cases:
        g = vg.Geometry()
        sid, pv = W.build_single_shape(g, kind, params)
        lo, hi = g.shape_extent(sid)

        def q_gpu(fn, dtype, *cols):
            t = [torch.from_numpy(np.ascontiguousarray(c)).to(dev) for c in cols]
            o = torch.empty(len(cols[0]), dtype=dtype, device=dev)
            fn(pv, *t, o)
            return o.cpu().numpy()

        if cfg == "cfg1":
            pts, dirs = W.shape_points_box(lo, hi, n, args.seed)
        else:
            pts, dirs = W.shape_points_mixed(lo, hi, n, args.seed, lambda *c: q_gpu(g.inside, torch.int32, *c),
                                             lambda *c: q_gpu(g.distance_to_out, torch.float64, *c))
        t = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in (*pts, *dirs)]
        o_geo = o_pv = None
        if oracle:
            o_geo = OracleGeometry()
            _, o_pv = W.build_single_shape(o_geo, kind, params)
            host_cols = [np.ascontiguousarray(a) for a in (*pts, *dirs)]
        outs = {"inside": torch.empty(n, dtype=torch.int32, device=dev),
                "contains": torch.empty(n, dtype=torch.uint8, device=dev)}
        for prec_name, prec in (("fp64", vg.PREC_FP64), ("mixed", vg.PREC_MIXED)):
            for q in QUERY_BYTES:
                o = outs.get(q, None)
                if o is None:
                    o = torch.empty(n, dtype=torch.float64, device=dev)
                fn = getattr(g, q)
                args_q = (pv, *t, o) if q.startswith("distance") else (pv, *t[:3], o)

                def call():
                    fn(*args_q, flags=prec)

                ms = timed_graph(torch, call, args.shape_reps)
                gbs = QUERY_BYTES[q] * n / (ms * 1e-3) / 1e9
                row = {"config": cfg, "shape": name, "query": q, "precision": prec_name, "n": n,
                       "input_bytes": QUERY_BYTES[q] * n, "l2_resident_inputs": QUERY_BYTES[q] * n < 129e6,
                       "queries_per_s": n / (ms * 1e-3), "GB_per_s": gbs, "hbm_frac": gbs / hbm_peak}
                if oracle:
                    if (q, "oracle") not in outs:
                        outs[(q, "oracle")] = o_geo.query(o_pv, QUERY_INDEX[q], *host_cols, nthreads=nthreads)[0]
                    got = o.cpu().numpy()
                    row.update(compare_to_oracle(got.astype(np.int32) if q == "contains" else got,
                                                 outs[(q, "oracle")]))
                if prec_name == "fp64":
                    outs[(q, "ref")] = o.clone()
                else:
                    ref = outs[(q, "ref")]
                    if o.dtype == torch.float64:
                        both = (ref < 1e300) & (o < 1e300)
                        row["max_abs_diff_vs_fp64"] = float((o - ref)[both].abs().max().item()) if bool(both.any()) else 0.0
                        row["sentinel_mismatch"] = int(((ref >= 1e300) != (o >= 1e300)).sum().item())
                    else:
                        row["mismatch_vs_fp64"] = int((o != ref).sum().item())
                rows.append(row)
    return rows


def cpu_time_steps(args, host_inputs, host_states, nthreads, reps=5):
    """Oracle port timing over the given sample: the median of `reps` repetitions after one
    warm-up, on `nthreads` host threads and on one thread; returns (all-thread steps/s,
    single-thread steps/s)."""
    from oracle.oracle import OracleGeometry
    o = OracleGeometry()
    builder(args.workload)(o)
    st = np.frombuffer(host_states.tobytes(), dtype=[("nav_ind", "<u4"), ("last_exited", "<u4"),
                                                    ("on_boundary", "u1"), ("pad", "u1", 3)]).copy()
    rates = []
    for threads in (nthreads, 1):
        o.step(*host_inputs, st, nthreads=threads)
        ts = sorted(o.step(*host_inputs, st, nthreads=threads)[3] for _ in range(reps))
        rates.append(len(host_inputs[0]) / ts[reps // 2])
    return rates[0], rates[1]


def run_reference(args, ws, rank):
    """CPU implementation of the path (the oracle port; the reference itself needs VecCore,
    which is not available) on all host cores, same metric and config. Each step is a
    bounded sample of the batch: the first --cpu-sample of the GPU arm's own step inputs,
    reproduced on the CPU (the same primaries transported by the oracle, the same seeded
    draw), so both arms' CPU figures step the very same tracks."""
    if rank != 0:
        return
    nthreads = os.cpu_count() or 1
    from oracle.oracle import OracleGeometry, transport_step_sample
    from vecgeom_gb300 import workloads as W
    o = OracleGeometry()
    builder(args.workload)(o)
    m = min(args.cpu_sample, args.tracks)
    if args.workload == "detector":
        sub, st, _ = transport_step_sample(o, args.tracks, args.seed, args.primaries, nthreads=nthreads, first=m)
        sample = ("the first %d of the %d step inputs of the GPU arm (its transport-history draw, reproduced "
                  "on the host by the oracle)" % (m, args.tracks))
    else:
        pts, dirs = W.tracks_in_cylinder(args.tracks, seed=args.seed)
        sub = [np.ascontiguousarray(a[:m]) for a in (*pts, *dirs)]
        st, _ = o.locate(*sub[:3], nthreads=nthreads)
        sample = "the first %d of the %d tracks of the GPU arm" % (m, args.tracks)
    for _ in range(args.warmup):
        o.step(*sub, st, nthreads=nthreads)
    times = []
    for _ in range(args.steps):
        _, _, _, t = o.step(*sub, st, nthreads=nthreads)
        times.append(t)
    tot = sum(times)
    value = m * args.steps / tot
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * tot / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": config_of(args), "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                             "sample": sample + ", every step", "note": PORT_NOTE},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
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
    if args.section == "shapes":
        try:
            hbm = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"]
        except (OSError, ValueError, KeyError):
            hbm = 6800.0
        if rank == 0:
            print(json.dumps({"section": "shape_queries", "rows": shape_rows(args, torch, dev, hbm)}), flush=True)
        return
    geo = vg.Geometry()
    builder(args.workload)(geo)
    t, st, pool = make_inputs(args, geo, torch, dev)
    n = args.tracks
    out = torch.empty_like(st)
    step = torch.empty(n, dtype=torch.float64, device=dev)
    status = torch.empty(n, dtype=torch.int32, device=dev)
    torch.cuda.synchronize()

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()

    spread = {}

    def timed(flags, graph=False):
        """ms per step; with graph=True the step (all its launches) is captured once into a
        CUDA graph after the warm-up and each timed step is one replay."""
        for _ in range(args.warmup):
            geo.compute_step_and_next_volume(*t, st, out, step, status=status, flags=flags)
        torch.cuda.synchronize()
        run = lambda: geo.compute_step_and_next_volume(*t, st, out, step, status=status, flags=flags)
        if graph:
            cg = torch.cuda.CUDAGraph()
            with torch.cuda.graph(cg):
                geo.compute_step_and_next_volume(*t, st, out, step, status=status, flags=flags)
            cg.replay()
            run = cg.replay
        torch.cuda.synchronize()
        barrier()
        evs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
        torch.cuda.synchronize()
        evs[0].record()
        for k in range(args.steps):
            run()
            evs[k + 1].record()
        torch.cuda.synchronize()
        barrier()
        per = [evs[k].elapsed_time(evs[k + 1]) for k in range(args.steps)]
        spread[flags] = (min(per), max(per))
        ms = max_over_ranks(evs[0].elapsed_time(evs[-1]), ws, dev)
        return ms / args.steps

    head = SCHEDULES[args.schedule]
    learned_info, model = None, None
    if any(f & vg.NAV_LEARNED for f in SCHEDULES.values()) and (args.variants or head & vg.NAV_LEARNED):
        model, learned_info = train_proposer(args, geo, torch, dev)
        nodes = torch.empty(n, dtype=torch.int32, device=dev)
        per = {}
        for name in ("fp64", "mixed_sort_queue", "mixed_sort_queue_learned"):
            geo.compute_step_and_next_volume(*t, st, out, step, status=status, flags=SCHEDULES[name],
                                             nodes_visited=nodes)
            per[name] = round(float(nodes.to(torch.float64).mean().item()), 3)
        learned_info["bvh_nodes_visited_per_step"] = per
    tuning = None
    if args.tune and head & (vg.NAV_SORT | vg.NAV_QUEUE):
        from vecgeom_gb300.tune import autotune
        cands = [(head, b, q) for b in (0, 7, 6, 5) for q in (tuple(range(1, 9)) if head & vg.NAV_QUEUE else (1,))]
        tuning = autotune(geo, t, st, candidates=cands, cache=None)
    elif args.cell_bits or args.queue_blocks:
        geo.set_tuning(args.cell_bits, args.queue_blocks)
    queue_cfg = (tuning["queue_blocks"] if tuning else args.queue_blocks) or 1
    split = queue_cfg >= 5
    ms_fp64 = timed(vg.PREC_FP64)
    out64, step64 = out.clone(), step.clone()
    variants = {"fp64": ms_fp64}
    identical = True
    if args.variants:
        for name, f in sorted(SCHEDULES.items()):
            if name in ("fp64", args.schedule):
                continue
            variants[name] = timed(f)
            identical &= bool(torch.equal(out64, out)) and bool(torch.equal(step64, step))
    ms_head_eager = timed(head) if args.graph else None
    with ClockSampler(local) as clocks:
        ms_head = timed(head, graph=bool(args.graph))
    variants[args.schedule] = ms_head
    n_err = int((status != 0).sum().item())
    ids_equal = bool(torch.equal(out64, out))
    step_err = float((step64 - step).abs().max().item())
    head_out, head_step = out.cpu().numpy(), step.cpu().numpy()

    # the track sort alone (part of every sorted step), to separate the step kernel's time
    ms_sort = 0.0
    passes = 0
    if head & vg.NAV_SORT:
        order = torch.empty(n, dtype=torch.int32, device=dev)
        wsp = torch.empty(vg.Geometry.step_workspace_bytes(n, vg.NAV_SORT), dtype=torch.uint8, device=dev)
        for _ in range(args.warmup):
            geo.sort_tracks(t[0], t[1], t[2], st, order, workspace=wsp)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(args.steps):
            geo.sort_tracks(t[0], t[1], t[2], st, order, workspace=wsp)
        e1.record()
        torch.cuda.synchronize()
        ms_sort = e0.elapsed_time(e1) / args.steps
        _, _, cb, lb = geo.sort_key_params()
        passes = (lb + 3 * cb + 8) // 9  # 9-bit radix digits
    # the learned proposal alone (features + MLP inference), also part of the headline step
    ms_propose = 0.0
    if head & vg.NAV_LEARNED:
        from vecgeom_gb300 import learned as L
        slot = torch.empty(n, dtype=torch.int8, device=dev)
        for _ in range(args.warmup):
            L.propose(geo, *t, st, out=slot)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(args.steps):
            L.propose(geo, *t, st, out=slot)
        e1.record()
        torch.cuda.synchronize()
        ms_propose = e0.elapsed_time(e1) / args.steps
    ms_kernel = ms_head - ms_sort - ms_propose

    stream = run_stream(args, geo, torch, dev, head, ClockSampler, local) if (args.stream and rank == 0) else None
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    shapes = shape_rows(args, torch, dev, hbm_peak) if (args.shapes and rank == 0) else None

    # e2e: host arrays through the host-pointer C-ABI entry point, copies inside the timed region
    hp = [a.cpu().pin_memory() for a in t]
    hst = st.cpu().pin_memory()
    hout = torch.empty_like(hst).pin_memory()
    hstep = torch.empty(n, dtype=torch.float64).pin_memory()
    for _ in range(max(3, args.warmup)):
        geo.compute_step_and_next_volume_host(*hp, hst, hout, hstep, flags=head)
    barrier()
    # each host-entry call returns with its results in host memory; the calls are timed one
    # by one (the spread shows host and link noise of a shared machine) and the value is the
    # whole run: all calls' steps over the total time
    ke = max(5, args.steps // 2)
    calls = []
    t0 = time.perf_counter()
    for _ in range(ke):
        c0 = time.perf_counter()
        geo.compute_step_and_next_volume_host(*hp, hst, hout, hstep, flags=head)
        calls.append(time.perf_counter() - c0)
    torch.cuda.synchronize()
    barrier()
    e2e_s = (time.perf_counter() - t0) / ke
    in_order = [round(1e3 * c, 3) for c in calls]
    calls.sort()
    e2e_calls = {"calls": ke, "min": round(1e3 * calls[0], 3), "median": round(1e3 * calls[ke // 2], 3),
                 "max": round(1e3 * calls[-1], 3)}

    value = ws * n / (ms_head * 1e-3)
    achieved = STEP_BYTES * n / (ms_kernel * 1e-3) / 1e9
    # FP64 roofline of the scheduled step (the bound of the navigation rows): FP64 pipe
    # thread-ops per step x steps/s over this GPU's measured FP64 FMA rate
    roofline_fp64 = None
    if head == SCHEDULES["mixed_sort_queue_learned"]:
        fp64_peak = vg.device_fp64_rate()
        ops = FP64_OPS_PER_STEP["split" if split else "fused"]
        roofline_fp64 = {"bound": "fp64", "achieved": ops * n / (ms_head * 1e-3), "peak": fp64_peak,
                         "unit": "FP64 thread-ops/s", "frac": ops * n / (ms_head * 1e-3) / fp64_peak,
                         "ops_per_step": ops,
                         "note": "ncu-counted ops per step of the build before the candidate-buffer change "
                                 "(an upper bound for the current kernels); peak = DFMA probe timed in this run"}
    m = {
        "value": value, "ms_per_step": ms_head, "n": n, "ws": ws, "args": args, "pool": pool,
        "ms_fp64": ms_fp64, "ms_fp64_sort": variants.get("fp64_sort"), "ids_equal": ids_equal, "step_err": step_err,
        "e2e_value": ws * n / e2e_s, "e2e_calls": e2e_calls, "head": head, "passes": passes,
        "step_kernels": 2 if (split and head & 4) else 1,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak,
                     "traffic": STEP_TRAFFIC_PER_STEP[queue_cfg] * n
                     if head & 4 and queue_cfg in STEP_TRAFFIC_PER_STEP else None,
                     "kernel": ("k_step_mixed_split (step + relocation launches)" if split else "k_step_mixed_queue")
                     if head & 4 else ("k_step_mixed" if head & 1 else "k_step"),
                     "queue_configuration": queue_cfg,
                     "note": "80 algorithmic B/step over the step kernel(s)' own time; traffic = ncu DRAM bytes "
                             "of the launch(es) (2^20-step capture scaled by steps); peak %s"
                             % ("of measured" if peaks else "of fallback")},
        "roofline_fp64": roofline_fp64, "n_err": n_err, "clocks": clocks.summary(),
    }
    if rank == 0:
        emit({"section": "schedules", "ms_per_step": variants, "all_identical_to_fp64": identical and ids_equal,
              "ms_per_step_min_max": [round(v, 4) for v in spread.get(head, (ms_head, ms_head))],
              "ms_per_step_eager": ms_head_eager, "cuda_graph": bool(args.graph),
              "sort_ms_per_step": ms_sort, "propose_ms_per_step": ms_propose, "step_kernel_ms_per_step": ms_kernel,
              "tuning": None if tuning is None else {k: tuning[k] for k in ("cell_bits", "queue_blocks", "timings")},
              "e2e_ms_per_call_in_order": in_order})
        if learned_info is not None:
            emit({"section": "learned", **learned_info})
        if stream is not None:
            emit({"section": "transport_stream", **stream})
        if shapes is not None:
            emit({"section": "shape_queries", "rows": shapes})
        # parity against the FP64 oracle over every one of the n step inputs (host cores,
        # untimed), for the headline schedule and for plain FP64
        nthreads = os.cpu_count() or 1
        from oracle.oracle import OracleGeometry
        og = OracleGeometry()
        builder(args.workload)(og)
        hin = [np.ascontiguousarray(a.cpu().numpy()) for a in t]
        hst_np = np.frombuffer(st.cpu().numpy().tobytes(), dtype=NAVSTATE_NP).copy()
        o_out, o_step, _, o_sec = og.step(*hin, hst_np, nthreads=nthreads)
        parity = {"section": "parity_vs_oracle", "tracks": n, "oracle_seconds": round(o_sec, 3),
                  "oracle_threads": nthreads,
                  "headline": nav_parity(head_out, head_step, o_out, o_step),
                  "plain_fp64": nav_parity(out64.cpu().numpy(), step64.cpu().numpy(), o_out, o_step)}
        if shapes is not None:
            parity["shapes"] = shape_parity_summary(shapes)
        emit(parity)
        m["parity"] = parity
        # CPU baseline: the oracle on the first cpu_sample step inputs (the same inputs the
        # reference arm reproduces and steps)
        k = min(args.cpu_sample, n)
        cv, cv1 = cpu_time_steps(args, [a[:k] for a in hin], hst_np[:k], nthreads)
        m["cpu_baseline"] = {"value": cv, "unit": UNIT, "cores": nthreads, "kind": "port",
                             "single_thread_value": cv1,
                             "sample": "the first %d of the %d step inputs, median of 5 after a warm-up" % (k, n), "note": PORT_NOTE}
        emit(headline_line(m))
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


NAVSTATE_NP = np.dtype([("nav_ind", "<u4"), ("last_exited", "<u4"), ("on_boundary", "u1"), ("pad", "u1", 3)])


def emit(obj):
    print(json.dumps(obj), flush=True)


def nav_parity(gpu_out, gpu_step, o_out, o_step):
    """Out-states (all three fields) must be bit-identical to the oracle's; steps within
    1e-9 mm + 1e-12 relative (reported: bit-identical count and largest difference)."""
    g = np.frombuffer(np.ascontiguousarray(gpu_out).tobytes(), dtype=NAVSTATE_NP)
    diff = ((g["nav_ind"] != o_out["nav_ind"]) | (g["last_exited"] != o_out["last_exited"])
            | (g["on_boundary"] != o_out["on_boundary"]))
    r = {"state_mismatch": int(diff.sum()), "next_volume_mismatch": int((g["nav_ind"] != o_out["nav_ind"]).sum())}
    r.update(compare_to_oracle(np.asarray(gpu_step, dtype=np.float64), o_step))
    return r


def shape_parity_summary(rows):
    """Totals of the shape rows' oracle comparison, per precision, with the largest error
    per shape; the mixed full-phi Tube safeties are lowered by their proven bound on purpose
    and are listed apart."""
    out = {}
    for prec in ("fp64", "mixed"):
        sel = [r for r in rows if r["precision"] == prec]
        # FP32 safeties with a proven bound below the FP64 value: the full-phi Tube's
        bounded = [r for r in sel if prec == "mixed" and r["shape"] == "tube" and r["query"].startswith("safety")]
        strict = [r for r in sel if r not in bounded]
        per_shape = {}
        for r in strict:
            e = r.get("max_abs_err_vs_oracle")
            if e is not None:
                per_shape[r["shape"]] = max(per_shape.get(r["shape"], 0.0), e)
        out[prec] = {"queries": sum(r["n"] for r in sel),
                     "int_mismatch": sum(r.get("mismatch_vs_oracle", 0) for r in strict),
                     "beyond_tol": sum(r.get("beyond_tol_vs_oracle", 0) for r in strict),
                     "max_abs_err_per_shape": per_shape}
        if bounded:
            out[prec]["fp32_safety_bounded_max_err"] = {
                k: max(r["max_abs_err_vs_oracle"] for r in bounded if r["shape"] == k)
                for k in sorted({r["shape"] for r in bounded})}
    return out


def headline_line(m):
    """The result line the driver parses (the last line of stdout, kept to a few KB): the
    contract keys, e2e, rooflines, CPU baseline, clocks and the identity/parity summary."""
    args, n, ws = m["args"], m["n"], m["ws"]
    cfg = {"workload": "config-4 detector nav step (150,213 placed volumes: 150k barrel box modules, 2x12 "
                       "Polycone holders, 2x2000 Trd wedges; depth 4)" if args.workload == "detector"
           else "config-3 barrel nav step (1e4 placed volumes, depth 4)",
           "tracks": args.tracks, "seed": args.seed, "schedule": args.schedule,
           "l2": "inputs %.0f MB > L2 (129 MB)" % (n * 60 / 1e6),
           "parallelism": "replicas" if ws > 1 else "single GPU"}
    line = {
        "metric": METRIC, "value": m["value"], "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": m["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64 (mixed: FP32 pruning, FP64 decisions)",
        "data": "synthetic (seeded; geometry built in code, tracks from GPU transport histories)", "config": cfg,
        "plain_fp64_value": ws * n / (m["ms_fp64"] * 1e-3),
        "speedup_vs_plain_fp64": m["ms_fp64"] / m["ms_per_step"],
        "speedup_vs_fp64_sort": (m["ms_fp64_sort"] / m["ms_per_step"]) if m.get("ms_fp64_sort") else None,
        "ids_identical_to_fp64": m["ids_equal"], "max_step_diff_vs_fp64_mm": m["step_err"],
        "e2e": {"value": m["e2e_value"], "unit": UNIT, "h2d_bytes_per_step": n * (48 + 12),
                "d2h_bytes_per_step": n * (12 + 8), "ms_per_call": m["e2e_calls"]},
        "roofline": m["roofline"], "roofline_fp64": m["roofline_fp64"],
        "gpu_launches": args.steps * (m.get("step_kernels", 1) + ((1 + 3 * m["passes"]) if m["head"] & 2 else 0)
                                      + (1 if m["head"] & 8 else 0)),
        "track_errors": m["n_err"], "clocks": m["clocks"],
    }
    par = m.get("parity")
    if par:
        h, f = par["headline"], par["plain_fp64"]
        line["vs_oracle"] = {"tracks": par["tracks"], "state_mismatch": h["state_mismatch"],
                             "step_beyond_tol": h["beyond_tol_vs_oracle"],
                             "step_max_abs_err": h["max_abs_err_vs_oracle"],
                             "plain_fp64_state_mismatch": f["state_mismatch"]}
        if "shapes" in par:
            line["vs_oracle"]["shape_queries"] = {p: {k: v for k, v in d.items() if k != "max_abs_err_per_shape"}
                                                  for p, d in par["shapes"].items()}
    if "cpu_baseline" in m:
        line["cpu_baseline"] = m["cpu_baseline"]
    return line


if __name__ == "__main__":
    main()
