"""Throughput benchmark of the GB300 synthesis engine.

Workload (one "step"): the render-texture enlarge -- a 128x128 RGBA corpus tile
of seeded value noise plus tileable stripes synthesized into a 1024x1024
target, random order, neighbours=16, trys=300, no context -- through
engine() (wavefront mode), all passes until the reference's termination rule.

  value   target px/s with the pixmaps already resident in device memory
          (engineDevice), timed with CUDA events per step, L2 flushed between
          steps (outside the timed intervals)
  e2e     the same metric through engineEx() with host Maps: host->device copy
          of the pixmaps, the synthesis and the device->host copy of the result
  roofline    the per-target synthesis kernel (k_wave), its launches timed live
          with CUDA events on the library stream
  cpu_baseline  the CPU engine on a bounded sample of the workload
  learned     learned proposals against the plain search on a 1024^2 heal
          (network trained on the GPU from pairs dumped by plain runs)

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
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

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = "render1024: 128x128 RGBA tile -> 1024x1024 target, random order, P=16, trys=300, engine()"
METRIC = "target px/s + candidate evals/s; learned vs plain GPU search at equal patch energy"


def term_bytes(nc: int, nm: int) -> int:
    """Algorithmic bytes of one neighbour term: the 4-byte corpus word (mask +
    colours), a 16-bit table read per colour channel, and per map channel the
    map byte and a 32-bit table read."""
    return 4 + 2 * nc + (1 + 4) * nm


def term_ops(nc: int, nm: int) -> int:
    """Integer ops of one neighbour term: bounds/mask, then (sub, index, add)
    per colour and map channel."""
    return 4 + 3 * (nc + nm)

# DRAM bytes (read + write) per k_wave launch, the mean over one synthesis, from
# an ncu launch list (dram__bytes_read.sum + dram__bytes_write.sum, one pass) of
#   python bench.py --profile-once --no-cpu --warps 16 --workload W
# ncu flushes the caches before each launch, so these are cold-cache figures:
# an upper bound for the warm launches timed here.
WAVE_DRAM_BYTES = {"render1024": 6.64e6, "heal4096": 67.63e6, "mapstyle2048": 28.58e6}
SAMPLE_SIDE = 256                 # CPU sample: 256x256 target from the same tile


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
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
        sm, mx, reasons = [], 0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx = max(mx, float(f[1]))
            except ValueError:
                continue
            for n, v in zip(names, f[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(value: float, device=None) -> float:
    """The largest value over the ranks of the default process group (the
    value itself without one): replicas report the slowest rank's time."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return value
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(world: int, steps: int, units_per_step: float, max_ms: float) -> float:
    """Whole-job throughput of `world` replicas that each processed `steps`
    steps of `units_per_step` units, timed by the slowest one."""
    return world * steps * units_per_step / (max_ms / 1000.0)


def cpu_sample(threads: int, side: int = SAMPLE_SIDE):
    """The CPU engine on a side x side sample of the workload: the reference
    built from its own sources where present, else the oracle port."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from resynthesizer_gb300 import workloads as W
    wl = W.render(tile=128, out=side)
    p = O.make_params(**wl["params"])
    kind = "port"
    if O.reference_available(threaded=threads > 1):
        ref = O.Reference(threaded=threads > 1)
        fmt = O.Oracle().format_indices(*wl["format"])
        t0 = time.perf_counter()
        rc, _, _, _ = ref.engine_state(p, fmt, wl["target"], wl["corpus"])
        dt = time.perf_counter() - t0
        kind = "reference"
        evals = None
    else:
        o = O.Oracle()
        fmt = o.format_indices(*wl["format"])
        t0 = time.perf_counter()
        rc, _, st = o.engine(p, fmt, wl["target"], wl["corpus"], threads=threads)
        dt = time.perf_counter() - t0
        evals = st.evals
    assert rc == 0
    px = side * side
    return dict(value=px / dt, seconds=dt, evals_per_s=(evals / dt) if evals else None, kind=kind, cores=threads,
                sample=f"{side}x{side} target from the same 128x128 tile (P=16, trys=300), one run")


def cpu_same_schedule(target, corpus, spec, params: dict, gpu_out, threads: int):
    """The wavefront schedule itself on the CPU: its plain-C restatement
    (oracle/wave_oracle.c) on the whole workload with `threads` threads, and
    whether it gives the GPU's output byte for byte.  Separates what the
    schedule gains over the reference's sequential engine from what the GPU
    gains over the same schedule on CPU cores."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    o = O.Oracle()
    fmt = o.format_indices(*spec)
    t0 = time.perf_counter()
    rc, out, passes, _ = o.wave_engine(O.make_params(**params), fmt, target, corpus, threads=threads)
    dt = time.perf_counter() - t0
    px = int((target[..., 0] != 0).sum())
    return {"value": px / dt, "unit": "target px/s", "cores": threads, "seconds": dt, "passes": passes,
            "identical_to_gpu": bool(rc == 0 and np.array_equal(out, gpu_out)),
            "what": "the wavefront schedule restated in C (oracle/wave_oracle.c), whole workload"}


def load_workload(name: str):
    """(name, target pixmap, corpus pixmap, prepareImageFormatIndices args, params) of a workload."""
    from resynthesizer_gb300 import workloads as W
    if name == "render1024":
        wl = W.render1024()
        return wl["name"], wl["target"], wl["corpus"], wl["format"], wl["params"]
    if name == "mapstyle2048":
        wl = W.mapstyle()
        return wl["name"], wl["target"], wl["corpus"], wl["format"], wl["params"]
    if name == "heal256":
        wl = W.heal256()
    elif name == "heal4096":
        wl = W.heal4096()
    else:
        raise SystemExit(f"unknown workload {name}")
    t, c = W.simple_to_pixmaps(wl["image"], wl["mask"])
    return wl["name"], t, c, (3, 0, 0, 0, 0), wl["params"]


def psnr(a, b):
    import numpy as np
    mse = float(np.mean((a.astype(np.float64) - b.astype(np.float64)) ** 2))
    return float("inf") if mse == 0 else 10 * np.log10(255.0 ** 2 / mse)


def run_quality(args):
    """Energy of the wavefront result against the CPU engine on the same input:
    the single-threaded engine once and the 8-thread engine (nondeterministic)
    `--quality-runs` times.  Energy = sum over target pixels of the full-patch
    metric at each pixel's final source, patches from the final state."""
    import numpy as np

    import resynthesizer_gb300 as R
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    name, tgt, cor, spec, kw = load_workload(args.workload)
    p = R.params(**kw)
    fmt = R.format_indices(*spec)
    sel = tgt[..., 0] != 0
    ys, xs = np.nonzero(sel)
    targets = np.stack([xs, ys], 1).astype(np.int32)
    nc = fmt.img_match_bpp

    def energy(out, hv, src):
        return R.patch_energy(p, fmt, out, cor, hv, src, targets)[0]

    g = R.engine(tgt, cor, fmt, p, opts=R.options(mode=R.MODE_WAVEFRONT, recordState=1))
    assert g.rc == 0, R.last_error()
    e_gpu = energy(g.out, g.has_value, g.source)
    o = O.Oracle()
    of = o.format_indices(*spec)
    op = O.make_params(**kw)
    t0 = time.perf_counter()
    rc, out_st, st_st, src_st, hv_st = o.engine(op, of, tgt, cor, threads=1, want_state=True)
    t_st = time.perf_counter() - t0
    e_st = energy(out_st, hv_st, src_st)
    e_mt, t_mt, out_mt = [], [], None
    for _ in range(args.quality_runs):
        t0 = time.perf_counter()
        rc, out_mt, st_mt, src_mt, hv_mt = o.engine(op, of, tgt, cor, threads=8, want_state=True)
        t_mt.append(time.perf_counter() - t0)
        e_mt.append(energy(out_mt, hv_mt, src_mt))
    mt_mean = float(np.mean(e_mt)) if e_mt else None
    ref_out = out_mt if out_mt is not None else out_st
    line = {"quality": name, "target_px": int(sel.sum()), "energy_gpu": e_gpu, "energy_cpu_st": e_st,
            "energy_cpu_mt": e_mt, "energy_cpu_mt_mean": mt_mean,
            "gpu_over_mt": e_gpu / mt_mean if mt_mean else None, "gpu_over_st": e_gpu / e_st,
            "mt_spread": (max(e_mt) - min(e_mt)) / mt_mean if mt_mean else None,
            "psnr_gpu_vs_ref": psnr(g.out[sel][:, 1:1 + nc], ref_out[sel][:, 1:1 + nc]),
            "psnr_ref": "8-thread CPU run" if out_mt is not None else "single-threaded CPU run",
            "gpu_passes": g.stats["passes"], "gpu_ms": g.stats["deviceMs"], "gpu_evals": g.stats["evals"],
            "cpu_st_s": t_st, "cpu_st_evals": st_st.evals, "cpu_mt_s": t_mt, "cpu_kind": "port",
            "cpu_threads_mt": 8}
    if int(sel.sum()) <= 100000:
        # sequential replay: byte-identical to the single-threaded engine
        r = R.engine(tgt, cor, fmt, p, opts=R.options(mode=R.MODE_REPLAY))
        line["replay_identical_to_cpu_st"] = bool(r.rc == 0 and np.array_equal(r.out, out_st))
        line["replay_ms"] = r.stats["deviceMs"]
    print(json.dumps(line), flush=True)


def run_batch(args):
    """Batched heal requests: independent heals of mixed sizes,
    layouts, holes and patch sizes through imageSynthBatch, end to end with
    host buffers.  value = all requests' target pixels / wall time."""
    import numpy as np

    import resynthesizer_gb300 as R
    from resynthesizer_gb300 import workloads as W
    n = int(args.workload[len("batch"):] or 512)
    t0 = time.perf_counter()
    reqs = W.batch_requests(n=n)
    gen_s = time.perf_counter() - t0
    items = [(r["image"], r["mask"], r["fmt"], R.params(**r["params"])) for r in reqs]
    target_px = sum(r["target_px"] for r in reqs)
    opts = R.options(mode=R.MODE_WAVEFRONT)
    for _ in range(max(1, args.warmup // 3)):
        rc, _, codes, _ = R.image_synth_batch(items[: min(16, n)], opts=opts, concurrency=args.concurrency)
        assert rc == 0, R.last_error()
    times, st = [], None
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            t1 = time.perf_counter()
            rc, outs, codes, st = R.image_synth_batch(items, opts=opts, concurrency=args.concurrency)
            times.append(time.perf_counter() - t1)
            assert rc == 0, R.last_error()
    wall = sum(times)
    line = {"metric": METRIC, "value": args.steps * target_px / wall, "unit": "target px/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * wall / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
            "config": {"workload": f"batch{n}: {n} heal requests, 128..1024 px sides, Gray/RGB/RGBA, holes 2-20 %, "
                                   f"P in {{9,16,30}}, trys=200, imageSynthBatch",
                       "requests": n, "target_px": target_px, "concurrency": args.concurrency,
                       "mode": "wavefront", "timing": "wall clock around imageSynthBatch (host buffers)"},
            "evals_per_s": st["evals"] / (wall / args.steps), "gpu_launches": st["launches"] * args.steps,
            "device_ms_sum_per_step": st["deviceMs"], "generation_s": gen_s,
            "e2e": {"value": args.steps * target_px / wall, "unit": "target px/s",
                    "h2d_bytes_per_step": st["h2dBytes"], "d2h_bytes_per_step": st["d2hBytes"]},
            "clocks": clk.summary()}
    print(json.dumps(line), flush=True)


def learned_comparison(size, train_images, train_pairs, train_steps, searches, reps=3):
    """Learned proposals against the plain search on the large-heal family
    (seeded value noise, union of 40 ellipses covering ~10 % of the image):
    pairs are dumped by plain wavefront runs over `train_images` images (seeds
    1..N), the network trains on the GPU with the tensor-core kernels, then a
    held-out image (seed 0) is synthesized with and without the network's 16
    proposals at the given probe counts.  Energy = sum of the full-patch metric
    over the targets at their final sources."""
    import numpy as np

    import resynthesizer_gb300 as R
    from resynthesizer_gb300 import workloads as W
    fmt = R.format_indices(3, 0, 0, 0, 0)

    def run(wl, trys, net=None, dump=None, stride=16, state=True):
        tgt, cor = W.simple_to_pixmaps(wl["image"], wl["mask"])
        kw = dict(wl["params"])
        kw["maxProbeCount"] = trys
        o = R.options(mode=R.MODE_WAVEFRONT, recordState=1 if state else 0, net=net, proposals=16 if net else 0,
                      dump=dump, dumpStride=stride)
        r = R.engine(tgt, cor, fmt, R.params(**kw), opts=o)
        assert r.rc == 0, R.last_error()
        e = None
        if state:
            ys, xs = np.nonzero(tgt[..., 0] != 0)
            t = np.stack([xs, ys], 1).astype(np.int32)
            e, _ = R.patch_energy(R.params(**kw), fmt, r.out, cor, r.has_value, r.source, t)
        return r, e

    t0 = time.perf_counter()
    pairs = R.Pairs(train_pairs)
    per_image = max(1, train_pairs // train_images)
    for i in range(1, train_images + 1):
        wl = W.heal4096(index=i, size=size)
        run(wl, 200, dump=pairs, stride=max(1, wl["target_px"] // per_image), state=False)
    dump_s = time.perf_counter() - t0
    net = R.Net(seed=1)
    t0 = time.perf_counter()
    loss = net.train(pairs, steps=train_steps, batch=512, lr=1e-3)
    train_s = time.perf_counter() - t0
    wl = W.heal4096(index=0, size=size)
    rows = []
    for trys, use in searches:
        ms = []
        for _ in range(reps):
            r, e = run(wl, trys, net=net if use else None)
            ms.append(r.stats["deviceMs"])
        rows.append({"search": ("learned+" if use else "plain ") + f"trys={trys}", "energy": e,
                     "ms": min(ms), "px_per_s": wl["target_px"] / (min(ms) / 1000.0), "evals": r.stats["evals"],
                     "passes": r.stats["passes"]})
    base = rows[0]["energy"]
    for row in rows:
        row["energy_vs_plain200"] = row["energy"] / base
    # the fastest learned search whose energy is at most the plain search's
    ok = [row for row in rows if row["search"].startswith("learned") and row["energy"] <= base]
    best = max(ok, key=lambda r: r["px_per_s"]) if ok else None
    net.close()
    pairs.close()
    return {"learned": f"heal{size}", "target_px": wl["target_px"], "train_images": train_images,
            "train_pairs": train_pairs, "dump_s": dump_s, "train_steps": train_steps, "train_s": train_s,
            "train_loss": loss, "rows": rows,
            "learned_vs_plain_px_per_s_at_equal_energy": (best["px_per_s"] / rows[0]["px_per_s"]) if best else None}


def run_learned(args):
    """The full learned-vs-plain table (see learned_comparison)."""
    line = learned_comparison(args.learned_size, args.train_images, args.train_pairs, args.train_steps,
                              [(200, False), (64, False), (16, False), (200, True), (64, True), (16, True),
                               (0, True)])
    print(json.dumps(line), flush=True)


def run_reference_arm(args):
    world, rank, _ = dist_setup()
    if rank != 0:
        return
    # The reference's threaded engine (THREAD_LIMIT = 8 worker threads,
    # lib/buildSwitches.h:89) on a bounded sample per step.
    vals = []
    for i in range(args.warmup + args.steps):
        r = cpu_sample(threads=8)
        if i >= args.warmup:
            vals.append(r)
    total_px = SAMPLE_SIDE * SAMPLE_SIDE * len(vals)
    total_s = sum(v["seconds"] for v in vals)
    value = total_px / total_s
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "target px/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * total_s / len(vals),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
            "config": {"workload": WORKLOAD, "sample": vals[0]["sample"], "threads": 8},
            "cpu_baseline": {"value": value, "unit": "target px/s", "cores": 8, "kind": vals[0]["kind"],
                             "sample": vals[0]["sample"]},
            "e2e": {"value": value, "unit": "target px/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--warps", type=int, default=0,
                    help="warps per CTA of the synthesis kernel (0 = autotuned; fix it when profiling, since the "
                         "tuner's timings are not meaningful under a profiler)")
    ap.add_argument("--profile-once", action="store_true",
                    help="one warm-up and one timed engineDevice call only (for ncu captures)")
    ap.add_argument("--workload", default="render1024",
                    help="render1024 (default), heal256, heal4096, mapstyle2048")
    ap.add_argument("--quality", action="store_true", help="energy against the CPU engine instead of speed")
    ap.add_argument("--quality-runs", type=int, default=3)
    ap.add_argument("--concurrency", type=int, default=8, help="host workers for batch workloads")
    ap.add_argument("--learned", action="store_true", help="learned proposals against the plain search")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-vs-plain object of the bench line")
    ap.add_argument("--learned-size", type=int, default=4096)
    ap.add_argument("--train-images", type=int, default=64)
    ap.add_argument("--train-pairs", type=int, default=2000000)
    ap.add_argument("--train-steps", type=int, default=4000)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference_arm(args)
    if args.quality:
        from resynthesizer_gb300 import build as B
        B.build()
        return run_quality(args)
    if args.learned:
        from resynthesizer_gb300 import build as B
        B.build()
        return run_learned(args)
    if args.workload.startswith("batch"):
        from resynthesizer_gb300 import build as B
        B.build()
        return run_batch(args)

    import numpy as np
    import torch

    import resynthesizer_gb300 as R
    from resynthesizer_gb300 import build as B
    from resynthesizer_gb300 import workloads as W

    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    if rank == 0 or world == 1:
        B.build()
    if world > 1:
        dist.barrier()
    L = R.lib()

    wname, w_target, w_corpus, w_spec, w_params = load_workload(args.workload)
    wl = {"target": w_target, "corpus": w_corpus, "format": w_spec, "params": w_params}
    p = R.params(**wl["params"])
    fmt = R.format_indices(*wl["format"])
    th, tw, _ = wl["target"].shape
    ch, cw, _ = wl["corpus"].shape
    target_px = int((wl["target"][..., 0] != 0).sum())
    dev = torch.device("cuda", local)
    t_init = torch.from_numpy(wl["target"]).to(dev)
    t_work = t_init.clone()
    c_dev = torch.from_numpy(wl["corpus"]).to(dev)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)   # > 129 MB L2
    stream = torch.cuda.current_stream()
    opts = R.options(mode=R.MODE_WAVEFRONT, warpsPerBlock=args.warps)

    def step(o=opts):
        t_work.copy_(t_init)
        rc, st = R.engine_device(p, fmt, t_work.data_ptr(), tw, th, c_dev.data_ptr(), cw, ch,
                                 stream=stream.cuda_stream, opts=o)
        if rc:
            raise RuntimeError(f"engineDevice rc={rc}: {R.last_error()}")
        return st

    if args.profile_once:
        step()
        torch.cuda.synchronize()
        st = step()
        torch.cuda.synchronize()
        print(json.dumps({"profile_once": True, "stats": st}), flush=True)
        return
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()

    # device-resident throughput
    ms, evals, launches = [], 0, 0
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.fill_(1)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            st = step()
            e1.record(stream)
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
            evals += st["evals"]
            launches += st["launches"]
    total_ms = max_over_ranks(sum(ms), dev)
    if world > 1:
        dist.barrier()
    value = replica_throughput(world, args.steps, target_px, total_ms)
    evals_per_s = world * evals / (total_ms / 1000.0)

    # end to end through the reference-facing call with host buffers
    e2e_ms, h2d, d2h = [], 0, 0
    for i in range(args.warmup + args.steps):
        tm, cm = R.PixmapMap(wl["target"]), R.PixmapMap(wl["corpus"])
        stt = R.Stats()
        t0 = time.perf_counter()
        rc = L.engineEx(R.C.byref(p), R.C.byref(fmt), R.C.byref(tm.map), R.C.byref(cm.map), None, None, None,
                        R.C.byref(opts), R.C.byref(stt))
        dt = time.perf_counter() - t0
        assert rc == 0, R.last_error()
        if i >= args.warmup:
            e2e_ms.append(dt * 1000)
            h2d, d2h = stt.h2dBytes, stt.d2hBytes
    e2e_value = world * args.steps * target_px / (sum(e2e_ms) / 1000.0)

    # dominant kernel: the per-target synthesis launches, timed live
    flush.fill_(1)
    torch.cuda.synchronize()
    prof = step(R.options(mode=R.MODE_WAVEFRONT, profile=1, warpsPerBlock=args.warps))
    wave_ms_per_launch = prof["waveMs"] / max(1, prof["waveLaunches"])
    terms_per_launch = prof["waveTerms"] / max(1, prof["waveLaunches"])
    tb, to = term_bytes(fmt.img_match_bpp, fmt.map_match_bpp), term_ops(fmt.img_match_bpp, fmt.map_match_bpp)
    achieved_gbs = terms_per_launch * tb / (wave_ms_per_launch / 1000.0) / 1e9
    peak, peak_kind = peaks()

    # quality of this run (outside every timed region)
    res = R.engine(wl["target"], wl["corpus"], fmt, p, opts=R.options(mode=R.MODE_WAVEFRONT, recordState=1))
    sel = wl["target"][..., 0] != 0
    ys, xs = np.nonzero(sel)
    targets = np.stack([xs, ys], 1).astype(np.int32)
    energy, _ = R.patch_energy(p, fmt, res.out, wl["corpus"], res.has_value, res.source, targets)

    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": "target px/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": {"workload": WORKLOAD if wname == "render1024" else wname, "target": f"{tw}x{th}",
                   "corpus": f"{cw}x{ch}", "target_px": target_px, "mode": "wavefront",
                   "l2": "flushed (256 MB write) between steps, outside the timed intervals",
                   "parallelism": "replicas" if world > 1 else "1 GPU"},
        "evals_per_s": evals_per_s,
        "energy_per_px": energy / target_px,
        "passes": res.stats["passes"],
        "gpu_launches": launches,
        "e2e": {"value": e2e_value, "unit": "target px/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "roofline": {"bound": "hbm", "achieved": achieved_gbs, "peak": peak, "unit": "GB/s",
                     "frac": achieved_gbs / peak, "traffic": WAVE_DRAM_BYTES.get(wname), "kernel": "k_wave",
                     "peak_kind": peak_kind, "launches": prof["waveLaunches"],
                     "ms_per_launch": wave_ms_per_launch, "terms_per_launch": terms_per_launch,
                     "bytes_per_term": tb, "int_ops_per_s": terms_per_launch * to /
                     (wave_ms_per_launch / 1000.0)},
        "clocks": clk.summary(),
    }
    if not args.no_cpu and wname == "render1024":
        mt = cpu_sample(threads=8)
        stt = cpu_sample(threads=1)
        line["cpu_baseline"] = {"value": mt["value"], "unit": "target px/s", "cores": 8, "kind": mt["kind"],
                                "sample": mt["sample"], "single_thread_value": stt["value"]}
        try:
            line["cpu_same_schedule"] = cpu_same_schedule(wl["target"], wl["corpus"], wl["format"], wl["params"],
                                                          res.out, min(16, os.cpu_count() or 1))
        except Exception as e:   # an informative extra: never fails the bench line
            line["cpu_same_schedule"] = {"error": repr(e)[:200]}
    if not args.no_learned and wname == "render1024" and rank == 0:
        # learned vs plain (outside every timed region above): a 1024^2 heal,
        # network trained on pairs from four plain runs, 200 probes each way
        c = learned_comparison(1024, 4, 400000, 1000, [(200, False), (200, True)])
        plain, learned = c["rows"]
        line["learned"] = {"workload": "heal1024: seeded value noise, 40 ellipses ~10 %, P=30, trys=200",
                           "train": {"images": 4, "pairs": c["train_pairs"], "steps": 1000, "seconds": c["train_s"]},
                           "plain_px_per_s": plain["px_per_s"], "learned_px_per_s": learned["px_per_s"],
                           "learned_vs_plain_px_per_s": learned["px_per_s"] / plain["px_per_s"],
                           "learned_energy_vs_plain": learned["energy"] / plain["energy"]}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
