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

# DRAM bytes (read + write) per launch of the wavefront synthesis kernel, the
# mean over the launches of one synthesis, from one ncu capture
# (dram__bytes_read.sum + dram__bytes_write.sum; profiles/k_wave_persistent_render1024.md):
#   ncu --set full --clock-control none -k regex:k_wave_persistent -s 6 -c 6 \
#       python bench.py --profile-once --no-cpu --no-extra --warps 16
# ncu flushes the caches before each launch, so these are cold-cache figures:
# an upper bound for the warm launches timed here.
WAVE_DRAM_BYTES = {"render1024": 12.84e6}
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


def learned_comparison(size, train_images, train_pairs, train_steps, searches, reps=3, pool=None):
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

    def run(wl, trys, net=None, dump=None, stride=16, state=True, passes=0):
        tgt, cor = W.simple_to_pixmaps(wl["image"], wl["mask"])
        kw = dict(wl["params"])
        kw["maxProbeCount"] = trys
        o = R.options(mode=R.MODE_WAVEFRONT, recordState=1 if state else 0, net=net, proposals=16 if net else 0,
                      dump=dump, dumpStride=stride, proposalPasses=passes)
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
    # training images (seeds 1..N) generated in spawned worker processes when a pool is given
    images = (pool.imap(_cpu_job, [("heal", i, size) for i in range(1, train_images + 1)]) if pool else
              (W.heal4096(index=i, size=size) for i in range(1, train_images + 1)))
    for wl in images:
        run(wl, 200, dump=pairs, stride=max(1, wl["target_px"] // per_image), state=False)
    dump_s = time.perf_counter() - t0
    net = R.Net(seed=1)
    t0 = time.perf_counter()
    loss = net.train(pairs, steps=train_steps, batch=512, lr=1e-3)
    train_s = time.perf_counter() - t0
    wl = W.heal4096(index=0, size=size)
    rows = []
    for search in searches:
        trys, use = search[0], search[1]
        passes = search[2] if len(search) > 2 else 0
        ms = []
        for _ in range(reps):
            r, e = run(wl, trys, net=net if use else None, passes=passes)
            ms.append(r.stats["deviceMs"])
        rows.append({"search": ("learned+" if use else "plain ") + f"trys={trys}" +
                               (f" (proposals in pass 0 only)" if passes == 1 else ""), "energy": e,
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


def learned_mapstyle(out=1024, train_images=8, steps=1000, reps=2):
    """Map-conditioned proposals on the map-guided family (a 512^2 corpus
    with its blurred-luma map -> an out^2 target guided by a smooth map, map
    weight 0.5, P=30): pairs from plain runs over `train_images` problems
    (seeds 1..N; the contexts carry the target map's first channel), the
    network trained on the GPU, then the held-out problem (seed 0) with and
    without its 16 proposals."""
    import numpy as np

    import resynthesizer_gb300 as R
    from resynthesizer_gb300 import workloads as W

    def run(wl, trys, net=None, dump=None):
        kw = dict(wl["params"], maxProbeCount=trys)
        fmt = R.format_indices(*wl["format"])
        r = R.engine(wl["target"], wl["corpus"], fmt, R.params(**kw),
                     opts=R.options(mode=R.MODE_WAVEFRONT, recordState=1, net=net, proposals=16 if net else 0,
                                    dump=dump, dumpStride=4))
        assert r.rc == 0, R.last_error()
        ys, xs = np.nonzero(wl["target"][..., 0] != 0)
        t = np.stack([xs, ys], 1).astype(np.int32)
        e, _ = R.patch_energy(R.params(**kw), fmt, r.out, wl["corpus"], r.has_value, r.source, t)
        return r, e

    pairs = R.Pairs(2000000)
    for i in range(1, train_images + 1):
        run(W.mapstyle(512, out, index=i), 200, dump=pairs)
    net = R.Net(seed=1)
    t0 = time.perf_counter()
    loss = net.train(pairs, steps=steps, batch=512, lr=1e-3)
    train_s = time.perf_counter() - t0
    wl = W.mapstyle(512, out, index=0)
    rows = []
    for trys, use in ((200, False), (64, False), (200, True), (64, True)):
        ms = []
        for _ in range(reps):
            r, e = run(wl, trys, net=net if use else None)
            ms.append(r.stats["deviceMs"])
        rows.append({"search": ("learned+" if use else "plain ") + f"trys={trys}", "energy": e, "ms": min(ms),
                     "px_per_s": out * out / (min(ms) / 1000.0)})
    for row in rows:
        row["energy_vs_plain200"] = row["energy"] / rows[0]["energy"]
    npairs = len(pairs)
    net.close()
    pairs.close()
    return {"learned": f"mapstyle{out}: 512^2 corpus + map, map weight 0.5, P=30, map channel in the context",
            "train_problems": train_images, "train_pairs": npairs, "train_steps": steps, "train_s": train_s,
            "train_loss": loss, "rows": rows}


def run_learned(args):
    """The full learned-vs-plain table (see learned_comparison)."""
    line = learned_comparison(args.learned_size, args.train_images, args.train_pairs, args.train_steps,
                              [(200, False), (64, False), (16, False), (200, True), (64, True), (16, True),
                               (0, True)])
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------ CPU helpers

def cpu_engine(name: str, threads: int, want_energy: bool = True):
    """The CPU engine (the reference built from its sources where present,
    else its oracle port) on the whole workload `name`: (seconds, energy,
    kind, output pixmap).  Energy = the full-patch metric summed over the
    targets at their final sources, computed by the oracle's restatement of
    computeBestFit (bit-exact with the GPU's resynthPatchEnergy)."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    _, tgt, cor, spec, kw = load_workload(name)
    o = O.Oracle()
    fmt = o.format_indices(*spec)
    p = O.make_params(**kw)
    kind = "port"
    t0 = time.perf_counter()
    if O.reference_available(threaded=threads > 1):
        rc, out, src, hv = O.Reference(threaded=threads > 1).engine_state(p, fmt, tgt, cor)
        kind = "reference"
    else:
        rc, out, _, src, hv = o.engine(p, fmt, tgt, cor, threads=threads, want_state=True)
    dt = time.perf_counter() - t0
    assert rc == 0
    e = None
    if want_energy:
        ys, xs = np.nonzero(tgt[..., 0] != 0)
        targets = np.stack([xs, ys], 1).astype(np.int32)
        e, _ = o.energy(p, fmt, out, cor, hv, src, targets)
    return dt, e, kind, out


def _cpu_job(job):
    """Pool worker (spawned processes, never forked from the GPU process)."""
    kind = job[0]
    if kind == "engine":
        dt, e, k, _ = cpu_engine(job[1], job[2])
        return dt, e, k
    from resynthesizer_gb300 import workloads as W
    if kind == "batch":
        return W.batch_request(job[1])
    if kind == "heal":
        return W.heal4096(index=job[1], size=job[2])
    raise ValueError(kind)


def spawn_pool(n: int):
    import multiprocessing as mp
    return mp.get_context("spawn").Pool(n)


def cpu_reference_energies(name: str, mt_runs: int):
    """The single-threaded engine once, alone (its time is the CPU baseline),
    then `mt_runs` runs of the threaded engine (8 threads, nondeterministic)
    in spawned processes, at most six side by side (more at once would load
    the host cores more than the earlier lines did and shift the threaded
    engine's interleaving), for their energies."""
    st_s, st_e, kind, st_out = cpu_engine(name, 1)
    mt = []
    if mt_runs:
        with spawn_pool(min(mt_runs, 6)) as pool:
            mt = pool.map(_cpu_job, [("engine", name, 8)] * mt_runs)
    return dict(st_seconds=st_s, st_energy=st_e, kind=kind, st_out=st_out,
                mt_energies=[m[1] for m in mt], mt_seconds=[m[0] for m in mt])


def energy_vs_reference(e_gpu: float, ref: dict) -> dict:
    import numpy as np
    mt = ref["mt_energies"]
    mt_mean = float(np.mean(mt)) if mt else None
    d = {"gpu_energy": e_gpu, "cpu_st_energy": ref["st_energy"], "gpu_over_st": e_gpu / ref["st_energy"],
         "cpu_mt_energies": mt, "cpu_mt_mean": mt_mean,
         "gpu_over_mt_mean": e_gpu / mt_mean if mt_mean else None,
         "mt_spread": (max(mt) - min(mt)) / mt_mean if mt_mean else None,
         # the threaded engine is nondeterministic: the standard error of its
         # mean, relative, says how far the gate's denominator moves run to run
         "mt_mean_rel_stderr": float(np.std(mt, ddof=1) / np.sqrt(len(mt)) / mt_mean) if len(mt) > 1 else None,
         "mt_seconds": ref.get("mt_seconds"),
         "mt_runs_at_or_above_gpu": sum(1 for m in mt if m >= e_gpu) if mt else None,
         "cpu_kind": ref["kind"],
         "gate": "wavefront energy at most 1.01 x the threaded reference's mean (one-sided: lower is better)"}
    if mt_mean:
        d["gate_pass"] = bool(e_gpu <= 1.01 * mt_mean)
    return d


# ------------------------------------------------------------ reference arm

def run_reference_arm(args):
    """The reference's CPU engine on this machine's host cores, on the same
    workload as the default GPU line (render1024, the whole 1024x1024 target
    every step).  Its single-threaded build is the value: the threaded build
    (THREAD_LIMIT 8 workers, lib/buildSwitches.h:89) serialises on a global
    mutex and one shared rand() and runs about 5x slower on the same input
    (one full-size run of it is reported beside).  Warm-up steps run a
    256x256 sample; every timed step the full workload."""
    world, rank, _ = dist_setup()
    if rank != 0:
        return
    for _ in range(args.warmup):
        cpu_sample(threads=1)
    secs, kind = [], None
    for _ in range(args.steps):
        dt, _, kind, _ = cpu_engine("render1024", 1, want_energy=False)
        secs.append(dt)
    px = 1024 * 1024
    value = px * len(secs) / sum(secs)
    mt_s, _, mt_kind, _ = cpu_engine("render1024", 8, want_energy=False)
    sample = "the whole workload (1024x1024 target) every timed step; single-threaded engine"
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "target px/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * sum(secs) / len(secs),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
            "config": {"workload": WORKLOAD, "target": "1024x1024", "corpus": "128x128", "target_px": px,
                       "threads": 1, "same_config": True, "warmup_sample": "256x256 target from the same tile"},
            "cpu_baseline": {"value": value, "unit": "target px/s", "cores": 1, "kind": kind, "sample": sample},
            "threaded": {"value": px / mt_s, "unit": "target px/s", "threads": 8, "kind": mt_kind,
                         "sample": "the whole workload, one run"},
            "e2e": {"value": value, "unit": "target px/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------- GPU measurements

def device_timing(R, torch, wl: dict, opts, steps: int, warmup: int, flush, stream):
    """engineDevice on pixmaps resident in device memory: per step a fresh
    target copy and an L2 flush (outside the timed interval), then the
    synthesis timed with CUDA events on the call's stream."""
    dev = flush.device
    tgt, cor = wl["target"], wl["corpus"]
    th, tw, _ = tgt.shape
    ch, cw, _ = cor.shape
    t_init = torch.from_numpy(tgt).to(dev)
    t_work = t_init.clone()
    c_dev = torch.from_numpy(cor).to(dev)
    p = R.params(**wl["params"])
    fmt = R.format_indices(*wl["format"])
    ms, stats = [], []
    for i in range(warmup + steps):
        t_work.copy_(t_init)
        flush.fill_(1)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        rc, st = R.engine_device(p, fmt, t_work.data_ptr(), tw, th, c_dev.data_ptr(), cw, ch,
                                 stream=stream.cuda_stream, opts=opts)
        e1.record(stream)
        torch.cuda.synchronize()
        if rc:
            raise RuntimeError(f"engineDevice rc={rc}: {R.last_error()}")
        if i >= warmup:
            ms.append(e0.elapsed_time(e1))
            stats.append(st)
    return ms, stats


def e2e_engine(R, wl: dict, opts, steps: int, warmup: int):
    """engineEx on host Maps (the reference's engine() call with options):
    host->device copies, synthesis and the device->host copy of the target,
    wall-clock timed around the C call."""
    L = R.lib()
    p = R.params(**wl["params"])
    fmt = R.format_indices(*wl["format"])
    ms, h2d, d2h = [], 0, 0
    for i in range(warmup + steps):
        tm, cm = R.PixmapMap(wl["target"]), R.PixmapMap(wl["corpus"])
        stt = R.Stats()
        t0 = time.perf_counter()
        rc = L.engineEx(R.C.byref(p), R.C.byref(fmt), R.C.byref(tm.map), R.C.byref(cm.map), None, None, None,
                        R.C.byref(opts), R.C.byref(stt))
        dt = time.perf_counter() - t0
        assert rc == 0, R.last_error()
        if i >= warmup:
            ms.append(dt * 1000)
            h2d, d2h = stt.h2dBytes, stt.d2hBytes
    return ms, h2d, d2h


def e2e_image_synth(R, image, mask, fmt: int, params: dict, opts, steps: int, warmup: int):
    """imageSynthEx on the caller's row buffers (the reference's imageSynth
    call with options), wall-clock timed around the C call; the image is
    restored between calls outside the timed interval."""
    import numpy as np
    L = R.lib()
    p = R.params(**params)
    img = np.ascontiguousarray(image).copy()
    m = np.ascontiguousarray(mask)
    ib, mb = R._buf(img), R._buf(m)
    cf = R.C.c_int(0)
    ms, h2d, d2h = [], 0, 0
    for i in range(warmup + steps):
        img[...] = image
        st = R.Stats()
        t0 = time.perf_counter()
        rc = L.imageSynthEx(R.C.byref(ib), R.C.byref(mb), None, fmt, R.C.byref(p), None, None, R.C.byref(cf),
                            R.C.byref(opts), R.C.byref(st))
        dt = time.perf_counter() - t0
        assert rc == 0, R.last_error()
        if i >= warmup:
            ms.append(dt * 1000)
            h2d, d2h = st.h2dBytes, st.d2hBytes
    return ms, h2d, d2h, img


def gpu_energy(R, wl: dict, out, has_value, source):
    import numpy as np
    sel = wl["target"][..., 0] != 0
    ys, xs = np.nonzero(sel)
    targets = np.stack([xs, ys], 1).astype(np.int32)
    e, _ = R.patch_energy(R.params(**wl["params"]), R.format_indices(*wl["format"]), out, wl["corpus"], has_value,
                          source, targets)
    return e


def workload_dict(name: str) -> dict:
    wname, t, c, spec, kw = load_workload(name)
    return {"name": wname, "target": t, "corpus": c, "format": spec, "params": kw,
            "target_px": int((t[..., 0] != 0).sum())}


def sub_line(R, torch, name, flush, stream, steps=5, warmup=2, pool=None, mt_runs=0):
    """Figures of one more workload of the survey's set, all outside the
    main line's timed region: device-resident and end-to-end px/s, energy,
    and -- where the CPU engine finishes in seconds -- its energy beside."""
    import numpy as np
    from resynthesizer_gb300 import workloads as W
    t0 = time.perf_counter()
    wl = workload_dict(name)
    gen_s = time.perf_counter() - t0
    opts = R.options(mode=R.MODE_WAVEFRONT)
    ms, stats = device_timing(R, torch, wl, opts, steps, warmup + 6, flush, stream)   # 6: the launch tuning
    d = {"workload": name, "target_px": wl["target_px"], "generation_s": gen_s,
         "device_px_per_s": wl["target_px"] / (min(ms) / 1000.0), "device_ms": ms,
         "evals_per_s": stats[0]["evals"] / (min(ms) / 1000.0), "passes": stats[0]["passes"],
         "launches": stats[0]["launches"]}
    if name.startswith("heal"):
        heal = W.heal256() if name == "heal256" else W.heal4096()
        ems, h2d, d2h, _ = e2e_image_synth(R, heal["image"], heal["mask"], heal["fmt"], heal["params"], opts, steps,
                                           warmup)
        d["e2e"] = {"value": wl["target_px"] / (np.median(ems) / 1000.0), "unit": "target px/s",
                    "call": "imageSynthEx on host row buffers", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h}
    else:
        ems, h2d, d2h = e2e_engine(R, wl, opts, steps, warmup)
        d["e2e"] = {"value": wl["target_px"] / (np.median(ems) / 1000.0), "unit": "target px/s",
                    "call": "engineEx on host Maps", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h}
    res = R.engine(wl["target"], wl["corpus"], R.format_indices(*wl["format"]), R.params(**wl["params"]),
                   opts=R.options(mode=R.MODE_WAVEFRONT, recordState=1))
    e = gpu_energy(R, wl, res.out, res.has_value, res.source)
    d["energy_per_px"] = e / wl["target_px"]
    if mt_runs:
        ref = cpu_reference_energies(name, mt_runs)
        d["energy_vs_reference"] = energy_vs_reference(e, ref)
        d["cpu_single_thread_px_per_s"] = wl["target_px"] / ref["st_seconds"]
        if name == "heal256":
            r = R.engine(wl["target"], wl["corpus"], R.format_indices(*wl["format"]), R.params(**wl["params"]),
                         opts=R.options(mode=R.MODE_REPLAY))
            d["replay"] = {"ms": r.stats["deviceMs"], "identical_to_cpu_single_thread":
                           bool(r.rc == 0 and np.array_equal(r.out, ref["st_out"]))}
    else:
        d["energy_vs_reference"] = ("not run here: the CPU engine needs minutes at this size "
                                    "(its offline figure is in the design notes)")
    return d


def batch_line(R, n: int, pool, steps=2):
    """Batched heal requests through imageSynthBatch with host buffers."""
    from resynthesizer_gb300 import workloads as W
    t0 = time.perf_counter()
    specs = W.batch_specs(n=n)
    reqs = pool.map(_cpu_job, [("batch", sp) for sp in specs], chunksize=4) if pool else \
        [W.batch_request(sp) for sp in specs]
    gen_s = time.perf_counter() - t0
    items = [(r["image"], r["mask"], r["fmt"], R.params(**r["params"])) for r in reqs]
    px = sum(r["target_px"] for r in reqs)
    opts = R.options(mode=R.MODE_WAVEFRONT)
    rc, _, _, _ = R.image_synth_batch(items[:16], opts=opts)
    assert rc == 0, R.last_error()
    ts, st = [], None
    for _ in range(steps):
        t1 = time.perf_counter()
        rc, _, codes, st = R.image_synth_batch(items, opts=opts)
        ts.append(time.perf_counter() - t1)
        assert rc == 0, R.last_error()
    return {"workload": f"batch{n}: {n} heal requests, 128..1024 px sides, Gray/RGB/RGBA, holes 2-20 %, "
                        f"P in {{9,16,30}}, trys=200, imageSynthBatch", "requests": n, "target_px": px,
            "generation_s": gen_s, "e2e": {"value": px / min(ts), "unit": "target px/s",
                                           "call": "imageSynthBatch on host row buffers (wall clock)",
                                           "h2d_bytes_per_step": st["h2dBytes"], "d2h_bytes_per_step": st["d2hBytes"]},
            "ms": [1000 * t for t in ts], "launches": st["launches"], "device_ms": st["deviceMs"],
            "evals_per_s": st["evals"] / min(ts)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baselines and energies")
    ap.add_argument("--no-extra", action="store_true",
                    help="only the main line (no other workloads, no learned comparison)")
    ap.add_argument("--warps", type=int, default=0,
                    help="warps per CTA of the synthesis kernel (0 = autotuned; fix it when profiling, since the "
                         "tuner's timings are not meaningful under a profiler)")
    ap.add_argument("--profile-once", action="store_true",
                    help="one warm-up and one timed engineDevice call only (for ncu captures)")
    ap.add_argument("--batch-launches", action="store_true",
                    help="one kernel launch per batch instead of one persistent launch per pass")
    ap.add_argument("--workload", default="render1024",
                    help="render1024 (default), heal256, heal4096, mapstyle2048, batchN")
    ap.add_argument("--quality", action="store_true", help="energy against the CPU engine instead of speed")
    ap.add_argument("--quality-runs", type=int, default=3)
    ap.add_argument("--mt-runs", type=int, default=12, help="threaded CPU runs for the energy gate")
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

    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    if rank == 0 or world == 1:
        B.build()
    if world > 1:
        dist.barrier()

    wl = workload_dict(args.workload)
    wname = wl["name"]
    p = R.params(**wl["params"])
    fmt = R.format_indices(*wl["format"])
    th, tw, _ = wl["target"].shape
    ch, cw, _ = wl["corpus"].shape
    target_px = wl["target_px"]
    dev = torch.device("cuda", local)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)   # > 129 MB L2
    stream = torch.cuda.current_stream()
    opts = R.options(mode=R.MODE_WAVEFRONT, warpsPerBlock=args.warps, batchLaunches=1 if args.batch_launches else 0)

    # The library picks how each problem class's passes are launched from the
    # device times of its first six calls (two of each configuration): those
    # calls run here, untimed, before the warm-up.
    tune_calls = 0 if (args.batch_launches or args.warps) else 6
    if args.profile_once:
        device_timing(R, torch, wl, opts, 0, tune_calls, flush, stream)
        ms, stats = device_timing(R, torch, wl, opts, 1, 1, flush, stream)
        print(json.dumps({"profile_once": True, "ms": ms, "stats": stats[0]}), flush=True)
        return
    device_timing(R, torch, wl, opts, 0, tune_calls + args.warmup, flush, stream)
    if world > 1:
        dist.barrier()

    # device-resident throughput (the timed region)
    with ClockSampler(local) as clk:
        ms, stats = device_timing(R, torch, wl, opts, args.steps, 0, flush, stream)
    total_ms = max_over_ranks(sum(ms), dev)
    if world > 1:
        dist.barrier()
    value = replica_throughput(world, args.steps, target_px, total_ms)
    evals_per_s = world * sum(s["evals"] for s in stats) / (total_ms / 1000.0)
    launches = sum(s["launches"] for s in stats)

    # end to end through the reference-facing call with host buffers
    e2e_ms, h2d, d2h = e2e_engine(R, wl, opts, args.steps, args.warmup)
    e2e_value = world * args.steps * target_px / (sum(e2e_ms) / 1000.0)

    # dominant kernel: the wavefront synthesis launches, timed live with CUDA
    # events on the library's stream, against the two on-chip peaks that
    # bound it (measured here) and, as a secondary figure, the HBM copy peak
    _, pst = device_timing(R, torch, wl, R.options(mode=R.MODE_WAVEFRONT, profile=1, warpsPerBlock=args.warps,
                                                   batchLaunches=1 if args.batch_launches else 0), 1, 0, flush,
                                  stream)
    prof = pst[0]
    wave_ms_per_launch = prof["waveMs"] / max(1, prof["waveLaunches"])
    terms_per_launch = prof["waveTerms"] / max(1, prof["waveLaunches"])
    tb, to = term_bytes(fmt.img_match_bpp, fmt.map_match_bpp), term_ops(fmt.img_match_bpp, fmt.map_match_bpp)
    smem_peak, _ = R.microbench(0)
    int_peak, _ = R.microbench(1)
    hbm_peak, hbm_kind = peaks()
    sec = wave_ms_per_launch / 1000.0
    smem_gbs = terms_per_launch * tb / sec / 1e9
    int_gops = terms_per_launch * to / sec / 1e9
    fr = {"smem": smem_gbs / smem_peak, "int32": int_gops / int_peak}
    bound = max(fr, key=fr.get)
    roof = {"bound": bound, "achieved": smem_gbs if bound == "smem" else int_gops,
            "peak": smem_peak if bound == "smem" else int_peak, "unit": "GB/s" if bound == "smem" else "G int ops/s",
            "frac": fr[bound], "traffic": WAVE_DRAM_BYTES.get(wname),
            "kernel": "k_wave" if prof.get("launchMode") == 2 else "k_wave_persistent",
            "launch_mode": {0: "persistent, 16 warps per CTA", 1: "persistent, 8 warps per CTA",
                            2: "one launch per batch", 3: "persistent"}.get(prof.get("launchMode")),
            "peak_source": "measured in this run: resynthMicrobench (conflict-free 16-byte shared loads; chains of "
                           "32-bit add and xor), best of five CUDA-event-timed launches",
            "smem": {"achieved": smem_gbs, "peak": smem_peak, "unit": "GB/s", "frac": fr["smem"],
                     "bytes_per_term": tb},
            "int32": {"achieved": int_gops, "peak": int_peak, "unit": "G ops/s", "frac": fr["int32"],
                      "ops_per_term": to},
            "hbm": {"achieved": smem_gbs, "peak": hbm_peak, "unit": "GB/s", "frac": smem_gbs / hbm_peak,
                    "peak_kind": hbm_kind, "note": "algorithmic bytes over the HBM copy peak; the corpus and "
                                                  "tables are read from shared memory and L1, DRAM traffic is the "
                                                  "'traffic' figure"},
            "launches": prof["waveLaunches"], "ms_per_launch": wave_ms_per_launch,
            "terms_per_launch": terms_per_launch}

    # quality of this run (outside every timed region)
    res = R.engine(wl["target"], wl["corpus"], fmt, p, opts=R.options(mode=R.MODE_WAVEFRONT, recordState=1))
    energy = gpu_energy(R, wl, res.out, res.has_value, res.source)

    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": "target px/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": {"workload": WORKLOAD if wname == "render1024" else wname, "target": f"{tw}x{th}",
                   "corpus": f"{cw}x{ch}", "target_px": target_px, "mode": "wavefront",
                   "launch": "one launch per batch" if args.batch_launches else
                             "tuned per problem class: persistent launches per pass or one launch per batch",
                   "l2": "flushed (256 MB write) between steps, outside the timed intervals",
                   "autotune_calls": f"{tune_calls} untimed calls before the warm-up, in which the library times "
                                     "its launch configurations",
                   "parallelism": "replicas" if world > 1 else "1 GPU"},
        "evals_per_s": evals_per_s,
        "energy_per_px": energy / target_px,
        "passes": res.stats["passes"],
        "gpu_launches": launches,
        "e2e": {"value": e2e_value, "unit": "target px/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "roofline": roof,
        "clocks": clk.summary(),
    }
    if not args.no_cpu and wname == "render1024":
        ref = cpu_reference_energies("render1024", args.mt_runs)
        line["cpu_baseline"] = {"value": target_px / ref["st_seconds"], "unit": "target px/s", "cores": 1,
                                "kind": ref["kind"], "sample": "the whole workload (1024x1024 target), one run of "
                                                              "the single-threaded engine"}
        line["energy_vs_reference"] = energy_vs_reference(energy, ref)
        line["energy_vs_reference"]["psnr_vs_cpu_st"] = psnr(res.out[..., 1:4], ref["st_out"][..., 1:4])
        try:
            line["cpu_same_schedule"] = cpu_same_schedule(wl["target"], wl["corpus"], wl["format"], wl["params"],
                                                          res.out, min(16, os.cpu_count() or 1))
        except Exception as e:   # an informative extra: never fails the bench line
            line["cpu_same_schedule"] = {"error": repr(e)[:200]}
    if not args.no_extra and wname == "render1024":
        extra = {}
        with spawn_pool(min(16, os.cpu_count() or 1)) as pool:
            for name in ("heal256", "heal4096", "mapstyle2048"):
                try:
                    extra[name] = sub_line(R, torch, name, flush, stream,
                                           mt_runs=0 if (args.no_cpu or name != "heal256") else 5)
                except Exception as e:
                    extra[name] = {"error": repr(e)[:300]}
            try:
                extra["batch512"] = batch_line(R, 512, pool)
            except Exception as e:
                extra["batch512"] = {"error": repr(e)[:300]}
            if not args.no_learned:
                try:
                    extra["learned_heal4096"] = learned_comparison(4096, 64, 2000000, 4000,
                                                                   [(200, False), (64, False), (16, False),
                                                                    (200, True), (64, True), (16, True),
                                                                    (64, True, 1), (16, True, 1)], reps=2,
                                                                   pool=pool)
                except Exception as e:
                    extra["learned_heal4096"] = {"error": repr(e)[:300]}
                try:
                    extra["learned_mapstyle1024"] = learned_mapstyle()
                except Exception as e:
                    extra["learned_mapstyle1024"] = {"error": repr(e)[:300]}
        line["workloads"] = extra
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
