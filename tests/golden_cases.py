"""Loads the golden fixtures of tests/golden/ (made by make_golden.py from the
reference engine) as plain dicts, for the oracle and the GPU parity tests."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(name):
    return np.load(os.path.join(GOLDEN, name), allow_pickle=False)


def params_kw(v):
    return dict(tileH=int(v[0]), tileV=int(v[1]), matchContextType=int(v[2]), mapWeight=float(v[3]),
                sensitivity=float(v[4]), patchSize=int(v[5]), maxProbeCount=int(v[6]))


def testsynth():
    z = _load("testsynth.npz")
    return [dict(name=str(z[f"{i}_name"]), image=z[f"{i}_image"], mask=z[f"{i}_mask"], fmt=int(z[f"{i}_fmt"]),
                 params=None if bool(z[f"{i}_null_params"]) else params_kw(z[f"{i}_params"]),
                 rc=int(z[f"{i}_rc"]), out=z[f"{i}_out"]) for i in range(int(z["count"]))]


def heal():
    z = _load("heal.npz")
    return [dict(image=z[f"{k}_image"], mask=z[f"{k}_mask"], fmt=int(z[f"{k}_fmt"]),
                 params=params_kw(z[f"{k}_params"]), out=z[f"{k}_out"]) for k in range(int(z["count"]))]


def heal256():
    z = _load("heal256.npz")
    return dict(image=z["image"], mask=z["mask"], fmt=int(z["fmt"]), params=params_kw(z["params"]),
                out_region=z["out_region"], sha256=str(z["sha256"]))


def engine():
    z = _load("engine.npz")
    return [dict(name=str(z[f"{k}_name"]), target=z[f"{k}_target"], corpus=z[f"{k}_corpus"],
                 format=tuple(int(v) for v in z[f"{k}_format"]), params=params_kw(z[f"{k}_params"]),
                 out=z[f"{k}_out"], source=z[f"{k}_source"], has=z[f"{k}_has"]) for k in range(int(z["count"]))]


def frozen():
    z = _load("frozen.npz")
    keys = ["target", "corpus", "has", "source", "targets", "start", "cands", "sum", "pt", "count"]
    out = []
    for k in range(int(z["count"])):
        d = {n: z[f"{k}_{n}"] for n in keys}
        d["format"] = tuple(int(v) for v in z[f"{k}_format"])
        d["params"] = params_kw(z[f"{k}_params"])
        out.append(d)
    return out


# sha256 of the target pixmap after engine() in the library's default mode
# (wavefront, default options), with the passes run and the betters of each
# pass.  The CPU wavefront oracle (oracle/wave_oracle.c) and the CUDA library
# on a GB300 give these same outputs.
WAVE_FULL = {
    "render1024": ("710baea67bc0c8500ffee84cb1251b01baeb669d22987efcde6304f5d6489edd", 3, [1048576, 51668, 23402]),
    "heal4096": ("6339cdc79ad835d4363eb096c3facba71d2cc81fc663fc10540c6c1cd4146d65", 2, [1523352, 59388]),
    "mapstyle2048": ("289dc9dd0a88eb8e04c691afe903695b2818f3472e1c91282c3eaacfc072eaf4", 2, [4194304, 71676]),
}


def wave_workload(name):
    """(target pixmap, corpus pixmap, prepareImageFormatIndices arguments, params) of a
    full-size workload, as bench.py builds it."""
    from resynthesizer_gb300 import workloads as W
    if name == "render1024":
        wl = W.render1024()
        return wl["target"], wl["corpus"], wl["format"], wl["params"]
    if name == "mapstyle2048":
        wl = W.mapstyle()
        return wl["target"], wl["corpus"], wl["format"], wl["params"]
    wl = W.heal4096()
    t, c = W.simple_to_pixmaps(wl["image"], wl["mask"])
    return t, c, (3, 0, 0, 0, 0), wl["params"]


# Small wavefront cases (corpus staged in shared memory, teams of warps per
# target, tiling, maps): output hash, passes, betters per pass.  The CUDA
# library and the CPU wavefront oracle give these same outputs.
WAVE_SMALL = {
    "heal": ("c242d24b4fd897e0f3b05f1f20d2c53a1b2334934f660664a5eb2ae4230e2eed", 3, [196, 39, 5]),
    "render": ("ab1318035955c00230beda01b7983e6105570027b8bdc5d8e9dc027a666a06ef", 3, [4096, 558, 217]),
    "render_tiled": ("3fedb93d5756a96d6ca9558a2285e458ab9a3cd3d148a05d755a976f38c985a0", 3, [4096, 762, 313]),
    "mapstyle": ("53045f164606779ffc8d67ff21b240a025e9e2b1e80ae75538d6581e8fdad6e9", 2, [4096, 292]),
}


def wave_small_case(case):
    """(target pixmap, corpus pixmap, prepareImageFormatIndices arguments, params) of a small
    wavefront case."""
    from resynthesizer_gb300 import workloads as W
    if case == "heal":
        wl = W.heal_small(size=48, hole=14, ctype=1, patch=16, trys=80)
        t, c = W.simple_to_pixmaps(wl["image"], wl["mask"])
        return t, c, (3, 0, 0, 0, 0), wl["params"]
    if case.startswith("render"):
        wl = W.render(tile=24, out=64)
        kw = dict(wl["params"])
        if case == "render_tiled":
            kw.update(tileH=1, tileV=1)
        return wl["target"], wl["corpus"], wl["format"], kw
    wl = W.mapstyle(corpus_size=40, out=64)
    return wl["target"], wl["corpus"], wl["format"], wl["params"]
