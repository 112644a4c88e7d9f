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
