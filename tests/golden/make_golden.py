"""Generates the golden fixtures in tests/golden/ from the reference engine
compiled from its own sources (oracle/build_ref.sh).

    sh oracle/build_ref.sh && python tests/golden/make_golden.py

Each .npz holds the exact inputs (so no generator has to reproduce them
bit-for-bit on another machine) and the reference's outputs:
  testsynth.npz   the known-answer cases of the reference's src/testSynth.c:87-224
                  (inputs restated from its buffers; outputs and return codes
                  from the reference run here)
  heal.npz        simple-API heals: 4 formats x orderings, small images
  heal256.npz     the 256x256 RGB heal workload: full input, target-region output
                  and the SHA-256 of the whole output image
  engine.npz      engine() on pixmaps: tiled render and map-guided cases, with the
                  final sourceOf/hasValue state
  frozen.npz      frozen-state best fits (random state, random candidate lists)
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from oracle import Reference, make_params  # noqa: E402
from resynthesizer_gb300 import workloads as W  # noqa: E402


def params_vec(p):
    return np.array([p.tileH, p.tileV, p.matchContextType, p.mapWeight, p.sensitivityToOutliers,
                     p.patchSize, p.maxProbeCount], np.float64)


def testsynth_cases():
    """The buffers of src/testSynth.c:91-147 without row padding (the padding
    bytes are never read), as (name, image, mask, format, params or None)."""
    P = make_params()
    img33 = np.array([[0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0],
                      [0, 0, 0, 0, 1, 1, 1, 1, 0, 0, 0, 0],
                      [0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 8]], np.uint8).reshape(3, 3, 4)
    m33 = np.array([[0, 0, 0], [0, 255, 0], [0, 0, 0]], np.uint8)
    img2 = np.array([[128, 128, 128, 255, 1, 1, 1, 1, 0, 0, 0, 0]], np.uint8).reshape(1, 3, 4)
    m2 = np.array([[0, 255, 0]], np.uint8)
    img3 = np.array([[128, 128, 128, 0, 1, 1, 1, 1, 0, 0, 0, 0]], np.uint8).reshape(1, 3, 4)
    rgb = np.array([[128, 128, 128, 1, 1, 1, 2, 2, 2], [64, 64, 64, 4, 4, 4, 3, 3, 3]], np.uint8).reshape(2, 3, 3)
    m3 = np.array([[0, 0, 0], [0, 255, 0]], np.uint8)
    ga = np.array([[128, 255, 64, 1, 1, 0]], np.uint8).reshape(1, 3, 2)
    g = np.array([[128, 64, 1]], np.uint8).reshape(1, 3, 1)
    big = make_params(patchSize=65)
    p10 = make_params(patchSize=10)
    return [
        ("center_rgba", img33, m33, W.T_RGBA, P),
        ("mixed_transparency", img2, m2, W.T_RGBA, P),
        ("rgb_no_alpha", rgb, m3, W.T_RGB, P),
        ("gray_alpha", ga, m2, W.T_GrayA, P),
        ("gray_null_params", g, m2, W.T_Gray, None),
        ("all_transparent", img3, m2, W.T_RGBA, P),
        ("patch_65", g, m2, W.T_Gray, big),
        ("mask_mismatch", g, np.array([[0]], np.uint8), W.T_Gray, p10),
        ("empty_mask", g, np.zeros((1, 3), np.uint8), W.T_Gray, p10),
        ("invalid_format", g, m2, 666, p10),
    ]


def main():
    ref = Reference()
    out = {}
    for i, (name, img, mask, fmt, p) in enumerate(testsynth_cases()):
        rc, res = ref.image_synth(img, mask, fmt, p)
        out[f"{i}_image"] = img
        out[f"{i}_mask"] = mask
        out[f"{i}_fmt"] = np.array(fmt)
        out[f"{i}_params"] = params_vec(p if p is not None else make_params())
        out[f"{i}_null_params"] = np.array(p is None)
        out[f"{i}_rc"] = np.array(rc)
        out[f"{i}_out"] = res
        out[f"{i}_name"] = np.array(name)
    out["count"] = np.array(len(testsynth_cases()))
    np.savez_compressed(os.path.join(HERE, "testsynth.npz"), **out)

    out, k = {}, 0
    for fmt in (W.T_RGB, W.T_RGBA, W.T_Gray, W.T_GrayA):
        for ctype in (1, 2, 5, 8):
            wl = W.heal_small(size=28, hole=9, fmt=fmt, ctype=ctype, patch=16, trys=40, index=ctype)
            p = make_params(**wl["params"])
            rc, res = ref.image_synth(wl["image"], wl["mask"], fmt, p)
            assert rc == 0
            out.update({f"{k}_image": wl["image"], f"{k}_mask": wl["mask"], f"{k}_fmt": np.array(fmt),
                        f"{k}_params": params_vec(p), f"{k}_out": res})
            k += 1
    out["count"] = np.array(k)
    np.savez_compressed(os.path.join(HERE, "heal.npz"), **out)

    wl = W.heal256()
    p = make_params(**wl["params"])
    rc, res = ref.image_synth(wl["image"], wl["mask"], wl["fmt"], p)
    assert rc == 0
    np.savez_compressed(os.path.join(HERE, "heal256.npz"), image=wl["image"], mask=wl["mask"],
                        fmt=np.array(wl["fmt"]), params=params_vec(p), out_region=res[96:160, 96:160],
                        sha256=np.array(hashlib.sha256(res.tobytes()).hexdigest()))

    out = {}
    cases = [("render_tiled", W.render(tile=16, out=40), dict(tileH=1, tileV=1)),
             ("render", W.render(tile=20, out=48), {}),
             ("mapstyle", W.mapstyle(corpus_size=24, out=40), {})]
    for k, (name, wl, extra) in enumerate(cases):
        p = make_params(**dict(wl["params"], **extra))
        from oracle import Format  # noqa: F401
        fmt = ref_format(wl["format"])
        rc, t, s, h = ref.engine_state(p, fmt, wl["target"], wl["corpus"])
        assert rc == 0
        out.update({f"{k}_target": wl["target"], f"{k}_corpus": wl["corpus"], f"{k}_format": np.array(wl["format"]),
                    f"{k}_params": params_vec(p), f"{k}_out": t, f"{k}_source": s, f"{k}_has": h,
                    f"{k}_name": np.array(name)})
    out["count"] = np.array(len(cases))
    np.savez_compressed(os.path.join(HERE, "engine.npz"), **out)

    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from test_oracle_pin import _random_state
    out = {}
    fmts = [(3, 0, 0, 0, 0), (3, 0, 1, 1, 0), (1, 0, 0, 0, 0), (3, 1, 0, 0, 1)]
    for k, fm in enumerate(fmts):
        target, corpus, hv, src, targets, start, cands = _random_state(10 + k, fmt=fm)
        p = make_params(patchSize=9 + 7 * k, mapWeight=0.7, tileH=k % 2, tileV=k % 2)
        s, pt, cnt = ref.frozen(p, ref_format(fm), target, corpus, hv, src, targets, start, cands)
        out.update({f"{k}_target": target, f"{k}_corpus": corpus, f"{k}_has": hv, f"{k}_source": src,
                    f"{k}_targets": targets, f"{k}_start": start, f"{k}_cands": cands,
                    f"{k}_format": np.array(fm), f"{k}_params": params_vec(p),
                    f"{k}_sum": s, f"{k}_pt": pt, f"{k}_count": cnt})
    out["count"] = np.array(len(fmts))
    np.savez_compressed(os.path.join(HERE, "frozen.npz"), **out)
    print("golden fixtures written to", HERE)


def ref_format(spec):
    """TFormatIndices from prepareImageFormatIndices arguments (lib/imageFormat.c:116-207)."""
    from oracle import Oracle
    return Oracle().format_indices(*spec)


if __name__ == "__main__":
    main()
