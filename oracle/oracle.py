"""ctypes wrappers for the CPU oracle and the reference built from its sources.

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke check in
__graft_entry__.py and by bench.py's CPU-baseline leg.  The product library
(resynthesizer_gb300) never imports this module.

* ``Oracle``   -- oracle/lib/liboracle.so, the plain-C restatement
  (oracle/resynth_oracle.c), built by ``make -C oracle``.
* ``Reference`` -- oracle/_ref/libref_{st,mt}.so, the reference engine compiled
  from its own sources by oracle/build_ref.sh (only where the reference tree
  exists, i.e. not on a machine that lacks it).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "lib", "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")
# Where the reference tree is read from (its sources are compiled in place by
# build_ref.sh): the environment variable RESYNTH_REFERENCE_ROOT, else the
# location build_ref.sh uses by default.  Where it does not exist (a machine
# without the reference), everything that needs it is skipped.
REFERENCE_ROOT = os.environ.get("RESYNTH_REFERENCE_ROOT", "/root/reference")


def reference_tree() -> str | None:
    """The reference tree's root if its engine sources are there, else None."""
    return REFERENCE_ROOT if os.path.exists(os.path.join(REFERENCE_ROOT, "lib", "engine.c")) else None


class Params(C.Structure):
    """Mirror of TImageSynthParameters (lib/engineParams.h:31-86)."""
    _fields_ = [("tileH", C.c_int), ("tileV", C.c_int), ("matchContextType", C.c_int),
                ("mapWeight", C.c_double), ("sensitivityToOutliers", C.c_double),
                ("patchSize", C.c_uint), ("maxProbeCount", C.c_uint)]


class Format(C.Structure):
    """Mirror of TFormatIndices (lib/imageFormatIndicies.h:46-58)."""
    _fields_ = [("colorEndBip", C.c_ubyte), ("alpha_bip", C.c_ubyte), ("map_start_bip", C.c_ubyte),
                ("map_end_bip", C.c_ubyte), ("img_match_bpp", C.c_ubyte), ("map_match_bpp", C.c_ubyte),
                ("total_bpp", C.c_ubyte), ("isAlphaTarget", C.c_int), ("isAlphaSource", C.c_int)]


class ImageBuffer(C.Structure):
    _fields_ = [("data", C.POINTER(C.c_ubyte)), ("width", C.c_uint), ("height", C.c_uint),
                ("rowBytes", C.c_size_t)]


class Stats(C.Structure):
    _fields_ = [("visits", C.c_ulonglong), ("evals", C.c_ulonglong), ("terms", C.c_ulonglong),
                ("draws", C.c_ulonglong), ("passes", C.c_uint), ("pass_len", C.c_uint * 6),
                ("betters", C.c_uint * 6)]


PROGRESS = C.CFUNCTYPE(None, C.c_int, C.c_void_p)


class WaveOpts(C.Structure):
    """orc_wave_opts: the wavefront schedule options (0 = default)."""
    _fields_ = [("firstBatch", C.c_uint), ("bandGrowth", C.c_uint), ("phaseSide", C.c_uint),
                ("minPasses", C.c_uint), ("probeShare", C.c_uint)]


def make_params(tileH=0, tileV=0, matchContextType=1, mapWeight=0.5, sensitivity=0.117,
                patchSize=30, maxProbeCount=200) -> Params:
    return Params(tileH, tileV, matchContextType, mapWeight, sensitivity, patchSize, maxProbeCount)


def _u8p(a: np.ndarray):
    assert a.dtype == np.uint8 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_ubyte))


def _vp(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def build_oracle() -> str:
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return ORACLE_SO


class Oracle:
    """The plain-C restatement of the reference engine."""

    def __init__(self, path: str = ORACLE_SO):
        if not os.path.exists(path):
            build_oracle()
        self.lib = L = C.CDLL(path)
        vp, u = C.c_void_p, C.c_uint
        L.orc_engine.argtypes = [C.POINTER(Params), C.POINTER(Format), vp, u, u, vp, u, u, C.c_int,
                                 vp, vp, C.POINTER(C.c_int), C.POINTER(Stats), vp, vp]
        L.orc_engine.restype = C.c_int
        L.orc_image_synth.argtypes = [C.POINTER(ImageBuffer), C.POINTER(ImageBuffer), vp, C.c_int,
                                      C.POINTER(Params), C.c_int, vp, vp, C.POINTER(C.c_int),
                                      C.POINTER(Stats)]
        L.orc_image_synth.restype = C.c_int
        L.orc_frozen.argtypes = [C.POINTER(Params), C.POINTER(Format), vp, u, u, vp, u, u, vp, vp,
                                 vp, u, vp, vp, vp, vp, vp]
        L.orc_frozen.restype = None
        L.orc_energy.argtypes = [C.POINTER(Params), C.POINTER(Format), vp, u, u, vp, u, u, vp, vp,
                                 vp, u, vp]
        L.orc_energy.restype = C.c_ulonglong
        L.orc_metric_tables.argtypes = [C.c_double, C.c_double, vp, vp]
        L.orc_sorted_offsets.argtypes = [u, u, u, u, vp]
        L.orc_sorted_offsets.restype = C.c_size_t
        L.orc_order_targets.argtypes = [C.c_int, vp, u]
        L.orc_order_targets.restype = C.c_int
        L.orc_format_indices.argtypes = [C.POINTER(Format), u, u, C.c_int, C.c_int, C.c_int]
        L.orc_format_from_type.argtypes = [C.POINTER(Format), C.c_int]
        L.orc_format_from_type.restype = C.c_int
        L.orc_rand_stream.argtypes = [u, u, vp]
        L.orc_wave_engine.argtypes = [C.POINTER(Params), C.POINTER(Format), vp, u, u, vp, u, u, u, C.c_int,
                                      C.POINTER(C.c_uint), vp]
        L.orc_wave_engine.restype = C.c_int
        L.orc_wave_engine_ex.argtypes = [C.POINTER(Params), C.POINTER(Format), vp, u, u, vp, u, u, u, C.c_int,
                                         C.POINTER(WaveOpts), C.POINTER(C.c_uint), vp, vp, vp, C.POINTER(C.c_uint)]
        L.orc_wave_engine_ex.restype = C.c_int
        L.orc_wave_image_synth.argtypes = [C.POINTER(ImageBuffer), C.POINTER(ImageBuffer), C.POINTER(ImageBuffer),
                                           C.c_int, C.POINTER(Params), u, C.c_int]
        L.orc_wave_image_synth.restype = C.c_int

    # -- helpers --------------------------------------------------------
    def format_indices(self, colors, mapColors, alphaT, alphaS, isMap) -> Format:
        f = Format()
        self.lib.orc_format_indices(C.byref(f), colors, mapColors, alphaT, alphaS, isMap)
        return f

    def format_from_type(self, t) -> Format:
        f = Format()
        rc = self.lib.orc_format_from_type(C.byref(f), t)
        if rc:
            raise ValueError(f"invalid image format {t}")
        return f

    def metric_tables(self, sensitivity=0.117, mapWeight=0.5):
        ct = np.zeros(512, np.uint16)
        mt = np.zeros(512, np.uint32)
        self.lib.orc_metric_tables(sensitivity, mapWeight, _vp(ct), _vp(mt))
        return ct, mt

    def sorted_offsets(self, tw, th, cw, ch) -> np.ndarray:
        n = (2 * min(tw, cw) - 1) * (2 * min(th, ch) - 1)
        out = np.zeros((n, 2), np.int32)
        self.lib.orc_sorted_offsets(tw, th, cw, ch, _vp(out))
        return out

    def order_targets(self, ctype, points: np.ndarray) -> np.ndarray:
        pts = np.ascontiguousarray(points, np.int32).copy()
        rc = self.lib.orc_order_targets(ctype, _vp(pts), len(pts))
        if rc:
            raise ValueError(f"matchContextType out of range: {ctype}")
        return pts

    def rand_stream(self, n, seed=1198472) -> np.ndarray:
        out = np.zeros(n, np.int32)
        self.lib.orc_rand_stream(seed, n, _vp(out))
        return out

    # -- engines --------------------------------------------------------
    def engine(self, params: Params, fmt: Format, target: np.ndarray, corpus: np.ndarray,
               threads: int = 1, cancel: int = 0, progress=None, want_state=False):
        """Runs the engine on interleaved pixmaps (H, W, total_bpp).  Returns
        (rc, target_out, stats[, sourceOf, hasValue])."""
        th, tw, _ = target.shape
        ch, cw, _ = corpus.shape
        tgt = np.ascontiguousarray(target, np.uint8).copy()
        cor = np.ascontiguousarray(corpus, np.uint8)
        st = Stats()
        cf = C.c_int(cancel)
        src = np.zeros((th, tw, 2), np.int32) if want_state else None
        hv = np.zeros((th, tw), np.uint8) if want_state else None
        cb = PROGRESS(progress) if progress else None
        rc = self.lib.orc_engine(C.byref(params), C.byref(fmt), _vp(tgt), tw, th, _vp(cor), cw, ch,
                                 threads, C.cast(cb, C.c_void_p) if cb else None, None, C.byref(cf),
                                 C.byref(st), _vp(src), _vp(hv))
        if want_state:
            return rc, tgt, st, src, hv
        return rc, tgt, st

    def wave_engine(self, params: Params, fmt: Format, target: np.ndarray, corpus: np.ndarray,
                    threads: int = 8, seed: int = 0):
        """The GPU library's wavefront mode restated on the CPU (every visit
        order, default options): (rc, target_out, passes, betters per pass)."""
        th, tw, _ = target.shape
        ch, cw, _ = corpus.shape
        tgt = np.ascontiguousarray(target, np.uint8).copy()
        cor = np.ascontiguousarray(corpus, np.uint8)
        passes = C.c_uint(0)
        betters = np.zeros(6, np.uint32)
        rc = self.lib.orc_wave_engine(C.byref(params), C.byref(fmt), _vp(tgt), tw, th, _vp(cor), cw, ch, seed,
                                      threads, C.byref(passes), _vp(betters))
        return rc, tgt, passes.value, betters[: passes.value].tolist()

    def wave_engine_state(self, params: Params, fmt: Format, target: np.ndarray, corpus: np.ndarray,
                          threads: int = 8, seed: int = 0, **schedule):
        """wave_engine with schedule options (firstBatch, bandGrowth, phaseSide,
        minPasses) and the final state: (rc, target_out, passes, betters,
        sourceOf (H, W, 2), hasValue (H, W), batches)."""
        th, tw, _ = target.shape
        ch, cw, _ = corpus.shape
        tgt = np.ascontiguousarray(target, np.uint8).copy()
        cor = np.ascontiguousarray(corpus, np.uint8)
        passes, batches = C.c_uint(0), C.c_uint(0)
        betters = np.zeros(6, np.uint32)
        src = np.zeros((th, tw, 2), np.int32)
        hv = np.zeros((th, tw), np.uint8)
        opts = WaveOpts(**schedule)
        rc = self.lib.orc_wave_engine_ex(C.byref(params), C.byref(fmt), _vp(tgt), tw, th, _vp(cor), cw, ch, seed,
                                         threads, C.byref(opts), C.byref(passes), _vp(betters), _vp(src), _vp(hv),
                                         C.byref(batches))
        return rc, tgt, passes.value, betters[: passes.value].tolist(), src, hv, batches.value

    def image_synth(self, image: np.ndarray, mask: np.ndarray, fmt: int, params: Params | None,
                    mask2: np.ndarray | None = None, threads=1, cancel=0, progress=None):
        """Simple API on (H, W, bpp) image and (H, W) mask (unpadded)."""
        img = np.ascontiguousarray(image, np.uint8).copy()
        h, w = img.shape[:2]
        bpp = img.shape[2] if img.ndim == 3 else 1
        ib = ImageBuffer(_u8p(img), w, h, w * bpp)
        m = np.ascontiguousarray(mask, np.uint8)
        mb = ImageBuffer(_u8p(m), m.shape[1], m.shape[0], m.shape[1])
        m2 = None
        if mask2 is not None:
            m2a = np.ascontiguousarray(mask2, np.uint8)
            m2 = ImageBuffer(_u8p(m2a), m2a.shape[1], m2a.shape[0], m2a.shape[1])
        st = Stats()
        cf = C.c_int(cancel)
        cb = PROGRESS(progress) if progress else None
        rc = self.lib.orc_image_synth(C.byref(ib), C.byref(mb), C.byref(m2) if m2 else None, fmt,
                                      C.byref(params) if params is not None else None, threads,
                                      C.cast(cb, C.c_void_p) if cb else None, None, C.byref(cf),
                                      C.byref(st))
        return rc, img, st

    def wave_image_synth(self, image: np.ndarray, mask: np.ndarray, fmt: int, params: Params | None,
                         mask2: np.ndarray | None = None, threads: int = 8, seed: int = 0):
        """The Simple API around the wavefront restatement (what the GPU
        library's imageSynth gives in wavefront mode): (rc, image_out)."""
        img = np.ascontiguousarray(image, np.uint8).copy()
        h, w = img.shape[:2]
        bpp = img.shape[2] if img.ndim == 3 else 1
        ib = ImageBuffer(_u8p(img), w, h, w * bpp)
        m = np.ascontiguousarray(mask, np.uint8)
        mb = ImageBuffer(_u8p(m), m.shape[1], m.shape[0], m.shape[1])
        m2 = None
        if mask2 is not None:
            m2a = np.ascontiguousarray(mask2, np.uint8)
            m2 = ImageBuffer(_u8p(m2a), m2a.shape[1], m2a.shape[0], m2a.shape[1])
        rc = self.lib.orc_wave_image_synth(C.byref(ib), C.byref(mb), C.byref(m2) if m2 else None, fmt,
                                           C.byref(params) if params is not None else None, seed, threads)
        return rc, img

    def frozen(self, params, fmt, target, corpus, hasValue, sourceOf, targets, candStart, cands):
        th, tw, _ = target.shape
        ch, cw, _ = corpus.shape
        n = len(targets)
        out_sum = np.zeros(n, np.uint32)
        out_pt = np.zeros((n, 2), np.int32)
        out_cnt = np.zeros(n, np.uint32)
        args = [np.ascontiguousarray(a) for a in (target, corpus, hasValue, sourceOf, targets,
                                                   candStart, cands)]
        self.lib.orc_frozen(C.byref(params), C.byref(fmt), _vp(args[0]), tw, th, _vp(args[1]), cw, ch,
                            _vp(args[2]), _vp(args[3]), _vp(args[4]), n, _vp(args[5]), _vp(args[6]),
                            _vp(out_sum), _vp(out_pt), _vp(out_cnt))
        return out_sum, out_pt, out_cnt

    def energy(self, params, fmt, target, corpus, hasValue, sourceOf, targets):
        th, tw, _ = target.shape
        ch, cw, _ = corpus.shape
        per = np.zeros(len(targets), np.uint32)
        a = [np.ascontiguousarray(x) for x in (target, corpus, hasValue, sourceOf, targets)]
        tot = self.lib.orc_energy(C.byref(params), C.byref(fmt), _vp(a[0]), tw, th, _vp(a[1]), cw, ch,
                                  _vp(a[2]), _vp(a[3]), _vp(a[4]), len(targets), _vp(per))
        return int(tot), per


def reference_available(threaded: bool = False) -> bool:
    return os.path.exists(os.path.join(REF_DIR, "libref_mt.so" if threaded else "libref_st.so"))


class Reference:
    """The reference engine compiled from its own sources (oracle/build_ref.sh)."""

    def __init__(self, threaded: bool = False):
        path = os.path.join(REF_DIR, "libref_mt.so" if threaded else "libref_st.so")
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = L = C.CDLL(path)
        vp, u = C.c_void_p, C.c_uint
        L.imageSynth.argtypes = [C.POINTER(ImageBuffer), C.POINTER(ImageBuffer), C.c_int,
                                 C.POINTER(Params), vp, vp, C.POINTER(C.c_int)]
        L.imageSynth.restype = C.c_int
        L.imageSynth2.argtypes = [C.POINTER(ImageBuffer), C.POINTER(ImageBuffer), C.POINTER(ImageBuffer),
                                  C.c_int, C.POINTER(Params), vp, vp, C.POINTER(C.c_int)]
        L.imageSynth2.restype = C.c_int
        L.ref_engine_state.argtypes = [C.POINTER(Params), C.POINTER(Format), vp, u, u, vp, u, u, vp, vp]
        L.ref_engine_state.restype = C.c_int
        L.ref_order_targets.argtypes = [C.POINTER(Params), C.POINTER(Format), vp, u, u, vp, C.POINTER(C.c_uint)]
        L.ref_order_targets.restype = C.c_int
        L.ref_sorted_offsets.argtypes = [u, u, u, u, vp]
        L.ref_sorted_offsets.restype = C.c_uint
        L.ref_metric_tables.argtypes = [C.c_double, C.c_double, vp, vp]
        L.ref_frozen.argtypes = [C.POINTER(Params), C.POINTER(Format), vp, u, u, vp, u, u, vp, vp, vp, u,
                                 vp, vp, vp, vp, vp, C.c_int]
        self._noop = PROGRESS(lambda p, c: None)

    def image_synth(self, image, mask, fmt, params, mask2=None, cancel=0, progress=None):
        img = np.ascontiguousarray(image, np.uint8).copy()
        h, w = img.shape[:2]
        bpp = img.shape[2] if img.ndim == 3 else 1
        ib = ImageBuffer(_u8p(img), w, h, w * bpp)
        m = np.ascontiguousarray(mask, np.uint8)
        mb = ImageBuffer(_u8p(m), m.shape[1], m.shape[0], m.shape[1])
        cf = C.c_int(cancel)
        cb = PROGRESS(progress) if progress else self._noop
        pp = C.byref(params) if params is not None else None
        if mask2 is None:
            rc = self.lib.imageSynth(C.byref(ib), C.byref(mb), fmt, pp, C.cast(cb, C.c_void_p), None,
                                     C.byref(cf))
        else:
            m2a = np.ascontiguousarray(mask2, np.uint8)
            m2 = ImageBuffer(_u8p(m2a), m2a.shape[1], m2a.shape[0], m2a.shape[1])
            rc = self.lib.imageSynth2(C.byref(ib), C.byref(mb), C.byref(m2), fmt, pp,
                                      C.cast(cb, C.c_void_p), None, C.byref(cf))
        return rc, img

    def engine_state(self, params, fmt, target, corpus):
        th, tw, _ = target.shape
        ch, cw, _ = corpus.shape
        tgt = np.ascontiguousarray(target, np.uint8).copy()
        cor = np.ascontiguousarray(corpus, np.uint8)
        src = np.zeros((th, tw, 2), np.int32)
        hv = np.zeros((th, tw), np.uint8)
        rc = self.lib.ref_engine_state(C.byref(params), C.byref(fmt), _vp(tgt), tw, th, _vp(cor), cw, ch,
                                       _vp(src), _vp(hv))
        return rc, tgt, src, hv

    def order_targets(self, params, fmt, target):
        th, tw, _ = target.shape
        out = np.zeros((th * tw, 2), np.int32)
        cnt = C.c_uint(0)
        tgt = np.ascontiguousarray(target, np.uint8)
        rc = self.lib.ref_order_targets(C.byref(params), C.byref(fmt), _vp(tgt), tw, th, _vp(out),
                                        C.byref(cnt))
        return rc, out[:cnt.value]

    def sorted_offsets(self, tw, th, cw, ch):
        n = (2 * min(tw, cw) - 1) * (2 * min(th, ch) - 1)
        out = np.zeros((n, 2), np.int32)
        self.lib.ref_sorted_offsets(tw, th, cw, ch, _vp(out))
        return out

    def metric_tables(self, sensitivity=0.117, mapWeight=0.5):
        ct = np.zeros(512, np.uint16)
        mt = np.zeros(512, np.uint32)
        self.lib.ref_metric_tables(sensitivity, mapWeight, _vp(ct), _vp(mt))
        return ct, mt

    def frozen(self, params, fmt, target, corpus, hasValue, sourceOf, targets, candStart, cands,
               full_sum=False):
        th, tw, _ = target.shape
        ch, cw, _ = corpus.shape
        n = len(targets)
        out_sum = np.zeros(n, np.uint32)
        out_pt = np.zeros((n, 2), np.int32)
        out_cnt = np.zeros(n, np.uint32)
        a = [np.ascontiguousarray(x) for x in (target, corpus, hasValue, sourceOf, targets, candStart, cands)]
        self.lib.ref_frozen(C.byref(params), C.byref(fmt), _vp(a[0]), tw, th, _vp(a[1]), cw, ch, _vp(a[2]),
                            _vp(a[3]), _vp(a[4]), n, _vp(a[5]), _vp(a[6]), _vp(out_sum), _vp(out_pt),
                            _vp(out_cnt), int(full_sum))
        return out_sum, out_pt, out_cnt
