"""resynthesizer_gb300 -- GB300 texture-synthesis engine (Python side of libresynthesizer.so).

The engine itself is the C ABI library built from resynthesizer_gb300/csrc
(see include/resynthesizer.h); this module loads it with ctypes and mirrors
the reference's API for Python callers and tests:

    image_synth(image, mask, fmt, params)       -- imageSynth / imageSynth2
    engine(target, corpus, fmt_spec, params)    -- engine() on interleaved pixmaps
    frozen_best_fit(...), patch_energy(...)     -- state-level extensions

There is no CPU fallback: if the library is missing, importing succeeds but
every call raises; if no GPU is usable, calls return RESYNTH_ERROR_DEVICE.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "lib", "libresynthesizer.so")

T_RGB, T_RGBA, T_Gray, T_GrayA = 0, 1, 2, 3
MODE_WAVEFRONT, MODE_REPLAY = 0, 1
ERRORS = {0: "SUCCESS", 1: "INVALID_IMAGE_FORMAT", 2: "IMAGE_MASK_MISMATCH", 3: "PATCH_SIZE_EXCEEDED",
          4: "MATCH_CONTEXT_TYPE_RANGE", 5: "EMPTY_TARGET", 6: "EMPTY_CORPUS", 100: "DEVICE", 101: "UNSUPPORTED",
          102: "ARGUMENT"}


class ImageSynthParameters(C.Structure):
    """TImageSynthParameters (lib/engineParams.h:31-86)."""
    _fields_ = [("isMakeSeamlesslyTileableHorizontally", C.c_int), ("isMakeSeamlesslyTileableVertically", C.c_int),
                ("matchContextType", C.c_int), ("mapWeight", C.c_double), ("sensitivityToOutliers", C.c_double),
                ("patchSize", C.c_uint), ("maxProbeCount", C.c_uint)]


class FormatIndices(C.Structure):
    """TFormatIndices (lib/imageFormatIndicies.h:46-58)."""
    _fields_ = [("colorEndBip", C.c_ubyte), ("alpha_bip", C.c_ubyte), ("map_start_bip", C.c_ubyte),
                ("map_end_bip", C.c_ubyte), ("img_match_bpp", C.c_ubyte), ("map_match_bpp", C.c_ubyte),
                ("total_bpp", C.c_ubyte), ("isAlphaTarget", C.c_int), ("isAlphaSource", C.c_int)]


class ImageBuffer(C.Structure):
    _fields_ = [("data", C.POINTER(C.c_ubyte)), ("width", C.c_uint), ("height", C.c_uint), ("rowBytes", C.c_size_t)]


class GArray(C.Structure):
    _fields_ = [("data", C.c_void_p), ("len", C.c_uint)]


class Map(C.Structure):
    _fields_ = [("width", C.c_uint), ("height", C.c_uint), ("depth", C.c_uint), ("data", C.POINTER(GArray))]


class Options(C.Structure):
    _fields_ = [("mode", C.c_int), ("seed", C.c_uint), ("firstBatch", C.c_uint), ("refineBatches", C.c_uint),
                ("warpsPerBlock", C.c_uint), ("recordState", C.c_int), ("profile", C.c_int),
                ("phaseSide", C.c_uint), ("bandGrowth", C.c_uint), ("minPasses", C.c_uint),
                ("net", C.c_void_p), ("proposals", C.c_uint), ("dumpPairs", C.c_void_p), ("dumpStride", C.c_uint),
                ("graphs", C.c_int), ("separateRequests", C.c_int), ("bandGrowthLarge", C.c_uint),
                ("batchLaunches", C.c_int), ("proposalPasses", C.c_uint), ("probeShare", C.c_int)]


class TrainOptions(C.Structure):
    _fields_ = [("steps", C.c_uint), ("batch", C.c_uint), ("learningRate", C.c_float), ("seed", C.c_uint)]


class Request(C.Structure):
    _fields_ = [("image", C.POINTER(ImageBuffer)), ("mask", C.POINTER(ImageBuffer)), ("mask2", C.POINTER(ImageBuffer)),
                ("format", C.c_int), ("parameters", C.POINTER(ImageSynthParameters)), ("result", C.c_int)]


class Stats(C.Structure):
    _fields_ = [("visits", C.c_ulonglong), ("evals", C.c_ulonglong), ("terms", C.c_ulonglong),
                ("passes", C.c_uint), ("passLength", C.c_uint * 6), ("betters", C.c_uint * 6),
                ("launches", C.c_uint), ("deviceMs", C.c_double), ("totalMs", C.c_double),
                ("h2dBytes", C.c_ulonglong), ("d2hBytes", C.c_ulonglong), ("waveMs", C.c_double),
                ("waveLaunches", C.c_uint), ("waveTerms", C.c_ulonglong), ("launchMode", C.c_int)]

    def as_dict(self) -> dict:
        return dict(visits=self.visits, evals=self.evals, terms=self.terms, passes=self.passes,
                    passLength=list(self.passLength)[: self.passes], betters=list(self.betters)[: self.passes],
                    launches=self.launches, deviceMs=self.deviceMs, totalMs=self.totalMs,
                    h2dBytes=self.h2dBytes, d2hBytes=self.d2hBytes, waveMs=self.waveMs,
                    waveLaunches=self.waveLaunches, waveTerms=self.waveTerms, launchMode=self.launchMode)


PROGRESS = C.CFUNCTYPE(None, C.c_int, C.c_void_p)

_lib = None


class LibraryMissing(RuntimeError):
    pass


def lib() -> C.CDLL:
    """The loaded libresynthesizer.so; raises if it was not built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise LibraryMissing(f"{LIB_PATH} not built: run `python -m resynthesizer_gb300.build`")
        L = C.CDLL(LIB_PATH)
        vp, u, P = C.c_void_p, C.c_uint, C.POINTER
        L.imageSynth.argtypes = [P(ImageBuffer), P(ImageBuffer), C.c_int, P(ImageSynthParameters), vp, vp, P(C.c_int)]
        L.imageSynth2.argtypes = [P(ImageBuffer), P(ImageBuffer), P(ImageBuffer), C.c_int, P(ImageSynthParameters),
                                  vp, vp, P(C.c_int)]
        L.imageSynthEx.argtypes = [P(ImageBuffer), P(ImageBuffer), P(ImageBuffer), C.c_int, P(ImageSynthParameters),
                                   vp, vp, P(C.c_int), P(Options), P(Stats)]
        L.engine.argtypes = [ImageSynthParameters, P(FormatIndices), P(Map), P(Map), vp, vp, P(C.c_int)]
        L.engineEx.argtypes = [P(ImageSynthParameters), P(FormatIndices), P(Map), P(Map), vp, vp, P(C.c_int),
                               P(Options), P(Stats)]
        L.imageSynthBatch.argtypes = [C.POINTER(Request), u, u, P(Options), P(Stats)]
        L.engineDevice.argtypes = [P(ImageSynthParameters), P(FormatIndices), vp, u, u, vp, u, u, vp, vp, vp,
                                   P(C.c_int), P(Options), P(Stats)]
        L.resynthFrozenBestFit.argtypes = [P(ImageSynthParameters), P(FormatIndices), vp, u, u, vp, u, u, vp, vp, vp,
                                           u, vp, vp, vp, vp, vp]
        L.resynthPatchEnergy.argtypes = [P(ImageSynthParameters), P(FormatIndices), vp, u, u, vp, u, u, vp, vp, vp, u,
                                         P(C.c_ulonglong), vp]
        L.resynthGetState.argtypes = [vp, vp, u, u]
        L.resynthLastError.restype = C.c_char_p
        L.resynthSetMode.argtypes = [C.c_int]
        L.resynthDefaultOptions.argtypes = [P(Options)]
        L.prepareImageFormatIndices.argtypes = [P(FormatIndices), u, u, C.c_int, C.c_int, C.c_int]
        L.prepareImageFormatIndicesFromFormatType.argtypes = [P(FormatIndices), C.c_int]
        L.countPixelelsPerPixelForFormat.argtypes = [C.c_int]
        L.countPixelelsPerPixelForFormat.restype = C.c_uint
        L.setDefaultParams.argtypes = [P(ImageSynthParameters)]
        for name in ("new_pixmap",):
            getattr(L, name).argtypes = [P(Map), u, u, u]
        for name in ("new_bytemap", "new_intmap", "new_coordmap"):
            getattr(L, name).argtypes = [P(Map), u, u]
        L.free_map.argtypes = [P(Map)]
        L.set_bytemap.argtypes = [P(Map), C.c_ubyte]
        L.invert_bytemap.argtypes = [P(Map)]
        L.interleave_mask.argtypes = [P(Map), P(Map)]
        L.resynthTcGemm.argtypes = [vp, vp, C.c_int, C.c_int, C.c_int, vp]
        L.resynthTcWaitTimeout.argtypes = []
        L.resynthPatchNeighbours.argtypes = [vp, u, u, u, vp, u, C.c_int, vp, vp]
        L.resynthNetParamCount.restype = u
        L.resynthNetCreate.argtypes = [u]
        L.resynthNetCreate.restype = vp
        L.resynthNetDestroy.argtypes = [vp]
        L.resynthNetGetParams.argtypes = [vp, vp]
        L.resynthNetSetParams.argtypes = [vp, vp]
        L.resynthNetForward.argtypes = [vp, vp, u, vp, C.c_int]
        L.resynthNetGradients.argtypes = [vp, vp, vp, u, vp, P(C.c_float)]
        L.resynthNetTrain.argtypes = [vp, vp, P(TrainOptions), P(C.c_float)]
        L.resynthPairsCreate.argtypes = [u]
        L.resynthPairsCreate.restype = vp
        L.resynthPairsDestroy.argtypes = [vp]
        L.resynthPairsCount.argtypes = [vp]
        L.resynthPairsCount.restype = u
        L.resynthPairsAdd.argtypes = [vp, vp, vp, u]
        L.resynthPairsAdd.restype = u
        L.resynthPairsRead.argtypes = [vp, u, u, vp, vp]
        _lib = L
    return _lib


def last_error() -> str:
    return lib().resynthLastError().decode()


def params(tileH=0, tileV=0, matchContextType=1, mapWeight=0.5, sensitivity=0.117, patchSize=30,
           maxProbeCount=200) -> ImageSynthParameters:
    return ImageSynthParameters(tileH, tileV, matchContextType, mapWeight, sensitivity, patchSize, maxProbeCount)


def default_params() -> ImageSynthParameters:
    p = ImageSynthParameters()
    lib().setDefaultParams(C.byref(p))
    return p


def format_indices(colors, mapColors=0, alphaTarget=0, alphaSource=0, isMap=0) -> FormatIndices:
    f = FormatIndices()
    lib().prepareImageFormatIndices(C.byref(f), colors, mapColors, alphaTarget, alphaSource, isMap)
    return f


def options(mode=None, seed=0, firstBatch=0, refineBatches=0, warpsPerBlock=0, recordState=0,
            profile=0, phaseSide=0, bandGrowth=0, minPasses=0, net=None, proposals=0, dump=None,
            dumpStride=0, graphs=0, separateRequests=0, bandGrowthLarge=0, batchLaunches=0,
            proposalPasses=0, probeShare=0) -> Options:
    o = Options()
    lib().resynthDefaultOptions(C.byref(o))
    if mode is not None:
        o.mode = mode
    o.seed, o.firstBatch, o.refineBatches, o.warpsPerBlock, o.recordState, o.profile = (
        seed, firstBatch, refineBatches, warpsPerBlock, recordState, profile)
    o.phaseSide, o.bandGrowth, o.minPasses = phaseSide, bandGrowth, minPasses
    o.net = net.handle if net is not None else None
    o.proposals = proposals if net is not None else 0
    o.dumpPairs = dump.handle if dump is not None else None
    o.dumpStride = dumpStride
    o.graphs = graphs
    o.separateRequests = separateRequests
    o.batchLaunches = batchLaunches
    o.proposalPasses = proposalPasses
    o.probeShare = probeShare
    o.bandGrowthLarge = bandGrowthLarge
    return o


def _vp(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _buf(a: np.ndarray) -> ImageBuffer:
    h, w = a.shape[:2]
    bpp = a.shape[2] if a.ndim == 3 else 1
    return ImageBuffer(a.ctypes.data_as(C.POINTER(C.c_ubyte)), w, h, w * bpp)


@dataclass
class Result:
    rc: int
    out: np.ndarray
    stats: dict
    source: np.ndarray | None = None
    has_value: np.ndarray | None = None


def _padded(a: np.ndarray, pad: int):
    """(row-padded copy, ImageBuffer over it): each row of `a` followed by
    `pad` bytes of 0xA5, as a caller's buffer with rowBytes > width * bpp."""
    h, w = a.shape[:2]
    bpp = a.shape[2] if a.ndim == 3 else 1
    buf = np.full((h, w * bpp + pad), 0xA5, np.uint8)
    buf[:, :w * bpp] = a.reshape(h, w * bpp)
    return buf, ImageBuffer(buf.ctypes.data_as(C.POINTER(C.c_ubyte)), w, h, w * bpp + pad)


def image_synth(image, mask, fmt, p: ImageSynthParameters | None = None, mask2=None, opts: Options | None = None,
                cancel=0, progress=None, raw_entry=False, row_pad: int = 0) -> Result:
    """Simple API on an (H, W, bpp) image and (H, W) mask.  raw_entry=True
    calls the reference-named imageSynth/imageSynth2 entry point itself.
    row_pad > 0 hands the library row-padded buffers (rowBytes = width * bpp
    + row_pad); the result is then checked to leave the padding untouched."""
    img = np.ascontiguousarray(image, np.uint8).copy()
    m = np.ascontiguousarray(mask, np.uint8)
    ib, mb = _buf(img), _buf(m)
    padded = None
    if row_pad:
        pimg, ib = _padded(img, row_pad)
        pm, mb = _padded(m, row_pad)
        padded = (pimg, pm)
    m2 = None
    if mask2 is not None:
        m2a = np.ascontiguousarray(mask2, np.uint8)
        m2 = _buf(m2a)
        if row_pad:
            pm2, m2 = _padded(m2a, row_pad)
            padded = padded + (pm2,)
    cf = C.c_int(cancel)
    cb = PROGRESS(progress) if progress else None
    cbp = C.cast(cb, C.c_void_p) if cb else None
    pp = C.byref(p) if p is not None else None
    st = Stats()
    if raw_entry:
        if m2 is None:
            rc = lib().imageSynth(C.byref(ib), C.byref(mb), fmt, pp, cbp, None, C.byref(cf))
        else:
            rc = lib().imageSynth2(C.byref(ib), C.byref(mb), C.byref(m2), fmt, pp, cbp, None, C.byref(cf))
    else:
        rc = lib().imageSynthEx(C.byref(ib), C.byref(mb), C.byref(m2) if m2 else None, fmt, pp, cbp, None,
                                C.byref(cf), C.byref(opts) if opts else None, C.byref(st))
    if padded is not None:
        h, w = m.shape
        rowb = img.size // h
        if not (padded[0][:, rowb:] == 0xA5).all():
            raise RuntimeError("the library wrote into the row padding of the image buffer")
        img = np.ascontiguousarray(padded[0][:, :rowb]).reshape(img.shape)
    r = Result(rc, img, st.as_dict())
    if opts is not None and opts.recordState and rc == 0:
        h, w = m.shape
        r.source, r.has_value = get_state(w, h)
    return r


class PixmapMap:
    """A reference Map (lib/map.h:28-33) owning a copy of an (H, W, depth) pixmap."""

    def __init__(self, pix: np.ndarray):
        h, w, d = pix.shape
        self.map = Map()
        lib().new_pixmap(C.byref(self.map), w, h, d)
        C.memmove(self.map.data.contents.data, np.ascontiguousarray(pix, np.uint8).ctypes.data, pix.nbytes)
        self.shape = pix.shape

    def array(self) -> np.ndarray:
        n = int(np.prod(self.shape))
        buf = (C.c_ubyte * n).from_address(self.map.data.contents.data)
        return np.frombuffer(buf, np.uint8, n).reshape(self.shape).copy()

    def __del__(self):
        try:
            lib().free_map(C.byref(self.map))
        except Exception:
            pass


def engine(target, corpus, fmt: FormatIndices, p: ImageSynthParameters, opts: Options | None = None, cancel=0,
           progress=None, raw_entry=False) -> Result:
    """engine() on interleaved pixmaps (H, W, total_bpp); returns the updated target."""
    tm, cm = PixmapMap(target), PixmapMap(corpus)
    cf = C.c_int(cancel)
    cb = PROGRESS(progress) if progress else None
    cbp = C.cast(cb, C.c_void_p) if cb else None
    st = Stats()
    if raw_entry:
        rc = lib().engine(p, C.byref(fmt), C.byref(tm.map), C.byref(cm.map), cbp, None, C.byref(cf))
    else:
        rc = lib().engineEx(C.byref(p), C.byref(fmt), C.byref(tm.map), C.byref(cm.map), cbp, None, C.byref(cf),
                            C.byref(opts) if opts else None, C.byref(st))
    r = Result(rc, tm.array(), st.as_dict())
    if opts is not None and opts.recordState and rc == 0:
        h, w = target.shape[:2]
        r.source, r.has_value = get_state(w, h)
    return r


def get_state(w, h):
    src = np.zeros((h, w, 2), np.int32)
    hv = np.zeros((h, w), np.uint8)
    rc = lib().resynthGetState(_vp(src), _vp(hv), w, h)
    if rc:
        raise RuntimeError(f"resynthGetState: {last_error()}")
    return src, hv


def engine_device(p, fmt, d_target: int, tw, th, d_corpus: int, cw, ch, stream: int = 0,
                  opts: Options | None = None) -> tuple[int, dict]:
    """engineDevice on device pointers (e.g. torch tensors' data_ptr())."""
    st = Stats()
    rc = lib().engineDevice(C.byref(p), C.byref(fmt), C.c_void_p(d_target), tw, th, C.c_void_p(d_corpus), cw, ch,
                            C.c_void_p(stream) if stream else None, None, None, None,
                            C.byref(opts) if opts else None, C.byref(st))
    return rc, st.as_dict()


def frozen_best_fit(p, fmt, target, corpus, has_value, source, targets, cand_start, cands):
    th, tw, _ = target.shape
    ch, cw, _ = corpus.shape
    n = len(targets)
    out_sum = np.zeros(n, np.uint32)
    out_pt = np.zeros((n, 2), np.int32)
    out_cnt = np.zeros(n, np.uint32)
    a = [np.ascontiguousarray(x) for x in (target, corpus, has_value, source, targets, cand_start, cands)]
    rc = lib().resynthFrozenBestFit(C.byref(p), C.byref(fmt), _vp(a[0]), tw, th, _vp(a[1]), cw, ch, _vp(a[2]),
                                    _vp(a[3]), _vp(a[4]), n, _vp(a[5]), _vp(a[6]), _vp(out_sum), _vp(out_pt),
                                    _vp(out_cnt))
    if rc:
        raise RuntimeError(f"resynthFrozenBestFit rc={rc}: {last_error()}")
    return out_sum, out_pt, out_cnt


def patch_energy(p, fmt, target, corpus, has_value, source, targets):
    th, tw, _ = target.shape
    ch, cw, _ = corpus.shape
    per = np.zeros(len(targets), np.uint32)
    e = C.c_ulonglong(0)
    a = [np.ascontiguousarray(x) for x in (target, corpus, has_value, source, targets)]
    rc = lib().resynthPatchEnergy(C.byref(p), C.byref(fmt), _vp(a[0]), tw, th, _vp(a[1]), cw, ch, _vp(a[2]),
                                  _vp(a[3]), _vp(a[4]), len(targets), C.byref(e), _vp(per))
    if rc:
        raise RuntimeError(f"resynthPatchEnergy rc={rc}: {last_error()}")
    return int(e.value), per


def image_synth_batch(items, opts: Options | None = None, concurrency: int = 8):
    """imageSynthBatch over [(image, mask, fmt, params or None), ...]; returns
    (rc, outputs, per-request codes, stats)."""
    keep, reqs = [], (Request * len(items))()
    for i, (image, mask, fmt, p) in enumerate(items):
        img = np.ascontiguousarray(image, np.uint8).copy()
        m = np.ascontiguousarray(mask, np.uint8)
        ib, mb = _buf(img), _buf(m)
        pp = C.pointer(p) if p is not None else None
        keep.append((img, m, ib, mb, pp))
        reqs[i].image = C.pointer(ib)
        reqs[i].mask = C.pointer(mb)
        reqs[i].mask2 = None
        reqs[i].format = fmt
        reqs[i].parameters = pp
    st = Stats()
    rc = lib().imageSynthBatch(reqs, len(items), concurrency, C.byref(opts) if opts else None, C.byref(st))
    return rc, [k[0] for k in keep], [reqs[i].result for i in range(len(items))], st.as_dict()


def order_targets_device(match_context_type: int, points: np.ndarray) -> np.ndarray:
    """resynthOrderTargets: the device-side visit order of a directional type."""
    L = lib()
    L.resynthOrderTargets.argtypes = [C.c_int, C.c_void_p, C.c_uint, C.c_void_p]
    pts = np.ascontiguousarray(points, np.int32)
    out = np.zeros_like(pts)
    rc = L.resynthOrderTargets(match_context_type, _vp(pts), len(pts), _vp(out))
    if rc:
        raise RuntimeError(f"resynthOrderTargets rc={rc}: {last_error()}")
    return out


def grid_barrier_probe(rounds: int, absent_cta: int = -1, timeout_ns: int = 1_000_000_000):
    """resynthGridBarrierProbe: (barriers passed summed over CTAs, error bits)."""
    L = lib()
    L.resynthGridBarrierProbe.argtypes = [C.c_int, C.c_int, C.c_longlong, C.POINTER(C.c_uint), C.POINTER(C.c_uint)]
    passed, err = C.c_uint(0), C.c_uint(0)
    rc = L.resynthGridBarrierProbe(rounds, absent_cta, timeout_ns, C.byref(passed), C.byref(err))
    if rc:
        raise RuntimeError(f"resynthGridBarrierProbe rc={rc}: {last_error()}")
    return passed.value, err.value


def microbench(which: int):
    """resynthMicrobench: (peak, ms): which 0 = shared-memory load GB/s, 1 = INT32 ALU G ops/s."""
    L = lib()
    L.resynthMicrobench.argtypes = [C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    v, ms = C.c_double(0), C.c_double(0)
    rc = L.resynthMicrobench(which, C.byref(v), C.byref(ms))
    if rc:
        raise RuntimeError(f"resynthMicrobench rc={rc}: {last_error()}")
    return v.value, ms.value


def sm_count() -> int:
    import torch
    return torch.cuda.get_device_properties(0).multi_processor_count


def tc_gemm(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """D = bf16(a) . bf16(b)^T on the tensor cores (fp32 accumulation)."""
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    m, k = a.shape
    n = b.shape[0]
    d = np.zeros((m, n), np.float32)
    rc = lib().resynthTcGemm(_vp(a), _vp(b), m, n, k, _vp(d))
    if rc:
        raise RuntimeError(f"resynthTcGemm rc={rc}: {last_error()}")
    return d


# ------------------------------------------------------- learned proposals

CTX_SHAPE = (11, 11, 16)


class Net:
    """The proposal network (resynthNetCreate ... resynthNetDestroy)."""

    def __init__(self, seed: int = 1):
        self.handle = lib().resynthNetCreate(seed)
        if not self.handle:
            raise RuntimeError(f"resynthNetCreate: {last_error()}")

    def close(self):
        if self.handle:
            lib().resynthNetDestroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def param_count() -> int:
        return int(lib().resynthNetParamCount())

    def get_params(self) -> np.ndarray:
        p = np.zeros(self.param_count(), np.float32)
        _check(lib().resynthNetGetParams(self.handle, _vp(p)), "resynthNetGetParams")
        return p

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.param_count()
        _check(lib().resynthNetSetParams(self.handle, _vp(p)), "resynthNetSetParams")

    def forward(self, contexts: np.ndarray, path: int = 0) -> np.ndarray:
        """contexts: uint16 bf16 bits [n, 11, 11, 16] -> outputs [n, 32]."""
        x = np.ascontiguousarray(contexts, np.uint16)
        n = x.shape[0]
        out = np.zeros((n, 32), np.float32)
        _check(lib().resynthNetForward(self.handle, _vp(x), n, _vp(out), path), "resynthNetForward")
        return out

    def gradients(self, contexts: np.ndarray, labels: np.ndarray):
        x = np.ascontiguousarray(contexts, np.uint16)
        y = np.ascontiguousarray(labels, np.float32)
        g = np.zeros(self.param_count(), np.float32)
        loss = C.c_float(0)
        _check(lib().resynthNetGradients(self.handle, _vp(x), _vp(y), x.shape[0], _vp(g), C.byref(loss)),
               "resynthNetGradients")
        return float(loss.value), g

    def train(self, pairs: "Pairs", steps=2000, batch=512, lr=1e-3, seed=0) -> float:
        o = TrainOptions(steps, batch, lr, seed)
        loss = C.c_float(0)
        _check(lib().resynthNetTrain(self.handle, pairs.handle, C.byref(o), C.byref(loss)), "resynthNetTrain")
        return float(loss.value)


class Pairs:
    """Device-resident training pairs (resynthPairsCreate ... resynthPairsDestroy)."""

    def __init__(self, capacity: int):
        self.handle = lib().resynthPairsCreate(capacity)
        if not self.handle:
            raise RuntimeError(f"resynthPairsCreate: {last_error()}")

    def close(self):
        if self.handle:
            lib().resynthPairsDestroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __len__(self):
        return int(lib().resynthPairsCount(self.handle))

    def add(self, contexts: np.ndarray, labels: np.ndarray) -> int:
        x = np.ascontiguousarray(contexts, np.uint16)
        y = np.ascontiguousarray(labels, np.float32)
        return int(lib().resynthPairsAdd(self.handle, _vp(x), _vp(y), x.shape[0]))

    def read(self, first=0, n=None):
        n = len(self) - first if n is None else n
        x = np.zeros((n,) + CTX_SHAPE, np.uint16)
        y = np.zeros((n, 2), np.float32)
        _check(lib().resynthPairsRead(self.handle, first, n, _vp(x), _vp(y)), "resynthPairsRead")
        return x, y


def _check(rc, what):
    if rc:
        raise RuntimeError(f"{what} rc={rc}: {last_error()}")


def patch_neighbours(has_value: np.ndarray, patch_size: int, targets: np.ndarray, use_grid: bool):
    """resynthPatchNeighbours: per target, the (dx, dy) of its patch neighbours."""
    hv = np.ascontiguousarray(has_value, np.uint8)
    h, w = hv.shape
    t = np.ascontiguousarray(targets, np.int32)
    off = np.zeros((len(t), 63, 2), np.int32)
    cnt = np.zeros(len(t), np.uint32)
    _check(lib().resynthPatchNeighbours(_vp(hv), w, h, patch_size, _vp(t), len(t), int(use_grid), _vp(off), _vp(cnt)),
           "resynthPatchNeighbours")
    return [off[i, :cnt[i]] for i in range(len(t))]
