"""CPU-side checks of libresynthesizer.so: it builds, exports every entry point
include/resynthesizer.h declares, answers the reference's argument and data
errors before touching a device, and links with the reference's own test
program (src/testSynth.c) unchanged.  No synthesis runs here (no GPU)."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

import resynthesizer_gb300 as R
from resynthesizer_gb300 import build as B

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "resynthesizer.h")


@pytest.fixture(scope="module")
def lib():
    B.build()
    return R.lib()


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(\w+)\s*\(", text, flags=re.M)) - {"if"})


def test_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert "imageSynth" in names and "engine" in names and "resynthFrozenBestFit" in names
    out = subprocess.run(["nm", "-D", "--defined-only", B.LIB], capture_output=True, text=True, check=True).stdout
    exported = {l.split()[-1] for l in out.splitlines() if " T " in l}
    missing = [n for n in names if n not in exported]
    assert not missing, missing


def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def test_host_side_errors(lib):
    img = np.array([[[128], [64], [1]]], np.uint8)
    mask = np.array([[0, 255, 0]], np.uint8)
    cases = [
        (R.params(patchSize=65), mask, R.T_Gray, 3),
        (R.params(), np.array([[0]], np.uint8), R.T_Gray, 2),
        (R.params(), np.zeros((1, 3), np.uint8), R.T_Gray, 5),
        (R.params(), mask, 7, 1),
        (R.params(matchContextType=9), mask, R.T_Gray, 4),
    ]
    for p, m, fmt, expect in cases:
        for raw in (False, True):
            r = R.image_synth(img, m, fmt, p, raw_entry=raw)
            assert r.rc == expect
            assert (r.out == img).all()
    rgba = np.array([[[128, 128, 128, 0], [1, 1, 1, 1], [0, 0, 0, 0]]], np.uint8)
    assert R.image_synth(rgba, mask, R.T_RGBA, R.params()).rc == 6


@pytest.mark.skipif(has_gpu(), reason="checks the no-GPU path")
def test_no_gpu_fails_loudly(lib):
    img = np.array([[[128], [64], [1]]], np.uint8)
    r = R.image_synth(img, np.array([[0, 255, 0]], np.uint8), R.T_Gray, R.params())
    assert r.rc == 100 and "CUDA" in R.last_error() or "device" in R.last_error().lower()
    assert (r.out == img).all()


def test_format_and_map_helpers(lib):
    f = R.FormatIndices()
    assert lib.prepareImageFormatIndicesFromFormatType(C.byref(f), R.T_RGBA) == 0
    assert (f.colorEndBip, f.alpha_bip, f.map_start_bip, f.total_bpp, f.img_match_bpp) == (4, 4, 5, 5, 3)
    assert lib.prepareImageFormatIndicesFromFormatType(C.byref(f), 9) == 1
    g = R.format_indices(3, 1, 0, 0, 1)
    assert (g.colorEndBip, g.map_start_bip, g.map_end_bip, g.total_bpp, g.map_match_bpp) == (4, 4, 5, 5, 1)
    assert [lib.countPixelelsPerPixelForFormat(t) for t in range(5)] == [3, 4, 1, 2, 0]
    p = R.default_params()
    assert (p.matchContextType, p.patchSize, p.maxProbeCount) == (1, 30, 200)
    assert abs(p.sensitivityToOutliers - 0.117) < 1e-12 and p.mapWeight == 0.5
    pix, mask = R.Map(), R.Map()
    lib.new_pixmap(C.byref(pix), 3, 2, 4)
    lib.new_bytemap(C.byref(mask), 3, 2)
    lib.set_bytemap(C.byref(mask), 0x0F)
    lib.invert_bytemap(C.byref(mask))
    lib.interleave_mask(C.byref(pix), C.byref(mask))
    data = (C.c_ubyte * 24).from_address(pix.data.contents.data)
    assert list(data)[0::4] == [0xF0] * 6 and sum(data) == 0xF0 * 6
    lib.free_map(C.byref(pix))
    lib.free_map(C.byref(mask))
    assert not pix.data


def test_reference_testsynth_links_unchanged(lib, tmp_path):
    """The reference's own test harness, compiled against the reference's
    headers, links against this library with no source change."""
    from oracle import reference_tree
    ref = reference_tree()
    if not ref or not os.path.exists(os.path.join(ref, "src", "testSynth.c")):
        pytest.skip("reference tree not present")
    shim = tmp_path / "shim"
    shim.mkdir()
    (shim / "buildSwitches.h").write_text("#define USE_GLIB_PROXY TRUE\n#define THREAD_LIMIT 1\n")
    (shim / "engineParams.h").write_text(
        f'#ifndef EP_GUARD\n#define EP_GUARD\n#include "{ref}/lib/engineParams.h"\n#endif\n')
    exe = tmp_path / "testSynth"
    cmd = ["gcc", "-std=gnu99", "-DSYNTH_LIB_ALONE", "-w", f"-I{shim}", "-I-", f"-I{ref}/lib",
           f"{ref}/src/testSynth.c", "-o", str(exe), f"-L{os.path.dirname(B.LIB)}", "-lresynthesizer",
           f"-Wl,-rpath,{os.path.dirname(B.LIB)}"]
    subprocess.run(cmd, check=True, capture_output=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0
    assert "Test Gray w/o alpha" in r.stdout


def test_layouts_reaching_past_the_pixel_are_rejected(lib):
    """A TFormatIndices whose colour, map or alpha bytes lie past total_bpp is
    refused with RESYNTH_ERROR_UNSUPPORTED before any device work (the
    kernels would otherwise read past the end of the caller's buffers).  The
    pointers are never dereferenced: the call must answer from the layout
    alone."""
    P = C.POINTER
    lib.resynthFrozenBestFitNoAlloc.argtypes = [P(R.ImageSynthParameters), P(R.FormatIndices)] + [
        C.c_void_p, C.c_uint, C.c_uint, C.c_void_p, C.c_uint, C.c_uint, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint,
        C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    p = R.params()
    bad = []
    f = R.format_indices(3, 1, 0, 0, 1)
    f.total_bpp = 4                        # the map byte would be byte 4 of a 4-byte pixel
    bad.append(f)
    f = R.format_indices(3, 0, 0, 0, 0)
    f.total_bpp = 3                        # colours end at byte 4
    bad.append(f)
    f = R.format_indices(2, 2, 0, 0, 1)
    f.map_start_bip = 4                    # map channels 4..5 of a 5-byte pixel
    bad.append(f)
    dummy = C.c_void_p(16)
    buf = np.zeros(4096, np.uint8)            # host buffers, large enough for any of these layouts
    hb = C.c_void_p(buf.ctypes.data)
    for f in bad:
        rc = lib.resynthFrozenBestFitNoAlloc(C.byref(p), C.byref(f), dummy, 8, 8, dummy, 8, 8, dummy, dummy, dummy,
                                             1, dummy, dummy, dummy, dummy, dummy, None)
        assert rc == 101 and "layout" in R.last_error()
        rc = lib.resynthFrozenBestFit(C.byref(p), C.byref(f), hb, 8, 8, hb, 8, 8, hb, hb, hb, 0, hb, hb, hb, hb, hb)
        assert rc == 101
    # alpha byte outside the pixel, through engine() on host maps
    f = R.format_indices(3, 0, 1, 1, 0)
    f.alpha_bip = 9
    t = np.zeros((4, 4, f.total_bpp), np.uint8)
    t[1:3, 1:3, 0] = 255
    r = R.engine(t, t.copy(), f, R.params())
    assert r.rc == 101
