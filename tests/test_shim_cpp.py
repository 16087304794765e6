"""The C++ drop-in classes (imagecodingutils_gb300/shim/vppgpu_vpp.hpp): they
compile standalone and against vpp's own interface headers, and a codec-style
program built on them gives the oracle's results on the GPU."""
import os
import subprocess

import numpy as np
import pytest

from imagecodingutils_gb300 import synth
from oracle.oracle import REF_TREE

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHIM = os.path.join(ROOT, "imagecodingutils_gb300", "shim")
REF_INC = os.path.join(REF_TREE, "include")  # vpp's headers, only where the reference tree is present


def gxx(args):
    return subprocess.run(["g++", "-std=c++11", "-Wall", "-Wno-pragma-once-outside-header", *args],
                          capture_output=True, text=True)


def test_shim_compiles_standalone():
    r = gxx(["-fsyntax-only", "-I", SHIM, os.path.join(SHIM, "example_estimate.cpp")])
    assert r.returncode == 0, r.stderr


@pytest.mark.skipif(not os.path.isdir(REF_INC), reason="vpp headers not present on this host")
def test_shim_compiles_against_vpp_interfaces():
    r = gxx(["-fsyntax-only", "-DVPPGPU_WITH_VPP", "-include", "math.h", "-x", "c++",
             *[f"-I{REF_INC}/{d}" for d in ("CodecUtils", "GeneralUtils", "ImageUtils")],
             os.path.join(SHIM, "vppgpu_vpp.hpp")])
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["full", "multires", "mrc", "mrc2", "mrc2lam", "cross", "sad", "umhs", "fhs", "impl1",
                                  "impl2", "h263mrc2"])
def test_codec_style_program_on_gpu(tmp_path, vpp, orc, kind):
    from imagecodingutils_gb300 import build
    exe = tmp_path / "example_estimate"
    r = subprocess.run(["g++", "-std=c++11", "-O2", "-I", SHIM, os.path.join(SHIM, "example_estimate.cpp"),
                        "-L", os.path.dirname(build.LIB), "-lvppgpu", f"-Wl,-rpath,{os.path.dirname(build.LIB)}",
                        "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    w, h, mr = 176, 144, 128
    fr = synth.pan_sequence(77, w, h, 2)
    pair = tmp_path / "pair.bin"
    pair.write_bytes(fr[1].astype(np.int16).tobytes() + fr[0].astype(np.int16).tobytes())
    out = tmp_path / "out.bin"
    r = subprocess.run([str(exe), str(pair), str(w), str(h), str(mr), str(out), kind], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    nmb = (w // 16) * (h // 16)
    raw = out.read_bytes()
    if kind in ("impl1", "impl2"):  # the SimpleMotionVectorList's char vectors and the average
        mv = np.frombuffer(raw[:4 * nmb], np.int16).reshape(nmb, 2)
        # SetMode(0) at 176x144 (area below 40000) is Impl2's two-level mode 1
        mv_o, _, avg_o = orc.me_impl1(fr[1], fr[0], 16) if kind == "impl1" else orc.me_impl2(fr[1], fr[0], 16, 1)
        np.testing.assert_array_equal(mv, mv_o)
        assert np.frombuffer(raw[4 * nmb:4 * nmb + 8], np.int64)[0] == avg_o
        return
    mv = np.frombuffer(raw[:4 * nmb], np.int16).reshape(nmb, 2)
    avg = np.frombuffer(raw[4 * nmb:4 * nmb + 8], np.int64)[0]
    pred = np.frombuffer(raw[4 * nmb + 8:12 * nmb + 8], np.int32).reshape(nmb, 2)
    rest = np.frombuffer(raw[12 * nmb + 8:], np.int16)
    nblk = (w // 4) * 4
    levels, recon = rest[:16 * nblk], rest[16 * nblk:32 * nblk]
    dc_lev, dc_rec = rest[32 * nblk:32 * nblk + w], rest[32 * nblk + w:32 * nblk + 2 * w]
    tail = raw[12 * nmb + 8 + 2 * (32 * nblk + 2 * w):]
    pdist = np.frombuffer(tail[:4 * nmb], np.int32)
    prev_mv = np.frombuffer(tail[4 * nmb:], np.int16).reshape(-1, 2)
    ones = np.ones(nmb, np.uint8)
    if kind == "full":
        mv_o, _, avg_o = orc.me_full(fr[1], fr[0], mr, dist_incl=ones)
    elif kind == "multires":
        mv_o, _, avg_o = orc.me_multires(fr[1], fr[0], mr, mode=0, dist_incl=ones)
    elif kind == "mrc":
        mv_o, _, avg_o = orc.me_multires_cross(fr[1], fr[0], mr, mode=0, dist_incl=ones)
    elif kind == "h263mrc2":  # half pels, the predictor object is not called
        mv_o, _, avg_o = orc.me_h263_multires_cross_ver2(fr[1], fr[0], mr // 2, mode=0, dist_incl=ones)
    elif kind == "cross":
        mv_o, _, avg_o = orc.me_cross(fr[1], fr[0], mr, mode=0, dist_incl=ones)
    elif kind == "mrc2lam":
        mv_o, _, avg_o = orc.me_multires_cross_v2_lambda(fr[1], fr[0], mr, 2.5, mode=0, dist_incl=ones)
    elif kind == "sad":
        mv_o, d_o = orc.me_full_intpel(fr[1], fr[0], mr, metric=1)
        avg_o = int(d_o.sum()) // nmb
    elif kind == "umhs":
        mv0, _, _ = orc.me_umhs(fr[1], fr[0], mr)
        np.testing.assert_array_equal(prev_mv, mv0)
        mv_o, d_o, avg_o = orc.me_umhs(fr[1], fr[0], mr, dist_incl=ones, prev_mv=mv0)
        np.testing.assert_array_equal(pdist, d_o)  # the predictor receives each vector with its distortion
    elif kind == "fhs":
        mv_o, d_o, avg_o = orc.me_fhs(fr[1], fr[0], mr, dist_incl=ones)
        np.testing.assert_array_equal(pdist, d_o)
    else:
        mv_o, _, avg_o = orc.me_multires_cross_v2(fr[1], fr[0], mr, mode=0, dist_incl=ones)
    np.testing.assert_array_equal(mv, mv_o)
    assert avg == avg_o
    if kind not in ("mrc", "h263mrc2"):  # MultiresCross has no predictor, the H.263 one sets none
        np.testing.assert_array_equal(pred, mv_o.astype(np.int32))
    res = (fr[1][:16].astype(np.int32) - fr[0][:16]).astype(np.int16)
    blocks = res.reshape(4, 4, w // 4, 4).transpose(0, 2, 1, 3).reshape(-1, 16)
    lev_o = orc.fwd4x4(blocks, 0, 0, 28, 0)
    np.testing.assert_array_equal(levels.reshape(-1, 16), lev_o)
    np.testing.assert_array_equal(recon.reshape(-1, 16), orc.inv4x4(lev_o, 0, 0, 28))
    coeffs = orc.fwd4x4(blocks, 0, 1, 1, 1).reshape(4, w // 16, 4, 16)   # (block row, MB, block col, coeff)
    dc = coeffs[:, :, :, 0].transpose(1, 0, 2).reshape(-1, 16)
    dc_lev_o = orc.fwd_dc(dc, 4, 0, 28)
    np.testing.assert_array_equal(dc_lev.reshape(-1, 16), dc_lev_o)
    np.testing.assert_array_equal(dc_rec.reshape(-1, 16), orc.inv_dc(dc_lev_o, 4, 0, 28))
