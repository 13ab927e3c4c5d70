"""The C++ drop-in classes on the GPU: a program compiled against
include/serstacker_gb300.hpp runs c_frame_registration::setup_reference_frame,
register_frame (the reference's registration options: ecc.scale 0.5, an IC
pyramid of 3 levels with the translation estimate first) with its remap of
each frame, and c_weigthed_average::add of the warped frames with their masks,
as the stacking pipeline's loop body does (c_image_stacking_pipeline.cc:
1539-1790). Checked against the FP64 oracle:
  - every frame's transform within 0.02 px RMS of the oracle's register_frame;
  - every frame's current remap within 1e-3 px of its transform's warp;
  - the stack within 1e-5 relative (1 % floor) of FP64 sums of the frames
    sampled at the program's own remap positions (FP32 coordinates, as the
    reference's cv::Mat2f maps hold them), on every settled pixel.
"""
import math
import os
import shutil
import subprocess

import numpy as np
import pytest

from serstacker_gb300 import synth

pytestmark = pytest.mark.gpu

PROGRAM = r'''
#include "serstacker_gb300.hpp"
#include <cstdio>
#include <vector>

static bool load(const char * path, void * dst, size_t bytes)
{
  FILE * f = std::fopen(path, "rb");
  if( !f ) return false;
  const bool ok = std::fread(dst, 1, bytes, f) == bytes;
  std::fclose(f);
  return ok;
}

static bool save(const char * path, const void * src, size_t bytes)
{
  FILE * f = std::fopen(path, "wb");
  if( !f ) return false;
  const bool ok = std::fwrite(src, 1, bytes, f) == bytes;
  std::fclose(f);
  return ok;
}

int main(int argc, char ** argv)
{
  const int W = 256, H = 192, N = 3;
  const char * dir = argv[1];
  char path[4096];
  std::vector<float> ref((size_t) W * H);
  std::vector<uint16_t> frames((size_t) N * W * H);
  std::snprintf(path, sizeof(path), "%s/ref.f32", dir);
  if( !load(path, ref.data(), ref.size() * 4) ) return 1;
  std::snprintf(path, sizeof(path), "%s/frames.u16", dir);
  if( !load(path, frames.data(), frames.size() * 2) ) return 2;

  sst_gb300::c_image_registration_options o;
  o.motion_type = SST_MOTION_AFFINE;
  o.enable_feature_registration = false;
  o.enable_ecc_registration = true;
  o.ecc.scale = 0.5;
  o.ecc.ecc_method = SST_ECC_INVERSE_COMPOSITIONAL;
  o.ecc.ecch_max_level = 3;
  o.ecc.eps = 0.01;
  sst_gb300::c_frame_registration reg(o);
  if( !reg.setup_reference_frame(sst_gb300::image_view(ref.data(), W, H, SST_DEPTH_F32, W * 4)) ) {
    std::fprintf(stderr, "setup_reference_frame: %s\n", sst_gb300::last_error().c_str());
    return 3;
  }
  sst_gb300::c_weigthed_average acc;
  std::vector<float> params((size_t) N * 12, 0.f);
  std::vector<float> rmaps;
  std::vector<float> dst;
  std::vector<uint8_t> dmask;
  for( int i = 0; i < N; ++i ) {
    sst_gb300::image_view cur(frames.data() + (size_t) i * W * H, W, H, SST_DEPTH_U16, W * 2);
    if( !reg.register_frame(cur, &dst, &dmask, 1.0 / 65535.0) ) {
      std::fprintf(stderr, "register_frame %d: status %d, %s\n", i, reg.status().frame_status,
          sst_gb300::last_error().c_str());
      return 4;
    }
    const std::vector<float> & p = reg.image_transform_ref().parameters;
    for( size_t j = 0; j < p.size(); ++j ) params[(size_t) i * 12 + j] = p[j];
    if( reg.current_remap().size() != (size_t) W * H * 2 ) return 5;
    rmaps.insert(rmaps.end(), reg.current_remap().begin(), reg.current_remap().end());
    if( !acc.add(sst_gb300::image_view(dst.data(), W, H, SST_DEPTH_F32, W * 4),
            sst_gb300::image_view(dmask.data(), W, H, SST_DEPTH_U8, W)) ) {
      std::fprintf(stderr, "add: %s\n", sst_gb300::last_error().c_str());
      return 6;
    }
  }
  std::vector<float> avg;
  std::vector<uint8_t> mask;
  if( !acc.compute(avg, mask) ) return 7;
  std::snprintf(path, sizeof(path), "%s/params.f32", dir);
  if( !save(path, params.data(), params.size() * 4) ) return 8;
  std::snprintf(path, sizeof(path), "%s/avg.f32", dir);
  if( !save(path, avg.data(), avg.size() * 4) ) return 9;
  std::snprintf(path, sizeof(path), "%s/mask.u8", dir);
  if( !save(path, mask.data(), mask.size()) ) return 10;
  std::snprintf(path, sizeof(path), "%s/rmaps.f32", dir);
  if( !save(path, rmaps.data(), rmaps.size() * 4) ) return 11;
  std::printf("ok\n");
  return 0;
}
'''


def _remap_fp64(img, rmap):
    """base_remap in FP64 at given map positions: bilinear, BORDER_REFLECT_101;
    the mask is the in-image bilinear weight >= 254.5 / 255, eroded 5 x 5 with
    the window clipped to the image."""
    from scipy.ndimage import minimum_filter
    h, w = img.shape
    X, Y = rmap[..., 0], rmap[..., 1]
    x0, y0 = np.floor(X).astype(np.int64), np.floor(Y).astype(np.int64)
    fx, fy = X - x0, Y - y0

    def r101(p, n):
        p = np.abs(p)
        p = p % (2 * (n - 1))
        return np.where(p >= n, 2 * (n - 1) - p, p)

    def tap(xi, yi):
        return img[r101(yi, h), r101(xi, w)]

    val = ((1 - fy) * ((1 - fx) * tap(x0, y0) + fx * tap(x0 + 1, y0)) +
           fy * ((1 - fx) * tap(x0, y0 + 1) + fx * tap(x0 + 1, y0 + 1)))
    inx0, inx1 = (x0 >= 0) & (x0 < w), (x0 + 1 >= 0) & (x0 + 1 < w)
    iny0, iny1 = (y0 >= 0) & (y0 < h), (y0 + 1 >= 0) & (y0 + 1 < h)
    cov = (np.where(inx0, 1 - fx, 0) + np.where(inx1, fx, 0)) * (np.where(iny0, 1 - fy, 0) + np.where(iny1, fy, 0))
    raw = (255 * cov + 0.5 >= 255).astype(np.uint8)
    return val, minimum_filter(raw, 5, mode="nearest")


def test_cpp_register_frame_remap_add_matches_oracle(gpu, oracle, tmp_path):
    C, O = gpu, oracle
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    w, h, n = 256, 192, 3
    sc = synth.Scene(w, h, 0.3 * min(w, h), band_period=16.0)
    frames, _, _ = synth.make_sequence_np(sc, n, seed=71, kind="config1", dtype=np.uint16, gain=64.0,
                                          blur_range=(0.8, 2.0))
    scale = 1.0 / 65535.0
    ref = (synth.reference_np(sc) * 64.0 * scale).astype(np.float32)
    ref.tofile(tmp_path / "ref.f32")
    frames.tofile(tmp_path / "frames.u16")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = tmp_path / "t.cc"
    src.write_text(PROGRAM)
    libdir = os.path.dirname(C.LIB_PATH)
    exe = tmp_path / "t"
    subprocess.check_call([gxx, "-std=c++17", "-O2", "-I", os.path.join(root, "include"), str(src), "-o", str(exe),
                           "-L", libdir, "-lsst_gb300", f"-Wl,-rpath,{libdir}"])
    out = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True)
    assert out.returncode == 0, (out.returncode, out.stderr)
    params = np.fromfile(tmp_path / "params.f32", np.float32).reshape(n, 12)
    rmaps = np.fromfile(tmp_path / "rmaps.f32", np.float32).reshape(n, h, w, 2)
    avg = np.fromfile(tmp_path / "avg.f32", np.float32).reshape(h, w)
    mask = np.fromfile(tmp_path / "mask.u8", np.uint8).reshape(h, w)

    oo = O.registration_opts(motion_type=O.AFFINE, method=O.IC, ecch_max_level=3, eps=0.01)
    m = O.model(O.AFFINE)
    S = np.zeros((h, w))
    W = np.zeros((h, w))
    ms = []
    for i in range(n):
        img = frames[i].astype(np.float64) * scale
        status, st, rho, _ = O.register_frame(oo, ref.astype(np.float64), img)
        assert status == 0
        s_g = O.set_params(m, O.identity(m), params[i, :6].astype(np.float64))
        xa, ya = O.warp_grid(m, s_g, w, h)
        xb, yb = O.warp_grid(m, st, w, h)
        rms = math.sqrt(float(((xa - xb) ** 2 + (ya - yb) ** 2).mean()))
        assert rms <= 0.02, (i, rms)
        ms.append((m, s_g))
        assert np.abs(rmaps[i, ..., 0] - xa).max() < 1e-3 and np.abs(rmaps[i, ..., 1] - ya).max() < 1e-3
        dst, msk = _remap_fp64(img, rmaps[i].astype(np.float64))
        wt = (msk > 0).astype(np.float64)
        S += wt * dst
        W += wt
    keep = O.stack_compare_region(ms, w, h, w, h)
    assert np.array_equal((mask > 0)[keep], (W > 0)[keep])
    both = keep & (W > 0)
    rel = O.stack_rel_err(avg[both], S[both] / W[both])
    assert rel.max() <= 1e-5, rel.max()
