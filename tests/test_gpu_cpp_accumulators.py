"""The C++ drop-in classes of the other accumulators and of LPG on the GPU: a
program compiled against include/serstacker_gb300.hpp runs
c_lpg_sharpness_measure::compute, c_frame_accumulation_with_fft::add /
compute, c_laplacian_pyramid_focus_stacking::add / compute,
c_canvas_average::add / compute and linear_interpolation_inpaint on frames
written by this test; the results are checked against the FP64 oracle with
the tolerances of the C ABI tests (2e-5 of the maximum; 2e-6 for the canvas
and the inpaint)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

W, H, N = 96, 72, 4

PROGRAM = r'''
#include "serstacker_gb300.hpp"
#include <cstdio>
#include <vector>

static bool io(const char * dir, const char * name, void * p, size_t bytes, bool write)
{
  char path[4096];
  std::snprintf(path, sizeof(path), "%s/%s", dir, name);
  FILE * f = std::fopen(path, write ? "wb" : "rb");
  if( !f ) return false;
  const bool ok = (write ? std::fwrite(p, 1, bytes, f) : std::fread(p, 1, bytes, f)) == bytes;
  std::fclose(f);
  return ok;
}

int main(int argc, char ** argv)
{
  const int W = 96, H = 72, N = 4;
  const char * dir = argv[1];
  std::vector<float> frames((size_t) N * W * H);
  std::vector<uint8_t> masks((size_t) N * W * H);
  std::vector<float> rmap((size_t) 80 * 60 * 2);
  if( !io(dir, "frames.f32", frames.data(), frames.size() * 4, false) ) return 1;
  if( !io(dir, "masks.u8", masks.data(), masks.size(), false) ) return 2;
  if( !io(dir, "rmap.f32", rmap.data(), rmap.size() * 4, false) ) return 3;
  auto view = [&](int i) { return sst_gb300::image_view(frames.data() + (size_t) i * W * H, W, H, SST_DEPTH_F32, W * 4); };
  auto mview = [&](int i) { return sst_gb300::image_view(masks.data() + (size_t) i * W * H, W, H, SST_DEPTH_U8, W); };

  sst_gb300::c_lpg_sharpness_measure lpg;
  std::vector<float> map;
  double metric = 0;
  if( !lpg.compute(view(0), map, &metric) ) return 4;
  if( !io(dir, "lpg.f32", map.data(), map.size() * 4, true) || !io(dir, "lpg_metric.f64", &metric, 8, true) ) return 5;

  sst_gb300::c_frame_accumulation_with_fft fft;
  for( int i = 0; i < N; ++i ) if( !fft.add(view(i)) ) return 6;
  std::vector<float> avg;
  std::vector<uint8_t> mask;
  if( !fft.compute(avg, mask) || !io(dir, "fft.f32", avg.data(), avg.size() * 4, true) ) return 7;

  sst_gb300::c_laplacian_pyramid_focus_stacking fs;
  for( int i = 0; i < N; ++i ) if( !fs.add(view(i), mview(i)) ) return 8;
  if( !fs.compute(avg) || !io(dir, "focus.f32", avg.data(), avg.size() * 4, true) ) return 9;

  sst_gb300::c_canvas_average canvas;
  canvas.setCanvasSize(300, 200);
  std::vector<float> none;
  if( !canvas.add(view(0), mview(0), none, sst_gb300::rect()) ) return 10;
  if( !canvas.add(view(1), mview(1), rmap, sst_gb300::rect(150, 90, 80, 60)) ) return 11;
  sst_gb300::rect ob;
  if( !canvas.compute(avg, mask, 1.0, sst_gb300::rect(), &ob) ) return 12;
  if( ob.width != 300 || ob.height != 200 ) return 13;
  if( !io(dir, "canvas.f32", avg.data(), avg.size() * 4, true) || !io(dir, "canvas_mask.u8", mask.data(), mask.size(), true) )
    return 14;

  std::vector<float> img(frames.begin() + (size_t) W * H, frames.begin() + (size_t) 2 * W * H);
  std::vector<uint8_t> m1(masks.begin() + (size_t) W * H, masks.begin() + (size_t) 2 * W * H);
  if( !sst_gb300::linear_interpolation_inpaint(img, m1, W, H) || !io(dir, "inpaint.f32", img.data(), img.size() * 4, true) )
    return 15;
  std::printf("ok\n");
  return 0;
}
'''


def test_cpp_accumulators_match_oracle(gpu, oracle, tmp_path):
    C, O = gpu, oracle
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    rng = np.random.default_rng(12)
    y, x = np.mgrid[0:H, 0:W].astype(np.float64)
    frames = np.stack([0.5 + 0.3 * np.sin(x / (4.0 + i)) * np.cos(y / 5.0) + 0.02 * rng.standard_normal((H, W))
                       for i in range(N)]).astype(np.float32)
    masks = np.full((N, H, W), 255, np.uint8)
    for i in range(N):
        masks[i, :, : 1 + i] = 0
        masks[i, 20 + 3 * i:26 + 3 * i, 40:47] = 0
    masks[0::2] = 255                                  # every other frame whole (see the focus tests)
    yy, xx = np.mgrid[0:60, 0:80].astype(np.float64)
    rmap = np.stack([xx * 1.01 + 3.3, yy * 0.99 + 2.1], axis=-1).astype(np.float32)
    frames.tofile(tmp_path / "frames.f32")
    masks.tofile(tmp_path / "masks.u8")
    rmap.tofile(tmp_path / "rmap.f32")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = tmp_path / "t.cc"
    src.write_text(PROGRAM)
    libdir = os.path.dirname(C.LIB_PATH)
    exe = tmp_path / "t"
    subprocess.check_call([gxx, "-std=c++17", "-O2", "-I", os.path.join(root, "include"), str(src), "-o", str(exe),
                           "-L", libdir, "-lsst_gb300", f"-Wl,-rpath,{libdir}"])
    out = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True)
    assert out.returncode == 0, (out.returncode, out.stderr)

    def rel(got, want):
        return np.abs(got - want).max() / np.abs(want).max()

    f64 = frames.astype(np.float64)
    lpg = np.fromfile(tmp_path / "lpg.f32", np.float32).reshape(H, W)
    met = np.fromfile(tmp_path / "lpg_metric.f64", np.float64)[0]
    want, wmet = O.lpg(f64[0])
    assert rel(lpg, want) <= 2e-5 and met == pytest.approx(wmet, rel=2e-5)
    fft = np.fromfile(tmp_path / "fft.f32", np.float32).reshape(H, W)
    assert rel(fft, O.fft_average(f64)) <= 2e-5
    focus = np.fromfile(tmp_path / "focus.f32", np.float32).reshape(H, W)
    assert rel(focus, O.focus_stack(f64, masks)) <= 2e-5
    canvas = np.fromfile(tmp_path / "canvas.f32", np.float32).reshape(200, 300)
    cmask = np.fromfile(tmp_path / "canvas_mask.u8", np.uint8).reshape(200, 300)
    boxes = np.array([[0, 0, 0, 0], [150, 90, 80, 60]], np.int32)
    oacc, oW, _, _ = O.canvas_average(f64[:2], weights=masks[:2], boxes=boxes, rmaps=[None, rmap.astype(np.float64)],
                                      canvas=(300, 200))
    assert np.array_equal(cmask > 0, oW > 0) and rel(canvas, oacc) <= 2e-6
    inp = np.fromfile(tmp_path / "inpaint.f32", np.float32).reshape(H, W)
    assert (masks[1] == 0).sum() > 100
    assert rel(inp, O.linear_inpaint(f64[1], masks[1])) <= 2e-6
