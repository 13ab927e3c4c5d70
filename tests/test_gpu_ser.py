"""sst_stack_ser on the GPU: frames streamed from a SER file (pinned chunk
buffers, the next chunk read while the current one is registered and
stacked) give exactly what sst_stack_frames / sst_stack_bayer_frames give on
the same frames with the same chunking and the read_input_frame scale
1 / 2^bits_per_plane (bitwise: parameters, statuses and accumulator state)."""
import numpy as np
import pytest

from serstacker_gb300 import synth
from ser_files import write_ser

pytestmark = pytest.mark.gpu


def _registration(C, ref, scale, chunk):
    reg = C.c_ecch(C.default_options(method=1, maxlevel=2, max_iterations=30, epsx=0.01, minimum_image_size=16))
    reg.set_reference_image(ref.astype(np.float32), scale=scale)
    reg.set_chunk_frames(chunk)
    return reg


@pytest.mark.parametrize("first,count", [(0, -1), (2, 3)])
def test_stack_ser_equals_stack_frames(gpu, tmp_path, first, count):
    C = gpu
    w, h, n = 160, 120, 7
    sc = synth.Scene(w, h, 0.3 * min(w, h))
    frames, _, _ = synth.make_sequence_np(sc, n, seed=41, kind="config1", dtype=np.uint16, gain=64.0)
    ref = synth.reference_np(sc) * 64.0
    ts = np.arange(n, dtype=np.uint64) + 1000
    path = str(write_ser(tmp_path / "mono.ser", frames, bits=16, timestamps=ts))
    scale = 1.0 / 65536
    m = n - first if count < 0 else count
    sel = frames[first:first + m]
    reg = _registration(C, ref, scale, 4)
    acc = C.c_weigthed_average(w, h)
    ser = C.c_ser_reader(path)
    out = C.stack_ser(reg, acc, ser, [3, 4], first=first, count=count, chunk=4)
    reg2 = _registration(C, ref, scale, 4)
    acc2 = C.c_weigthed_average(w, h)
    outs = [C.stack_frames(reg2, acc2, sel[k:k + 4], [3, 4], scale) for k in range(0, m, 4)]
    want = {k: np.concatenate([o[k] for o in outs]) for k in ("params", "status", "rho", "weight")}
    for k in ("params", "status", "rho", "weight"):
        assert np.array_equal(out[k], want[k]), k
    s1, f1 = acc.save_state()
    s2, f2 = acc2.save_state()
    assert f1 == f2 == int((want["status"] == 0).sum())
    assert np.array_equal(s1, s2)


def test_stack_ser_bayer_equals_stack_bayer_frames(gpu, tmp_path):
    from test_gpu_bayer import _raw_sequence
    C, W_, H_, n = gpu, 192, 128, 5
    frames, ref_raw, _ = _raw_sequence(n, W_, H_, 17)
    path = str(write_ser(tmp_path / "bayer.ser", frames, color_id=8, bits=12))
    import oracle as O
    ref_bin = O.average_bayer_planes(ref_raw).astype(np.float32)
    scale = 1.0 / 4096
    res = []
    for mode in ("ser", "frames"):
        reg = _registration(C, ref_bin, scale, 3)
        accs = [C.c_weigthed_average(W_ // 2, H_ // 2) for _ in range(4)]
        if mode == "ser":
            out = C.stack_ser(reg, accs, C.c_ser_reader(path), [C.TRANSLATION], chunk=3)
        else:
            parts = [C.stack_bayer_frames(reg, accs, frames[k:k + 3], [C.TRANSLATION], scale) for k in range(0, n, 3)]
            out = {k: np.concatenate([o[k] for o in parts]) for k in ("params", "status", "rho", "weight")}
        res.append((out, [a.save_state()[0] for a in accs]))
    for k in ("params", "status", "rho", "weight"):
        assert np.array_equal(res[0][0][k], res[1][0][k]), k
    for p in range(4):
        assert np.array_equal(res[0][1][p], res[1][1][p]), p


def test_stack_ser_rejects_unsupported_files(gpu, tmp_path):
    C = gpu
    rgb = np.zeros((2, 64, 64, 3), np.uint8)
    path = str(write_ser(tmp_path / "rgb.ser", rgb, color_id=100, bits=8))
    y, x = np.mgrid[0:64, 0:64]
    reg = _registration(C, np.sin(x / 5.0) * np.cos(y / 7.0), 1.0, 4)
    ser = C.c_ser_reader(path)
    acc = C.c_weigthed_average(64, 64)
    with pytest.raises(C.SSTError):
        C.stack_ser(reg, acc, ser, [0])
