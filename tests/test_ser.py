"""SER v3 input through the C ABI on the CPU: sst_ser_* against files written
by tests/ser_files.py. Covers c_ser_reader's header checks, the inverted
LittleEndian field (0 = little-endian pixel data, c_ser_file.cc:304-305), the
bits-per-plane extension (-32, -64, 17..32), timestamps, seek / curpos and
truncated files. Byte-for-byte: every read is compared exactly."""
import ctypes as C

import numpy as np
import pytest

from ser_files import write_ser


@pytest.fixture(scope="module")
def capi():
    from serstacker_gb300 import capi
    capi.lib()
    return capi


def _frames(n, h, w, dtype, seed=0):
    rng = np.random.default_rng(seed)
    if np.issubdtype(dtype, np.integer):
        info = np.iinfo(dtype)
        return rng.integers(max(info.min, -2 ** 31), min(info.max, 2 ** 31 - 1), size=(n, h, w), dtype=np.int64,
                            endpoint=True).astype(dtype)
    return rng.standard_normal((n, h, w)).astype(dtype)


def test_mono_u16_with_timestamps(capi, tmp_path):
    fr = _frames(5, 7, 9, np.uint16)
    ts = np.arange(5, dtype=np.uint64) * 10_000_000 + 638_000_000_000_000_000
    p = write_ser(tmp_path / "a.ser", fr, bits=12, timestamps=ts, luid=3, observer=b"obs", instrument=b"cam",
                  telescope=b"scope", date_time=123, date_time_utc=456)
    r = capi.c_ser_reader(str(p))
    i = r.info
    assert (i.width, i.height, i.frames, i.bits_per_plane, i.color_id, i.luid) == (9, 7, 5, 12, 0, 3)
    assert (i.channels, i.bytes_per_plane, i.depth, i.data_little_endian) == (1, 2, capi.DEPTH_U16, 1)
    assert (i.observer, i.instrument, i.telescope) == (b"obs", b"cam", b"scope")
    assert (i.date_time, i.date_time_utc) == (123, 456)
    assert i.has_timestamps == 1 and np.array_equal(r.timestamps(), ts)
    got = r.read(3)
    assert np.array_equal(got, fr[:3]) and r.curpos() == 3
    assert np.array_equal(r.read(10), fr[3:]) and r.curpos() == 5
    assert r.read(1).shape[0] == 0          # at the end: nothing more


def test_big_endian_data_is_swapped(capi, tmp_path):
    fr = _frames(3, 4, 6, np.uint16, 1)
    ts = np.array([1, 2, 3 << 40], np.uint64)
    r = capi.c_ser_reader(str(write_ser(tmp_path / "b.ser", fr, le_field=1, timestamps=ts)))
    assert r.info.data_little_endian == 0
    assert np.array_equal(r.read(3), fr)
    assert np.array_equal(r.timestamps(), ts)


@pytest.mark.parametrize("dtype,bits,depth_name", [
    (np.uint8, 8, "DEPTH_U8"), (np.uint8, 6, "DEPTH_U8"), (np.uint16, 16, "DEPTH_U16"),
    (np.int32, 24, None), (np.float32, -32, "DEPTH_F32"), (np.float64, -64, None)])
@pytest.mark.parametrize("le_field", [0, 1])
def test_pixel_formats(capi, tmp_path, dtype, bits, depth_name, le_field):
    fr = _frames(2, 5, 3, dtype, 2)
    r = capi.c_ser_reader(str(write_ser(tmp_path / "c.ser", fr, bits=bits, le_field=le_field)))
    assert r.info.bytes_per_plane == np.dtype(dtype).itemsize
    if depth_name:
        assert r.info.depth == getattr(capi, depth_name)
    assert r.info.has_timestamps == 0
    assert np.array_equal(r.read(2), fr)


def test_rgb_frames_have_three_channels(capi, tmp_path):
    fr = _frames(2, 4, 5 * 3, np.uint8, 3).reshape(2, 4, 5, 3)
    r = capi.c_ser_reader(str(write_ser(tmp_path / "d.ser", fr, color_id=100, bits=8)))
    assert r.info.channels == 3 and r.info.width == 5
    assert np.array_equal(r.read(2), fr)


def test_seek_follows_the_reference(capi, tmp_path):
    fr = _frames(4, 3, 3, np.uint16, 4)
    r = capi.c_ser_reader(str(write_ser(tmp_path / "e.ser", fr)))
    r.seek(2)
    assert r.curpos() == 2 and np.array_equal(r.read(1)[0], fr[2])
    r.seek(-5)                                # negative positions seek to frame 0
    assert r.curpos() == 0
    with pytest.raises(capi.SSTError):
        r.seek(4)                             # past the last frame
    r.seek(3)
    r.read(1)
    r.seek(4)                                 # equal to the current position: accepted as is
    assert r.curpos() == 4


def test_strided_reads(capi, tmp_path):
    fr = _frames(3, 4, 5, np.uint16, 5)
    r = capi.c_ser_reader(str(write_ser(tmp_path / "f.ser", fr)))
    stride = 4 * 5 * 2 + 24
    buf = np.zeros(3 * stride, np.uint8)
    got = C.c_int()
    assert capi.lib().sst_ser_read(r.handle, 3, buf.ctypes.data, stride, C.byref(got)) == 0 and got.value == 3
    for k in range(3):
        assert np.array_equal(buf[k * stride:k * stride + 40].view(np.uint16).reshape(4, 5), fr[k])
    assert capi.lib().sst_ser_read(r.handle, 1, buf.ctypes.data, 8, C.byref(got)) != 0   # stride below a frame


@pytest.mark.parametrize("kw,code", [
    ({"magic": b"NOT-A-SER-FILE"}, -3),
    ({"color_id": 5}, -3),
    ({"bits": 0}, -3),
    ({"bits": 40}, -3),
])
def test_rejected_headers(capi, tmp_path, kw, code):
    p = write_ser(tmp_path / "g.ser", _frames(1, 2, 2, np.uint16), **kw)
    h = C.c_void_p()
    assert capi.lib().sst_ser_open(C.byref(h), str(p).encode()) == code
    assert not h.value


def test_zero_width_and_short_files(capi, tmp_path):
    p = write_ser(tmp_path / "h.ser", np.zeros((1, 2, 0), np.uint16))
    h = C.c_void_p()
    assert capi.lib().sst_ser_open(C.byref(h), str(p).encode()) == -3
    (tmp_path / "i.ser").write_bytes(b"LUCAM-RECORDER" + bytes(20))
    assert capi.lib().sst_ser_open(C.byref(h), str(tmp_path / "i.ser").encode()) == -7
    assert capi.lib().sst_ser_open(C.byref(h), str(tmp_path / "missing.ser").encode()) == -7


def test_truncated_file_fails_to_read(capi, tmp_path):
    fr = _frames(2, 3, 4, np.uint16, 6)
    r = capi.c_ser_reader(str(write_ser(tmp_path / "j.ser", fr, frames_count=3)))
    assert r.info.frames == 3 and r.info.has_timestamps == 0
    assert np.array_equal(r.read(2), fr)
    with pytest.raises(capi.SSTError):
        r.read(1)


@pytest.mark.parametrize("le_field", [0, 1])
def test_large_reads_split_over_threads(capi, tmp_path, le_field):
    """reads above 64 MB go through several host threads (1 MB pieces, frames
    for strided reads and byte swaps); the bytes are the same"""
    fr = _frames(40, 512, 1024, np.uint16, 7)                 # 40 MB of frames
    fr = np.concatenate([fr, fr[::-1] ^ np.uint16(0x5a5a)])   # 80 MB, no two frames alike
    p = write_ser(tmp_path / "k.ser", fr, le_field=le_field)
    r = capi.c_ser_reader(str(p))
    assert np.array_equal(r.read(80), fr)
    r.seek(3)
    stride = 512 * 1024 * 2 + 64
    buf = np.zeros(70 * stride, np.uint8)
    got = C.c_int()
    assert capi.lib().sst_ser_read(r.handle, 70, buf.ctypes.data, stride, C.byref(got)) == 0 and got.value == 70
    for k in (0, 33, 69):
        assert np.array_equal(buf[k * stride:k * stride + stride - 64].view(np.uint16).reshape(512, 1024), fr[3 + k])
    t = capi.c_ser_reader(str(write_ser(tmp_path / "l.ser", fr[:40], frames_count=80)))
    with pytest.raises(capi.SSTError):
        t.read(80)                                            # truncated: a piece past the end fails


def test_writer_round_trip_and_layout(capi, tmp_path):
    """c_ser_writer: the file equals the reference writer's layout (header with
    LittleEndian 0, FrameCount and DateTime of the first frame, frames, then
    the little-endian timestamps) and reads back exactly"""
    fr = _frames(4, 5, 7, np.uint16, 8)
    ts = np.array([5, 6, 7, 8], np.uint64) << np.uint64(33)
    w = capi.c_ser_writer(str(tmp_path / "w.ser"), 7, 5, 0, 12)
    w.write(fr[:1], ts[:1])
    w.write(fr[1:], ts[1:])
    w.close()
    want = write_ser(tmp_path / "ref.ser", fr, bits=12, timestamps=ts, date_time=int(ts[0]), date_time_utc=int(ts[0]))
    assert (tmp_path / "w.ser").read_bytes() == want.read_bytes()
    r = capi.c_ser_reader(str(tmp_path / "w.ser"))
    assert r.info.frames == 4 and np.array_equal(r.read(4), fr) and np.array_equal(r.timestamps(), ts)


def test_writer_defaults_and_checks(capi, tmp_path):
    rgb = _frames(2, 3, 4 * 3, np.uint8, 9).reshape(2, 3, 4, 3)
    w = capi.c_ser_writer(str(tmp_path / "x.ser"), 4, 3, 100, 8)
    w.write(rgb)                                   # no timestamps: UINT64_MAX each
    w.close()
    r = capi.c_ser_reader(str(tmp_path / "x.ser"))
    assert r.info.channels == 3 and np.array_equal(r.read(2), rgb)
    assert np.array_equal(r.timestamps(), np.full(2, np.iinfo(np.uint64).max, np.uint64))
    assert r.info.date_time == np.iinfo(np.uint64).max
    for args in ((0, 3, 0, 16), (4, 3, 5, 16), (4, 3, 0, 40)):
        with pytest.raises(capi.SSTError):
            capi.c_ser_writer(str(tmp_path / "y.ser"), *args)
