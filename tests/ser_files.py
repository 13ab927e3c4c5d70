"""Writes SER v3 files for the tests: the 178-byte LUCAM-RECORDER header
(little-endian fields), the frames, and an optional trailer of 64-bit
timestamps. `le_field` is the header's LittleEndian field as stored; the
reader takes 0 to mean little-endian pixel data (the reference's reading), so
frames are written big-endian when le_field != 0."""
import struct

import numpy as np


def write_ser(path, frames, color_id=0, bits=16, le_field=0, timestamps=None, frames_count=None, luid=0,
              observer=b"", instrument=b"", telescope=b"", date_time=0, date_time_utc=0, magic=b"LUCAM-RECORDER"):
    frames = np.asarray(frames)
    n, h, w = frames.shape[:3]
    count = n if frames_count is None else frames_count
    head = struct.pack("<14s7i40s40s40sQQ", magic, luid, color_id, le_field, w, h, bits, count,
                       observer, instrument, telescope, date_time, date_time_utc)
    assert len(head) == 178
    data = frames.astype(frames.dtype.newbyteorder(">" if le_field else "<"))
    with open(path, "wb") as f:
        f.write(head)
        f.write(data.tobytes())
        if timestamps is not None:
            ts = np.asarray(timestamps, np.uint64).astype(">u8" if le_field else "<u8")
            f.write(ts.tobytes())
    return path
