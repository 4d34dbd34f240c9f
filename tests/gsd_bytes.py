"""Builds GSD files byte by byte for the reader tests (published GSD file-layer
layout: 256-byte header, 32-byte index entries, the name list, then chunk data),
in file-layer 1.0 (64-byte name entries) or 2.0 (packed zero-terminated names)."""

import struct

import numpy as np

MAGIC = 0x65DF65DF65DF65DF
TYPE_IDS = {np.dtype("u1"): 1, np.dtype("u2"): 2, np.dtype("u4"): 3, np.dtype("u8"): 4, np.dtype("i1"): 5,
            np.dtype("i2"): 6, np.dtype("i4"): 7, np.dtype("i8"): 8, np.dtype("f4"): 9, np.dtype("f8"): 10}


def gsd_bytes(frames, version=2, schema=b"hoomd", magic=MAGIC):
    """frames: list of {name: array} (a 1-D array is one column). Returns bytes."""
    names = []
    for fr in frames:
        for nm in fr:
            if nm not in names:
                names.append(nm)
    entries = []
    data = b""
    n_index = max(1, sum(len(fr) for fr in frames))
    n_names = max(16, len(names))
    index_loc = 256
    names_loc = index_loc + 32 * n_index
    data_loc = names_loc + 64 * n_names
    for f, fr in enumerate(frames):
        for nm, arr in fr.items():
            a = np.ascontiguousarray(arr)
            a2 = a.reshape(len(a), -1) if a.ndim > 1 else a.reshape(-1, 1)
            entries.append(struct.pack("<QQqIHBB", f, a2.shape[0], data_loc + len(data), a2.shape[1],
                                       names.index(nm), TYPE_IDS[a.dtype], 0))
            data += a.tobytes()
    index = b"".join(entries).ljust(32 * n_index, b"\0")
    if version == 1:
        namelist = b"".join(nm.encode().ljust(64, b"\0") for nm in names).ljust(64 * n_names, b"\0")
        gsd_version = 1 << 16
    else:
        namelist = b"".join(nm.encode() + b"\0" for nm in names).ljust(64 * n_names, b"\0")
        gsd_version = 2 << 16
    header = struct.pack("<QQQQQII64s64s80s", magic, index_loc, n_index, names_loc, n_names, (1 << 16) | 4,
                         gsd_version, b"tests", schema, b"")
    return header + index + namelist + data


def trajectory_bytes(boxes, positions, dims=3, version=2):
    """HOOMD-schema frames with configuration/box, configuration/dimensions
    (frame 0 only), configuration/step, particles/N and particles/position."""
    frames = []
    for f, (b, p) in enumerate(zip(boxes, positions)):
        fr = {"configuration/step": np.array([1000 * f], np.uint64),
              "configuration/box": np.asarray(b, np.float32)[:6],
              "particles/N": np.array([len(p)], np.uint32),
              "particles/position": np.asarray(p, np.float32)}
        if f == 0:
            fr["configuration/dimensions"] = np.array([dims], np.uint8)
        frames.append(fr)
    return gsd_bytes(frames, version=version)
