"""Reader for HOOMD-schema GSD trajectories, the format of the reference's
trajectory fixtures, feeding ``(box, points)`` frames and ``FrameBatch``.

Written from the published GSD file-layer description (GSD 1.x and 2.x files):

* a 256-byte header: magic 0x65DF65DF65DF65DF, index location and allocated
  entries, name-list location and allocated entries, schema version, file-layer
  version, 64-byte application and schema strings;
* the index: 32-byte entries (frame u64, N u64, location i64, M u32, id u16,
  type u8, flags u8); entries with location 0 are unused, and a chunk's data is
  N x M elements of its type at its location;
* the name list: file layer 1.x stores 64-byte zero-padded names, 2.x a buffer of
  ``allocated entries`` x 64 bytes holding zero-terminated names one after
  another; a chunk's id is its name's position in the list.

HOOMD schema rules used here: ``configuration/box`` is (Lx, Ly, Lz, xy, xz, yz),
``configuration/dimensions`` 2 or 3, ``particles/position`` (N, 3) float32; a
chunk missing from frame f takes its frame-0 value, and one missing from frame 0
too takes the schema default (box 1, 1, 1, 0, 0, 0; dimensions 3; N 0).

The reference reads these files through the ``gsd`` package in its tests
(tests/integration/test_reader_integrations.py:55-57,
tests/validation/test_steinhardt_average.py:14-22) and accepts its frames as
systems (freud/locality.py:327-336); ``Frame`` here has the same attribute paths
(``configuration.box``, ``configuration.dimensions``, ``particles.position``).
"""

import builtins
import mmap
import struct

import numpy as np

__all__ = ["Frame", "HOOMDTrajectory", "open"]

_MAGIC = 0x65DF65DF65DF65DF
_HEADER = struct.Struct("<QQQQQII64s64s80s")
_ENTRY = np.dtype([("frame", "<u8"), ("N", "<u8"), ("location", "<i8"), ("M", "<u4"), ("id", "<u2"),
                   ("type", "u1"), ("flags", "u1")])
_NAME_SIZE = 64
_TYPES = {1: "<u1", 2: "<u2", 3: "<u4", 4: "<u8", 5: "<i1", 6: "<i2", 7: "<i4", 8: "<i8", 9: "<f4", 10: "<f8",
          11: "<u1"}
_DEFAULTS = {
    "configuration/box": np.array([1, 1, 1, 0, 0, 0], dtype=np.float32),
    "configuration/dimensions": np.uint8(3),
    "configuration/step": np.uint64(0),
    "particles/N": np.uint32(0),
}


class _Section:
    pass


class Frame:
    """One trajectory frame: ``configuration.box`` (6 floats),
    ``configuration.dimensions``, ``configuration.step``, ``particles.N`` and
    ``particles.position`` ((N, 3) float32)."""

    def __init__(self, box, dimensions, step, position):
        self.configuration = _Section()
        self.configuration.box = np.asarray(box, dtype=np.float32)
        self.configuration.dimensions = int(dimensions)
        self.configuration.step = int(step)
        self.particles = _Section()
        self.particles.position = np.ascontiguousarray(position, dtype=np.float32).reshape(-1, 3)
        self.particles.N = len(self.particles.position)

    def system(self):
        """The frame as a ``(box, points)`` system (2D frames zero Lz, xz, yz as
        the reference does for gsd frames, freud/locality.py:327-336)."""
        box = np.array(self.configuration.box, dtype=np.float64)
        if self.configuration.dimensions == 2:
            box[[2, 4, 5]] = 0
        return box, self.particles.position


class HOOMDTrajectory:
    """The frames of one GSD file (read-only, random access, ``len``, iteration)."""

    def __init__(self, path):
        with builtins.open(path, "rb") as fh:
            try:
                self._buf = mmap.mmap(fh.fileno(), 0, access=mmap.ACCESS_READ)
            except ValueError as err:  # empty file
                raise RuntimeError(f"{path}: not a GSD file (empty)") from err
        size = len(self._buf)
        if size < _HEADER.size:
            raise RuntimeError(f"{path}: not a GSD file (shorter than the header)")
        (magic, index_loc, index_n, names_loc, names_n, schema_version, gsd_version, _app, schema,
         _reserved) = _HEADER.unpack_from(self._buf, 0)
        if magic != _MAGIC:
            raise RuntimeError(f"{path}: not a GSD file (bad magic number)")
        major = gsd_version >> 16
        if major not in (1, 2):
            raise RuntimeError(f"{path}: GSD file layer version {major} is not supported")
        schema = schema.split(b"\0")[0]
        if schema != b"hoomd":
            raise RuntimeError(f"{path}: schema {schema!r} is not the HOOMD schema")
        self.schema_version = (schema_version >> 16, schema_version & 0xFFFF)
        self.gsd_version = (major, gsd_version & 0xFFFF)
        if index_loc + index_n * _ENTRY.itemsize > size or names_loc + names_n * _NAME_SIZE > size:
            raise RuntimeError(f"{path}: truncated GSD file (index or name list past the end)")

        raw_names = bytes(self._buf[names_loc:names_loc + names_n * _NAME_SIZE])
        if major == 1:
            names = [raw_names[k * _NAME_SIZE:(k + 1) * _NAME_SIZE].split(b"\0")[0] for k in range(names_n)]
        else:
            names = raw_names.split(b"\0")
        self._names = []
        for nm in names:
            if not nm:
                break
            self._names.append(nm.decode("ascii"))

        index = np.frombuffer(self._buf, dtype=_ENTRY, count=index_n, offset=index_loc)
        index = index[index["location"] != 0]
        self._chunks = {}
        for e in index:
            kind = int(e["type"])
            ident = int(e["id"])
            if kind not in _TYPES or ident >= len(self._names):
                raise RuntimeError(f"{path}: bad index entry (type {kind}, id {ident})")
            n, m, loc = int(e["N"]), int(e["M"]), int(e["location"])
            nbytes = n * m * np.dtype(_TYPES[kind]).itemsize
            if loc < 0 or loc + nbytes > size:
                raise RuntimeError(f"{path}: chunk {self._names[ident]} of frame {int(e['frame'])} past the end")
            self._chunks[(int(e["frame"]), self._names[ident])] = (kind, n, m, loc)
        self._nframes = int(index["frame"].max()) + 1 if len(index) else 0
        self._path = path

    def close(self):
        if self._buf is not None:
            self._buf.close()
            self._buf = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __len__(self):
        return self._nframes

    @property
    def names(self):
        """Chunk names in the file's name list."""
        return list(self._names)

    def read_chunk(self, frame, name):
        """The data of chunk ``name`` in ``frame`` as an (N, M) array (a copy), or
        None when that frame does not hold it."""
        ent = self._chunks.get((frame, name))
        if ent is None:
            return None
        kind, n, m, loc = ent
        arr = np.frombuffer(self._buf, dtype=_TYPES[kind], count=n * m, offset=loc)
        return arr.reshape(n, m).copy() if m > 1 else arr.copy()

    def _value(self, frame, name):
        v = self.read_chunk(frame, name)
        if v is None and frame != 0:
            v = self.read_chunk(0, name)
        if v is None:
            return _DEFAULTS.get(name)
        return v

    def __getitem__(self, f):
        if isinstance(f, slice):
            return [self[k] for k in range(*f.indices(len(self)))]
        if f < 0:
            f += len(self)
        if not 0 <= f < len(self):
            raise IndexError(f"frame {f} out of range for {len(self)} frames")
        box = self._value(f, "configuration/box")
        dims = self._value(f, "configuration/dimensions")
        step = self._value(f, "configuration/step")
        n = int(np.asarray(self._value(f, "particles/N")).reshape(-1)[0])
        pos = self._value(f, "particles/position")
        if pos is None:
            pos = np.zeros((n, 3), dtype=np.float32)
        pos = np.asarray(pos, dtype=np.float32).reshape(-1, 3)
        if len(pos) != n:
            raise RuntimeError(f"{self._path}: frame {f} has {len(pos)} positions for N = {n}")
        return Frame(np.asarray(box).reshape(-1), np.asarray(dims).reshape(-1)[0], np.asarray(step).reshape(-1)[0],
                     pos)

    def __iter__(self):
        for f in range(len(self)):
            yield self[f]


def open(path, mode="rb"):  # noqa: A001 - the gsd.hoomd.open name
    """Open a HOOMD-schema GSD file for reading (the ``gsd.hoomd.open`` call of
    the reference's tests; only read modes)."""
    if mode not in ("rb", "r"):
        raise ValueError("only reading is supported")
    return HOOMDTrajectory(path)
