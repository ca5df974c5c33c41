"""MRC2014 reading and writing of result maps (no third-party dependency).

Leopard-EM writes its search results with ``mrcfile`` (utils/data_io.py:50-160,
``write_mrc_from_tensor``: ``mrcfile.new(path, overwrite)`` then
``set_data``).  This module writes the same files: a 1024-byte MRC2014 header
(dimensions, mode from the dtype, sampling = dimensions, unit cell angles 90,
axis order 1 2 3, data min / max / mean / rms, space group 0 for images and 1
for volumes, 'MAP ' stamp, little-endian machine stamp, version 20141, no
extended header) followed by the data in C order (x fastest).
"""

from __future__ import annotations

import os
import struct

import numpy as np

HEADER_BYTES = 1024
_MODES = {np.dtype(np.int8): 0, np.dtype(np.int16): 1, np.dtype(np.float32): 2, np.dtype(np.complex64): 4,
          np.dtype(np.uint16): 6, np.dtype(np.float16): 12}
_DTYPES = {v: k for k, v in _MODES.items()}


def _as_numpy(data) -> np.ndarray:
    if hasattr(data, "detach"):  # torch tensor
        data = data.detach().cpu().numpy()
    arr = np.ascontiguousarray(data)
    if arr.dtype == np.float64:
        arr = arr.astype(np.float32)
    if arr.dtype not in _MODES:
        raise ValueError(f"dtype {arr.dtype} has no MRC mode")
    if arr.ndim not in (2, 3):
        raise ValueError("MRC data must be 2-D (an image) or 3-D (a volume or stack)")
    return arr.astype(arr.dtype.newbyteorder("<"), copy=False)


def mrc_header(arr: np.ndarray, voxel_size: float = 0.0) -> bytes:
    """The 1024-byte MRC2014 header describing ``arr`` (2-D or 3-D)."""
    nz, ny, nx = (1,) + arr.shape if arr.ndim == 2 else arr.shape
    h = bytearray(HEADER_BYTES)
    real = arr.real.astype(np.float64) if np.iscomplexobj(arr) else arr.astype(np.float64)
    struct.pack_into("<3i", h, 0, nx, ny, nz)
    struct.pack_into("<i", h, 12, _MODES[arr.dtype.newbyteorder("=")])
    struct.pack_into("<3i", h, 16, 0, 0, 0)                       # nxstart, nystart, nzstart
    struct.pack_into("<3i", h, 28, nx, ny, nz)                    # mx, my, mz
    struct.pack_into("<3f", h, 40, nx * voxel_size, ny * voxel_size, nz * voxel_size)  # cell lengths
    struct.pack_into("<3f", h, 52, 90.0, 90.0, 90.0)              # cell angles
    struct.pack_into("<3i", h, 64, 1, 2, 3)                       # mapc, mapr, maps
    struct.pack_into("<3f", h, 76, real.min(), real.max(), real.mean())  # dmin, dmax, dmean
    struct.pack_into("<i", h, 88, 0 if arr.ndim == 2 else 1)      # ispg
    struct.pack_into("<i", h, 92, 0)                              # nsymbt (no extended header)
    h[104:108] = b"MRCO"                                          # exttyp
    struct.pack_into("<i", h, 108, 20141)                         # nversion
    struct.pack_into("<3f", h, 196, 0.0, 0.0, 0.0)                # origin
    h[208:212] = b"MAP "
    h[212:216] = bytes([0x44, 0x44, 0x00, 0x00])                  # little-endian machine stamp
    struct.pack_into("<f", h, 216, real.std())                    # rms
    struct.pack_into("<i", h, 220, 0)                             # nlabl
    return bytes(h)


def write_mrc(path, data, voxel_size: float = 0.0, overwrite: bool = False) -> None:
    """Write a 2-D or 3-D array (numpy or torch) as an MRC2014 file."""
    if os.path.exists(path) and not overwrite:
        raise FileExistsError(f"{path} exists (overwrite=False)")
    arr = _as_numpy(data)
    with open(path, "wb") as f:
        f.write(mrc_header(arr, voxel_size))
        f.write(arr.tobytes(order="C"))


def read_mrc(path) -> np.ndarray:
    """Data of an MRC2014 file (modes 0, 1, 2, 4, 6, 12) as a numpy array,
    shape (ny, nx) for nz = 1 else (nz, ny, nx)."""
    with open(path, "rb") as f:
        head = f.read(HEADER_BYTES)
        if len(head) < HEADER_BYTES or head[208:212] != b"MAP ":
            raise ValueError(f"{path} is not an MRC2014 file")
        little = head[212] == 0x44
        e = "<" if little else ">"
        nx, ny, nz = struct.unpack_from(e + "3i", head, 0)
        mode = struct.unpack_from(e + "i", head, 12)[0]
        next_bytes = struct.unpack_from(e + "i", head, 92)[0]
        if mode not in _DTYPES:
            raise ValueError(f"MRC mode {mode} is not supported")
        f.seek(HEADER_BYTES + next_bytes)
        dt = _DTYPES[mode].newbyteorder(e)
        data = np.fromfile(f, dtype=dt, count=nx * ny * nz)
    if data.size != nx * ny * nz:
        raise ValueError(f"{path}: truncated data")
    data = data.astype(dt.newbyteorder("="))
    return data.reshape(ny, nx) if nz == 1 else data.reshape(nz, ny, nx)
