"""Writes minimal NIfTI-1 files for the ingest and command-line tests: a
352-byte header read the way the reference reads it (shorts: dim[0..7] at
20..27, datatype at 35, bitpix at 36), then the voxel data."""
import numpy as np


def write_nifti(path, data, datatype):
    """data: [T][Z][Y][X] (or [Z][Y][X]) array; datatype 2 (uint8), 16
    (float32) or 64 (float64)."""
    data = np.asarray(data)
    if data.ndim == 3:
        data = data[None]
    T, Z, Y, X = data.shape
    hdr = np.zeros(176, np.int16)
    hdr[0] = 348          # sizeof_hdr (low half of the int32 at byte 0)
    hdr[20] = 4 if T > 1 else 3
    hdr[21], hdr[22], hdr[23], hdr[24] = X, Y, Z, T
    dt = {2: np.uint8, 16: np.float32, 64: np.float64}[datatype]
    hdr[35] = datatype
    hdr[36] = np.dtype(dt).itemsize * 8
    raw = hdr.tobytes()
    raw = raw[:108] + np.float32(352.0).tobytes() + raw[112:]  # vox_offset
    with open(path, "wb") as f:
        f.write(raw)
        f.write(np.ascontiguousarray(data, dtype=dt).tobytes())
