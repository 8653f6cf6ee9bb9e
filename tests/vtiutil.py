"""Minimal reader/writer for VTK XML ImageData (.vti) files, test helper.

Supports what the NS3D files use: one DataArray, "appended" data encoded in
base64 or raw, optional vtkZLibDataCompressor blocks, UInt32 or UInt64
headers, little endian.  Returns numpy arrays in C order (x, y, z) with z
fastest, the axis order of the solver's index maps.
"""
import base64
import re
import struct
import zlib

import numpy as np

_TYPES = {"UInt8": np.uint8, "Int8": np.int8, "UInt16": np.uint16, "Int16": np.int16,
          "UInt32": np.uint32, "Int32": np.int32, "Float32": np.float32, "Float64": np.float64,
          "UInt64": np.uint64, "Int64": np.int64}


def _attr(tag, name, default=None):
    m = re.search(r'\b%s="([^"]*)"' % name, tag)
    return m.group(1) if m else default


def read_vti(path):
    """Return (array, ncomp); array shape (nx, ny, nz) or (nx, ny, nz, ncomp)."""
    data = open(path, "rb").read()
    head_end = data.find(b"<AppendedData")
    head = data[:head_end if head_end >= 0 else len(data)].decode("latin-1")
    vtk = re.search(r"<VTKFile[^>]*>", head).group(0)
    hdr_t = _attr(vtk, "header_type", "UInt32")
    hfmt, hsize = ("<I", 4) if hdr_t == "UInt32" else ("<Q", 8)
    compressed = _attr(vtk, "compressor") is not None
    ext = [int(v) for v in _attr(re.search(r"<ImageData[^>]*>", head).group(0), "WholeExtent").split()]
    dims = (ext[1] - ext[0] + 1, ext[3] - ext[2] + 1, ext[5] - ext[4] + 1)
    darr = re.search(r"<DataArray[^>]*>", head).group(0)
    dtype = _TYPES[_attr(darr, "type")]
    ncomp = int(_attr(darr, "NumberOfComponents", "1"))
    offset = int(_attr(darr, "offset", "0"))
    app = data[head_end:]
    enc = _attr(app[:200].decode("latin-1"), "encoding", "base64")
    start = app.find(b"_") + 1
    body = app[start:]
    body = body[:body.rfind(b"</AppendedData>")].rstrip()
    nbytes_total = dims[0] * dims[1] * dims[2] * ncomp * np.dtype(dtype).itemsize
    if enc == "base64":
        body = body[offset:]
        if compressed:
            # header: [nblocks, blocksize, lastsize, csize...]
            nblocks = struct.unpack(hfmt, base64.b64decode(body[:((3 * hsize + 2) // 3) * 4])[:hsize])[0]
            hlen = (3 + nblocks) * hsize
            henc = ((hlen + 2) // 3) * 4
            hdr = base64.b64decode(body[:henc])[:hlen]
            vals = struct.unpack("<" + hfmt[1] * (3 + nblocks), hdr)
            csizes = vals[3:]
            raw = base64.b64decode(body[henc:henc + ((sum(csizes) + 2) // 3) * 4])
            out, pos = [], 0
            for cs in csizes:
                out.append(zlib.decompress(raw[pos:pos + cs]))
                pos += cs
            buf = b"".join(out)
        else:
            raw = base64.b64decode(body[:((hsize + nbytes_total + 2) // 3) * 4])
            buf = raw[hsize:hsize + nbytes_total]
    else:
        raise NotImplementedError("raw appended encoding")
    arr = np.frombuffer(buf[:nbytes_total], dtype=dtype)
    if ncomp == 1:
        arr = arr.reshape(dims[2], dims[1], dims[0]).transpose(2, 1, 0)
    else:
        arr = arr.reshape(dims[2], dims[1], dims[0], ncomp).transpose(2, 1, 0, 3)
    return np.ascontiguousarray(arr), ncomp


def read_raw_xfastest(path):
    """Voxel buffer in file order (x fastest) and dims (nx, ny, nz)."""
    arr, _ = read_vti(path)
    nx, ny, nz = arr.shape[:3]
    return np.ascontiguousarray(arr.transpose(2, 1, 0)).reshape(-1), (nx, ny, nz)
