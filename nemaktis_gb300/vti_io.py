"""VTK XML ImageData (.vti) input and output without VTK, for the file-based entry of the
backend (the reference's `bpm-solver -x` command line).

Reading follows BeamPropagationSolver/src/UtilitiesLib/VTIReader.cpp:11-203:

* point arrays "n" (director, 3 components), "Q" (Q-tensor, 6 components: xx, yy, zz, xy,
  xz, yz) and "S" are looked up by name; a director field needs "n"; a Q-tensor field takes
  "Q" if present, else rebuilds Q from "n" (and "S" when present) with the reference's
  formulas (:142-199);
* the basis convention (XYZ, YZX, ZXY) permutes the mesh axes and the vector components
  (:83-99, 103-126);
* a NaN in the director is an error (:113-124).

The reader accepts what VTK's XML writers produce: inline ascii, inline binary (base64) and
appended data (raw or base64), UInt32 or UInt64 block headers, little- or big-endian, and
zlib-compressed blocks (vtkZLibDataCompressor).
"""
import base64
import re
import struct
import xml.etree.ElementTree as ET
import zlib

import numpy as np

_DT = {"Float64": "f8", "Float32": "f4", "Int8": "i1", "UInt8": "u1", "Int16": "i2", "UInt16": "u2",
       "Int32": "i4", "UInt32": "u4", "Int64": "i8", "UInt64": "u8"}


class VtiError(ValueError):
    pass


def _split_appended(raw):
    """Header XML text and the appended payload (bytes after the '_' marker)."""
    tag = b"<AppendedData"
    i = raw.find(tag)
    if i < 0:
        return raw, None, None
    j = raw.index(b">", i) + 1
    enc = re.search(rb'encoding="(\w+)"', raw[i:j])
    k = raw.index(b"_", j) + 1
    end = raw.rfind(b"</AppendedData>")
    payload = raw[k:end]
    head = raw[:i] + b"<AppendedData/>" + raw[end + len(b"</AppendedData>"):]
    return head, payload, (enc.group(1).decode() if enc else "raw")


def _decode_block(buf, dtype, header, compressed, base64_encoded):
    """Data bytes of one DataArray given its encoded bytes (with VTK's size headers)."""
    ht = np.dtype(header)
    if base64_encoded:
        if compressed:
            # header block first (base64 of its own), then the compressed blocks
            hb = base64.b64decode(buf[: _b64len(3 * ht.itemsize)])
            nb = int(np.frombuffer(hb[: ht.itemsize], ht)[0])
            hlen = (3 + nb) * ht.itemsize
            hb = base64.b64decode(buf[: _b64len(hlen)])
            data = base64.b64decode(buf[_b64len(hlen):].strip())
            return _inflate(np.frombuffer(hb, ht), data, ht)
        b = base64.b64decode(buf.strip())
        n = int(np.frombuffer(b[: ht.itemsize], ht)[0])
        return b[ht.itemsize: ht.itemsize + n]
    if compressed:
        nb = int(np.frombuffer(buf[: ht.itemsize], ht)[0])
        hdr = np.frombuffer(buf[: (3 + nb) * ht.itemsize], ht)
        return _inflate(hdr, buf[(3 + nb) * ht.itemsize:], ht)
    n = int(np.frombuffer(buf[: ht.itemsize], ht)[0])
    return buf[ht.itemsize: ht.itemsize + n]


def _b64len(n):
    return 4 * ((n + 2) // 3)


def _inflate(hdr, data, ht):
    nb = int(hdr[0])
    sizes = [int(v) for v in hdr[3: 3 + nb]]
    out, o = [], 0
    for s in sizes:
        out.append(zlib.decompress(data[o: o + s]))
        o += s
    return b"".join(out)


def read_vti(path):
    """{"dims": (nx, ny, nz), "spacing", "origin", "point": {name: array (n, ncomp)},
    "field": {name: array}} of a .vti file."""
    raw = open(path, "rb").read()
    head, payload, enc = _split_appended(raw)
    try:
        root = ET.fromstring(head)
    except ET.ParseError as e:
        raise VtiError("not a VTK XML file: %s" % e)
    if root.tag != "VTKFile" or root.get("type") != "ImageData":
        raise VtiError("not a VTK ImageData file")
    big = root.get("byte_order", "LittleEndian") == "BigEndian"
    header = {"UInt32": "u4", "UInt64": "u8"}[root.get("header_type", "UInt32")]
    header = (">" if big else "<") + header
    compressed = root.get("compressor") is not None
    img = root.find("ImageData")
    ext = [int(v) for v in img.get("WholeExtent").split()]
    dims = (ext[1] - ext[0] + 1, ext[3] - ext[2] + 1, ext[5] - ext[4] + 1)
    spacing = tuple(float(v) for v in img.get("Spacing", "1 1 1").split())
    origin = tuple(float(v) for v in img.get("Origin", "0 0 0").split())

    def read_array(da):
        dt = np.dtype((">" if big else "<") + _DT[da.get("type")])
        nc = int(da.get("NumberOfComponents", "1"))
        fmt = da.get("format")
        if fmt == "ascii":
            a = np.array((da.text or "").split(), dtype=dt)
        elif fmt == "binary":
            a = np.frombuffer(_decode_block(da.text.strip().encode(), dt, header, compressed, True), dt)
        elif fmt == "appended":
            if payload is None:
                raise VtiError("appended array without AppendedData")
            off = int(da.get("offset"))
            a = np.frombuffer(_decode_block(payload[off:], dt, header, compressed, enc == "base64"), dt)
        else:
            raise VtiError("unknown DataArray format %r" % fmt)
        a = a.astype(np.float64)
        return a.reshape(-1, nc) if nc > 1 else a

    out = {"dims": dims, "spacing": spacing, "origin": origin, "point": {}, "field": {}}
    fd = img.find("FieldData")
    if fd is not None:
        for da in fd.findall("DataArray"):
            out["field"][da.get("Name")] = read_array(da)
    piece = img.find("Piece")
    pd = piece.find("PointData") if piece is not None else None
    if pd is not None:
        for da in pd.findall("DataArray"):
            out["point"][da.get("Name")] = read_array(da)
    return out


_PERM = {"XYZ": (0, 1, 2), "YZX": (1, 2, 0), "ZXY": (2, 0, 1)}


def lc_field_from_vti(path, lc_dim, basis="XYZ"):
    """(values (Nz, Ny, Nx, lc_dim) in the backend's layout, dims (Nx, Ny, Nz), spacings) of an
    LC field file, as VTIReader::fill_solution_vector builds it (VTIReader.cpp:77-203)."""
    import os
    if not os.path.exists(path):
        raise VtiError("The given input vti file does not exists")
    d = read_vti(path)
    pts = d["point"]
    if lc_dim == 3 and "n" not in pts:
        raise VtiError('Could not find the director array "n" in the given vti file')
    if lc_dim == 6 and "Q" not in pts and "n" not in pts:
        raise VtiError('Could not find the director array "n" in the given vti file')
    I = _PERM[basis]
    dim = d["dims"]
    odims = (dim[I[0]], dim[I[1]], dim[I[2]])
    ospac = (d["spacing"][I[0]], d["spacing"][I[1]], d["spacing"][I[2]])
    # input point index i_in = ix + dim0*(iy + dim1*iz); output index follows the permuted axes
    shape_in = (dim[2], dim[1], dim[0])  # (iz, iy, ix)

    def to_out(a, nc):
        a = a.reshape(shape_in + (nc,))           # [iz][iy][ix][c]
        axes_in = {0: 2, 1: 1, 2: 0}              # mesh axis -> array axis of a
        # output array [k3][k2][k1][c] with k1 along input axis I1, k2 along I2, k3 along I3
        return np.ascontiguousarray(np.transpose(a, (axes_in[I[2]], axes_in[I[1]], axes_in[I[0]], 3)))

    if lc_dim == 3:
        n = pts["n"]
        if np.isnan(n).any():
            raise VtiError("Error: NaN value in the given vti file")
        vals = to_out(n[:, list(I)], 3)
    elif "Q" in pts:
        vals = to_out(pts["Q"], 6)
    else:
        n = pts["n"]
        f = 1 - pts["S"].reshape(-1) if "S" in pts else np.ones(len(n))
        q = np.stack([0.5 * f * (3 * n[:, 0] ** 2 - 1), 0.5 * f * (3 * n[:, 1] ** 2 - 1), 0.5 * f * (3 * n[:, 2] ** 2 - 1),
                      1.5 * f * n[:, 0] * n[:, 1], 1.5 * f * n[:, 0] * n[:, 2], 1.5 * f * n[:, 1] * n[:, 2]], axis=1)
        vals = to_out(q, 6)
    return vals, odims, ospac


def write_vti(path, dims, spacing, origin, point=(), field=()):
    """Writes a VTK XML ImageData file with raw appended Float64 arrays (UInt64 headers).
    point / field: sequences of (name, array (n, ncomp) or (n,))."""
    parts, decl_f, decl_p, off = [], [], [], 0

    def decl(name, a, indent):
        nonlocal off
        a = np.ascontiguousarray(np.asarray(a, np.float64))
        nc = a.shape[1] if a.ndim > 1 else 1
        s = '%s<DataArray type="Float64" Name="%s" NumberOfComponents="%d" format="appended" offset="%d"/>\n' % (
            indent, name, nc, off)
        b = a.tobytes()
        parts.append(struct.pack("<Q", len(b)) + b)
        off += 8 + len(b)
        return s

    for name, a in field:
        decl_f.append(decl(name, a, "      "))
    for name, a in point:
        decl_p.append(decl(name, a, "        "))
    ext = "0 %d 0 %d 0 %d" % (dims[0] - 1, dims[1] - 1, dims[2] - 1)
    head = ('<?xml version="1.0"?>\n<VTKFile type="ImageData" version="1.0" byte_order="LittleEndian" '
            'header_type="UInt64">\n  <ImageData WholeExtent="%s" Origin="%r %r %r" Spacing="%r %r %r">\n'
            % (ext, *[float(v) for v in origin], *[float(v) for v in spacing]))
    head += "    <FieldData>\n" + "".join(decl_f) + "    </FieldData>\n"
    head += '    <Piece Extent="%s">\n      <PointData>\n' % ext + "".join(decl_p)
    head += "      </PointData>\n      <CellData>\n      </CellData>\n    </Piece>\n  </ImageData>\n"
    head += '  <AppendedData encoding="raw">\n   _'
    with open(path, "wb") as f:
        f.write(head.encode())
        for p in parts:
            f.write(p)
        f.write(b"\n  </AppendedData>\n</VTKFile>\n")
