"""Minimal reader of VTK XML ImageData files with raw appended Float64 arrays (the bulk-output
files the backend writes), for the tests."""
import re

import numpy as np


def read_vti(path):
    raw = open(path, "rb").read()
    head, _, rest = raw.partition(b"<AppendedData encoding=\"raw\">")
    start = rest.index(b"_") + 1
    blob = rest[start:]
    text = head.decode()
    hdr = "UInt64" if 'header_type="UInt64"' in text else "UInt32"
    ht = np.uint64 if hdr == "UInt64" else np.uint32
    hs = np.dtype(ht).itemsize
    m = re.search(r'WholeExtent="([^"]+)"', text)
    ext = [int(v) for v in m.group(1).split()]
    dims = (ext[1] - ext[0] + 1, ext[3] - ext[2] + 1, ext[5] - ext[4] + 1)
    info = {k: [float(v) for v in re.search(k + r'="([^"]+)"', text).group(1).split()] for k in ("Origin", "Spacing")}
    arrays = {}
    for a in re.finditer(r'<DataArray ([^>]*)/>', text):
        attrs = dict(re.findall(r'(\w+)="([^"]*)"', a.group(1)))
        off = int(attrs["offset"])
        nb = int(np.frombuffer(blob[off:off + hs], ht)[0])
        data = np.frombuffer(blob[off + hs:off + hs + nb], np.float64)
        nc = int(attrs.get("NumberOfComponents", "1"))
        arrays[attrs["Name"]] = data.reshape(-1, nc) if nc > 1 else data
    return {"dims": dims, "origin": info["Origin"], "spacing": info["Spacing"], "arrays": arrays}
