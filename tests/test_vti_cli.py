"""LC-field .vti reading (VTIReader.cpp semantics) and the file-based command line (bpm-solver -x):
reader formats and basis conventions on the CPU, the command line against a direct backend call
on the GPU."""
import base64
import json
import os
import struct
import zlib

import numpy as np
import pytest

from nemaktis_gb300 import vti_io, workloads


def _vti_bytes(dims, arrays, mode="raw", header="UInt64", compress=False):
    """A .vti file in one of VTK's XML encodings (written here independently of vti_io)."""
    hfmt = {"UInt64": "<Q", "UInt32": "<I"}[header]
    decls, blobs, off = [], [], 0
    for name, a in arrays:
        a = np.ascontiguousarray(np.asarray(a, np.float64))
        nc = a.shape[1] if a.ndim > 1 else 1
        raw = a.tobytes()
        if compress:
            comp = zlib.compress(raw)
            head = struct.pack(hfmt, 1) + struct.pack(hfmt, len(raw)) + struct.pack(hfmt, len(raw)) + \
                struct.pack(hfmt, len(comp))
            body = head + comp if mode != "base64" else base64.b64encode(head) + base64.b64encode(comp)
        else:
            body = struct.pack(hfmt, len(raw)) + raw
            if mode == "base64":
                body = base64.b64encode(body)
        if mode == "ascii":
            decls.append('<DataArray type="Float64" Name="%s" NumberOfComponents="%d" format="ascii">%s</DataArray>'
                         % (name, nc, " ".join(repr(float(v)) for v in a.ravel())))
        elif mode == "binary":
            decls.append('<DataArray type="Float64" Name="%s" NumberOfComponents="%d" format="binary">%s</DataArray>'
                         % (name, nc, base64.b64encode(struct.pack(hfmt, len(raw)) + raw).decode()))
        else:
            decls.append('<DataArray type="Float64" Name="%s" NumberOfComponents="%d" format="appended" offset="%d"/>'
                         % (name, nc, off))
            blobs.append(body)
            off += len(body)
    comp_attr = ' compressor="vtkZLibDataCompressor"' if compress else ""
    ext = "0 %d 0 %d 0 %d" % (dims[0] - 1, dims[1] - 1, dims[2] - 1)
    x = ('<?xml version="1.0"?>\n<VTKFile type="ImageData" version="1.0" byte_order="LittleEndian" '
         'header_type="%s"%s>\n<ImageData WholeExtent="%s" Origin="0 0 0" Spacing="0.2 0.3 0.4">\n'
         '<Piece Extent="%s"><PointData>%s</PointData><CellData></CellData></Piece>\n</ImageData>\n'
         % (header, comp_attr, ext, ext, "".join(decls)))
    if blobs:
        x = x.encode() + ('<AppendedData encoding="%s">\n_' % ("base64" if mode == "base64" else "raw")).encode() + \
            b"".join(blobs) + b"\n</AppendedData>\n</VTKFile>\n"
    else:
        x = (x + "</VTKFile>\n").encode()
    return x


def _director(dims, seed=0):
    rng = np.random.default_rng(seed)
    n = rng.normal(size=(dims[2] * dims[1] * dims[0], 3))
    return n / np.linalg.norm(n, axis=1, keepdims=True)


@pytest.mark.parametrize("mode,header,compress", [("raw", "UInt64", False), ("raw", "UInt32", False),
                                                  ("base64", "UInt32", False), ("base64", "UInt64", True),
                                                  ("raw", "UInt64", True), ("ascii", "UInt32", False),
                                                  ("binary", "UInt32", False)])
def test_reader_formats(tmp_path, mode, header, compress):
    dims = (5, 4, 3)
    n = _director(dims)
    S = np.linspace(0, 0.5, len(n))
    p = tmp_path / "f.vti"
    p.write_bytes(_vti_bytes(dims, [("n", n), ("S", S)], mode, header, compress))
    d = vti_io.read_vti(str(p))
    assert d["dims"] == dims
    np.testing.assert_allclose(d["spacing"], (0.2, 0.3, 0.4))
    np.testing.assert_array_equal(d["point"]["n"], n)
    np.testing.assert_array_equal(d["point"]["S"], S)


@pytest.mark.parametrize("basis", ["XYZ", "YZX", "ZXY"])
def test_basis_conventions(tmp_path, basis):
    dims = (5, 4, 3)
    n = _director(dims, 1)
    p = tmp_path / "f.vti"
    p.write_bytes(_vti_bytes(dims, [("n", n)]))
    vals, odims, spac = vti_io.lc_field_from_vti(str(p), 3, basis)
    I = {"XYZ": (0, 1, 2), "YZX": (1, 2, 0), "ZXY": (2, 0, 1)}[basis]
    assert odims == tuple(dims[i] for i in I)
    np.testing.assert_allclose(spac, [(0.2, 0.3, 0.4)[i] for i in I])
    # VTIReader.cpp:103-126, one element at a time
    for ix in range(dims[0]):
        for iy in range(dims[1]):
            for iz in range(dims[2]):
                idx = (ix, iy, iz)
                i_in = ix + dims[0] * (iy + dims[1] * iz)
                o = (idx[I[0]], idx[I[1]], idx[I[2]])
                np.testing.assert_array_equal(vals[o[2], o[1], o[0]], n[i_in, list(I)])


def test_qtensor_from_director_and_order(tmp_path):
    dims = (4, 3, 2)
    n = _director(dims, 2)
    S = np.linspace(0.1, 0.4, len(n))
    p = tmp_path / "f.vti"
    p.write_bytes(_vti_bytes(dims, [("n", n), ("S", S)]))
    q, _, _ = vti_io.lc_field_from_vti(str(p), 6, "XYZ")
    f = 1 - S  # VTIReader.cpp:145-170 uses (1 - S)
    ref = np.stack([0.5 * f * (3 * n[:, 0] ** 2 - 1), 0.5 * f * (3 * n[:, 1] ** 2 - 1), 0.5 * f * (3 * n[:, 2] ** 2 - 1),
                    1.5 * f * n[:, 0] * n[:, 1], 1.5 * f * n[:, 0] * n[:, 2], 1.5 * f * n[:, 1] * n[:, 2]], 1)
    np.testing.assert_allclose(q.reshape(-1, 6), ref, rtol=0, atol=1e-15)
    raw_q = np.random.default_rng(3).normal(size=(len(n), 6))
    p.write_bytes(_vti_bytes(dims, [("n", n), ("Q", raw_q)]))
    q2, od, _ = vti_io.lc_field_from_vti(str(p), 6, "YZX")  # Q is copied without permuting components
    assert od == (dims[1], dims[2], dims[0]) and q2.shape == (dims[0], dims[2], dims[1], 6)
    for ix in range(dims[0]):
        for iy in range(dims[1]):
            for iz in range(dims[2]):
                np.testing.assert_array_equal(q2[ix, iz, iy], raw_q[ix + dims[0] * (iy + dims[1] * iz)])


def test_reader_errors(tmp_path):
    with pytest.raises(vti_io.VtiError, match="does not exists"):
        vti_io.lc_field_from_vti(str(tmp_path / "missing.vti"), 3)
    dims = (3, 3, 2)
    p = tmp_path / "f.vti"
    p.write_bytes(_vti_bytes(dims, [("m", np.zeros((18, 3)))]))
    with pytest.raises(vti_io.VtiError, match='director array "n"'):
        vti_io.lc_field_from_vti(str(p), 3)
    n = _director(dims)
    n[4, 1] = np.nan
    p.write_bytes(_vti_bytes(dims, [("n", n)]))
    with pytest.raises(vti_io.VtiError, match="NaN"):
        vti_io.lc_field_from_vti(str(p), 3)


def test_writer_roundtrip(tmp_path):
    a = np.random.default_rng(0).normal(size=(12, 3))
    vti_io.write_vti(str(tmp_path / "w.vti"), (4, 3, 1), (0.5, 0.25, 0), (-0.75, -0.25, 0), [("E", a)],
                     [("lambda", np.array([0.5, 0.6]))])
    d = vti_io.read_vti(str(tmp_path / "w.vti"))
    assert d["dims"] == (4, 3, 1)
    np.testing.assert_array_equal(d["point"]["E"], a)
    np.testing.assert_array_equal(d["field"]["lambda"], [0.5, 0.6])


def test_minify_drops_comments_and_blank_lines(tmp_path):
    from nemaktis_gb300 import cli
    p = tmp_path / "s.json"
    p.write_text('# comment\n{\n\n  "a": 1,   \n   # another\n  "b": [2, 3]\n}\n')
    assert json.loads(cli.minify_json(str(p))) == {"a": 1, "b": [2, 3]}


@pytest.mark.gpu
@pytest.mark.parametrize("basis", ["XYZ", "ZXY"])
def test_cli_matches_backend_call(gpu, tmp_path, basis):
    """bpm-solver -x on a .vti director with a hole (zero director = outside the LC domain) gives
    the backend's fields for the same director and mask, and writes them as the screen file."""
    from nemaktis_gb300 import api, cli
    dims = (14, 12, 6)  # file axes
    n = _director(dims, 4)
    n[:10] = 0.0  # outside the domain
    p = tmp_path / "lc.vti"
    p.write_bytes(_vti_bytes(dims, [("n", n)]))
    folder = str(tmp_path / "out")
    js = json.loads(workloads.settings_json((1, 1, 1), (1, 1, 1), [0.5, 0.6], [(0.0, 0.0), (0.05, 0.02)], no="1.5",
                                            ne="1.7", nhost="1.45", results_folder=folder))
    js["Physics settings"]["Initial conditions"].update({"LC field file": str(p), "Basis convention": basis})
    js["Postprocessor settings"]["Screen output"]["Base name"] = "screen"
    sp = tmp_path / "settings.json"
    sp.write_text("# settings\n" + json.dumps(js, indent=1) + "\n")
    assert cli.main(["-x", str(sp)]) == 0
    vals, odims, spac = vti_io.lc_field_from_vti(str(p), 3, basis)
    js2 = workloads.settings_json(odims, spac, [0.5, 0.6], [(0.0, 0.0), (0.05, 0.02)], no="1.5", ne="1.7", nhost="1.45")
    E = np.zeros((2, 2, 4, odims[1], odims[0]), np.complex128)
    mask = np.where(np.linalg.norm(vals, axis=-1) > 1e-8, 1.0, -1.0)
    api.run(js2, vals, E, mask=mask)
    d = vti_io.read_vti(os.path.join(folder, "screen.vti"))
    assert d["dims"] == (odims[0], odims[1], 1)
    for w in range(2):
        for q in range(2):
            for pol, tag in enumerate(("inputX_", "inputY_")):
                re_ = d["point"]["E_real_%s%d_%d" % (tag, w, q)]
                im_ = d["point"]["E_imag_%s%d_%d" % (tag, w, q)]
                got = (re_[:, :2] + 1j * im_[:, :2]).T.reshape(2, odims[1], odims[0])
                np.testing.assert_array_equal(got, E[w, q, 2 * pol: 2 * pol + 2])


def test_cli_failures_print_the_reference_frame(tmp_path, capsys):
    """bpm-solver -x on a missing settings file, or on an LC field that is not a .vti file,
    exits with status 1 and the reference's framed message on stderr (main.cpp:169-257)."""
    from nemaktis_gb300 import cli
    assert cli.main(["-x", str(tmp_path / "missing.json")]) == 1
    err = capsys.readouterr().err
    assert "Could not open the specified setting file" in err and "Aborting!" in err
    js = json.loads(workloads.settings_json((4, 4, 4), (1, 1, 1), [0.5], [(0.0, 0.0)]))
    js["Physics settings"]["Initial conditions"]["LC field file"] = str(tmp_path / "lc.dat")
    p = tmp_path / "s.json"
    p.write_text(json.dumps(js))
    assert cli.main(["-x", str(p)]) == 1
    assert "must be a path to a vti file" in capsys.readouterr().err
    js["Physics settings"]["Initial conditions"]["LC field file"] = str(tmp_path / "absent.vti")
    p.write_text(json.dumps(js))
    assert cli.main(["-x", str(p)]) == 1
    assert "does not exists" in capsys.readouterr().err


def test_reader_big_endian_and_integer_arrays(tmp_path):
    """Big-endian files and integer/single-precision arrays, as VTK writes them on other hosts."""
    dims = (3, 2, 2)
    n = _director(dims, 8).astype(">f4")
    ids = np.arange(12, dtype=">i4")
    raw_n, raw_i = n.tobytes(), ids.tobytes()
    blob_n = struct.pack(">Q", len(raw_n)) + raw_n
    blob_i = struct.pack(">Q", len(raw_i)) + raw_i
    ext = "0 2 0 1 0 1"
    x = ('<?xml version="1.0"?>\n<VTKFile type="ImageData" version="1.0" byte_order="BigEndian" header_type="UInt64">\n'
         '<ImageData WholeExtent="%s" Origin="0 0 0" Spacing="1 1 1"><Piece Extent="%s"><PointData>'
         '<DataArray type="Float32" Name="n" NumberOfComponents="3" format="appended" offset="0"/>'
         '<DataArray type="Int32" Name="id" NumberOfComponents="1" format="appended" offset="%d"/>'
         '</PointData></Piece></ImageData>\n<AppendedData encoding="raw">\n_' % (ext, ext, len(blob_n)))
    (tmp_path / "b.vti").write_bytes(x.encode() + blob_n + blob_i + b"\n</AppendedData>\n</VTKFile>\n")
    d = vti_io.read_vti(str(tmp_path / "b.vti"))
    np.testing.assert_array_equal(d["point"]["n"], n.astype(np.float64))
    np.testing.assert_array_equal(d["point"]["id"], ids.astype(np.float64))
