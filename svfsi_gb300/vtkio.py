"""VTK XML meshes (.vtu volumes, .vtp faces): the formats the reference reads
its meshes from (READVTU / READVTP, Code/Source/svFSI/VTKXML.f:39-150, on
the vtkXMLParser module) and writes its results to.

Supported, as the reference's parser: DataArrays in ``ascii``, ``binary``
(base64) and ``appended`` (``raw`` or ``base64``) formats, header types
UInt32 and UInt64, and ``vtkZLibDataCompressor`` blocks.  Volume meshes are
tet4 (VTK cell type 10); faces are triangles (type 5).  As in READVTP, a
face's ``GlobalNodeID`` point array maps its points to the volume mesh's
(1-based) node numbers and ``GlobalElementID`` names the adjacent volume
element of each face triangle.

Host-side I/O (numpy, zlib, base64): the decoded arrays feed
``gsls_mesh_create`` and the boundary-condition calls unchanged.
"""
from __future__ import annotations

import base64
import re
import struct
import xml.etree.ElementTree as ET
import zlib
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

_DTYPES = {"Int8": "i1", "UInt8": "u1", "Int16": "i2", "UInt16": "u2", "Int32": "i4",
           "UInt32": "u4", "Int64": "i8", "UInt64": "u8", "Float32": "f4", "Float64": "f8"}
VTK_TRIANGLE, VTK_TETRA = 5, 10


@dataclass
class VtkPiece:
    points: np.ndarray                      # (n, 3) float64
    cells: np.ndarray                       # (m, k) int64, 0-based
    cell_types: np.ndarray | None = None    # (m,) (unstructured grids)
    point_data: dict = field(default_factory=dict)
    cell_data: dict = field(default_factory=dict)


class VtkError(ValueError):
    pass


# ---------------------------------------------------------------------------
# decoding
def _header_dtype(root):
    return np.dtype("<u8") if root.get("header_type", "UInt32") == "UInt64" else np.dtype("<u4")


def _byte_order(root):
    return "<" if root.get("byte_order", "LittleEndian") == "LittleEndian" else ">"


def _decode_block(buf: bytes, hdr: np.dtype, compressed: bool):
    """One binary DataArray payload (already base64-decoded when needed):
    returns (data bytes, bytes consumed)."""
    hs = hdr.itemsize
    if not compressed:
        n = int(np.frombuffer(buf[:hs], dtype=hdr)[0])
        return buf[hs:hs + n], hs + n
    nb, bs, last = (int(v) for v in np.frombuffer(buf[:3 * hs], dtype=hdr))
    sizes = np.frombuffer(buf[3 * hs:(3 + nb) * hs], dtype=hdr).astype(np.int64)
    pos, out = (3 + nb) * hs, []
    for b in range(nb):
        raw = zlib.decompress(buf[pos:pos + sizes[b]])
        expect = last if (b == nb - 1 and last) else bs
        if len(raw) != expect:
            raise VtkError("compressed block of unexpected size")
        out.append(raw)
        pos += int(sizes[b])
    return b"".join(out), pos


def _b64len(nbytes: int) -> int:
    return ((nbytes + 2) // 3) * 4


def _decode_b64_inline(text: str, hdr: np.dtype, compressed: bool):
    """A base64 DataArray payload (inline, or at an offset of an appended
    base64 block, so trailing characters of other arrays are ignored).  The
    header and the data may be encoded together or separately, as writers
    differ; compressed payloads are always encoded separately."""
    s = "".join(text.split()) if len(text) < (1 << 16) else re.sub(r"\s+", "", text)
    hs = hdr.itemsize
    if compressed:
        h0 = base64.b64decode(s[:_b64len(3 * hs)])
        nb = int(np.frombuffer(h0[:hs], dtype=hdr)[0])
        hch = _b64len((3 + nb) * hs)
        header = base64.b64decode(s[:hch])[:(3 + nb) * hs]
        sizes = np.frombuffer(header[3 * hs:], dtype=hdr).astype(np.int64)
        body = base64.b64decode(s[hch:hch + _b64len(int(sizes.sum()))])
        return _decode_block(header + body, hdr, True)[0]
    hch = _b64len(hs)
    h0 = base64.b64decode(s[:hch])
    n = int(np.frombuffer(h0[:hs], dtype=hdr)[0])
    if "=" in s[:hch]:  # header encoded on its own
        return base64.b64decode(s[hch:hch + _b64len(n)])[:n]
    return base64.b64decode(s[:_b64len(hs + n)])[hs:hs + n]


class _Reader:
    def __init__(self, path):
        data = Path(path).read_bytes()
        self.appended = b""
        self.app_enc = "raw"
        i = data.find(b"<AppendedData")
        if i >= 0:
            j = data.index(b">", i)
            tag = data[i:j + 1].decode("ascii", "replace")
            m = re.search(r'encoding="(\w+)"', tag)
            self.app_enc = m.group(1) if m else "raw"
            k = data.index(b"_", j) + 1
            end = data.rfind(b"</AppendedData>")
            self.appended = data[k:end]
            if self.app_enc == "base64":
                self.appended = self.appended.strip()
            xml = data[:i] + b"</VTKFile>"  # the grid is closed before AppendedData
        else:
            xml = data
        try:
            self.root = ET.fromstring(xml)
        except ET.ParseError as e:
            raise VtkError(f"not a VTK XML file: {e}") from None
        if self.root.tag != "VTKFile":
            raise VtkError("not a VTK XML file")
        self.hdr = _header_dtype(self.root)
        self.bo = _byte_order(self.root)
        self.compressed = self.root.get("compressor", "") == "vtkZLibDataCompressor"
        if self.root.get("compressor") not in (None, "", "vtkZLibDataCompressor"):
            raise VtkError(f"unsupported compressor {self.root.get('compressor')}")

    def array(self, el) -> np.ndarray:
        t = el.get("type")
        if t not in _DTYPES:
            raise VtkError(f"unsupported DataArray type {t}")
        dt = np.dtype(self.bo + _DTYPES[t])
        fmt = el.get("format", "ascii")
        nc = int(el.get("NumberOfComponents", "1"))
        if fmt == "ascii":
            a = np.array((el.text or "").split(), dtype=dt.newbyteorder("="))
        elif fmt == "binary":
            raw = _decode_b64_inline(el.text or "", self.hdr, self.compressed)
            a = np.frombuffer(raw, dtype=dt)
        elif fmt == "appended":
            off = int(el.get("offset"))
            if self.app_enc == "raw":
                raw, _ = _decode_block(self.appended[off:], self.hdr, self.compressed)
            else:
                raw = _decode_b64_inline(self.appended[off:].decode("ascii"), self.hdr,
                                         self.compressed)
            a = np.frombuffer(raw, dtype=dt)
        else:
            raise VtkError(f"unsupported DataArray format {fmt}")
        a = a.astype(dt.newbyteorder("="), copy=False)
        return a.reshape(-1, nc) if nc > 1 else a

    def named(self, parent, name):
        if parent is None:
            return None
        for el in parent.findall("DataArray"):
            if el.get("Name") == name:
                return self.array(el)
        return None

    def data_dict(self, parent):
        out = {}
        if parent is not None:
            for el in parent.findall("DataArray"):
                out[el.get("Name")] = self.array(el)
        return out


def _cells_from(conn, offsets):
    sizes = np.diff(np.concatenate([[0], offsets]))
    if sizes.size and np.all(sizes == sizes[0]):
        return conn.reshape(-1, int(sizes[0])).astype(np.int64)
    raise VtkError("mixed cell sizes are not supported")


def read_vtu(path) -> VtkPiece:
    """Points, cells, cell types and point/cell arrays of a .vtu file."""
    r = _Reader(path)
    piece = r.root.find("UnstructuredGrid/Piece")
    if piece is None:
        raise VtkError("no UnstructuredGrid piece")
    n, m = int(piece.get("NumberOfPoints")), int(piece.get("NumberOfCells"))
    pts = r.array(piece.find("Points/DataArray")).reshape(n, -1).astype(np.float64)
    cel = piece.find("Cells")
    conn = r.named(cel, "connectivity")
    offs = r.named(cel, "offsets")
    types = r.named(cel, "types")
    cells = _cells_from(conn, offs) if m else np.zeros((0, 0), np.int64)
    if cells.shape[0] != m:
        raise VtkError("cell count mismatch")
    return VtkPiece(pts, cells, None if types is None else types.astype(np.int64),
                    r.data_dict(piece.find("PointData")), r.data_dict(piece.find("CellData")))


def read_vtp(path) -> VtkPiece:
    """Points, polygons and point/cell arrays of a .vtp file."""
    r = _Reader(path)
    piece = r.root.find("PolyData/Piece")
    if piece is None:
        raise VtkError("no PolyData piece")
    n = int(piece.get("NumberOfPoints"))
    m = int(piece.get("NumberOfPolys", "0"))
    pts = r.array(piece.find("Points/DataArray")).reshape(n, -1).astype(np.float64)
    pol = piece.find("Polys")
    cells = _cells_from(r.named(pol, "connectivity"), r.named(pol, "offsets")) if m else \
        np.zeros((0, 3), np.int64)
    if cells.shape[0] != m:
        raise VtkError("polygon count mismatch")
    return VtkPiece(pts, cells, None, r.data_dict(piece.find("PointData")),
                    r.data_dict(piece.find("CellData")))


# ---------------------------------------------------------------------------
# encoding
def _vtk_type(a: np.ndarray):
    for k, v in _DTYPES.items():
        if np.dtype(v) == a.dtype.newbyteorder("="):
            return k
    raise VtkError(f"no VTK type for {a.dtype}")


def _encode(a: np.ndarray, hdr: np.dtype, compress: bool, blocksize=1 << 15):
    raw = np.ascontiguousarray(a).astype(a.dtype.newbyteorder("<"), copy=False).tobytes()
    if not compress:
        return np.array([len(raw)], dtype=hdr).tobytes(), raw
    blocks = [raw[i:i + blocksize] for i in range(0, len(raw), blocksize)] or [b""]
    comp = [zlib.compress(b) for b in blocks]
    last = len(blocks[-1]) if len(blocks[-1]) != blocksize else 0
    head = np.array([len(blocks), blocksize, last] + [len(c) for c in comp], dtype=hdr).tobytes()
    return head, b"".join(comp)


def _write(path, kind, piece_attrs, sections, fmt="appended", compress=True, header="UInt64"):
    """sections: list of (tag, [(name, array, extra_attrs)])."""
    if fmt not in ("ascii", "binary", "appended"):
        raise VtkError(f"unknown format {fmt}")
    hdr = np.dtype("<u8") if header == "UInt64" else np.dtype("<u4")
    comp = compress and fmt != "ascii"
    attrs = f'type="{kind}" version="1.0" byte_order="LittleEndian" header_type="{header}"'
    if comp:
        attrs += ' compressor="vtkZLibDataCompressor"'
    out = [f'<?xml version="1.0"?>\n<VTKFile {attrs}>\n  <{kind}>\n    <Piece {piece_attrs}>\n']
    app, off = [], 0
    for tag, arrays in sections:
        out.append(f"      <{tag}>\n")
        for name, a, extra in arrays:
            a = np.asarray(a)
            nc = a.shape[1] if a.ndim == 2 else 1
            head = (f'        <DataArray type="{_vtk_type(a)}" '
                    + (f'Name="{name}" ' if name else "")
                    + (f'NumberOfComponents="{nc}" ' if nc > 1 else "") + extra)
            if fmt == "ascii":
                body = " ".join(repr(float(v)) if a.dtype.kind == "f" else str(int(v))
                                for v in a.ravel())
                out.append(head + f'format="ascii">\n          {body}\n        </DataArray>\n')
            elif fmt == "binary":
                h, d = _encode(a, hdr, comp)
                if comp:
                    b64 = base64.b64encode(h).decode() + base64.b64encode(d).decode()
                else:
                    b64 = base64.b64encode(h + d).decode()
                out.append(head + f'format="binary">\n          {b64}\n        </DataArray>\n')
            else:
                h, d = _encode(a, hdr, comp)
                out.append(head + f'format="appended" offset="{off}"/>\n')
                app.append(h + d)
                off += len(h) + len(d)
        out.append(f"      </{tag}>\n")
    out.append(f"    </Piece>\n  </{kind}>\n")
    with open(path, "wb") as f:
        f.write("".join(out).encode())
        if fmt == "appended":
            f.write(b'  <AppendedData encoding="raw">\n   _')
            for blob in app:
                f.write(blob)
            f.write(b"\n  </AppendedData>\n")
        f.write(b"</VTKFile>\n")


def write_vtu(path, points, cells, point_data=None, cell_data=None, cell_type=VTK_TETRA,
              fmt="appended", compress=True, header="UInt64"):
    """Unstructured grid of equal-size cells (0-based connectivity)."""
    points = np.asarray(points, np.float64)
    cells = np.asarray(cells, np.int64)
    m, k = cells.shape
    secs = []
    if point_data:
        secs.append(("PointData", [(n, v, "") for n, v in point_data.items()]))
    if cell_data:
        secs.append(("CellData", [(n, v, "") for n, v in cell_data.items()]))
    secs.append(("Points", [("", points, "")]))
    secs.append(("Cells", [("connectivity", cells.ravel(), ""),
                           ("offsets", np.arange(1, m + 1, dtype=np.int64) * k, ""),
                           ("types", np.full(m, cell_type, np.uint8), "")]))
    _write(path, "UnstructuredGrid", f'NumberOfPoints="{points.shape[0]}" NumberOfCells="{m}"',
           secs, fmt, compress, header)


def write_vtp(path, points, polys, point_data=None, cell_data=None, fmt="appended",
              compress=True, header="UInt64"):
    """Poly data of equal-size polygons (0-based connectivity)."""
    points = np.asarray(points, np.float64)
    polys = np.asarray(polys, np.int64)
    m, k = polys.shape
    secs = []
    if point_data:
        secs.append(("PointData", [(n, v, "") for n, v in point_data.items()]))
    if cell_data:
        secs.append(("CellData", [(n, v, "") for n, v in cell_data.items()]))
    secs.append(("Points", [("", points, "")]))
    secs.append(("Polys", [("connectivity", polys.ravel(), ""),
                           ("offsets", np.arange(1, m + 1, dtype=np.int64) * k, "")]))
    _write(path, "PolyData", f'NumberOfPoints="{points.shape[0]}" NumberOfPolys="{m}"', secs,
           fmt, compress, header)


# ---------------------------------------------------------------------------
# svFSI meshes
@dataclass
class SvMesh:
    x: np.ndarray          # (nNo, 3)
    ien: np.ndarray        # (nEl, 4) 0-based, int32
    faces: dict            # name -> dict(nodes (0-based, sorted), tris (0-based), elems)


def load_mesh(vtu_path, faces: dict | None = None) -> SvMesh:
    """A tet4 volume mesh and its named faces, as READVTU/READVTP load them:
    face points are mapped to volume nodes through GlobalNodeID (1-based),
    face triangles keep their GlobalElementID when present."""
    v = read_vtu(vtu_path)
    if v.cells.shape[1] != 4 or (v.cell_types is not None and np.any(v.cell_types != VTK_TETRA)):
        raise VtkError("the volume mesh must be linear tetrahedra (VTK type 10)")
    out = {}
    for name, fp in (faces or {}).items():
        f = read_vtp(fp)
        gn = f.point_data.get("GlobalNodeID")
        if gn is None:
            raise VtkError(f"face {name}: no GlobalNodeID point array")
        gn = np.asarray(gn, np.int64).ravel() - 1
        if gn.min() < 0 or gn.max() >= v.points.shape[0]:
            raise VtkError(f"face {name}: GlobalNodeID outside the volume mesh")
        ge = f.cell_data.get("GlobalElementID")
        out[name] = dict(nodes=np.unique(gn).astype(np.int32), tris=gn[f.cells].astype(np.int32),
                         elems=None if ge is None else np.asarray(ge, np.int64).ravel() - 1)
    return SvMesh(v.points[:, :3].copy(), v.cells.astype(np.int32), out)


def _fibre_block(piece: VtkPiece, name: str, nEl: int, src) -> np.ndarray:
    a = piece.cell_data.get(name)
    if a is None:
        raise VtkError(f"{src}: no cell array {name}")
    a = np.asarray(a, np.float64).reshape(piece.cells.shape[0], -1)
    if a.shape[0] != nEl:
        raise VtkError(f"{src}: {a.shape[0]} cells for {name}, the mesh has {nEl} elements")
    out = np.zeros((nEl, 3))
    k = min(3, a.shape[1])
    out[:, :k] = a[:, :k]
    return out


def load_fibers(nEl: int, file=None, files=None, directions=None,
                nFn: int | None = None) -> np.ndarray | None:
    """Per-element fibre directions (the reference's lM%fN), nEl x 3 nFn in
    element order, from the first of the reference's three sources that
    gives fibres (Code/Source/svFSI/READMSH.f:336-420):

    * ``file``: one .vtu whose cell arrays FIB_DIR1, FIB_DIR2, ... hold the
      families (READFIBNFSF, READMSH.f:895-965); ``nFn`` families, or as
      many as the largest index among the FIB_DIR<i> names (one digit, as
      the reference parses it);
    * ``files``: one .vtu per family, each with the cell array FIB_DIR
      (READFIBNFF, READMSH.f:968-1003);
    * ``directions``: one constant vector per family ("Fiber direction").

    Every direction is normalised to unit length unless its length is zero
    (ISZERO), as READMSH does after reading.  None when no source gives a
    family.  The result is what ``gsls_eq_params.fN`` expects."""
    fN = None
    if file is not None:
        v = read_vtu(file)
        n = nFn or 0
        if not n:
            for name in v.cell_data:
                if name.startswith("FIB_DIR") and len(name) >= 8:
                    if not name[7].isdigit():
                        raise VtkError(f"{file}: cannot read the fibre index of {name}")
                    n = max(n, int(name[7]))
        if n:
            fN = np.concatenate([_fibre_block(v, f"FIB_DIR{i}", nEl, file)
                                 for i in range(1, n + 1)], axis=1)
    if fN is None and files:
        fN = np.concatenate([_fibre_block(read_vtu(p), "FIB_DIR", nEl, p) for p in files], axis=1)
    if fN is None and directions is not None and len(directions):
        d = np.asarray(directions, np.float64).reshape(-1, 3)
        fN = np.tile(d.ravel(), (nEl, 1))
    if fN is None:
        return None
    fam = fN.reshape(nEl, -1, 3)
    nrm = np.linalg.norm(fam, axis=2, keepdims=True)
    # ISZERO: |x| / max(|x|, eps) < eps, i.e. |x| < eps^2, is zero
    ok = nrm >= np.finfo(np.float64).eps ** 2
    fam = np.where(ok, fam / np.where(ok, nrm, 1.0), fam)
    return np.ascontiguousarray(fam.reshape(nEl, -1))


def pack_struct_header(hdr_type: str, nblocks: int, bs: int, last: int, sizes) -> bytes:
    """vtkZLibDataCompressor block header (for tests and writers)."""
    c = "Q" if hdr_type == "UInt64" else "I"
    return struct.pack("<" + c * (3 + nblocks), nblocks, bs, last, *sizes)
