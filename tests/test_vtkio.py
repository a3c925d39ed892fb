"""VTK XML mesh I/O (READVTU / READVTP, Code/Source/svFSI/VTKXML.f:39-150):
hand-written ASCII fixtures (tests/golden/two_tets.vtu, two_tets_face.vtp,
two_tets_fibers.vtu, written from the VTK XML format description), a
zlib-compressed inline array encoded independently in the test, round
trips through the writer in every format / header / compression
combination, and the three fibre sources of READMSH."""
import base64
import struct
import zlib
from pathlib import Path

import numpy as np
import pytest

from svfsi_gb300 import meshgen, vtkio

GOLD = Path(__file__).parent / "golden"


def test_ascii_fixture_and_face_mapping():
    m = vtkio.load_mesh(GOLD / "two_tets.vtu", {"top": GOLD / "two_tets_face.vtp"})
    assert m.x.shape == (5, 3) and m.ien.tolist() == [[0, 1, 2, 3], [1, 2, 3, 4]]
    f = m.faces["top"]
    assert f["nodes"].tolist() == [1, 3, 4]          # GlobalNodeID 2 5 4 -> 0-based
    assert f["tris"].tolist() == [[1, 4, 3]]
    assert f["elems"].tolist() == [1]
    # face coordinates agree with the volume nodes they map to
    v = vtkio.read_vtp(GOLD / "two_tets_face.vtp")
    assert np.allclose(v.points, m.x[[1, 4, 3]])


def _compressed_inline(values: np.ndarray, blocksize: int, header="UInt32"):
    raw = values.astype("<f8").tobytes()
    blocks = [raw[i:i + blocksize] for i in range(0, len(raw), blocksize)]
    comp = [zlib.compress(b, 9) for b in blocks]
    last = len(blocks[-1]) if len(blocks[-1]) != blocksize else 0
    c = "Q" if header == "UInt64" else "I"
    head = struct.pack("<" + c * (3 + len(comp)), len(comp), blocksize, last, *[len(x) for x in comp])
    return base64.b64encode(head).decode() + base64.b64encode(b"".join(comp)).decode()


@pytest.mark.parametrize("header", ["UInt32", "UInt64"])
def test_independently_encoded_compressed_array(tmp_path, header):
    pts = np.random.default_rng(0).standard_normal((7, 3))
    b64 = _compressed_inline(pts.ravel(), blocksize=40, header=header)
    xml = f'''<?xml version="1.0"?>
<VTKFile type="UnstructuredGrid" version="1.0" byte_order="LittleEndian" header_type="{header}" compressor="vtkZLibDataCompressor">
 <UnstructuredGrid><Piece NumberOfPoints="7" NumberOfCells="1">
  <Points><DataArray type="Float64" NumberOfComponents="3" format="binary">{b64}</DataArray></Points>
  <Cells>
   <DataArray type="Int32" Name="connectivity" format="ascii">0 1 2 3</DataArray>
   <DataArray type="Int32" Name="offsets" format="ascii">4</DataArray>
   <DataArray type="UInt8" Name="types" format="ascii">10</DataArray>
  </Cells></Piece></UnstructuredGrid></VTKFile>'''
    f = tmp_path / "c.vtu"
    f.write_text(xml)
    v = vtkio.read_vtu(f)
    assert np.array_equal(v.points, pts) and v.cells.tolist() == [[0, 1, 2, 3]]


@pytest.mark.parametrize("fmt", ["ascii", "binary", "appended"])
@pytest.mark.parametrize("compress", [False, True])
@pytest.mark.parametrize("header", ["UInt32", "UInt64"])
def test_round_trip(tmp_path, fmt, compress, header):
    x, ien = meshgen.kuhn_box(3, 2, 2)
    gid = np.arange(1, x.shape[0] + 1, dtype=np.int32)
    eid = np.arange(1, ien.shape[0] + 1, dtype=np.int32)
    f = tmp_path / "m.vtu"
    vtkio.write_vtu(f, x, ien, {"GlobalNodeID": gid}, {"GlobalElementID": eid}, fmt=fmt,
                    compress=compress, header=header)
    faces = meshgen.faces_on_plane(x, ien, 0, 1.0)
    fn = np.unique(faces)
    loc = np.searchsorted(fn, faces)
    fp = tmp_path / "f.vtp"
    vtkio.write_vtp(fp, x[fn], loc, {"GlobalNodeID": gid[fn]}, fmt=fmt, compress=compress,
                    header=header)
    m = vtkio.load_mesh(f, {"right": fp})
    assert np.array_equal(m.x, x) and np.array_equal(m.ien, ien)
    assert np.array_equal(m.faces["right"]["nodes"], fn)
    assert np.array_equal(m.faces["right"]["tris"], faces)
    v = vtkio.read_vtu(f)
    assert np.array_equal(v.point_data["GlobalNodeID"], gid)
    assert np.array_equal(v.cell_data["GlobalElementID"], eid)
    assert np.all(v.cell_types == vtkio.VTK_TETRA)


def test_appended_base64(tmp_path):
    """Appended data in base64 (offsets in characters), compressed."""
    x, ien = meshgen.kuhn_box(2, 2, 2)
    f = tmp_path / "a.vtu"
    vtkio.write_vtu(f, x, ien, fmt="appended", compress=True)
    # re-encode the appended block as base64 by hand
    v = vtkio.read_vtu(f)
    arrays = [x.ravel(), ien.ravel().astype(np.int64),
              np.arange(1, ien.shape[0] + 1, dtype=np.int64) * 4,
              np.full(ien.shape[0], 10, np.uint8)]
    names = ["", "connectivity", "offsets", "types"]
    types = ["Float64", "Int64", "Int64", "UInt8"]
    chunks, offs, off = [], [], 0
    for a in arrays:
        raw = a.astype(a.dtype.newbyteorder("<")).tobytes()
        comp = zlib.compress(raw)
        head = struct.pack("<QQQQ", 1, len(raw), len(raw), len(comp))
        s = base64.b64encode(head).decode() + base64.b64encode(comp).decode()
        offs.append(off)
        chunks.append(s)
        off += len(s)
    da = [f'<DataArray type="{t}" ' + (f'Name="{n}" ' if n else 'NumberOfComponents="3" ')
          + f'format="appended" offset="{o}"/>' for t, n, o in zip(types, names, offs)]
    xml = (f'<?xml version="1.0"?>\n<VTKFile type="UnstructuredGrid" version="1.0" '
           f'byte_order="LittleEndian" header_type="UInt64" compressor="vtkZLibDataCompressor">'
           f'<UnstructuredGrid><Piece NumberOfPoints="{x.shape[0]}" NumberOfCells="{ien.shape[0]}">'
           f'<Points>{da[0]}</Points><Cells>{"".join(da[1:])}</Cells></Piece></UnstructuredGrid>'
           f'<AppendedData encoding="base64">\n _{"".join(chunks)}\n</AppendedData></VTKFile>')
    g = tmp_path / "b.vtu"
    g.write_text(xml)
    w = vtkio.read_vtu(g)
    assert np.array_equal(w.points, v.points) and np.array_equal(w.cells, v.cells)


def test_rejects_non_tet_volume(tmp_path):
    f = tmp_path / "h.vtu"
    vtkio.write_vtu(f, np.zeros((8, 3)), np.arange(8).reshape(1, 8), cell_type=12, fmt="ascii")
    with pytest.raises(vtkio.VtkError):
        vtkio.load_mesh(f)


def test_fibres_from_one_file_fixture():
    """READFIBNFSF: FIB_DIR1, FIB_DIR2 cell arrays, the family count from the
    names, each direction normalised, a zero direction left zero."""
    f = vtkio.load_fibers(2, file=GOLD / "two_tets_fibers.vtu")
    assert f.shape == (2, 6)
    assert np.allclose(f, [[1, 0, 0, 0, 0, 1], [0, 0.6, 0.8, 0, 0, 0]], atol=1e-15)
    f1 = vtkio.load_fibers(2, file=GOLD / "two_tets_fibers.vtu", nFn=1)
    assert np.array_equal(f1, f[:, :3])


def test_fibres_from_one_file_per_family_and_uniform(tmp_path):
    x, ien = meshgen.kuhn_box(2, 2, 1, 1.0, 1.0, 1.0)
    rng = np.random.default_rng(3)
    fams = [rng.standard_normal((ien.shape[0], 3)) for _ in range(2)]
    paths = []
    for i, a in enumerate(fams):
        p = tmp_path / f"fib{i}.vtu"
        vtkio.write_vtu(p, x, ien, cell_data={"FIB_DIR": a})
        paths.append(p)
    f = vtkio.load_fibers(ien.shape[0], files=paths)
    want = np.concatenate([a / np.linalg.norm(a, axis=1, keepdims=True) for a in fams], axis=1)
    assert np.allclose(f, want, atol=1e-15)
    # a file without FIB_DIR<i> arrays gives no fibres: the next source is read
    plain = tmp_path / "plain.vtu"
    vtkio.write_vtu(plain, x, ien)
    assert np.allclose(vtkio.load_fibers(ien.shape[0], file=plain, files=paths), want, atol=1e-15)
    u = vtkio.load_fibers(ien.shape[0], directions=[[0, 0, 2.0], [1, 1, 0]])
    assert np.allclose(u, np.tile([0, 0, 1, 2 ** -0.5, 2 ** -0.5, 0], (ien.shape[0], 1)))
    assert vtkio.load_fibers(ien.shape[0]) is None
    with pytest.raises(vtkio.VtkError):
        vtkio.load_fibers(ien.shape[0] + 1, files=paths)
