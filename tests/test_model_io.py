"""Mesh import: tests/unit/stl.test.ts, obj/obj.test.ts and threemf/threemf.test.ts
of the reference, restated on the host importers (the fixture files are the
reference's, committed as base64 in tests/golden/model_fixtures.json)."""
import base64
import io
import json
import math
import struct
import zipfile
from pathlib import Path

import numpy as np
import pytest

from pocketwind_gb300 import model_io as M
from pocketwind_gb300._lib import RangeError

FIXTURES = json.loads((Path(__file__).parent / "golden" / "model_fixtures.json").read_text())["files"]


def fixture(name: str) -> bytes:
    return base64.b64decode(FIXTURES[name])


def ascii(text: str) -> bytes:
    return text.encode("utf-8")


def bounds(mesh, lo, hi):
    p = mesh.positions.reshape(-1, 3)
    np.testing.assert_allclose(p.min(0), lo, atol=1e-3)
    np.testing.assert_allclose(p.max(0), hi, atol=1e-3)


# ---------------------------------------------------------------- STL
@pytest.mark.parametrize("name", ["cube-binary", "cube-ascii-crlf", "solid-header-binary"])
def test_stl_reads_the_cube(name):
    mesh = M.parse_stl(fixture(f"stl/{name}.stl"))
    assert mesh.triangle_count == 12 and mesh.positions.size == 108
    ref = M.parse_stl(fixture("stl/cube-binary.stl"))
    assert np.array_equal(mesh.positions, ref.positions)
    assert set(mesh.positions.tolist()) == {0.0, 1.0}


def test_stl_errors_from_fixtures():
    data = fixture("stl/truncated.stl")
    e = M.parse_stl(data)
    assert (e.kind, e.byte_offset) == ("truncated", len(data))
    assert (M.parse_stl(fixture("stl/random.stl")).kind, M.parse_stl(fixture("stl/random.stl")).byte_offset) == ("not-stl", 0)
    e = M.parse_stl(fixture("stl/empty.stl"))
    assert (e.kind, e.byte_offset) == ("empty", 80)
    e = M.parse_stl(fixture("stl/nan-vertex.stl"))
    assert e.kind == "non-finite" and e.byte_offset >= 84 + 12


@pytest.mark.parametrize("name", ["cube-binary", "cube-ascii-crlf"])
def test_stl_triangle_limit(name):
    assert M.parse_stl(fixture(f"stl/{name}.stl"), 11).kind == "too-many-triangles"


def test_stl_binary_normals_ignored_and_trailing_bytes_rejected():
    data = bytearray(fixture("stl/cube-binary.stl"))
    for t in range(12):
        data[84 + 50 * t: 84 + 50 * t + 12] = b"\xff" * 12  # NaN normals
        data[84 + 50 * t + 48: 84 + 50 * t + 50] = b"\x07\x07"
    assert M.parse_stl(bytes(data)).triangle_count == 12
    assert M.parse_stl(bytes(fixture("stl/cube-binary.stl")) + b"\0").kind == "not-stl"


def test_stl_ascii_errors():
    assert M.parse_stl(ascii("solid empty\nendsolid empty\n")).kind == "empty"
    data = ascii("solid t\nfacet normal 0 0 0\nouter loop\nvertex 0 0 0\n")
    e = M.parse_stl(data)
    assert (e.kind, e.byte_offset) == ("truncated", len(data))
    text = "solid t\nfacet normal 0 0 0\nouter lop\n"
    e = M.parse_stl(ascii(text))
    assert (e.kind, e.byte_offset) == ("not-stl", text.index("lop"))
    for value in ("1e39", "-1e39", "Infinity"):
        text = f"solid t\nfacet normal 0 0 0\nouter loop\nvertex {value} 0 0\n"
        e = M.parse_stl(ascii(text))
        assert (e.kind, e.byte_offset) == ("non-finite", text.index(value))


def test_stl_offsets_after_utf8_name_and_bad_tokens():
    prefix = "solid é\nfacet normal 0 0 0\nouter loop\nvertex "
    e = M.parse_stl(ascii(prefix + "NaN 0 0"))
    assert (e.kind, e.byte_offset) == ("non-finite", len(prefix.encode()))
    e = M.parse_stl(ascii(prefix + "wrong 0 0"))
    assert (e.kind, e.byte_offset) == ("not-stl", len(prefix.encode()))
    text = "solid t\nfacet normal 0 0 0\nouter loop\nvertex 0 0 0\nvertex 1 0 0\nvertex 0 1 0\nendloop\nendfacet\nendsolid t\n"
    e = M.parse_stl(ascii(text + "facet"))
    assert (e.kind, e.byte_offset) == ("not-stl", len(text))


def test_stl_signed_and_scientific_coordinates():
    text = ("solid t\nfacet normal 0 0 0\nouter loop\nvertex -1e-2 +.5 1.\nvertex 1 0 0\nvertex 0 1 0\n"
            "endloop\nendfacet\nendsolid t\n")
    mesh = M.parse_stl(ascii(text))
    assert mesh.positions[:3].tolist() == [np.float32(-0.01), 0.5, 1.0]


def test_stl_invalid_limits_and_default_cap():
    for limit in (-1, 1.5, 2 ** 53):
        with pytest.raises(RangeError):
            M.parse_stl(fixture("stl/empty.stl"), limit)
    data = bytearray(84)
    struct.pack_into("<I", data, 80, M.DEFAULT_MAX_TRIANGLES + 1)
    e = M.parse_stl(bytes(data))
    assert (e.kind, e.byte_offset) == ("too-many-triangles", 80)


# ---------------------------------------------------------------- OBJ
VERTS = "v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\n"


def test_obj_quad_cube_fans_to_twelve():
    mesh = M.parse_obj(fixture("obj/quad-cube.obj"))
    assert mesh.triangle_count == 12


@pytest.mark.parametrize("face", ["1 2 3 4", "1/1 2/2 3/3 4/4", "1//1 2//2 3//3 4//4", "1/1/1 2/2/2 3/3/3 4/4/4",
                                  "-4 -3 -2 -1"])
def test_obj_face_forms(face):
    mesh = M.parse_obj(ascii(f"{VERTS}f {face}"))
    assert mesh.triangle_count == 2
    assert mesh.positions.tolist() == [0, 0, 0, 1, 0, 0, 1, 1, 0, 0, 0, 0, 1, 1, 0, 0, 1, 0]


def test_obj_negative_indices_resolve_at_the_face():
    assert M.parse_obj(ascii(f"{VERTS}f -4 -3 -2\nv 9 9 9")).triangle_count == 1


@pytest.mark.parametrize("face", ["1 2", "0 1 2", "1 2 5", "1 2 x", "1/ 2 3", "-5 1 2"])
def test_obj_invalid_faces(face):
    assert M.parse_obj(ascii(f"{VERTS}f {face}")).kind == "not-stl"


def test_obj_coordinates_limits_and_offsets():
    assert M.parse_obj(ascii("v 1 2")).kind == "not-stl"
    assert M.parse_obj(ascii("v 1e50 0 0")).kind == "non-finite"
    assert M.parse_obj(ascii("v NaN 0 0")).kind == "not-stl"
    prefix = f"# é\r\n{VERTS}\r"
    e = M.parse_obj(ascii(f"{prefix}f 0 1 2"))
    assert (e.kind, e.byte_offset) == ("not-stl", len(prefix.encode()))
    assert M.parse_obj(ascii(f"{VERTS}f 1 2 3 4"), 1).kind == "too-many-triangles"
    assert M.parse_obj(ascii(VERTS)).kind == "empty"


# ---------------------------------------------------------------- 3MF
MODEL_PATH = "3D/3dmodel.model"
_CUBE_V = [(0, 0, 0), (300, 0, 0), (300, 300, 0), (0, 300, 0), (0, 0, 300), (300, 0, 300), (300, 300, 300), (0, 300, 300)]
_CUBE_T = [(0, 2, 1), (0, 3, 2), (4, 5, 6), (4, 6, 7), (0, 1, 5), (0, 5, 4), (1, 2, 6), (1, 6, 5), (2, 3, 7), (2, 7, 6),
           (3, 0, 4), (3, 4, 7)]
CUBE_OBJECT = ('<object id="1" type="model"><mesh><vertices>'
               + "".join(f'<vertex x="{x}" y="{y}" z="{z}"/>' for x, y, z in _CUBE_V)
               + "</vertices><triangles>"
               + "".join(f'<triangle v1="{a}" v2="{b}" v3="{c}"/>' for a, b, c in _CUBE_T)
               + "</triangles></mesh></object>")


def model_xml(objects=CUBE_OBJECT, build='<item objectid="1"/>', unit="millimeter"):
    return ('<?xml version="1.0" encoding="UTF-8"?>'
            f'<model unit="{unit}" xml:lang="en-US" xmlns="http://schemas.microsoft.com/3dmanufacturing/core/2015/02" '
            'xmlns:p="http://schemas.microsoft.com/3dmanufacturing/production/2015/06">'
            f"<resources>{objects}</resources><build>{build}</build></model>")


def make_archive(members, method=zipfile.ZIP_DEFLATED):
    buf = io.BytesIO()
    with zipfile.ZipFile(buf, "w", method) as z:
        for name, text in members:
            z.writestr(name, text)
    return buf.getvalue()


def model_archive(text):
    rels = ('<?xml version="1.0" encoding="UTF-8"?><Relationships xmlns="http://schemas.openxmlformats.org/package/'
            '2006/relationships"><Relationship Target="/3D/3dmodel.model" Id="rel0" '
            'Type="http://schemas.microsoft.com/3dmanufacturing/2013/01/3dmodel"/></Relationships>')
    return make_archive([("_rels/.rels", rels), (MODEL_PATH, text)])


@pytest.mark.parametrize("name,count,lo,hi,items,unit", [
    ("single-object", 12, [0, 0, 0], [300, 300, 300], 1, 1),
    ("stored", 12, [0, 0, 0], [300, 300, 300], 1, 1),
    ("inch", 12, [0, 0, 0], [7620, 7620, 7620], 1, 25.4),
    ("components", 24, [-300, 0, 0], [980, 310, 330], 2, 1),
    ("external-part", 12, [10, 20, 30], [310, 320, 330], 1, 1),
])
def test_3mf_fixtures(name, count, lo, hi, items, unit):
    mesh, unit_mm, item_count = M.parse_three_mf(fixture(f"3mf/{name}.3mf"))
    assert mesh.triangle_count == count and unit_mm == unit and item_count == items
    bounds(mesh, lo, hi)


@pytest.mark.parametrize("unit,mm", [("micron", 0.001), ("millimeter", 1), ("centimeter", 10), ("inch", 25.4),
                                     ("foot", 304.8), ("meter", 1000)])
def test_3mf_units(unit, mm):
    mesh, unit_mm, _ = M.parse_three_mf(model_archive(model_xml(unit=unit)))
    assert unit_mm == mm
    bounds(mesh, [0, 0, 0], [300 * mm] * 3)


@pytest.mark.parametrize("name,kind", [("zip64", "zip-unsupported"), ("encrypted", "zip-unsupported"),
                                       ("unsupported-method", "zip-unsupported"), ("missing-model", "no-model-part")])
def test_3mf_archive_errors(name, kind):
    assert M.parse_three_mf(fixture(f"3mf/{name}.3mf")).kind == kind


def test_3mf_start_relationship_prefixes_quotes_and_escaped_paths():
    text = (model_xml().replace('"', "'").replace("<model", "<c:model").replace("</model>", "</c:model>")
            .replace("xmlns=", "xmlns:c="))
    data = make_archive([("_rels/.rels", '<r:Relationships xmlns:r="urn:rels"><r:Relationship Type="StartPart" '
                                         'Target="/3D/a&amp;b.model"/></r:Relationships>'), ("3D/a&b.model", text)])
    mesh, _, _ = M.parse_three_mf(data)
    assert mesh.triangle_count == 12


def test_3mf_default_path_and_unit():
    data = make_archive([(MODEL_PATH, model_xml().replace(' unit="millimeter"', ""))])
    mesh, unit, _ = M.parse_three_mf(data)
    assert unit == 1 and mesh.triangle_count == 12


def test_3mf_ignores_metadata_comments_colours_and_unused_resources():
    text = model_xml(CUBE_OBJECT + '<object id="2"/>').replace(
        "<resources>", '<!-- <bad> --><metadata name="x"><![CDATA[a < b]]></metadata><resources><colorgroup id="3"/>')
    assert M.parse_three_mf(model_archive(text))[0].triangle_count == 12


@pytest.mark.parametrize("text", [
    "<model><resources></model>",
    "<!DOCTYPE model><model/>",
    "<model unit=millimeter/>",
    model_xml().replace('v1="0"', 'v1="900"'),
    model_xml().replace('x="0"', 'x="no"'),
    model_xml().replace('id="1"', 'id="1" id="2"'),
    model_xml(CUBE_OBJECT, '<item objectid="9"/>'),
    model_xml(CUBE_OBJECT, '<item objectid="1" transform="1 2"/>'),
    model_xml(CUBE_OBJECT, '<item objectid="1"/>', "yard"),
    model_xml('<object id="1"><components><component objectid="1"/></components></object>'),
])
def test_3mf_invalid_models(text):
    e = M.parse_three_mf(model_archive(text))
    assert (e.kind, e.part) == ("bad-xml", MODEL_PATH)


def test_3mf_missing_external_part():
    text = model_xml('<object id="1"><components><component objectid="2" p:path="Objects/missing.model"/>'
                     '</components></object>')
    e = M.parse_three_mf(model_archive(text))
    assert (e.kind, e.part) == ("no-model-part", "3D/Objects/missing.model")


def test_3mf_limits_and_overflow():
    assert M.parse_three_mf(fixture("3mf/single-object.3mf"), 11).kind == "too-many-triangles"
    two = model_archive(model_xml(CUBE_OBJECT, '<item objectid="1"/><item objectid="1"/>'))
    assert M.parse_three_mf(two, 12).kind == "too-many-triangles"
    big = model_archive(model_xml(CUBE_OBJECT, '<item objectid="1" transform="1e40 0 0 0 1 0 0 0 1 0 0 0"/>'))
    assert M.parse_three_mf(big).kind == "non-finite"


# ---------------------------------------------------------------- dispatch
def test_parse_model_sniffs_content():
    assert M.parse_model(fixture("stl/cube-binary.stl"), "x.obj").format == "stl"
    assert M.parse_model(fixture("obj/quad-cube.obj"), "x.stl").format == "obj"
    r = M.parse_model(fixture("3mf/single-object.3mf"), "x.bin")
    assert (r.format, r.unit_mm, r.item_count) == ("3mf", 1, 1)
    assert M.parse_model(b"ISO-10303-21;", "part.step").kind == "unsupported-cad"


@pytest.mark.parametrize("path,fmt,unit", [
    ("stl/cube-binary.stl", "stl", None), ("stl/cube-ascii-crlf.stl", "stl", None),
    ("stl/solid-header-binary.stl", "stl", None), ("3mf/single-object.3mf", "3mf", 1),
    ("obj/quad-cube.obj", "obj", None), ("3mf/inch.3mf", "3mf", 25.4)])
def test_parse_model_detects_content_regardless_of_extension(path, fmt, unit):
    """tests/unit/model/model.test.ts:6-22."""
    r = M.parse_model(fixture(path), "misnamed.step")
    assert (r.format, r.unit_mm, r.item_count, r.mesh.triangle_count) == (fmt, unit, 1, 12)


@pytest.mark.parametrize("name", ["part.step", "part.STP", "part.iges", "part.IGS"])
def test_parse_model_gives_an_export_hint_for_cad(name):
    """model.test.ts:23-29."""
    r = M.parse_model(b"ISO-10303-21;", name)
    assert r.kind == "unsupported-cad" and "Export" in r.message


def test_parse_model_keeps_errors_limits_and_dispatch():
    """model.test.ts:30-49: STL errors survive dispatch, the triangle limit holds
    in every format, invalid limits raise, and OBJ vertex text inside a binary
    STL header does not change the dispatch."""
    assert M.parse_model(fixture("stl/truncated.stl"), "bad.stl").kind == "truncated"
    for name in ("stl/cube-binary.stl", "3mf/single-object.3mf", "obj/quad-cube.obj"):
        assert M.parse_model(fixture(name), name, 11).kind == "too-many-triangles"
    for limit in (-1, math.nan, 0.5):
        with pytest.raises(RangeError):
            M.parse_model(b"", "x", limit)
    data = bytearray(fixture("stl/cube-binary.stl"))
    data[:8] = b"v 0 0 0\n"
    assert M.parse_model(bytes(data), "cube.obj").format == "stl"
