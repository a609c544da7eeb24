"""Mesh files for the voxelizer: STL (binary and ASCII), OBJ and 3MF.

Host-side restatement of the reference's importers with the same results and
error kinds (kind, byte offset, part):
* ``parse_stl``: src/geometry/stl.ts:118-150 (exact binary layout first, then
  ASCII ``solid`` grammar; triangle limit; finite float32 vertices);
* ``parse_obj``: src/geometry/obj.ts:63-88 (polygons as triangle fans, negative
  indices resolved at the face);
* ``read_zip`` / ``inflate_part``: src/geometry/zip.ts:40-191 (single-disk,
  stored or deflated, no encryption or ZIP64, sizes and CRC-32 checked);
* ``parse_three_mf``: src/geometry/threemf.ts:264-350 (start part from
  _rels/.rels, build items and nested components with row-vector transforms,
  units to millimetres);
* ``parse_model``: src/geometry/model.ts:25-52 (content sniffing).
Positions are float32, nine per triangle, as ``meshes.Mesh``.
"""
from __future__ import annotations

import math
import re
import struct
import urllib.parse
import zlib
from dataclasses import dataclass, field
from typing import Callable, Dict, List, Optional, Tuple, Union

import numpy as np

from ._lib import RangeError
from .meshes import Mesh

DEFAULT_MAX_TRIANGLES = 2_000_000
_DECIMAL = re.compile(r"^[+-]?(?:\d+(?:\.\d*)?|\.\d+)(?:[eE][+-]?\d+)?$")
_F32_MAX = float(np.finfo(np.float32).max)


@dataclass
class ModelParseError:
    kind: str  # truncated not-stl too-many-triangles empty non-finite zip-unsupported no-model-part bad-xml unsupported-cad
    byte_offset: int
    message: str
    part: Optional[str] = None


@dataclass
class ParsedModel:
    mesh: Mesh
    format: str  # 'stl' | '3mf' | 'obj'
    unit_mm: Optional[float]
    item_count: int


def _f32_finite(v: float) -> bool:
    """Math.fround(v) is finite: |v| rounds below the float32 overflow threshold."""
    if not math.isfinite(v):
        return False
    if abs(v) <= _F32_MAX:
        return True
    with np.errstate(over="ignore"):
        return bool(np.isfinite(np.float32(v)))


def _check_limit(max_triangles):
    if not isinstance(max_triangles, int) or isinstance(max_triangles, bool) or max_triangles < 0 \
            or max_triangles > 2 ** 53 - 1:
        raise RangeError("maxTriangles must be a non-negative safe integer.")


# ---------------------------------------------------------------- STL
_STL_MESSAGES = {
    "truncated": "The STL ends before the mesh is complete.",
    "not-stl": "The file does not contain a valid STL mesh.",
    "too-many-triangles": "The STL exceeds the triangle limit.",
    "empty": "The STL contains no triangles.",
    "non-finite": "A vertex cannot be represented as a finite float32 coordinate.",
}


def _stl_error(kind, offset):
    return ModelParseError(kind, offset, _STL_MESSAGES[kind])


_FACET = ("normal", None, None, None, "outer", "loop", "vertex", 0, 0, 0, "vertex", 0, 0, 0, "vertex", 0, 0, 0,
          "endloop", "endfacet")
_SPECIAL = re.compile(r"^[+-]?(?:NaN|Infinity)$", re.IGNORECASE)


def _parse_stl_ascii(text: str, max_triangles: int):
    head = re.match(r"solid[^\r\n]*(?:\r\n|[\r\n]|$)", text)
    if not head:
        return _stl_error("not-stl", 0)
    tokens = re.compile(r"\S+")
    pos = head.end()
    positions: List[float] = []
    count = 0
    while True:
        m = tokens.search(text, pos)
        if not m:
            return _stl_error("truncated", len(text))
        pos = m.end()
        word = m.group(0)
        if word == "endsolid":
            line_end = re.search(r"[\r\n]", text[pos:])
            if line_end:
                extra_at = pos + line_end.start()
                extra = re.search(r"\S", text[extra_at:])
                if extra:
                    return _stl_error("not-stl", extra_at + extra.start())
            if count == 0:
                return _stl_error("empty", m.start())
            return Mesh(np.asarray(positions, np.float32), count)
        if word != "facet":
            return _stl_error("not-stl", m.start())
        if count >= max_triangles:
            return _stl_error("too-many-triangles", m.start())
        for expected in _FACET:
            t = tokens.search(text, pos)
            if not t:
                return _stl_error("truncated", len(text))
            pos = t.end()
            tok = t.group(0)
            if expected is None:
                continue
            if expected != 0:
                if tok != expected:
                    return _stl_error("not-stl", t.start())
                continue
            if not _DECIMAL.match(tok) and not _SPECIAL.match(tok):
                return _stl_error("not-stl", t.start())
            value = float(tok) if _DECIMAL.match(tok) else float("nan")
            if not _f32_finite(value):
                return _stl_error("non-finite", t.start())
            positions.append(value)
        count += 1


def parse_stl(data: bytes, max_triangles: int = DEFAULT_MAX_TRIANGLES):
    """stl.ts:118-150: an exact binary record layout wins over ASCII."""
    _check_limit(max_triangles)
    data = bytes(data)
    has_count = len(data) >= 84
    count = struct.unpack_from("<I", data, 80)[0] if has_count else 0
    expected = 84 + 50 * count
    if has_count and expected == len(data):
        if count > max_triangles:
            return _stl_error("too-many-triangles", 80)
        if count == 0:
            return _stl_error("empty", 80)
        rec = np.frombuffer(data, np.uint8, count * 50, 84).reshape(count, 50)
        pos = rec[:, 12:48].copy().view("<f4").reshape(count, 9)
        bad = ~np.isfinite(pos)
        if bad.any():
            t, k = np.argwhere(bad)[0]
            return _stl_error("non-finite", 84 + 50 * int(t) + 12 + 4 * int(k))
        return Mesh(pos.astype(np.float32).reshape(-1), count)
    text = data.decode("latin-1")  # one character per byte keeps offsets
    if re.match(r"solid(?:\s|$)", text[:6]):
        return _parse_stl_ascii(text, max_triangles)
    if has_count and expected > len(data):
        if count > max_triangles:
            return _stl_error("too-many-triangles", 80)
        return _stl_error("truncated", len(data))
    return _stl_error("not-stl", 0)


# ---------------------------------------------------------------- OBJ
_FACE_REF = re.compile(r"^[+-]?\d+(?:/[+-]?\d+(?:/[+-]?\d+)?|//[+-]?\d+)?$")


def parse_obj(data: bytes, max_triangles: int = DEFAULT_MAX_TRIANGLES):
    """obj.ts:63-88: 'v' and 'f' records; faces as triangle fans."""
    _check_limit(max_triangles)
    text = bytes(data).decode("utf-8", errors="replace")
    if text.startswith("﻿"):
        text = text[1:]
    vertices: List[Tuple[float, float, float]] = []
    positions: List[float] = []
    offset = 0
    for m in re.finditer(r"[^\r\n]*(?:\r\n|[\r\n]|$)", text):
        line = m.group(0)
        if m.start() == len(text) and line == "":
            break
        fields = line.split("#", 1)[0].strip().split()
        tag = fields.pop(0) if fields else None
        if tag == "v":
            coords = fields[:3]
            if len(coords) != 3 or not all(_DECIMAL.match(c) for c in coords):
                return ModelParseError("not-stl", offset, "An OBJ vertex needs three numeric coordinates.")
            v = tuple(float(c) for c in coords)
            if not all(_f32_finite(c) for c in v):
                return ModelParseError("non-finite", offset, "An OBJ vertex exceeds the finite float32 range.")
            vertices.append(v)
        elif tag == "f":
            if len(fields) < 3:
                return ModelParseError("not-stl", offset, "An OBJ face needs at least three vertices.")
            face: List[Tuple[float, float, float]] = []
            for f in fields:
                if not _FACE_REF.match(f):
                    return ModelParseError("not-stl", offset, "An OBJ face contains an invalid vertex reference.")
                idx = int(f.split("/")[0])
                k = idx - 1 if idx > 0 else len(vertices) + idx
                if idx == 0 or not (0 <= k < len(vertices)):
                    return ModelParseError("not-stl", offset, "An OBJ face references a missing vertex.")
                face.append(vertices[k])
            if len(positions) // 9 + len(face) - 2 > max_triangles:
                return ModelParseError("too-many-triangles", offset, "The OBJ exceeds the triangle limit.")
            for i in range(1, len(face) - 1):
                positions.extend(face[0] + face[i] + face[i + 1])
        offset += len(line.encode("utf-8"))
    if not positions:
        return ModelParseError("empty", 0, "The OBJ contains no faces.")
    return Mesh(np.asarray(positions, np.float32), len(positions) // 9)


# ---------------------------------------------------------------- ZIP
MAX_EXPANDED_BYTES = 512 * 1024 * 1024


@dataclass
class ZipPart:
    name: str
    method: int
    size: int
    crc: int
    byte_offset: int
    compressed: bytes


def _zip64_extra(data: bytes, start: int, end: int) -> bool:
    off = start
    while off < end:
        if off + 4 > end:
            return True
        tag, length = struct.unpack_from("<HH", data, off)
        if tag == 1 or off + 4 + length > end:
            return True
        off += 4 + length
    return False


def read_zip(data: bytes):
    """zip.ts:40-150: index the members of an ordinary single-disk archive."""
    data = bytes(data)
    u16 = lambda o: struct.unpack_from("<H", data, o)[0]
    u32 = lambda o: struct.unpack_from("<I", data, o)[0]
    end = len(data) - 22
    minimum = max(0, end - 65535)
    while end >= minimum:
        if u32(end) == 0x06054B50 and end + 22 + u16(end + 20) == len(data):
            break
        end -= 1
    if end < minimum:
        return ModelParseError("truncated", len(data), "The ZIP directory is missing.")
    count, dir_size, off = u16(end + 10), u32(end + 12), u32(end + 16)
    if (count == 0xFFFF or dir_size == 0xFFFFFFFF or off == 0xFFFFFFFF
            or (end >= 20 and u32(end - 20) == 0x07064B50)
            or u16(end + 4) != 0 or u16(end + 6) != 0 or u16(end + 8) != count):
        return ModelParseError("zip-unsupported", end, "ZIP64 and multi-disk archives are unsupported.")
    if off + dir_size != end:
        return ModelParseError("truncated", off, "The ZIP directory has an invalid size or offset.")
    parts: Dict[str, ZipPart] = {}
    expanded = 0
    for _ in range(count):
        if off + 46 > end or u32(off) != 0x02014B50:
            return ModelParseError("truncated", off, "A ZIP directory entry is incomplete.")
        flags, method = u16(off + 8), u16(off + 10)
        csize, size = u32(off + 20), u32(off + 24)
        nlen, xlen, clen = u16(off + 28), u16(off + 30), u16(off + 32)
        nxt = off + 46 + nlen + xlen + clen
        local = u32(off + 42)
        if nxt > end:
            return ModelParseError("truncated", off, "A ZIP entry extends beyond its directory.")
        if ((flags & 0x41) != 0 or method not in (0, 8) or size == 0xFFFFFFFF or csize == 0xFFFFFFFF
                or local == 0xFFFFFFFF or u16(off + 34) != 0
                or _zip64_extra(data, off + 46 + nlen, off + 46 + nlen + xlen)):
            return ModelParseError("zip-unsupported", off, "Use a ZIP without encryption or ZIP64, stored or deflated.")
        if local + 30 > off or u32(local) != 0x04034B50:
            return ModelParseError("truncated", local, "A ZIP local header is missing.")
        if (u16(local + 6) & 0x41) != 0 or u16(local + 8) != method:
            return ModelParseError("zip-unsupported", local, "ZIP local compression flags disagree with the directory.")
        lnlen, lxlen = u16(local + 26), u16(local + 28)
        start = local + 30 + lnlen + lxlen
        if start + csize > off:
            return ModelParseError("truncated", start, "A ZIP member is incomplete.")
        if _zip64_extra(data, start - lxlen, start):
            return ModelParseError("zip-unsupported", local, "ZIP64 members are unsupported.")
        name = data[off + 46:off + 46 + nlen].decode("utf-8", errors="replace")
        lname = data[local + 30:local + 30 + lnlen].decode("utf-8", errors="replace")
        if name != lname or name in parts:
            return ModelParseError("zip-unsupported", local, "ZIP member names disagree or are duplicated.")
        expanded += size
        if expanded > MAX_EXPANDED_BYTES:
            return ModelParseError("zip-unsupported", off, "The expanded ZIP exceeds 512 MiB.")
        parts[name] = ZipPart(name, method, size, u32(off + 16), start, data[start:start + csize])
        off = nxt
    if off != end:
        return ModelParseError("truncated", off, "The ZIP directory count is incorrect.")
    return parts


def inflate_part(part: ZipPart):
    """zip.ts:153-191: expand a member, checking its size and CRC-32."""
    def fail(msg):
        return ModelParseError("truncated", part.byte_offset, msg, part.name)
    out = part.compressed
    if part.method == 8:
        try:
            d = zlib.decompressobj(-15)
            out = d.decompress(part.compressed, part.size + 1)
            if len(out) > part.size:
                return fail("The ZIP member expands beyond its declared size.")
            if not d.eof:
                rest = d.decompress(d.unconsumed_tail, 1)
                if rest:
                    return fail("The ZIP member expands beyond its declared size.")
        except zlib.error:
            return fail("The ZIP member contains invalid raw-deflate data.")
        if len(out) != part.size:
            return fail("The ZIP member expands to an incorrect size.")
    if len(out) != part.size or (zlib.crc32(out) & 0xFFFFFFFF) != part.crc:
        return fail("The ZIP member size or checksum is incorrect.")
    return out


# ---------------------------------------------------------------- 3MF
class _BadXml(Exception):
    pass


class _TooMany(Exception):
    pass


_UNITS = {"micron": 0.001, "millimeter": 1.0, "centimeter": 10.0, "inch": 25.4, "foot": 304.8, "meter": 1000.0}
_IDENTITY = [1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0]
_TAGS = re.compile(r"<!--[\s\S]*?-->|<\?[\s\S]*?\?>|<!\[CDATA\[[\s\S]*?\]\]>|"
                   r"</?[A-Za-z_][\w.:-]*(?:[^<>\"']|\"[^\"]*\"|'[^']*')*>")
_ATTR = re.compile(r"\s+([A-Za-z_][\w.:-]*)\s*=\s*(?:\"([^\"<]*)\"|'([^'<]*)')")


def _unescape(value: str) -> str:
    named = {"amp": "&", "lt": "<", "gt": ">", "quot": '"', "apos": "'"}

    def sub(m):
        ent = m.group(1)
        if ent is not None and ent in named:
            return named[ent]
        if ent is not None and re.match(r"^#(?:\d+|x[\da-fA-F]+)$", ent):
            code = int(ent[2:], 16) if ent.startswith("#x") else int(ent[1:])
            if 0 < code <= 0x10FFFF and not (0xD800 <= code <= 0xDFFF):
                return chr(code)
        raise _BadXml("The XML contains an unknown or invalid entity.")
    return re.sub(r"&([^;]*);|&", sub, value)


def _attributes(token: str, name: str) -> Dict[str, str]:
    attrs: Dict[str, str] = {}
    cursor = len(name) + 1
    while True:
        m = _ATTR.match(token, cursor)
        if not m:
            break
        key = m.group(1)
        if key in attrs:
            raise _BadXml("The XML has duplicate attributes.")
        value = m.group(2) if m.group(2) is not None else (m.group(3) or "")
        attrs[key] = _unescape(value) if "&" in value else value
        cursor = m.end()
    if not re.match(r"^\s*/?>$", token[cursor:]):
        raise _BadXml("The XML attributes must be quoted.")
    return attrs


def _scan_xml(text: str, visit: Callable[[str, Dict[str, str]], None]) -> None:
    """A strict scanner of the XML the 3MF parts use: element paths by local
    name, attributes, comments, processing instructions and CDATA skipped."""
    stack: List[str] = []
    paths: List[str] = []
    offset = 0
    roots = 0
    for m in _TAGS.finditer(text):
        gap = text[offset:m.start()]
        if "<" in gap or (not stack and gap.strip()):
            raise _BadXml("The XML contains malformed text.")
        token = m.group(0)
        offset = m.end()
        if token.startswith("<?") or token.startswith("<!"):
            continue
        nm = re.match(r"^</?([\w.:-]+)", token)
        if not nm:
            raise _BadXml("The XML element has no name.")
        name = nm.group(1)
        if token.startswith("</"):
            if not re.match(r"^</[\w.:-]+\s*>$", token):
                raise _BadXml("The XML closing tag is malformed.")
            if not stack or stack.pop() != name:
                raise _BadXml("The XML elements are not balanced.")
            paths.pop()
            continue
        if not stack:
            roots += 1
        local = name[name.rfind(":") + 1:]
        path = f"{paths[-1]}/{local}" if paths else local
        visit(path, _attributes(token, name))
        if not token.endswith("/>"):
            stack.append(name)
            paths.append(path)
    if stack or roots != 1 or text[offset:].strip():
        raise _BadXml("The XML document is incomplete.")


def _number(v: Optional[str]) -> float:
    if v is None or not _DECIMAL.match(v) or not math.isfinite(float(v)):
        raise _BadXml("A model coordinate or transform is not a finite number.")
    return float(v)


@dataclass
class _Ref:
    id: str
    path: str
    transform: List[float]


@dataclass
class _Object:
    vertices: List[float] = field(default_factory=list)
    indices: List[int] = field(default_factory=list)
    components: List[_Ref] = field(default_factory=list)


def _reference(attrs: Dict[str, str]) -> _Ref:
    oid = attrs.get("objectid")
    if not oid:
        raise _BadXml("A component or build item is missing its object ID.")
    t = _IDENTITY if "transform" not in attrs else [_number(v) for v in attrs["transform"].strip().split()]
    if len(t) != 12:
        raise _BadXml("A 3MF transform must contain twelve numbers.")
    path = next((v for k, v in attrs.items() if k.endswith(":path")), "")
    return _Ref(oid, path, t)


def _index(v: Optional[str]) -> int:
    if v is None or not re.match(r"^\d+$", v) or int(v) > 2 ** 53 - 1:
        raise _BadXml("A triangle index is invalid.")
    return int(v)


def _parse_part(text: str, max_triangles: int):
    objects: Dict[str, _Object] = {}
    items: List[_Ref] = []
    state = {"unit": 1.0, "model": False, "current": None}

    def visit(path, attrs):
        if path == "model":
            state["model"] = True
            unit = attrs.get("unit", "millimeter")
            if unit not in _UNITS:
                raise _BadXml("The 3MF unit is unsupported.")
            state["unit"] = _UNITS[unit]
        elif path == "model/resources/object":
            oid = attrs.get("id")
            if not oid or oid in objects:
                raise _BadXml("An object ID is missing or duplicated.")
            state["current"] = objects[oid] = _Object()
        elif path == "model/resources/object/mesh/vertices/vertex":
            if state["current"] is not None:
                state["current"].vertices.extend((_number(attrs.get("x")), _number(attrs.get("y")),
                                                  _number(attrs.get("z"))))
        elif path == "model/resources/object/mesh/triangles/triangle":
            cur = state["current"]
            if cur is not None:
                if len(cur.indices) // 3 >= max_triangles:
                    raise _TooMany("The 3MF exceeds the triangle limit.")
                cur.indices.extend((_index(attrs.get("v1")), _index(attrs.get("v2")), _index(attrs.get("v3"))))
        elif path == "model/resources/object/components/component":
            if state["current"] is not None:
                state["current"].components.append(_reference(attrs))
        elif path == "model/build/item":
            items.append(_reference(attrs))

    _scan_xml(text, visit)
    if not state["model"]:
        raise _BadXml("The model part has no model root.")
    for obj in objects.values():
        if obj.components and obj.indices:
            raise _BadXml("An object cannot contain both a mesh and components.")
        if any(i * 3 >= len(obj.vertices) for i in obj.indices):
            raise _BadXml("A triangle references a missing vertex.")
    return objects, items, state["unit"]


def _part_path(base: str, target: str) -> str:
    decoded = urllib.parse.unquote(target)
    if re.search(r"[?#\\]", decoded) or re.match(r"^[a-z]+:", decoded, re.IGNORECASE):
        raise _BadXml("A model part path is invalid.")
    segments = [] if decoded.startswith("/") else base.split("/")[:-1]
    for seg in decoded.split("/"):
        if seg == "..":
            if not segments or not segments.pop():
                raise _BadXml("A model part path leaves the archive root.")
        elif seg and seg != ".":
            segments.append(seg)
    return "/".join(segments)


def parse_three_mf(data: bytes, max_triangles: int = DEFAULT_MAX_TRIANGLES):
    """threemf.ts:264-350: merge all build items and component instances into
    millimetre triangle positions; (mesh, unit_mm, item_count) or an error."""
    _check_limit(max_triangles)
    parts = read_zip(data)
    if isinstance(parts, ModelParseError):
        return parts
    active = ["_rels/.rels"]

    def read_text(path):
        part = parts.get(path)
        if part is None:
            return ModelParseError("no-model-part", 0, "The referenced 3MF part is missing.", path)
        raw = inflate_part(part)
        if isinstance(raw, ModelParseError):
            return raw
        try:
            return raw.decode("utf-8")
        except UnicodeDecodeError:
            raise _BadXml("The model part is not valid UTF-8.")

    try:
        root_path = "3D/3dmodel.model"
        if active[0] in parts:
            rels = read_text(active[0])
            if isinstance(rels, ModelParseError):
                return rels
            found = []

            def visit_rel(path, attrs):
                if path == "Relationships/Relationship" and re.search(r"(?:/3dmodel|/StartPart|^StartPart)$",
                                                                      attrs.get("Type", "")):
                    if attrs.get("TargetMode") == "External" or not attrs.get("Target"):
                        raise _BadXml("The start model must be an archive part.")
                    found.append(_part_path("", attrs["Target"]))
            _scan_xml(rels, visit_rel)
            if found:
                root_path = found[-1]
        cache = {}

        def load(path):
            active[0] = path
            if path in cache:
                return cache[path]
            text = read_text(path)
            if isinstance(text, ModelParseError):
                return text
            cache[path] = _parse_part(text, max_triangles)
            return cache[path]

        root = load(root_path)
        if isinstance(root, ModelParseError):
            return root
        unit = root[2]
        instances = []
        total = [0]

        def expand(ref: _Ref, path: str, transforms: list, ancestors: set):
            target = _part_path(path, ref.path) if ref.path else path
            key = f"{target}#{ref.id}"
            if key in ancestors or len(ancestors) >= 128:
                raise _BadXml("The component hierarchy is cyclic or too deep.")
            model = load(target)
            if isinstance(model, ModelParseError):
                return model
            if model[2] != unit:
                raise _BadXml("All 3MF model parts must use the same unit.")
            obj = model[0].get(ref.id)
            if obj is None:
                raise _BadXml("A build item or component references a missing object.")
            chain = [ref.transform] + transforms  # component transforms act first (row vectors)
            ancestors.add(key)
            for child in obj.components:
                err = expand(child, target, chain, ancestors)
                if err is not None:
                    return err
            ancestors.discard(key)
            total[0] += len(obj.indices) // 3
            if total[0] > max_triangles:
                raise _TooMany("The 3MF exceeds the triangle limit.")
            instances.append((obj, chain))
            return None

        for item in root[1]:
            err = expand(item, root_path, [], set())
            if err is not None:
                return err
        if total[0] == 0:
            return ModelParseError("empty", 0, "The 3MF build contains no triangles.", root_path)
        out = []
        for obj, chain in instances:
            v = np.asarray(obj.vertices, np.float64).reshape(-1, 3)
            for m in chain:
                a, b, c, d, e, f, g, h, i, tx, ty, tz = m
                v = np.stack([v[:, 0] * a + v[:, 1] * d + v[:, 2] * g + tx,
                              v[:, 0] * b + v[:, 1] * e + v[:, 2] * h + ty,
                              v[:, 0] * c + v[:, 1] * f + v[:, 2] * i + tz], axis=1)
            with np.errstate(over="ignore", invalid="ignore"):
                vf = (v * unit).astype(np.float32)
            if not np.isfinite(vf).all():
                return ModelParseError("non-finite", 0, "A transformed 3MF vertex exceeds the finite float32 range.")
            out.append(vf[np.asarray(obj.indices, np.int64)].reshape(-1))
        positions = np.concatenate(out).astype(np.float32)
        return Mesh(positions, total[0]), unit, len(root[1])
    except _TooMany as e:
        return ModelParseError("too-many-triangles", 0, str(e), active[0])
    except _BadXml as e:
        return ModelParseError("bad-xml", 0, str(e), active[0])


# ---------------------------------------------------------------- dispatch
def _text_format(data: bytes):
    if len(data) >= 84 and 84 + struct.unpack_from("<I", data, 80)[0] * 50 == len(data):
        return "stl"
    text = data.decode("utf-8", errors="replace")
    if re.match(r"solid(?:\s|$)", text):
        return "stl"
    return "obj" if re.search(r"^\s*v[ \t]+", text, re.MULTILINE) else None


def parse_model(data: bytes, file_name: str = "", max_triangles: int = DEFAULT_MAX_TRIANGLES):
    """model.ts:25-52: sniff the content (not the name); CAD files get an export hint."""
    _check_limit(max_triangles)
    data = bytes(data)
    if len(data) >= 4 and struct.unpack_from("<I", data, 0)[0] == 0x04034B50:
        r = parse_three_mf(data, max_triangles)
        if isinstance(r, ModelParseError):
            return r
        mesh, unit, items = r
        return ParsedModel(mesh, "3mf", unit, items)
    fmt = _text_format(data)
    if fmt is None and re.search(r"\.(?:step|stp|iges|igs)$", file_name, re.IGNORECASE):
        return ModelParseError("unsupported-cad", 0, "Export this CAD model as STL, 3MF or OBJ before importing it.")
    fmt = fmt or "stl"
    mesh = parse_obj(data, max_triangles) if fmt == "obj" else parse_stl(data, max_triangles)
    if isinstance(mesh, ModelParseError):
        return mesh
    return ParsedModel(mesh, fmt, None, 1)
