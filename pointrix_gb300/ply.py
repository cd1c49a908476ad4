"""Gaussian scenes as PLY files, in the layout Pointrix saves and loads.

``PointCloud.save_ply`` / ``load_ply`` (``pointrix/model/point_cloud/points.py:360-426``)
write one ``vertex`` element of float32 properties through the ``plyfile``
package: ``x y z nx ny nz`` (normals all zero), then every registered
attribute but the position, flattened row-major as ``<name>_<i>``.  For a
``GaussianPointCloud`` (``gaussian_points.py:28-52``) the attributes are, in
order, ``features`` [N,1,3] (the SH DC term), ``features_rest`` [N,K-1,3],
``scaling`` [N,3] (log scale), ``rotation`` [N,4] (wxyz, not normalised) and
``opacity`` [N,1] (logit): the raw parameters, before activation.

This module reads and writes that format without ``plyfile``: the header is
parsed here, and the vertex block of a binary file is read in one
``numpy.fromfile`` as a structured array (no Python loop over records), so
a 1M-Gaussian SH-3 scene (248 MB) loads at disk speed.  Reading follows the
PLY 1.0 format: ``ascii``, ``binary_little_endian`` and
``binary_big_endian``; every scalar type under both its names; list
properties (read record by record, as they have no fixed stride).  Writing
produces what ``plyfile`` writes for Pointrix: ``binary_little_endian``,
canonical type names, no comments.
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field

import numpy as np
import torch

# PLY type names (both spellings of the format) -> numpy type codes
_TYPES = {
    "char": "i1", "int8": "i1", "uchar": "u1", "uint8": "u1",
    "short": "i2", "int16": "i2", "ushort": "u2", "uint16": "u2",
    "int": "i4", "int32": "i4", "uint": "u4", "uint32": "u4",
    "float": "f4", "float32": "f4", "double": "f8", "float64": "f8",
}
# numpy type codes -> the canonical name a writer uses
_NAMES = {"i1": "char", "u1": "uchar", "i2": "short", "u2": "ushort",
          "i4": "int", "u4": "uint", "f4": "float", "f8": "double"}
_FORMATS = {"ascii": None, "binary_little_endian": "<", "binary_big_endian": ">"}


@dataclass
class PlyProperty:
    name: str
    type: str                    # numpy code of a scalar, or of a list's items
    count_type: str | None = None  # numpy code of a list's length, None for a scalar


@dataclass
class PlyElement:
    name: str
    count: int
    properties: list = field(default_factory=list)


def _parse_header(f):
    """(format, elements, offset of the data) of an open binary file."""
    if f.readline().rstrip(b"\r\n") != b"ply":
        raise ValueError("not a PLY file (no 'ply' magic line)")
    fmt, elements = None, []
    while True:
        raw = f.readline()
        if not raw:
            raise ValueError("PLY header has no end_header line")
        words = raw.decode("ascii").split()
        if not words or words[0] in ("comment", "obj_info"):
            continue
        if words[0] == "end_header":
            break
        if words[0] == "format":
            if len(words) != 3 or words[1] not in _FORMATS or words[2] != "1.0":
                raise ValueError(f"unsupported PLY format line: {raw!r}")
            fmt = words[1]
        elif words[0] == "element":
            if len(words) != 3:
                raise ValueError(f"bad PLY element line: {raw!r}")
            elements.append(PlyElement(words[1], int(words[2])))
        elif words[0] == "property":
            if not elements:
                raise ValueError("PLY property before any element")
            if words[1] == "list":
                if len(words) != 5 or words[2] not in _TYPES or words[3] not in _TYPES:
                    raise ValueError(f"bad PLY list property line: {raw!r}")
                prop = PlyProperty(words[4], _TYPES[words[3]], _TYPES[words[2]])
            else:
                if len(words) != 3 or words[1] not in _TYPES:
                    raise ValueError(f"bad PLY property line: {raw!r}")
                prop = PlyProperty(words[2], _TYPES[words[1]])
            elements[-1].properties.append(prop)
        else:
            raise ValueError(f"unknown PLY header line: {raw!r}")
    if fmt is None:
        raise ValueError("PLY header has no format line")
    return fmt, elements, f.tell()


def _scalar_dtype(el: PlyElement, order: str) -> np.dtype:
    names = [p.name for p in el.properties]
    if len(set(names)) != len(names):
        raise ValueError(f"PLY element {el.name!r} repeats a property name")
    return np.dtype([(p.name, order + p.type) for p in el.properties])


def _record_dtype(el: PlyElement, order: str) -> np.dtype:
    # lists become object fields (one array per record)
    return np.dtype([(p.name, object if p.count_type else order + p.type)
                     for p in el.properties])


def _read_binary(f, order: str, elements, offset: int) -> dict:
    out, pos = {}, offset
    for el in elements:
        f.seek(pos)
        if all(p.count_type is None for p in el.properties):
            dt = _scalar_dtype(el, order)
            arr = np.fromfile(f, dtype=dt, count=el.count)
            if arr.shape[0] != el.count:
                raise ValueError(f"PLY element {el.name!r} is truncated: "
                                 f"{arr.shape[0]} of {el.count} records")
            pos += dt.itemsize * el.count
        else:  # no fixed stride: one record at a time
            arr = np.empty(el.count, dtype=_record_dtype(el, order))
            for r in range(el.count):
                for p in el.properties:
                    if p.count_type is None:
                        arr[p.name][r] = _take(f, order + p.type, 1, el)[0]
                    else:
                        n = int(_take(f, order + p.count_type, 1, el)[0])
                        arr[p.name][r] = _take(f, order + p.type, n, el)
            pos = f.tell()
        out[el.name] = arr
    return out


def _take(f, code: str, n: int, el: PlyElement) -> np.ndarray:
    dt = np.dtype(code)
    raw = f.read(dt.itemsize * n)
    if len(raw) != dt.itemsize * n:
        raise ValueError(f"PLY element {el.name!r} is truncated")
    return np.frombuffer(raw, dtype=dt, count=n).copy()


def _read_ascii(f, elements, offset: int) -> dict:
    f.seek(offset)
    tokens = f.read().split()
    out, at = {}, 0
    for el in elements:
        if all(p.count_type is None for p in el.properties):
            width = len(el.properties)
            need = width * el.count
            if at + need > len(tokens):
                raise ValueError(f"PLY element {el.name!r} is truncated")
            table = np.array(tokens[at:at + need], dtype=object).reshape(el.count, width)
            arr = np.empty(el.count, dtype=_scalar_dtype(el, "<"))
            for j, p in enumerate(el.properties):
                arr[p.name] = _parse_column(table[:, j], p.type)
            at += need
        else:
            arr = np.empty(el.count, dtype=_record_dtype(el, "<"))
            for r in range(el.count):
                for p in el.properties:
                    if p.count_type is None:
                        arr[p.name][r] = _parse_column([_word(tokens, at, el)], p.type)[0]
                        at += 1
                    else:
                        n = int(_word(tokens, at, el))
                        _word(tokens, at + n, el)  # the list's last item is there
                        arr[p.name][r] = _parse_column(tokens[at + 1:at + 1 + n], p.type)
                        at += 1 + n
        out[el.name] = arr
    return out


def _word(tokens, at: int, el: PlyElement):
    if at >= len(tokens):
        raise ValueError(f"PLY element {el.name!r} is truncated")
    return tokens[at]


def _parse_column(words, code: str) -> np.ndarray:
    text = np.array([w.decode("ascii") for w in words])
    if code[0] == "f":
        return text.astype(np.float64).astype(code)
    return text.astype(np.int64).astype(code)


def read_ply(path) -> dict:
    """Every element of a PLY file, as ``{element name: structured array}``
    with one field per property (list properties as object fields holding
    one array per record)."""
    with open(path, "rb") as f:
        fmt, elements, offset = _parse_header(f)
        if fmt == "ascii":
            return _read_ascii(f, elements, offset)
        return _read_binary(f, _FORMATS[fmt], elements, offset)


def write_ply(path, element: str, properties: dict) -> None:
    """One element of scalar properties, in the given order, as a
    ``binary_little_endian`` PLY file (the layout ``plyfile`` writes)."""
    names = list(properties)
    if not names:
        raise ValueError("write_ply needs at least one property")
    cols = [np.asarray(properties[n]) for n in names]
    count = cols[0].shape[0]
    codes = []
    for n, c in zip(names, cols):
        if c.ndim != 1 or c.shape[0] != count:
            raise ValueError(f"property {n!r} must be 1-D with {count} entries")
        code = c.dtype.str[1:]
        if code not in _NAMES:
            raise ValueError(f"property {n!r} has a type PLY cannot store: {c.dtype}")
        codes.append(code)
    arr = np.empty(count, dtype=np.dtype([(n, "<" + c) for n, c in zip(names, codes)]))
    for n, c in zip(names, cols):
        arr[n] = c
    head = ["ply", "format binary_little_endian 1.0", f"element {element} {count}"]
    head += [f"property {_NAMES[c]} {n}" for n, c in zip(names, codes)]
    head.append("end_header")
    parent = os.path.dirname(os.fspath(path))
    if parent:
        os.makedirs(parent, exist_ok=True)
    with open(path, "wb") as f:
        f.write(("\n".join(head) + "\n").encode("ascii"))
        arr.tofile(f)


# -- the Gaussian point cloud layout -----------------------------------------

def _attribute_widths(k: int):
    """(attribute, floats per Gaussian) after the position and the normals,
    in the order ``GaussianPointCloud`` registers them (features first, from
    ``points.py:51-59``, then ``gaussian_points.py:48-51``)."""
    return (("features", 3), ("features_rest", 3 * (k - 1)), ("scaling", 3),
            ("rotation", 4), ("opacity", 1))


def gaussian_property_names(sh_degree: int = 3) -> list:
    """The vertex properties of a Gaussian point cloud's PLY file, in file
    order (``points.py:360-370``): 62 for SH degree 3."""
    if sh_degree < 0:
        raise ValueError("sh_degree must be >= 0")
    names = ["x", "y", "z", "nx", "ny", "nz"]
    for attr, width in _attribute_widths((sh_degree + 1) ** 2):
        names += [f"{attr}_{i}" for i in range(width)]
    return names


def _sh_degree_of(k: int) -> int:
    d = int(round(k ** 0.5)) - 1
    if d < 0 or (d + 1) ** 2 != k:
        raise ValueError(f"{k} SH coefficients per channel is not (degree + 1)^2")
    return d


def save_gaussians(path, scene) -> None:
    """Writes a :class:`~pointrix_gb300.workloads.Scene` (raw parameters:
    position, log scale, unnormalised wxyz quaternion, opacity logit, SH
    [N,K,3]) as ``GaussianPointCloud.save_ply`` lays it out."""
    n, k = scene.n, scene.shs.shape[1]
    names = gaussian_property_names(_sh_degree_of(k))
    host = lambda t: t.detach().to("cpu", torch.float32).reshape(n, -1)  # noqa: E731
    table = torch.cat([host(scene.position), torch.zeros(n, 3),
                       host(scene.shs[:, :1, :]), host(scene.shs[:, 1:, :]),
                       host(scene.log_scale), host(scene.quat_raw),
                       host(scene.opacity_logit)], dim=1).numpy()
    if table.shape[1] != len(names):
        raise ValueError(f"scene has {table.shape[1]} floats per Gaussian, "
                         f"the layout {len(names)}")
    head = ["ply", "format binary_little_endian 1.0", f"element vertex {n}"]
    head += [f"property float {x}" for x in names]
    head.append("end_header")
    parent = os.path.dirname(os.fspath(path))
    if parent:
        os.makedirs(parent, exist_ok=True)
    with open(path, "wb") as f:
        f.write(("\n".join(head) + "\n").encode("ascii"))
        np.ascontiguousarray(table, dtype="<f4").tofile(f)


def load_gaussians(path, device="cpu"):
    """Reads a Gaussian point cloud PLY file (``GaussianPointCloud.load_ply``,
    ``points.py:399-426``: properties found by name, the SH degree from the
    number of ``features_rest_*``) into a
    :class:`~pointrix_gb300.workloads.Scene` of float32 tensors on
    ``device``.  A file in the exact layout ``save_ply`` writes is reinterpreted
    in place as an [N, 62] table and copied to the device in one transfer."""
    from .workloads import Scene

    data = read_ply(path)
    if "vertex" not in data:
        raise ValueError(f"{path}: no 'vertex' element")
    v = data["vertex"]
    have = v.dtype.names or ()
    rest = sum(1 for x in have if x.startswith("features_rest_"))
    if rest % 3:
        raise ValueError(f"{path}: {rest} features_rest properties is not a multiple of 3")
    k = rest // 3 + 1
    names = gaussian_property_names(_sh_degree_of(k))
    missing = [x for x in names if x not in have]
    if missing:
        raise ValueError(f"{path}: missing properties {missing[:6]}")
    n = v.shape[0]
    if have == tuple(names) and all(v.dtype[i] == np.dtype("<f4") for i in range(len(names))):
        table = v.view("<f4").reshape(n, len(names))  # the file's own bytes
    else:
        table = np.stack([v[x].astype(np.float32) for x in names], axis=1)
    t = torch.from_numpy(np.ascontiguousarray(table, dtype=np.float32)).to(device)
    at, parts = 6, {}
    for attr, width in _attribute_widths(k):
        parts[attr] = t[:, at:at + width]
        at += width
    shs = torch.cat([parts["features"].reshape(n, 1, 3),
                     parts["features_rest"].reshape(n, k - 1, 3)], dim=1)
    return Scene(t[:, 0:3].contiguous(), parts["scaling"].contiguous(),
                 parts["rotation"].contiguous(), parts["opacity"].contiguous(),
                 shs.contiguous())


def resident_scene(path, device="cuda"):
    """A PLY file loaded straight into a scene the render server keeps on
    the device (activated parameters)."""
    from .serve import ResidentScene

    return ResidentScene(*load_gaussians(path, device).activated(), device=device)
