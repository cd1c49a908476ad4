"""PLY scenes on CPU: the Gaussian point cloud layout Pointrix writes
(``pointrix/model/point_cloud/points.py:360-426``), round trips, files
written by hand in every PLY 1.0 encoding, and malformed files."""
import struct

import numpy as np
import pytest
import torch

from pointrix_gb300 import ply
from pointrix_gb300 import workloads as WL


def _equal_scenes(a, b):
    for x, y in zip((a.position, a.log_scale, a.quat_raw, a.opacity_logit, a.shs),
                    (b.position, b.log_scale, b.quat_raw, b.opacity_logit, b.shs)):
        assert x.shape == y.shape and torch.equal(x.float(), y), (x.shape, y.shape)


def test_property_names_follow_the_attribute_order():
    names = ply.gaussian_property_names(3)
    # points.py:363-370: position and normals, then each attribute flattened
    expect = ["x", "y", "z", "nx", "ny", "nz"] + [f"features_{i}" for i in range(3)]
    expect += [f"features_rest_{i}" for i in range(45)] + [f"scaling_{i}" for i in range(3)]
    expect += [f"rotation_{i}" for i in range(4)] + ["opacity_0"]
    assert names == expect and len(names) == 62
    assert len(ply.gaussian_property_names(0)) == 17


@pytest.mark.parametrize("maker", ["sh0", "sh3"])
def test_round_trip_is_exact(tmp_path, maker):
    scene = WL.scene_small(0, 500)[0] if maker == "sh0" else WL.scene_sh3(4, 777)
    path = tmp_path / "point_cloud" / "scene.ply"  # the parent is created, as save_ply does
    ply.save_gaussians(path, scene)
    _equal_scenes(scene, ply.load_gaussians(path))
    k = scene.shs.shape[1]
    assert path.stat().st_size == len(_header(scene.n, k)) + scene.n * 4 * (14 + 3 * k)


def _header(n, k):
    names = ply.gaussian_property_names(int(round(k ** 0.5)) - 1)
    lines = ["ply", "format binary_little_endian 1.0", f"element vertex {n}"]
    lines += [f"property float {x}" for x in names] + ["end_header"]
    return ("\n".join(lines) + "\n").encode()


def test_file_bytes_are_the_plyfile_layout(tmp_path):
    scene = WL.scene_sh3(5, 3)
    path = tmp_path / "s.ply"
    ply.save_gaussians(path, scene)
    raw = path.read_bytes()
    head = _header(3, 16)
    assert raw.startswith(head)
    body = np.frombuffer(raw[len(head):], dtype="<f4").reshape(3, 62)
    # the record of Gaussian 1, field by field
    assert np.array_equal(body[1, 0:3], scene.position[1].numpy())
    assert np.array_equal(body[1, 3:6], np.zeros(3, np.float32))
    assert np.array_equal(body[1, 6:9], scene.shs[1, 0].numpy())
    # features_rest_{3j+c} is coefficient j+1 of channel c (row-major [K-1, 3])
    assert np.array_equal(body[1, 9:54].reshape(15, 3), scene.shs[1, 1:].numpy())
    assert np.array_equal(body[1, 54:57], scene.log_scale[1].numpy())
    assert np.array_equal(body[1, 57:61], scene.quat_raw[1].numpy())
    assert body[1, 61] == scene.opacity_logit[1, 0]


def _sh0_columns(n, seed=0):
    g = np.random.default_rng(seed)
    return {x: g.standard_normal(n).astype(np.float32) for x in ply.gaussian_property_names(0)}


def test_properties_found_by_name_in_any_order_and_type(tmp_path):
    cols = _sh0_columns(6)
    names = list(cols)[::-1]  # reversed order, one column double, an extra property
    props = {x: cols[x] for x in names}
    props["opacity_0"] = props["opacity_0"].astype(np.float64)
    props["label"] = np.arange(6, dtype=np.int32)
    ply.write_ply(tmp_path / "r.ply", "vertex", props)
    s = ply.load_gaussians(tmp_path / "r.ply")
    assert torch.equal(s.position, torch.from_numpy(np.stack([cols[c] for c in "xyz"], 1)))
    assert torch.equal(s.opacity_logit[:, 0], torch.from_numpy(cols["opacity_0"]))
    assert torch.equal(s.shs[:, 0], torch.from_numpy(
        np.stack([cols[f"features_{i}"] for i in range(3)], 1)))


def test_resident_scene_holds_activated_parameters(tmp_path):
    scene = WL.scene_sh3(6, 64)
    ply.save_gaussians(tmp_path / "s.ply", scene)
    r = ply.resident_scene(tmp_path / "s.ply", device="cpu")
    pos, sc, q, op, shs = scene.activated()
    assert torch.equal(r.position, pos) and torch.equal(r.scaling, sc)
    assert torch.equal(r.rotation, q) and torch.equal(r.opacity, op) and torch.equal(r.shs, shs)


# -- files written by hand --------------------------------------------------

ASCII = b"""ply
format ascii 1.0
comment made by hand
element vertex 3
property float x
property uchar red
property int16 t
element face 2
property list uchar int vertex_indices
end_header
0.5 255 -3
-1e-3 0 7
2 17 -32768
3 0 1 2
0
"""


def test_ascii_with_a_list_element(tmp_path):
    (tmp_path / "a.ply").write_bytes(ASCII)
    d = ply.read_ply(tmp_path / "a.ply")
    v, f = d["vertex"], d["face"]
    assert v["x"].dtype == np.float32 and np.array_equal(v["x"], np.float32([0.5, -1e-3, 2]))
    assert v["red"].dtype == np.uint8 and list(v["red"]) == [255, 0, 17]
    assert v["t"].dtype == np.int16 and list(v["t"]) == [-3, 7, -32768]
    assert list(f["vertex_indices"][0]) == [0, 1, 2] and len(f["vertex_indices"][1]) == 0


def _binary(order):
    fmt = "binary_big_endian" if order == ">" else "binary_little_endian"
    head = (f"ply\nformat {fmt} 1.0\nobj_info hand\nelement face 2\n"
            "property list uchar uint vertex_indices\nproperty double w\n"
            "element vertex 2\nproperty float x\nproperty ushort k\nproperty char c\n"
            "end_header\n").encode()
    body = struct.pack(order + "B3Id", 3, 4, 5, 6, 0.25) + struct.pack(order + "Bd", 0, -2.0)
    body += struct.pack(order + "fHb", 1.5, 65535, -128) + struct.pack(order + "fHb", -0.0, 1, 127)
    return head + body


@pytest.mark.parametrize("order", ["<", ">"])
def test_binary_both_byte_orders_lists_before_the_vertices(tmp_path, order):
    (tmp_path / "b.ply").write_bytes(_binary(order))
    d = ply.read_ply(tmp_path / "b.ply")
    f, v = d["face"], d["vertex"]
    assert list(f["vertex_indices"][0]) == [4, 5, 6] and len(f["vertex_indices"][1]) == 0
    assert list(f["w"]) == [0.25, -2.0]
    assert list(v["x"]) == [1.5, 0.0] and list(v["k"]) == [65535, 1] and list(v["c"]) == [-128, 127]


def test_write_then_read_keeps_types(tmp_path):
    props = {"a": np.arange(5, dtype=np.uint16), "b": np.linspace(0, 1, 5),
             "c": np.array([-1, 0, 1, 2, 3], dtype=np.int8)}
    ply.write_ply(tmp_path / "w.ply", "pts", props)
    raw = (tmp_path / "w.ply").read_bytes()
    assert b"property ushort a\nproperty double b\nproperty char c\nend_header\n" in raw
    v = ply.read_ply(tmp_path / "w.ply")["pts"]
    for k, x in props.items():
        assert v[k].dtype == x.dtype and np.array_equal(v[k], x)


# -- malformed files ----------------------------------------------------------

@pytest.mark.parametrize("raw,msg", [
    (b"plx\n", "magic"),
    (b"ply\nformat binary_little_endian 1.0\nelement vertex 1\nproperty float x\n", "end_header"),
    (b"ply\nelement vertex 1\nproperty float x\nend_header\n", "format"),
    (b"ply\nformat binary_middle_endian 1.0\nend_header\n", "format"),
    (b"ply\nformat ascii 1.0\nproperty float x\nend_header\n", "before any element"),
    (b"ply\nformat ascii 1.0\nelement v 1\nproperty float16 x\nend_header\n", "property"),
    (b"ply\nformat ascii 1.0\nelement v 1\nproperty float x\nproperty float x\nend_header\n1 2\n",
     "repeats"),
    (b"ply\nformat binary_little_endian 1.0\nelement v 3\nproperty float x\nend_header\n"
     + b"\0" * 8, "truncated"),
    (b"ply\nformat ascii 1.0\nelement v 3\nproperty float x\nend_header\n1 2\n", "truncated"),
    (b"ply\nformat ascii 1.0\nelement f 1\nproperty list uchar int i\nend_header\n3 1 2\n",
     "truncated"),
    (b"ply\nformat binary_little_endian 1.0\nelement f 1\nproperty list uchar int i\n"
     b"end_header\n\x02\x01\x00\x00\x00", "truncated"),
])
def test_malformed_files_raise(tmp_path, raw, msg):
    (tmp_path / "m.ply").write_bytes(raw)
    with pytest.raises(ValueError, match=msg):
        ply.read_ply(tmp_path / "m.ply")


def test_gaussian_layout_errors(tmp_path):
    cols = _sh0_columns(2)
    del cols["rotation_3"]
    ply.write_ply(tmp_path / "m.ply", "vertex", cols)
    with pytest.raises(ValueError, match="missing properties"):
        ply.load_gaussians(tmp_path / "m.ply")
    cols = _sh0_columns(2)
    cols.update({f"features_rest_{i}": np.zeros(2, np.float32) for i in range(6)})
    ply.write_ply(tmp_path / "k.ply", "vertex", cols)  # K = 3: not (degree + 1)^2
    with pytest.raises(ValueError, match="degree"):
        ply.load_gaussians(tmp_path / "k.ply")
    ply.write_ply(tmp_path / "e.ply", "point", _sh0_columns(2))
    with pytest.raises(ValueError, match="no 'vertex'"):
        ply.load_gaussians(tmp_path / "e.ply")
    with pytest.raises(ValueError, match="1-D"):
        ply.write_ply(tmp_path / "x.ply", "vertex", {"a": np.zeros(2), "b": np.zeros(3)})
    with pytest.raises(ValueError, match="cannot store"):
        ply.write_ply(tmp_path / "x.ply", "vertex", {"a": np.zeros(2, np.int64)})
