"""Scene import (Utils/Importer.cpp) and image files (Utils/Image.cpp),
host code of libcraystal_gb300.so, checked without a GPU.

The reference reads OBJ/MTL with assimp 5.4.3, XML with pugixml 1.15 and
images with tinyexr / stb; none of them is in this image, so the expected
values here are derived by hand from those libraries' published behaviour
(named in each test) or built by independent encoders written in the test
(Python's zlib for compressed EXR and PNG files)."""
import struct
import zlib

import numpy as np
import pytest

from craystal_gb300._lib import CrayError
from craystal_gb300.api import Image, Importer, MaterialFlags


def write_scene(tmp_path, obj, mtl=None, xml=None, name="scene"):
    xml = xml if xml is not None else (
        '<?xml version="1.0"?>\n<camera width="32" height="24" fovy="45">'
        '<eye x="0" y="1" z="5"/><lookat x="0" y="1" z="0"/><up x="0" y="1" z="0"/></camera>\n'
        '<light mtlname="Lamp" radiance="10, 8,6"/>\n')
    (tmp_path / f"{name}.xml").write_text(xml)
    (tmp_path / f"{name}.obj").write_text(obj)
    if mtl is not None:
        (tmp_path / f"{name}.mtl").write_text(mtl)
    return str(tmp_path / f"{name}.xml")


# --- assimp's fast_atof (fast_atof.h) for float, restated in numpy -----------
FRAC = [0.0] + [10.0 ** -k for k in range(1, 16)]


def fast_atof(s):
    i, inv = 0, s[0] == "-"
    if s[0] in "+-":
        i += 1
    f = np.float32(0)

    def digits(i, cap=None):
        j, v, n = i, 0, 0
        while j < len(s) and s[j].isdigit():
            if cap is None or n < cap:
                v, n = v * 10 + int(s[j]), n + 1
            j += 1
        return v, n, j

    if s[i] not in ".,":
        v, _, i = digits(i)
        f = np.float32(v)
    if i < len(s) and s[i] in ".," and i + 1 < len(s) and s[i + 1].isdigit():
        v, n, i = digits(i + 1, 15)
        f = np.float32(f + np.float32(float(v) * FRAC[n]))
    elif i < len(s) and s[i] == ".":
        i += 1
    if i < len(s) and s[i] in "eE":
        i += 1
        einv = s[i] == "-"
        if s[i] in "+-":
            i += 1
        v, _, i = digits(i)
        e = np.float32(-v if einv else v)
        f = np.float32(f * np.power(np.float32(10.0), e))
    return np.float32(-f if inv else f)


def test_fast_atof_numbers(tmp_path):
    nums = ["0.1", "0.7", "123.456", "-2.5e+2", "1.0000000000000000001", "3.14159265358979323846", ".5", "7.",
            "1e-3", "2.5E-1", "16777217", "0.333333333333333333", "-0", "1,5", "0.30000001", "1234567.891",
            "9.999999999999999e-8", "-0.000001", "4.2e10", "-154.6256e-12", "780.549e5", "-602.9739e2"]
    while len(nums) % 3:
        nums.append("1")
    lines = [f"v {nums[i]} {nums[i + 1]} {nums[i + 2]}" for i in range(0, len(nums), 3)]
    faces = [f"f {a} {a + 1} {a + 2}" for a in range(1, len(lines) - 1)]
    data, _ = Importer().load(write_scene(tmp_path, "\n".join(lines + faces) + "\n"))
    got = np.concatenate([m.position for m in data.meshes]).reshape(-1)
    want = np.array([fast_atof(s) for s in nums], np.float32)
    # every vertex is used; compare the sets of bit patterns (corners repeat with their face normals)
    assert set(got.view(np.uint32).tolist()) == set(want.view(np.uint32).tolist())
    # a difference from a correctly rounded parse exists in this list
    assert any(np.float32(fast_atof(s)) != np.float32(float(s.replace(",", "."))) for s in nums)


def test_materials_meshes_and_emitters(tmp_path):
    mtl = ("newmtl Red\nKd 0.8 0.1 0.1\nKs 0.2 0.2 0.2\nNs 32\n"
           "newmtl Mono\nKd 0.5\n"  # one value: (0.5, 0, 0)
           "newmtl Lamp\nKd 0.9 0.9 0.9\n")
    obj = ("mtllib scene.mtl\n"
           "v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nv 0 0 1\nv 1 0 1\n"
           "f 1 2 3\n"                # no object yet: a default object whose mesh takes the last MTL material
           "usemtl Red\nf 1 3 4\n"    # another material after faces: a new mesh
           "usemtl Red\nf 2 3 4\n"    # same material: ignored
           "o second\nusemtl Mystery\nf 1 5 6\n"  # unknown name: a new default material
           "usemtl Lamp\nf 2 5 6\nf 3 5 6\n"
           "g\n"
           "usemtl Mono\nf 4 5 6\n")
    data, cam = Importer().load(write_scene(tmp_path, obj, mtl))
    names = [m.name for m in data.materials]
    assert names == ["DefaultMaterial", "Red", "Mono", "Lamp", "Mystery"]
    md = {m.name: m for m in data.materials}
    assert md["DefaultMaterial"].diffuseRefl == pytest.approx((0.6, 0.6, 0.6))
    assert md["Mystery"].diffuseRefl == pytest.approx((0.6, 0.6, 0.6))
    assert md["Mono"].diffuseRefl == pytest.approx((0.5, 0.0, 0.0))
    assert md["Red"].specularRefl == pytest.approx((0.2, 0.2, 0.2)) and md["Red"].shininess == 32.0
    assert all(int(m.type) == 2 for m in data.materials)  # Phong
    assert md["Lamp"].emission == pytest.approx((10.0, 8.0, 6.0)) and md["Lamp"].isEmissive()
    mesh_mats = [names[m.materialID] for m in data.meshes]
    assert mesh_mats == ["Lamp", "Red", "Mystery", "Lamp", "Mono"]
    tris_per_mesh = [len(m.index) // 3 for m in data.meshes]
    assert tris_per_mesh == [1, 2, 1, 2, 1]
    # emitters: every triangle of the meshes with the emissive material, numbered over all meshes
    assert data.emissiveIndex == [0, 4, 5]
    assert cam.sensor.size == (32, 24) and cam.fovY == 45.0 and cam.posW == (0.0, 1.0, 5.0)


def test_quad_split_from_concave_corner(tmp_path):
    # corner 2 (0.4, 0.4) is concave: fan from it -> (2, 3, 0), (2, 0, 1)
    obj = "v 0 0 0\nv 1 0 0\nv 0.4 0.4 0\nv 0 1 0\nf 1 2 3 4\nv 0 0 1\nv 1 0 1\nv 1 1 1\nv 0 1 1\nf 5 6 7 8\n"
    data, _ = Importer().load(write_scene(tmp_path, obj))
    m = data.meshes[0]
    tri = m.position[m.index.reshape(-1, 3)]
    np.testing.assert_allclose(tri[0], [[0.4, 0.4, 0], [0, 1, 0], [0, 0, 0]], atol=1e-7)
    np.testing.assert_allclose(tri[1], [[0.4, 0.4, 0], [0, 0, 0], [1, 0, 0]], atol=1e-7)
    # the convex quad splits from corner 0
    np.testing.assert_allclose(tri[2], [[0, 0, 1], [1, 0, 1], [1, 1, 1]])
    np.testing.assert_allclose(tri[3], [[0, 0, 1], [1, 1, 1], [0, 1, 1]])
    # a pentagon is fanned from corner 0
    obj5 = "v 0 0 0\nv 1 0 0\nv 1.5 1 0\nv 0.5 1.5 0\nv -0.5 1 0\nf 1 2 3 4 5\n"
    d5, _ = Importer().load(write_scene(tmp_path, obj5, name="pent"))
    assert d5.meshes[0].index.reshape(-1, 3).tolist() == [[0, 1, 2], [0, 2, 3], [0, 3, 4]]


def test_normals_texcoords_indices_and_joining(tmp_path):
    obj = ("v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\n"
           "vt 0 0\nvt 1 0\nvt 1 1\nvt 0 1\nvn 0 0 1\n"
           "o a\nf -4/-4/1 -3/-3/1 -2/-2/1\nf 1/1/1 3/3/1 4/4/1\n"   # negative indices count back
           "o b\nf 1 2 3\nf 1 3 4\n")                                # no normals: flat normals generated
    data, _ = Importer().load(write_scene(tmp_path, obj))
    a, b = data.meshes
    # identical corners joined in first-use order: 6 corners, 4 distinct
    assert len(a.position) == 4 and a.index.tolist() == [0, 1, 2, 0, 2, 3]
    np.testing.assert_array_equal(a.texCrd, [[0, 0], [1, 0], [1, 1], [0, 1]])
    np.testing.assert_array_equal(a.normal, np.tile([0, 0, 1], (4, 1)))
    assert len(b.position) == 4
    np.testing.assert_array_equal(b.normal, np.tile([0, 0, 1], (4, 1)))
    assert not b.texCrd.any()  # mesh b names no texture coordinates


def test_import_errors(tmp_path):
    with pytest.raises(CrayError, match="xml"):
        Importer().load(str(tmp_path / "scene.txt"))
    p = write_scene(tmp_path, "v 0 0 0\n", xml="<scene><camera/></scene>")
    with pytest.raises(CrayError, match="camera"):
        Importer().load(p)
    (tmp_path / "lonely.xml").write_text('<camera width="4" height="4" fovy="30"/>')
    with pytest.raises(CrayError):
        Importer().load(str(tmp_path / "lonely.xml"))
    p = write_scene(tmp_path, "v 0 0 0\nf 1 2 3\n", name="badidx")
    with pytest.raises(CrayError, match="range"):
        Importer().load(p)


def test_map_kd_texture_is_flipped_and_linearised(tmp_path):
    tex = np.zeros((2, 3, 3), np.float32)
    tex[0] = [[1, 0, 0], [0, 1, 0], [0, 0, 1]]
    tex[1] = [[0.2, 0.4, 0.6], [0.5, 0.5, 0.5], [1, 1, 1]]
    Image(data=tex).writePNG(str(tmp_path / "wood.png"), False)
    mtl = "newmtl Wood\nKd 1 1 1\nmap_Kd -s 1 1 1 wood.png\n"
    obj = "mtllib scene.mtl\nv 0 0 0\nv 1 0 0\nv 0 1 0\nvt 0 0\nvt 1 0\nvt 0 1\nusemtl Wood\nf 1/1 2/2 3/3\n"
    data, _ = Importer().load(write_scene(tmp_path, obj, mtl))
    m = data.materials[1]
    assert m.flags & MaterialFlags.hasDiffuseTexture and m.diffuseHandle == 0
    t = data.textureImages[0]
    assert t.shape == (2, 3, 4)
    # bytes trunc(v * 255) / 255, raised to 2.2, rows bottom-up, alpha 0
    bytes_ = np.floor(tex * np.float32(255.0)).astype(np.float32)
    want = (np.power((bytes_ / np.float32(255.0)).astype(np.float64), 2.2)).astype(np.float32)[::-1]
    np.testing.assert_array_equal(t[..., :3], want)
    assert not t[..., 3].any()


# --- EXR ---------------------------------------------------------------------
def parse_exr_header(b):
    assert b[:4] == bytes([0x76, 0x2F, 0x31, 0x01]) and struct.unpack("<I", b[4:8])[0] == 2
    pos, attrs = 8, {}
    while b[pos] != 0:
        e = b.index(0, pos)
        name = b[pos:e].decode()
        e2 = b.index(0, e + 1)
        typ = b[e + 1:e2].decode()
        size = struct.unpack("<I", b[e2 + 1:e2 + 5])[0]
        attrs[name] = (typ, b[e2 + 5:e2 + 5 + size])
        pos = e2 + 5 + size
    return attrs, pos + 1


def test_exr_layout_and_roundtrip(tmp_path):
    img = Image(5, 3, 3)
    img.setPixel(1, 2, 0, 0.25)
    img.setPixel(1, 2, 1, 0.5)
    img.setPixel(1, 2, 2, 0.75)
    img.setPixel(4, 0, 0, 1000.0)
    p = str(tmp_path / "film.exr")
    img.writeEXR(p)
    b = open(p, "rb").read()
    attrs, table = parse_exr_header(b)
    assert attrs["compression"] == ("compression", b"\x00")
    chl = attrs["channels"][1]
    assert chl.startswith(b"B\x00\x01\x00\x00\x00") and b"G\x00" in chl and b"R\x00" in chl
    offs = struct.unpack("<3Q", b[table:table + 24])
    y, size = struct.unpack("<iI", b[offs[2]:offs[2] + 8])
    assert (y, size) == (2, 5 * 3 * 2)
    line = np.frombuffer(b[offs[2] + 8:offs[2] + 8 + size], np.float16).reshape(3, 5)  # B, G, R planes
    assert (line[0, 1], line[1, 1], line[2, 1]) == (0.75, 0.5, 0.25)
    back = Image.load(p)
    assert (back.getWidth(), back.getHeight(), back.getChannels()) == (5, 3, 3)
    np.testing.assert_array_equal(back.data, img.data)
    with pytest.raises(CrayError, match="exr"):
        img.writeEXR(str(tmp_path / "film.png"))


def test_exr_half_rounding_ties_up(tmp_path):
    # tinyexr's float -> half adds one unit when the first dropped bit is set
    vals = np.array([1.0 + 2.0 ** -11, 1.0 + 3 * 2.0 ** -11, 2.0 ** -20, 65520.0, -0.1, 1e-9, np.inf],
                    np.float32)
    img = Image(data=np.stack([vals, vals, vals], -1)[None])
    p = str(tmp_path / "r.exr")
    img.writeEXR(p)
    got = Image.load(p).data[0, :, 0]
    want = np.array([1.0 + 2.0 ** -10, 1.0 + 2.0 ** -9, 2.0 ** -20, np.inf, -0.0999755859375, 0.0, np.inf],
                    np.float32)
    np.testing.assert_array_equal(got, want)
    assert np.float16(vals[0]) == np.float16(1.0)  # round-to-nearest-even would differ


def exr_zip_float(path, w, h, planes):
    """A ZIP-compressed FLOAT EXR written from the OpenEXR layout description."""
    names = sorted(planes)
    chl = b"".join(n.encode() + b"\x00" + struct.pack("<iBxxxii", 2, 0, 1, 1) for n in names) + b"\x00"

    def attr(n, t, v):
        return n.encode() + b"\x00" + t.encode() + b"\x00" + struct.pack("<I", len(v)) + v
    box = struct.pack("<4i", 0, 0, w - 1, h - 1)
    hdr = (bytes([0x76, 0x2F, 0x31, 0x01]) + struct.pack("<I", 2) + attr("channels", "chlist", chl) +
           attr("compression", "compression", b"\x03") + attr("dataWindow", "box2i", box) +
           attr("displayWindow", "box2i", box) + attr("lineOrder", "lineOrder", b"\x00") +
           attr("pixelAspectRatio", "float", struct.pack("<f", 1)) +
           attr("screenWindowCenter", "v2f", struct.pack("<2f", 0, 0)) +
           attr("screenWindowWidth", "float", struct.pack("<f", 1)) + b"\x00")
    blocks = []
    for y0 in range(0, h, 16):
        raw = b"".join(planes[n][y].astype("<f4").tobytes() for y in range(y0, min(h, y0 + 16)) for n in names)
        t = bytes(raw[0::2]) + bytes(raw[1::2])
        d = bytearray(t)
        for i in range(len(d) - 1, 0, -1):
            d[i] = (t[i] - t[i - 1] + 128 + 256) & 0xFF
        z = zlib.compress(bytes(d))
        assert len(z) < len(raw)  # a block that does not shrink would be stored raw
        blocks.append((y0, z))
    table_at = len(hdr)
    data_at = table_at + 8 * len(blocks)
    offs, body = [], b""
    for y0, z in blocks:
        offs.append(data_at + len(body))
        body += struct.pack("<iI", y0, len(z)) + z
    open(path, "wb").write(hdr + struct.pack(f"<{len(offs)}Q", *offs) + body)


def test_exr_reader_zip_float_and_channel_mapping(tmp_path):
    rng = np.random.default_rng(1)
    w, h = 7, 37
    planes = {c: (rng.integers(-8, 8, (h, w)) / 4).astype(np.float32) for c in ("A", "B", "G", "R")}
    p = str(tmp_path / "z.exr")
    exr_zip_float(p, w, h, planes)
    img = Image.load(p)
    assert img.getChannels() == 4  # channels beyond R, G, B are kept as zeros
    np.testing.assert_array_equal(img.data[..., 0], planes["R"])
    np.testing.assert_array_equal(img.data[..., 1], planes["G"])
    np.testing.assert_array_equal(img.data[..., 2], planes["B"])
    assert not img.data[..., 3].any()


# --- PNG ---------------------------------------------------------------------
def test_png_roundtrip_truncation_and_flip(tmp_path):
    rng = np.random.default_rng(2)
    vals = (rng.integers(0, 256, (4, 6, 3)) / 255.0 + 1e-4).astype(np.float32)
    p = str(tmp_path / "a.png")
    Image(data=vals).writePNG(p, False)
    back = Image.load(p, toLinear=False)
    want = (np.floor(vals * np.float32(255.0)) / np.float32(255.0)).astype(np.float32)[::-1]
    np.testing.assert_array_equal(back.data, want)
    # out-of-range values without gamma wrap as the reference's x86 conversion does
    odd = np.array([[[1.5, -1.0, np.nan]]], np.float32)
    Image(data=odd).writePNG(str(tmp_path / "o.png"), False)
    got = np.round(Image.load(str(tmp_path / "o.png"), toLinear=False).data * 255).astype(int)
    assert got.reshape(-1).tolist() == [382 & 255, (-255) & 255, 0]
    # gamma-corrected: pow(v, 1/2.2), clamped
    g = np.array([[[0.0, 0.5, 4.0]]], np.float32)
    Image(data=g).writePNG(str(tmp_path / "g.png"), True)
    got = np.round(Image.load(str(tmp_path / "g.png"), toLinear=False).data * 255).astype(int).reshape(-1)
    assert got.tolist() == [0, int(np.float32(np.power(np.float32(0.5), np.float32(1 / 2.2))) * np.float32(255)), 255]
    with pytest.raises(CrayError, match="png"):
        Image(data=g).writePNG(str(tmp_path / "g.jpg"), True)


def png_file(path, w, h, ctype, depth, rows, plte=None, trns=None, filters=None):
    def chunk(t, d):
        return struct.pack(">I", len(d)) + t + d + struct.pack(">I", zlib.crc32(t + d) & 0xFFFFFFFF)
    bpp = max(1, {0: 1, 2: 3, 3: 1, 6: 4}[ctype] * depth // 8)
    raw, prev = b"", bytes(len(rows[0]))
    for y, row in enumerate(rows):
        ft = filters[y % len(filters)] if filters else 0
        out = bytearray()
        for i, x in enumerate(row):
            a = row[i - bpp] if i >= bpp else 0
            b = prev[i]
            c = prev[i - bpp] if i >= bpp else 0
            pred = [0, a, b, (a + b) // 2,
                    (lambda p: a if abs(p - a) <= abs(p - b) and abs(p - a) <= abs(p - c)
                     else (b if abs(p - b) <= abs(p - c) else c))(a + b - c)][ft]
            out.append((x - pred) & 0xFF)
        raw += bytes([ft]) + bytes(out)
        prev = row
    body = chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, 0))
    if plte is not None:
        body += chunk(b"PLTE", bytes(plte))
    if trns is not None:
        body += chunk(b"tRNS", bytes(trns))
    body += chunk(b"IDAT", zlib.compress(raw, 9)) + chunk(b"IEND", b"")
    open(path, "wb").write(b"\x89PNG\r\n\x1a\n" + body)


def test_png_reader_filters_palette_depths(tmp_path):
    rng = np.random.default_rng(3)
    w, h = 9, 5
    rgb = rng.integers(0, 256, (h, w, 3), dtype=np.uint8)
    png_file(str(tmp_path / "f.png"), w, h, 2, 8, [bytes(r.reshape(-1)) for r in rgb], filters=[0, 1, 2, 3, 4])
    got = Image.load(str(tmp_path / "f.png"), toLinear=False).data
    np.testing.assert_array_equal(got, (rgb[::-1].astype(np.float32) / np.float32(255.0)))
    # 16-bit: the high byte is kept
    v16 = rng.integers(0, 65536, (h, w, 3), dtype=np.uint16)
    png_file(str(tmp_path / "s.png"), w, h, 2, 16, [v16[y].astype(">u2").tobytes() for y in range(h)], filters=[4])
    got = Image.load(str(tmp_path / "s.png"), toLinear=False).data
    np.testing.assert_array_equal(got, ((v16[::-1] >> 8).astype(np.float32) / np.float32(255.0)))
    # palette with transparency -> 4 channels
    pal = rng.integers(0, 256, (4, 3), dtype=np.uint8)
    ind = rng.integers(0, 4, (h, w), dtype=np.uint8)
    png_file(str(tmp_path / "p.png"), w, h, 3, 8, [bytes(r) for r in ind], plte=pal.reshape(-1), trns=[0, 128])
    got = Image.load(str(tmp_path / "p.png"), toLinear=False).data
    alpha = np.array([0, 128, 255, 255])[ind]
    want = np.concatenate([pal[ind], alpha[..., None]], -1)[::-1].astype(np.float32) / np.float32(255.0)
    np.testing.assert_array_equal(got, want)
    # 1-bit grey scales 0/1 to 0/255
    bits = rng.integers(0, 2, (h, 16), dtype=np.uint8)
    png_file(str(tmp_path / "b.png"), 16, h, 0, 1, [bytes(np.packbits(r)) for r in bits])
    got = Image.load(str(tmp_path / "b.png"), toLinear=False).data[..., 0]
    np.testing.assert_array_equal(got, bits[::-1].astype(np.float32))
    # linearisation: (v / 255) ** 2.2 in double, rounded to float
    lin = Image.load(str(tmp_path / "f.png")).data
    np.testing.assert_array_equal(lin, np.power((rgb[::-1] / 255.0).astype(np.float32).astype(np.float64), 2.2)
                                  .astype(np.float32))
