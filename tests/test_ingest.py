"""Mesh ingest: the oracle readers against known answers, then the device
readers (file and memory, binary bodies decoded by kernels) against the
oracle, bit-exact, over the format variants and edge cases, and an
end-to-end render of an ingested mesh."""
import numpy as np
import pytest

from oracle import formats as F


def _same(dev: dict, ref: dict):
    for k in ("vertices", "triangles", "colors", "normals", "uv"):
        assert (k in dev) == (k in ref and ref[k] is not None and len(ref[k]) > 0 or k in ("vertices", "triangles")), k
        if k in dev and k in ref:
            a, b = np.asarray(dev[k]), np.asarray(ref[k])
            assert a.shape == b.shape, (k, a.shape, b.shape)
            assert np.array_equal(a.view(np.uint32), b.astype(a.dtype).view(np.uint32)), k


def _ico(level=2, seed=0x6A3D0050):
    from j3d_gb300 import workloads as W
    return W.icosphere(level, seed)


# ----------------------------------------------------------------- CPU: oracle

def test_sscanf_subset_known_answers():
    assert F.sscanf("f 1/2 3/4 5/6", "f %d/%d %d/%d %d/%d %d/%d\n") == (6, [1, 2, 3, 4, 5, 6])
    assert F.sscanf("f 1 2 3", "f %d/%d %d/%d %d/%d %d/%d\n")[0] == 1
    assert F.sscanf("f 1/1/1 2/2/2 3/3/3", "f %d/%d/ %d/%d/ %d/%d/ %d/%d/\n")[0] == 3
    assert F.sscanf("f 1//1 2//2 3//3", "f %d/%d/%d %d/%d/%d %d/%d/%d %d/%d/%d\n")[0] == 1
    assert F.sscanf("v", "v %f")[0] == -1
    assert F.sscanf("v 1 2", "v %f %f %f")[0] == 2
    n, v = F.sscanf("  12", "%d\n")
    assert n == 1 and v == [12]


def test_obj_oracle_known_answer():
    obj = (b"# quad with colours and texture coordinates\n"
           b"mtllib none.mtl\n"
           b"v 0 0 0 1 0 0\n"
           b"v 1 0 0 0 1 0\n"
           b"  v 1 1 0 0 0 1\n"
           b"v 0 1 0 0.5 0.5 0.5\n"
           b"vt 0 0\nvt 1 0\nvt 1 1\nvt 0 1\n"
           b"f 1/1 2/2 3/3 4/4\n")
    r = F.read_obj(obj)
    assert r["vertices"].tolist() == [[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]]
    assert r["triangles"].tolist() == [[0, 1, 2], [0, 2, 3]]
    assert [hex(c) for c in r["colors"]] == ["0xff0000ff", "0xff00ff00", "0xffff0000", "0xff7f7f7f"]
    assert r["uv"].tolist() == [[0, 1, 1, 1, 1, 0], [0, 1, 1, 0, 0, 0]]
    # 1-based indices above the vertex count are shifted down by the minimum (io.cpp:232-262)
    r = F.read_obj(b"v 0 0 0\nv 1 0 0\nv 0 1 0\nf 11 12 13\n")
    assert r["triangles"].tolist() == [[0, 1, 2]]
    with pytest.raises(F.FormatError):
        F.read_obj(b"v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1//1 2//1 3//1\n")


def test_ply_oracle_known_answer():
    ply = (b"ply\nformat ascii 1.0\ncomment hand written\nelement vertex 4\n"
           b"property float x\nproperty float y\nproperty float z\n"
           b"property uchar red\nproperty uchar green\nproperty uchar blue\n"
           b"element face 2\nproperty list uchar int vertex_indices\nend_header\n"
           b"0 0 0 255 0 0\n1 0 0 0 255 0\n1 1 0 0 0 255\n0 1 0 10 20 30\n"
           b"4 0 1 2 3\n3 3 2 1\n")
    r = F.read_ply(ply)
    assert r["triangles"].tolist() == [[0, 1, 2], [0, 2, 3], [3, 2, 1]]
    assert [hex(c) for c in r["colors"]] == ["0xff0000ff", "0xff00ff00", "0xffff0000", "0xff1e140a"]
    be = F.write_ply(r["vertices"], [[0, 1, 2, 3], [3, 2, 1]], encoding="binary_big_endian",
                     colors=[[255, 0, 0], [0, 255, 0], [0, 0, 255], [10, 20, 30]])
    r2 = F.read_ply(be)
    _same(r2, r)


def test_pts_xyz_stl_off_oracle_known_answers():
    r = F.read_pts(b"2\n1 2 3 5 10 20 30\n4 5 6 5 1 2 3\n")
    assert r["vertices"].tolist() == [[1, 2, 3], [4, 5, 6]]
    assert [hex(c) for c in r["colors"]] == ["0xff1e140a", "0xff030201"]
    with pytest.raises(F.FormatError):
        F.read_pts(b"3\n1 2 3\n")
    r = F.read_xyz(b"1 2 3\n\n4 5\n")
    assert r["vertices"].tolist() == [[1, 2, 3], [4, 5, 0]]
    V = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], np.float32)
    T = np.array([[0, 1, 2], [0, 2, 3]], np.uint32)
    for data in (F.write_stl_binary(V, T), F.write_stl_ascii(V, T)):
        r = F.read_stl(data)
        assert r["vertices"].tolist() == V[T].reshape(-1, 3).tolist()
        assert r["triangles"].tolist() == [[0, 1, 2], [3, 4, 5]]
    r = F.read_off(b"OFF\n# comment\n4 1 0\n0 0 0\n1 0 0\n1 1 0\n0 1 0 \n4 0 1 2 3\n")
    assert r["triangles"].tolist() == [[0, 1, 2], [0, 2, 3]]


def test_writers_round_trip_through_the_oracle(product_lib):
    V, T = _ico(2)
    for enc in ("ascii", "binary_little_endian", "binary_big_endian"):
        r = F.read_ply(F.write_ply(V, T, encoding=enc))
        assert np.array_equal(r["vertices"], V) and np.array_equal(r["triangles"], T), enc
    r = F.read_ply(F.write_ply_triangles_fast(V, T, big_endian=True))
    assert np.array_equal(r["vertices"], V) and np.array_equal(r["triangles"], T)
    r = F.read_obj(F.write_obj(V, T))
    assert np.array_equal(r["vertices"], V) and np.array_equal(r["triangles"], T)
    r = F.read_off(F.write_off(V, T))
    assert np.array_equal(r["vertices"], V) and np.array_equal(r["triangles"], T)


# ------------------------------------------------------------- GPU: device readers

def _read_both(ctx, data: bytes, fmt: str, tmp_path):
    from j3d_gb300 import Geometry
    g1 = Geometry.read_memory(ctx, data, fmt)
    p = tmp_path / f"m.{fmt}"
    p.write_bytes(data)
    g2 = Geometry.read_file(ctx, p)
    a1, a2 = g1.arrays(), g2.arrays()
    assert a1.keys() == a2.keys()
    for k in a1:
        assert np.array_equal(a1[k], a2[k]), k
    assert g2.info.file_bytes == len(data)
    return a1, g2.info


def _ply_variants():
    V, T = _ico(2, 0x6A3D0051)
    n = len(V)
    rng = np.random.default_rng(5)
    col = rng.integers(0, 256, (n, 3))
    colf = rng.uniform(-0.1, 1.1, (n, 3)).astype(np.float32)
    nrm = rng.normal(size=(n, 3)).astype(np.float32)
    quads = [list(T[i]) + [int(T[i + 1][2])] for i in range(0, len(T) - 1, 2)]
    mixed = [list(t) for t in T[:40]] + quads[:30] + [[1, 2], [5, 6, 7, 8, 9]] + [list(t) for t in T[40:80]]
    tc_tri = [list(rng.uniform(0, 1, 6).astype(np.float32)) for _ in range(len(T))]
    out = {
        "le_plain": dict(faces=T),
        "be_plain": dict(faces=T, encoding="binary_big_endian"),
        "ascii_plain": dict(faces=T, encoding="ascii"),
        "double_coords": dict(faces=T, coord="double"),
        "int_count_uint_index": dict(faces=T, count_type="int", index_type="uint"),
        "ushort_index_be": dict(faces=T, index_type="ushort", encoding="binary_big_endian"),
        "colors_normals": dict(faces=T, colors=col, normals=nrm),
        "float_colors_ascii": dict(faces=T, colors=colf, color_type="float", encoding="ascii"),
        "odd_stride": dict(faces=T, extra_vertex=[("confidence", "float", rng.uniform(size=n)),
                                                  ("intensity", "uchar", rng.integers(0, 255, n))]),
        "wide_stride": dict(faces=T, extra_vertex=[(f"q{k}", "double", rng.uniform(size=n)) for k in range(50)]),
        "quads": dict(faces=quads),
        "mixed_polygons": dict(faces=mixed),
        "mixed_polygons_be": dict(faces=mixed, encoding="binary_big_endian"),
        "texcoords": dict(faces=T, texcoords=tc_tri),
        "list_element_before": dict(faces=T, pre_elements=[("edge_loop", [("ids", ("uchar", "int"))],
                                                            [[[1, 2, 3]], [[4]], [[]]])]),
        "fixed_element_after": dict(faces=T, extra_elements=[("material", [("a", "float"), ("b", "uchar")],
                                                              [[1.5, 2], [2.5, 3]])]),
        "point_cloud": dict(faces=[], colors=col),
    }
    return V, out


@pytest.mark.gpu
@pytest.mark.parametrize("variant", list(_ply_variants()[1].keys()))
def test_ply_device_decode_matches_oracle(gpu_ctx, tmp_path, variant):
    V, variants = _ply_variants()
    kw = variants[variant]
    data = F.write_ply(V, **kw)
    dev, info = _read_both(gpu_ctx, data, "ply", tmp_path)
    ref = F.read_ply(data)
    _same(dev, ref)
    assert info.encoding == {"ascii": 0, "binary_big_endian": 2}.get(kw.get("encoding"), 1)
    assert info.device_decoded == (info.encoding != 0)


@pytest.mark.gpu
def test_stl_binary_and_ascii(gpu_ctx, tmp_path):
    V, T = _ico(3)
    for data in (F.write_stl_binary(V, T), F.write_stl_ascii(V[:200], T[T.max(1) < 200])):
        dev, info = _read_both(gpu_ctx, data, "stl", tmp_path)
        _same(dev, F.read_stl(data))


@pytest.mark.gpu
@pytest.mark.parametrize("style", ["plain", "slash", "slash2", "triple", "colors", "quads", "lead", "crlf", "long_lines"])
def test_obj_matches_oracle(gpu_ctx, tmp_path, style):
    V, T = _ico(2, 0x6A3D0052)
    rng = np.random.default_rng(3)
    uv = rng.uniform(0, 1, (3 * len(T) + 2, 2)).astype(np.float32)
    if style == "colors":
        data = F.write_obj(V, T, colors=rng.uniform(-0.2, 1.2, (len(V), 3)).astype(np.float32))
    elif style == "quads":
        Q = [list(T[i]) + [int(T[i + 1][2])] for i in range(0, len(T) - 1, 2)]
        data = F.write_obj(V, Q, uv=uv, style="slash")
    elif style == "lead":
        data = F.write_obj(V, T, lead=" \t ", normals=True)
    elif style == "crlf":
        data = F.write_obj(V, T, uv=uv, style="triple").replace(b"\n", b"\r\n")
    elif style == "long_lines":
        # lines longer than 255 bytes are read in 255-byte pieces; a piece
        # that starts with "v " is a vertex line of its own
        pad = b"# " + b"x" * 253 + b"v 9 9 9\n"
        data = pad + F.write_obj(V, T) + pad
    elif style == "plain":
        data = F.write_obj(V, T)
    else:
        data = F.write_obj(V, T, uv=uv, style=style)
    dev, info = _read_both(gpu_ctx, data, "obj", tmp_path)
    _same(dev, F.read_obj(data))
    if style == "long_lines":
        assert len(dev["vertices"]) == len(V) + 2


@pytest.mark.gpu
def test_off_xyz_pts(gpu_ctx, tmp_path):
    V, T = _ico(2, 0x6A3D0053)
    rng = np.random.default_rng(4)
    col = rng.integers(0, 256, (len(V), 3))
    Q = [list(T[i]) + [int(T[i + 1][2])] for i in range(0, len(T) - 1, 2)]
    cases = [(F.write_off(V, T), "off"), (F.write_off(V, Q, colors=col), "off"), (F.write_xyz(V), "xyz"),
             (F.write_pts(V), "pts"), (F.write_pts(V, intensity=np.arange(len(V)), colors=col), "pts"),
             (F.write_pts(V, count_line=False), "pts")]
    for data, fmt in cases:
        dev, _ = _read_both(gpu_ctx, data, fmt, tmp_path)
        _same(dev, F.read(data, fmt))


@pytest.mark.gpu
def test_ingest_errors_are_reported(gpu_ctx, tmp_path):
    from j3d_gb300 import Geometry, J3dgError, mesh_from_geometry
    V, T = _ico(1)
    good = F.write_ply_triangles_fast(V, T)
    bad = [(good[:-7], "ply"),                                   # body shorter than the header says
           (good.replace(b"end_header", b"end_headr"), "ply"),   # unknown header line
           (b"ply\nformat binary_little_endian 1.0\n", "ply"),  # no end_header
           (b"", "ply"),
           (b"v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1//1 2//1 3//1\n", "obj"),
           (b"3\n1 2 3\n", "pts"),
           (b"hello", "auto")]
    for data, fmt in bad:
        with pytest.raises(J3dgError):
            Geometry.read_memory(gpu_ctx, data, fmt)
    with pytest.raises(J3dgError):
        Geometry.read_file(gpu_ctx, tmp_path / "missing.ply")
    p = tmp_path / "mesh.unknown"
    p.write_bytes(good)
    with pytest.raises(J3dgError):
        Geometry.read_file(gpu_ctx, p)
    # out-of-range indices are decoded as written and refused by the build
    T2 = T.copy()
    T2[3, 1] = len(V) + 5
    g = Geometry.read_memory(gpu_ctx, F.write_ply_triangles_fast(V, T2), "ply")
    with pytest.raises(J3dgError):
        mesh_from_geometry(gpu_ctx, g)
    # a point cloud has no mesh
    pc = Geometry.read_memory(gpu_ctx, F.write_xyz(V), "xyz")
    with pytest.raises(J3dgError):
        mesh_from_geometry(gpu_ctx, pc)


@pytest.mark.gpu
def test_large_binary_ply_round_trip(gpu_ctx, tmp_path):
    """2.1M triangles through the file path (pinned chunks, device decode):
    the arrays come back exactly as written, both byte orders."""
    from j3d_gb300 import Geometry, workloads as W
    V, T = W.torus(1030, 1030, seed=W.SEED_BASE + 73)
    for be in (False, True):
        p = tmp_path / "torus.ply"
        p.write_bytes(F.write_ply_triangles_fast(V, T, big_endian=be))
        g = Geometry.read_file(gpu_ctx, p)
        a = g.arrays()
        assert np.array_equal(a["vertices"], V) and np.array_equal(a["triangles"], T)
        assert g.info.device_decoded == 1 and g.info.file_bytes > 32 << 20  # more than one pinned chunk


@pytest.mark.gpu
def test_ingested_mesh_renders_like_the_arrays(gpu_ctx, oracle_mod):
    """mesh_from_geometry(read(PLY)) gives the same frame as Mesh(V, T),
    and PLY vertex colours shade like set_vertex_colors of the converted
    colours (mesh.cpp:216-228)."""
    from j3d_gb300 import Canvas, Geometry, Matcap, Mesh, Scene, mesh_from_geometry, settings
    from j3d_gb300 import workloads as W
    V, T = W.icosphere(4, W.SEED_BASE + 74)
    rng = np.random.default_rng(9)
    col = rng.integers(0, 256, (len(V), 3))
    g = Geometry.read_memory(gpu_ctx, F.write_ply(V, T, colors=col), "ply")
    m1 = mesh_from_geometry(gpu_ctx, g)
    m2 = Mesh(gpu_ctx, V, T)
    colf = (col.astype(np.float32) / np.float32(255.0)).astype(np.float32)
    m2.set_vertex_colors(np.ascontiguousarray(colf))
    mc = Matcap.make(gpu_ctx, 0)
    out = []
    for mesh in (m1, m2):
        sc = Scene()
        sc.add_object(mesh, None, 1)
        sc.prepare_scene()
        sc.unzoom()
        cv = Canvas(gpu_ctx, 320, 240)
        cv.update_settings(settings(shadow=True, edges=False, vertexcolors=True))
        cv.render_frame(sc, mc)
        out.append((cv.get_pixels(), cv.get_image()))
    assert np.array_equal(out[0][0].view(np.uint8), out[1][0].view(np.uint8))
    assert np.array_equal(out[0][1], out[1][1])
    assert (out[0][0]["db_id"] != 0).mean() > 0.2
