"""Mesh / point-cloud file readers and writers -- TEST INFRASTRUCTURE ONLY.

CPU restatement of the reader dispatch of read_from_file (j3d/mesh.cpp:76-176,
j3d/pc.cpp:32-110) used as the oracle of the device ingest path, plus writers
that make the test files. Only tests/, smoke() and the bench's CPU-baseline
leg use it.

* OBJ follows j3d/io.cpp:292-480 line by line: fgets pieces of at most 255
  bytes, the leading-blank skip (at most 250), the four face patterns tried
  in order with sscanf semantics, vertex colours packed as
  0xff000000 | b << 16 | g << 8 | r from (uint8_t)(c * 255.f) on x86,
  correct_vertices_and_triangles (io.cpp:232-262) and the 1 - v flip.
* PTS follows io.cpp:590-640 (1023-byte pieces, 7 / 3 / 1 value lines),
  XYZ io.cpp:659-685 (missing values read as 0, blank lines skipped).
* PLY, OFF and STL go through jtk in the reference, which is not shipped
  (parity unpinned for those three); this file restates the published
  formats: PLY (Turk 1994) with any scalar type and byte order, faces fan
  triangulated (i0, ik+1, ik+2), a `texcoord` list of 2 values per corner as
  per-triangle uv; OFF with optional colours; STL binary (80-byte header,
  count, 50-byte records) and ASCII, unwelded (V = 3T).

Decimal strings are parsed through Python floats then rounded to float32;
the test files write float32 values in their shortest round-trip form, for
which this equals a direct strtof.
"""
from __future__ import annotations

import re
import struct

import numpy as np

PLY_TYPES = {"char": "i1", "int8": "i1", "uchar": "u1", "uint8": "u1", "short": "i2", "int16": "i2",
             "ushort": "u2", "uint16": "u2", "int": "i4", "int32": "i4", "uint": "u4", "uint32": "u4",
             "float": "f4", "float32": "f4", "double": "f8", "float64": "f8"}


class FormatError(ValueError):
    pass


def _f32(s: str) -> np.float32:
    return np.float32(float(s))


# ------------------------------------------------------------------ sscanf

_WS = " \t\n\v\f\r"
_FLOAT_RE = re.compile(r"[+-]?(?:(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?|inf(?:inity)?|nan)", re.IGNORECASE)
_INT_RE = re.compile(r"[+-]?\d+")


def sscanf(s: str, fmt: str):
    """The subset of C sscanf the readers use: %f, %d, %s, whitespace
    directives and literal characters. Returns (count, values); count is -1
    when the input ends before the first conversion."""
    vals = []
    i = 0
    k = 0
    n = len(s)
    while k < len(fmt):
        c = fmt[k]
        if c in _WS:
            while k < len(fmt) and fmt[k] in _WS:
                k += 1
            while i < n and s[i] in _WS:
                i += 1
            continue
        if c == "%":
            conv = fmt[k + 1]
            k += 2
            while i < n and s[i] in _WS:
                i += 1
            if i >= n:
                return (len(vals) if vals else -1), vals
            if conv == "f":
                m = _FLOAT_RE.match(s, i)
                if not m:
                    return len(vals), vals
                vals.append(_f32(m.group(0)))
            elif conv == "d":
                m = _INT_RE.match(s, i)
                if not m:
                    return len(vals), vals
                v = int(m.group(0))
                v = max(-(1 << 63), min((1 << 63) - 1, v))  # strtol clamps to long
                vals.append(((v + (1 << 31)) % (1 << 32)) - (1 << 31))  # then (int)
            elif conv == "s":
                m = re.compile(r"[^ \t\n\v\f\r]+").match(s, i)
                vals.append(m.group(0)[:255])
            i = m.end()
            continue
        if i >= n:
            return (len(vals) if vals else -1), vals
        if s[i] != c:
            return len(vals), vals
        i += 1
        k += 1
    return len(vals), vals


def _pieces(data: bytes, cap: int):
    """fgets(buf, cap + 1) pieces of the byte stream, as str (latin-1), cut at NUL."""
    i = 0
    n = len(data)
    while i < n:
        j = data.find(b"\n", i, i + cap)
        end = j + 1 if j >= 0 else min(n, i + cap)
        piece = data[i:end]
        z = piece.find(b"\0")
        yield (piece[:z] if z >= 0 else piece).decode("latin-1")
        i = end


def _byte_x86(x: np.float32) -> int:
    y = np.float32(x) * np.float32(255.0)
    if not (-2147483648.0 < float(y) < 2147483648.0):
        return 0
    return int(np.int32(int(y))) & 255  # truncation toward zero, low byte


def _u32(v: int) -> int:
    return v & 0xFFFFFFFF


# -------------------------------------------------------------------- OBJ

def read_obj(data: bytes) -> dict:
    """io.cpp:292-480 (_read_obj); texture files are not loaded."""
    V, clr, VN, VT, tri, tuv = [], [], [], [], [], []
    for b in _pieces(data, 255):
        ws = 0
        while ws < 250 and ws < len(b) and b[ws] in " \t":
            ws += 1
        q = b[ws:]
        g = lambda k: q[k] if k < len(q) else "\0"  # noqa: E731
        b2 = b[2] if len(b) > 2 else "\0"
        if g(0) == "v" and g(1) == " ":
            cnt, v = sscanf(q, "v %f %f %f %f %f %f\n")
            if cnt not in (3, 6):
                raise FormatError("obj: bad vertex line")
            V.append(v[:3])
            if cnt == 6:
                clr.append(0xFF000000 | (_byte_x86(v[5]) << 16) | (_byte_x86(v[4]) << 8) | _byte_x86(v[3]))
        elif g(0) == "v" and g(1) == "n" and b2 == " ":
            cnt, v = sscanf(q, "vn %f %f %f\n")
            if cnt != 3:
                raise FormatError("obj: bad normal line")
            VN.append(v)
        elif g(0) == "v" and g(1) == "t" and b2 == " ":
            cnt, v = sscanf(q, "vt %f %f\n")
            if cnt != 2:
                raise FormatError("obj: bad texture coordinate line")
            VT.append(v)
        elif g(0) == "f" and g(1) == " ":
            cnt, v = sscanf(q, "f %d/%d %d/%d %d/%d %d/%d\n")
            if cnt not in (6, 8):
                cnt, v = sscanf(q, "f %d/%d/ %d/%d/ %d/%d/ %d/%d/\n")
            if cnt in (6, 8):
                t = v[0::2]
                u = v[1::2]
                tuv.append([u[0] - 1, u[1] - 1, u[2] - 1])
                tri.append([t[0] - 1, t[1] - 1, t[2] - 1])
                if cnt == 8:
                    tuv.append([u[0] - 1, u[2] - 1, u[3] - 1])
                    tri.append([t[0] - 1, t[2] - 1, t[3] - 1])
                continue
            cnt, v = sscanf(q, "f %d %d %d %d\n")
            if cnt in (3, 4):
                tri.append([v[0] - 1, v[1] - 1, v[2] - 1])
                if cnt == 4:
                    tri.append([v[0] - 1, v[2] - 1, v[3] - 1])
                continue
            cnt, v = sscanf(q, "f %d/%d/%d %d/%d/%d %d/%d/%d %d/%d/%d\n")
            if cnt in (9, 12):
                t = v[0::3]
                u = v[1::3]
                tuv.append([u[0] - 1, u[1] - 1, u[2] - 1])
                tri.append([t[0] - 1, t[1] - 1, t[2] - 1])
                if cnt == 12:
                    tuv.append([u[0] - 1, u[2] - 1, u[3] - 1])
                    tri.append([t[0] - 1, t[2] - 1, t[3] - 1])
                continue
            raise FormatError("obj: unsupported face line")
    if tuv and len(tri) != len(tuv):
        raise FormatError("obj: faces with and without texture coordinates")
    T = np.array([[_u32(x) for x in t] for t in tri], np.uint32).reshape(-1, 3)
    TU = np.array([[_u32(x) for x in t] for t in tuv], np.uint32).reshape(-1, 3)
    nv = len(V)
    if T.size:
        lo, hi = int(T.min()), int(T.max())
        if hi >= nv and lo > 0:
            T = (T - np.uint32(lo)).astype(np.uint32)
            TU = (TU - np.uint32(lo)).astype(np.uint32)
    out = {"vertices": np.array(V, np.float32).reshape(-1, 3), "triangles": T}
    if TU.size:
        vt = np.array(VT, np.float32).reshape(-1, 2)
        if int(TU.max()) >= len(vt):
            raise FormatError("obj: texture coordinate index out of range")
        vt = vt.copy()
        vt[:, 1] = np.float32(1.0) - vt[:, 1]
        out["uv"] = vt[TU.reshape(-1)].reshape(-1, 6)
    if len(clr) == nv:
        out["colors"] = np.array(clr, np.uint32)
    if len(VN) == nv and nv:
        out["normals"] = np.array(VN, np.float32).reshape(-1, 3)
    return out


# -------------------------------------------------------------- PTS / XYZ

def read_pts(data: bytes) -> dict:
    """io.cpp:590-640 (_read_pts)."""
    V, clr = [], []
    count = None
    for b in _pieces(data, 1023):
        ws = 0
        while ws < 250 and ws < len(b) and b[ws] in " \t":
            ws += 1
        q = b[ws:]
        cnt, v = sscanf(q, "%f %f %f %d %d %d %d\n")
        if cnt == 7:
            V.append(v[:3])
            r, g, bl = (_u32(x) for x in v[4:7])
            clr.append(_u32(0xFF000000 | (bl << 16) | (g << 8) | r))
            continue
        cnt, v = sscanf(q, "%f %f %f\n")
        if cnt == 3:
            V.append(v)
            continue
        cnt, v = sscanf(q, "%d\n")
        if cnt != 1:
            raise FormatError("pts: invalid line")
        count = _u32(v[0])
    if count and len(V) != count:
        raise FormatError("pts: point count does not match the header")
    out = {"vertices": np.array(V, np.float32).reshape(-1, 3), "triangles": np.zeros((0, 3), np.uint32)}
    if len(clr) == len(V):
        out["colors"] = np.array(clr, np.uint32)
    return out


def read_xyz(data: bytes) -> dict:
    """io.cpp:659-685 (_read_xyz): three numbers per non-blank line."""
    V = []
    for line in data.decode("latin-1").split("\n"):
        if not line.strip():
            continue
        vals = [np.float32(0.0)] * 3
        i = 0
        for k in range(3):
            while i < len(line) and line[i] in _WS:
                i += 1
            m = _FLOAT_RE.match(line, i)
            if not m:
                break
            vals[k] = _f32(m.group(0))
            i = m.end()
        V.append(vals)
    return {"vertices": np.array(V, np.float32).reshape(-1, 3), "triangles": np.zeros((0, 3), np.uint32)}


# -------------------------------------------------------------------- PLY

def parse_ply_header(data: bytes):
    end = data.find(b"end_header")
    if not data.startswith(b"ply") or end < 0:
        raise FormatError("ply: bad header")
    nl = data.find(b"\n", end)
    if nl < 0:
        raise FormatError("ply: bad header")
    head = data[:nl + 1].decode("latin-1").replace("\r", "")
    enc = None
    elements = []
    for line in head.split("\n")[1:]:
        w = line.split()
        if not w or w[0] in ("comment", "obj_info", "end_header"):
            continue
        if w[0] == "format":
            enc = {"ascii": 0, "binary_little_endian": 1, "binary_big_endian": 2}[w[1]]
        elif w[0] == "element":
            elements.append({"name": w[1], "count": int(w[2]), "props": []})
        elif w[0] == "property":
            if w[1] == "list":
                elements[-1]["props"].append({"name": w[4], "list": True, "ct": PLY_TYPES[w[2]],
                                              "it": PLY_TYPES[w[3]]})
            else:
                elements[-1]["props"].append({"name": w[2], "list": False, "t": PLY_TYPES[w[1]]})
    return enc, elements, nl + 1


def _channel(t: str, v) -> int:
    if t[0] == "f":
        x = np.float32(v) * np.float32(255.0)
        if np.isnan(x):
            return 0
        return int(min(max(float(x), 0.0), 255.0))
    return int(min(255, max(0, int(v))))


def read_ply(data: bytes) -> dict:
    enc, elements, at = parse_ply_header(data)
    bo = ">" if enc == 2 else "<"
    out_v = out_c = out_n = None
    tris, uv, uv_ok = [], [], True
    toks = data[at:].split() if enc == 0 else None
    ti = 0

    def take(t):
        nonlocal ti
        s = toks[ti].decode()
        ti += 1
        if t[0] == "f":
            return np.float32(float(s)) if t == "f4" else np.float32(np.float64(float(s)))
        return int(s)

    for e in elements:
        names = [p["name"] for p in e["props"]]
        rows = []
        if enc == 0:
            for _ in range(e["count"]):
                rec = {}
                for p in e["props"]:
                    if p["list"]:
                        c = take(p["ct"])
                        rec[p["name"]] = [take(p["it"]) for _ in range(c)]
                    else:
                        rec[p["name"]] = take(p["t"])
                rows.append(rec)
        elif not any(p["list"] for p in e["props"]):
            dt = np.dtype([(p["name"], bo + p["t"]) for p in e["props"]])
            arr = np.frombuffer(data, dt, e["count"], at) if e["count"] else np.zeros(0, dt)
            at += dt.itemsize * e["count"]
            rows = arr
        else:
            for _ in range(e["count"]):
                rec = {}
                for p in e["props"]:
                    if p["list"]:
                        ct = np.dtype(bo + p["ct"])
                        c = int(np.frombuffer(data, ct, 1, at)[0])
                        at += ct.itemsize
                        it = np.dtype(bo + p["it"])
                        rec[p["name"]] = list(np.frombuffer(data, it, c, at)) if c else []
                        at += it.itemsize * c
                    else:
                        t = np.dtype(bo + p["t"])
                        rec[p["name"]] = np.frombuffer(data, t, 1, at)[0]
                        at += t.itemsize
                rows.append(rec)
        if e["name"] == "vertex":
            def col(n, rows=rows):
                if isinstance(rows, np.ndarray):
                    return rows[n]
                return [r[n] for r in rows]
            t_of = {p["name"]: p.get("t") for p in e["props"]}
            out_v = np.stack([np.asarray(col(n)).astype(np.float64).astype(np.float32)
                              if t_of[n] == "f8" else np.asarray(col(n)).astype(np.float32)
                              for n in ("x", "y", "z")], 1).reshape(-1, 3)
            if all(n in names for n in ("nx", "ny", "nz")):
                out_n = np.stack([np.asarray(col(n)).astype(np.float32) for n in ("nx", "ny", "nz")], 1).reshape(-1, 3)
            if all(n in names for n in ("red", "green", "blue")):
                ch = [[_channel(t_of[n], v) for v in col(n)] for n in ("red", "green", "blue")]
                out_c = np.array([0xFF000000 | (b << 16) | (g << 8) | r for r, g, b in zip(*ch)], np.uint32)
        if e["name"] == "face":
            il = "vertex_indices" if "vertex_indices" in names else "vertex_index"
            tc = "texcoord" if "texcoord" in names else ("texcoords" if "texcoords" in names else None)
            for r in rows:
                idx = [_u32(int(x)) for x in r[il]]
                t = [np.float32(x) for x in r[tc]] if tc else []
                has = tc is not None and len(t) == 2 * len(idx)
                if tc is not None and not has and len(idx) >= 3:
                    uv_ok = False
                for k in range(len(idx) - 2):
                    tris.append([idx[0], idx[k + 1], idx[k + 2]])
                    if has:
                        c = (0, k + 1, k + 2)
                        uv.append([t[2 * c[0]], t[2 * c[0] + 1], t[2 * c[1]], t[2 * c[1] + 1], t[2 * c[2]],
                                   t[2 * c[2] + 1]])
    out = {"vertices": out_v, "triangles": np.array(tris, np.uint32).reshape(-1, 3)}
    if out_c is not None:
        out["colors"] = out_c
    if out_n is not None:
        out["normals"] = out_n
    if uv_ok and uv and len(uv) == len(tris):
        out["uv"] = np.array(uv, np.float32).reshape(-1, 6)
    return out


# -------------------------------------------------------------- OFF / STL

def read_off(data: bytes) -> dict:
    lines = []
    for line in data.decode("latin-1").split("\n"):
        line = line.split("#")[0]
        w = line.split()
        if w:
            lines.append(w)
    if not lines or lines[0][0] not in ("OFF", "COFF"):
        raise FormatError("off: missing OFF magic")
    w = lines[0][1:]
    k = 1
    if not w:
        w = lines[1]
        k = 2
    nv, nf = int(w[0]), int(w[1])
    V, clr, tris = [], [], []
    for i in range(nv):
        w = lines[k + i]
        V.append([_f32(x) for x in w[:3]])
        if len(w) >= 6:
            ch = [_channel("f4", _f32(s)) if any(c in s for c in ".eE") else _channel("i4", int(s)) for s in w[3:6]]
            clr.append(0xFF000000 | (ch[2] << 16) | (ch[1] << 8) | ch[0])
    k += nv
    for i in range(nf):
        w = lines[k + i]
        c = int(w[0])
        idx = [_u32(int(x)) for x in w[1:1 + c]]
        for j in range(c - 2):
            tris.append([idx[0], idx[j + 1], idx[j + 2]])
    out = {"vertices": np.array(V, np.float32).reshape(-1, 3), "triangles": np.array(tris, np.uint32).reshape(-1, 3)}
    if len(clr) == nv:
        out["colors"] = np.array(clr, np.uint32)
    return out


def read_stl(data: bytes) -> dict:
    if len(data) >= 84:
        n = struct.unpack_from("<I", data, 80)[0]
        if len(data) == 84 + 50 * n:
            rec = np.frombuffer(data, np.dtype([("n", "<f4", 3), ("v", "<f4", 9), ("a", "<u2")]), n, 84)
            V = rec["v"].reshape(-1, 3).astype(np.float32)
            return {"vertices": V, "triangles": np.arange(3 * n, dtype=np.uint32).reshape(-1, 3)}
    toks = data.split()
    if not toks or toks[0] != b"solid":
        raise FormatError("stl: not an STL file")
    V = []
    for i, t in enumerate(toks):
        if t == b"vertex":
            V.append([_f32(toks[i + 1].decode()), _f32(toks[i + 2].decode()), _f32(toks[i + 3].decode())])
    n = len(V) // 3
    return {"vertices": np.array(V, np.float32).reshape(-1, 3), "triangles": np.arange(3 * n, dtype=np.uint32).reshape(-1, 3)}


READERS = {"ply": read_ply, "stl": read_stl, "obj": read_obj, "off": read_off, "xyz": read_xyz, "pts": read_pts}


def read(data: bytes, fmt: str) -> dict:
    return READERS[fmt](data)


# ---------------------------------------------------------------- writers

def fstr(x) -> str:
    """Shortest string that reads back as the same float32."""
    return np.format_float_positional(np.float32(x), unique=True, trim="-") if np.isfinite(x) else repr(float(x))


def write_ply(V, faces, encoding="binary_little_endian", coord="float", count_type="uchar", index_type="int",
              colors=None, color_type="uchar", normals=None, texcoords=None, extra_vertex=(), extra_elements=(),
              pre_elements=(), comments=("made by the ingest tests",)) -> bytes:
    """faces: list of index lists (or a (T, k) array). colors: (V, 3) values
    in color_type. texcoords: per face, a list of 2k floats. extra_vertex:
    [(name, type, values)], extra_elements / pre_elements: [(name, [(prop,
    type)], rows)] written after / before the vertex element."""
    V = np.asarray(V)
    faces = [list(map(int, f)) for f in faces]
    head = ["ply", f"format {encoding} 1.0"] + [f"comment {c}" for c in comments]

    def elem_head(name, props, count):
        head.append(f"element {name} {count}")
        for p, t in props:
            head.append(f"property {t} {p}" if not isinstance(t, tuple) else f"property list {t[0]} {t[1]} {p}")

    for name, props, rows in pre_elements:
        elem_head(name, props, len(rows))
    vprops = [("x", coord), ("y", coord), ("z", coord)]
    if normals is not None:
        vprops += [("nx", "float"), ("ny", "float"), ("nz", "float")]
    for n, t, _ in extra_vertex:
        vprops.append((n, t))
    if colors is not None:
        vprops += [("red", color_type), ("green", color_type), ("blue", color_type)]
    elem_head("vertex", vprops, len(V))
    if faces:
        fprops = [("vertex_indices", (count_type, index_type))]
        if texcoords is not None:
            fprops.append(("texcoord", ("uchar", "float")))
        elem_head("face", fprops, len(faces))
    for name, props, rows in extra_elements:
        elem_head(name, props, len(rows))
    head.append("end_header")
    out = bytearray(("\n".join(head) + "\n").encode())
    bo = ">" if encoding == "binary_big_endian" else "<"
    tnp = {k: v for k, v in PLY_TYPES.items()}

    def put(t, v):
        if encoding == "ascii":
            return (fstr(v) if tnp[t][0] == "f" else str(int(v))).encode() + b" "
        return np.array([v], bo + tnp[t]).tobytes()

    def write_rows(props, rows):
        for row in rows:
            line = bytearray()
            for (p, t), v in zip(props, row):
                if isinstance(t, tuple):
                    line += put(t[0], len(v))
                    for x in v:
                        line += put(t[1], x)
                else:
                    line += put(t, v)
            out.extend(line)
            if encoding == "ascii":
                out[-1:] = b"\n"

    for name, props, rows in pre_elements:
        write_rows(props, rows)
    vrows = []
    for i in range(len(V)):
        r = list(V[i])
        if normals is not None:
            r += list(normals[i])
        for _, _, vals in extra_vertex:
            r.append(vals[i])
        if colors is not None:
            r += list(colors[i])
        vrows.append(r)
    if encoding != "ascii" and not extra_vertex and normals is None and colors is None:
        out.extend(np.ascontiguousarray(V, bo + tnp[coord]).tobytes())  # fast path
    else:
        write_rows(vprops, vrows)
    if faces:
        frows = [[f] + ([texcoords[i]] if texcoords is not None else []) for i, f in enumerate(faces)]
        write_rows(fprops, frows)
    for name, props, rows in extra_elements:
        write_rows(props, rows)
    return bytes(out)


def write_ply_triangles_fast(V: np.ndarray, T: np.ndarray, big_endian=False) -> bytes:
    """Binary PLY of float vertices and uchar-count int-index triangles (the
    Stanford scan layout), written with numpy for large meshes."""
    bo = ">" if big_endian else "<"
    head = (f"ply\nformat binary_{'big' if big_endian else 'little'}_endian 1.0\nelement vertex {len(V)}\n"
            "property float x\nproperty float y\nproperty float z\n"
            f"element face {len(T)}\nproperty list uchar int vertex_indices\nend_header\n").encode()
    fd = np.dtype([("n", "u1"), ("i", bo + "i4", 3)])
    f = np.empty(len(T), fd)
    f["n"] = 3
    f["i"] = T
    return head + np.ascontiguousarray(V, bo + "f4").tobytes() + f.tobytes()


def write_stl_binary(V, T) -> bytes:
    V = np.asarray(V, np.float32)
    T = np.asarray(T)
    rec = np.zeros(len(T), np.dtype([("n", "<f4", 3), ("v", "<f4", 9), ("a", "<u2")]))
    rec["v"] = V[T].reshape(-1, 9)
    return b"binary stl written by the ingest tests".ljust(80, b" ") + struct.pack("<I", len(T)) + rec.tobytes()


def write_stl_ascii(V, T) -> bytes:
    lines = ["solid test"]
    for t in T:
        lines += ["  facet normal 0 0 1", "    outer loop"]
        lines += [f"      vertex {fstr(V[i][0])} {fstr(V[i][1])} {fstr(V[i][2])}" for i in t]
        lines += ["    endloop", "  endfacet"]
    lines.append("endsolid test")
    return ("\n".join(lines) + "\n").encode()


def write_off(V, faces, colors=None) -> bytes:
    lines = ["OFF", f"{len(V)} {len(faces)} 0"]
    for i, v in enumerate(V):
        s = " ".join(fstr(x) for x in v)
        if colors is not None:
            s += " " + " ".join(str(int(c)) for c in colors[i])
        lines.append(s)
    for f in faces:
        lines.append(" ".join(str(int(x)) for x in [len(f)] + list(f)))
    return ("\n".join(lines) + "\n").encode()


def write_xyz(V) -> bytes:
    return ("".join(f"{fstr(v[0])} {fstr(v[1])} {fstr(v[2])}\n" for v in V)).encode()


def write_pts(V, intensity=None, colors=None, count_line=True) -> bytes:
    lines = [str(len(V))] if count_line else []
    for i, v in enumerate(V):
        s = f"{fstr(v[0])} {fstr(v[1])} {fstr(v[2])}"
        if colors is not None:
            s += f" {int(intensity[i]) if intensity is not None else 0} " + " ".join(str(int(c)) for c in colors[i])
        lines.append(s)
    return ("\n".join(lines) + "\n").encode()


def write_obj(V, T, colors=None, uv=None, quads=None, style="plain", normals=False, lead="") -> bytes:
    """style: plain 'f a b c', slash 'f a/t b/t c/t', slash2 'f a/t/ ...',
    triple 'f a/t/n ...'. colors: (V, 3) floats in 0..1 written after xyz.
    uv: (K, 2) texture coordinates, face i using corners 3i..3i+2."""
    lines = ["# written by the ingest tests", "mtllib test.mtl"]
    for i, v in enumerate(V):
        s = f"{lead}v {fstr(v[0])} {fstr(v[1])} {fstr(v[2])}"
        if colors is not None:
            s += " " + " ".join(fstr(c) for c in colors[i])
        lines.append(s)
    if normals:
        for v in V:
            lines.append(f"vn {fstr(v[0])} {fstr(v[1])} {fstr(v[2])}")
    if uv is not None:
        for t in uv:
            lines.append(f"vt {fstr(t[0])} {fstr(t[1])}")
    for i, t in enumerate(T):
        idx = [int(x) + 1 for x in t]
        if style == "plain" or uv is None:
            lines.append(lead + "f " + " ".join(map(str, idx)))
        else:
            tx = [3 * i + k + 1 for k in range(len(idx))]
            if style == "slash":
                lines.append(lead + "f " + " ".join(f"{a}/{b}" for a, b in zip(idx, tx)))
            elif style == "slash2":
                lines.append(lead + "f " + " ".join(f"{a}/{b}/" for a, b in zip(idx, tx)))
            else:
                lines.append(lead + "f " + " ".join(f"{a}/{b}/{a}" for a, b in zip(idx, tx)))
    return ("\n".join(lines) + "\n").encode()
