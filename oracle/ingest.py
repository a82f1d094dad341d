"""CPU restatement of the reference's asset ingest.

TEST INFRASTRUCTURE ONLY: imported by tests/ to check the library's ingest entry points
(sr_image_load, sr_texture_load, sr_obj_load).  The product never imports this module.

Follows, step by step:
  - ObjLexer                      obj.cs:20-128   (tokens, comments, word buffers of 512 / 64 chars)
  - ObjLoader.Parse / BuildObject obj.cs:145-259  (v, vt with V flipped, vn, f, o/g, mtllib, usemtl)
  - ObjLoader.ParseMtl            obj.cs:261-401  (newmtl, Kd, Ke, Pr, Pm, Ns, Ni, d, Tr, texture maps)
  - TriangulateFace / ReadFace    obj.cs:403-470  (triangle fan, default uvs, 1-based / negative indices)
  - ReadFloat / ReadInt           obj.cs:487-511  (float.TryParse Float+Invariant, int.TryParse)
  - Image.Load / LoadTga          image.cs:214-282
  - ImageHdr.LoadHdr / ReadLine   image.cs:300-397
  - Color.FromPixel, FromPixelLinear, FromPixel(PixelHdr), ClampLuminance  math.cs:115-125, 184-202
Triangles (face / smooth normals, tangents) come from the render oracle's Triangle constructors
(oracle_triangles_from_corners in sr_oracle.cpp).

Parity unpinned against the C# binary: the reference ships no tests or fixtures for ingest and its
sample assets are Git LFS pointers, so this restatement is checked against hand-made files whose
expected values follow from the format definitions (tests/test_ingest.py).
"""
from __future__ import annotations

import ctypes as C
import ctypes.util
import os
import re
import stat
from fractions import Fraction

import numpy as np

from . import oracle

_libm = C.CDLL(ctypes.util.find_library("m") or "libm.so.6")
_libm.powf.restype = C.c_float
_libm.powf.argtypes = [C.c_float, C.c_float]

F32 = np.float32
F32_MAX = float(np.finfo(np.float32).max)


class IngestError(Exception):
    pass


# ---- System.IO.Path on Unix ('/' only) -----------------------------------------------------------

def path_extension(path: str) -> str:
    base = path[path.rfind("/") + 1:]
    dot = base.rfind(".")
    return "" if dot < 0 or dot == len(base) - 1 else base[dot:]


def path_directory(path: str) -> str:
    i = path.rfind("/")
    return "" if i < 0 else ("/" if i == 0 else path[:i])


def path_combine(a: str, b: str) -> str:
    if not a or b.startswith("/"):
        return b
    if not b:
        return a
    return a + b if a.endswith("/") else a + "/" + b


def path_stem(path: str) -> str:
    base = path[path.rfind("/") + 1:]
    dot = base.rfind(".")
    return base if dot < 0 else base[:dot]


def read_file(path: str) -> bytes:
    """File.OpenRead: a missing or unreadable file is a load error."""
    try:
        with open(path, "rb") as f:
            return f.read()
    except OSError as e:
        raise IngestError(f"cannot open '{path}': {e.strerror}") from None


def file_exists(path: str) -> bool:
    try:
        return bool(path) and stat.S_ISREG(os.stat(path).st_mode)
    except OSError:
        return False


# ---- number parsing ------------------------------------------------------------------------------

_FLOAT_RE = re.compile(r"[+-]?(\d+\.?\d*|\.\d+)([eE][+-]?\d+)?")
_INT_RE = re.compile(r"[+-]?\d+")


def round_to_f32(v: Fraction) -> float:
    """The float32 nearest to the exact rational v, ties to even; +-inf past the largest finite."""
    if v == 0:
        return 0.0
    limit = Fraction(F32_MAX) + Fraction(2) ** 103  # half an ulp above the largest finite float
    if abs(v) >= limit:
        return float("inf") if v > 0 else float("-inf")
    guess = np.float32(float(v))
    best = None
    with np.errstate(over="ignore"):
        cands = (np.nextafter(guess, np.float32(-np.inf)), guess, np.nextafter(guess, np.float32(np.inf)))
    for c in cands:
        if not np.isfinite(c):
            continue
        err = abs(Fraction(float(c)) - v)
        key = (err, int(np.array(c, np.float32).view(np.uint32)) & 1)
        if best is None or key < best[0]:
            best = (key, c)
    return float(best[1])


def _trim_number(s: str) -> str:
    """.NET number parsing: white space (tab to carriage return, space) around, NULs after."""
    return s.rstrip("\0").strip(" \t\n\v\f\r")


def parse_float(word: str):
    """float.TryParse(s, NumberStyles.Float, InvariantCulture): sign, digits with an optional point,
    optional exponent, or (any case) Infinity / +Infinity / -Infinity / NaN / +NaN / -NaN; the
    correctly rounded float."""
    s = _trim_number(word)
    low = s.lower()
    if low in ("infinity", "+infinity"):
        return float("inf")
    if low == "-infinity":
        return float("-inf")
    if low in ("nan", "+nan", "-nan"):
        return float("nan")
    if not _FLOAT_RE.fullmatch(s):
        return None
    v = Fraction(s)
    if v == 0:
        return -0.0 if s.startswith("-") else 0.0
    return round_to_f32(v)


def parse_int(word: str):
    """int.TryParse(s): optional sign and decimal digits within int range."""
    s = _trim_number(word)
    if not _INT_RE.fullmatch(s):
        return None
    v = int(s)
    return v if -2**31 <= v < 2**31 else None


# ---- ObjLexer ------------------------------------------------------------------------------------

WORD, SLASH, NEWLINE, END = "Word", "Slash", "Newline", "End"


class Lexer:
    def __init__(self, data: bytes):
        self.d, self.i = data, 3 if data.startswith(b"\xef\xbb\xbf") else 0  # StreamReader drops a UTF-8 BOM
        self.peeked = None  # (kind, word)

    def _read(self, limit: int):
        d = self.d
        while True:
            if self.i >= len(d):
                return END, ""
            c = d[self.i]
            self.i += 1
            if c == 0x0A:
                return NEWLINE, ""
            if c == 0x2F:
                return SLASH, ""
            if c in (0x20, 0x09, 0x0D):
                continue
            if c == 0x23:  # '#': comment to the end of the line
                j = d.find(b"\n", self.i)
                if j < 0:
                    self.i = len(d)
                    return END, ""
                self.i = j + 1
                return NEWLINE, ""
            j = self.i - 1
            while self.i < len(d) and d[self.i] not in (0x20, 0x09, 0x0D, 0x0A, 0x2F):
                self.i += 1
            word = d[j:self.i].decode("latin-1")
            if len(word) > limit:  # ReadWord past the end of its span
                raise IngestError(f"OBJ: word longer than {limit} characters")
            return WORD, word

    def peek(self):
        if self.peeked is None:
            self.peeked = self._read(512)
        return self.peeked[0]

    def next_word(self):
        if self.peeked is not None:
            p, self.peeked = self.peeked, None
            return p
        return self._read(512)

    def next(self):
        if self.peeked is not None:
            p, self.peeked = self.peeked, None
            return p[0]
        return self._read(64)[0]

    def skip_line(self):
        while self.next() not in (NEWLINE, END):
            pass


def read_float(lx: Lexer) -> float:
    kind, w = lx.next_word()
    if kind != WORD:
        raise IngestError(f"OBJ: expected number, got {kind}")
    v = parse_float(w) if len(w) <= 32 else None
    if v is None:
        raise IngestError(f"OBJ: invalid number '{w}'")
    return v


def read_int(lx: Lexer) -> int:
    kind, w = lx.next_word()
    if kind != WORD:
        raise IngestError(f"OBJ: expected int, got {kind}")
    v = parse_int(w) if len(w) <= 16 else None
    if v is None:
        raise IngestError(f"OBJ: invalid int '{w}'")
    return v


def read_index(lx: Lexer, count: int) -> int:
    idx = read_int(lx)
    idx = count + idx if idx < 0 else idx - 1
    if idx < 0 or idx >= count:
        raise IngestError(f"OBJ: index out of bounds ({idx}, count: {count})")
    return idx


# ---- images --------------------------------------------------------------------------------------

def load_tga(path: str) -> np.ndarray:
    """Image.LoadTga: (H, W, 3) RGB8, rows top-down."""
    d = read_file(path)
    if len(d) < 18:
        raise IngestError("TGA: truncated header")
    cmap, itype = d[1], d[2]
    w, h = d[12] | d[13] << 8, d[14] | d[15] << 8
    bpp, desc = d[16], d[17]
    if cmap != 0:
        raise IngestError("TGA: Color-mapped images not supported")
    if itype not in (2, 3):
        raise IngestError(f"TGA: Unsupported image type {itype}")
    if itype == 2 and bpp != 24:
        raise IngestError(f"TGA: Only 24-bit TrueColor images supported, got {bpp}-bit")
    if itype == 3 and bpp != 8:
        raise IngestError(f"TGA: Only 8-bit Grayscale images supported, got {bpp}-bit")
    if w == 0 or h == 0:
        raise IngestError("TGA: empty image")
    ch = 1 if itype == 3 else 3
    body = d[18:18 + w * h * ch]  # the id field is not skipped: pixels start right after the header
    if len(body) < w * h * ch:
        raise IngestError("TGA: truncated pixel data")
    px = np.frombuffer(body, np.uint8).reshape(h, w, ch)
    img = np.repeat(px, 3, axis=2) if ch == 1 else px[:, :, ::-1]
    if (desc & 0x20) == 0:  # bottom-left origin
        img = img[::-1]
    return np.ascontiguousarray(img)


def load_image(path: str) -> np.ndarray:
    ext = path_extension(path)
    if ext == ".tga":
        return load_tga(path)
    if ext in (".ppm", ".bmp"):
        raise IngestError(f"Image: Loading not supported for format '{ext[1:].capitalize()}'")
    raise IngestError(f"Image: Unsupported file format '{ext}'")


def _parse_uint(s: str):
    """uint.Parse(span): white space around, trailing NULs, '+' or '-' (zero only), digits."""
    s = s.rstrip("\0").strip(" \t\n\v\f\r")
    m = re.fullmatch(r"([+-]?)(\d+)", s)
    if not m:
        return None
    v = int(m.group(2))
    if v >= 2**32 or (m.group(1) == "-" and v != 0):
        return None
    return v


def load_hdr(path: str) -> np.ndarray:
    """ImageHdr.LoadHdr: (H, W, 4) RGBE8, rows top-down."""
    d = read_file(path)
    pos = 0

    def byte():
        nonlocal pos
        if pos >= len(d):
            raise IngestError("ImageHdr: unexpected end of file")
        pos += 1
        return d[pos - 1]

    def some(n):  # BinaryReader.Read(Span): a short read at the end of the file
        nonlocal pos
        out = d[pos:pos + n]
        pos += len(out)
        return out

    def line():
        s = []
        while True:
            c = byte()
            if c == 0x0A:
                return "".join(s)
            if c != 0x0D:
                s.append(chr(c))
            if len(s) > 256:
                raise IngestError("ImageHdr: header line longer than 256 characters")

    magic = line()
    if not (magic.startswith("#?RADIANCE") or magic.startswith("#?RGBE")):
        raise IngestError(f"ImageHdr: Invalid magic '{magic}'")
    while line():
        pass
    size = line()
    parts = size.split(" ", 3)
    if len(parts) != 4 or parts[0] != "-Y" or parts[2] != "+X":
        raise IngestError(f"ImageHdr: Unsupported size/orientation '{size}'")
    h, w = _parse_uint(parts[1]), _parse_uint(parts[3])
    if h is None or w is None:
        raise IngestError(f"ImageHdr: invalid size '{size}'")
    if w == 0 or h == 0 or w * h > 2**31:
        raise IngestError(f"ImageHdr: bad size '{size}'")
    out = np.zeros((h, w, 4), np.uint8)
    scan = bytearray(4 * w)
    head = bytearray(4)
    for y in range(h):
        got = some(4)
        head[:len(got)] = got
        if head[0] == 2 and head[1] == 2 and (head[2] & 0x80) == 0:
            lw = head[2] << 8 | head[3]
            if lw != w:
                raise IngestError(f"ImageHdr: Scanline width mismatch ({lw} vs {w})")
            for ch in range(4):
                x = 0
                while x < w:
                    code = byte()
                    if code > 128:
                        n, v = code - 128, byte()
                        if x + n > w:
                            raise IngestError("ImageHdr: run past the scanline")
                        for _ in range(n):
                            scan[4 * x + ch] = v
                            x += 1
                    else:
                        if code == 0:
                            raise IngestError("ImageHdr: empty run")
                        for _ in range(code):
                            if x >= w:
                                raise IngestError("ImageHdr: run past the scanline")
                            scan[4 * x + ch] = byte()
                            x += 1
        else:
            if head[0] == 1 and head[1] == 1 and head[2] == 1:
                raise IngestError("ImageHdr: Old RLE format not supported")
            scan[0:4] = head
            got = some(4 * w - 4)
            scan[4:4 + len(got)] = got
        out[y] = np.frombuffer(bytes(scan), np.uint8).reshape(w, 4)
    return out


# ---- texel conversions ---------------------------------------------------------------------------

def srgb_texels(rgb: np.ndarray) -> np.ndarray:
    """Color.FromPixel: MathF.Pow(c / 255f, 2.233333333f) (the C runtime's powf)."""
    table = np.array([_libm.powf(float(F32(i) / F32(255)), float(F32(2.233333333))) for i in range(256)], np.float32)
    return table[rgb]


def linear_texels(rgb: np.ndarray) -> np.ndarray:
    return rgb.astype(np.float32) / np.float32(255)


def hdr_texels(rgbe: np.ndarray, max_luminance: float = F32_MAX) -> np.ndarray:
    """Color.FromPixel(PixelHdr) then ClampLuminance(max)."""
    e = rgbe[..., 3].astype(np.int32)
    scale = np.array([_libm.powf(2.0, float(k - 128)) for k in range(256)], np.float32)[e] / np.float32(256)
    scale = np.where(e == 0, np.float32(0), scale).astype(np.float32)
    c = rgbe[..., :3].astype(np.float32) * scale[..., None]
    c = np.where((e == 0)[..., None], np.float32(0), c).astype(np.float32)
    r, g, b = c[..., 0], c[..., 1], c[..., 2]
    lum = np.float32(0.2126) * r + np.float32(0.7152) * g + np.float32(0.0722) * b
    mx = np.float32(max_luminance)
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        k = mx / lum
        clamp = lum > mx
        return np.where(clamp[..., None], c * k[..., None], c).astype(np.float32)


# ---- MTL + OBJ -----------------------------------------------------------------------------------

def _material_defaults():
    return dict(albedo=(1.0, 1.0, 1.0), roughness=1.0, metallic=0.0, transparency=0.0, ior=1.5,
                radiance=(0.0, 0.0, 0.0), color_map=None, roughness_map=None, metallic_map=None, normal_map=None)


def parse_mtl(path: str, out: dict) -> None:
    directory = path_directory(path)
    lx = Lexer(read_file(path))
    name = None
    m = _material_defaults()
    pr, has_pr, ns = 1.0, False, 0.0

    def build():
        if name is None:
            return
        with np.errstate(divide="ignore", invalid="ignore"):
            r = pr if has_pr else float(np.sqrt(F32(2) / (F32(ns) + F32(2)), dtype=np.float32))
        done = dict(m)
        done["roughness"] = min(max(r, 0.0), 1.0)
        out[name] = done

    while True:
        kind, w = lx.next_word()
        if kind == END:
            break
        if kind != WORD:
            continue
        if w == "newmtl":
            build()
            _, name = lx.next_word()
            m = _material_defaults()
            pr, has_pr, ns = 1.0, False, 0.0
        elif w in ("Kd", "Ke"):
            c = (read_float(lx), read_float(lx), read_float(lx))
            m["albedo" if w == "Kd" else "radiance"] = c
        elif w == "Pr":
            pr, has_pr = read_float(lx), True
        elif w == "Pm":
            m["metallic"] = read_float(lx)
        elif w == "Ns":
            ns = read_float(lx)
        elif w == "Ni":
            m["ior"] = read_float(lx)
        elif w == "d":
            m["transparency"] = float(F32(1) - F32(read_float(lx)))
        elif w == "Tr":
            m["transparency"] = read_float(lx)
        elif w in ("map_Kd", "map_Pm", "map_Pr", "map_roughness", "map_bump", "norm", "map_Kn"):
            _, file = lx.next_word()
            img = load_image(path_combine(directory, file))
            texels = srgb_texels(img) if w == "map_Kd" else linear_texels(img)
            slot = {"map_Kd": "color_map", "map_Pm": "metallic_map", "map_Pr": "roughness_map",
                    "map_roughness": "roughness_map"}.get(w, "normal_map")
            m[slot] = texels
        lx.skip_line()
    build()


def _triangles(corners) -> np.ndarray:
    """SrTriangles of one object: corners = [(positions (3,3), uvs (3,2), normals (3,3) or None)]."""
    out = np.zeros((len(corners), 36), np.float32)
    plain = [i for i, c in enumerate(corners) if c[2] is None]
    full = [i for i, c in enumerate(corners) if c[2] is not None]
    if plain:
        p = np.array([corners[i][0] for i in plain], np.float32)
        u = np.array([corners[i][1] for i in plain], np.float32)
        out[plain] = oracle.triangles_from_corners(p, u, None, False)
    if full:
        p = np.array([corners[i][0] for i in full], np.float32)
        u = np.array([corners[i][1] for i in full], np.float32)
        n = np.array([corners[i][2] for i in full], np.float32)
        out[full] = oracle.triangles_from_corners(p, u, n, False)
    return out


def parse_obj(path: str, smooth_normals: bool = True) -> list:
    """ObjLoader.Load: a list of objects {name, triangles (N, 36), material (dict) or None}."""
    lx = Lexer(read_file(path))
    positions, normals, uvs = [], [], []
    corners = []
    materials = {}
    file_name = path_stem(path)
    material_name = None
    object_name = None
    objects = []

    def build_object():
        nonlocal corners
        if not corners:
            return
        if smooth_normals and not normals:
            p = np.array([c[0] for c in corners], np.float32)
            u = np.array([c[1] for c in corners], np.float32)
            tris = oracle.triangles_from_corners(p, u, None, True)
        else:
            tris = _triangles(corners)
        name = f"{file_name}_{object_name}" if object_name is not None else f"{file_name}_{len(objects)}"
        mat = dict(materials[material_name]) if material_name is not None and material_name in materials else None
        objects.append(dict(name=name, triangles=tris, material=mat))
        corners = []

    while True:
        kind, w = lx.next_word()
        if kind == END:
            break
        if kind != WORD:
            continue
        if w == "v" or w == "vn":
            (positions if w == "v" else normals).append((read_float(lx), read_float(lx), read_float(lx)))
            lx.skip_line()
        elif w == "vt":
            u, v = read_float(lx), read_float(lx)
            uvs.append((u, float(F32(1) - F32(v))))
            lx.skip_line()
        elif w == "f":
            face = []
            while lx.peek() == WORD:
                pos = read_index(lx, len(positions))
                uv = norm = -1
                if lx.peek() == SLASH:
                    lx.next()
                    if lx.peek() == WORD:
                        uv = read_index(lx, len(uvs))
                    if lx.peek() == SLASH:
                        lx.next()
                        if lx.peek() == WORD:
                            norm = read_index(lx, len(normals))
                face.append((pos, norm, uv))
            if len(face) < 3:
                raise IngestError("OBJ: face has fewer than 3 vertices")
            a = face[0]
            uva = uvs[a[2]] if a[2] >= 0 else (0.0, 0.0)
            for i in range(2, len(face)):
                b, c = face[i - 1], face[i]
                uvb = uvs[b[2]] if b[2] >= 0 else (1.0, 0.0)
                uvc = uvs[c[2]] if c[2] >= 0 else (0.0, 1.0)
                ns = None
                if a[1] >= 0 and b[1] >= 0 and c[1] >= 0:
                    ns = (normals[a[1]], normals[b[1]], normals[c[1]])
                corners.append(((positions[a[0]], positions[b[0]], positions[c[0]]), (uva, uvb, uvc), ns))
        elif w in ("o", "g"):
            build_object()
            if lx.peek() == WORD:
                _, object_name = lx.next_word()
            lx.skip_line()
        elif w == "mtllib":
            _, file = lx.next_word()
            mtl = path_combine(path_directory(path), file)
            if file_exists(mtl):
                parse_mtl(mtl, materials)
            lx.skip_line()
        elif w == "usemtl":
            build_object()
            _, material_name = lx.next_word()
            lx.skip_line()
        else:
            lx.skip_line()
    build_object()
    if not objects:
        raise IngestError("OBJ: no objects found")
    return objects


# ---- image files (Image.WriteTga / WritePpm / WriteBmp image.cs:95-196) -------------------------

def image_bytes(ext: str, rgb: np.ndarray) -> bytes:
    """The bytes Image.Save writes for an (H, W, 3) RGB8 image and an extension."""
    h, w = rgb.shape[:2]
    if ext == ".tga":
        head = bytes([0, 0, 2]) + bytes(9) + (w & 0xFFFF).to_bytes(2, "little") + (h & 0xFFFF).to_bytes(2, "little")
        return head + bytes([24, 0x20]) + rgb[:, :, ::-1].tobytes()
    if ext == ".ppm":
        return f"P6\n{w} {h}\n255\n".encode("ascii") + rgb.tobytes()
    if ext == ".bmp":
        stride = (w * 3 + 3) & ~3
        size = stride * h
        out = bytearray(b"BM")
        for v in (14 + 40 + size, 0, 54, 40, w, (-h) & 0xFFFFFFFF):
            out += int(v).to_bytes(4, "little")
        out += (1).to_bytes(2, "little") + (24).to_bytes(2, "little")
        out += (0).to_bytes(4, "little") + size.to_bytes(4, "little") + bytes(16)
        pad = bytes(stride - w * 3)
        for y in range(h):
            out += rgb[y, :, ::-1].tobytes() + pad
        return bytes(out)
    raise IngestError(f"Image: Unsupported file format '{ext}'")
