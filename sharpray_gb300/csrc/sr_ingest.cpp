// sr_ingest.cpp — asset ingest on the host: Wavefront OBJ + MTL (obj.cs), uncompressed TGA
// (Image.LoadTga image.cs:226-273) and Radiance HDR (ImageHdr.LoadHdr image.cs:307-382), with the
// reference's accepted forms, defaults and error cases.  Parsing only; sr_host.cpp turns the
// results into textures, meshes and scene objects.
#include "sr_ingest.h"

#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <algorithm>
#include <cstring>
#include <fstream>
#include <iterator>
#include <map>
#include <sys/stat.h>

#include "sr_bvh.h"

namespace sr {
namespace host {
namespace {

std::vector<uint8_t> read_file(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw IngestError("cannot open '" + path + "'");
    return std::vector<uint8_t>(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
}

// System.IO.Path on Unix: '/' is the only separator.
std::string extension(const std::string& path) {  // Path.GetExtension: "" when the dot ends the name
    size_t slash = path.find_last_of('/');
    size_t dot = path.find_last_of('.');
    if (dot == std::string::npos || (slash != std::string::npos && dot < slash) || dot + 1 == path.size()) return "";
    return path.substr(dot);
}

std::string directory(const std::string& path) {  // Path.GetDirectoryName ("/" for a file in the root)
    size_t slash = path.find_last_of('/');
    if (slash == std::string::npos) return std::string();
    return slash == 0 ? std::string("/") : path.substr(0, slash);
}

std::string join(const std::string& dir, const std::string& name) {  // Path.Combine
    if (dir.empty() || (!name.empty() && name[0] == '/')) return name;
    if (name.empty()) return dir;
    return dir.back() == '/' ? dir + name : dir + "/" + name;
}

bool is_file(const std::string& path) {  // File.Exists: a regular file (not a directory)
    struct stat st;
    return !path.empty() && ::stat(path.c_str(), &st) == 0 && S_ISREG(st.st_mode);
}

std::string stem(const std::string& path) {
    size_t slash = path.find_last_of('/');
    std::string base = slash == std::string::npos ? path : path.substr(slash + 1);
    size_t dot = base.find_last_of('.');
    return dot == std::string::npos ? base : base.substr(0, dot);
}

// ---- OBJ lexer (ObjLexer obj.cs:20-128): words, '/', newlines; '#' comments to end of line;
// spaces, tabs and carriage returns separate words.  A word longer than the buffer it is read into
// fails the load: 512 characters for words the parser keeps, 64 for words it skips (Next() without
// a buffer reads into a 64-character scratch span).
enum class Tok { Word, Slash, Newline, End };

class Lexer {
public:
    explicit Lexer(std::vector<uint8_t> data) : d_(std::move(data)) {
        // StreamReader drops a UTF-8 byte order mark
        if (d_.size() >= 3 && d_[0] == 0xEF && d_[1] == 0xBB && d_[2] == 0xBF) pos_ = 3;
    }

    Tok peek() {
        if (!has_peek_) {
            peek_kind_ = read(peek_word_, 512);
            has_peek_ = true;
        }
        return peek_kind_;
    }
    Tok next(std::string& word) {
        if (has_peek_) {
            has_peek_ = false;
            word = peek_word_;
            return peek_kind_;
        }
        return read(word, 512);
    }
    Tok next() {
        if (has_peek_) {
            has_peek_ = false;
            return peek_kind_;
        }
        std::string scratch;
        return read(scratch, 64);
    }
    void skip_line() {
        Tok k;
        do {
            k = next();
        } while (k != Tok::Newline && k != Tok::End);
    }

private:
    static bool word_end(int c) { return c == ' ' || c == '\t' || c == '\r' || c == '\n' || c == '/'; }
    Tok read(std::string& word, size_t limit) {
        word.clear();
        for (;;) {
            if (pos_ >= d_.size()) return Tok::End;
            int c = d_[pos_++];
            switch (c) {
                case '\n': return Tok::Newline;
                case '/': return Tok::Slash;
                case ' ':
                case '\t':
                case '\r': continue;
                case '#':
                    for (;;) {
                        if (pos_ >= d_.size()) return Tok::End;
                        if (d_[pos_++] == '\n') return Tok::Newline;
                    }
                default:
                    word.push_back((char)c);
                    while (pos_ < d_.size() && !word_end(d_[pos_])) word.push_back((char)d_[pos_++]);
                    if (word.size() > limit)
                        throw IngestError("OBJ: word longer than " + std::to_string(limit) + " characters");
                    return Tok::Word;
            }
        }
    }
    std::vector<uint8_t> d_;
    size_t pos_ = 0;
    bool has_peek_ = false;
    Tok peek_kind_ = Tok::End;
    std::string peek_word_;
};

const char* tok_name(Tok k) {
    switch (k) {
        case Tok::Word: return "Word";
        case Tok::Slash: return "Slash";
        case Tok::Newline: return "Newline";
        default: return "End";
    }
}

// .NET number parsing trims white space (tab to carriage return, space) around the text and NULs
// after it.
std::string trim_number(const std::string& s) {
    auto white = [](char c) { return c == ' ' || (c >= '\t' && c <= '\r'); };
    size_t b = 0, e = s.size();
    while (e > 0 && s[e - 1] == '\0') --e;
    while (b < e && white(s[b])) ++b;
    while (e > b && white(s[e - 1])) --e;
    return s.substr(b, e - b);
}

bool equals_ci(const std::string& a, const char* b) {
    size_t n = std::strlen(b);
    if (a.size() != n) return false;
    for (size_t i = 0; i < n; ++i) {
        char x = a[i], y = b[i];
        if (x >= 'A' && x <= 'Z') x = (char)(x - 'A' + 'a');
        if (y >= 'A' && y <= 'Z') y = (char)(y - 'A' + 'a');
        if (x != y) return false;
    }
    return true;
}

// float.TryParse(NumberStyles.Float, InvariantCulture): optional sign, digits with an optional
// decimal point (at least one digit), optional exponent; or, ignoring case, the invariant symbols
// Infinity, -Infinity and NaN (also +Infinity, +NaN, -NaN).  The value is the correctly rounded
// float (strtof), +-infinity past the float range.
bool parse_float(const std::string& word, float& out) {
    const std::string s = trim_number(word);
    if (equals_ci(s, "Infinity") || equals_ci(s, "+Infinity")) return out = INFINITY, true;
    if (equals_ci(s, "-Infinity")) return out = -INFINITY, true;
    if (equals_ci(s, "NaN") || equals_ci(s, "+NaN") || equals_ci(s, "-NaN")) return out = NAN, true;
    size_t i = 0, n = s.size();
    if (i < n && (s[i] == '+' || s[i] == '-')) ++i;
    size_t digits = 0;
    while (i < n && s[i] >= '0' && s[i] <= '9') ++i, ++digits;
    if (i < n && s[i] == '.') {
        ++i;
        while (i < n && s[i] >= '0' && s[i] <= '9') ++i, ++digits;
    }
    if (digits == 0) return false;
    if (i < n && (s[i] == 'e' || s[i] == 'E')) {
        ++i;
        if (i < n && (s[i] == '+' || s[i] == '-')) ++i;
        size_t ed = 0;
        while (i < n && s[i] >= '0' && s[i] <= '9') ++i, ++ed;
        if (ed == 0) return false;
    }
    if (i != n) return false;
    out = std::strtof(s.c_str(), nullptr);
    return true;
}

// int.TryParse (NumberStyles.Integer): optional sign and decimal digits, within int range.
bool parse_int(const std::string& word, int& out) {
    const std::string s = trim_number(word);
    size_t i = 0, n = s.size();
    bool neg = false;
    if (i < n && (s[i] == '+' || s[i] == '-')) neg = s[i++] == '-';
    if (i == n) return false;
    long long v = 0;
    for (; i < n; ++i) {
        if (s[i] < '0' || s[i] > '9') return false;
        v = v * 10 + (s[i] - '0');
        if (v > 2147483648LL) return false;
    }
    if (neg) v = -v;
    if (v > 2147483647LL || v < -2147483648LL) return false;
    out = (int)v;
    return true;
}

float read_float(Lexer& lx) {
    std::string w;
    Tok k = lx.next(w);
    if (k != Tok::Word) throw IngestError(std::string("OBJ: expected number, got ") + tok_name(k));
    if (w.size() > 32) throw IngestError("OBJ: invalid number '" + w + "'");
    float v;
    if (!parse_float(w, v)) throw IngestError("OBJ: invalid number '" + w + "'");
    return v;
}

int read_int(Lexer& lx) {
    std::string w;
    Tok k = lx.next(w);
    if (k != Tok::Word) throw IngestError(std::string("OBJ: expected int, got ") + tok_name(k));
    int v;
    if (w.size() > 16 || !parse_int(w, v)) throw IngestError("OBJ: invalid int '" + w + "'");
    return v;
}

// ObjLoader.ReadIndex obj.cs:472-480: 1-based, negative = relative to the end.
int read_index(Lexer& lx, int count) {
    int idx = read_int(lx);
    idx = idx < 0 ? count + idx : idx - 1;
    if (idx < 0 || idx >= count)
        throw IngestError("OBJ: index out of bounds (" + std::to_string(idx) + ", count: " + std::to_string(count) + ")");
    return idx;
}

struct V3f {
    float v[3];
};
struct V2f {
    float v[2];
};

// ObjLoader.ParseMtl obj.cs:261-401.
void parse_mtl(const std::string& path, std::map<std::string, ObjMaterial>& out) {
    const std::string dir = directory(path);
    Lexer lx(read_file(path));
    bool have = false;
    std::string name;
    ObjMaterial m;
    float roughness = 1.0f, ns = 0.0f;
    bool has_pr = false;
    auto reset = [&]() {
        m = ObjMaterial{};
        roughness = 1.0f, ns = 0.0f, has_pr = false;
    };
    auto build = [&]() {
        if (!have) return;
        // Math.Clamp(hasPr ? roughness : MathF.Sqrt(2 / (ns + 2)), 0, 1)
        float r = has_pr ? roughness : std::sqrt(2.0f / (ns + 2.0f));
        m.roughness = r < 0.0f ? 0.0f : (r > 1.0f ? 1.0f : r);
        out[name] = m;
    };
    reset();
    std::string w;
    for (;;) {
        Tok k = lx.next(w);
        if (k == Tok::End) break;
        if (k != Tok::Word) continue;
        if (w == "newmtl") {
            build();
            std::string nm;
            lx.next(nm);
            name = nm;
            have = true;
            reset();
            lx.skip_line();
        } else if (w == "Kd" || w == "Ke") {
            float c[3];
            for (float& x : c) x = read_float(lx);
            std::memcpy(w == "Kd" ? m.albedo : m.radiance, c, sizeof(c));
            lx.skip_line();
        } else if (w == "Pr") {
            roughness = read_float(lx), has_pr = true;
            lx.skip_line();
        } else if (w == "Pm") {
            m.metallic = read_float(lx);
            lx.skip_line();
        } else if (w == "Ns") {
            ns = read_float(lx);
            lx.skip_line();
        } else if (w == "Ni") {
            m.ior = read_float(lx);
            lx.skip_line();
        } else if (w == "d") {
            m.transparency = 1.0f - read_float(lx);  // d = 1 is opaque
            lx.skip_line();
        } else if (w == "Tr") {
            m.transparency = read_float(lx);
            lx.skip_line();
        } else if (w == "map_Kd" || w == "map_Pm" || w == "map_Pr" || w == "map_roughness" || w == "map_bump" ||
                   w == "norm" || w == "map_Kn") {
            // Texture.FromSrgb(Image.Load(..)) for map_Kd, FromLinear for the others (obj.cs:365-390)
            std::string file;
            lx.next(file);
            ObjImagePtr* slot = w == "map_Kd" ? &m.color_map
                              : w == "map_Pm" ? &m.metallic_map
                              : (w == "map_Pr" || w == "map_roughness") ? &m.roughness_map
                                                                          : &m.normal_map;
            auto img = std::make_shared<ObjImage>();
            img->path = join(dir, file);
            std::vector<uint8_t> rgb;
            load_image(img->path, img->width, img->height, rgb);
            img->texels.resize((size_t)img->width * img->height * 3);
            rgb8_to_texels(rgb.data(), (size_t)img->width * img->height, w == "map_Kd", img->texels.data());
            *slot = std::move(img);
            lx.skip_line();
        } else {
            lx.skip_line();
        }
    }
    build();
}

}  // namespace

// ObjLoader.Load + Parse obj.cs:139-259 (objects are returned, not added: see ObjResult).
ObjResult parse_obj(const std::string& path, bool smooth_normals) {
    Lexer lx(read_file(path));
    ObjResult res;
    std::vector<V3f> positions, normals;
    std::vector<V2f> uvs;
    std::vector<SrTriangle> triangles;
    struct Entry {
        int pos, norm, uv;
    };
    std::vector<Entry> face;
    const std::string file_name = stem(path);
    bool has_material = false, has_object_name = false;
    std::string material_name, object_name;
    int object_count = 0;

    auto build_object = [&]() {
        if (triangles.empty()) return;
        if (smooth_normals && normals.empty()) compute_smooth_normals(triangles.data(), (uint32_t)triangles.size());
        ObjObject o;
        o.name = has_object_name ? file_name + "_" + object_name : file_name + "_" + std::to_string(object_count);
        auto found = has_material ? res.materials.find(material_name) : res.materials.end();
        o.has_material = found != res.materials.end();
        if (o.has_material) o.material_name = material_name, o.material = found->second;
        o.triangles.swap(triangles);
        res.objects.push_back(std::move(o));
        triangles.clear();
        ++object_count;
    };

    std::string w;
    for (;;) {
        Tok k = lx.next(w);
        if (k == Tok::End) break;
        if (k != Tok::Word) continue;
        if (w == "v" || w == "vn") {
            V3f p;
            for (float& x : p.v) x = read_float(lx);
            (w == "v" ? positions : normals).push_back(p);
            lx.skip_line();
        } else if (w == "vt") {
            V2f t;
            t.v[0] = read_float(lx);
            float v = read_float(lx);
            t.v[1] = 1.0f - v;  // OBJ is bottom-left, textures top-left
            uvs.push_back(t);
            lx.skip_line();
        } else if (w == "f") {
            // ReadFace obj.cs:445-470
            face.clear();
            while (lx.peek() == Tok::Word) {
                Entry e{read_index(lx, (int)positions.size()), -1, -1};
                if (lx.peek() == Tok::Slash) {
                    lx.next();
                    if (lx.peek() == Tok::Word) e.uv = read_index(lx, (int)uvs.size());
                    if (lx.peek() == Tok::Slash) {
                        lx.next();
                        if (lx.peek() == Tok::Word) e.norm = read_index(lx, (int)normals.size());
                    }
                }
                face.push_back(e);
            }
            // TriangulateFace obj.cs:403-443: a fan from the first vertex
            if (face.size() < 3) throw IngestError("OBJ: face has fewer than 3 vertices");
            static const float kUvA[2] = {0, 0}, kUvB[2] = {1, 0}, kUvC[2] = {0, 1};
            const Entry& a = face[0];
            const float* uva = a.uv >= 0 ? uvs[a.uv].v : kUvA;
            for (size_t i = 2; i < face.size(); ++i) {
                const Entry& b = face[i - 1];
                const Entry& c = face[i];
                const float* uvb = b.uv >= 0 ? uvs[b.uv].v : kUvB;
                const float* uvc = c.uv >= 0 ? uvs[c.uv].v : kUvC;
                SrTriangle t;
                if (a.norm >= 0 && b.norm >= 0 && c.norm >= 0) {
                    float ns[9];
                    std::memcpy(ns, normals[a.norm].v, 12);
                    std::memcpy(ns + 3, normals[b.norm].v, 12);
                    std::memcpy(ns + 6, normals[c.norm].v, 12);
                    make_triangle_corners(positions[a.pos].v, positions[b.pos].v, positions[c.pos].v, ns, uva, uvb, uvc, &t);
                } else {
                    make_triangle_corners(positions[a.pos].v, positions[b.pos].v, positions[c.pos].v, nullptr, uva, uvb,
                                          uvc, &t);
                }
                triangles.push_back(t);
            }
        } else if (w == "o" || w == "g") {
            build_object();
            if (lx.peek() == Tok::Word) {
                lx.next(object_name);
                has_object_name = true;
            }
            lx.skip_line();
        } else if (w == "mtllib") {
            std::string file;
            lx.next(file);
            std::string mtl = join(directory(path), file);
            if (is_file(mtl)) parse_mtl(mtl, res.materials);
            lx.skip_line();
        } else if (w == "usemtl") {
            build_object();
            std::string nm;
            lx.next(nm);
            material_name = nm;
            has_material = true;
            lx.skip_line();
        } else {
            lx.skip_line();
        }
    }
    build_object();
    if (object_count == 0) throw IngestError("OBJ: no objects found");
    return res;
}

// Image.LoadTga image.cs:226-273: uncompressed 24-bit TrueColor or 8-bit Grayscale, rows flipped
// to top-down unless the descriptor says top-left origin.  Pixels as RGB8.
void load_tga(const std::string& path, uint32_t& width, uint32_t& height, std::vector<uint8_t>& rgb) {
    std::vector<uint8_t> d = read_file(path);
    if (d.size() < 18) throw IngestError("TGA: truncated header");
    const uint8_t id_length = d[0];
    (void)id_length;  // the reference skips it without skipping the id field itself
    const uint8_t color_map_type = d[1], image_type = d[2];
    width = (uint32_t)d[12] | ((uint32_t)d[13] << 8);
    height = (uint32_t)d[14] | ((uint32_t)d[15] << 8);
    const uint8_t bpp = d[16], descriptor = d[17];
    if (color_map_type != 0) throw IngestError("TGA: Color-mapped images not supported");
    if (image_type != 2 && image_type != 3)
        throw IngestError("TGA: Unsupported image type " + std::to_string(image_type) +
                          " (only uncompressed TrueColor and Grayscale supported)");
    if (image_type == 2 && bpp != 24)
        throw IngestError("TGA: Only 24-bit TrueColor images supported, got " + std::to_string(bpp) + "-bit");
    if (image_type == 3 && bpp != 8)
        throw IngestError("TGA: Only 8-bit Grayscale images supported, got " + std::to_string(bpp) + "-bit");
    if (width == 0 || height == 0) throw IngestError("TGA: empty image");
    const size_t n = (size_t)width * height;
    const size_t need = 18 + n * (image_type == 3 ? 1 : 3);
    if (d.size() < need) throw IngestError("TGA: truncated pixel data");
    rgb.resize(n * 3);
    const uint8_t* p = d.data() + 18;
    for (size_t i = 0; i < n; ++i) {
        if (image_type == 3) {
            rgb[3 * i] = rgb[3 * i + 1] = rgb[3 * i + 2] = p[i];
        } else {
            rgb[3 * i] = p[3 * i + 2], rgb[3 * i + 1] = p[3 * i + 1], rgb[3 * i + 2] = p[3 * i];  // BGR on disk
        }
    }
    if ((descriptor & 0x20) == 0) {  // bottom-left origin: Image.FlipVertical
        for (uint32_t y = 0; y < height / 2; ++y)
            for (uint32_t x = 0; x < 3 * width; ++x)
                std::swap(rgb[(size_t)y * 3 * width + x], rgb[(size_t)(height - 1 - y) * 3 * width + x]);
    }
}

// ImageHdr.LoadHdr image.cs:307-382: "#?RADIANCE" or "#?RGBE" magic, header lines to an empty
// line, "-Y h +X w", then scanlines either new-style RLE (per channel runs) or flat RGBE.
void load_hdr(const std::string& path, uint32_t& width, uint32_t& height, std::vector<uint8_t>& rgbe) {
    std::vector<uint8_t> d = read_file(path);
    size_t pos = 0;
    auto byte = [&]() -> uint8_t {  // BinaryReader.ReadByte: the end of the file is an error
        if (pos >= d.size()) throw IngestError("ImageHdr: unexpected end of file");
        return d[pos++];
    };
    auto read_some = [&](uint8_t* dst, size_t n) {  // BinaryReader.Read(Span): short at the end, no error
        size_t k = std::min(n, d.size() - pos);
        std::memcpy(dst, d.data() + pos, k);
        pos += k;
    };
    auto line = [&]() {
        std::string s;
        for (;;) {
            uint8_t c = byte();
            if (c == '\n') return s;
            if (c != '\r') s.push_back((char)c);
            if (s.size() > 256) throw IngestError("ImageHdr: header line longer than 256 characters");
        }
    };
    std::string magic = line();
    if (magic.rfind("#?RADIANCE", 0) != 0 && magic.rfind("#?RGBE", 0) != 0)
        throw IngestError("ImageHdr: Invalid magic '" + magic + "'");
    while (!line().empty()) {
    }
    std::string size = line();
    // MemoryExtensions.Split(span, Range[4], ' '): at most 4 parts, the last one keeps the rest.
    std::vector<std::string> parts;
    for (size_t i = 0;;) {
        size_t j = parts.size() == 3 ? std::string::npos : size.find(' ', i);
        parts.push_back(size.substr(i, j == std::string::npos ? std::string::npos : j - i));
        if (j == std::string::npos) break;
        i = j + 1;
    }
    // uint.Parse (NumberStyles.Integer): surrounding white space, trailing NULs, a sign ("-" only
    // for zero), decimal digits within uint range.
    auto parse_u = [&](const std::string& str, uint32_t& v) {
        auto white = [](char c) { return c == ' ' || (c >= '\t' && c <= '\r'); };
        size_t b0 = 0, e0 = str.size();
        while (e0 > 0 && str[e0 - 1] == '\0') --e0;
        while (b0 < e0 && white(str[b0])) ++b0;
        while (e0 > b0 && white(str[e0 - 1])) --e0;
        bool neg = false;
        if (b0 < e0 && (str[b0] == '+' || str[b0] == '-')) neg = str[b0++] == '-';
        if (b0 == e0) return false;
        unsigned long long x = 0;
        for (size_t i = b0; i < e0; ++i) {
            if (str[i] < '0' || str[i] > '9') return false;
            x = x * 10 + (uint32_t)(str[i] - '0');
            if (x > 0xffffffffull) return false;
        }
        if (neg && x != 0) return false;
        v = (uint32_t)x;
        return true;
    };
    if (parts.size() != 4 || parts[0] != "-Y" || parts[2] != "+X")
        throw IngestError("ImageHdr: Unsupported size/orientation '" + size + "'");
    if (!parse_u(parts[1], height) || !parse_u(parts[3], width))
        throw IngestError("ImageHdr: invalid size '" + size + "'");
    if (width == 0 || height == 0 || (uint64_t)width * height > (1ull << 31))
        throw IngestError("ImageHdr: bad size '" + size + "'");
    rgbe.assign((size_t)width * height * 4, 0);
    // Both buffers live across scanlines and start zeroed: a short read at the end of the file leaves
    // the previous scanline's bytes in place, as the reference's stack buffers do.
    std::vector<uint8_t> scan((size_t)width * 4, 0);
    uint8_t hdr[4] = {0, 0, 0, 0};
    for (uint32_t y = 0; y < height; ++y) {
        read_some(hdr, 4);
        if (hdr[0] == 2 && hdr[1] == 2 && (hdr[2] & 0x80) == 0) {
            uint32_t line_width = ((uint32_t)hdr[2] << 8) | hdr[3];
            if (line_width != width)
                throw IngestError("ImageHdr: Scanline width mismatch (" + std::to_string(line_width) + " vs " +
                                  std::to_string(width) + ")");
            for (int ch = 0; ch < 4; ++ch) {
                for (uint32_t x = 0; x < width;) {
                    uint8_t code = byte();
                    if (code > 128) {
                        uint32_t count = code - 128u;
                        uint8_t v = byte();
                        if (x + count > width) throw IngestError("ImageHdr: run past the scanline");
                        for (uint32_t i = 0; i < count; ++i) scan[4 * (size_t)x++ + ch] = v;
                    } else {
                        // a zero-length literal never advances: the reference loops forever on it
                        if (code == 0) throw IngestError("ImageHdr: empty run");
                        for (uint32_t i = 0; i < code; ++i) {
                            if (x >= width) throw IngestError("ImageHdr: run past the scanline");
                            scan[4 * (size_t)x++ + ch] = byte();
                        }
                    }
                }
            }
        } else {
            if (hdr[0] == 1 && hdr[1] == 1 && hdr[2] == 1) throw IngestError("ImageHdr: Old RLE format not supported");
            std::memcpy(scan.data(), hdr, 4);
            read_some(scan.data() + 4, scan.size() - 4);
        }
        std::memcpy(rgbe.data() + (size_t)y * width * 4, scan.data(), scan.size());
    }
}

// Color.FromPixel (sRGB decode) math.cs:184-191, FromPixelLinear :193-194, FromPixel(PixelHdr)
// :196-202 + ClampLuminance :118-122 (Texture.FromSrgb/FromLinear/FromHdr texture.cs:138-163).
void rgb8_to_texels(const uint8_t* rgb, size_t n, bool srgb, float* out) {
    for (size_t i = 0; i < 3 * n; ++i) {
        float c = (float)rgb[i] / 255.0f;
        out[i] = srgb ? std::pow(c, 2.233333333f) : c;
    }
}

void rgbe_to_texels(const uint8_t* rgbe, size_t n, float max_luminance, float* out) {
    for (size_t i = 0; i < n; ++i) {
        const uint8_t* p = rgbe + 4 * i;
        float r = 0, g = 0, b = 0;
        if (p[3] != 0) {
            float scale = std::pow(2.0f, (float)((int)p[3] - 128)) / 256.0f;
            r = (float)p[0] * scale, g = (float)p[1] * scale, b = (float)p[2] * scale;
        }
        float lum = 0.2126f * r + 0.7152f * g + 0.0722f * b;
        if (lum > max_luminance) {
            float k = max_luminance / lum;
            r *= k, g *= k, b *= k;
        }
        out[3 * i] = r, out[3 * i + 1] = g, out[3 * i + 2] = b;
    }
}

// Image.Load by extension (image.cs:214-224, FormatFromPath :275-282): only .tga loads.
void load_image(const std::string& path, uint32_t& width, uint32_t& height, std::vector<uint8_t>& rgb) {
    std::string ext = extension(path);
    if (ext == ".tga") return load_tga(path, width, height, rgb);
    if (ext == ".ppm" || ext == ".bmp") {
        std::string fmt = ext == ".ppm" ? "Ppm" : "Bmp";
        throw IngestError("Image: Loading not supported for format '" + fmt + "'");
    }
    throw IngestError("Image: Unsupported file format '" + ext + "'");
}

}  // namespace host
}  // namespace sr
