// sr_image.cpp — host side of the image conveniences: Color.ToPixel for overlay colours, the
// overlay's projection and text layout (View.Project math.cs:1638-1663, Overlay.Draw and
// RasterizeText overlay.cs:54-196), the samples-image table (program.cs:247-256) and the
// Image.Save writers (image.cs:88-212).  The device draws what this plans (sr_overlay.cu).
#include "sr_image.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "sr_bvh.h"

namespace sr {
namespace host {
namespace {

// (byte)f in .NET 8: truncation to int (0 for NaN and outside the int range), low 8 bits.
uint8_t net_byte(float f) {
    if (!(std::fabs(f) < 2147483648.0f)) return 0;
    return (uint8_t)(uint32_t)(int32_t)f;
}

float clamp01(float x) { return x < 0.0f ? 0.0f : (x > 1.0f ? 1.0f : x); }  // Math.Clamp: NaN passes

// Vec2.RoundToInt math.cs:261: MathF.Round (half to even), then (int).  False outside the int range.
bool round_to_int(float v, int32_t& out) {
    float r = std::nearbyint(v);
    if (!(std::fabs(r) < 2147483648.0f)) return false;
    out = (int32_t)r;
    return true;
}

// View.Project math.cs:1638-1663.
bool project(const SrView& v, F3 p, float aspect, float& sx, float& sy, float& depth) {
    const SrTransform& t = v.transform;
    Quat inv{-t.rot[0], -t.rot[1], -t.rot[2], t.rot[3]};
    F3 local = rotate(inv, p - F3{t.pos[0], t.pos[1], t.pos[2]}) / F3{t.scale[0], t.scale[1], t.scale[2]};
    if (local.z <= v.near_plane) return false;
    float th, tv;
    if (aspect >= 1.0f) {
        th = std::tan(v.fov * 0.5f);
        tv = th / aspect;
    } else {
        tv = std::tan(v.fov * 0.5f);
        th = tv * aspect;
    }
    F3 from_near{local.x, local.y, local.z - v.near_plane};
    float ndc_x = (from_near.x / from_near.z) / th;
    float ndc_y = (from_near.y / from_near.z) / tv;
    sx = (ndc_x + 1.0f) * 0.5f;
    sy = (1.0f - ndc_y) * 0.5f;
    depth = magnitude(from_near);
    return true;
}

// RasterizeText overlay.cs:172-196: '\n' separated lines (at most 64 ranges, the last one keeps the
// rest), optionally centred on the coordinate; one glyph op per character the font has.
void layout_text(const char* text, int32_t x, int32_t y, int32_t align, const SrFont& font, int32_t entry,
                 std::vector<OverlayGlyphOp>& out) {
    std::vector<std::string> lines;
    std::string s(text ? text : "");
    for (size_t i = 0;;) {
        size_t j = lines.size() == 63 ? std::string::npos : s.find('\n', i);
        lines.push_back(s.substr(i, j == std::string::npos ? std::string::npos : j - i));
        if (j == std::string::npos) break;
        i = j + 1;
    }
    if (align == SR_ALIGN_CENTER) {
        int32_t width = 0;
        for (const std::string& l : lines) width = std::max(width, (int32_t)l.size());
        x -= width * 8 / 2;
        y -= (int32_t)lines.size() * 8 / 2;
    }
    for (size_t li = 0; li < lines.size(); ++li) {
        const std::string& l = lines[li];
        for (size_t c = 0; c < l.size(); ++c) {
            int32_t ch = (unsigned char)l[c];
            if (ch < font.first_char || ch > font.last_char) continue;
            out.push_back(OverlayGlyphOp{x + (int32_t)c * 8, y + (int32_t)li * 8, ch - font.first_char, entry});
        }
    }
}

void put16(std::vector<uint8_t>& b, uint32_t v) {
    b.push_back((uint8_t)v), b.push_back((uint8_t)(v >> 8));
}
void put32(std::vector<uint8_t>& b, uint32_t v) {
    for (int i = 0; i < 4; ++i) b.push_back((uint8_t)(v >> (8 * i)));
}

std::string extension(const std::string& path) {  // Path.GetExtension on Unix
    size_t slash = path.find_last_of('/');
    size_t dot = path.find_last_of('.');
    if (dot == std::string::npos || (slash != std::string::npos && dot < slash) || dot + 1 == path.size()) return "";
    return path.substr(dot);
}

}  // namespace

uint32_t color_to_pixel(const float rgb[3]) {
    uint32_t out = 0;
    for (int k = 0; k < 3; ++k) {
        float c = clamp01(rgb[k]);
        float e = net_max(1.055f * std::pow(c, 0.416666667f) - 0.055f, 0.0f);
        out |= (uint32_t)net_byte(e * 255.0f + 0.5f) << (8 * k);
    }
    return out;
}

OverlayPlan plan_overlay(uint32_t width, uint32_t height, const SrView& view, const SrOverlayLine* lines,
                         uint32_t line_count, const SrOverlayText* texts, uint32_t text_count, const SrFont* font) {
    OverlayPlan plan;
    const float aspect = (float)width / (float)height;
    const float size_x = (float)width, size_y = (float)height;
    int32_t entry = 0;
    for (uint32_t i = 0; i < line_count; ++i) {
        const SrOverlayLine& l = lines[i];
        float ax, ay, da, bx, by, db;
        if (project(view, F3{l.a[0], l.a[1], l.a[2]}, aspect, ax, ay, da) &&
            project(view, F3{l.b[0], l.b[1], l.b[2]}, aspect, bx, by, db)) {
            OverlayLineOp op{};
            if (!round_to_int(ax * size_x, op.ax) || !round_to_int(ay * size_y, op.ay) ||
                !round_to_int(bx * size_x, op.bx) || !round_to_int(by * size_y, op.by))
                throw ImageError("overlay line " + std::to_string(i) + ": end point outside the int range");
            const int64_t span = std::max(std::llabs((int64_t)op.bx - op.ax), std::llabs((int64_t)op.by - op.ay));
            if (span > (1 << 24))
                throw ImageError("overlay line " + std::to_string(i) + " spans " + std::to_string(span) +
                                 " pixels (limit 2^24)");
            const float bias = 1.0f - l.depth_bias;
            op.inv_a = 1.0f / (da * bias);
            op.inv_b = 1.0f / (db * bias);
            op.depth_test = l.depth_test != 0;
            op.entry = entry;
            plan.lines.push_back(op);
        }
        plan.colors.push_back(color_to_pixel(l.color));
        ++entry;
    }
    for (int pass = 0; pass < 2; ++pass) {  // world-space texts, then screen-space texts
        for (uint32_t i = 0; i < text_count; ++i) {
            const SrOverlayText& t = texts[i];
            if ((t.in_world != 0) != (pass == 0)) continue;
            int32_t x = t.screen_pos[0], y = t.screen_pos[1];
            bool draw = true;
            if (pass == 0) {
                float sx, sy, d;
                draw = project(view, F3{t.world_pos[0], t.world_pos[1], t.world_pos[2]}, aspect, sx, sy, d) &&
                       round_to_int(sx * size_x, x) && round_to_int(sy * size_y, y);
            }
            if (draw && font && font->glyphs) layout_text(t.text, x, y, t.align, *font, entry, plan.glyphs);
            plan.colors.push_back(color_to_pixel(t.color));
            ++entry;
        }
    }
    return plan;
}

std::vector<uint8_t> samples_table(uint32_t min_samples, uint32_t max_samples, float* log_range) {
    const float range = std::log2((float)max_samples / (float)min_samples);
    std::vector<uint8_t> t((size_t)max_samples + 2);
    for (size_t s = 0; s < t.size(); ++s)
        t[s] = net_byte(std::log2((float)s / (float)min_samples) / range * 255.0f);
    if (log_range) *log_range = range;
    return t;
}

void save_image(const std::string& path, uint32_t width, uint32_t height, const uint8_t* rgb) {
    const std::string ext = extension(path);
    const size_t n = (size_t)width * height;
    std::vector<uint8_t> b;
    if (ext == ".tga") {  // WriteTga image.cs:95-123
        b = {0, 0, 2, 0, 0, 0, 0, 0, 0, 0, 0, 0};
        put16(b, width & 0xffff);
        put16(b, height & 0xffff);
        b.push_back(24);
        b.push_back(0x20);
        for (size_t i = 0; i < n; ++i) b.push_back(rgb[3 * i + 2]), b.push_back(rgb[3 * i + 1]), b.push_back(rgb[3 * i]);
    } else if (ext == ".ppm") {  // WritePpm image.cs:125-146
        char head[64];
        int k = std::snprintf(head, sizeof(head), "P6\n%u %u\n255\n", width, height);
        b.assign(head, head + k);
        b.insert(b.end(), rgb, rgb + 3 * n);
    } else if (ext == ".bmp") {  // WriteBmp image.cs:148-196
        const uint32_t stride = (width * 3u + 3u) & ~3u;
        const uint32_t data = stride * height;
        b = {'B', 'M'};
        put32(b, 14u + 40u + data);
        put32(b, 0);
        put32(b, 54);
        put32(b, 40);
        put32(b, width);
        put32(b, (uint32_t)(-(int32_t)height));
        put16(b, 1);
        put16(b, 24);
        put32(b, 0);
        put32(b, data);
        b.insert(b.end(), 16, 0);
        const uint32_t pad = stride - width * 3u;
        for (uint32_t y = 0; y < height; ++y) {
            for (uint32_t x = 0; x < width; ++x) {
                const uint8_t* p = rgb + 3 * ((size_t)y * width + x);
                b.push_back(p[2]), b.push_back(p[1]), b.push_back(p[0]);
            }
            b.insert(b.end(), pad, 0);
        }
    } else {
        throw ImageError("Image: Unsupported file format '" + ext + "'");
    }
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) throw ImageError("cannot write '" + path + "'");
    const bool ok = std::fwrite(b.data(), 1, b.size(), f) == b.size();
    if (std::fclose(f) != 0 || !ok) throw ImageError("cannot write '" + path + "'");
}

}  // namespace host
}  // namespace sr
