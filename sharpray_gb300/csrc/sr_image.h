// sr_image.h — host side of the image conveniences (sr_image.cpp): overlay planning (projection,
// text layout, colours), the samples-image table and the image file writers.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/sharpray.h"
#include "sr_kernels.h"

namespace sr {
namespace host {

struct ImageError : std::runtime_error {
    explicit ImageError(const std::string& m) : std::runtime_error(m) {}
};

// Color.ToPixel math.cs:127-136 packed as r | g << 8 | b << 16.
uint32_t color_to_pixel(const float rgb[3]);

// Overlay.Draw overlay.cs:54-96 flattened into device work: line end points and depths, glyph
// cells, and one packed colour per draw entry (lines, then world texts, then screen texts).
struct OverlayPlan {
    std::vector<OverlayLineOp> lines;
    std::vector<OverlayGlyphOp> glyphs;
    std::vector<uint32_t> colors;
};
// Throws ImageError for end points outside the int range and lines longer than 2^24 steps.
OverlayPlan plan_overlay(uint32_t width, uint32_t height, const SrView& view, const SrOverlayLine* lines,
                         uint32_t line_count, const SrOverlayText* texts, uint32_t text_count, const SrFont* font);

// Bytes of the samples image (program.cs:247-256) for counts 0 .. max_samples + 1.
std::vector<uint8_t> samples_table(uint32_t min_samples, uint32_t max_samples, float* log_range);

// Image.Save image.cs:88-212 by extension (.tga / .ppm / .bmp).  Throws ImageError.
void save_image(const std::string& path, uint32_t width, uint32_t height, const uint8_t* rgb8);

}  // namespace host
}  // namespace sr
