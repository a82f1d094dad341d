// sr_ingest.h — asset ingest (sr_ingest.cpp): OBJ + MTL, TGA and Radiance HDR files.
#pragma once

#include <cstdint>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/sharpray.h"

namespace sr {
namespace host {

// A malformed or unsupported file; the message is the reference's exception text where it has one.
struct IngestError : std::runtime_error {
    explicit IngestError(const std::string& m) : std::runtime_error(m) {}
};

// A texture map of an MTL material, decoded when the MTL is parsed (as the reference does: a broken
// map fails the load even when no object uses its material).
struct ObjImage {
    std::string path;
    uint32_t width = 0, height = 0;
    std::vector<float> texels;  // RGB, rows top-down
};
using ObjImagePtr = std::shared_ptr<const ObjImage>;

// One `newmtl` of an MTL file with the reference's defaults (ParseMtl obj.cs:261-401).
struct ObjMaterial {
    float albedo[3] = {1.0f, 1.0f, 1.0f};
    float roughness = 1.0f;  // final value: Pr, or sqrt(2 / (Ns + 2)), clamped to [0, 1]
    float metallic = 0.0f;
    float transparency = 0.0f;
    float ior = 1.5f;
    float radiance[3] = {0.0f, 0.0f, 0.0f};
    ObjImagePtr color_map, roughness_map, metallic_map, normal_map;  // sRGB / linear / linear / linear
};

// One object of an OBJ file (BuildObject obj.cs:171-189), its triangles already smoothed when the
// loader smooths them, and the material its `usemtl` named as defined when the object ended.
struct ObjObject {
    std::string name;
    std::vector<SrTriangle> triangles;
    bool has_material = false;  // false: the caller's default material
    std::string material_name;
    ObjMaterial material;
};

struct ObjResult {
    std::vector<ObjObject> objects;
    std::map<std::string, ObjMaterial> materials;
};

// ObjLoader.Load(path, ..., SmoothNormals) without the scene side effects.  Throws IngestError.
ObjResult parse_obj(const std::string& path, bool smooth_normals);
// Image.Load (.tga only, as the reference) -> RGB8 rows top-down.  Throws IngestError.
void load_image(const std::string& path, uint32_t& width, uint32_t& height, std::vector<uint8_t>& rgb);
void load_tga(const std::string& path, uint32_t& width, uint32_t& height, std::vector<uint8_t>& rgb);
// ImageHdr.Load -> RGBE8 rows top-down.  Throws IngestError.
void load_hdr(const std::string& path, uint32_t& width, uint32_t& height, std::vector<uint8_t>& rgbe);
// Texture.FromSrgb / FromLinear / FromHdr texel conversions (3 floats per texel).
void rgb8_to_texels(const uint8_t* rgb, size_t n, bool srgb, float* out);
void rgbe_to_texels(const uint8_t* rgbe, size_t n, float max_luminance, float* out);

}  // namespace host
}  // namespace sr
