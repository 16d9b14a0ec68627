// Minimal OpenEXR writer for linear-radiance frames: one part, scanline
// storage, NO_COMPRESSION, 32-bit FLOAT channels, no external library. Layout
// per the published OpenEXR file format ("The OpenEXR File Layout"): magic
// 20000630, version 2 with no flag bits, the required header attributes
// (channels, compression, dataWindow, displayWindow, lineOrder,
// pixelAspectRatio, screenWindowCenter, screenWindowWidth) each as
// name\0 type\0 int32 size value, a null byte, the line offset table (one
// uint64 file offset per chunk; an uncompressed chunk holds one scanline), then
// per scanline int32 y, int32 byte count and the channels' values in the
// channel list's (alphabetical) order. All numbers little-endian.
#pragma once

#include <cstdint>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace rtgb::exr {

namespace detail {

inline void put_u8(std::vector<uint8_t>& out, uint8_t v) { out.push_back(v); }

inline void put_i32(std::vector<uint8_t>& out, int32_t v) {
    const uint32_t u = static_cast<uint32_t>(v);
    for (int k = 0; k < 4; ++k) out.push_back(static_cast<uint8_t>(u >> (8 * k)));
}

inline void put_u64(std::vector<uint8_t>& out, uint64_t v) {
    for (int k = 0; k < 8; ++k) out.push_back(static_cast<uint8_t>(v >> (8 * k)));
}

inline void put_f32(std::vector<uint8_t>& out, float v) {
    uint32_t u;
    std::memcpy(&u, &v, 4);
    put_i32(out, static_cast<int32_t>(u));
}

inline void put_str(std::vector<uint8_t>& out, const std::string& s) {
    out.insert(out.end(), s.begin(), s.end());
    out.push_back(0);
}

// name\0 type\0 int32 size, then `value` (already encoded)
inline void attribute(std::vector<uint8_t>& out, const char* name, const char* type, const std::vector<uint8_t>& value) {
    put_str(out, name);
    put_str(out, type);
    put_i32(out, static_cast<int32_t>(value.size()));
    out.insert(out.end(), value.begin(), value.end());
}

}  // namespace detail

// Writes `width` x `height` pixels of `channels` interleaved floats (rows top to
// bottom) under the given channel names. Names must be in strictly increasing
// byte order (the order OpenEXR readers expect the channel list in), e.g.
// {"B", "G", "R"} with the interleaved data then in B, G, R order per pixel,
// or use write_rgba below, which reorders for you.
inline std::vector<uint8_t> encode(int width, int height, const std::vector<std::string>& names, const float* pixels) {
    if (width <= 0 || height <= 0) throw std::runtime_error("exr: image size must be positive");
    if (names.empty()) throw std::runtime_error("exr: no channels");
    for (size_t c = 1; c < names.size(); ++c) {
        if (!(names[c - 1] < names[c])) throw std::runtime_error("exr: channel names must be sorted and unique");
    }
    using namespace detail;
    std::vector<uint8_t> out;
    put_i32(out, 20000630);
    put_i32(out, 2);

    std::vector<uint8_t> v;
    for (const std::string& n : names) {
        put_str(v, n);
        put_i32(v, 2);  // pixel type FLOAT
        put_u8(v, 0);   // pLinear
        put_u8(v, 0);
        put_u8(v, 0);
        put_u8(v, 0);   // reserved
        put_i32(v, 1);  // xSampling
        put_i32(v, 1);  // ySampling
    }
    put_u8(v, 0);
    attribute(out, "channels", "chlist", v);
    attribute(out, "compression", "compression", {0});
    v.clear();
    put_i32(v, 0);
    put_i32(v, 0);
    put_i32(v, width - 1);
    put_i32(v, height - 1);
    attribute(out, "dataWindow", "box2i", v);
    attribute(out, "displayWindow", "box2i", v);
    attribute(out, "lineOrder", "lineOrder", {0});  // INCREASING_Y
    v.clear();
    put_f32(v, 1.0f);
    attribute(out, "pixelAspectRatio", "float", v);
    v.clear();
    put_f32(v, 0.0f);
    put_f32(v, 0.0f);
    attribute(out, "screenWindowCenter", "v2f", v);
    v.clear();
    put_f32(v, 1.0f);
    attribute(out, "screenWindowWidth", "float", v);
    put_u8(out, 0);  // end of header

    const size_t nc = names.size();
    const size_t line_bytes = static_cast<size_t>(width) * nc * 4;
    const size_t table_at = out.size();
    const size_t first_chunk = table_at + 8 * static_cast<size_t>(height);
    for (int y = 0; y < height; ++y) put_u64(out, first_chunk + static_cast<size_t>(y) * (8 + line_bytes));
    out.reserve(first_chunk + static_cast<size_t>(height) * (8 + line_bytes));
    for (int y = 0; y < height; ++y) {
        put_i32(out, y);
        put_i32(out, static_cast<int32_t>(line_bytes));
        const float* row = pixels + static_cast<size_t>(y) * width * nc;
        for (size_t c = 0; c < nc; ++c) {
            for (int x = 0; x < width; ++x) put_f32(out, row[static_cast<size_t>(x) * nc + c]);
        }
    }
    return out;
}

inline void write_file(const std::filesystem::path& path, const std::vector<uint8_t>& bytes) {
    std::ofstream f(path, std::ios::binary);
    if (!f.is_open()) throw std::runtime_error("failed to open " + path.string());
    f.write(reinterpret_cast<const char*>(bytes.data()), static_cast<std::streamsize>(bytes.size()));
    if (!f) throw std::runtime_error("failed to write " + path.string());
}

// RGBA floats per pixel (rtgb_download_frame's beauty layout) -> channels A, B,
// G, R, or B, G, R when `alpha` is false.
inline void write_rgba(const std::filesystem::path& path, int width, int height, const float* rgba, bool alpha = false) {
    const size_t px = static_cast<size_t>(width) * height;
    const size_t nc = alpha ? 4 : 3;
    std::vector<float> sorted(px * nc);
    for (size_t i = 0; i < px; ++i) {
        float* d = &sorted[i * nc];
        if (alpha) *d++ = rgba[4 * i + 3];
        d[0] = rgba[4 * i + 2];
        d[1] = rgba[4 * i + 1];
        d[2] = rgba[4 * i];
    }
    const std::vector<std::string> names = alpha ? std::vector<std::string>{"A", "B", "G", "R"}
                                                 : std::vector<std::string>{"B", "G", "R"};
    write_file(path, encode(width, height, names, sorted.data()));
}

}  // namespace rtgb::exr
