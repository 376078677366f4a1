// Image output: the reference's FrameBuffer::output / WriteImage step
// (src/renderer/framebuffer.cpp:11-26, imageio.cpp:59-82) on the host.
//
// PNG: each channel through the sRGB curve of GammaCorrect (spectrum.h:62-72),
// 8 bits as clamp(255 g + 0.5, 0, 255) truncated, rows written bottom-up (the
// reference sets stbi_flip_vertically_on_write). The file is a plain PNG:
// IHDR, one IDAT holding a zlib stream of stored (uncompressed) deflate blocks,
// IEND — any reader decodes it; the CRC-32 and Adler-32 are computed here.
// PFM: linear 32-bit floats, little-endian (scale -1), rows bottom-up as the
// format stores them, so the first framebuffer row is the file's last.
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "render.h"

namespace {

uint32_t crc_table_entry(uint32_t c) {
    for (int k = 0; k < 8; ++k) c = (c & 1u) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
    return c;
}

// CRC-32 (ISO 3309 / ITU-T V.42, the polynomial PNG uses), byte at a time.
struct Crc32 {
    uint32_t table[256];
    Crc32() {
        for (uint32_t n = 0; n < 256; ++n) table[n] = crc_table_entry(n);
    }
    uint32_t update(uint32_t crc, const uint8_t* p, size_t n) const {
        uint32_t c = crc ^ 0xFFFFFFFFu;
        for (size_t i = 0; i < n; ++i) c = table[(c ^ p[i]) & 0xFFu] ^ (c >> 8);
        return c ^ 0xFFFFFFFFu;
    }
};

void put_be32(std::vector<uint8_t>& v, uint32_t x) {
    v.push_back((uint8_t)(x >> 24));
    v.push_back((uint8_t)(x >> 16));
    v.push_back((uint8_t)(x >> 8));
    v.push_back((uint8_t)x);
}

void chunk(std::vector<uint8_t>& png, const Crc32& crc, const char* tag, const std::vector<uint8_t>& data) {
    put_be32(png, (uint32_t)data.size());
    const size_t at = png.size();
    png.insert(png.end(), tag, tag + 4);
    png.insert(png.end(), data.begin(), data.end());
    put_be32(png, crc.update(0, png.data() + at, png.size() - at));
}

// GammaCorrect (spectrum.h:62-72) and the 8-bit rounding of FrameBuffer::output.
uint8_t srgb8(float v) {
    const float g = v <= 0.0031308f ? 12.92f * v : 1.055f * std::pow(v, 1.0f / 2.4f) - 0.055f;
    float x = 255.0f * g + 0.5f;
    if (!(x > 0.0f)) x = 0.0f;  // also a NaN sample
    if (x > 255.0f) x = 255.0f;
    return (uint8_t)x;
}

bool ends_with(const std::string& s, const char* suffix) {
    const size_t n = std::strlen(suffix);
    if (s.size() < n) return false;
    for (size_t i = 0; i < n; ++i)
        if (std::tolower((unsigned char)s[s.size() - n + i]) != suffix[i]) return false;
    return true;
}

bool write_file(const char* path, const std::vector<uint8_t>& bytes) {
    FILE* f = std::fopen(path, "wb");
    if (!f) return false;
    const bool ok = std::fwrite(bytes.data(), 1, bytes.size(), f) == bytes.size();
    return std::fclose(f) == 0 && ok;
}

std::vector<uint8_t> encode_png(const float* rgb, uint32_t w, uint32_t h) {
    static const Crc32 crc;
    // filtered scanlines (filter type 0), bottom row first
    const size_t stride = 1 + 3ull * w;
    std::vector<uint8_t> raw(stride * h);
    for (uint32_t y = 0; y < h; ++y) {
        uint8_t* row = raw.data() + stride * y;
        row[0] = 0;
        const float* src = rgb + 3ull * w * (h - 1 - y);
        for (size_t i = 0; i < 3ull * w; ++i) row[1 + i] = srgb8(src[i]);
    }
    // zlib stream: header, stored deflate blocks of at most 65,535 bytes, Adler-32
    std::vector<uint8_t> z;
    z.reserve(raw.size() + raw.size() / 65535 * 5 + 16);
    z.push_back(0x78);
    z.push_back(0x01);
    size_t pos = 0;
    do {
        const size_t len = std::min<size_t>(65535, raw.size() - pos);
        const bool last = pos + len == raw.size();
        z.push_back(last ? 1 : 0);
        z.push_back((uint8_t)len);
        z.push_back((uint8_t)(len >> 8));
        z.push_back((uint8_t)~len);
        z.push_back((uint8_t)(~len >> 8));
        z.insert(z.end(), raw.begin() + pos, raw.begin() + pos + len);
        pos += len;
    } while (pos < raw.size());
    uint32_t a = 1, b = 0;
    for (uint8_t c : raw) {
        a = (a + c) % 65521u;
        b = (b + a) % 65521u;
    }
    put_be32(z, (b << 16) | a);
    std::vector<uint8_t> png = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1A, '\n'};
    std::vector<uint8_t> ihdr;
    put_be32(ihdr, w);
    put_be32(ihdr, h);
    ihdr.insert(ihdr.end(), {8, 2, 0, 0, 0});  // 8 bits, RGB, deflate, filter set 0, no interlace
    chunk(png, crc, "IHDR", ihdr);
    chunk(png, crc, "IDAT", z);
    chunk(png, crc, "IEND", {});
    return png;
}

std::vector<uint8_t> encode_pfm(const float* rgb, uint32_t w, uint32_t h) {
    const std::string head = "PF\n" + std::to_string(w) + " " + std::to_string(h) + "\n-1.0\n";
    std::vector<uint8_t> out(head.begin(), head.end());
    const size_t body = 12ull * w * h;
    out.resize(head.size() + body);
    // rows bottom-up: the first framebuffer row is written last
    uint8_t* dst = out.data() + head.size();
    for (uint32_t y = 0; y < h; ++y) {
        const float* src = rgb + 3ull * w * (h - 1 - y);
        for (size_t i = 0; i < 3ull * w; ++i) {
            uint32_t bits;
            std::memcpy(&bits, src + i, 4);
            uint8_t* d = dst + 12ull * w * y + 4 * i;
            d[0] = (uint8_t)bits;
            d[1] = (uint8_t)(bits >> 8);
            d[2] = (uint8_t)(bits >> 16);
            d[3] = (uint8_t)(bits >> 24);
        }
    }
    return out;
}

}  // namespace

extern "C" {

gr_status gr_image_write(const char* path, const float* rgb, uint32_t width, uint32_t height) {
    if (!path || !rgb || width == 0 || height == 0 || (uint64_t)width * height > (1ull << 31)) return GR_ERR_INVALID;
    const std::string p(path);
    std::vector<uint8_t> bytes;
    if (ends_with(p, ".png")) bytes = encode_png(rgb, width, height);
    else if (ends_with(p, ".pfm")) bytes = encode_pfm(rgb, width, height);
    else return GR_ERR_INVALID;
    return write_file(path, bytes) ? GR_OK : GR_ERR_IO;
}

gr_status gr_scene_write_image(gr_scene* sc, const char* path) {
    if (!sc || !path) return GR_ERR_INVALID;
    uint32_t w = 0, h = 0, tris = 0, lights = 0;
    gr_status st = gr_scene_info(sc, &w, &h, &tris, &lights);
    if (st != GR_OK) return st;
    const size_t npix = (size_t)w * h;
    std::vector<double> sum(3 * npix);
    std::vector<uint32_t> count(npix);
    if ((st = gr_scene_accumulation(sc, sum.data(), count.data())) != GR_OK) return st;
    // mean radiance, buffer[i] / sample_num[i] (framebuffer.cpp:18); a pixel without samples is black
    std::vector<float> rgb(3 * npix);
    for (size_t i = 0; i < npix; ++i)
        for (int c = 0; c < 3; ++c) rgb[3 * i + c] = count[i] ? (float)(sum[3 * i + c] / count[i]) : 0.0f;
    st = gr_image_write(path, rgb.data(), w, h);
    if (st != GR_OK) sc->ctx->last_error = std::string("gr_scene_write_image: cannot write ") + path;
    return st;
}

}  // extern "C"
