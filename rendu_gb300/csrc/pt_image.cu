// Image output of the path tracer's command-line render (include/rendu_gb300.h,
// pt_image_save): what renderOneShot does after PathTracer::render
// (src/apps/pathtracer/main.cpp:106-119 of kosua20/Rendu): for 8-bit formats the
// exponential tone map 1 - exp(-c), then Image::saveAsLDR (Image.cpp:126-160) -- pow(v,
// 1/2.2) on colour channels, 255 v clamped to [0, 255] and truncated -- written as PNG;
// for ".exr" Image::saveAsHDR (Image.cpp:162-290): half-precision channels, no tone map.
// Host code: the per-pixel arithmetic follows the reference's float operations so that the
// bytes written equal the reference's.
#include <cuda_fp16.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "rt_context.hpp"

namespace {

uint32_t crc_table[256];
bool crc_ready = false;

uint32_t crc32(const uint8_t *p, size_t n, uint32_t c = 0xFFFFFFFFu) {
    if (!crc_ready) {
        for (uint32_t i = 0; i < 256; ++i) {
            uint32_t v = i;
            for (int k = 0; k < 8; ++k) v = (v & 1) ? 0xEDB88320u ^ (v >> 1) : v >> 1;
            crc_table[i] = v;
        }
        crc_ready = true;
    }
    for (size_t i = 0; i < n; ++i) c = crc_table[(c ^ p[i]) & 0xFF] ^ (c >> 8);
    return c;
}

void put_be32(std::vector<uint8_t> &o, uint32_t v) {
    for (int s = 24; s >= 0; s -= 8) o.push_back((uint8_t)(v >> s));
}

void png_chunk(std::vector<uint8_t> &o, const char *type, const std::vector<uint8_t> &data) {
    put_be32(o, (uint32_t)data.size());
    const size_t start = o.size();
    o.insert(o.end(), type, type + 4);
    o.insert(o.end(), data.begin(), data.end());
    put_be32(o, crc32(o.data() + start, o.size() - start) ^ 0xFFFFFFFFu);
}

// PNG (RGB or RGBA, 8 bits, no filter) with the image data in stored (uncompressed)
// deflate blocks.
std::vector<uint8_t> encode_png(const uint8_t *px, uint32_t w, uint32_t h, uint32_t ch) {
    std::vector<uint8_t> raw;
    raw.reserve((size_t)h * (1 + (size_t)w * ch));
    for (uint32_t y = 0; y < h; ++y) {
        raw.push_back(0);
        raw.insert(raw.end(), px + (size_t)y * w * ch, px + (size_t)(y + 1) * w * ch);
    }
    std::vector<uint8_t> z{0x78, 0x01};
    uint32_t a = 1, b = 0;  // Adler-32
    for (uint8_t v : raw) {
        a = (a + v) % 65521u;
        b = (b + a) % 65521u;
    }
    for (size_t off = 0; off < raw.size() || off == 0; off += 65535) {
        const size_t len = std::min<size_t>(65535, raw.size() - off);
        const bool last = off + len >= raw.size();
        z.push_back(last ? 1 : 0);
        z.push_back((uint8_t)(len & 0xFF));
        z.push_back((uint8_t)(len >> 8));
        z.push_back((uint8_t)(~len & 0xFF));
        z.push_back((uint8_t)((~len >> 8) & 0xFF));
        z.insert(z.end(), raw.begin() + off, raw.begin() + off + len);
        if (raw.empty()) break;
    }
    put_be32(z, (b << 16) | a);
    std::vector<uint8_t> o{0x89, 'P', 'N', 'G', '\r', '\n', 0x1A, '\n'};
    std::vector<uint8_t> ihdr;
    put_be32(ihdr, w);
    put_be32(ihdr, h);
    ihdr.push_back(8);
    ihdr.push_back(ch == 4 ? 6 : 2);
    ihdr.push_back(0);
    ihdr.push_back(0);
    ihdr.push_back(0);
    png_chunk(o, "IHDR", ihdr);
    png_chunk(o, "IDAT", z);
    png_chunk(o, "IEND", {});
    return o;
}

void put_le32(std::vector<uint8_t> &o, uint32_t v) {
    for (int s = 0; s < 32; s += 8) o.push_back((uint8_t)(v >> s));
}
void put_le64(std::vector<uint8_t> &o, uint64_t v) {
    for (int s = 0; s < 64; s += 8) o.push_back((uint8_t)(v >> s));
}
void put_str(std::vector<uint8_t> &o, const char *s) { o.insert(o.end(), s, s + std::strlen(s) + 1); }
void exr_attr(std::vector<uint8_t> &o, const char *name, const char *type, const std::vector<uint8_t> &v) {
    put_str(o, name);
    put_str(o, type);
    put_le32(o, (uint32_t)v.size());
    o.insert(o.end(), v.begin(), v.end());
}

// OpenEXR, single part, scanlines without compression, half channels: B, G, R (and A for
// 4-component images), stored in the alphabetical order the format requires.
std::vector<uint8_t> encode_exr(const float *px, uint32_t w, uint32_t h, uint32_t comps, bool ignore_alpha) {
    const int nch = comps == 4 ? 4 : (comps == 1 ? 1 : 3);
    // channel names in file order and the source component of each
    const char *names4[4] = {"A", "B", "G", "R"};
    const int src4[4] = {3, 2, 1, 0};
    const char *names3[3] = {"B", "G", "R"};
    const int src3[3] = {2, 1, 0};
    const char *names1[1] = {"A"};
    const int src1[1] = {0};
    const char **names = nch == 4 ? names4 : (nch == 3 ? names3 : names1);
    const int *src = nch == 4 ? src4 : (nch == 3 ? src3 : src1);
    std::vector<uint8_t> o{0x76, 0x2F, 0x31, 0x01, 2, 0, 0, 0};  // magic, version 2, scanline
    std::vector<uint8_t> chl;
    for (int c = 0; c < nch; ++c) {
        put_str(chl, names[c]);
        put_le32(chl, 1);  // HALF
        chl.insert(chl.end(), {0, 0, 0, 0});  // pLinear, reserved
        put_le32(chl, 1);
        put_le32(chl, 1);  // x/y sampling
    }
    chl.push_back(0);
    exr_attr(o, "channels", "chlist", chl);
    exr_attr(o, "compression", "compression", {0});
    std::vector<uint8_t> box;
    put_le32(box, 0);
    put_le32(box, 0);
    put_le32(box, w - 1);
    put_le32(box, h - 1);
    exr_attr(o, "dataWindow", "box2i", box);
    exr_attr(o, "displayWindow", "box2i", box);
    exr_attr(o, "lineOrder", "lineOrder", {0});
    std::vector<uint8_t> one;
    float f1 = 1.0f, f0 = 0.0f;
    uint32_t u1, u0;
    std::memcpy(&u1, &f1, 4);
    std::memcpy(&u0, &f0, 4);
    put_le32(one, u1);
    exr_attr(o, "pixelAspectRatio", "float", one);
    std::vector<uint8_t> v2;
    put_le32(v2, u0);
    put_le32(v2, u0);
    exr_attr(o, "screenWindowCenter", "v2f", v2);
    exr_attr(o, "screenWindowWidth", "float", one);
    o.push_back(0);  // end of header
    const size_t line_bytes = (size_t)w * nch * 2;
    const size_t table = o.size();
    for (uint32_t y = 0; y < h; ++y) put_le64(o, table + (size_t)h * 8 + (size_t)y * (8 + line_bytes));
    for (uint32_t y = 0; y < h; ++y) {
        put_le32(o, y);
        put_le32(o, (uint32_t)line_bytes);
        for (int c = 0; c < nch; ++c)
            for (uint32_t x = 0; x < w; ++x) {
                const size_t p = (size_t)y * w + x;
                float v;
                if (src[c] == 3) v = ignore_alpha ? 1.0f : px[p * comps + 3];
                else v = src[c] < (int)comps ? px[p * comps + src[c]] : 0.0f;
                const __half hv = __float2half_rn(v);
                uint16_t bits;
                std::memcpy(&bits, &hv, 2);
                o.push_back((uint8_t)(bits & 0xFF));
                o.push_back((uint8_t)(bits >> 8));
            }
    }
    return o;
}

bool ends_with(const std::string &s, const std::string &suf) {
    return s.size() >= suf.size() && s.compare(s.size() - suf.size(), suf.size(), suf) == 0;
}

}  // namespace

extern "C" {

int pt_image_save(const float *image, uint32_t width, uint32_t height, uint32_t components, const char *path,
                  int32_t tonemap) {
    rgb::clear_error();
    if (!image || !path) {
        rgb::set_error("null argument");
        return RT_ERR_ARG;
    }
    if (width == 0 || height == 0 || components == 0 || components > 4 || (uint64_t)width * height >= (1ull << 31)) {
        rgb::set_error("invalid image size");
        return RT_ERR_ARG;
    }
    const std::string p(path);
    const size_t npix = (size_t)width * height;
    std::vector<uint8_t> bytes;
    if (ends_with(p, ".exr")) {
        // Image::saveAsHDR refuses images under 16 x 16 (Image.cpp:165-168).
        if (width < 16 || height < 16) {
            rgb::set_error("EXR output needs at least 16 x 16 pixels");
            return RT_ERR_ARG;
        }
        bytes = encode_exr(image, width, height, components, true);
    } else {
        if (components < 3) {
            rgb::set_error("8-bit output needs an RGB or RGBA image");
            return RT_ERR_ARG;
        }
        // main.cpp:109-116 (colour only, in place) then Image::saveAsLDR with SRGB_LDR and
        // IGNORE_ALPHA: every channel but alpha gamma-corrected, alpha written as 255.
        const uint32_t ch = components == 4 ? 4 : 3;
        std::vector<uint8_t> ldr(npix * ch);
        for (size_t i = 0; i < npix; ++i)
            for (uint32_t c = 0; c < ch; ++c) {
                float v = c < components ? image[i * components + c] : 0.0f;
                if (c == 3) {
                    ldr[i * ch + c] = 255;
                    continue;
                }
                if (tonemap) v = 1.0f - std::exp(-v * 1.0f);
                v = std::pow(v, 1.0f / 2.2f);
                const float s = 255.0f * v;
                const float m = (0.0f < s) ? s : 0.0f;       // std::max(0.0f, s)
                const float q = (m < 255.0f) ? m : 255.0f;    // std::min(255.0f, m)
                ldr[i * ch + c] = static_cast<unsigned char>(q);
            }
        bytes = encode_png(ldr.data(), width, height, ch);
    }
    FILE *f = std::fopen(path, "wb");
    if (!f) {
        rgb::set_error("cannot open " + p + " for writing");
        return RT_ERR_ARG;
    }
    const size_t wrote = std::fwrite(bytes.data(), 1, bytes.size(), f);
    const bool ok = std::fclose(f) == 0 && wrote == bytes.size();
    if (!ok) {
        rgb::set_error("writing " + p + " failed");
        return RT_ERR_ARG;
    }
    return RT_OK;
}

// PNG filters (None, Sub, Up, Average, Paeth), each byte predicted from the byte one pixel
// to the left (a), the byte above (b) and the byte above-left (c); the first row sees a zero
// row above it.
int pt_png_unfilter(const uint8_t *filtered, uint32_t rows, uint32_t row_bytes, uint32_t pixel_bytes, uint8_t *out) {
    rgb::clear_error();
    if ((!filtered || !out) && rows && row_bytes) {
        rgb::set_error("null argument");
        return RT_ERR_ARG;
    }
    if (pixel_bytes == 0 || pixel_bytes > 8) {
        rgb::set_error("pixel_bytes must be 1..8");
        return RT_ERR_ARG;
    }
    const size_t fb = pixel_bytes;
    for (uint32_t y = 0; y < rows; ++y) {
        const uint8_t *in = filtered + (size_t)y * (row_bytes + 1);
        const uint8_t type = in[0];
        ++in;
        uint8_t *cur = out + (size_t)y * row_bytes;
        const uint8_t *up = y ? cur - row_bytes : nullptr;
        if (type > 4) {
            rgb::set_error("PNG filter type " + std::to_string(type) + " is invalid");
            return RT_ERR_ARG;
        }
        for (size_t x = 0; x < row_bytes; ++x) {
            const int a = x >= fb ? cur[x - fb] : 0;
            const int b = up ? up[x] : 0;
            const int c = (up && x >= fb) ? up[x - fb] : 0;
            int pred = 0;
            switch (type) {
            case 1: pred = a; break;
            case 2: pred = b; break;
            case 3: pred = (a + b) >> 1; break;
            case 4: {
                const int p = a + b - c;
                const int pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
                pred = (pa <= pb && pa <= pc) ? a : (pb <= pc ? b : c);
                break;
            }
            default: break;
            }
            cur[x] = (uint8_t)(in[x] + pred);
        }
    }
    return RT_OK;
}

}  // extern "C"
