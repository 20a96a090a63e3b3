// JPEG decoding for scene textures (include/rendu_gb300.h, pt_jpeg_decode): the part of
// Image::loadLDR (src/engine/resources/Image.cpp:291-333 of kosua20/Rendu, through
// stb_image) that reads .jpg / .jpeg files. Host code.
//
// ITU-T T.81 Huffman-coded JPEG, sequential (SOF0, SOF1) and progressive (SOF2: spectral
// selection and successive approximation), 1 or 3 components, any sampling factors, restart
// intervals. Coefficients are gathered for the whole image first, then each 8x8 block is
// dequantised and inverse-transformed (separable float DCT-III, +128, rounded, clamped).
// Subsampled chroma is upsampled with the triangle ("fancy") filter for factors of 2 and
// replicated otherwise; YCbCr goes to RGB with the JFIF equations (an Adobe marker with
// transform 0 means the 3 components are RGB already). The requested channel count
// expands grey to RGB, adds alpha 255, or takes luminance (77 R + 150 G + 29 B) >> 8.
//
// Malformed input returns RT_ERR_ARG with a message; no read or write goes out of bounds.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "rt_context.hpp"

namespace {

const uint8_t kZigzag[64] = {0,  1,  8,  16, 9,  2,  3,  10, 17, 24, 32, 25, 18, 11, 4,  5,  12, 19, 26, 33, 40, 48,
                             41, 34, 27, 20, 13, 6,  7,  14, 21, 28, 35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23,
                             30, 37, 44, 51, 58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63};

struct JpegError {
    std::string msg;
};

[[noreturn]] void fail(const std::string &m) { throw JpegError{m}; }

struct Huffman {
    // canonical code -> value: for each length the first code, count and offset into vals
    int mincode[17], maxcode[18], valptr[17];
    uint8_t vals[256];
    uint8_t fast_len[512], fast_val[512];  // 9-bit lookup, len 0 = not resolved
    bool defined = false;
};

struct Component {
    int id, h, v, tq;
    int bw, bh;          // blocks per line / column, padded to whole MCUs
    int cw, ch;          // blocks covering the component's own size (non-interleaved scans)
    int dc_table, ac_table;
    int dc_pred;
    std::vector<int16_t> coef;  // bw * bh * 64, natural order
    std::vector<uint8_t> pixels;  // bw * 8 x bh * 8
};

struct Decoder {
    const uint8_t *p;
    size_t n, pos = 0;
    uint16_t qt[4][64];
    bool qt_defined[4] = {false, false, false, false};
    Huffman dc[4], ac[4];
    std::vector<Component> comp;
    int width = 0, height = 0, hmax = 1, vmax = 1, mcux = 0, mcuy = 0;
    bool progressive = false, frame = false, adobe = false;
    int adobe_transform = -1;
    bool jfif = false;
    int restart_interval = 0;
    // bit reader
    uint32_t bitbuf = 0;
    int bitcnt = 0;
    bool hit_marker = false;
    int eobrun = 0;

    uint8_t byte() {
        if (pos >= n) fail("unexpected end of data");
        return p[pos++];
    }
    int u16() {
        const int a = byte();
        return (a << 8) | byte();
    }

    // ---- entropy-coded segment bit reader (0xFF00 stuffing; a marker stops the stream,
    // after which zeros are read as the standard allows) ----
    void fill() {
        while (bitcnt <= 24) {
            uint32_t b = 0;
            if (!hit_marker && pos < n) {
                b = p[pos];
                if (b == 0xFF) {
                    const uint8_t nx = pos + 1 < n ? p[pos + 1] : 0;
                    if (nx == 0x00) {
                        pos += 2;
                    } else {
                        hit_marker = true;
                        b = 0;
                    }
                } else {
                    ++pos;
                }
            }
            bitbuf |= b << (24 - bitcnt);
            bitcnt += 8;
        }
    }
    int bits(int k) {
        if (k == 0) return 0;
        fill();
        const int v = (int)(bitbuf >> (32 - k));
        bitbuf <<= k;
        bitcnt -= k;
        return v;
    }
    int bit() { return bits(1); }
    static int extend(int v, int s) { return v < (1 << (s - 1)) ? v - (1 << s) + 1 : v; }
    int receive_extend(int s) {
        if (s == 0) return 0;
        if (s > 16) fail("bad coefficient size");
        return extend(bits(s), s);
    }
    int decode(const Huffman &h) {
        if (!h.defined) fail("undefined Huffman table");
        fill();
        const uint32_t top9 = bitbuf >> 23;
        if (h.fast_len[top9]) {
            const int l = h.fast_len[top9];
            bitbuf <<= l;
            bitcnt -= l;
            return h.fast_val[top9];
        }
        int code = 0;
        for (int l = 1; l <= 16; ++l) {
            code = (code << 1) | bit();
            if (h.maxcode[l] >= 0 && code <= h.maxcode[l] && code >= h.mincode[l]) {
                const int idx = h.valptr[l] + code - h.mincode[l];
                if (idx < 0 || idx > 255) fail("bad Huffman code");
                return h.vals[idx];
            }
        }
        fail("bad Huffman code");
    }
    void reset_bits() {
        bitbuf = 0;
        bitcnt = 0;
        hit_marker = false;
    }

    // ---- marker segments ----
    void read_dqt(int len) {
        const size_t end = pos + len;
        while (pos < end) {
            const int pq_tq = byte();
            const int pq = pq_tq >> 4, tq = pq_tq & 15;
            if (tq > 3 || pq > 1) fail("bad quantisation table");
            for (int k = 0; k < 64; ++k) qt[tq][kZigzag[k]] = (uint16_t)(pq ? u16() : byte());
            qt_defined[tq] = true;
        }
        if (pos != end) fail("bad DQT length");
    }
    void read_dht(int len) {
        const size_t end = pos + len;
        while (pos < end) {
            const int tc_th = byte();
            const int tc = tc_th >> 4, th = tc_th & 15;
            if (tc > 1 || th > 3) fail("bad Huffman table");
            Huffman &h = tc ? ac[th] : dc[th];
            int counts[17] = {0}, total = 0;
            for (int l = 1; l <= 16; ++l) total += counts[l] = byte();
            if (total > 256) fail("bad Huffman table");
            for (int k = 0; k < total; ++k) h.vals[k] = byte();
            int code = 0, k = 0;
            std::memset(h.fast_len, 0, sizeof(h.fast_len));
            for (int l = 1; l <= 16; ++l) {
                h.valptr[l] = k;
                h.mincode[l] = code;
                h.maxcode[l] = counts[l] ? code + counts[l] - 1 : -1;
                for (int c = 0; c < counts[l]; ++c, ++code, ++k) {
                    if (l <= 9) {
                        const int shift = 9 - l;
                        for (int f = 0; f < (1 << shift); ++f) {
                            const int idx = (code << shift) | f;
                            if (idx < 512) {
                                h.fast_len[idx] = (uint8_t)l;
                                h.fast_val[idx] = h.vals[k];
                            }
                        }
                    }
                }
                if (code > (1 << l)) fail("bad Huffman code lengths");
                code <<= 1;
            }
            h.maxcode[17] = -1;
            h.defined = true;
        }
        if (pos != end) fail("bad DHT length");
    }
    void read_sof(int len, int marker) {
        if (frame) fail("more than one frame");
        frame = true;
        progressive = marker == 0xC2;
        const int precision = byte();
        if (precision != 8) fail("only 8-bit JPEG is supported");
        height = u16();
        width = u16();
        const int nc = byte();
        if (width <= 0 || height <= 0) fail("JPEG without a size (DNL) is not supported");
        if ((int64_t)width * height > (1ll << 28)) fail("JPEG too large");
        if (nc != 1 && nc != 3) fail("only 1- and 3-component JPEG is supported");
        if (len != 6 + 3 * nc) fail("bad SOF length");
        comp.resize(nc);
        for (auto &c : comp) {
            c.id = byte();
            const int hv = byte();
            c.h = hv >> 4;
            c.v = hv & 15;
            c.tq = byte();
            if (c.h < 1 || c.h > 4 || c.v < 1 || c.v > 4 || c.tq > 3) fail("bad component");
            hmax = std::max(hmax, c.h);
            vmax = std::max(vmax, c.v);
        }
        mcux = (width + 8 * hmax - 1) / (8 * hmax);
        mcuy = (height + 8 * vmax - 1) / (8 * vmax);
        for (auto &c : comp) {
            c.bw = mcux * c.h;
            c.bh = mcuy * c.v;
            c.cw = ((width * c.h + hmax - 1) / hmax + 7) / 8;
            c.ch = ((height * c.v + vmax - 1) / vmax + 7) / 8;
            c.coef.assign((size_t)c.bw * c.bh * 64, 0);
        }
    }

    // ---- scans ----
    void decode_block_baseline(Component &c, int16_t *blk) {
        const int t = decode(dc[c.dc_table]);
        const int diff = receive_extend(t);
        c.dc_pred += diff;
        blk[0] = (int16_t)c.dc_pred;
        for (int k = 1; k < 64;) {
            const int rs = decode(ac[c.ac_table]);
            const int r = rs >> 4, s = rs & 15;
            if (s == 0) {
                if (r != 15) break;
                k += 16;
                continue;
            }
            k += r;
            if (k > 63) fail("AC coefficient index out of range");
            blk[kZigzag[k]] = (int16_t)receive_extend(s);
            ++k;
        }
    }
    void decode_dc_first(Component &c, int16_t *blk, int al) {
        const int t = decode(dc[c.dc_table]);
        c.dc_pred += receive_extend(t);
        blk[0] = (int16_t)(c.dc_pred * (1 << al));
    }
    void decode_dc_refine(int16_t *blk, int al) {
        if (bit()) blk[0] = (int16_t)(blk[0] | (1 << al));
    }
    void decode_ac_first(Component &c, int16_t *blk, int ss, int se, int al) {
        if (eobrun > 0) {
            --eobrun;
            return;
        }
        for (int k = ss; k <= se;) {
            const int rs = decode(ac[c.ac_table]);
            const int r = rs >> 4, s = rs & 15;
            if (s == 0) {
                if (r < 15) {
                    eobrun = (1 << r) - 1;
                    if (r) eobrun += bits(r);
                    break;
                }
                k += 16;
                continue;
            }
            k += r;
            if (k > 63) fail("AC coefficient index out of range");
            blk[kZigzag[k]] = (int16_t)(receive_extend(s) * (1 << al));
            ++k;
        }
    }
    void decode_ac_refine(Component &c, int16_t *blk, int ss, int se, int al) {
        const int p1 = 1 << al, m1 = -1 * (1 << al);
        int k = ss;
        if (eobrun <= 0) {
            for (; k <= se;) {
                const int rs = decode(ac[c.ac_table]);
                int r = rs >> 4;
                const int s = rs & 15;
                int value = 0;
                if (s == 0) {
                    if (r < 15) {
                        eobrun = 1 << r;
                        if (r) eobrun += bits(r);
                        break;  // the rest of the band is refined under the EOB run below
                    }
                    // ZRL: skip 16 zero coefficients (refining the nonzero ones met)
                } else {
                    if (s != 1) fail("bad refinement coefficient size");
                    value = bit() ? p1 : m1;
                }
                for (; k <= se; ++k) {
                    int16_t &co = blk[kZigzag[k]];
                    if (co != 0) {
                        if (bit() && (co & p1) == 0) co = (int16_t)(co >= 0 ? co + p1 : co + m1);
                    } else {
                        if (r == 0) {
                            if (value) co = (int16_t)value;
                            ++k;
                            break;
                        }
                        --r;
                    }
                }
            }
        }
        if (eobrun > 0) {
            for (; k <= se; ++k) {
                int16_t &co = blk[kZigzag[k]];
                if (co != 0 && bit() && (co & p1) == 0) co = (int16_t)(co >= 0 ? co + p1 : co + m1);
            }
            --eobrun;
        }
    }

    void read_restart() {
        // align to the marker, which must be RSTn
        reset_bits();
        while (pos + 1 < n && !(p[pos] == 0xFF && p[pos + 1] >= 0xD0 && p[pos + 1] <= 0xD7)) {
            if (p[pos] == 0xFF && p[pos + 1] != 0x00 && p[pos + 1] != 0xFF) break;
            ++pos;
        }
        if (pos + 1 < n && p[pos] == 0xFF && p[pos + 1] >= 0xD0 && p[pos + 1] <= 0xD7) pos += 2;
        for (auto &c : comp) c.dc_pred = 0;
        eobrun = 0;
    }

    void read_sos(int len) {
        if (!frame) fail("scan before frame");
        const int ns = byte();
        if (ns < 1 || ns > 4 || len != 4 + 2 * ns) fail("bad SOS");
        std::vector<Component *> sc;
        for (int k = 0; k < ns; ++k) {
            const int id = byte(), tables = byte();
            Component *found = nullptr;
            for (auto &c : comp)
                if (c.id == id) found = &c;
            if (!found) fail("scan names an unknown component");
            found->dc_table = tables >> 4;
            found->ac_table = tables & 15;
            if (found->dc_table > 3 || found->ac_table > 3) fail("bad table selector");
            sc.push_back(found);
        }
        const int ss = byte(), se = byte(), a = byte();
        const int ah = a >> 4, al = a & 15;
        if (progressive) {
            if (ss > se || se > 63 || (ss == 0 && se != 0) || (ss > 0 && ns != 1) || al > 13) fail("bad progressive scan");
        } else if (ss != 0 || se != 63 || a != 0) {
            fail("bad sequential scan");
        }
        for (auto *c : sc) c->dc_pred = 0;
        eobrun = 0;
        reset_bits();
        auto block = [&](Component &c, int bx, int by) {
            int16_t *blk = &c.coef[((size_t)by * c.bw + bx) * 64];
            if (!progressive) {
                decode_block_baseline(c, blk);
            } else if (ss == 0) {
                if (ah == 0) decode_dc_first(c, blk, al);
                else decode_dc_refine(blk, al);
            } else if (ah == 0) {
                decode_ac_first(c, blk, ss, se, al);
            } else {
                decode_ac_refine(c, blk, ss, se, al);
            }
        };
        int todo = restart_interval;
        if (ns == 1) {
            Component &c = *sc[0];
            for (int by = 0; by < c.ch; ++by)
                for (int bx = 0; bx < c.cw; ++bx) {
                    block(c, bx, by);
                    if (restart_interval && --todo == 0 && !(by == c.ch - 1 && bx == c.cw - 1)) {
                        read_restart();
                        todo = restart_interval;
                    }
                }
        } else {
            for (int my = 0; my < mcuy; ++my)
                for (int mx = 0; mx < mcux; ++mx) {
                    for (auto *c : sc)
                        for (int v = 0; v < c->v; ++v)
                            for (int h = 0; h < c->h; ++h) block(*c, mx * c->h + h, my * c->v + v);
                    if (restart_interval && --todo == 0 && !(my == mcuy - 1 && mx == mcux - 1)) {
                        read_restart();
                        todo = restart_interval;
                    }
                }
        }
        // skip to the next marker
        reset_bits();
        while (pos + 1 < n && !(p[pos] == 0xFF && p[pos + 1] != 0x00 && !(p[pos + 1] >= 0xD0 && p[pos + 1] <= 0xD7)))
            ++pos;
    }

    // headers_only: stop at the frame header (size query)
    void parse(bool headers_only) {
        if (n < 4 || p[0] != 0xFF || p[1] != 0xD8) fail("not a JPEG file");
        pos = 2;
        for (;;) {
            // find the next marker
            while (pos < n && p[pos] != 0xFF) ++pos;
            while (pos < n && p[pos] == 0xFF) ++pos;
            if (pos >= n) fail("missing end of image");
            const int m = p[pos++];
            if (m == 0xD9) break;  // EOI
            if (m >= 0xD0 && m <= 0xD7) continue;
            const int len = u16() - 2;
            if (len < 0 || pos + (size_t)len > n) fail("bad marker length");
            const size_t next = pos + len;
            if (m == 0xDB) {
                read_dqt(len);
            } else if (m == 0xC4) {
                read_dht(len);
            } else if (m == 0xC0 || m == 0xC1 || m == 0xC2) {
                read_sof(len, m);
                if (headers_only) return;
            } else if (m == 0xDD) {
                if (len != 2) fail("bad DRI");
                restart_interval = u16();
            } else if (m == 0xDA) {
                read_sos(len);
                continue;
            } else if ((m >= 0xC3 && m <= 0xCF) && m != 0xC4 && m != 0xC8 && m != 0xCC) {
                fail("unsupported JPEG process (lossless, hierarchical or arithmetic coding)");
            } else if (m == 0xEE && len >= 12 && std::memcmp(p + pos, "Adobe", 5) == 0) {
                adobe = true;
                adobe_transform = p[pos + 11];
            } else if (m == 0xE0 && len >= 5 && std::memcmp(p + pos, "JFIF", 5) == 0) {
                jfif = true;
            }
            pos = next;
        }
        if (!frame) fail("JPEG without a frame");
    }

    // ---- reconstruction ----
    void idct_all() {
        // DCT-III basis: c(u) cos((2x + 1) u pi / 16)
        float basis[8][8];
        for (int x = 0; x < 8; ++x)
            for (int u = 0; u < 8; ++u)
                basis[x][u] = (float)((u == 0 ? std::sqrt(0.125) : 0.5) * std::cos((2 * x + 1) * u * M_PI / 16.0));
        for (auto &c : comp) {
            if (!qt_defined[c.tq]) fail("undefined quantisation table");
            const uint16_t *q = qt[c.tq];
            const int pw = c.bw * 8;
            c.pixels.assign((size_t)pw * c.bh * 8, 0);
            for (int by = 0; by < c.bh; ++by)
                for (int bx = 0; bx < c.bw; ++bx) {
                    const int16_t *blk = &c.coef[((size_t)by * c.bw + bx) * 64];
                    float f[64], tmp[64];
                    for (int k = 0; k < 64; ++k) f[k] = (float)blk[k] * (float)q[k];
                    for (int y = 0; y < 8; ++y)  // columns: tmp[y][u] = sum_v basis[y][v] f[v][u]
                        for (int u = 0; u < 8; ++u) {
                            float s = 0.0f;
                            for (int v = 0; v < 8; ++v) s += basis[y][v] * f[v * 8 + u];
                            tmp[y * 8 + u] = s;
                        }
                    for (int y = 0; y < 8; ++y)
                        for (int x = 0; x < 8; ++x) {
                            float s = 0.0f;
                            for (int u = 0; u < 8; ++u) s += basis[x][u] * tmp[y * 8 + u];
                            const float v = std::nearbyint(s + 128.0f);
                            c.pixels[(size_t)(by * 8 + y) * pw + bx * 8 + x] =
                                (uint8_t)(v < 0.0f ? 0.0f : (v > 255.0f ? 255.0f : v));
                        }
                }
        }
    }

    // sample of component c at full-resolution pixel (x, y)
    void upsample(const Component &c, std::vector<uint8_t> &out) const {
        const int pw = c.bw * 8;
        const int sw = (width * c.h + hmax - 1) / hmax, sh = (height * c.v + vmax - 1) / vmax;
        const int fx = hmax / c.h, fy = vmax / c.v;
        out.resize((size_t)width * height);
        const bool fancy = hmax % c.h == 0 && vmax % c.v == 0 && fx <= 2 && fy <= 2 && (fx == 2 || fy == 2);
        auto at = [&](int x, int y) -> int {
            x = x < 0 ? 0 : (x >= sw ? sw - 1 : x);
            y = y < 0 ? 0 : (y >= sh ? sh - 1 : y);
            return c.pixels[(size_t)y * pw + x];
        };
        for (int y = 0; y < height; ++y)
            for (int x = 0; x < width; ++x) {
                int v;
                if (fx == 1 && fy == 1) {
                    v = c.pixels[(size_t)y * pw + x];
                } else if (fancy) {
                    // triangle filter: 3/4 nearer sample, 1/4 farther, in each upsampled axis
                    const int sx = x / fx, sy = y / fy;
                    const int nx = fx == 2 ? (x & 1 ? sx + 1 : sx - 1) : sx;
                    const int ny = fy == 2 ? (y & 1 ? sy + 1 : sy - 1) : sy;
                    if (fx == 2 && fy == 2) {
                        const int near_col = 3 * at(sx, sy) + at(sx, ny);
                        const int far_col = 3 * at(nx, sy) + at(nx, ny);
                        v = (3 * near_col + far_col + 8) >> 4;
                    } else if (fx == 2) {
                        v = (3 * at(sx, sy) + at(nx, sy) + 2) >> 2;
                    } else {
                        v = (3 * at(sx, sy) + at(sx, ny) + 2) >> 2;
                    }
                } else {
                    v = at(x * c.h / hmax, y * c.v / vmax);
                }
                out[(size_t)y * width + x] = (uint8_t)v;
            }
    }

    void output(uint32_t channels, uint8_t *dst) {
        std::vector<uint8_t> planes[3];
        for (size_t k = 0; k < comp.size(); ++k) upsample(comp[k], planes[k]);
        // components already RGB: named 'R', 'G', 'B', or an Adobe marker with transform 0
        // in a file without a JFIF marker
        const bool rgb_direct = comp.size() == 3 && ((comp[0].id == 'R' && comp[1].id == 'G' && comp[2].id == 'B') ||
                                                     (adobe && adobe_transform == 0 && !jfif));
        const size_t np = (size_t)width * height;
        for (size_t i = 0; i < np; ++i) {
            int r, g, b;
            if (comp.size() == 1) {
                r = g = b = planes[0][i];
            } else if (rgb_direct) {
                r = planes[0][i];
                g = planes[1][i];
                b = planes[2][i];
            } else {
                const float Y = planes[0][i], cb = planes[1][i] - 128.0f, cr = planes[2][i] - 128.0f;
                const float fr = std::nearbyint(Y + 1.402f * cr);
                const float fg = std::nearbyint(Y - 0.344136f * cb - 0.714136f * cr);
                const float fb = std::nearbyint(Y + 1.772f * cb);
                r = fr < 0 ? 0 : (fr > 255 ? 255 : (int)fr);
                g = fg < 0 ? 0 : (fg > 255 ? 255 : (int)fg);
                b = fb < 0 ? 0 : (fb > 255 ? 255 : (int)fb);
            }
            uint8_t *o = dst + i * channels;
            if (channels == 1 || channels == 2) {
                o[0] = comp.size() == 1 ? (uint8_t)r : (uint8_t)((r * 77 + g * 150 + b * 29) >> 8);
                if (channels == 2) o[1] = 255;
            } else {
                o[0] = (uint8_t)r;
                o[1] = (uint8_t)g;
                o[2] = (uint8_t)b;
                if (channels == 4) o[3] = 255;
            }
        }
    }
};

}  // namespace

extern "C" {

int pt_jpeg_decode(const uint8_t *data, size_t size, uint32_t channels, uint8_t *out, size_t out_capacity,
                   uint32_t *width, uint32_t *height) {
    rgb::clear_error();
    if (!data || !width || !height) {
        rgb::set_error("null argument");
        return RT_ERR_ARG;
    }
    if (channels < 1 || channels > 4) {
        rgb::set_error("channels must be 1..4");
        return RT_ERR_ARG;
    }
    try {
        Decoder d;
        d.p = data;
        d.n = size;
        d.parse(out == nullptr);
        *width = (uint32_t)d.width;
        *height = (uint32_t)d.height;
        if (!out) return RT_OK;  // size query
        if (out_capacity < (size_t)d.width * d.height * channels) {
            rgb::set_error("output buffer too small");
            return RT_ERR_ARG;
        }
        d.idct_all();
        d.output(channels, out);
    } catch (const JpegError &e) {
        rgb::set_error("JPEG: " + e.msg);
        return RT_ERR_ARG;
    } catch (const std::bad_alloc &) {
        rgb::set_error("JPEG: out of memory");
        return RT_ERR_OOM;
    }
    return RT_OK;
}

}  // extern "C"
