// image_io.cpp -- PNG and Radiance RGBE I/O plus image metrics (host code).
//
// The renderer's PNG output replaces the reference's CoreGraphics writer
// (src/metal_bridge.mm:2072-2160); the RGBE reader follows
// src/metal_bridge.mm:2184-2259 and the metrics follow
// src/metal_bridge.mm:2383-2495 and 6078-6104.
#include "image_io.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>

namespace fpt {

// ------------------------------------------------------------------ checksums
static uint32_t crc_table[256];
static bool crc_ready = false;
static uint32_t crc32_update(uint32_t crc, const uint8_t *p, size_t n) {
    if (!crc_ready) {
        for (uint32_t i = 0; i < 256; ++i) {
            uint32_t c = i;
            for (int k = 0; k < 8; ++k) c = (c & 1u) ? 0xedb88320u ^ (c >> 1) : c >> 1;
            crc_table[i] = c;
        }
        crc_ready = true;
    }
    crc = ~crc;
    for (size_t i = 0; i < n; ++i) crc = crc_table[(crc ^ p[i]) & 0xffu] ^ (crc >> 8);
    return ~crc;
}
static uint32_t adler32(const uint8_t *p, size_t n) {
    uint32_t a = 1, b = 0;
    for (size_t i = 0; i < n; ++i) { a = (a + p[i]) % 65521u; b = (b + a) % 65521u; }
    return (b << 16) | a;
}
static void put32(std::vector<uint8_t> &v, uint32_t x) {
    v.push_back(uint8_t(x >> 24)); v.push_back(uint8_t(x >> 16)); v.push_back(uint8_t(x >> 8)); v.push_back(uint8_t(x));
}
static void chunk(std::vector<uint8_t> &out, const char *type, const std::vector<uint8_t> &data) {
    put32(out, uint32_t(data.size()));
    size_t start = out.size();
    out.insert(out.end(), type, type + 4);
    out.insert(out.end(), data.begin(), data.end());
    put32(out, crc32_update(0, out.data() + start, out.size() - start));
}

bool write_png(const char *path, uint32_t w, uint32_t h, const uint8_t *rgba, std::string &err) {
    std::vector<uint8_t> raw;
    raw.reserve(size_t(h) * (size_t(w) * 4 + 1));
    for (uint32_t y = 0; y < h; ++y) {
        raw.push_back(0);  // filter: none
        raw.insert(raw.end(), rgba + size_t(y) * w * 4, rgba + size_t(y + 1) * w * 4);
    }
    std::vector<uint8_t> z;
    z.push_back(0x78); z.push_back(0x01);
    size_t pos = 0;
    do {
        size_t n = std::min<size_t>(65535, raw.size() - pos);
        bool last = pos + n == raw.size();
        z.push_back(last ? 1 : 0);
        z.push_back(uint8_t(n)); z.push_back(uint8_t(n >> 8));
        z.push_back(uint8_t(~n)); z.push_back(uint8_t((~n) >> 8));
        z.insert(z.end(), raw.begin() + pos, raw.begin() + pos + n);
        pos += n;
    } while (pos < raw.size());
    put32(z, adler32(raw.data(), raw.size()));
    std::vector<uint8_t> out = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1a, '\n'};
    std::vector<uint8_t> ihdr;
    put32(ihdr, w); put32(ihdr, h);
    ihdr.push_back(8); ihdr.push_back(6); ihdr.push_back(0); ihdr.push_back(0); ihdr.push_back(0);
    chunk(out, "IHDR", ihdr);
    chunk(out, "IDAT", z);
    chunk(out, "IEND", {});
    FILE *f = std::fopen(path, "wb");
    if (!f) { err = std::string("failed to open ") + path + " for writing"; return false; }
    bool ok = std::fwrite(out.data(), 1, out.size(), f) == out.size();
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) err = std::string("failed to write ") + path;
    return ok;
}

// ------------------------------------------------------------------ inflate (RFC 1951)
namespace {
struct BitReader {
    const uint8_t *p; size_t n, pos = 0; uint32_t bit = 0; bool bad = false;
    uint32_t get(int count) {
        uint32_t v = 0;
        for (int i = 0; i < count; ++i) {
            if (pos >= n) { bad = true; return 0; }
            v |= uint32_t((p[pos] >> bit) & 1u) << i;
            if (++bit == 8) { bit = 0; ++pos; }
        }
        return v;
    }
};
struct Huffman {
    uint16_t counts[16] = {0};
    std::vector<uint16_t> symbols;
    bool build(const uint8_t *lengths, int n) {
        std::fill(counts, counts + 16, 0);
        for (int i = 0; i < n; ++i) counts[lengths[i]]++;
        counts[0] = 0;
        uint16_t offs[16] = {0};
        for (int i = 1; i < 16; ++i) offs[i] = uint16_t(offs[i - 1] + counts[i - 1]);
        symbols.assign(n, 0);
        for (int i = 0; i < n; ++i) if (lengths[i]) symbols[offs[lengths[i]]++] = uint16_t(i);
        return true;
    }
    int decode(BitReader &br) const {
        int code = 0, first = 0, index = 0;
        for (int len = 1; len < 16; ++len) {
            code |= int(br.get(1));
            int count = counts[len];
            if (code - count < first) return symbols[index + (code - first)];
            index += count; first += count; first <<= 1; code <<= 1;
            if (br.bad) return -1;
        }
        return -1;
    }
};
const uint16_t kLenBase[] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129, 193, 257, 385, 513, 769, 1025, 1537, 2049, 3073,
                              4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

bool inflate_block(BitReader &br, const Huffman &lit, const Huffman &dist, std::vector<uint8_t> &out) {
    while (true) {
        int sym = lit.decode(br);
        if (sym < 0) return false;
        if (sym < 256) { out.push_back(uint8_t(sym)); continue; }
        if (sym == 256) return true;
        sym -= 257;
        if (sym >= 29) return false;
        size_t len = kLenBase[sym] + br.get(kLenExtra[sym]);
        int ds = dist.decode(br);
        if (ds < 0 || ds >= 30) return false;
        size_t d = kDistBase[ds] + br.get(kDistExtra[ds]);
        if (d > out.size() || br.bad) return false;
        size_t from = out.size() - d;
        for (size_t i = 0; i < len; ++i) out.push_back(out[from + i]);
    }
}
bool zlib_inflate(const uint8_t *p, size_t n, std::vector<uint8_t> &out) {
    if (n < 6) return false;
    BitReader br{p + 2, n - 6};
    int final_block = 0;
    do {
        final_block = int(br.get(1));
        int type = int(br.get(2));
        if (br.bad) return false;
        if (type == 0) {
            if (br.bit) { br.bit = 0; ++br.pos; }
            if (br.pos + 4 > br.n) return false;
            size_t len = size_t(br.p[br.pos]) | size_t(br.p[br.pos + 1]) << 8;
            br.pos += 4;
            if (br.pos + len > br.n) return false;
            out.insert(out.end(), br.p + br.pos, br.p + br.pos + len);
            br.pos += len;
        } else if (type == 1) {
            uint8_t l[288], d[30];
            for (int i = 0; i < 144; ++i) l[i] = 8;
            for (int i = 144; i < 256; ++i) l[i] = 9;
            for (int i = 256; i < 280; ++i) l[i] = 7;
            for (int i = 280; i < 288; ++i) l[i] = 8;
            for (int i = 0; i < 30; ++i) d[i] = 5;
            Huffman hl, hd;
            hl.build(l, 288); hd.build(d, 30);
            if (!inflate_block(br, hl, hd, out)) return false;
        } else if (type == 2) {
            int hlit = int(br.get(5)) + 257, hdist = int(br.get(5)) + 1, hclen = int(br.get(4)) + 4;
            static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
            uint8_t cl[19] = {0};
            for (int i = 0; i < hclen; ++i) cl[order[i]] = uint8_t(br.get(3));
            Huffman hc;
            hc.build(cl, 19);
            uint8_t lens[320] = {0};
            int idx = 0;
            while (idx < hlit + hdist) {
                int sym = hc.decode(br);
                if (sym < 0) return false;
                if (sym < 16) lens[idx++] = uint8_t(sym);
                else {
                    int rep = 0; uint8_t val = 0;
                    if (sym == 16) { if (idx == 0) return false; val = lens[idx - 1]; rep = 3 + int(br.get(2)); }
                    else if (sym == 17) rep = 3 + int(br.get(3));
                    else rep = 11 + int(br.get(7));
                    if (idx + rep > hlit + hdist) return false;
                    while (rep--) lens[idx++] = val;
                }
            }
            Huffman hl, hd;
            hl.build(lens, hlit); hd.build(lens + hlit, hdist);
            if (!inflate_block(br, hl, hd, out)) return false;
        } else {
            return false;
        }
    } while (!final_block);
    return !br.bad;
}
uint32_t be32(const uint8_t *p) { return uint32_t(p[0]) << 24 | uint32_t(p[1]) << 16 | uint32_t(p[2]) << 8 | p[3]; }
int paeth(int a, int b, int c) {
    int p = a + b - c, pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
    return (pa <= pb && pa <= pc) ? a : (pb <= pc ? b : c);
}
}  // namespace

bool read_png(const char *path, Image &out, std::string &err) {
    std::ifstream f(path, std::ios::binary);
    if (!f) { err = std::string("failed to open image ") + path; return false; }
    std::vector<uint8_t> data((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    static const uint8_t sig[8] = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1a, '\n'};
    if (data.size() < 8 || std::memcmp(data.data(), sig, 8) != 0) { err = std::string("not a PNG: ") + path; return false; }
    size_t pos = 8;
    uint32_t w = 0, h = 0; int depth = 0, ctype = 0, interlace = 0;
    std::vector<uint8_t> idat;
    while (pos + 12 <= data.size()) {
        uint32_t len = be32(&data[pos]);
        const char *type = reinterpret_cast<const char *>(&data[pos + 4]);
        if (pos + 12 + len > data.size()) break;
        const uint8_t *body = &data[pos + 8];
        if (!std::memcmp(type, "IHDR", 4)) { w = be32(body); h = be32(body + 4); depth = body[8]; ctype = body[9]; interlace = body[12]; }
        else if (!std::memcmp(type, "IDAT", 4)) idat.insert(idat.end(), body, body + len);
        else if (!std::memcmp(type, "IEND", 4)) break;
        pos += 12 + len;
    }
    int channels = ctype == 6 ? 4 : (ctype == 2 ? 3 : (ctype == 0 ? 1 : (ctype == 4 ? 2 : 0)));
    if (!w || !h || depth != 8 || !channels || interlace) { err = std::string("unsupported PNG format in ") + path; return false; }
    std::vector<uint8_t> raw;
    if (!zlib_inflate(idat.data(), idat.size(), raw)) { err = std::string("corrupt PNG data in ") + path; return false; }
    size_t stride = size_t(w) * channels;
    if (raw.size() < size_t(h) * (stride + 1)) { err = std::string("truncated PNG data in ") + path; return false; }
    std::vector<uint8_t> px(size_t(h) * stride);
    for (uint32_t y = 0; y < h; ++y) {
        const uint8_t *src = &raw[size_t(y) * (stride + 1)];
        uint8_t *dst = &px[size_t(y) * stride];
        const uint8_t *prev = y ? &px[size_t(y - 1) * stride] : nullptr;
        int filter = src[0];
        for (size_t i = 0; i < stride; ++i) {
            int a = i >= size_t(channels) ? dst[i - channels] : 0, b = prev ? prev[i] : 0,
                c = (prev && i >= size_t(channels)) ? prev[i - channels] : 0;
            int v = src[i + 1];
            switch (filter) {
                case 1: v += a; break;
                case 2: v += b; break;
                case 3: v += (a + b) / 2; break;
                case 4: v += paeth(a, b, c); break;
                default: break;
            }
            dst[i] = uint8_t(v);
        }
    }
    out.width = w; out.height = h;
    out.rgba.assign(size_t(w) * h * 4, 255);
    for (size_t i = 0; i < size_t(w) * h; ++i) {
        const uint8_t *s = &px[i * channels];
        uint8_t *d = &out.rgba[i * 4];
        if (channels >= 3) { d[0] = s[0]; d[1] = s[1]; d[2] = s[2]; if (channels == 4) d[3] = s[3]; }
        else { d[0] = d[1] = d[2] = s[0]; if (channels == 2) d[3] = s[1]; }
    }
    return true;
}

// ------------------------------------------------------------------ RGBE
bool read_radiance_hdr(const char *path, HdrImage &out, std::string &err) {
    std::ifstream stream(path, std::ios::binary);
    if (!stream) { err = std::string("failed to open HDRI ") + path; return false; }
    std::string line;
    bool format_ok = false;
    while (std::getline(stream, line)) {
        if (!line.empty() && line.back() == '\r') line.pop_back();
        if (line.rfind("FORMAT=32-bit_rle_rgbe", 0) == 0) format_ok = true;
        if (line.empty()) break;
    }
    if (!std::getline(stream, line)) { err = std::string("missing HDRI resolution in ") + path; return false; }
    char ys = 0, xs = 0;
    int width = 0, height = 0;
    if (std::sscanf(line.c_str(), " %cY %d %cX %d", &ys, &height, &xs, &width) != 4 || width <= 0 || height <= 0) {
        err = "unsupported HDRI resolution line '" + line + "'";
        return false;
    }
    if (!format_ok || width < 8 || width > 32767) { err = std::string("unsupported non-RLE Radiance HDRI ") + path; return false; }
    // The reference bounds the width only; the height is bounded too, so a
    // corrupt header cannot ask for more than 32767^2 pixels of floats.
    if (height > 32767) { err = "HDRI height " + std::to_string(height) + " exceeds 32767 in " + path; return false; }
    out.width = uint32_t(width); out.height = uint32_t(height);
    out.rgb.assign(size_t(width) * height * 3, 0.0f);
    std::vector<uint8_t> scan(size_t(width) * 4);
    for (int fy = 0; fy < height; ++fy) {
        uint8_t hd[4] = {0};
        stream.read(reinterpret_cast<char *>(hd), 4);
        if (!stream || hd[0] != 2u || hd[1] != 2u || ((uint32_t(hd[2]) << 8) | hd[3]) != uint32_t(width)) {
            err = "invalid HDRI scanline " + std::to_string(fy) + " in " + path;
            return false;
        }
        for (int ch = 0; ch < 4; ++ch) {
            int x = 0;
            while (x < width) {
                uint8_t code = 0;
                stream.read(reinterpret_cast<char *>(&code), 1);
                if (!stream || code == 0u) { err = "truncated HDRI scanline " + std::to_string(fy) + " in " + path; return false; }
                if (code > 128u) {
                    int count = int(code - 128u);
                    uint8_t v = 0;
                    stream.read(reinterpret_cast<char *>(&v), 1);
                    if (!stream || x + count > width) { err = "corrupt HDRI run in " + std::string(path); return false; }
                    for (int i = 0; i < count; ++i) scan[size_t(x++) * 4 + ch] = v;
                } else {
                    int count = int(code);
                    if (x + count > width) { err = "corrupt HDRI literal in " + std::string(path); return false; }
                    for (int i = 0; i < count; ++i) {
                        uint8_t v = 0;
                        stream.read(reinterpret_cast<char *>(&v), 1);
                        scan[size_t(x++) * 4 + ch] = v;
                    }
                }
            }
        }
        int oy = ys == '-' ? fy : height - 1 - fy;
        for (int fx = 0; fx < width; ++fx) {
            int ox = xs == '+' ? fx : width - 1 - fx;
            uint8_t e = scan[size_t(fx) * 4 + 3];
            float sc = e == 0u ? 0.0f : std::ldexp(1.0f, int(e) - (128 + 8));
            size_t dst = (size_t(oy) * width + ox) * 3;
            for (int k = 0; k < 3; ++k) out.rgb[dst + k] = (float(scan[size_t(fx) * 4 + k]) + 0.5f) * sc;
        }
    }
    return true;
}


uint16_t reference_float_to_half(float value) {
    uint32_t bits = 0;
    std::memcpy(&bits, &value, sizeof(bits));
    const uint32_t sign = (bits >> 16u) & 0x8000u;
    int exponent = int((bits >> 23u) & 0xffu) - 127 + 15;
    uint32_t mantissa = bits & 0x7fffffu;
    if (exponent <= 0) {
        if (exponent < -10) return uint16_t(sign);
        mantissa = (mantissa | 0x800000u) >> uint32_t(1 - exponent);
        return uint16_t(sign | ((mantissa + 0x1000u) >> 13u));
    }
    if (exponent >= 31) return uint16_t(sign | 0x7c00u);
    return uint16_t(sign | (uint32_t(exponent) << 10u) | ((mantissa + 0x1000u) >> 13u));
}

// ------------------------------------------------------------------ metrics
size_t unique_colour_sample(const uint8_t *rgba, size_t pixels) {
    std::vector<uint32_t> colours;
    colours.reserve(256);
    for (size_t i = 0; i < pixels; ++i) {
        const uint8_t *p = rgba + i * 4;
        uint32_t c = uint32_t(p[0]) << 24 | uint32_t(p[1]) << 16 | uint32_t(p[2]) << 8 | p[3];
        if (std::find(colours.begin(), colours.end(), c) == colours.end()) {
            colours.push_back(c);
            if (colours.size() >= 2048) break;
        }
    }
    return colours.size();
}

static inline double luma(const uint8_t *img, size_t p) {
    const uint8_t *q = img + p * 4;
    return 0.2126 * double(q[0]) + 0.7152 * double(q[1]) + 0.0722 * double(q[2]);
}

ImageMetrics compare_rgba(const uint8_t *a, const uint8_t *b, uint32_t W, uint32_t H) {
    ImageMetrics m{};
    double abs_sum = 0, sq = 0;
    uint32_t maxd = 0;
    uint64_t changed = 0;
    size_t px = size_t(W) * H;
    for (size_t p = 0; p < px; ++p) {
        bool ch = false;
        for (int k = 0; k < 3; ++k) {
            uint32_t d = uint32_t(std::abs(int(a[p * 4 + k]) - int(b[p * 4 + k])));
            abs_sum += d; sq += double(d) * d; maxd = std::max(maxd, d);
            if (d) ch = true;
        }
        if (ch) ++changed;
    }
    double n = double(px * 3);
    m.mae = abs_sum / n; m.rmse = std::sqrt(sq / n); m.max_abs = maxd;
    m.changed_pct = px ? 100.0 * double(changed) / double(px) : 0.0;
    const double c1 = 6.5025, c2 = 58.5225;
    double ws = 0, wt = 0;
    for (uint32_t by = 0; by < H; by += 8)
        for (uint32_t bx = 0; bx < W; bx += 8) {
            uint32_t ye = std::min(H, by + 8), xe = std::min(W, bx + 8);
            double cnt = double((ye - by) * (xe - bx)), ma = 0, mb = 0;
            for (uint32_t y = by; y < ye; ++y)
                for (uint32_t x = bx; x < xe; ++x) { size_t p = size_t(y) * W + x; ma += luma(a, p); mb += luma(b, p); }
            ma /= cnt; mb /= cnt;
            double va = 0, vb = 0, cv = 0;
            for (uint32_t y = by; y < ye; ++y)
                for (uint32_t x = bx; x < xe; ++x) {
                    size_t p = size_t(y) * W + x;
                    double da = luma(a, p) - ma, db = luma(b, p) - mb;
                    va += da * da; vb += db * db; cv += da * db;
                }
            double den = std::max(1.0, cnt - 1.0);
            va /= den; vb /= den; cv /= den;
            double num = (2 * ma * mb + c1) * (2 * cv + c2), dd = (ma * ma + mb * mb + c1) * (va + vb + c2);
            ws += (dd > 0 ? num / dd : 1.0) * cnt;
            wt += cnt;
        }
    m.ssim = wt > 0 ? std::clamp(ws / wt, -1.0, 1.0) : 0.0;
    std::vector<double> A(64 * 64), B(64 * 64);
    for (uint32_t y = 0; y < 64; ++y) {
        uint32_t y0 = uint32_t((uint64_t(y) * H) / 64), y1 = std::max(uint32_t((uint64_t(y + 1) * H) / 64), y0 + 1);
        for (uint32_t x = 0; x < 64; ++x) {
            uint32_t x0 = uint32_t((uint64_t(x) * W) / 64), x1 = std::max(uint32_t((uint64_t(x + 1) * W) / 64), x0 + 1);
            double sa = 0, sb = 0, cnt = 0;
            for (uint32_t sy = y0; sy < y1; ++sy)
                for (uint32_t sx = x0; sx < x1; ++sx) { size_t p = size_t(sy) * W + sx; sa += luma(a, p); sb += luma(b, p); cnt += 1; }
            A[y * 64 + x] = sa / cnt; B[y * 64 + x] = sb / cnt;
        }
    }
    double ma = 0, mb = 0, nn = double(A.size());
    for (size_t i = 0; i < A.size(); ++i) { ma += A[i]; mb += B[i]; }
    ma /= nn; mb /= nn;
    double va = 0, vb = 0, cv = 0;
    for (size_t i = 0; i < A.size(); ++i) { double da = A[i] - ma, db = B[i] - mb; va += da * da; vb += db * db; cv += da * db; }
    double den = std::max(1.0, nn - 1.0);
    va /= den; vb /= den; cv /= den;
    double num = (2 * ma * mb + c1) * (2 * cv + c2), dd = (ma * ma + mb * mb + c1) * (va + vb + c2);
    m.lf_ssim = dd > 0 ? std::clamp(num / dd, -1.0, 1.0) : 1.0;
    m.unique_baseline = unique_colour_sample(a, px);
    m.unique_candidate = unique_colour_sample(b, px);
    return m;
}

}  // namespace fpt
