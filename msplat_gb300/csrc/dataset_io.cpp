// Dataset ingestion: on-disk layouts, point clouds and image decoding (see
// dataset_io.h).  Loader behaviour follows core/src/loaders/load_colmap.cpp,
// load_nerfstudio.cpp, load_polycam.cpp and load_ply.cpp; the decoders
// implement the published formats (PNG: ISO/IEC 15948 with DEFLATE, RFC 1951
// and zlib, RFC 1950; JPEG: ITU-T T.81 baseline and extended sequential
// Huffman, JFIF colour conversion).
#include "dataset_io.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <unordered_map>

namespace fs = std::filesystem;

namespace msplat {
namespace io {

static std::vector<uint8_t> read_file(const std::string &path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("cannot open " + path);
    f.seekg(0, std::ios::end);
    const std::streamoff n = f.tellg();
    f.seekg(0, std::ios::beg);
    std::vector<uint8_t> b((size_t)std::max<std::streamoff>(n, 0));
    if (n > 0) f.read(reinterpret_cast<char *>(b.data()), n);
    return b;
}

// ===========================================================================
// DEFLATE (RFC 1951) inside a zlib stream (RFC 1950)
// ===========================================================================

namespace {

struct BitIn {
    const uint8_t *p;
    size_t n, pos = 0;
    uint32_t buf = 0;
    int cnt = 0;
    BitIn(const uint8_t *d, size_t len) : p(d), n(len) {}
    uint32_t bits(int k) {   // k <= 24, LSB first
        while (cnt < k) {
            if (pos >= n) throw std::runtime_error("deflate: unexpected end of data");
            buf |= (uint32_t)p[pos++] << cnt;
            cnt += 8;
        }
        const uint32_t v = buf & ((1u << k) - 1u);
        buf >>= k;
        cnt -= k;
        return v;
    }
    void align() {
        buf = 0;
        cnt = 0;
    }
};

// Canonical Huffman code: symbols ordered by (length, value); decoded one
// bit at a time (codes are at most 15 bits).
struct Huff {
    uint16_t count[16] = {0};
    std::vector<uint16_t> sym;
    void build(const uint8_t *len, int n) {
        std::fill(count, count + 16, 0);
        for (int i = 0; i < n; i++) count[len[i]]++;
        count[0] = 0;
        uint16_t offs[16] = {0};
        for (int l = 1; l < 16; l++) offs[l] = offs[l - 1] + count[l - 1];
        sym.assign(n, 0);
        for (int i = 0; i < n; i++)
            if (len[i]) sym[offs[len[i]]++] = (uint16_t)i;
    }
    int decode(BitIn &in) const {
        int code = 0, first = 0, index = 0;
        for (int l = 1; l < 16; l++) {
            code |= (int)in.bits(1);
            const int c = count[l];
            if (code - first < c) return sym[index + (code - first)];
            index += c;
            first = (first + c) << 1;
            code <<= 1;
        }
        throw std::runtime_error("deflate: bad Huffman code");
    }
};

const uint16_t kLenBase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31,
                               35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129, 193,
                                257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8,
                                9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

void inflate_block(BitIn &in, const Huff &lit, const Huff &dist, std::vector<uint8_t> &out) {
    for (;;) {
        const int s = lit.decode(in);
        if (s < 256) {
            out.push_back((uint8_t)s);
        } else if (s == 256) {
            return;
        } else {
            const int li = s - 257;
            if (li >= 29) throw std::runtime_error("deflate: bad length symbol");
            const int len = kLenBase[li] + (int)in.bits(kLenExtra[li]);
            const int di = dist.decode(in);
            if (di >= 30) throw std::runtime_error("deflate: bad distance symbol");
            const size_t d = kDistBase[di] + in.bits(kDistExtra[di]);
            if (d > out.size()) throw std::runtime_error("deflate: distance past the start");
            const size_t from = out.size() - d;
            for (int k = 0; k < len; k++) out.push_back(out[from + k]);
        }
    }
}

std::vector<uint8_t> zlib_inflate(const uint8_t *data, size_t n, size_t expect) {
    if (n < 2) throw std::runtime_error("zlib: stream too short");
    if ((data[0] & 15) != 8 || ((data[0] << 8) | data[1]) % 31 != 0) throw std::runtime_error("zlib: bad header");
    if (data[1] & 0x20) throw std::runtime_error("zlib: preset dictionary not supported");
    BitIn in(data + 2, n - 2);
    std::vector<uint8_t> out;
    out.reserve(expect);
    Huff fl, fd;
    {
        uint8_t l[288];
        for (int i = 0; i < 144; i++) l[i] = 8;
        for (int i = 144; i < 256; i++) l[i] = 9;
        for (int i = 256; i < 280; i++) l[i] = 7;
        for (int i = 280; i < 288; i++) l[i] = 8;
        fl.build(l, 288);
        uint8_t d[30];
        std::fill(d, d + 30, 5);
        fd.build(d, 30);
    }
    int last = 0;
    while (!last) {
        last = (int)in.bits(1);
        const int type = (int)in.bits(2);
        if (type == 0) {
            in.align();
            if (in.pos + 4 > in.n) throw std::runtime_error("deflate: truncated stored block");
            const unsigned len = in.p[in.pos] | (in.p[in.pos + 1] << 8);
            in.pos += 4;
            if (in.pos + len > in.n) throw std::runtime_error("deflate: truncated stored block");
            out.insert(out.end(), in.p + in.pos, in.p + in.pos + len);
            in.pos += len;
        } else if (type == 1) {
            inflate_block(in, fl, fd, out);
        } else if (type == 2) {
            const int hlit = (int)in.bits(5) + 257, hdist = (int)in.bits(5) + 1, hclen = (int)in.bits(4) + 4;
            static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
            uint8_t cl[19] = {0};
            for (int i = 0; i < hclen; i++) cl[order[i]] = (uint8_t)in.bits(3);
            Huff hc;
            hc.build(cl, 19);
            uint8_t lens[320] = {0};
            int i = 0;
            while (i < hlit + hdist) {
                const int s = hc.decode(in);
                if (s < 16) {
                    lens[i++] = (uint8_t)s;
                } else {
                    int rep = 0;
                    uint8_t v = 0;
                    if (s == 16) {
                        if (i == 0) throw std::runtime_error("deflate: repeat without a length");
                        v = lens[i - 1];
                        rep = 3 + (int)in.bits(2);
                    } else if (s == 17) {
                        rep = 3 + (int)in.bits(3);
                    } else {
                        rep = 11 + (int)in.bits(7);
                    }
                    if (i + rep > hlit + hdist) throw std::runtime_error("deflate: code lengths overflow");
                    while (rep--) lens[i++] = v;
                }
            }
            Huff dl, dd;
            dl.build(lens, hlit);
            dd.build(lens + hlit, hdist);
            inflate_block(in, dl, dd, out);
        } else {
            throw std::runtime_error("deflate: bad block type");
        }
    }
    return out;
}

uint32_t be32(const uint8_t *p) { return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3]; }

// ===========================================================================
// PNG
// ===========================================================================

Image decode_png(const std::vector<uint8_t> &f) {
    static const uint8_t sig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
    if (f.size() < 8 || std::memcmp(f.data(), sig, 8) != 0) throw std::runtime_error("png: bad signature");
    size_t pos = 8;
    uint32_t W = 0, H = 0;
    int depth = 0, ctype = -1, interlace = 0;
    std::vector<uint8_t> idat, plte;
    while (pos + 8 <= f.size()) {
        const uint32_t len = be32(&f[pos]);
        const std::string type(reinterpret_cast<const char *>(&f[pos + 4]), 4);
        if (pos + 12 + (size_t)len > f.size()) throw std::runtime_error("png: truncated chunk " + type);
        const uint8_t *d = &f[pos + 8];
        if (type == "IHDR") {
            if (len < 13) throw std::runtime_error("png: short IHDR");
            W = be32(d);
            H = be32(d + 4);
            depth = d[8];
            ctype = d[9];
            interlace = d[12];
        } else if (type == "PLTE") {
            plte.assign(d, d + len);
        } else if (type == "IDAT") {
            idat.insert(idat.end(), d, d + len);
        } else if (type == "IEND") {
            break;
        }
        pos += 12 + len;
    }
    if (W == 0 || H == 0 || W > 65535 || H > 65535) throw std::runtime_error("png: bad size");
    if (interlace) throw std::runtime_error("png: interlaced images are not supported");
    int ch = 0;
    switch (ctype) {
        case 0: ch = 1; break;
        case 2: ch = 3; break;
        case 3: ch = 1; break;
        case 4: ch = 2; break;
        case 6: ch = 4; break;
        default: throw std::runtime_error("png: bad colour type");
    }
    const bool ok_depth = (ctype == 3) ? (depth == 1 || depth == 2 || depth == 4 || depth == 8)
                          : (ctype == 0) ? (depth == 1 || depth == 2 || depth == 4 || depth == 8 || depth == 16)
                                         : (depth == 8 || depth == 16);
    if (!ok_depth) throw std::runtime_error("png: bad bit depth");
    const size_t bits_pp = (size_t)ch * depth;
    const size_t stride = (W * bits_pp + 7) / 8;
    const size_t bpp = std::max<size_t>(1, bits_pp / 8);
    std::vector<uint8_t> raw = zlib_inflate(idat.data(), idat.size(), (stride + 1) * H);
    if (raw.size() < (stride + 1) * H) throw std::runtime_error("png: image data too short");
    // undo the per-row filters in place
    std::vector<uint8_t> img(stride * H);
    for (uint32_t y = 0; y < H; y++) {
        const uint8_t ft = raw[y * (stride + 1)];
        const uint8_t *src = &raw[y * (stride + 1) + 1];
        uint8_t *row = &img[y * stride];
        const uint8_t *up = y ? &img[(y - 1) * stride] : nullptr;
        for (size_t x = 0; x < stride; x++) {
            const int a = x >= bpp ? row[x - bpp] : 0, b = up ? up[x] : 0, c = (up && x >= bpp) ? up[x - bpp] : 0;
            int v = src[x];
            switch (ft) {
                case 0: break;
                case 1: v += a; break;
                case 2: v += b; break;
                case 3: v += (a + b) >> 1; break;
                case 4: {
                    const int p = a + b - c, pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
                    v += (pa <= pb && pa <= pc) ? a : (pb <= pc ? b : c);
                    break;
                }
                default: throw std::runtime_error("png: bad filter type");
            }
            row[x] = (uint8_t)v;
        }
    }
    Image out;
    out.width = (int)W;
    out.height = (int)H;
    out.rgb.resize((size_t)W * H * 3);
    for (uint32_t y = 0; y < H; y++) {
        const uint8_t *row = &img[y * stride];
        for (uint32_t x = 0; x < W; x++) {
            float v[4];
            for (int c = 0; c < ch; c++) {
                if (depth == 16) {
                    const size_t o = ((size_t)x * ch + c) * 2;
                    v[c] = (float)((row[o] << 8) | row[o + 1]) / 65535.0f;
                } else if (depth == 8) {
                    v[c] = (float)row[(size_t)x * ch + c] / 255.0f;
                } else {   // 1, 2, 4 bits, one channel
                    const size_t bit = (size_t)x * depth;
                    const int s = (row[bit / 8] >> (8 - depth - (int)(bit % 8))) & ((1 << depth) - 1);
                    v[c] = (ctype == 3) ? (float)s : (float)s / (float)((1 << depth) - 1);
                }
            }
            float *o = &out.rgb[((size_t)y * W + x) * 3];
            if (ctype == 3) {
                const int idx = depth == 8 ? row[x] : (int)v[0];
                if ((size_t)idx * 3 + 2 >= plte.size()) throw std::runtime_error("png: palette index out of range");
                for (int c = 0; c < 3; c++) o[c] = (float)plte[idx * 3 + c] / 255.0f;
            } else if (ch <= 2) {
                o[0] = o[1] = o[2] = v[0];
            } else {
                o[0] = v[0]; o[1] = v[1]; o[2] = v[2];
            }
        }
    }
    return out;
}

// ===========================================================================
// JPEG: baseline / extended sequential, Huffman, 8-bit samples
// ===========================================================================

const uint8_t kZigzag[64] = {0,  1,  8,  16, 9,  2,  3,  10, 17, 24, 32, 25, 18, 11, 4,  5,
                             12, 19, 26, 33, 40, 48, 41, 34, 27, 20, 13, 6,  7,  14, 21, 28,
                             35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51,
                             58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63};

struct JHuff {
    // canonical code: maxcode/valptr per length (T.81 Annex F)
    int mincode[17], maxcode[18], valptr[17];
    std::vector<uint8_t> vals;
    bool present = false;
};

struct JComp {
    int id, h, v, tq, td = 0, ta = 0, pred = 0;
    int bw, bh;                      // blocks across / down (padded to whole MCUs)
    std::vector<float> plane;        // samples, bw*8 x bh*8
};

struct JBits {
    const uint8_t *p;
    size_t n, pos;
    uint32_t buf = 0;
    int cnt = 0;
    bool marker_hit = false;
    int bit() {
        if (cnt == 0) {
            uint8_t b = 0;
            if (!marker_hit && pos < n) {
                b = p[pos];
                if (b == 0xFF) {
                    const uint8_t nx = pos + 1 < n ? p[pos + 1] : 0;
                    if (nx == 0x00) {
                        pos += 2;
                    } else {
                        marker_hit = true;   // a marker: feed zeros from here
                        b = 0;
                    }
                } else {
                    pos++;
                }
            }
            buf = b;
            cnt = 8;
        }
        cnt--;
        return (buf >> cnt) & 1;
    }
    int bits(int k) {
        int v = 0;
        for (int i = 0; i < k; i++) v = (v << 1) | bit();
        return v;
    }
    void reset() {
        cnt = 0;
        marker_hit = false;
    }
};

int jdecode(JBits &in, const JHuff &h) {
    int code = in.bit();
    for (int l = 1; l <= 16; l++) {
        if (code <= h.maxcode[l]) return h.vals[h.valptr[l] + code - h.mincode[l]];
        code = (code << 1) | in.bit();
    }
    throw std::runtime_error("jpeg: bad Huffman code");
}

int extend(int v, int t) { return t == 0 ? 0 : (v < (1 << (t - 1)) ? v - (1 << t) + 1 : v); }

// 8x8 inverse DCT from the definition, separable:
// f(x) = sum_u C(u)/2 F(u) cos((2x+1) u pi / 16), C(0) = 1/sqrt(2)
struct Idct {
    float c[8][8];
    Idct() {
        const double pi = 3.14159265358979323846;
        for (int x = 0; x < 8; x++)
            for (int u = 0; u < 8; u++)
                c[x][u] = (float)(0.5 * (u == 0 ? 1.0 / std::sqrt(2.0) : 1.0) * std::cos((2 * x + 1) * u * pi / 16.0));
    }
    void run(const float in[64], float out[64]) const {
        float tmp[64];
        for (int y = 0; y < 8; y++)          // rows: over u
            for (int x = 0; x < 8; x++) {
                float s = 0.f;
                for (int u = 0; u < 8; u++) s += c[x][u] * in[y * 8 + u];
                tmp[y * 8 + x] = s;
            }
        for (int x = 0; x < 8; x++)          // columns: over v
            for (int y = 0; y < 8; y++) {
                float s = 0.f;
                for (int v = 0; v < 8; v++) s += c[y][v] * tmp[v * 8 + x];
                out[y * 8 + x] = s;
            }
    }
};

Image decode_jpeg(const std::vector<uint8_t> &f) {
    if (f.size() < 4 || f[0] != 0xFF || f[1] != 0xD8) throw std::runtime_error("jpeg: no SOI marker");
    uint16_t qt[4][64];
    bool qt_ok[4] = {false, false, false, false};
    JHuff hdc[4], hac[4];
    std::vector<JComp> comps;
    int W = 0, H = 0, hmax = 1, vmax = 1, restart = 0;
    bool frame = false, done = false;
    size_t pos = 2;
    static const Idct idct;
    while (!done && pos + 4 <= f.size()) {
        if (f[pos] != 0xFF) { pos++; continue; }
        const uint8_t m = f[pos + 1];
        pos += 2;
        if (m == 0xD8 || m == 0x01 || (m >= 0xD0 && m <= 0xD7) || m == 0xFF) {
            if (m == 0xFF) pos--;
            continue;
        }
        if (m == 0xD9) break;
        if (pos + 2 > f.size()) break;
        const size_t len = ((size_t)f[pos] << 8) | f[pos + 1];
        if (len < 2 || pos + len > f.size()) throw std::runtime_error("jpeg: truncated segment");
        const uint8_t *d = &f[pos + 2];
        const size_t dl = len - 2;
        if (m == 0xDB) {   // DQT
            size_t i = 0;
            while (i < dl) {
                const int pq = d[i] >> 4, tq = d[i] & 3;
                i++;
                for (int k = 0; k < 64; k++) {
                    qt[tq][kZigzag[k]] = pq ? (uint16_t)((d[i] << 8) | d[i + 1]) : d[i];
                    i += pq ? 2 : 1;
                }
                qt_ok[tq] = true;
            }
        } else if (m == 0xC4) {   // DHT
            size_t i = 0;
            while (i < dl) {
                const int tc = d[i] >> 4, th = d[i] & 3;
                i++;
                JHuff &h = tc ? hac[th] : hdc[th];
                int counts[17] = {0}, total = 0;
                for (int l = 1; l <= 16; l++) total += (counts[l] = d[i + l - 1]);
                i += 16;
                h.vals.assign(d + i, d + i + total);
                i += total;
                int code = 0, k = 0;
                for (int l = 1; l <= 16; l++) {
                    h.valptr[l] = k;
                    h.mincode[l] = code;
                    code += counts[l];
                    k += counts[l];
                    h.maxcode[l] = counts[l] ? code - 1 : -1;
                    code <<= 1;
                }
                h.maxcode[17] = 0x7fffffff;
                h.present = true;
            }
        } else if (m == 0xDD) {   // DRI
            restart = (d[0] << 8) | d[1];
        } else if (m == 0xC0 || m == 0xC1) {   // SOF0 / SOF1
            if (d[0] != 8) throw std::runtime_error("jpeg: only 8-bit samples are supported");
            H = (d[1] << 8) | d[2];
            W = (d[3] << 8) | d[4];
            const int nc = d[5];
            if (W <= 0 || H <= 0 || (nc != 1 && nc != 3)) throw std::runtime_error("jpeg: bad frame header");
            comps.resize(nc);
            for (int c = 0; c < nc; c++) {
                comps[c].id = d[6 + 3 * c];
                comps[c].h = d[7 + 3 * c] >> 4;
                comps[c].v = d[7 + 3 * c] & 15;
                comps[c].tq = d[8 + 3 * c] & 3;
                if (comps[c].h < 1 || comps[c].h > 4 || comps[c].v < 1 || comps[c].v > 4)
                    throw std::runtime_error("jpeg: bad sampling factors");
                hmax = std::max(hmax, comps[c].h);
                vmax = std::max(vmax, comps[c].v);
            }
            frame = true;
        } else if (m >= 0xC2 && m <= 0xCF && m != 0xC4 && m != 0xC8 && m != 0xCC) {
            throw std::runtime_error("jpeg: progressive, lossless and arithmetic-coded JPEG are not supported");
        } else if (m == 0xDA) {   // SOS
            if (!frame) throw std::runtime_error("jpeg: scan before frame");
            const int ns = d[0];
            std::vector<JComp *> sc;
            for (int k = 0; k < ns; k++) {
                const int cid = d[1 + 2 * k];
                JComp *cp = nullptr;
                for (auto &c : comps)
                    if (c.id == cid) cp = &c;
                if (!cp) throw std::runtime_error("jpeg: scan names an unknown component");
                cp->td = d[2 + 2 * k] >> 4;
                cp->ta = d[2 + 2 * k] & 3;
                sc.push_back(cp);
            }
            const int mcux = (W + 8 * hmax - 1) / (8 * hmax), mcuy = (H + 8 * vmax - 1) / (8 * vmax);
            for (auto &c : comps) {
                c.bw = mcux * c.h;
                c.bh = mcuy * c.v;
                if (c.plane.empty()) c.plane.assign((size_t)c.bw * 8 * c.bh * 8, 0.f);
                c.pred = 0;
                if (!qt_ok[c.tq]) throw std::runtime_error("jpeg: missing quantisation table");
            }
            JBits in{f.data(), f.size(), pos + len};
            auto block = [&](JComp &c, int bx, int by) {
                const JHuff &dc = hdc[c.td], &ac = hac[c.ta];
                if (!dc.present || !ac.present) throw std::runtime_error("jpeg: missing Huffman table");
                float coef[64] = {0.f};
                const int t = jdecode(in, dc);
                c.pred += extend(in.bits(t), t);
                coef[0] = (float)c.pred * qt[c.tq][0];
                for (int k = 1; k < 64;) {
                    const int rs = jdecode(in, ac), r = rs >> 4, s = rs & 15;
                    if (s == 0) {
                        if (r != 15) break;   // end of block
                        k += 16;
                        continue;
                    }
                    k += r;
                    if (k > 63) break;
                    coef[kZigzag[k]] = (float)extend(in.bits(s), s) * qt[c.tq][kZigzag[k]];
                    k++;
                }
                float px[64];
                idct.run(coef, px);
                const int stride = c.bw * 8;
                for (int y = 0; y < 8; y++)
                    for (int x = 0; x < 8; x++)
                        c.plane[(size_t)(by * 8 + y) * stride + bx * 8 + x] = px[y * 8 + x] + 128.f;
            };
            int todo = restart;
            if (ns == 1) {   // non-interleaved: the component's own block grid
                JComp &c = *sc[0];
                const int cw = (W * c.h + hmax - 1) / hmax, chh = (H * c.v + vmax - 1) / vmax;
                const int bw = (cw + 7) / 8, bh = (chh + 7) / 8;
                for (int by = 0; by < bh; by++)
                    for (int bx = 0; bx < bw; bx++) {
                        if (restart && todo == 0) {
                            in.reset();
                            while (in.pos + 1 < in.n && !(in.p[in.pos] == 0xFF && in.p[in.pos + 1] >= 0xD0 &&
                                                           in.p[in.pos + 1] <= 0xD7))
                                in.pos++;
                            in.pos += 2;
                            c.pred = 0;
                            todo = restart;
                        }
                        block(c, bx, by);
                        if (restart) todo--;
                    }
            } else {
                for (int my = 0; my < mcuy; my++)
                    for (int mx = 0; mx < mcux; mx++) {
                        if (restart && todo == 0) {
                            in.reset();
                            while (in.pos + 1 < in.n && !(in.p[in.pos] == 0xFF && in.p[in.pos + 1] >= 0xD0 &&
                                                           in.p[in.pos + 1] <= 0xD7))
                                in.pos++;
                            in.pos += 2;
                            for (auto *c : sc) c->pred = 0;
                            todo = restart;
                        }
                        for (auto *c : sc)
                            for (int v = 0; v < c->v; v++)
                                for (int h = 0; h < c->h; h++) block(*c, mx * c->h + h, my * c->v + v);
                        if (restart) todo--;
                    }
            }
            // continue after the entropy-coded data: find the next marker
            size_t q = in.pos;
            while (q + 1 < f.size() && !(f[q] == 0xFF && f[q + 1] != 0x00 && !(f[q + 1] >= 0xD0 && f[q + 1] <= 0xD7)))
                q++;
            pos = q;
            done = (comps.size() == 1 || ns == (int)comps.size());
            continue;
        }
        pos += len;
    }
    if (!frame || comps.empty() || comps[0].plane.empty()) throw std::runtime_error("jpeg: no image data");
    Image out;
    out.width = W;
    out.height = H;
    out.rgb.resize((size_t)W * H * 3);
    auto sample = [&](const JComp &c, int x, int y) {   // nearest upsampling of subsampled planes
        const int sx = x * c.h / hmax, sy = y * c.v / vmax;
        return c.plane[(size_t)sy * (c.bw * 8) + sx];
    };
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            float *o = &out.rgb[((size_t)y * W + x) * 3];
            const float Y = sample(comps[0], x, y);
            if (comps.size() == 1) {
                o[0] = o[1] = o[2] = std::min(std::max(Y, 0.f), 255.f) / 255.f;
                continue;
            }
            const float cb = sample(comps[1], x, y) - 128.f, cr = sample(comps[2], x, y) - 128.f;
            const float r = Y + 1.402f * cr, g = Y - 0.344136f * cb - 0.714136f * cr, b = Y + 1.772f * cb;
            o[0] = std::min(std::max(r, 0.f), 255.f) / 255.f;
            o[1] = std::min(std::max(g, 0.f), 255.f) / 255.f;
            o[2] = std::min(std::max(b, 0.f), 255.f) / 255.f;
        }
    return out;
}

// ===========================================================================
// PPM / PGM (binary)
// ===========================================================================

Image decode_pnm(const std::vector<uint8_t> &f) {
    size_t pos = 2;
    auto token = [&]() {
        while (pos < f.size()) {
            if (f[pos] == '#') {
                while (pos < f.size() && f[pos] != '\n') pos++;
            } else if (std::isspace(f[pos])) {
                pos++;
            } else {
                break;
            }
        }
        long v = 0;
        while (pos < f.size() && std::isdigit(f[pos])) v = v * 10 + (f[pos++] - '0');
        return v;
    };
    const bool color = f[1] == '6';
    const long W = token(), H = token(), maxv = token();
    pos++;
    if (W <= 0 || H <= 0 || maxv <= 0 || maxv > 65535) throw std::runtime_error("pnm: bad header");
    const int ch = color ? 3 : 1, bs = maxv > 255 ? 2 : 1;
    if (pos + (size_t)W * H * ch * bs > f.size()) throw std::runtime_error("pnm: truncated");
    Image out;
    out.width = (int)W;
    out.height = (int)H;
    out.rgb.resize((size_t)W * H * 3);
    for (size_t i = 0; i < (size_t)W * H; i++)
        for (int c = 0; c < 3; c++) {
            const size_t o = (i * ch + (color ? c : 0)) * bs;
            const int v = bs == 2 ? (f[pos + o] << 8) | f[pos + o + 1] : f[pos + o];
            out.rgb[i * 3 + c] = (float)v / (float)maxv;
        }
    return out;
}

}  // namespace

Image read_image(const std::string &path) {
    const std::vector<uint8_t> f = read_file(path);
    if (f.size() >= 8 && f[0] == 137 && f[1] == 'P' && f[2] == 'N' && f[3] == 'G') return decode_png(f);
    if (f.size() >= 2 && f[0] == 0xFF && f[1] == 0xD8) return decode_jpeg(f);
    if (f.size() >= 2 && f[0] == 'P' && (f[1] == '6' || f[1] == '5')) return decode_pnm(f);
    throw std::runtime_error("unsupported image format: " + path);
}

Image resize_area(const Image &src, int dst_w, int dst_h) {
    if (dst_w <= 0 || dst_h <= 0) throw std::runtime_error("resize: bad size");
    Image dst;
    dst.width = dst_w;
    dst.height = dst_h;
    dst.rgb.assign((size_t)dst_w * dst_h * 3, 0.f);
    const float sx = (float)src.width / dst_w, sy = (float)src.height / dst_h;
    for (int dy = 0; dy < dst_h; dy++) {
        const float y0 = dy * sy, y1 = (dy + 1) * sy;
        const int iy0 = (int)y0, iy1 = std::min((int)std::ceil(y1), src.height);
        for (int dx = 0; dx < dst_w; dx++) {
            const float x0 = dx * sx, x1 = (dx + 1) * sx;
            const int ix0 = (int)x0, ix1 = std::min((int)std::ceil(x1), src.width);
            float acc[3] = {0.f, 0.f, 0.f}, area = 0.f;
            for (int iy = iy0; iy < iy1; iy++) {
                const float wy = std::min((float)(iy + 1), y1) - std::max((float)iy, y0);
                for (int ix = ix0; ix < ix1; ix++) {
                    const float w = wy * (std::min((float)(ix + 1), x1) - std::max((float)ix, x0));
                    const float *p = &src.rgb[((size_t)iy * src.width + ix) * 3];
                    acc[0] += p[0] * w;
                    acc[1] += p[1] * w;
                    acc[2] += p[2] * w;
                    area += w;
                }
            }
            float *o = &dst.rgb[((size_t)dy * dst_w + dx) * 3];
            const float inv = area > 0.f ? 1.f / area : 0.f;
            o[0] = acc[0] * inv;
            o[1] = acc[1] * inv;
            o[2] = acc[2] * inv;
        }
    }
    return dst;
}

Image undistort(const Image &src, float fx, float fy, float cx, float cy, float k1, float k2, float p1, float p2,
                float k3) {
    Image out;
    out.width = src.width;
    out.height = src.height;
    out.rgb.assign(src.rgb.size(), 0.f);
    for (int y = 0; y < src.height; y++)
        for (int x = 0; x < src.width; x++) {
            const float u = (x - cx) / fx, v = (y - cy) / fy;
            const float r2 = u * u + v * v, rad = 1.f + r2 * (k1 + r2 * (k2 + r2 * k3));
            const float ud = u * rad + 2.f * p1 * u * v + p2 * (r2 + 2.f * u * u);
            const float vd = v * rad + p1 * (r2 + 2.f * v * v) + 2.f * p2 * u * v;
            const float sx = ud * fx + cx, sy = vd * fy + cy;
            const int x0 = (int)std::floor(sx), y0 = (int)std::floor(sy);
            if (x0 < 0 || y0 < 0 || x0 + 1 >= src.width || y0 + 1 >= src.height) continue;
            const float ax = sx - x0, ay = sy - y0;
            float *o = &out.rgb[((size_t)y * src.width + x) * 3];
            for (int c = 0; c < 3; c++) {
                const float a = src.rgb[((size_t)y0 * src.width + x0) * 3 + c];
                const float b = src.rgb[((size_t)y0 * src.width + x0 + 1) * 3 + c];
                const float d = src.rgb[((size_t)(y0 + 1) * src.width + x0) * 3 + c];
                const float e = src.rgb[((size_t)(y0 + 1) * src.width + x0 + 1) * 3 + c];
                o[c] = (a * (1 - ax) + b * ax) * (1 - ay) + (d * (1 - ax) + e * ax) * ay;
            }
        }
    return out;
}

// ===========================================================================
// JSON (enough for transforms.json and the Polycam camera files)
// ===========================================================================

namespace {

struct Json {
    enum Kind { Null, Bool, Num, Str, Arr, Obj } kind = Null;
    double num = 0;
    bool b = false;
    std::string str;
    std::vector<Json> arr;
    std::map<std::string, Json> obj;

    bool has(const std::string &k) const { return kind == Obj && obj.count(k); }
    const Json &operator[](const std::string &k) const {
        static const Json null;
        auto it = obj.find(k);
        return it == obj.end() ? null : it->second;
    }
    double number(const std::string &k, double dflt) const {
        if (!has(k)) return dflt;
        const Json &v = (*this)[k];
        return v.kind == Num ? v.num : dflt;
    }
    std::string string(const std::string &k, const std::string &dflt) const {
        if (!has(k)) return dflt;
        const Json &v = (*this)[k];
        return v.kind == Str ? v.str : dflt;
    }
};

struct JsonParser {
    const std::string &s;
    size_t i = 0;
    explicit JsonParser(const std::string &src) : s(src) {}
    [[noreturn]] void fail(const char *what) { throw std::runtime_error(std::string("json: ") + what); }
    void ws() {
        while (i < s.size() && std::isspace((unsigned char)s[i])) i++;
    }
    Json value() {
        ws();
        if (i >= s.size()) fail("unexpected end");
        const char c = s[i];
        Json v;
        if (c == '{') {
            v.kind = Json::Obj;
            i++;
            ws();
            if (i < s.size() && s[i] == '}') { i++; return v; }
            for (;;) {
                ws();
                if (i >= s.size() || s[i] != '"') fail("expected a key");
                std::string k = string_lit();
                ws();
                if (i >= s.size() || s[i] != ':') fail("expected ':'");
                i++;
                v.obj[k] = value();
                ws();
                if (i < s.size() && s[i] == ',') { i++; continue; }
                if (i < s.size() && s[i] == '}') { i++; return v; }
                fail("expected ',' or '}'");
            }
        }
        if (c == '[') {
            v.kind = Json::Arr;
            i++;
            ws();
            if (i < s.size() && s[i] == ']') { i++; return v; }
            for (;;) {
                v.arr.push_back(value());
                ws();
                if (i < s.size() && s[i] == ',') { i++; continue; }
                if (i < s.size() && s[i] == ']') { i++; return v; }
                fail("expected ',' or ']'");
            }
        }
        if (c == '"') {
            v.kind = Json::Str;
            v.str = string_lit();
            return v;
        }
        if (s.compare(i, 4, "true") == 0) { i += 4; v.kind = Json::Bool; v.b = true; return v; }
        if (s.compare(i, 5, "false") == 0) { i += 5; v.kind = Json::Bool; return v; }
        if (s.compare(i, 4, "null") == 0) { i += 4; return v; }
        if (c == '-' || std::isdigit((unsigned char)c)) {
            const char *b = s.c_str() + i;
            char *e = nullptr;
            v.num = std::strtod(b, &e);
            if (e == b) fail("bad number");
            i += (size_t)(e - b);
            v.kind = Json::Num;
            return v;
        }
        fail("unexpected character");
    }
    std::string string_lit() {
        std::string out;
        i++;   // opening quote
        while (i < s.size() && s[i] != '"') {
            char c = s[i++];
            if (c != '\\') { out += c; continue; }
            if (i >= s.size()) fail("bad escape");
            c = s[i++];
            switch (c) {
                case 'n': out += '\n'; break;
                case 't': out += '\t'; break;
                case 'r': out += '\r'; break;
                case 'b': out += '\b'; break;
                case 'f': out += '\f'; break;
                case 'u': {
                    if (i + 4 > s.size()) fail("bad \\u escape");
                    const unsigned cp = (unsigned)std::stoul(s.substr(i, 4), nullptr, 16);
                    i += 4;
                    if (cp < 0x80) out += (char)cp;
                    else if (cp < 0x800) { out += (char)(0xC0 | (cp >> 6)); out += (char)(0x80 | (cp & 63)); }
                    else {
                        out += (char)(0xE0 | (cp >> 12));
                        out += (char)(0x80 | ((cp >> 6) & 63));
                        out += (char)(0x80 | (cp & 63));
                    }
                    break;
                }
                default: out += c;
            }
        }
        if (i >= s.size()) fail("unterminated string");
        i++;
        return out;
    }
};

Json read_json(const std::string &path) {
    const std::vector<uint8_t> b = read_file(path);
    const std::string s(b.begin(), b.end());
    JsonParser p(s);
    return p.value();
}

std::string resolve_image(const std::string &path) {
    if (fs::exists(path)) return path;
    for (const char *ext : {".png", ".jpg", ".jpeg", ".JPG"})
        if (fs::exists(path + ext)) return path + ext;
    return path;
}

void identity(float m[16]) {
    for (int k = 0; k < 16; k++) m[k] = (k % 5 == 0) ? 1.f : 0.f;
}

}  // namespace

// ===========================================================================
// Point clouds
// ===========================================================================

void read_ply_points(const std::string &path, std::vector<float> &xyz, std::vector<uint8_t> &rgb) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("cannot open PLY " + path);
    std::string line;
    std::getline(f, line);
    if (line.rfind("ply", 0) != 0) throw std::runtime_error("not a PLY file: " + path);
    std::string format;
    long long n = 0;
    bool in_vertex = false;
    struct Prop { std::string name, type; };
    std::vector<Prop> props;
    while (std::getline(f, line)) {
        if (!line.empty() && line.back() == '\r') line.pop_back();
        std::istringstream ss(line);
        std::string w;
        ss >> w;
        if (w == "format") ss >> format;
        else if (w == "element") {
            std::string name;
            ss >> name;
            in_vertex = name == "vertex";
            if (in_vertex) ss >> n;
        } else if (w == "property" && in_vertex) {
            Prop p;
            ss >> p.type;
            if (p.type == "list") throw std::runtime_error("PLY: list properties on vertices are not supported");
            ss >> p.name;
            props.push_back(p);
        } else if (w == "end_header") {
            break;
        }
    }
    auto size_of = [](const std::string &t) -> int {
        if (t == "char" || t == "uchar" || t == "int8" || t == "uint8") return 1;
        if (t == "short" || t == "ushort" || t == "int16" || t == "uint16") return 2;
        if (t == "int" || t == "uint" || t == "float" || t == "int32" || t == "uint32" || t == "float32") return 4;
        if (t == "double" || t == "float64") return 8;
        throw std::runtime_error("PLY: unknown property type " + t);
    };
    int ix = -1, iy = -1, iz = -1, ir = -1, ig = -1, ib = -1;
    for (int k = 0; k < (int)props.size(); k++) {
        const std::string &nm = props[k].name;
        if (nm == "x") ix = k; else if (nm == "y") iy = k; else if (nm == "z") iz = k;
        else if (nm == "red" || nm == "r") ir = k; else if (nm == "green" || nm == "g") ig = k;
        else if (nm == "blue" || nm == "b") ib = k;
    }
    if (ix < 0 || iy < 0 || iz < 0) throw std::runtime_error("PLY: no x/y/z properties in " + path);
    xyz.assign(3 * (size_t)n, 0.f);
    rgb.assign(3 * (size_t)n, 255);
    std::vector<double> vals(props.size());
    const bool ascii = format == "ascii";
    if (!ascii && format != "binary_little_endian") throw std::runtime_error("PLY: unsupported format " + format);
    for (long long i = 0; i < n; i++) {
        for (size_t k = 0; k < props.size(); k++) {
            const std::string &t = props[k].type;
            if (ascii) {
                f >> vals[k];
                continue;
            }
            unsigned char b[8];
            const int sz = size_of(t);
            f.read(reinterpret_cast<char *>(b), sz);
            if (t == "float" || t == "float32") { float v; std::memcpy(&v, b, 4); vals[k] = v; }
            else if (t == "double" || t == "float64") { double v; std::memcpy(&v, b, 8); vals[k] = v; }
            else if (t == "uchar" || t == "uint8") vals[k] = b[0];
            else if (t == "char" || t == "int8") vals[k] = (int8_t)b[0];
            else if (t == "ushort" || t == "uint16") { uint16_t v; std::memcpy(&v, b, 2); vals[k] = v; }
            else if (t == "short" || t == "int16") { int16_t v; std::memcpy(&v, b, 2); vals[k] = v; }
            else if (t == "uint" || t == "uint32") { uint32_t v; std::memcpy(&v, b, 4); vals[k] = v; }
            else { int32_t v; std::memcpy(&v, b, 4); vals[k] = v; }
        }
        if (!f) throw std::runtime_error("PLY: truncated " + path);
        xyz[3 * i] = (float)vals[ix];
        xyz[3 * i + 1] = (float)vals[iy];
        xyz[3 * i + 2] = (float)vals[iz];
        if (ir >= 0 && ig >= 0 && ib >= 0) {
            rgb[3 * i] = (uint8_t)std::min(std::max(vals[ir], 0.0), 255.0);
            rgb[3 * i + 1] = (uint8_t)std::min(std::max(vals[ig], 0.0), 255.0);
            rgb[3 * i + 2] = (uint8_t)std::min(std::max(vals[ib], 0.0), 255.0);
        }
    }
}

// ===========================================================================
// COLMAP (sparse model, binary or text)
// ===========================================================================

namespace {

struct ColmapCam {
    int width = 0, height = 0;
    float fx = 0, fy = 0, cx = 0, cy = 0, k1 = 0, k2 = 0, p1 = 0, p2 = 0;
};

// camera model id -> (name, parameter count)
void colmap_params(int model, const std::vector<double> &p, ColmapCam &c) {
    auto need = [&](size_t k) {
        if (p.size() < k) throw std::runtime_error("COLMAP: too few camera parameters");
    };
    switch (model) {
        case 0: need(3); c.fx = c.fy = (float)p[0]; c.cx = (float)p[1]; c.cy = (float)p[2]; break;   // SIMPLE_PINHOLE
        case 1: need(4); c.fx = (float)p[0]; c.fy = (float)p[1]; c.cx = (float)p[2]; c.cy = (float)p[3]; break;
        case 2: need(4); c.fx = c.fy = (float)p[0]; c.cx = (float)p[1]; c.cy = (float)p[2]; c.k1 = (float)p[3]; break;
        case 3: need(5); c.fx = c.fy = (float)p[0]; c.cx = (float)p[1]; c.cy = (float)p[2];
                c.k1 = (float)p[3]; c.k2 = (float)p[4]; break;                                            // RADIAL
        case 4: need(8); c.fx = (float)p[0]; c.fy = (float)p[1]; c.cx = (float)p[2]; c.cy = (float)p[3];
                c.k1 = (float)p[4]; c.k2 = (float)p[5]; c.p1 = (float)p[6]; c.p2 = (float)p[7]; break;   // OPENCV
        default: throw std::runtime_error("unsupported COLMAP camera model " + std::to_string(model));
    }
}

int colmap_model_id(const std::string &name) {
    static const char *names[] = {"SIMPLE_PINHOLE", "PINHOLE", "SIMPLE_RADIAL", "RADIAL", "OPENCV"};
    for (int k = 0; k < 5; k++)
        if (name == names[k]) return k;
    throw std::runtime_error("unsupported COLMAP camera model " + name);
}

int colmap_param_count(int model) {
    static const int n[] = {3, 4, 4, 5, 8};
    return (model >= 0 && model < 5) ? n[model] : -1;
}

struct ColmapImg {
    uint32_t cam;
    double q[4], t[3];
    std::string name;
};

template <class T> T rd(std::ifstream &f) {
    T v;
    f.read(reinterpret_cast<char *>(&v), sizeof(T));
    if (!f) throw std::runtime_error("COLMAP: truncated file");
    return v;
}

// world-to-camera (q, t) -> camera-to-world with OpenGL axes (columns 1 and
// 2 negated), as the reference's loader builds it
void colmap_c2w(const double qin[4], const double t[3], float out[16]) {
    double w = qin[0], x = qin[1], y = qin[2], z = qin[3];
    const double n = std::sqrt(w * w + x * x + y * y + z * z);
    w /= n; x /= n; y /= n; z /= n;
    const float R[9] = {(float)(1 - 2 * (y * y + z * z)), (float)(2 * (x * y - w * z)), (float)(2 * (x * z + w * y)),
                        (float)(2 * (x * y + w * z)), (float)(1 - 2 * (x * x + z * z)), (float)(2 * (y * z - w * x)),
                        (float)(2 * (x * z - w * y)), (float)(2 * (y * z + w * x)), (float)(1 - 2 * (x * x + y * y))};
    const float Ri[9] = {R[0], R[3], R[6], R[1], R[4], R[7], R[2], R[5], R[8]};
    float T[3];
    for (int r = 0; r < 3; r++)
        T[r] = -(Ri[3 * r] * (float)t[0] + Ri[3 * r + 1] * (float)t[1] + Ri[3 * r + 2] * (float)t[2]);
    for (int r = 0; r < 3; r++) {
        out[4 * r + 0] = Ri[3 * r];
        out[4 * r + 1] = -Ri[3 * r + 1];
        out[4 * r + 2] = -Ri[3 * r + 2];
        out[4 * r + 3] = T[r];
    }
    out[12] = out[13] = out[14] = 0.f;
    out[15] = 1.f;
}

void load_colmap(const std::string &root, const std::string &image_dir_in, LoadedScene &sc) {
    const fs::path r(root);
    std::string sparse;
    for (const fs::path &d : {r, r / "sparse" / "0", r / "sparse"})
        if (fs::exists(d / "cameras.bin") || fs::exists(d / "cameras.txt")) { sparse = d.string(); break; }
    if (sparse.empty()) throw std::runtime_error("COLMAP: no cameras.bin / cameras.txt under " + root);
    const std::string image_dir = !image_dir_in.empty() ? image_dir_in
                                  : fs::exists(r / "images") ? (r / "images").string()
                                                             : root;
    std::unordered_map<uint32_t, ColmapCam> cams;
    std::vector<ColmapImg> imgs;
    const fs::path sp(sparse);
    if (fs::exists(sp / "cameras.bin")) {
        std::ifstream f((sp / "cameras.bin").string(), std::ios::binary);
        const uint64_t n = rd<uint64_t>(f);
        for (uint64_t i = 0; i < n; i++) {
            const uint32_t id = rd<uint32_t>(f);
            const int model = rd<int32_t>(f);
            ColmapCam c;
            c.width = (int)rd<uint64_t>(f);
            c.height = (int)rd<uint64_t>(f);
            const int np = colmap_param_count(model);
            if (np < 0) throw std::runtime_error("unsupported COLMAP camera model " + std::to_string(model));
            std::vector<double> p(np);
            for (auto &v : p) v = rd<double>(f);
            colmap_params(model, p, c);
            cams[id] = c;
        }
        std::ifstream g((sp / "images.bin").string(), std::ios::binary);
        const uint64_t m = rd<uint64_t>(g);
        for (uint64_t i = 0; i < m; i++) {
            ColmapImg im;
            rd<uint32_t>(g);
            for (auto &v : im.q) v = rd<double>(g);
            for (auto &v : im.t) v = rd<double>(g);
            im.cam = rd<uint32_t>(g);
            char ch;
            while (g.get(ch) && ch != '\0') im.name += ch;
            const uint64_t np2 = rd<uint64_t>(g);
            g.seekg((std::streamoff)(np2 * 24), std::ios::cur);
            imgs.push_back(im);
        }
    } else {
        std::ifstream f((sp / "cameras.txt").string());
        std::string line;
        while (std::getline(f, line)) {
            if (line.empty() || line[0] == '#') continue;
            std::istringstream ss(line);
            uint32_t id;
            std::string model;
            ColmapCam c;
            ss >> id >> model >> c.width >> c.height;
            std::vector<double> p;
            double v;
            while (ss >> v) p.push_back(v);
            colmap_params(colmap_model_id(model), p, c);
            cams[id] = c;
        }
        std::ifstream g((sp / "images.txt").string());
        bool points_line = false;
        while (std::getline(g, line)) {
            if (line.empty() || line[0] == '#') continue;
            if (points_line) { points_line = false; continue; }
            std::istringstream ss(line);
            ColmapImg im;
            uint32_t id;
            ss >> id >> im.q[0] >> im.q[1] >> im.q[2] >> im.q[3] >> im.t[0] >> im.t[1] >> im.t[2] >> im.cam >> im.name;
            imgs.push_back(im);
            points_line = true;
        }
    }
    std::sort(imgs.begin(), imgs.end(), [](const ColmapImg &a, const ColmapImg &b) { return a.name < b.name; });
    for (auto &im : imgs) {
        auto it = cams.find(im.cam);
        if (it == cams.end()) continue;
        const ColmapCam &c = it->second;
        LoadedCamera lc;
        lc.width = c.width; lc.height = c.height;
        lc.fx = c.fx; lc.fy = c.fy; lc.cx = c.cx; lc.cy = c.cy;
        lc.k1 = c.k1; lc.k2 = c.k2; lc.p1 = c.p1; lc.p2 = c.p2;
        lc.path = (fs::path(image_dir) / im.name).string();
        lc.relative_name = im.name;
        colmap_c2w(im.q, im.t, lc.c2w);
        sc.cameras.push_back(lc);
    }
    // seed points
    if (fs::exists(sp / "points3D.bin")) {
        std::ifstream f((sp / "points3D.bin").string(), std::ios::binary);
        const uint64_t n = rd<uint64_t>(f);
        sc.xyz.reserve(3 * n);
        sc.rgb.reserve(3 * n);
        for (uint64_t i = 0; i < n; i++) {
            rd<uint64_t>(f);
            for (int k = 0; k < 3; k++) sc.xyz.push_back((float)rd<double>(f));
            for (int k = 0; k < 3; k++) sc.rgb.push_back(rd<uint8_t>(f));
            rd<double>(f);
            const uint64_t tl = rd<uint64_t>(f);
            f.seekg((std::streamoff)(tl * 8), std::ios::cur);
        }
    } else if (fs::exists(sp / "points3D.txt")) {
        std::ifstream f((sp / "points3D.txt").string());
        std::string line;
        while (std::getline(f, line)) {
            if (line.empty() || line[0] == '#') continue;
            std::istringstream ss(line);
            uint64_t id;
            double x, y, z;
            int cr, cg, cb;
            ss >> id >> x >> y >> z >> cr >> cg >> cb;
            sc.xyz.insert(sc.xyz.end(), {(float)x, (float)y, (float)z});
            sc.rgb.insert(sc.rgb.end(), {(uint8_t)cr, (uint8_t)cg, (uint8_t)cb});
        }
    } else if (fs::exists(sp / "points3D.ply")) {
        read_ply_points((sp / "points3D.ply").string(), sc.xyz, sc.rgb);
    }
}

// ===========================================================================
// Nerfstudio (transforms.json) and Polycam
// ===========================================================================

void load_nerfstudio(const std::string &root, LoadedScene &sc) {
    const fs::path r(root);
    const Json j = read_json((r / "transforms.json").string());
    const int gw = (int)j.number("w", 0), gh = (int)j.number("h", 0);
    const float gfx = (float)j.number("fl_x", 0), gfy = (float)j.number("fl_y", 0);
    const float gcx = (float)j.number("cx", 0), gcy = (float)j.number("cy", 0);
    const float gk1 = (float)j.number("k1", 0), gk2 = (float)j.number("k2", 0), gk3 = (float)j.number("k3", 0);
    const float gp1 = (float)j.number("p1", 0), gp2 = (float)j.number("p2", 0);
    const Json &frames = j["frames"];
    if (frames.kind != Json::Arr) throw std::runtime_error("transforms.json has no frames");
    for (const Json &fr : frames.arr) {
        LoadedCamera c;
        c.width = (int)fr.number("w", gw);
        c.height = (int)fr.number("h", gh);
        c.fx = (float)fr.number("fl_x", gfx); c.fy = (float)fr.number("fl_y", gfy);
        c.cx = (float)fr.number("cx", gcx); c.cy = (float)fr.number("cy", gcy);
        c.k1 = (float)fr.number("k1", gk1); c.k2 = (float)fr.number("k2", gk2); c.k3 = (float)fr.number("k3", gk3);
        c.p1 = (float)fr.number("p1", gp1); c.p2 = (float)fr.number("p2", gp2);
        const std::string fp = fr.string("file_path", "");
        c.path = (!fp.empty() && (fp[0] == '/' || fp[0] == '.')) ? resolve_image(fp) : resolve_image((r / fp).string());
        // no relative_name: the reference's loadNerfstudio leaves relativeName
        // empty, so training masks (--mask-dir) apply to COLMAP datasets only
        const Json &tm = fr["transform_matrix"];
        if (tm.kind != Json::Arr || tm.arr.size() < 4) throw std::runtime_error("frame without transform_matrix");
        for (int a = 0; a < 4; a++)
            for (int b = 0; b < 4; b++) c.c2w[4 * a + b] = (float)tm.arr[a].arr.at(b).num;
        sc.cameras.push_back(c);
    }
    std::sort(sc.cameras.begin(), sc.cameras.end(),
              [](const LoadedCamera &a, const LoadedCamera &b) { return a.path < b.path; });
    std::string ply;
    if (j.has("ply_file_path")) {
        ply = j.string("ply_file_path", "");
        if (!ply.empty() && ply[0] != '/') ply = (r / ply).string();
    }
    if (ply.empty() || !fs::exists(ply)) {
        ply.clear();
        for (const char *p : {"sparse/0/points3D.ply", "points3D.ply"})
            if (fs::exists(r / p)) { ply = (r / p).string(); break; }
    }
    if (!ply.empty()) read_ply_points(ply, sc.xyz, sc.rgb);
}

void load_polycam(const std::string &root, LoadedScene &sc) {
    const fs::path r(root);
    const fs::path kdir = r / "keyframes" / "corrected_cameras", idir = r / "keyframes" / "corrected_images";
    auto frame_camera = [](const Json &fr, LoadedCamera &c) {
        c.width = (int)fr.number("width", 0);
        c.height = (int)fr.number("height", 0);
        c.fx = (float)fr.number("fx", 0); c.fy = (float)fr.number("fy", 0);
        c.cx = (float)fr.number("cx", c.width / 2.0); c.cy = (float)fr.number("cy", c.height / 2.0);
    };
    if (fs::exists(kdir)) {
        std::vector<fs::path> files;
        for (auto &e : fs::directory_iterator(kdir))
            if (e.path().extension() == ".json") files.push_back(e.path());
        std::sort(files.begin(), files.end());
        for (auto &p : files) {
            const Json j = read_json(p.string());
            LoadedCamera c;
            frame_camera(j, c);
            float R[9];
            for (int a = 0; a < 3; a++)
                for (int b = 0; b < 3; b++)
                    R[3 * a + b] = (float)j.number("R_" + std::to_string(a) + std::to_string(b), 0);
            const float T[3] = {(float)j.number("t_20", 0), (float)j.number("t_21", 0), (float)j.number("t_22", 0)};
            // camera-to-world with the Y and Z rows flipped (OpenGL axes)
            for (int b = 0; b < 3; b++) {
                c.c2w[b] = R[b];
                c.c2w[4 + b] = -R[3 + b];
                c.c2w[8 + b] = -R[6 + b];
            }
            c.c2w[3] = T[0]; c.c2w[7] = -T[1]; c.c2w[11] = -T[2];
            c.c2w[12] = c.c2w[13] = c.c2w[14] = 0.f;
            c.c2w[15] = 1.f;
            const std::string stem = p.stem().string();
            c.path = (idir / (stem + ".png")).string();
            for (const char *ext : {".png", ".jpg", ".jpeg", ".JPG"})
                if (fs::exists(idir / (stem + ext))) { c.path = (idir / (stem + ext)).string(); break; }
            sc.cameras.push_back(c);
        }
    } else {
        const Json j = read_json((r / "cameras.json").string());
        const Json &frames = j.has("frames") ? j["frames"] : j;
        if (frames.kind != Json::Arr) throw std::runtime_error("cameras.json has no frames");
        for (const Json &fr : frames.arr) {
            LoadedCamera c;
            frame_camera(fr, c);
            identity(c.c2w);
            const Json &tm = fr["transform_matrix"];
            if (tm.kind == Json::Arr && tm.arr.size() >= 4)
                for (int a = 0; a < 4; a++)
                    for (int b = 0; b < 4; b++) c.c2w[4 * a + b] = (float)tm.arr[a].arr.at(b).num;
            c.path = fr.string("file_path", "");
            if (!c.path.empty() && c.path[0] != '/') c.path = (r / c.path).string();
            // no relative_name: the reference's loadPolycam leaves it empty (masks are COLMAP's)
            sc.cameras.push_back(c);
        }
    }
    for (const char *p : {"keyframes/point_cloud.ply", "point_cloud.ply", "sparse.ply"})
        if (fs::exists(r / p)) { read_ply_points((r / p).string(), sc.xyz, sc.rgb); break; }
}

}  // namespace

LoadedScene load_scene(const std::string &root, const std::string &colmap_image_dir) {
    const fs::path r(root);
    LoadedScene sc;
    if (fs::exists(r / "transforms.json")) {
        load_nerfstudio(root, sc);
    } else if (fs::exists(r / "cameras.bin") || fs::exists(r / "sparse" / "0" / "cameras.bin") ||
               fs::exists(r / "cameras.txt") || fs::exists(r / "sparse" / "0" / "cameras.txt")) {
        load_colmap(root, colmap_image_dir, sc);
    } else if (fs::exists(r / "keyframes" / "corrected_cameras") || fs::exists(r / "cameras.json")) {
        load_polycam(root, sc);
    } else {
        throw std::runtime_error("unrecognized dataset layout in " + root +
                                 " (COLMAP cameras.bin/txt, Nerfstudio transforms.json, Polycam keyframes/)");
    }
    if (sc.cameras.empty()) throw std::runtime_error("dataset has no cameras: " + root);
    return sc;
}

}  // namespace io
}  // namespace msplat
