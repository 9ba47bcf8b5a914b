// Baseline JPEG encoder restating crates/codecs/mjpeg/src/encoder.rs, with two
// stream-generation options the reference does not have: the standard Annex K
// Huffman tables (ITU-T T.81 K.3) and a restart interval (DRI + RSTn markers).
// Compiled with -ffp-contract=off: the forward DCT (transform.rs:111-138) must
// round every binary64 multiply and add as Rust does, for byte-identical output.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "common.h"
#include "encode.h"
#include "tables.h"

namespace mmr {

namespace {

const int kZigzag[64] = MMR_ZIGZAG_INIT;
const double kIdct[64] = MMR_IDCT_MATRIX_INIT;

// tables.rs:7-17 (natural order, Annex K.1 / K.2)
const uint8_t kLumaQ[64] = {16, 11, 10, 16, 24,  40,  51,  61,  12, 12, 14, 19, 26,  58,  60,  55,
                            14, 13, 16, 24, 40,  57,  69,  56,  14, 17, 22, 29, 51,  87,  80,  62,
                            18, 22, 37, 56, 68,  109, 103, 77,  24, 35, 55, 64, 81,  104, 113, 92,
                            49, 64, 78, 87, 103, 121, 120, 101, 72, 92, 95, 98, 112, 100, 103, 99};
const uint8_t kChromaQ[64] = {17, 18, 24, 47, 99, 99, 99, 99, 18, 21, 26, 66, 99, 99, 99, 99,
                              24, 26, 56, 99, 99, 99, 99, 99, 47, 66, 99, 99, 99, 99, 99, 99,
                              99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99,
                              99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99};

// ITU-T T.81 Annex K.3 typical Huffman tables (counts per length 1..16, then symbols).
const uint8_t kDcLumaBits[16] = {0, 1, 5, 1, 1, 1, 1, 1, 1, 0, 0, 0, 0, 0, 0, 0};
const uint8_t kDcChromaBits[16] = {0, 3, 1, 1, 1, 1, 1, 1, 1, 1, 1, 0, 0, 0, 0, 0};
const uint8_t kDcVals[12] = {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11};
const uint8_t kAcLumaBits[16] = {0, 2, 1, 3, 3, 2, 4, 3, 5, 5, 4, 4, 0, 0, 1, 0x7d};
const uint8_t kAcLumaVals[162] = {
    0x01, 0x02, 0x03, 0x00, 0x04, 0x11, 0x05, 0x12, 0x21, 0x31, 0x41, 0x06, 0x13, 0x51, 0x61, 0x07, 0x22, 0x71,
    0x14, 0x32, 0x81, 0x91, 0xa1, 0x08, 0x23, 0x42, 0xb1, 0xc1, 0x15, 0x52, 0xd1, 0xf0, 0x24, 0x33, 0x62, 0x72,
    0x82, 0x09, 0x0a, 0x16, 0x17, 0x18, 0x19, 0x1a, 0x25, 0x26, 0x27, 0x28, 0x29, 0x2a, 0x34, 0x35, 0x36, 0x37,
    0x38, 0x39, 0x3a, 0x43, 0x44, 0x45, 0x46, 0x47, 0x48, 0x49, 0x4a, 0x53, 0x54, 0x55, 0x56, 0x57, 0x58, 0x59,
    0x5a, 0x63, 0x64, 0x65, 0x66, 0x67, 0x68, 0x69, 0x6a, 0x73, 0x74, 0x75, 0x76, 0x77, 0x78, 0x79, 0x7a, 0x83,
    0x84, 0x85, 0x86, 0x87, 0x88, 0x89, 0x8a, 0x92, 0x93, 0x94, 0x95, 0x96, 0x97, 0x98, 0x99, 0x9a, 0xa2, 0xa3,
    0xa4, 0xa5, 0xa6, 0xa7, 0xa8, 0xa9, 0xaa, 0xb2, 0xb3, 0xb4, 0xb5, 0xb6, 0xb7, 0xb8, 0xb9, 0xba, 0xc2, 0xc3,
    0xc4, 0xc5, 0xc6, 0xc7, 0xc8, 0xc9, 0xca, 0xd2, 0xd3, 0xd4, 0xd5, 0xd6, 0xd7, 0xd8, 0xd9, 0xda, 0xe1, 0xe2,
    0xe3, 0xe4, 0xe5, 0xe6, 0xe7, 0xe8, 0xe9, 0xea, 0xf1, 0xf2, 0xf3, 0xf4, 0xf5, 0xf6, 0xf7, 0xf8, 0xf9, 0xfa};
const uint8_t kAcChromaBits[16] = {0, 2, 1, 2, 4, 4, 3, 4, 7, 5, 4, 4, 0, 1, 2, 0x77};
const uint8_t kAcChromaVals[162] = {
    0x00, 0x01, 0x02, 0x03, 0x11, 0x04, 0x05, 0x21, 0x31, 0x06, 0x12, 0x41, 0x51, 0x07, 0x61, 0x71, 0x13, 0x22,
    0x32, 0x81, 0x08, 0x14, 0x42, 0x91, 0xa1, 0xb1, 0xc1, 0x09, 0x23, 0x33, 0x52, 0xf0, 0x15, 0x62, 0x72, 0xd1,
    0x0a, 0x16, 0x24, 0x34, 0xe1, 0x25, 0xf1, 0x17, 0x18, 0x19, 0x1a, 0x26, 0x27, 0x28, 0x29, 0x2a, 0x35, 0x36,
    0x37, 0x38, 0x39, 0x3a, 0x43, 0x44, 0x45, 0x46, 0x47, 0x48, 0x49, 0x4a, 0x53, 0x54, 0x55, 0x56, 0x57, 0x58,
    0x59, 0x5a, 0x63, 0x64, 0x65, 0x66, 0x67, 0x68, 0x69, 0x6a, 0x73, 0x74, 0x75, 0x76, 0x77, 0x78, 0x79, 0x7a,
    0x82, 0x83, 0x84, 0x85, 0x86, 0x87, 0x88, 0x89, 0x8a, 0x92, 0x93, 0x94, 0x95, 0x96, 0x97, 0x98, 0x99, 0x9a,
    0xa2, 0xa3, 0xa4, 0xa5, 0xa6, 0xa7, 0xa8, 0xa9, 0xaa, 0xb2, 0xb3, 0xb4, 0xb5, 0xb6, 0xb7, 0xb8, 0xb9, 0xba,
    0xc2, 0xc3, 0xc4, 0xc5, 0xc6, 0xc7, 0xc8, 0xc9, 0xca, 0xd2, 0xd3, 0xd4, 0xd5, 0xd6, 0xd7, 0xd8, 0xd9, 0xda,
    0xe2, 0xe3, 0xe4, 0xe5, 0xe6, 0xe7, 0xe8, 0xe9, 0xea, 0xf2, 0xf3, 0xf4, 0xf5, 0xf6, 0xf7, 0xf8, 0xf9, 0xfa};

struct Table {
    uint8_t cls, id;
    uint8_t counts[16];
    std::vector<uint8_t> symbols;
};

// encoder.rs:230-256 simple tables
Table simple_dc() {
    Table t{0, 0, {0}, {}};
    t.counts[3] = 12;
    for (int s = 0; s <= 11; s++) t.symbols.push_back((uint8_t)s);
    return t;
}
Table simple_ac() {
    Table t{1, 0, {0}, {}};
    t.counts[7] = 162;
    t.symbols = {0x00, 0xf0};
    for (int run = 0; run <= 15; run++)
        for (int size = 1; size <= 10; size++) t.symbols.push_back((uint8_t)((run << 4) | size));
    return t;
}
Table annex(uint8_t cls, uint8_t id, const uint8_t *bits, const uint8_t *vals, size_t n) {
    Table t{cls, id, {0}, std::vector<uint8_t>(vals, vals + n)};
    memcpy(t.counts, bits, 16);
    return t;
}

// encoder.rs:427-473 HuffmanEncoder::new
bool huffman_encoder(const Table &t, HuffCode codes[256]) {
    for (int i = 0; i < 256; i++) codes[i] = {0, 0, false};
    uint32_t code = 0;
    size_t si = 0;
    for (int li = 0; li < 16; li++) {
        uint32_t length = (uint32_t)li + 1;
        if (code + t.counts[li] > (1u << length)) return false;
        for (int k = 0; k < t.counts[li]; k++) {
            if (si >= t.symbols.size()) return false;
            codes[t.symbols[si]] = {(uint16_t)code, (uint8_t)length, true};
            si++;
            code++;
        }
        code <<= 1;
    }
    return si == t.symbols.size();
}

// encoder.rs:495-543 EntropyWriter
struct Writer {
    std::vector<uint8_t> data;
    uint8_t cur = 0;
    uint8_t nbits = 0;
    void bits(uint32_t value, int count) {
        for (int i = count - 1; i >= 0; i--) {
            cur = (uint8_t)((cur << 1) | ((value >> i) & 1));
            if (++nbits == 8) push();
        }
    }
    void push() {
        data.push_back(cur);
        if (cur == 0xff) data.push_back(0);
        cur = 0;
        nbits = 0;
    }
    void pad() {
        while (nbits != 0) bits(1, 1);
    }
};

void segment(std::vector<uint8_t> &out, uint8_t marker, const std::vector<uint8_t> &payload) {
    size_t length = payload.size() + 2;
    out.push_back(0xff);
    out.push_back(marker);
    out.push_back((uint8_t)(length >> 8));
    out.push_back((uint8_t)length);
    out.insert(out.end(), payload.begin(), payload.end());
}

// encoder.rs:217-228 scale_quantization
void scale_quant(const uint8_t *base, uint8_t q, uint8_t *out) {
    uint32_t quality = q;
    uint32_t scale = quality < 50 ? 5000 / quality : 200 - quality * 2;
    for (int i = 0; i < 64; i++) {
        uint32_t v = (base[i] * scale + 50) / 100;
        out[i] = (uint8_t)std::min<uint32_t>(std::max<uint32_t>(v, 1), 255);
    }
}

// transform.rs:111-138 forward_dct_quantize
void fdct_quantize(const uint8_t s[64], const uint8_t q[64], int32_t out[64]) {
    double t[64];
    for (int i = 0; i < 64; i++) t[i] = 0.0;
    for (int y = 0; y < 8; y++)
        for (int u = 0; u < 8; u++)
            for (int x = 0; x < 8; x++) t[y * 8 + u] += kIdct[x * 8 + u] * ((double)s[y * 8 + x] - 128.0);
    for (int v = 0; v < 8; v++)
        for (int u = 0; u < 8; u++) {
            double value = 0.0;
            for (int y = 0; y < 8; y++) value += kIdct[y * 8 + v] * t[y * 8 + u];
            out[v * 8 + u] = (int32_t)round(value / (double)q[v * 8 + u]);
        }
}

uint8_t category(int32_t v) {
    uint32_t m = (uint32_t)(v < 0 ? -(int64_t)v : v);
    uint8_t n = 0;
    while (m) {
        n++;
        m >>= 1;
    }
    return n;
}

struct Comp {
    uint8_t id, h, v, tq;
};

}  // namespace

bool plan_jpeg_encode(const FrameIn &f, const JpegEncodeOptions &opt, JpegEncodePlan *plan) {
    JpegEncodePlan &P = *plan;
    auto fail = [&](int32_t st, const char *m) {
        P.status = st;
        P.message = m;
        return false;
    };
    // validate_frame (encoder.rs:101-160)
    if (f.width == 0 || f.height == 0 || f.width > 65535 || f.height > 65535)
        return fail(kInvalidData, "JPEG frame dimensions must be between 1 and 65535");
    if (f.range == kRangeLimited)
        return fail(kUnsupported, "limited-range input requires conversion to full-range JPEG samples");
    Comp comps[3] = {{1, 1, 1, 0}, {2, 1, 1, 1}, {3, 1, 1, 1}};
    size_t nc = 3;
    switch (f.format) {
    case kGray8: nc = 1; break;
    case kYuv420: comps[0].h = comps[0].v = 2; break;
    case kYuv422: comps[0].h = 2; break;
    case kYuv444: break;
    default: return fail(kUnsupported, "pixel format is not supported by JPEG");
    }
    uint8_t hmax = 1, vmax = 1;
    for (size_t i = 0; i < nc; i++) {
        hmax = std::max(hmax, comps[i].h);
        vmax = std::max(vmax, comps[i].v);
    }
    // validate_input_planes (encoder.rs:177-215)
    if (f.plane_count != nc) {
        char m[128];
        snprintf(m, sizeof m, "JPEG input requires %zu plane(s), found %zu", nc, f.plane_count);
        return fail(kInvalidData, m);
    }
    for (size_t i = 0; i < nc; i++) {
        size_t w = (f.width * comps[i].h + hmax - 1) / hmax, h = (f.height * comps[i].v + vmax - 1) / vmax;
        const PlaneIn &p = f.planes[i];
        if (p.width != w || p.height != h || p.stride < w || p.data_len < p.stride * p.height) {
            char m[128];
            snprintf(m, sizeof m, "JPEG input plane %zu has inconsistent dimensions, stride, or storage", i);
            return fail(kInvalidData, m);
        }
    }
    if (opt.quality < 1 || opt.quality > 100) return fail(kInvalidData, "JPEG quality must be between 1 and 100");

    P.ncomp = (uint32_t)nc;
    for (size_t i = 0; i < nc; i++) {
        P.comp_h[i] = comps[i].h;
        P.comp_v[i] = comps[i].v;
        P.comp_tq[i] = comps[i].tq;
        P.comp_table[i] = opt.annex_k ? comps[i].tq : 0;
    }
    P.hmax = hmax;
    P.vmax = vmax;
    P.mcu_cols = (f.width + (size_t)hmax * 8 - 1) / ((size_t)hmax * 8);
    P.mcu_rows = (f.height + (size_t)vmax * 8 - 1) / ((size_t)vmax * 8);
    P.restart_interval = opt.restart_interval;
    scale_quant(kLumaQ, opt.quality, P.qt[0]);
    scale_quant(kChromaQ, opt.quality, P.qt[1]);
    const bool multi = nc > 1;
    std::vector<Table> tables;
    if (opt.annex_k) {
        tables.push_back(annex(0, 0, kDcLumaBits, kDcVals, 12));
        tables.push_back(annex(1, 0, kAcLumaBits, kAcLumaVals, 162));
        if (multi) {
            tables.push_back(annex(0, 1, kDcChromaBits, kDcVals, 12));
            tables.push_back(annex(1, 1, kAcChromaBits, kAcChromaVals, 162));
        }
    } else {
        tables.push_back(simple_dc());
        tables.push_back(simple_ac());
    }
    for (int k = 0; k < 2; k++)
        for (int i = 0; i < 256; i++) P.dc[k][i] = P.ac[k][i] = {0, 0, false};
    for (auto &t : tables)
        if (!huffman_encoder(t, t.cls ? P.ac[t.id] : P.dc[t.id]))
            return fail(kInvalidData, "JPEG Huffman table is oversubscribed");

    std::vector<uint8_t> &out = P.header;
    out = {0xff, 0xd8};
    segment(out, 0xe0, {'J', 'F', 'I', 'F', 0, 1, 2, 0, 0, 1, 0, 1, 0, 0});
    {  // DQT (encoder.rs:269-283)
        std::vector<uint8_t> p;
        p.push_back(0);
        for (int k = 0; k < 64; k++) p.push_back(P.qt[0][kZigzag[k]]);
        if (multi) {
            p.push_back(1);
            for (int k = 0; k < 64; k++) p.push_back(P.qt[1][kZigzag[k]]);
        }
        segment(out, 0xdb, p);
    }
    {  // SOF0 (encoder.rs:285-310)
        std::vector<uint8_t> p = {8, (uint8_t)(f.height >> 8), (uint8_t)f.height, (uint8_t)(f.width >> 8),
                                  (uint8_t)f.width, (uint8_t)nc};
        for (size_t i = 0; i < nc; i++) {
            p.push_back(comps[i].id);
            p.push_back((uint8_t)((comps[i].h << 4) | comps[i].v));
            p.push_back(comps[i].tq);
        }
        segment(out, 0xc0, p);
    }
    {  // DHT (encoder.rs:312-325)
        std::vector<uint8_t> p;
        for (auto &t : tables) {
            p.push_back((uint8_t)((t.cls << 4) | t.id));
            p.insert(p.end(), t.counts, t.counts + 16);
            p.insert(p.end(), t.symbols.begin(), t.symbols.end());
        }
        segment(out, 0xc4, p);
    }
    if (opt.restart_interval) segment(out, 0xdd, {(uint8_t)(opt.restart_interval >> 8), (uint8_t)opt.restart_interval});
    {  // SOS (encoder.rs:327-335)
        std::vector<uint8_t> p = {(uint8_t)nc};
        for (size_t i = 0; i < nc; i++) {
            p.push_back(comps[i].id);
            p.push_back((uint8_t)((P.comp_table[i] << 4) | P.comp_table[i]));
        }
        p.push_back(0);
        p.push_back(63);
        p.push_back(0);
        segment(out, 0xda, p);
    }
    return true;
}

EncodeResult encode_jpeg(const FrameIn &f, const JpegEncodeOptions &opt) {
    EncodeResult r;
    JpegEncodePlan P;
    if (!plan_jpeg_encode(f, opt, &P)) {
        r.status = P.status;
        r.message = P.message;
        return r;
    }
    auto fail = [&](int32_t st, const char *m) {
        r.status = st;
        r.message = m;
        r.data.clear();
        return r;
    };
    std::vector<uint8_t> &out = r.data;
    out = P.header;
    // encode_scan (encoder.rs:346-390)
    std::vector<int32_t> pred(P.ncomp, 0);
    Writer w;
    w.data.reserve(f.width * f.height);
    uint8_t block[64];
    int32_t coef[64];
    uint32_t rst = 0;
    size_t mcu_index = 0;
    for (size_t my = 0; my < P.mcu_rows; my++)
        for (size_t mx = 0; mx < P.mcu_cols; mx++, mcu_index++) {
            if (P.restart_interval && mcu_index > 0 && mcu_index % P.restart_interval == 0) {
                w.pad();
                w.data.push_back(0xff);
                w.data.push_back((uint8_t)(0xd0 + (rst & 7)));
                rst++;
                std::fill(pred.begin(), pred.end(), 0);
            }
            for (size_t ci = 0; ci < P.ncomp; ci++) {
                const PlaneIn &pl = f.planes[ci];
                const uint8_t *q = P.qt[P.comp_tq[ci]];
                const HuffCode *dcc = P.dc[P.comp_table[ci]], *acc = P.ac[P.comp_table[ci]];
                for (size_t by = 0; by < P.comp_v[ci]; by++)
                    for (size_t bx = 0; bx < P.comp_h[ci]; bx++) {
                        size_t x = (mx * P.comp_h[ci] + bx) * 8, y = (my * P.comp_v[ci] + by) * 8;
                        // read_block (encoder.rs:392-402): edge replication
                        for (size_t yy = 0; yy < 8; yy++) {
                            size_t sy = std::min(y + yy, pl.height - 1);
                            for (size_t xx = 0; xx < 8; xx++) {
                                size_t sx = std::min(x + xx, pl.width - 1);
                                block[yy * 8 + xx] = pl.data[sy * pl.stride + sx];
                            }
                        }
                        fdct_quantize(block, q, coef);
                        for (int k = 1; k < 64; k++) coef[k] = std::min(std::max(coef[k], -1023), 1023);
                        // encode_block (encoder.rs:404-425)
                        int32_t diff = coef[0] - pred[ci];
                        pred[ci] = coef[0];
                        uint8_t dsz = category(diff);
                        if (!dcc[dsz].present) return fail(kInvalidData, "JPEG Huffman table has no DC symbol");
                        w.bits(dcc[dsz].bits, dcc[dsz].length);
                        if (dsz) w.bits((uint32_t)(diff < 0 ? diff + (1 << dsz) - 1 : diff), dsz);
                        int run = 0;
                        for (int k = 1; k < 64; k++) {
                            int32_t v = coef[kZigzag[k]];
                            if (v == 0) {
                                run++;
                                continue;
                            }
                            while (run >= 16) {
                                w.bits(acc[0xf0].bits, acc[0xf0].length);
                                run -= 16;
                            }
                            uint8_t sz = category(v);
                            uint8_t sym = (uint8_t)((run << 4) | sz);
                            if (!acc[sym].present) return fail(kInvalidData, "JPEG Huffman table has no AC symbol");
                            w.bits(acc[sym].bits, acc[sym].length);
                            w.bits((uint32_t)(v < 0 ? v + (1 << sz) - 1 : v), sz);
                            run = 0;
                        }
                        if (run != 0) w.bits(acc[0x00].bits, acc[0x00].length);
                    }
            }
        }
    w.pad();
    out.insert(out.end(), w.data.begin(), w.data.end());
    out.push_back(0xff);
    out.push_back(0xd9);
    return r;
}

}  // namespace mmr
