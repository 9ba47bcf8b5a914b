// DV25 video encoder restating crates/codecs/dv/src/encoder.rs (encode_video
// without audio or timecode), plus one generation option the reference lacks:
// per-block 2-4-8 DCT mode chosen by an inter-field activity test, with the
// 2-4-8 forward transform that the reference decoder's inverse_248 inverts.
// Compiled with -ffp-contract=off (binary64 forward DCT, as in Rust).
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "common.h"
#include "encode.h"
#include "tables.h"

namespace mmr {

namespace {

const double kCos16[128] = {
#include "cos_table.inc"
};
const int kZz88[64] = MMR_ZIGZAG_INIT;
const int kZz248[64] = MMR_DV_ZIGZAG_248_INIT;
const uint8_t kShifts[88] = MMR_DV_QUANT_SHIFTS_INIT;
const int kQoff[4] = MMR_DV_QUANT_OFFSET_INIT;
const int32_t kW88[64] = MMR_DV_IWEIGHT_88_INIT;
const int32_t kW248[64] = MMR_DV_IWEIGHT_248_INIT;
const size_t kBlockBits[6] = {112, 112, 112, 112, 80, 80};
const double kFrac = 0.7071067811865476;

struct Vlc {
    uint16_t code;
    uint8_t len, run;
    int16_t level;
};

// decoder.rs:319-354 vlc_entries (stable-sorted by length)
const std::vector<Vlc> &vlc_entries() {
    static std::vector<Vlc> entries = [] {
        std::vector<Vlc> tmp;
        uint8_t len_of[409];
        int n = 0;
        for (auto &r : kDvVlcLenRuns)
            for (int k = 0; k < r[1]; k++) len_of[n++] = (uint8_t)r[0];
        uint32_t canonical = 0;
        for (int i = 0; i < 409; i++) {
            uint8_t len = len_of[i];
            uint32_t code = canonical >> (32 - len);
            canonical += 1u << (32 - len);
            uint8_t run = i < 153 ? kDvVlcRunHead[i] : 0;
            int16_t level = (int16_t)(i < 153 ? kDvVlcLevelHead[i] : i - 153);
            if (level == 0) tmp.push_back({(uint16_t)code, len, run, 0});
            else {
                tmp.push_back({(uint16_t)(code << 1), (uint8_t)(len + 1), run, level});
                tmp.push_back({(uint16_t)((code << 1) | 1), (uint8_t)(len + 1), run, (int16_t)-level});
            }
        }
        std::stable_sort(tmp.begin(), tmp.end(), [](const Vlc &a, const Vlc &b) { return a.len < b.len; });
        return tmp;
    }();
    return entries;
}

// The first shortest entry for each (run, level), as min_by_key over the sorted
// entries picks it; precomputed once instead of scanning 746 entries per call.
const Vlc *min_entry(int run, int level) {
    static std::vector<const Vlc *> table = [] {
        std::vector<const Vlc *> t(128 * 511, nullptr);
        for (auto &e : vlc_entries()) {
            const Vlc *&slot = t[(size_t)e.run * 511 + (size_t)(e.level + 255)];
            if (!slot || e.len < slot->len) slot = &e;
        }
        return t;
    }();
    if (run < 0 || run > 127 || level < -255 || level > 255) return nullptr;
    return table[(size_t)run * 511 + (size_t)(level + 255)];
}

void push_bits(std::vector<uint8_t> &out, uint32_t value, int count) {
    for (int s = count - 1; s >= 0; s--) out.push_back((value >> s) & 1);
}

// decoder.rs:356-393 vlc_for_encoding
bool vlc_for_encoding(int run, int level, std::vector<uint8_t> &out) {
    if (run > 255 || level > 32767 || level < -32768) return false;
    if (const Vlc *e = min_entry(run, level)) {
        push_bits(out, e->code, e->len);
        return true;
    }
    if (run == 0 || level == 0) return false;
    const Vlc *r = min_entry(run - 1, 0), *l = min_entry(0, level);
    if (!r || !l) return false;
    push_bits(out, r->code, r->len);
    push_bits(out, l->code, l->len);
    return true;
}

// decoder.rs:290-310 inverse_factor_for_encoding
int32_t inverse_factor(size_t q, size_t cls, bool mode248, size_t pos) {
    size_t qq = q + (size_t)kQoff[cls];
    size_t area = pos <= 5 ? 0 : pos <= 20 ? 1 : pos <= 42 ? 2 : 3;
    int32_t weight = mode248 ? kW248[pos] : kW88[pos];
    return weight << (kShifts[qq * 4 + area] + 1 + (cls == 3));
}

// decoder.rs:395-422 macroblock_coordinates
void mb_coords(bool pal, size_t seqs, size_t sequence, size_t slot, size_t xy[5][2]) {
    static const size_t OFF[5] = {2, 6, 8, 0, 4}, SHUF3[5] = {18, 9, 27, 0, 36}, LS[5] = {9, 4, 13, 0, 18};
    static const size_t S1[27] = {0, 1, 2, 2, 1, 0, 0, 1, 2, 2, 1, 0, 0, 1, 2, 2, 1, 0, 0, 1, 2, 2, 1, 0, 0, 1, 2};
    static const size_t S2[30] = {0, 1, 2, 3, 4, 5, 5, 4, 3, 2, 1, 0, 0, 1, 2, 3, 4, 5, 5, 4, 3, 2, 1, 0, 0, 1, 2, 3, 4, 5};
    for (size_t m = 0; m < 5; m++) {
        if (pal) {
            size_t x = SHUF3[m] + slot / 3, y = S1[slot] + ((sequence + OFF[m]) % seqs) * 3;
            xy[m][0] = x * 2;
            xy[m][1] = y * 2;
        } else {
            size_t row = (sequence + OFF[m]) % seqs, k = slot + (size_t)(m == 1 || m == 2) * 3;
            size_t x = LS[m] + k / 6, y = S2[k] + row * 6;
            if (x > 21) y = y * 2 - row * 6;
            xy[m][0] = x * 4;
            xy[m][1] = y;
        }
    }
}

// encoder.rs:555-583 forward_dct (direct binary64 form)
void forward_88(const uint8_t px[64], int32_t out[64]) {
    for (int v = 0; v < 8; v++)
        for (int u = 0; u < 8; u++) {
            double cu = u == 0 ? kFrac : 1.0, cv = v == 0 ? kFrac : 1.0;
            double sum = 0.0;
            for (int y = 0; y < 8; y++)
                for (int x = 0; x < 8; x++)
                    sum += (double)px[y * 8 + x] * kCos16[(2 * x + 1) * u] * kCos16[(2 * y + 1) * v];
            out[v * 8 + u] = (int32_t)round(cu * cv * sum / 4.0);
        }
}

// Forward transform inverted by inverse_248 (decoder.rs:555-602): per field f,
// B_f[v][u] = 1/2 cu cv sum_{y<4,x<8} s_f[y][x] cos((2x+1)u pi/16) cos((2y+1)v pi/8);
// coefficient rows 2v / 2v+1 hold (B_0 + B_1)/2 and (B_0 - B_1)/2.
void forward_248(const uint8_t px[64], int32_t out[64]) {
    double B[2][4][8];
    for (int f = 0; f < 2; f++)
        for (int v = 0; v < 4; v++)
            for (int u = 0; u < 8; u++) {
                double sum = 0.0;
                for (int y = 0; y < 4; y++)
                    for (int x = 0; x < 8; x++)
                        sum += (double)px[(2 * y + f) * 8 + x] * kCos16[(2 * x + 1) * u] * kCos16[2 * (2 * y + 1) * v];
                double cu = u == 0 ? kFrac : 1.0, cv = v == 0 ? kFrac : 1.0;
                B[f][v][u] = 0.5 * cu * cv * sum;
            }
    for (int v = 0; v < 4; v++)
        for (int u = 0; u < 8; u++) {
            out[(2 * v) * 8 + u] = (int32_t)round((B[0][v][u] + B[1][v][u]) / 2.0);
            out[(2 * v + 1) * 8 + u] = (int32_t)round((B[0][v][u] - B[1][v][u]) / 2.0);
        }
}

bool prefer_248(const uint8_t px[64]) {
    int64_t frame = 0, field = 0;
    for (int y = 0; y < 7; y++)
        for (int x = 0; x < 8; x++) frame += std::abs((int)px[(y + 1) * 8 + x] - (int)px[y * 8 + x]);
    for (int y = 0; y < 6; y++)
        for (int x = 0; x < 8; x++) field += std::abs((int)px[(y + 2) * 8 + x] - (int)px[y * 8 + x]);
    return frame > field;
}

struct Cell {
    int32_t dc = 0;
    size_t cls = 0;
    bool mode = false;
    std::vector<uint8_t> ac;
};

// encoder.rs:470-488 quantized_levels
void quantized_levels(const int32_t c[64], size_t q, size_t cls, bool mode, int32_t levels[64]) {
    levels[0] = 0;
    const int *zz = mode ? kZz248 : kZz88;
    for (int pos = 1; pos < 64; pos++) {
        int32_t coefficient = c[zz[pos]];
        int32_t factor = inverse_factor(q, cls, mode, (size_t)pos);
        int64_t mag = ((int64_t)std::llabs(coefficient) * 16384 + factor / 2) / factor;
        int32_t level = mag > INT32_MAX ? INT32_MAX : (int32_t)mag;
        levels[pos] = coefficient < 0 ? -level : level;
    }
}

// encoder.rs:414-444 quantize_block
bool quantize_block(const int32_t c[64], bool mode, size_t q, Cell &cell, std::string &err) {
    size_t cls = 2;
    int32_t levels[64];
    quantized_levels(c, q, cls, mode, levels);
    for (int i = 0; i < 64; i++)
        if (std::abs((int64_t)levels[i]) > 255) {
            cls = 3;
            quantized_levels(c, q, cls, mode, levels);
            break;
        }
    cell.ac.clear();
    int previous = 0;
    for (int pos = 1; pos < 64; pos++) {
        if (levels[pos] == 0) continue;
        if (std::abs((int64_t)levels[pos]) > 255) {
            err = "DV coefficient exceeds encodable level after class selection";
            return false;
        }
        if (!vlc_for_encoding(pos - previous - 1, levels[pos], cell.ac)) {
            err = "DV has no VLC for this run and level";
            return false;
        }
        previous = pos;
    }
    vlc_for_encoding(127, 0, cell.ac);
    int32_t dd = c[0] - 1024;
    int32_t dc = dd >= 0 ? (dd + 2) / 4 : (dd - 2) / 4;
    cell.dc = std::min(std::max(dc, -256), 255);
    cell.cls = cls;
    cell.mode = mode;
    return true;
}

struct Packed {
    int32_t dc;
    size_t cls;
    bool mode;
    std::vector<uint8_t> storage;
    size_t used;
    std::vector<uint8_t> ac;
    size_t ac_offset;
    bool complete() const { return ac_offset == ac.size(); }
};

// encoder.rs:490-553 pack_segment, available_positions, fill_pending
size_t fill_pending(std::vector<Packed> &cells, size_t lo, size_t hi, const std::vector<std::pair<size_t, size_t>> &pos) {
    size_t p = 0;
    for (size_t pending = lo; pending < hi; pending++)
        while (!cells[pending].complete() && p < pos.size()) {
            cells[pos[p].first].storage[pos[p].second] = cells[pending].ac[cells[pending].ac_offset];
            cells[pending].ac_offset++;
            p++;
        }
    return pos.size() - p;
}

bool pack_segment(const std::vector<Cell> &cells, std::vector<Packed> &packed) {
    packed.clear();
    for (size_t i = 0; i < cells.size(); i++) {
        size_t cap = kBlockBits[i % 6] - 12;
        size_t used = std::min(cap, cells[i].ac.size());
        Packed p{cells[i].dc, cells[i].cls, cells[i].mode, std::vector<uint8_t>(cap, 1), used, cells[i].ac, used};
        std::copy(cells[i].ac.begin(), cells[i].ac.begin() + used, p.storage.begin());
        packed.push_back(std::move(p));
    }
    std::vector<std::pair<size_t, size_t>> segment_positions;
    for (size_t m = 0; m < 5; m++) {
        std::vector<std::pair<size_t, size_t>> pool;
        for (size_t i = m * 6; i < m * 6 + 6; i++)
            if (packed[i].complete())
                for (size_t b = packed[i].used; b < packed[i].storage.size(); b++) pool.push_back({i, b});
        size_t unused = fill_pending(packed, m * 6, m * 6 + 6, pool);
        bool all = true;
        for (size_t i = m * 6; i < m * 6 + 6; i++) all = all && packed[i].complete();
        if (all) segment_positions.insert(segment_positions.end(), pool.end() - unused, pool.end());
    }
    fill_pending(packed, 0, packed.size(), segment_positions);
    for (auto &p : packed)
        if (!p.complete()) return false;
    return true;
}

void read_block(const PlaneIn &p, size_t x, size_t y, uint8_t out[64]) {
    for (int i = 0; i < 64; i++) out[i] = p.data[(y + i / 8) * p.stride + x + i % 8];
}
void read_split_chroma(const PlaneIn &p, size_t x, size_t y, uint8_t out[64]) {
    for (int i = 0; i < 64; i++) {
        size_t row = i / 8, col = i % 8;
        out[i] = col < 4 ? p.data[(y + row) * p.stride + x + col] : p.data[(y + 8 + row) * p.stride + x + col - 4];
    }
}

// encoder.rs:256-330 initialize_dif_frame (+ header, subcode and VAUX packs)
void initialize_dif_frame(bool pal, size_t seqs, std::vector<uint8_t> &d) {
    d.assign(pal ? 144000 : 120000, 0xff);
    for (size_t s = 0; s < seqs; s++) {
        for (size_t pos = 0; pos < 150; pos++) {
            size_t off = (s * 150 + pos) * 80;
            uint8_t section;
            size_t number;
            if (pos == 0) {
                section = 0x1f;
                number = 0;
            } else if (pos <= 2) {
                section = 0x3f;
                number = pos - 1;
            } else if (pos <= 5) {
                section = 0x56;
                number = pos - 3;
            } else if ((pos - 6) % 16 == 0) {
                section = 0x76;
                number = (pos - 6) / 16;
            } else {
                section = 0x96;
                number = (pos - 7) - (pos - 6) / 16;
            }
            d[off] = section;
            d[off + 1] = (uint8_t)((s << 4) | 0x07);
            d[off + 2] = (uint8_t)number;
        }
        size_t h = s * 150 * 80;
        uint8_t dsf = pal ? 0xbf : 0x3f, app = pal ? 0xf8 : 0xf9;
        d[h + 3] = dsf;
        d[h + 4] = app;
        for (int k = 5; k < 8; k++) d[h + k] = app & 0x7f;
        for (size_t b = 0; b < 2; b++) {
            size_t base = (s * 150 + 1 + b) * 80;
            for (size_t sync = 0; sync < 6; sync++) {
                size_t o = base + 3 + sync * 8;
                d[o] = 0x8f;
                d[o + 1] = (uint8_t)(0xf0 | sync);
                d[o + 2] = 0xff;
            }
        }
        const uint8_t packs[4][5] = {{0x60, 0xff, 0xff, (uint8_t)(pal ? 0xe0 : 0xc0), 0xff},
                                     {0x61, 0x3f, 0xc8, 0xfc, 0xff},
                                     {0x62, 0xff, 0xc1, 0x01, 0x70},
                                     {0x63, 0xff, 0x80, 0x80, 0xc0}};
        for (size_t b = 0; b < 3; b++) {
            size_t base = (s * 150 + 3 + b) * 80;
            for (size_t start : {(size_t)3, (size_t)48})
                for (size_t i = 0; i < 4; i++) memcpy(&d[base + start + i * 5], packs[i], 5);
        }
    }
}

}  // namespace

EncodeResult encode_dv(const FrameIn &f, uint32_t policy) {
    EncodeResult r;
    auto fail = [&](int32_t st, const std::string &m) {
        r.status = st;
        r.message = m;
        r.data.clear();
        return r;
    };
    // profile_for_frame (encoder.rs:219-230)
    bool pal;
    if (f.width == 720 && f.height == 480 && f.format == kYuv411) pal = false;
    else if (f.width == 720 && f.height == 576 && f.format == kYuv420) pal = true;
    else {
        static const char *names[6] = {"?", "Gray8", "Yuv420p8", "Yuv422p8", "Yuv444p8", "Yuv411p8"};
        char m[160];
        snprintf(m, sizeof m, "DV25 encoding requires 720x480 Yuv411p8 or 720x576 Yuv420p8, found %zux%zu %s", f.width,
                 f.height, f.format < 6 ? names[f.format] : "?");
        return fail(kUnsupported, m);
    }
    // validate_frame (encoder.rs:232-254)
    size_t cw = pal ? 360 : 180, ch = pal ? 288 : 480;
    if (f.plane_count != 3) return fail(kInvalidData, "DV25 input requires three planes");
    size_t ew[3] = {720, cw, cw}, eh[3] = {f.height, ch, ch};
    for (size_t i = 0; i < 3; i++) {
        const PlaneIn &p = f.planes[i];
        if (p.width != ew[i] || p.height != eh[i] || p.stride < ew[i] || p.data_len < p.stride * eh[i]) {
            char m[64];
            snprintf(m, sizeof m, "DV input plane %zu has an invalid layout", i);
            return fail(kInvalidData, m);
        }
    }
    size_t seqs = pal ? 12 : 10;
    initialize_dif_frame(pal, seqs, r.data);
    std::vector<uint8_t> &out = r.data;
    std::vector<Cell> cells(30);
    std::vector<Packed> packed;
    for (size_t sequence = 0; sequence < seqs; sequence++)
        for (size_t slot = 0; slot < 27; slot++) {
            // encode_segment (encoder.rs:332-412)
            size_t xy[5][2];
            mb_coords(pal, seqs, sequence, slot, xy);
            int32_t coef[30][64];
            bool mode[30];
            for (size_t m = 0; m < 5; m++) {
                size_t x = xy[m][0] * 8, y = xy[m][1] * 8;
                uint8_t px[6][64];
                if (pal) {
                    read_block(f.planes[0], x, y, px[0]);
                    read_block(f.planes[0], x + 8, y, px[1]);
                    read_block(f.planes[0], x, y + 8, px[2]);
                    read_block(f.planes[0], x + 8, y + 8, px[3]);
                    read_block(f.planes[2], x / 2, y / 2, px[4]);
                    read_block(f.planes[1], x / 2, y / 2, px[5]);
                } else if (xy[m][0] < 88) {
                    for (int b = 0; b < 4; b++) read_block(f.planes[0], x + b * 8, y, px[b]);
                    read_block(f.planes[2], x / 4, y, px[4]);
                    read_block(f.planes[1], x / 4, y, px[5]);
                } else {
                    read_block(f.planes[0], x, y, px[0]);
                    read_block(f.planes[0], x + 8, y, px[1]);
                    read_block(f.planes[0], x, y + 8, px[2]);
                    read_block(f.planes[0], x + 8, y + 8, px[3]);
                    read_split_chroma(f.planes[2], x / 4, y, px[4]);
                    read_split_chroma(f.planes[1], x / 4, y, px[5]);
                }
                for (int b = 0; b < 6; b++) {
                    bool m248 = policy == kDvModeActivity && prefer_248(px[b]);
                    mode[m * 6 + b] = m248;
                    if (m248) forward_248(px[b], coef[m * 6 + b]);
                    else forward_88(px[b], coef[m * 6 + b]);
                }
            }
            int selected = -1;
            for (int q = 15; q >= 0; q--) {
                size_t total = 0;
                std::string err;
                for (int b = 0; b < 30; b++) {
                    if (!quantize_block(coef[b], mode[b], (size_t)q, cells[b], err)) return fail(kInvalidData, err);
                    total += cells[b].ac.size();
                }
                if (total <= 2680) {
                    selected = q;
                    break;
                }
            }
            if (selected < 0) {
                char m[128];
                snprintf(m, sizeof m, "DV segment %zu in sequence %zu cannot fit its coefficient budget", slot, sequence);
                return fail(kInvalidData, m);
            }
            if (!pack_segment(cells, packed)) return fail(kInvalidData, "DV coefficient spill overflow");
            for (size_t m = 0; m < 5; m++) {
                size_t vn = slot * 5 + m;
                size_t bi = sequence * 150 + 7 + (vn / 15) * 16 + vn % 15;
                size_t off = bi * 80;
                out[off + 3] = (uint8_t)selected;
                std::vector<uint8_t> bits;
                bits.reserve(608);
                for (size_t c = m * 6; c < m * 6 + 6; c++) {
                    push_bits(bits, (uint32_t)packed[c].dc & 0x1ff, 9);
                    bits.push_back(packed[c].mode ? 1 : 0);
                    push_bits(bits, (uint32_t)packed[c].cls, 2);
                    bits.insert(bits.end(), packed[c].storage.begin(), packed[c].storage.end());
                }
                for (size_t k = 0; k < 76; k++) {
                    uint8_t byte = 0;
                    for (int b = 0; b < 8; b++) byte = (uint8_t)((byte << 1) | bits[k * 8 + b]);
                    out[off + 4 + k] = byte;
                }
            }
        }
    return r;
}

}  // namespace mmr
