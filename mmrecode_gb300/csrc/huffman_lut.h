// Host construction of a baseline Huffman table's lookup records (HuffLut, plan.h)
// from its DHT counts and symbols (crates/codecs/mjpeg/src/entropy.rs:18-70 builds
// the same canonical code). Shared by the engine and the table tests.
#pragma once

#include <string.h>

#include "plan.h"

namespace mmr {

// key: 16 counts then the symbols; sym_off: the table's first symbol in the
// batch's symbol pool; ac: an AC table (run/size symbols, EOB, ZRL) or a DC one.
inline void build_lut(const uint8_t *key, size_t key_len, uint32_t sym_off, bool ac, HuffLut *lut) {
    memset(lut, 0, sizeof(*lut));
    for (int l = 0; l < 18; l++) lut->maxcode[l] = -1;
    const uint8_t *counts = key;
    const uint8_t *symbols = key + 16;
    constexpr uint32_t FB = kHuffFastBits;
    uint32_t code = 0, k = 0;
    for (int l = 1; l <= 16; l++) {
        uint32_t n = counts[l - 1];
        if (n) {
            lut->valptr[l] = (int32_t)k - (int32_t)code;
            lut->maxcode[l] = (int32_t)(code + n - 1);
        }
        for (uint32_t i = 0; i < n; i++) {
            const uint8_t sym = symbols[k];
            if (l <= 9) {
                uint32_t first = code << (9 - l), cnt = 1u << (9 - l);
                for (uint32_t j = 0; j < cnt; j++)  // the first code of each 9-bit pattern wins
                    if (!lut->fast[first + j]) lut->fast[first + j] = (uint16_t)((l << 8) | sym);
            }
            if ((uint32_t)l <= FB) {
                uint32_t size = 0, adv = 1, eob = 0;
                bool ok;
                if (ac) {
                    size = sym & 15;
                    adv = (sym >> 4) + 1;
                    if (sym == 0x00) eob = kFastEob, adv = 0, ok = true;
                    else if (sym == 0xf0) adv = 16, ok = true;
                    else ok = size >= 1 && size <= 10;
                } else {
                    size = sym;
                    ok = size <= 11;
                }
                if (ok && l + size > FB) {  // the code alone: the magnitude follows it
                    const uint32_t e = (size << 16) | kFastCode | (adv << 5) | (uint32_t)l;
                    const uint32_t base = code << (FB - l);
                    for (uint32_t j = 0; j < (1u << (FB - l)); j++)
                        if (!lut->fastv[base + j]) lut->fastv[base + j] = e;
                }
                if (ok && l + size <= FB) {
                    const uint32_t rest = FB - l - size;  // bits after the magnitude
                    for (uint32_t m = 0; m < (1u << size); m++) {
                        int32_t v = 0;
                        if (size) {
                            v = (int32_t)m;
                            if (v < (1 << (size - 1))) v += 1 - (1 << size);  // receive_extend
                        }
                        const uint32_t e = ((uint32_t)v << 16) | eob | (adv << 5) | (l + size);
                        const uint32_t base = (code << (FB - l)) | (m << rest);
                        for (uint32_t j = 0; j < (1u << rest); j++)
                            if (!lut->fastv[base + j]) lut->fastv[base + j] = e;
                    }
                }
            }
            code++;
            k++;
        }
        code <<= 1;
    }
    // pairs: an AC symbol whose bits leave room for the whole next one
    for (uint32_t x = 0; x < (1u << FB); x++) {
        const uint32_t e1 = lut->fastv[x];
        lut->fastp[x] = e1;
        if (!ac || !e1 || (e1 & (kFastCode | kFastEob))) continue;
        const uint32_t l1 = e1 & 31, adv1 = (e1 >> 5) & 127;
        const int32_t v1 = (int32_t)e1 >> 16;
        if (l1 + 2 > FB || v1 < -64 || v1 > 63) continue;
        const uint32_t e2 = lut->fastv[(x << l1) & ((1u << FB) - 1)];
        if (!e2 || (e2 & kFastCode)) continue;
        const uint32_t l2 = e2 & 31;  // the entry depends only on its first l2 bits
        if (l2 > FB - l1) continue;
        const int32_t v2 = (int32_t)e2 >> 16;
        const uint32_t adv2 = (e2 & kFastEob) ? 0 : (e2 >> 5) & 127;
        if (v2 < -32 || v2 > 31) continue;
        lut->fastp[x] = ((uint32_t)v2 << 26) | (((uint32_t)v1 & 127) << 19) | (adv2 << 14) | kFastPair | (adv1 << 5) |
                        (l1 + l2);
    }
    lut->sym_off = sym_off;
    lut->nsym = (uint32_t)(key_len - 16);
}

}  // namespace mmr
