// The DV25 VLC lookup table (entry layout in kernels.h), built from the
// canonical codes of crates/codecs/dv/src/decoder.rs:319-354: codes assigned
// in index order from VLC_LEN, level != 0 entries with a sign bit appended.
// Shared by the batch engine and the allocation-free entry point.
#pragma once

#include <stddef.h>
#include <stdint.h>
#include <string.h>

#include "kernels.h"
#include "tables.h"

namespace mmr {

// Largest table the two-level layout can need: the level-1 block plus one
// level-2 block for each level-1 prefix.
constexpr size_t kDvVlcMaxEntries = ((size_t)1 << kDvVlcL1Bits) + ((size_t)1 << kDvVlcL1Bits) * ((size_t)1 << (16 - kDvVlcL1Bits));

// Fills table[0, capacity) and returns the entries used; 0 when capacity is too
// small (nothing past table[capacity - 1] is ever written).
inline size_t fill_dv_vlc(uint32_t *table, size_t capacity) {
    const uint32_t l1 = kDvVlcL1Bits, l2 = 16 - kDvVlcL1Bits;
    size_t size = (size_t)1 << l1;
    if (capacity < size) return 0;
    memset(table, 0, capacity * sizeof(uint32_t));
    auto put = [&](uint32_t code, uint32_t len, uint32_t run, int32_t level) -> bool {
        const uint32_t packed = len | (run << 5) | ((uint32_t)(level + 256) << 12);
        if (len <= l1) {
            for (uint32_t j = 0; j < (1u << (l1 - len)); j++) table[(code << (l1 - len)) + j] = packed;
            return true;
        }
        const uint32_t prefix = code >> (len - l1);
        if (!(table[prefix] & 0x80000000u)) {
            if (size + ((size_t)1 << l2) > capacity) return false;
            table[prefix] = 0x80000000u | (uint32_t)size;
            size += (size_t)1 << l2;
        }
        const uint32_t off = table[prefix] & 0xffffu, rest = code & ((1u << (len - l1)) - 1);
        for (uint32_t j = 0; j < (1u << (16 - len)); j++) table[off + (rest << (16 - len)) + j] = packed;
        return true;
    };
    uint32_t canonical = 0;
    int i = 0;
    for (auto &r : kDvVlcLenRuns)
        for (int k = 0; k < r[1]; k++, i++) {
            const uint32_t len = (uint32_t)r[0];
            const uint32_t code = canonical >> (32 - len);
            canonical += 1u << (32 - len);
            const uint32_t run = i < 153 ? kDvVlcRunHead[i] : 0;
            const int32_t level = i < 153 ? kDvVlcLevelHead[i] : i - 153;
            if (level == 0) {
                if (!put(code, len, run, 0)) return 0;
            } else if (!put(code << 1, len + 1, run, level) || !put((code << 1) | 1, len + 1, run, -level)) {
                return 0;
            }
        }
    return size;
}

}  // namespace mmr
