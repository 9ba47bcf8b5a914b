// Host-only harness for the Huffman lookup tables the engine builds
// (mmrecode_gb300/csrc/huffman_lut.h): builds one table's HuffLut for the CPU tests.
#include <stddef.h>
#include <stdint.h>

#include "huffman_lut.h"

extern "C" size_t mmr_test_lut_size() { return sizeof(mmr::HuffLut); }

// key: 16 counts then the symbols (a DHT table body); ac: 1 for an AC table.
extern "C" int mmr_test_build_lut(const uint8_t *key, size_t key_len, int ac, void *out, size_t out_size) {
    if (key_len < 16 || out_size < sizeof(mmr::HuffLut)) return -1;
    mmr::build_lut(key, key_len, 0, ac != 0, static_cast<mmr::HuffLut *>(out));
    return 0;
}
