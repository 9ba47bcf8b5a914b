// Host-only harness for the DV VLC lookup table the engine builds
// (mmrecode_gb300/csrc/dv_vlc.h): fills one table for the CPU tests.
#include <stddef.h>
#include <stdint.h>

#include "dv_vlc.h"

extern "C" size_t mmr_test_dv_vlc_capacity() { return mmr::kDvVlcMaxEntries; }

extern "C" size_t mmr_test_fill_dv_vlc(uint32_t *table, size_t capacity) { return mmr::fill_dv_vlc(table, capacity); }
