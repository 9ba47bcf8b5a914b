// Host-only harness for the exact transforms' second decision stage
// (mmrecode_gb300/csrc/exact_fixed.h): the fixed-point weight tables the engine
// uploads and the decision that rounds a fixed-point sum, for the CPU tests.
#include <stddef.h>
#include <stdint.h>

#include "exact_fixed.h"

extern "C" int mmr_test_fix_entries() { return mmr::kFixEntries; }

// MJPEG, DV 8-8 and DV 2-4-8 tables, kFixEntries each.
extern "C" void mmr_test_fixed_tables(long long *jpeg, long long *w88, long long *w248) {
    mmr::build_jpeg_fixed(jpeg);
    mmr::build_dv_fixed(w88, w248);
}

// out[i] = fixed_round(t[i], c1[i], offset) for n sums.
extern "C" void mmr_test_fixed_round_many(const long long *t, const int32_t *c1, int offset, int32_t *out, size_t n) {
    for (size_t i = 0; i < n; i++) out[i] = mmr::fixed_round(t[i], c1[i], offset);
}
