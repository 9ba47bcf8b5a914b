// Baseline JPEG Huffman symbol decoding shared by the entropy kernels.
//
// Bits come from the unstuffed token stream as big-endian 32-bit words. A
// reader may hold bits past its interval's barrier, so every use of bits is
// checked against the count before the barrier (`avail`), which is exactly
// where the reference reader (crates/codecs/mjpeg/src/entropy.rs:74-166) would
// meet the next marker or the end of the data.
#pragma once

#include <cuda_runtime.h>

#include "plan.h"

namespace mmr {

__device__ __forceinline__ uint32_t bswap32(uint32_t x) { return __byte_perm(x, 0, 0x0123); }

struct Bits {
    const uint32_t *words;
    uint32_t wpos;  // next word to load
    int nbits;      // bits held in buf (>= 32 after refill)
    uint64_t buf;   // next bits, MSB first
    uint32_t used;  // bits consumed, counted from the reader's base position
    uint32_t pf;    // the word after buf's bits, loaded one refill ahead (byte order as stored)
};

// Reader at token-stream bit `bit`; `used` is the base-relative position there.
// Every frame's token stream is followed by padding (256-byte aligned frames and 64
// bytes past the last), so the one-ahead load of the last word stays inside the
// buffer.
__device__ __forceinline__ void bits_init(Bits &r, const uint8_t *tok, unsigned long long bit, uint32_t used) {
    r.words = reinterpret_cast<const uint32_t *>(tok);
    const uint32_t w0 = (uint32_t)(bit >> 5), skip = (uint32_t)bit & 31;
    r.buf = (uint64_t)bswap32(__ldg(r.words + w0)) << (32 + skip);
    r.pf = __ldg(r.words + w0 + 1);
    r.nbits = 32 - (int)skip;
    r.wpos = w0 + 2;
    r.used = used;
}

// Tops buf up to at least 33 bits from the prefetched word and starts the load
// of the next one, which the refill after this one uses (about 32 bits later).
__device__ __forceinline__ void refill(Bits &r) {
    if (r.nbits <= 32) {
        r.buf |= (uint64_t)bswap32(r.pf) << (32 - r.nbits);
        r.pf = __ldg(r.words + r.wpos);
        r.wpos++;
        r.nbits += 32;
    }
}

__device__ __forceinline__ void take(Bits &r, int n) {
    r.buf <<= n;
    r.nbits -= n;
    r.used += n;
}

// Code length of the next Huffman code (entropy.rs:57-70), 0 when none of
// length <= 16 matches; *sym its symbol.
__device__ __forceinline__ int slow_symbol(const HuffLut *__restrict__ T, const uint8_t *__restrict__ symbols,
                                           uint64_t buf, uint32_t *sym) {
    const uint32_t e = __ldg(&T->fast[buf >> 55]);
    if (e) {
        *sym = e & 0xff;
        return (int)(e >> 8);
    }
    const uint32_t code16 = (uint32_t)(buf >> 48);
#pragma unroll 1
    for (int l = 10; l <= 16; l++) {
        const int32_t c = (int32_t)(code16 >> (16 - l));
        if (c <= __ldg(&T->maxcode[l])) {
            *sym = __ldg(&symbols[__ldg(&T->sym_off) + __ldg(&T->valptr[l]) + c]);
            return l;
        }
    }
    return 0;
}

constexpr uint16_t kBarrierErr = 0xffff;  // the symbol runs into the interval's barrier

// Decodes one symbol for coefficient index k (0: the DC symbol), in the
// reference's order of checks (decoder.rs:501-546); with kPairs, two where
// HuffLut::fastp holds a pair (see decode_step). On success returns true, moves k
// (1 after the DC difference, past an AC level, 16 on for ZRL, 64 at EOB) and sets
// val: the DC difference or the AC level, 0 for EOB and ZRL, to be stored at
// zigzag index k - 1 (a zero stored past the last level changes nothing). On
// failure returns false with err (kBarrierErr when the symbol runs into the
// barrier) and errbit, the reader position the reference reports.
template <bool kPairs>
__device__ __forceinline__ bool decode_symbol_t(Bits &r, uint32_t avail, uint32_t stop, const HuffLut *__restrict__ T,
                                                const uint8_t *__restrict__ symbols, int &k, int32_t &val,
                                                int32_t &val2, int &k_mid, uint16_t &err, uint32_t &errbit) {
    refill(r);
    const uint32_t fv = __ldg(kPairs ? &T->fastp[r.buf >> (64 - kHuffFastBits)] : &T->fastv[r.buf >> (64 - kHuffFastBits)]);
    const uint32_t fl = fv & 31;
    if (kPairs) {
        k_mid = 0;
        val2 = 0;
    }
    if (kPairs && (fv & kFastPair) == kFastPair) {
        const int k1 = k + (int)((fv >> 5) & 127);
        const uint32_t adv2 = (fv >> 14) & 31;
        const int k2 = adv2 ? k1 + (int)adv2 : 64;
        if (fl - 1u < avail && fl <= stop && k1 < 64 && k2 <= 64) {
            val = (int32_t)(fv << 6) >> 25;
            val2 = (int32_t)fv >> 26;
            take(r, (int)fl);
            k_mid = k1;
            k = k2;
            return true;
        }
        // otherwise the first symbol alone, by the canonical search below
    } else {
        const int kn = (fv & kFastEob) ? 64 : k + (int)((fv >> 5) & 127);
        if (fv & kFastCode) {  // code resolved, magnitude after it (receive_extend, entropy.rs:168-182)
            const uint32_t size = (fv >> 16) & 15, total = fl + size;
            if (total - 1u < avail && kn <= 64) {
                const int32_t v = (int32_t)((r.buf << fl) >> (64 - size));
                val = v < (1 << (size - 1)) ? v + 1 - (1 << size) : v;
                take(r, (int)total);
                k = kn;
                return true;
            }
        } else if (fl - 1u < avail && kn <= 64) {
            val = (int32_t)fv >> 16;
            take(r, (int)fl);
            k = kn;
            return true;
        }
    }
    uint32_t sym;
    const int l = slow_symbol(T, symbols, r.buf, &sym);
    if (l == 0 || (uint32_t)l > avail) {
        err = (l == 0 && avail >= 16) ? (uint16_t)kJNoHuffCode : kBarrierErr;
        errbit = r.used + 16;
        return false;
    }
    int size, run;
    if (k == 0) {
        size = (int)sym;
        run = 0;
        if (size > 11) {
            take(r, l);
            err = kJDcCategory;
            errbit = r.used;
            return false;
        }
    } else {
        run = (int)(sym >> 4);
        size = (int)(sym & 15);
        if (size == 0) {
            take(r, l);
            val = 0;
            if (run == 0) {
                k = 64;
                return true;
            }
            if (run != 15) {
                err = kJAcZeroSize;
                errbit = r.used;
                return false;
            }
            if (k + 16 > 64) {
                err = kJZrlOverrun;
                errbit = r.used;
                return false;
            }
            k += 16;
            return true;
        }
        if (size > 10) {
            take(r, l);
            err = kJAcCategory;
            errbit = r.used;
            return false;
        }
        if (k + run >= 64) {
            take(r, l);
            err = kJAcRun;
            errbit = r.used;
            return false;
        }
    }
    if ((uint32_t)(l + size) > avail) {
        err = kBarrierErr;
        errbit = r.used;
        return false;
    }
    int32_t v = 0;
    if (size) {  // receive_extend (entropy.rs:168-182)
        v = (int32_t)((r.buf << l) >> (64 - size));
        v = v < (1 << (size - 1)) ? v + 1 - (1 << size) : v;
    }
    take(r, l + size);
    val = v;
    k += run + 1;
    return true;
}

// Decodes one symbol, or two AC symbols from one pair entry (HuffLut::fastp) when
// both lie within the next 11 bits and end at most `stop` bits on, the first
// leaves k below 64 and the second keeps it at most 64: the same steps one
// symbol at a time would take. The pair's inner boundary lies before `stop`, so
// a decode that records or compares states at the first symbol boundary at or
// past some position (a checkpoint, the slice end) passing that position as
// stop meets exactly the boundaries a one-symbol decode meets there. On a pair
// val is the first level (at zigzag index k_mid - 1) and val2 the second (at
// k - 1; 0 for EOB, with k 64); otherwise k_mid is 0 and val2 0.
__device__ __forceinline__ bool decode_step(Bits &r, uint32_t avail, uint32_t stop, const HuffLut *__restrict__ T,
                                            const uint8_t *__restrict__ symbols, int &k, int32_t &val,
                                            int32_t &val2, int &k_mid, uint16_t &err, uint32_t &errbit) {
    return decode_symbol_t<true>(r, avail, stop, T, symbols, k, val, val2, k_mid, err, errbit);
}

__device__ __forceinline__ bool decode_symbol(Bits &r, uint32_t avail, const HuffLut *__restrict__ T,
                                              const uint8_t *__restrict__ symbols, int &k, int32_t &val,
                                              uint16_t &err, uint32_t &errbit) {
    int32_t v2;
    int km;
    return decode_symbol_t<false>(r, avail, 0, T, symbols, k, val, v2, km, err, errbit);
}

}  // namespace mmr
