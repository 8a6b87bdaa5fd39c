// cr_laz.cpp -- LAZ reading and writing (include/cr_laz.h).
//
// LASzip (Isenburg, "LASzip: lossless compression of LiDAR data", 2013;
// vendored by the reference as libs/laszip) codes each chunk of points with
// an adaptive range coder -- the fast arithmetic coder of A. Said
// ("Introduction to Arithmetic Coding - Theory and Practice", HPL-2004-76):
// a 32-bit interval renormalised byte by byte below 2^24, frequency models
// rebuilt on a growing period -- over per-field predictors.  Every quantity
// that fixes the bytes (model periods, product widths, predictor contexts,
// corrector classes) is the format's; file:line cites are into
// libs/laszip/src.  The code here is organised for parallel chunk decoding:
// one self-contained codec state per host thread, chunks handed out by an
// atomic counter, models re-initialised per chunk as the format requires.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstring>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/cr_laz.h"
#include "../../include/cr_synth.h"
#include "cr_internal.h"

namespace {

constexpr uint32_t kMinLength = 1u << 24;  // arithmeticmodel.hpp:47
constexpr uint32_t kBitShift = 13;         // arithmeticmodel.hpp:53: binary product width
constexpr uint32_t kSymShift = 15;         // arithmeticmodel.hpp:57: multi-symbol product width

inline uint32_t ld32(const uint8_t* p) {
    uint32_t v;
    std::memcpy(&v, p, 4);
    return v;
}
inline int32_t ld32s(const uint8_t* p) {
    int32_t v;
    std::memcpy(&v, p, 4);
    return v;
}
inline uint64_t ld64(const uint8_t* p) {
    uint64_t v;
    std::memcpy(&v, p, 8);
    return v;
}
inline uint16_t ld16(const uint8_t* p) {
    uint16_t v;
    std::memcpy(&v, p, 2);
    return v;
}
inline void st32(uint8_t* p, uint32_t v) { std::memcpy(p, &v, 4); }
inline void st64(uint8_t* p, uint64_t v) { std::memcpy(p, &v, 8); }
inline void st16(uint8_t* p, uint16_t v) { std::memcpy(p, &v, 2); }

// ---- adaptive models -------------------------------------------------------

// Binary model (arithmeticmodel.cpp:165-212): P(0) in 13-bit fixed point from
// a zero count and a total, both halved past 2^13; recomputed after `left`
// more bits, the period growing by 5/4 up to 64.
struct BitModel {
    uint32_t p0, zeros, total, period, left;
    void reset() {
        zeros = 1;
        total = 2;
        p0 = 1u << (kBitShift - 1);
        period = left = 4;
    }
    void refresh() {
        total += period;
        if (total > (1u << kBitShift)) {
            total = (total + 1) >> 1;
            zeros = (zeros + 1) >> 1;
            if (zeros == total) ++total;
        }
        p0 = (zeros * (0x80000000u / total)) >> (31 - kBitShift);
        period = std::min((5 * period) >> 2, 64u);
        left = period;
    }
};

// Multi-symbol model (arithmeticmodel.cpp:60-160): per-symbol counts (halved
// once their sum would pass 2^15), the cumulative distribution in 15-bit fixed
// point rebuilt after `left` more symbols, the period starting at (n + 6) / 2
// and growing by 5/4 up to 8 (n + 6).  The decoder also keeps a bucket table:
// bucket t holds the largest symbol whose cumulative value is at most
// t << shift, so a symbol lies between the entries of its bucket and the next.
struct SymModel {
    uint32_t n = 0, shift = 0, buckets = 0;
    uint32_t total = 0, period = 0, left = 0;
    uint32_t* cdf = nullptr;   // n
    uint32_t* count = nullptr; // n
    uint16_t* lut = nullptr;   // buckets + 1 (decoder only)
    std::unique_ptr<uint32_t[]> mem;

    void create(uint32_t symbols, bool decoder) {
        n = symbols;
        uint32_t bits = 1;
        while ((1u << bits) < n) ++bits;
        bits = decoder ? std::min(bits + 1, 12u) : 0;
        buckets = decoder ? 1u << bits : 0;
        shift = kSymShift - bits;
        const size_t words = 2 * (size_t)n + (decoder ? (buckets + 2) / 2 + 1 : 0);
        mem.reset(new uint32_t[words]);
        cdf = mem.get();
        count = cdf + n;
        lut = decoder ? reinterpret_cast<uint16_t*>(count + n) : nullptr;
    }
    void reset() {
        for (uint32_t k = 0; k < n; k++) count[k] = 1;
        total = 0;
        period = n;
        rebuild();
        period = left = (n + 6) >> 1;
    }
    void rebuild() {
        total += period;
        if (total > (1u << kSymShift)) {
            total = 0;
            for (uint32_t k = 0; k < n; k++) total += (count[k] = (count[k] + 1) >> 1);
        }
        const uint32_t scale = 0x80000000u / total;
        uint32_t sum = 0;
        for (uint32_t k = 0; k < n; k++) {
            cdf[k] = (scale * sum) >> (31 - kSymShift);
            sum += count[k];
        }
        if (lut) {
            uint32_t k = 0;
            for (uint32_t t = 0; t < buckets; t++) {
                const uint32_t at = t << shift;
                while (k + 1 < n && cdf[k + 1] <= at) ++k;
                lut[t] = (uint16_t)k;
            }
            lut[buckets] = (uint16_t)(n - 1);
        }
        period = std::min((5 * period) >> 2, (n + 6) << 3);
        left = period;
    }
};

// ---- range decoder / encoder (arithmeticdecoder.cpp, arithmeticencoder.cpp)

struct Decoder {
    const uint8_t* p = nullptr;
    const uint8_t* end = nullptr;
    uint32_t value = 0, length = 0;
    bool bad = false;

    uint8_t byte() {
        if (p < end) return *p++;
        bad = true;
        return 0;
    }
    void start() {
        length = 0xFFFFFFFFu;
        value = (uint32_t)byte() << 24;
        value |= (uint32_t)byte() << 16;
        value |= (uint32_t)byte() << 8;
        value |= (uint32_t)byte();
    }
    void renorm() {
        do {
            value = (value << 8) | byte();
        } while ((length <<= 8) < kMinLength);
    }
    uint32_t bit(BitModel& m) {
        const uint32_t x = m.p0 * (length >> kBitShift);
        const uint32_t b = value >= x;
        if (!b) {
            length = x;
            ++m.zeros;
        } else {
            value -= x;
            length -= x;
        }
        if (length < kMinLength) renorm();
        if (--m.left == 0) m.refresh();
        return b;
    }
    uint32_t sym(SymModel& m) {
        const uint32_t full = length;
        const uint32_t l = length >> kSymShift;
        const uint32_t dv = value / l;
        // dv passes 2^15 by up to length mod 2^15 / l inside the last symbol's
        // interval (its upper end is the full length)
        const uint32_t t = std::min(dv >> m.shift, m.buckets - 1);
        uint32_t lo = m.lut[t], hi = m.lut[t + 1];
        while (lo < hi) {
            const uint32_t mid = (lo + hi + 1) >> 1;
            if (m.cdf[mid] <= dv)
                lo = mid;
            else
                hi = mid - 1;
        }
        const uint32_t x = m.cdf[lo] * l;
        const uint32_t y = lo + 1 == m.n ? full : m.cdf[lo + 1] * l;
        value -= x;
        length = y - x;
        if (length < kMinLength) renorm();
        ++m.count[lo];
        if (--m.left == 0) m.rebuild();
        return lo;
    }
    // `bits` raw bits, more than 19 as a low 16 and the rest (readBits)
    uint32_t raw(uint32_t bits) {
        if (bits > 19) {
            const uint32_t low = raw(16);
            return (raw(bits - 16) << 16) | low;
        }
        length >>= bits;
        const uint32_t s = value / length;
        value -= length * s;
        if (length < kMinLength) renorm();
        if (s >> bits) bad = true;
        return s;
    }
    uint32_t raw32() {
        const uint32_t low = raw(16);
        return (raw(16) << 16) | low;
    }
};

struct Encoder {
    std::vector<uint8_t>* out = nullptr;
    uint32_t base = 0, length = 0;

    void start(std::vector<uint8_t>* o) {
        out = o;
        base = 0;
        length = 0xFFFFFFFFu;
    }
    void carry() {  // the interval base overflowed: add one to the bytes written
        size_t i = out->size();
        while (i > 0 && (*out)[i - 1] == 0xFF) (*out)[--i] = 0;
        if (i > 0) ++(*out)[i - 1];
    }
    void renorm() {
        do {
            out->push_back((uint8_t)(base >> 24));
            base <<= 8;
        } while ((length <<= 8) < kMinLength);
    }
    void add(uint32_t x) {
        const uint32_t b0 = base;
        base += x;
        if (base < b0) carry();
    }
    void bit(BitModel& m, uint32_t b) {
        const uint32_t x = m.p0 * (length >> kBitShift);
        if (!b) {
            length = x;
            ++m.zeros;
        } else {
            add(x);
            length -= x;
        }
        if (length < kMinLength) renorm();
        if (--m.left == 0) m.refresh();
    }
    void sym(SymModel& m, uint32_t s) {
        if (s + 1 == m.n) {
            const uint32_t x = m.cdf[s] * (length >> kSymShift);
            add(x);
            length -= x;
        } else {
            length >>= kSymShift;
            const uint32_t x = m.cdf[s] * length;
            add(x);
            length = m.cdf[s + 1] * length - x;
        }
        if (length < kMinLength) renorm();
        ++m.count[s];
        if (--m.left == 0) m.rebuild();
    }
    void raw(uint32_t bits, uint32_t v) {
        if (bits > 19) {
            raw(16, v & 0xFFFFu);
            v >>= 16;
            bits -= 16;
        }
        length >>= bits;
        add(v * length);
        if (length < kMinLength) renorm();
    }
    void raw32(uint32_t v) {
        raw(16, v & 0xFFFFu);
        raw(16, v >> 16);
    }
    // arithmeticencoder.cpp done(): one or two final bytes of the base, then
    // zeros so that the decoder's four-byte look-ahead ends on the chunk end.
    void finish() {
        bool three_zeros = true;
        if (length > 2 * kMinLength) {
            add(kMinLength);
            length = kMinLength >> 1;
        } else {
            add(kMinLength >> 1);
            length = kMinLength >> 9;
            three_zeros = false;
        }
        renorm();
        out->push_back(0);
        out->push_back(0);
        if (three_zeros) out->push_back(0);
        out = nullptr;
    }
};

// ---- integer corrector (integercompressor.cpp) -----------------------------
// real - pred is coded as its class k (bit length of c - 1 for c > 0, of -c
// for c <= 0; one model per context), then its offset inside the class: k = 0
// (c = 0 or 1) by a binary model, k <= 8 by a model of 2^k symbols, larger k
// by a model of the top 8 bits and k - 8 raw bits; k = 32 is the one value
// -2^31.  Values of fewer than 32 bits wrap modulo 2^bits.
struct IntCoder {
    uint32_t bits = 0, contexts = 0, cbits = 0, range = 0;
    int32_t cmin = 0, cmax = 0;
    uint32_t k = 0;
    std::vector<SymModel> kmodel;
    BitModel zero_one;
    std::vector<SymModel> corr;  // [1, cbits]

    void create(uint32_t b, uint32_t ctx, bool decoder) {
        bits = b;
        contexts = ctx;
        if (bits < 32) {
            cbits = bits;
            range = 1u << bits;
            cmin = -(int32_t)(range / 2);
            cmax = cmin + (int32_t)range - 1;
        } else {
            cbits = 32;
            range = 0;
            cmin = INT32_MIN;
            cmax = INT32_MAX;
        }
        kmodel.resize(ctx);
        for (auto& m : kmodel) m.create(cbits + 1, decoder);
        corr.resize(cbits + 1);
        for (uint32_t i = 1; i <= cbits; i++) corr[i].create(1u << std::min(i, 8u), decoder);
    }
    void reset() {
        for (auto& m : kmodel) m.reset();
        zero_one.reset();
        for (uint32_t i = 1; i <= cbits; i++) corr[i].reset();
    }
    int32_t decode(Decoder& d, int32_t pred, uint32_t ctx) {
        k = d.sym(kmodel[ctx]);
        uint32_t c;
        if (k == 0) {
            c = d.bit(zero_one);
        } else if (k < 32) {
            uint32_t u;
            if (k <= 8) {
                u = d.sym(corr[k]);
            } else {
                const uint32_t k1 = k - 8;
                u = d.sym(corr[k]);
                u = (u << k1) | d.raw(k1);
            }
            c = u >= (1u << (k - 1)) ? u + 1 : u - ((1u << k) - 1);
        } else {
            c = (uint32_t)cmin;
        }
        int32_t real = (int32_t)((uint32_t)pred + c);
        if (real < 0)
            real = (int32_t)((uint32_t)real + range);
        else if ((uint32_t)real >= range)
            real = (int32_t)((uint32_t)real - range);
        return real;
    }
    void encode(Encoder& e, int32_t pred, int32_t real, uint32_t ctx) {
        int32_t c = (int32_t)((uint32_t)real - (uint32_t)pred);
        if (c < cmin)
            c = (int32_t)((uint32_t)c + range);
        else if (c > cmax)
            c = (int32_t)((uint32_t)c - range);
        uint32_t c1 = c <= 0 ? 0u - (uint32_t)c : (uint32_t)c - 1;
        k = 0;
        while (c1) {
            c1 >>= 1;
            ++k;
        }
        e.sym(kmodel[ctx], k);
        if (k == 0) {
            e.bit(zero_one, (uint32_t)c);
        } else if (k < 32) {
            const uint32_t u = c < 0 ? (uint32_t)c + ((1u << k) - 1) : (uint32_t)c - 1;
            if (k <= 8) {
                e.sym(corr[k], u);
            } else {
                const uint32_t k1 = k - 8;
                e.sym(corr[k], u >> k1);
                e.raw(k1, u & ((1u << k1) - 1));
            }
        }
    }
};

// ---- item codecs, version 2 (lasreaditemcompressed_v2.cpp,
// laswriteitemcompressed_v2.cpp) ---------------------------------------------

inline int32_t fold8(int32_t v) { return v < 0 ? v + 256 : (v > 255 ? v - 256 : v); }
inline int32_t clamp8(int32_t v) { return v <= 0 ? 0 : (v >= 255 ? 255 : v); }

// Return-number contexts (laszip_common_v2.hpp): [number of returns][return].
const uint8_t kReturnMap[8][8] = {
    {15, 14, 13, 12, 11, 10, 9, 8}, {14, 0, 1, 3, 6, 10, 10, 9},   {13, 1, 2, 4, 7, 11, 11, 10},
    {12, 3, 4, 5, 8, 12, 12, 11},   {11, 6, 7, 8, 9, 13, 13, 12},  {10, 10, 11, 12, 13, 14, 14, 13},
    {9, 10, 11, 12, 13, 14, 15, 14}, {8, 9, 10, 11, 12, 13, 14, 15}};
// Height contexts: |number of returns - return|.
inline uint32_t return_level(uint32_t n, uint32_t r) { return n > r ? n - r : r - n; }

// Streaming median of the last five deltas (laszip_common_v2.hpp
// StreamingMedian5): a sorted five-array that alternately drops its maximum
// and its minimum to make room for the new value, switching side when the
// value falls on the other side of the median.
struct Median5 {
    int32_t v[5];
    bool drop_high;
    void reset() {
        for (int i = 0; i < 5; i++) v[i] = 0;
        drop_high = true;
    }
    int32_t get() const { return v[2]; }
    void add(int32_t x) {
        const int32_t mid = v[2];
        if (drop_high) {
            int j = 4;
            while (j > 0 && v[j - 1] > x) {
                v[j] = v[j - 1];
                --j;
            }
            v[j] = x;
            drop_high = x < mid;
        } else {
            int j = 0;
            while (j < 4 && v[j + 1] < x) {
                v[j] = v[j + 1];
                ++j;
            }
            v[j] = x;
            drop_high = !(mid < x);
        }
    }
};

// Byte models chosen by the previous byte value, created on first use and
// reset on first use in each chunk.
struct LazyModels {
    std::unique_ptr<SymModel> m[256];
    uint32_t stamp[256] = {};
    SymModel& get(uint32_t prev, uint32_t chunk, bool decoder) {
        if (!m[prev]) {
            m[prev].reset(new SymModel());
            m[prev]->create(256, decoder);
        }
        if (stamp[prev] != chunk) {
            stamp[prev] = chunk;
            m[prev]->reset();
        }
        return *m[prev];
    }
};

// POINT10 (20 bytes: X, Y, Z, intensity, return byte, classification, scan
// angle, user data, point source ID).  A 6-bit mask says which of the
// attribute bytes changed; X and Y deltas are predicted by the median of the
// last five deltas of the same return context, Z by the last Z of the same
// level; the context of Y and Z follows the class k of the X (and Y) corrector.
struct Point10 {
    bool decoder;
    uint8_t last[20];
    uint16_t last_intensity[16];
    int32_t last_height[8];
    Median5 mx[16], my[16];
    SymModel changed, scan_angle[2];
    LazyModels bit_byte, classification, user_data;
    IntCoder ic_intensity, ic_source, ic_dx, ic_dy, ic_z;

    explicit Point10(bool dec) : decoder(dec) {
        changed.create(64, dec);
        scan_angle[0].create(256, dec);
        scan_angle[1].create(256, dec);
        ic_intensity.create(16, 4, dec);
        ic_source.create(16, 1, dec);
        ic_dx.create(32, 2, dec);
        ic_dy.create(32, 22, dec);
        ic_z.create(32, 20, dec);
    }
    void init(const uint8_t* item) {
        for (int i = 0; i < 16; i++) {
            mx[i].reset();
            my[i].reset();
            last_intensity[i] = 0;
        }
        for (int i = 0; i < 8; i++) last_height[i] = 0;
        changed.reset();
        scan_angle[0].reset();
        scan_angle[1].reset();
        ic_intensity.reset();
        ic_source.reset();
        ic_dx.reset();
        ic_dy.reset();
        ic_z.reset();
        std::memcpy(last, item, 20);
        if (decoder) last[12] = last[13] = 0;  // the reader starts from intensity 0
    }
    void decode(Decoder& d, uint32_t chunk, uint8_t* item) {
        const uint32_t cv = d.sym(changed);
        uint32_t r, n, m, l;
        if (cv) {
            if (cv & 32) last[14] = (uint8_t)d.sym(bit_byte.get(last[14], chunk, true));
            r = last[14] & 7u;
            n = (last[14] >> 3) & 7u;
            m = kReturnMap[n][r];
            l = return_level(n, r);
            if (cv & 16) {
                const uint16_t v = (uint16_t)ic_intensity.decode(d, last_intensity[m], m < 3 ? m : 3);
                last_intensity[m] = v;
                st16(last + 12, v);
            } else {
                st16(last + 12, last_intensity[m]);
            }
            if (cv & 8) last[15] = (uint8_t)d.sym(classification.get(last[15], chunk, true));
            if (cv & 4) {
                const int32_t v = (int32_t)d.sym(scan_angle[(last[14] >> 6) & 1u]);
                last[16] = (uint8_t)fold8(v + last[16]);
            }
            if (cv & 2) last[17] = (uint8_t)d.sym(user_data.get(last[17], chunk, true));
            if (cv & 1) st16(last + 18, (uint16_t)ic_source.decode(d, ld16(last + 18), 0));
        } else {
            r = last[14] & 7u;
            n = (last[14] >> 3) & 7u;
            m = kReturnMap[n][r];
            l = return_level(n, r);
        }
        const uint32_t one = n == 1;
        const int32_t dx = ic_dx.decode(d, mx[m].get(), one);
        st32(last, (uint32_t)ld32s(last) + (uint32_t)dx);
        mx[m].add(dx);
        const uint32_t kx = ic_dx.k;
        const int32_t dy = ic_dy.decode(d, my[m].get(), one + (kx < 20 ? kx & ~1u : 20));
        st32(last + 4, (uint32_t)ld32s(last + 4) + (uint32_t)dy);
        my[m].add(dy);
        const uint32_t kz = (ic_dx.k + ic_dy.k) / 2;
        const int32_t z = ic_z.decode(d, last_height[l], one + (kz < 18 ? kz & ~1u : 18));
        st32(last + 8, (uint32_t)z);
        last_height[l] = z;
        std::memcpy(item, last, 20);
    }
    void encode(Encoder& e, uint32_t chunk, const uint8_t* item) {
        const uint32_t r = item[14] & 7u, n = (item[14] >> 3) & 7u;
        const uint32_t m = kReturnMap[n][r], l = return_level(n, r);
        const uint16_t inten = ld16(item + 12);
        const uint32_t cv = ((uint32_t)(last[14] != item[14]) << 5) |
                            ((uint32_t)(last_intensity[m] != inten) << 4) |
                            ((uint32_t)(last[15] != item[15]) << 3) | ((uint32_t)(last[16] != item[16]) << 2) |
                            ((uint32_t)(last[17] != item[17]) << 1) |
                            (uint32_t)(ld16(last + 18) != ld16(item + 18));
        e.sym(changed, cv);
        if (cv & 32) e.sym(bit_byte.get(last[14], chunk, false), item[14]);
        if (cv & 16) {
            ic_intensity.encode(e, last_intensity[m], inten, m < 3 ? m : 3);
            last_intensity[m] = inten;
        }
        if (cv & 8) e.sym(classification.get(last[15], chunk, false), item[15]);
        if (cv & 4) e.sym(scan_angle[(item[14] >> 6) & 1u], (uint32_t)fold8((int32_t)item[16] - last[16]));
        if (cv & 2) e.sym(user_data.get(last[17], chunk, false), item[17]);
        if (cv & 1) ic_source.encode(e, ld16(last + 18), ld16(item + 18), 0);
        const uint32_t one = n == 1;
        const int32_t dx = (int32_t)((uint32_t)ld32s(item) - (uint32_t)ld32s(last));
        ic_dx.encode(e, mx[m].get(), dx, one);
        mx[m].add(dx);
        const uint32_t kx = ic_dx.k;
        const int32_t dy = (int32_t)((uint32_t)ld32s(item + 4) - (uint32_t)ld32s(last + 4));
        ic_dy.encode(e, my[m].get(), dy, one + (kx < 20 ? kx & ~1u : 20));
        my[m].add(dy);
        const uint32_t kz = (ic_dx.k + ic_dy.k) / 2;
        const int32_t z = ld32s(item + 8);
        ic_z.encode(e, last_height[l], z, one + (kz < 18 ? kz & ~1u : 18));
        last_height[l] = z;
        std::memcpy(last, item, 20);
    }
};

// GPSTIME11 (8-byte double, coded as its 64-bit pattern): up to four
// interleaved time sequences, each with its last value and last 32-bit delta;
// a delta is coded as a rounded multiple of the last delta plus a corrector,
// a jump to another sequence, or a full 64-bit value.  The layered POINT14
// coder (lasreaditemcompressed_v3.cpp read_gps_time) uses the same scheme
// without the "unchanged" symbols (its change flag rides with the point):
// 5 and 515 symbols, full value at 1 and 511.
constexpr uint32_t kGpsMulti = 500, kGpsUnchanged = 511, kGpsFull = 512, kGpsSymbols = 516;
constexpr int32_t kGpsMinus = -10;

struct GpsTime11 {
    SymModel multi, zero_diff;
    IntCoder ic;
    uint64_t t[4];
    int32_t diff[4], extreme[4];
    uint32_t last, next;
    uint32_t zd_diff, zd_full, m_full;  // symbol layout: point-wise or layered

    explicit GpsTime11(bool dec, bool layered = false) {
        multi.create(layered ? kGpsSymbols - 1 : kGpsSymbols, dec);
        zero_diff.create(layered ? 5 : 6, dec);
        ic.create(32, 9, dec);
        zd_diff = layered ? 0 : 1;
        zd_full = layered ? 1 : 2;
        m_full = layered ? kGpsFull - 1 : kGpsFull;
    }
    void init_time(uint64_t t0) {
        last = next = 0;
        for (int i = 0; i < 4; i++) diff[i] = extreme[i] = 0, t[i] = 0;
        t[0] = t0;
        multi.reset();
        zero_diff.reset();
        ic.reset();
    }
    void init(const uint8_t* item) { init_time(ld64(item)); }
    static int32_t times(int32_t a, int32_t b) { return (int32_t)((uint32_t)a * (uint32_t)b); }
    void count_extreme(int32_t g) {
        if (++extreme[last] > 3) {
            diff[last] = g;
            extreme[last] = 0;
        }
    }
    void decode_full(Decoder& d) {
        next = (next + 1) & 3;
        const uint64_t hi = (uint32_t)ic.decode(d, (int32_t)(uint32_t)(t[last] >> 32), 8);
        t[next] = (hi << 32) | d.raw32();
        last = next;
        diff[last] = 0;
        extreme[last] = 0;
    }
    // one time value into t[last]
    void decode_time(Decoder& d) {
        for (;;) {
            if (diff[last] == 0) {
                const uint32_t s = d.sym(zero_diff);
                if (s == zd_diff) {
                    diff[last] = ic.decode(d, 0, 0);
                    t[last] += (uint64_t)(int64_t)diff[last];
                    extreme[last] = 0;
                } else if (s == zd_full) {
                    decode_full(d);
                } else if (s > zd_full) {
                    last = (last + s - zd_full) & 3;
                    continue;
                }
            } else {
                const uint32_t s = d.sym(multi);
                if (s == 1) {
                    t[last] += (uint64_t)(int64_t)ic.decode(d, diff[last], 1);
                    extreme[last] = 0;
                } else if (s < kGpsUnchanged) {
                    int32_t g;
                    if (s == 0) {
                        g = ic.decode(d, 0, 7);
                        count_extreme(g);
                    } else if (s < kGpsMulti) {
                        g = ic.decode(d, times((int32_t)s, diff[last]), s < 10 ? 2 : 3);
                    } else if (s == kGpsMulti) {
                        g = ic.decode(d, times((int32_t)kGpsMulti, diff[last]), 4);
                        count_extreme(g);
                    } else {
                        const int32_t mm = (int32_t)kGpsMulti - (int32_t)s;
                        if (mm > kGpsMinus) {
                            g = ic.decode(d, times(mm, diff[last]), 5);
                        } else {
                            g = ic.decode(d, times(kGpsMinus, diff[last]), 6);
                            count_extreme(g);
                        }
                    }
                    t[last] += (uint64_t)(int64_t)g;
                } else if (s == m_full) {
                    decode_full(d);
                } else if (s > m_full) {
                    last = (last + s - m_full) & 3;
                    continue;
                }
            }
            break;
        }
    }
    void decode(Decoder& d, uint8_t* item) {
        decode_time(d);
        st64(item, t[last]);
    }
    // float ratio of the deltas rounded half away from zero (I32_QUANTIZE);
    // LASzip's cast is undefined past the int32 range, saturated here.
    static int32_t quantize(float f) {
        const float r = f >= 0.0f ? f + 0.5f : f - 0.5f;
        if (!(r < 2147483648.0f)) return INT32_MAX;
        if (!(r > -2147483904.0f)) return INT32_MIN;
        return (int32_t)r;
    }
    void encode_full(Encoder& e, uint64_t now) {
        ic.encode(e, (int32_t)(uint32_t)(t[last] >> 32), (int32_t)(uint32_t)(now >> 32), 8);
        e.raw32((uint32_t)now);
        next = (next + 1) & 3;
        last = next;
        diff[last] = 0;
        extreme[last] = 0;
    }
    // another sequence within a 32-bit delta, or 0
    uint32_t other_sequence(uint64_t now) const {
        for (uint32_t i = 1; i < 4; i++) {
            const int64_t dd = (int64_t)(now - t[(last + i) & 3]);
            if (dd == (int64_t)(int32_t)dd) return i;
        }
        return 0;
    }
    void encode(Encoder& e, const uint8_t* item) {
        const uint64_t now = ld64(item);
        for (;;) {
            const int64_t d64 = (int64_t)(now - t[last]);
            const int32_t d32 = (int32_t)d64;
            const bool fits = d64 == (int64_t)d32;
            if (diff[last] == 0) {
                if (now == t[last]) {
                    e.sym(zero_diff, 0);
                    return;
                }
                if (fits) {
                    e.sym(zero_diff, 1);
                    ic.encode(e, 0, d32, 0);
                    diff[last] = d32;
                    extreme[last] = 0;
                } else {
                    const uint32_t i = other_sequence(now);
                    if (i) {
                        e.sym(zero_diff, i + 2);
                        last = (last + i) & 3;
                        continue;
                    }
                    e.sym(zero_diff, 2);
                    encode_full(e, now);
                }
                t[last] = now;
                return;
            }
            if (now == t[last]) {
                e.sym(multi, kGpsUnchanged);
                return;
            }
            if (fits) {
                const int32_t mlt = quantize((float)d32 / (float)diff[last]);
                if (mlt == 1) {
                    e.sym(multi, 1);
                    ic.encode(e, diff[last], d32, 1);
                    extreme[last] = 0;
                } else if (mlt > 0) {
                    if (mlt < (int32_t)kGpsMulti) {
                        e.sym(multi, (uint32_t)mlt);
                        ic.encode(e, times(mlt, diff[last]), d32, mlt < 10 ? 2 : 3);
                    } else {
                        e.sym(multi, kGpsMulti);
                        ic.encode(e, times((int32_t)kGpsMulti, diff[last]), d32, 4);
                        count_extreme(d32);
                    }
                } else if (mlt < 0) {
                    if (mlt > kGpsMinus) {
                        e.sym(multi, (uint32_t)((int32_t)kGpsMulti - mlt));
                        ic.encode(e, times(mlt, diff[last]), d32, 5);
                    } else {
                        e.sym(multi, (uint32_t)((int32_t)kGpsMulti - kGpsMinus));
                        ic.encode(e, times(kGpsMinus, diff[last]), d32, 6);
                        count_extreme(d32);
                    }
                } else {
                    e.sym(multi, 0);
                    ic.encode(e, 0, d32, 7);
                    count_extreme(d32);
                }
            } else {
                const uint32_t i = other_sequence(now);
                if (i) {
                    e.sym(multi, kGpsFull + i);
                    last = (last + i) & 3;
                    continue;
                }
                e.sym(multi, kGpsFull);
                encode_full(e, now);
            }
            t[last] = now;
            return;
        }
    }
};

// RGB12 (three 16-bit channels): a 7-bit mask of which bytes changed (bit 6:
// the channels differ from each other); green and blue bytes are predicted
// from red's change (lasreaditemcompressed_v2.cpp RGB12).
// The channels of one RGB value from the previous one `last` (RGB12 v2, and
// per scanner channel the RGB14 / RGBNIR14 v3 layers).
void rgb_decode(Decoder& d, SymModel& used, SymModel* diff, const uint16_t* last, uint16_t* v) {
    const uint32_t s = d.sym(used);
    v[0] = (s & 1) ? (uint16_t)fold8((int32_t)d.sym(diff[0]) + (last[0] & 255)) : (uint16_t)(last[0] & 0xFF);
    if (s & 2)
        v[0] |= (uint16_t)(fold8((int32_t)d.sym(diff[1]) + (last[0] >> 8)) << 8);
    else
        v[0] |= (uint16_t)(last[0] & 0xFF00);
    if (s & 64) {
        int32_t dl = (v[0] & 0xFF) - (last[0] & 0xFF);
        if (s & 4)
            v[1] = (uint16_t)fold8((int32_t)d.sym(diff[2]) + clamp8(dl + (last[1] & 255)));
        else
            v[1] = (uint16_t)(last[1] & 0xFF);
        if (s & 16) {
            const int32_t c = (int32_t)d.sym(diff[4]);
            dl = (dl + ((v[1] & 0xFF) - (last[1] & 0xFF))) / 2;
            v[2] = (uint16_t)fold8(c + clamp8(dl + (last[2] & 255)));
        } else {
            v[2] = (uint16_t)(last[2] & 0xFF);
        }
        int32_t dh = (v[0] >> 8) - (last[0] >> 8);
        if (s & 8)
            v[1] |= (uint16_t)(fold8((int32_t)d.sym(diff[3]) + clamp8(dh + (last[1] >> 8))) << 8);
        else
            v[1] |= (uint16_t)(last[1] & 0xFF00);
        if (s & 32) {
            const int32_t c = (int32_t)d.sym(diff[5]);
            dh = (dh + ((v[1] >> 8) - (last[1] >> 8))) / 2;
            v[2] |= (uint16_t)(fold8(c + clamp8(dh + (last[2] >> 8))) << 8);
        } else {
            v[2] |= (uint16_t)(last[2] & 0xFF00);
        }
    } else {
        v[1] = v[2] = v[0];
    }
}

struct Rgb12 {
    SymModel used, diff[6];
    uint16_t last[3];
    explicit Rgb12(bool dec) {
        used.create(128, dec);
        for (auto& m : diff) m.create(256, dec);
    }
    void init(const uint8_t* item) {
        used.reset();
        for (auto& m : diff) m.reset();
        for (int c = 0; c < 3; c++) last[c] = ld16(item + 2 * c);
    }
    void decode(Decoder& d, uint8_t* item) {
        uint16_t v[3];
        rgb_decode(d, used, diff, last, v);
        for (int c = 0; c < 3; c++) {
            last[c] = v[c];
            st16(item + 2 * c, v[c]);
        }
    }
    void encode(Encoder& e, const uint8_t* item) {
        uint16_t v[3];
        for (int c = 0; c < 3; c++) v[c] = ld16(item + 2 * c);
        uint32_t s = 0;
        for (int c = 0; c < 3; c++) {
            s |= (uint32_t)((last[c] & 0x00FF) != (v[c] & 0x00FF)) << (2 * c);
            s |= (uint32_t)((last[c] & 0xFF00) != (v[c] & 0xFF00)) << (2 * c + 1);
        }
        s |= (uint32_t)(((v[0] & 0xFF) != (v[1] & 0xFF)) || ((v[0] & 0xFF) != (v[2] & 0xFF)) ||
                        ((v[0] & 0xFF00) != (v[1] & 0xFF00)) || ((v[0] & 0xFF00) != (v[2] & 0xFF00)))
             << 6;
        e.sym(used, s);
        int32_t dl = 0, dh = 0;
        if (s & 1) {
            dl = (int32_t)(v[0] & 255) - (last[0] & 255);
            e.sym(diff[0], (uint32_t)fold8(dl));
        }
        if (s & 2) {
            dh = (int32_t)(v[0] >> 8) - (last[0] >> 8);
            e.sym(diff[1], (uint32_t)fold8(dh));
        }
        if (s & 64) {
            if (s & 4) e.sym(diff[2], (uint32_t)fold8((int32_t)(v[1] & 255) - clamp8(dl + (last[1] & 255))));
            if (s & 16) {
                dl = (dl + (v[1] & 255) - (last[1] & 255)) / 2;
                e.sym(diff[4], (uint32_t)fold8((int32_t)(v[2] & 255) - clamp8(dl + (last[2] & 255))));
            }
            if (s & 8) e.sym(diff[3], (uint32_t)fold8((int32_t)(v[1] >> 8) - clamp8(dh + (last[1] >> 8))));
            if (s & 32) {
                dh = (dh + (v[1] >> 8) - (last[1] >> 8)) / 2;
                e.sym(diff[5], (uint32_t)fold8((int32_t)(v[2] >> 8) - clamp8(dh + (last[2] >> 8))));
            }
        }
        for (int c = 0; c < 3; c++) last[c] = v[c];
    }
};

// BYTE (extra bytes): each byte's change from the previous point by its own model.
struct Bytes {
    std::vector<SymModel> m;
    std::vector<uint8_t> last;
    Bytes(uint32_t count, bool dec) : m(count), last(count) {
        for (auto& x : m) x.create(256, dec);
    }
    void init(const uint8_t* item) {
        for (auto& x : m) x.reset();
        std::memcpy(last.data(), item, last.size());
    }
    void decode(Decoder& d, uint8_t* item) {
        for (size_t i = 0; i < last.size(); i++) item[i] = last[i] = (uint8_t)fold8(last[i] + (int32_t)d.sym(m[i]));
    }
    void encode(Encoder& e, const uint8_t* item) {
        for (size_t i = 0; i < last.size(); i++) {
            e.sym(m[i], (uint32_t)fold8((int32_t)item[i] - last[i]));
            last[i] = item[i];
        }
    }
};

// ---- layered items of LAS 1.4 points, version 3 (lasreaditemcompressed_v3.cpp)
//
// A layered chunk holds, after its raw first point, the point count and the
// byte size of every layer, then the layers: each attribute group has its own
// coder run, so a group that never changes in the chunk costs no bytes.
// Every item keeps one prediction context per scanner channel.  As in LASzip
// 3.4's version 3 items, the channel the POINT14 item hands the other items
// is the new channel on a point that switches channels and 0 on every other
// point, and an item switching to a context it already used keeps reading the
// previous context's last values: the bytes of such files follow that rule.

// number_return_map_6ctx of laszip_common_v3.hpp: [number of returns][return]
const uint8_t kReturnMap6[16][16] = {
    {0, 1, 2, 3, 4, 5, 3, 4, 4, 5, 5, 5, 5, 5, 5, 5}, {1, 0, 1, 3, 3, 3, 3, 3, 3, 3, 3, 3, 3, 3, 3, 3},
    {2, 1, 2, 4, 4, 4, 4, 4, 4, 4, 4, 3, 3, 3, 3, 3}, {3, 3, 4, 5, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4},
    {4, 3, 4, 4, 5, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4}, {5, 3, 4, 4, 4, 5, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4},
    {3, 3, 4, 4, 4, 4, 5, 4, 4, 4, 4, 4, 4, 4, 4, 4}, {4, 3, 4, 4, 4, 4, 4, 5, 4, 4, 4, 4, 4, 4, 4, 4},
    {4, 3, 4, 4, 4, 4, 4, 4, 5, 4, 4, 4, 4, 4, 4, 4}, {5, 3, 4, 4, 4, 4, 4, 4, 4, 5, 4, 4, 4, 4, 4, 4},
    {5, 3, 4, 4, 4, 4, 4, 4, 4, 4, 5, 4, 4, 4, 4, 4}, {5, 3, 3, 4, 4, 4, 4, 4, 4, 4, 4, 5, 5, 4, 4, 4},
    {5, 3, 3, 4, 4, 4, 4, 4, 4, 4, 4, 5, 5, 5, 4, 4}, {5, 3, 3, 4, 4, 4, 4, 4, 4, 4, 4, 4, 5, 5, 5, 4},
    {5, 3, 3, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 5, 5, 5}, {5, 3, 3, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 5, 5}};
// number_return_level_8ctx: |n - r| capped at 7
inline uint32_t return_level8(uint32_t n, uint32_t r) { return std::min(n > r ? n - r : r - n, 7u); }

// Models of one byte-valued context table, created on first use and reset on
// first use after their owner's context was (re)initialised (generation).
struct ModelBank {
    uint32_t symbols = 0;
    std::vector<std::unique_ptr<SymModel>> m;
    std::vector<uint32_t> gen;
    void create(uint32_t count, uint32_t syms) {
        symbols = syms;
        m.resize(count);
        gen.assign(count, 0);
    }
    SymModel& get(uint32_t i, uint32_t g) {
        if (!m[i]) {
            m[i].reset(new SymModel());
            m[i]->create(symbols, true);
        }
        if (gen[i] != g) {
            gen[i] = g;
            m[i]->reset();
        }
        return *m[i];
    }
};

// The 30-byte LAS 1.4 point record (formats 6-10).
struct Point14 {
    int32_t X, Y, Z;
    uint16_t intensity;
    uint32_t r, n, cflags, channel, sdir, edge, cls, user;
    int16_t scan_angle;
    uint16_t source;
    uint64_t gps;
    bool gps_change;
    void load(const uint8_t* p) {
        X = ld32s(p);
        Y = ld32s(p + 4);
        Z = ld32s(p + 8);
        intensity = ld16(p + 12);
        r = p[14] & 15u;
        n = p[14] >> 4;
        cflags = p[15] & 15u;
        channel = (p[15] >> 4) & 3u;
        sdir = (p[15] >> 6) & 1u;
        edge = p[15] >> 7;
        cls = p[16];
        user = p[17];
        scan_angle = (int16_t)ld16(p + 18);
        source = ld16(p + 20);
        gps = ld64(p + 22);
        gps_change = false;
    }
    void store(uint8_t* p) const {
        st32(p, (uint32_t)X);
        st32(p + 4, (uint32_t)Y);
        st32(p + 8, (uint32_t)Z);
        st16(p + 12, intensity);
        p[14] = (uint8_t)(r | (n << 4));
        p[15] = (uint8_t)(cflags | (channel << 4) | (sdir << 6) | (edge << 7));
        p[16] = (uint8_t)cls;
        p[17] = (uint8_t)user;
        st16(p + 18, (uint16_t)scan_angle);
        st16(p + 20, source);
        st64(p + 22, gps);
    }
};

// POINT14 layers, in stream order
enum { kLayerXY, kLayerZ, kLayerClass, kLayerFlags, kLayerIntensity, kLayerScanAngle, kLayerUser,
       kLayerSource, kLayerGps, kP14Layers };

// One scanner channel's POINT14 prediction state (createAndInitModelsAndDecompressors).
struct P14Context {
    bool used = false;
    uint32_t gen = 0;
    Point14 last;
    uint16_t last_intensity[8];
    int32_t last_Z[8];
    Median5 mx[12], my[12];
    SymModel changed[8], channel, rnum_gps_same;
    ModelBank nret, rnum, cls, flags, user;
    IntCoder ic_dx, ic_dy, ic_z, ic_intensity, ic_scan_angle, ic_source;
    GpsTime11 gps{true, true};

    P14Context() {
        for (auto& m : changed) m.create(128, true);
        channel.create(3, true);
        rnum_gps_same.create(13, true);
        nret.create(16, 16);
        rnum.create(16, 16);
        cls.create(64, 256);
        flags.create(64, 64);
        user.create(64, 256);
        ic_dx.create(32, 2, true);
        ic_dy.create(32, 22, true);
        ic_z.create(32, 20, true);
        ic_intensity.create(16, 4, true);
        ic_scan_angle.create(16, 2, true);
        ic_source.create(16, 1, true);
    }
    void init(const Point14& p, uint32_t chunk_gen) {
        gen = chunk_gen;
        for (auto& m : changed) m.reset();
        channel.reset();
        rnum_gps_same.reset();
        ic_dx.reset();
        ic_dy.reset();
        ic_z.reset();
        ic_intensity.reset();
        ic_scan_angle.reset();
        ic_source.reset();
        for (int i = 0; i < 12; i++) {
            mx[i].reset();
            my[i].reset();
        }
        for (int i = 0; i < 8; i++) {
            last_Z[i] = p.Z;
            last_intensity[i] = p.intensity;
        }
        gps.init_time(p.gps);
        last = p;
        last.gps_change = false;
        used = true;
    }
};

struct Point14Layered {
    bool v4;  // version 4 hands its channel to the other items on every point
    std::unique_ptr<P14Context> ctx[4];
    uint32_t cur = 0, gen = 0;
    Decoder d[kP14Layers];
    bool changed[kP14Layers];
    explicit Point14Layered(bool version4) : v4(version4) {}

    P14Context& context(uint32_t c) {
        if (!ctx[c]) ctx[c].reset(new P14Context());
        return *ctx[c];
    }
    // chunk start: every context unused; the first point's channel current
    void init(const uint8_t* item, uint32_t& shared) {
        for (auto& c : ctx)
            if (c) c->used = false;
        Point14 p;
        p.load(item);
        cur = p.channel;
        shared = cur;
        context(cur).init(p, ++gen);
    }
    void decode(uint8_t* item, uint32_t& shared) {
        P14Context* c = &context(cur);
        Decoder& dx = d[kLayerXY];
        uint32_t lpr = (c->last.r == 1 ? 1u : 0u) + (c->last.r >= c->last.n ? 2u : 0u) +
                       (c->last.gps_change ? 4u : 0u);
        const uint32_t cv = dx.sym(c->changed[lpr]);
        if (cv & (1u << 6)) {  // the scanner channel changed
            const uint32_t sc = (cur + dx.sym(c->channel) + 1) % 4;
            P14Context& nc = context(sc);
            if (!nc.used) nc.init(c->last, ++gen);
            cur = sc;
            shared = cur;
            c = &nc;
            c->last.channel = sc;
        }
        if (v4) shared = cur;
        Point14& L = c->last;
        const bool source_change = (cv & (1u << 5)) != 0;
        const uint32_t gps_change = (cv >> 4) & 1u;
        const bool angle_change = (cv & (1u << 3)) != 0;
        const uint32_t last_n = L.n, last_r = L.r;
        uint32_t n = last_n, r = last_r;
        if (cv & (1u << 2)) {
            n = dx.sym(c->nret.get(last_n, c->gen));
            L.n = n;
        }
        switch (cv & 3u) {
            case 0: break;
            case 1: r = (last_r + 1) % 16; break;
            case 2: r = (last_r + 15) % 16; break;
            default:
                if (gps_change) r = dx.sym(c->rnum.get(last_r, c->gen));
                else r = (last_r + dx.sym(c->rnum_gps_same) + 2) % 16;
                break;
        }
        L.r = r;
        const uint32_t m = kReturnMap6[n][r], l = return_level8(n, r);
        const uint32_t cpr = (r == 1 ? 2u : 0u) + (r >= n ? 1u : 0u);
        const uint32_t one = n == 1;
        const uint32_t mi = (m << 1) | gps_change;
        const int32_t ddx = c->ic_dx.decode(dx, c->mx[mi].get(), one);
        L.X = (int32_t)((uint32_t)L.X + (uint32_t)ddx);
        c->mx[mi].add(ddx);
        const uint32_t kx = c->ic_dx.k;
        const int32_t ddy = c->ic_dy.decode(dx, c->my[mi].get(), one + (kx < 20 ? kx & ~1u : 20));
        L.Y = (int32_t)((uint32_t)L.Y + (uint32_t)ddy);
        c->my[mi].add(ddy);
        if (changed[kLayerZ]) {
            const uint32_t kz = (c->ic_dx.k + c->ic_dy.k) / 2;
            L.Z = c->ic_z.decode(d[kLayerZ], c->last_Z[l], one + (kz < 18 ? kz & ~1u : 18));
            c->last_Z[l] = L.Z;
        }
        if (changed[kLayerClass]) {
            const uint32_t ccc = ((L.cls & 31u) << 1) + (cpr == 3 ? 1u : 0u);
            L.cls = d[kLayerClass].sym(c->cls.get(ccc, c->gen));
        }
        if (changed[kLayerFlags]) {
            const uint32_t lf = (L.edge << 5) | (L.sdir << 4) | L.cflags;
            const uint32_t f = d[kLayerFlags].sym(c->flags.get(lf, c->gen));
            L.edge = (f >> 5) & 1u;
            L.sdir = (f >> 4) & 1u;
            L.cflags = f & 15u;
        }
        if (changed[kLayerIntensity]) {
            const uint32_t ii = (cpr << 1) | gps_change;
            const uint16_t v = (uint16_t)c->ic_intensity.decode(d[kLayerIntensity], c->last_intensity[ii], cpr);
            c->last_intensity[ii] = v;
            L.intensity = v;
        }
        if (changed[kLayerScanAngle] && angle_change)
            L.scan_angle = (int16_t)c->ic_scan_angle.decode(d[kLayerScanAngle], L.scan_angle, gps_change);
        if (changed[kLayerUser]) L.user = d[kLayerUser].sym(c->user.get(L.user / 4, c->gen));
        if (changed[kLayerSource] && source_change)
            L.source = (uint16_t)c->ic_source.decode(d[kLayerSource], L.source, 0);
        if (changed[kLayerGps] && gps_change) {
            c->gps.decode_time(d[kLayerGps]);
            L.gps = c->gps.t[c->gps.last];
        }
        L.store(item);
        L.gps_change = gps_change != 0;
    }
};

// RGB14 / RGBNIR14 per scanner channel: the RGB12 predictor (and a two-byte
// NIR channel) with the item's own layers.
struct RgbCtx {
    bool used = false;
    SymModel used_m, diff[6], nir_used, nir_diff[2];
    uint16_t last[4];
    explicit RgbCtx(bool nir) {
        used_m.create(128, true);
        for (auto& m : diff) m.create(256, true);
        if (nir) {
            nir_used.create(4, true);
            nir_diff[0].create(256, true);
            nir_diff[1].create(256, true);
        }
    }
    void init(const uint16_t* item, bool nir) {
        used_m.reset();
        for (auto& m : diff) m.reset();
        if (nir) {
            nir_used.reset();
            nir_diff[0].reset();
            nir_diff[1].reset();
        }
        for (int c = 0; c < (nir ? 4 : 3); c++) last[c] = item[c];
        used = true;
    }
};

struct Rgb14Layered {
    bool nir, v4;  // version 4 also switches to a used context's own last values
    std::unique_ptr<RgbCtx> ctx[4];
    uint32_t cur = 0;
    Decoder d[2];  // RGB, NIR
    bool changed[2];
    Rgb14Layered(bool with_nir, bool version4) : nir(with_nir), v4(version4) {}

    RgbCtx& context(uint32_t c) {
        if (!ctx[c]) ctx[c].reset(new RgbCtx(nir));
        return *ctx[c];
    }
    void init(const uint8_t* item, uint32_t shared) {
        for (auto& c : ctx)
            if (c) c->used = false;
        uint16_t v[4];
        for (int c = 0; c < (nir ? 4 : 3); c++) v[c] = ld16(item + 2 * c);
        cur = shared;
        context(cur).init(v, nir);
    }
    void decode(uint8_t* item, uint32_t shared) {
        uint16_t* last = context(cur).last;
        if (cur != shared) {
            cur = shared;
            RgbCtx& nc = context(cur);
            if (!nc.used) {
                nc.init(last, nir);
                last = nc.last;
            } else if (v4) {
                last = nc.last;
            }
        }
        RgbCtx& c = context(cur);
        uint16_t v[3];
        if (changed[0]) {
            rgb_decode(d[0], c.used_m, c.diff, last, v);
            for (int k = 0; k < 3; k++) last[k] = v[k];
        } else {
            for (int k = 0; k < 3; k++) v[k] = last[k];
        }
        for (int k = 0; k < 3; k++) st16(item + 2 * k, v[k]);
        if (!nir) return;
        uint16_t w;
        if (changed[1]) {
            const uint32_t s = d[1].sym(c.nir_used);
            w = (s & 1) ? (uint16_t)fold8((int32_t)d[1].sym(c.nir_diff[0]) + (last[3] & 255))
                        : (uint16_t)(last[3] & 0xFF);
            if (s & 2)
                w |= (uint16_t)(fold8((int32_t)d[1].sym(c.nir_diff[1]) + (last[3] >> 8)) << 8);
            else
                w |= (uint16_t)(last[3] & 0xFF00);
            last[3] = w;
        } else {
            w = last[3];
        }
        st16(item + 6, w);
    }
};

// BYTE14: every extra byte its own layer and, per channel, its own model.
struct BytesCtx {
    bool used = false;
    std::vector<SymModel> m;
    std::vector<uint8_t> last;
    explicit BytesCtx(uint32_t count) : m(count), last(count) {
        for (auto& x : m) x.create(256, true);
    }
};

struct Bytes14Layered {
    uint32_t count;
    bool v4;
    std::unique_ptr<BytesCtx> ctx[4];
    uint32_t cur = 0;
    std::vector<Decoder> d;
    std::vector<uint8_t> changed;
    Bytes14Layered(uint32_t n, bool version4) : count(n), v4(version4), d(n), changed(n) {}

    BytesCtx& context(uint32_t c) {
        if (!ctx[c]) ctx[c].reset(new BytesCtx(count));
        return *ctx[c];
    }
    void init_context(BytesCtx& c, const uint8_t* item) {
        for (auto& x : c.m) x.reset();
        std::memcpy(c.last.data(), item, count);
        c.used = true;
    }
    void init(const uint8_t* item, uint32_t shared) {
        for (auto& c : ctx)
            if (c) c->used = false;
        cur = shared;
        init_context(context(cur), item);
    }
    void decode(uint8_t* item, uint32_t shared) {
        uint8_t* last = context(cur).last.data();
        if (cur != shared) {
            cur = shared;
            BytesCtx& nc = context(cur);
            if (!nc.used) {
                init_context(nc, last);
                last = nc.last.data();
            } else if (v4) {
                last = nc.last.data();
            }
        }
        BytesCtx& c = context(cur);
        for (uint32_t i = 0; i < count; i++) {
            if (changed[i]) {
                item[i] = (uint8_t)fold8(last[i] + (int32_t)d[i].sym(c.m[i]));
                last[i] = item[i];
            } else {
                item[i] = last[i];
            }
        }
    }
};

// ---- point layouts and one thread's chunk codec ----------------------------

struct Item {
    int32_t type, size, version;
};

struct Layout {
    std::vector<Item> items;
    int32_t bpp = 0;
    int32_t rgb_offset = -1;  // of the RGB12 / RGB14 / RGBNIR14 item in a record, -1 without one
    bool layered = false;     // LAS 1.4 items (compressor 3)
};

// Items of LAS point formats 0-3 plus extra bytes (laszip.cpp setup).
cr_status layout_for(int32_t fmt, int32_t bpp, Layout* out) {
    if (fmt < 0 || fmt > 10 || bpp <= 0) return CR_ERR_INVALID_ARG;
    if (fmt > 3) return CR_ERR_UNSUPPORTED;
    Layout L;
    L.items.push_back({CR_LAZ_ITEM_POINT10, 20, 2});
    if (fmt == 1 || fmt == 3) L.items.push_back({CR_LAZ_ITEM_GPSTIME11, 8, 2});
    if (fmt == 2 || fmt == 3) L.items.push_back({CR_LAZ_ITEM_RGB12, 6, 2});
    int32_t base = 0;
    for (const Item& it : L.items) {
        if (it.type == CR_LAZ_ITEM_RGB12) L.rgb_offset = base;
        base += it.size;
    }
    if (bpp < base || bpp - base > 0xFFFF) return CR_ERR_INVALID_ARG;
    if (bpp > base) L.items.push_back({CR_LAZ_ITEM_BYTE, bpp - base, 2});
    L.bpp = bpp;
    *out = std::move(L);
    return CR_OK;
}

class PointCodec {
  public:
    PointCodec(const Layout& L, bool decoder) : layout_(L), rec_(L.bpp) {
        for (const Item& it : L.items) {
            switch (it.type) {
                case CR_LAZ_ITEM_POINT10: p10_.reset(new Point10(decoder)); break;
                case CR_LAZ_ITEM_GPSTIME11: gps_.reset(new GpsTime11(decoder)); break;
                case CR_LAZ_ITEM_RGB12: rgb_.reset(new Rgb12(decoder)); break;
                case CR_LAZ_ITEM_POINT14: p14_.reset(new Point14Layered(it.version == 4)); break;
                case CR_LAZ_ITEM_RGB14: rgb14_.reset(new Rgb14Layered(false, it.version == 4)); break;
                case CR_LAZ_ITEM_RGBNIR14: rgb14_.reset(new Rgb14Layered(true, it.version == 4)); break;
                case CR_LAZ_ITEM_BYTE14:
                    bytes14_.reset(new Bytes14Layered((uint32_t)it.size, it.version == 4));
                    break;
                default: bytes_.reset(new Bytes((uint32_t)it.size, decoder)); break;
            }
        }
    }

    // Decodes points [0, stop) of a chunk of `count` points at `src` and copies
    // records [skip, take) (take <= stop) to `out`.  When stop == count, *end
    // receives the position after the chunk.  False if the stream ran out or
    // is corrupt.
    bool decode_chunk(const uint8_t* src, const uint8_t* file_end, int64_t count, int64_t skip, int64_t take,
                      int64_t stop, uint8_t* out, const uint8_t** end) {
        if (count <= 0) {
            *end = src;
            return true;
        }
        if (layout_.layered) return decode_layered(src, file_end, skip, take, stop, out, end);
        const int64_t bpp = layout_.bpp;
        if (file_end - src < bpp) return false;
        uint8_t* rec = rec_.data();
        std::memcpy(rec, src, (size_t)bpp);  // the chunk's first point is stored raw
        init_items(rec);
        if (skip == 0 && take > 0) std::memcpy(out, rec, (size_t)bpp);
        Decoder d;
        d.p = src + bpp;
        d.end = file_end;
        d.start();
        for (int64_t i = 1; i < stop; i++) {
            size_t off = 0;
            for (const Item& it : layout_.items) {
                uint8_t* at = rec + off;
                switch (it.type) {
                    case CR_LAZ_ITEM_POINT10: p10_->decode(d, chunk_no_, at); break;
                    case CR_LAZ_ITEM_GPSTIME11: gps_->decode(d, at); break;
                    case CR_LAZ_ITEM_RGB12: rgb_->decode(d, at); break;
                    default: bytes_->decode(d, at); break;
                }
                off += (size_t)it.size;
            }
            if (i >= skip && i < take) std::memcpy(out + (i - skip) * bpp, rec, (size_t)bpp);
        }
        if (stop == count) *end = d.p;
        return !d.bad;
    }

    // The chunk of `count` records: the first raw, then the coder's bytes.
    void encode_chunk(const uint8_t* records, int64_t count, std::vector<uint8_t>& out) {
        out.clear();
        if (count <= 0) return;
        const int64_t bpp = layout_.bpp;
        out.insert(out.end(), records, records + bpp);
        init_items(records);
        Encoder e;
        e.start(&out);
        for (int64_t i = 1; i < count; i++) {
            const uint8_t* rec = records + i * bpp;
            size_t off = 0;
            for (const Item& it : layout_.items) {
                const uint8_t* at = rec + off;
                switch (it.type) {
                    case CR_LAZ_ITEM_POINT10: p10_->encode(e, chunk_no_, at); break;
                    case CR_LAZ_ITEM_GPSTIME11: gps_->encode(e, at); break;
                    case CR_LAZ_ITEM_RGB12: rgb_->encode(e, at); break;
                    default: bytes_->encode(e, at); break;
                }
                off += (size_t)it.size;
            }
        }
        e.finish();
    }

  private:
    // lasreadpoint.cpp read() for layered chunks: the raw first point, the
    // point count, every item's layer sizes, then every item's layers.
    bool decode_layered(const uint8_t* src, const uint8_t* file_end, int64_t skip, int64_t take,
                        int64_t stop, uint8_t* out, const uint8_t** end) {
        const int64_t bpp = layout_.bpp;
        if (file_end - src < bpp + 4) return false;
        uint8_t* rec = rec_.data();
        std::memcpy(rec, src, (size_t)bpp);
        const uint8_t* q = src + bpp + 4;  // the stored point count is not needed
        std::vector<uint32_t>& sizes = sizes_;
        sizes.clear();
        for (const Item& it : layout_.items) {
            const int nl = it.type == CR_LAZ_ITEM_POINT14 ? kP14Layers
                           : it.type == CR_LAZ_ITEM_RGBNIR14 ? 2
                           : it.type == CR_LAZ_ITEM_RGB14 ? 1 : it.size;
            for (int k = 0; k < nl; k++) {
                if (file_end - q < 4) return false;
                sizes.push_back(ld32(q));
                q += 4;
            }
        }
        size_t li = 0;
        const uint8_t* at = q;
        bool overrun = false;
        auto layer = [&](Decoder& d, bool always) -> bool {  // one layer's bytes; false: empty
            const uint32_t n = sizes[li++];
            const bool fits = (int64_t)n <= file_end - at;
            d.p = at;
            d.end = fits ? at + n : file_end;  // never past the file
            d.bad = !fits;
            overrun |= !fits;
            at = fits ? at + n : file_end;
            if (n == 0 && !always) return false;
            d.start();
            return true;
        };
        for (const Item& it : layout_.items) {
            if (it.type == CR_LAZ_ITEM_POINT14) {
                for (int k = 0; k < kP14Layers; k++) p14_->changed[k] = layer(p14_->d[k], k == kLayerXY);
            } else if (it.type == CR_LAZ_ITEM_RGB14) {
                rgb14_->changed[0] = layer(rgb14_->d[0], false);
            } else if (it.type == CR_LAZ_ITEM_RGBNIR14) {
                rgb14_->changed[0] = layer(rgb14_->d[0], false);
                rgb14_->changed[1] = layer(rgb14_->d[1], false);
            } else {
                for (int k = 0; k < it.size; k++) bytes14_->changed[k] = layer(bytes14_->d[k], false);
            }
        }
        if (overrun) return false;
        // POINT14 comes first and hands its scanner channel to the others
        uint32_t shared = 0;
        size_t off = 0;
        for (const Item& it : layout_.items) {
            if (it.type == CR_LAZ_ITEM_POINT14) p14_->init(rec + off, shared);
            else if (it.type == CR_LAZ_ITEM_BYTE14) bytes14_->init(rec + off, shared);
            else rgb14_->init(rec + off, shared);
            off += (size_t)it.size;
        }
        if (skip == 0 && take > 0) std::memcpy(out, rec, (size_t)bpp);
        for (int64_t i = 1; i < stop; i++) {
            shared = 0;  // lasreadpoint.cpp read(): a fresh context per point
            off = 0;
            for (const Item& it : layout_.items) {
                if (it.type == CR_LAZ_ITEM_POINT14) p14_->decode(rec + off, shared);
                else if (it.type == CR_LAZ_ITEM_BYTE14) bytes14_->decode(rec + off, shared);
                else rgb14_->decode(rec + off, shared);
                off += (size_t)it.size;
            }
            if (i >= skip && i < take) std::memcpy(out + (i - skip) * bpp, rec, (size_t)bpp);
        }
        *end = at;
        bool bad = false;
        for (const Decoder& d : p14_->d) bad |= d.bad;
        if (rgb14_) bad |= rgb14_->d[0].bad || rgb14_->d[1].bad;
        if (bytes14_)
            for (const Decoder& d : bytes14_->d) bad |= d.bad;
        return !bad;
    }

    void init_items(const uint8_t* rec) {
        ++chunk_no_;
        size_t off = 0;
        for (const Item& it : layout_.items) {
            switch (it.type) {
                case CR_LAZ_ITEM_POINT10: p10_->init(rec + off); break;
                case CR_LAZ_ITEM_GPSTIME11: gps_->init(rec + off); break;
                case CR_LAZ_ITEM_RGB12: rgb_->init(rec + off); break;
                default: bytes_->init(rec + off); break;
            }
            off += (size_t)it.size;
        }
    }

    const Layout& layout_;
    std::vector<uint8_t> rec_;
    uint32_t chunk_no_ = 0;
    std::unique_ptr<Point10> p10_;
    std::unique_ptr<GpsTime11> gps_;
    std::unique_ptr<Rgb12> rgb_;
    std::unique_ptr<Bytes> bytes_;
    std::unique_ptr<Point14Layered> p14_;
    std::unique_ptr<Rgb14Layered> rgb14_;
    std::unique_ptr<Bytes14Layered> bytes14_;
    std::vector<uint32_t> sizes_;
};

int resolve_threads(int32_t threads, int64_t work) {
    int t = threads > 0 ? threads : (int)std::thread::hardware_concurrency();
    if (t < 1) t = 1;
    return (int)std::max<int64_t>(1, std::min<int64_t>(t, work));
}

// Runs job(worker) on `threads` threads (the caller's thread is worker 0).
template <typename F>
void run_workers(int threads, F&& job) {
    std::vector<std::thread> pool;
    for (int t = 1; t < threads; t++) pool.emplace_back(job, t);
    job(0);
    for (auto& th : pool) th.join();
}

}  // namespace

// ---- the opened file --------------------------------------------------------

struct cr_laz {
    const uint8_t* file = nullptr;
    int64_t size = 0;
    cr_laz_info info;
    Layout layout;
    std::vector<int64_t> chunk_start;  // byte offset of every chunk, plus the end of the last
    std::vector<int64_t> chunk_first;  // first point of every chunk, plus num_points
    bool sequential = false;           // chunk starts unknown: decode in order
    int64_t chunk_points = 0;          // fixed chunk size (sequential decoding)
};

namespace {

// Chunk table (lasreadpoint.cpp read_chunk_table): version, count, then the
// per-chunk point counts (variable chunking only) and byte sizes, each
// predicted by the previous one through a 32-bit corrector with 2 contexts.
cr_status read_chunk_table(cr_laz* z, int64_t table_at, int64_t chunks_at, bool variable, int64_t n) {
    const uint8_t* f = z->file;
    if (table_at < chunks_at || table_at + 8 > z->size) return CR_ERR_CORRUPT;
    if (ld32(f + table_at) != 0) return CR_ERR_CORRUPT;
    const int64_t count = ld32(f + table_at + 4);
    std::vector<uint32_t> bytes(count), points(count);
    if (count > 0) {
        Decoder d;
        d.p = f + table_at + 8;
        d.end = f + z->size;
        d.start();
        IntCoder ic;
        ic.create(32, 2, true);
        ic.reset();
        for (int64_t i = 0; i < count; i++) {
            if (variable) points[i] = (uint32_t)ic.decode(d, i ? (int32_t)points[i - 1] : 0, 0);
            bytes[i] = (uint32_t)ic.decode(d, i ? (int32_t)bytes[i - 1] : 0, 1);
        }
        if (d.bad) return CR_ERR_CORRUPT;
    }
    z->chunk_start.assign(1, chunks_at);
    z->chunk_first.assign(1, 0);
    for (int64_t i = 0; i < count; i++) {
        const int64_t s = z->chunk_start.back() + (int64_t)bytes[i];
        if (bytes[i] == 0 || s > table_at) return CR_ERR_CORRUPT;
        z->chunk_start.push_back(s);
        const int64_t first = z->chunk_first.back();
        if (first >= n) break;
        z->chunk_first.push_back(variable ? first + (int64_t)points[i] : first + z->chunk_points);
    }
    const int64_t used = (int64_t)z->chunk_first.size() - 1;
    if (z->chunk_first.back() < n) return CR_ERR_CORRUPT;  // the table covers fewer points
    z->chunk_first.back() = n;
    z->chunk_start.resize(used + 1);
    return CR_OK;
}

cr_status decode_range(const cr_laz* z, int64_t first, int64_t n, uint8_t* out, int32_t threads) {
    if (n <= 0) return CR_OK;
    const int64_t bpp = z->layout.bpp;
    const uint8_t* file_end = z->file + z->size;
    if (z->sequential) {  // chunk starts follow from decoding their predecessors
        PointCodec codec(z->layout, true);
        const int64_t N = z->info.las.num_points;
        int64_t pos = z->chunk_start[0];
        for (int64_t lo = 0; lo < first + n; lo += z->chunk_points) {
            const int64_t count = std::min(z->chunk_points, N - lo);
            const int64_t skip = std::min(std::max<int64_t>(first - lo, 0), count);
            const int64_t take = std::max(std::min(first + n - lo, count), skip);
            const uint8_t* end = nullptr;
            if (!codec.decode_chunk(z->file + pos, file_end, count, skip, take, count,
                                    take > skip ? out + (lo + skip - first) * bpp : out, &end))
                return CR_ERR_CORRUPT;
            pos = end - z->file;
        }
        return CR_OK;
    }
    const auto& cf = z->chunk_first;
    const int64_t c0 = (int64_t)(std::upper_bound(cf.begin(), cf.end(), first) - cf.begin()) - 1;
    const int64_t c1 = (int64_t)(std::upper_bound(cf.begin(), cf.end(), first + n - 1) - cf.begin()) - 1;
    std::atomic<int64_t> next(c0);
    std::atomic<int> status(CR_OK);
    const bool check_end = z->info.compressor != CR_LAZ_POINTWISE;
    run_workers(resolve_threads(threads, c1 - c0 + 1), [&](int) {
        PointCodec codec(z->layout, true);
        for (int64_t c = next++; c <= c1 && status.load() == CR_OK; c = next++) {
            const int64_t lo = cf[c], count = cf[c + 1] - lo;
            const int64_t skip = std::max<int64_t>(first - lo, 0);
            const int64_t stop = std::min(first + n, cf[c + 1]) - lo;
            const uint8_t* end = nullptr;
            const bool ok = codec.decode_chunk(z->file + z->chunk_start[c], file_end, count, skip, stop,
                                               stop, out + (lo + skip - first) * bpp, &end);
            if (!ok || (check_end && stop == count && end != z->file + z->chunk_start[c + 1]))
                status.store(CR_ERR_CORRUPT);
        }
    });
    return (cr_status)status.load();
}

}  // namespace

extern "C" {

// LasLoaderSparse.cpp:493-526 (the header) and laszip.cpp unpack (the VLR).
cr_status cr_laz_open(const void* file, int64_t size, cr_laz** out, cr_laz_info* info) {
    if (!file || !out || size <= 0) return CR_ERR_INVALID_ARG;
    *out = nullptr;
    const uint8_t* f = static_cast<const uint8_t*>(file);
    std::unique_ptr<cr_laz> z(new cr_laz());
    z->file = f;
    z->size = size;
    std::memset(&z->info, 0, sizeof(z->info));
    cr_status st = cr_las_parse_header(f, size, &z->info.las);
    if (st != CR_OK) return st;
    const int64_t header_size = ld16(f + 94);
    const int64_t num_vlrs = ld32(f + 100);
    const int64_t points_at = z->info.las.offset_to_points;
    z->info.points_at = points_at;
    const uint8_t* vlr = nullptr;
    int64_t vlr_len = 0;
    int64_t pos = header_size;
    for (int64_t v = 0; v < num_vlrs && pos + 54 <= std::min(size, points_at); v++) {
        const int64_t len = ld16(f + pos + 20);
        char user[17] = {0};
        std::memcpy(user, f + pos + 2, 16);
        if (std::strcmp(user, "laszip encoder") == 0 && ld16(f + pos + 18) == 22204) {
            vlr = f + pos + 54;
            vlr_len = len;
        }
        pos += 54 + len;
    }
    if (!vlr || vlr - f + vlr_len > size || vlr_len < 34) return CR_ERR_INVALID_ARG;
    const int32_t compressor = ld16(vlr), coder = ld16(vlr + 2);
    z->info.compressor = compressor;
    z->info.version_major = vlr[4];
    z->info.version_minor = vlr[5];
    const uint32_t chunk_size = ld32(vlr + 12);
    const int32_t num_items = ld16(vlr + 32);
    if (vlr_len < 34 + 6 * num_items || num_items < 1) return CR_ERR_INVALID_ARG;
    if (num_items > CR_LAZ_MAX_ITEMS) return CR_ERR_UNSUPPORTED;
    z->info.num_items = num_items;
    Layout& L = z->layout;
    int32_t off = 0;
    bool seen[16] = {false};
    for (int32_t i = 0; i < num_items; i++) {
        const Item it{ld16(vlr + 34 + 6 * i), ld16(vlr + 36 + 6 * i), ld16(vlr + 38 + 6 * i)};
        z->info.item_type[i] = it.type;
        z->info.item_size[i] = it.size;
        z->info.item_version[i] = it.version;
        const bool v2 = (it.type == CR_LAZ_ITEM_POINT10 && it.size == 20) ||
                        (it.type == CR_LAZ_ITEM_GPSTIME11 && it.size == 8) ||
                        (it.type == CR_LAZ_ITEM_RGB12 && it.size == 6) ||
                        (it.type == CR_LAZ_ITEM_BYTE && it.size >= 1);
        const bool v3 = (it.type == CR_LAZ_ITEM_POINT14 && it.size == 30) ||
                        (it.type == CR_LAZ_ITEM_RGB14 && it.size == 6) ||
                        (it.type == CR_LAZ_ITEM_RGBNIR14 && it.size == 8) ||
                        (it.type == CR_LAZ_ITEM_BYTE14 && it.size >= 1);
        if (!(v2 && it.version == 2) && !(v3 && (it.version == 3 || it.version == 4))) st = CR_ERR_UNSUPPORTED;
        else if (seen[it.type]) st = CR_ERR_INVALID_ARG;
        else seen[it.type] = true;
        if (it.type == CR_LAZ_ITEM_RGB12 || it.type == CR_LAZ_ITEM_RGB14 || it.type == CR_LAZ_ITEM_RGBNIR14)
            L.rgb_offset = off;
        if (v3) L.layered = true;
        L.items.push_back(it);
        off += it.size;
    }
    if (compressor != CR_LAZ_POINTWISE && compressor != CR_LAZ_POINTWISE_CHUNKED &&
        compressor != CR_LAZ_LAYERED_CHUNKED)
        return CR_ERR_UNSUPPORTED;
    if (coder != 0) return CR_ERR_UNSUPPORTED;
    if (st != CR_OK) return st;
    if (off != z->info.las.bytes_per_point) return CR_ERR_INVALID_ARG;
    if (L.layered) {  // LAS 1.4 items: layered chunks, POINT14 first, no point-wise items
        if (compressor != CR_LAZ_LAYERED_CHUNKED || L.items[0].type != CR_LAZ_ITEM_POINT14 ||
            seen[CR_LAZ_ITEM_POINT10] || seen[CR_LAZ_ITEM_GPSTIME11] || seen[CR_LAZ_ITEM_RGB12] ||
            seen[CR_LAZ_ITEM_BYTE] || (seen[CR_LAZ_ITEM_RGB14] && seen[CR_LAZ_ITEM_RGBNIR14]))
            return CR_ERR_INVALID_ARG;
    } else if (!seen[CR_LAZ_ITEM_POINT10] || compressor == CR_LAZ_LAYERED_CHUNKED) {
        return CR_ERR_INVALID_ARG;
    }
    L.bpp = off;
    const int64_t n = z->info.las.num_points;
    if (points_at < pos || points_at > size) return CR_ERR_INVALID_ARG;
    if (compressor == CR_LAZ_POINTWISE) {  // one coder run over all points
        z->info.chunk_size = n;
        z->chunk_points = std::max<int64_t>(n, 1);
        z->chunk_start = {points_at, size};
        z->chunk_first = {0, n};
        z->info.num_chunks = n > 0 ? 1 : 0;
    } else {
        const bool variable = chunk_size == 0xFFFFFFFFu;
        if (!variable && chunk_size == 0) return CR_ERR_INVALID_ARG;
        z->info.chunk_size = variable ? CR_LAZ_VARIABLE_CHUNKS : (int64_t)chunk_size;
        z->chunk_points = variable ? 0 : (int64_t)chunk_size;
        if (points_at + 8 > size) return CR_ERR_INVALID_ARG;
        int64_t table_at = (int64_t)ld64(f + points_at);
        const int64_t chunks_at = points_at + 8;
        if (table_at == -1) {  // written to a stream that could not seek: the position is at the end
            if (size < chunks_at + 8) return CR_ERR_CORRUPT;
            table_at = (int64_t)ld64(f + size - 8);
        }
        if (table_at + 8 == chunks_at) {  // the writer stopped before writing its table
            if (variable) return CR_ERR_CORRUPT;
            z->sequential = true;
            z->chunk_start = {chunks_at};
            z->chunk_first = {0};
        } else {
            st = read_chunk_table(z.get(), table_at, chunks_at, variable, n);
            if (st != CR_OK) return st;
            z->info.num_chunks = (int64_t)z->chunk_first.size() - 1;
        }
    }
    if (info) *info = z->info;
    *out = z.release();
    return CR_OK;
}

cr_status cr_laz_close(cr_laz* laz) {
    delete laz;
    return CR_OK;
}

cr_status cr_laz_decode(const cr_laz* laz, int64_t first, int64_t n, void* records, int32_t threads) {
    if (!laz || first < 0 || n < 0 || first + n > laz->info.las.num_points || (n > 0 && !records))
        return CR_ERR_INVALID_ARG;
    return decode_range(laz, first, n, static_cast<uint8_t*>(records), threads);
}

// LasLoaderSparse.cpp:556-575 (load tasks) and :214-429 (loadLaz).
cr_status cr_cloud_load_laz(cr_ctx* ctx, cr_cloud* cloud, const cr_laz* laz, int64_t point_offset,
                            int64_t batch_offset, int32_t file_index, int32_t threads, void* stream) {
    if (!ctx || !cloud || !laz || point_offset < 0 || batch_offset < 0 || file_index < 0)
        return CR_ERR_INVALID_ARG;
    const int64_t n = laz->info.las.num_points;
    if (point_offset + n > cr_cloud_num_points(cloud) ||
        batch_offset + cr_las_num_batches(n) > cr_cloud_num_batches(cloud))
        return CR_ERR_INVALID_ARG;
    if (n == 0) return CR_OK;
    cr_batch* batches = nullptr;
    uint32_t *lo = nullptr, *md = nullptr, *hi = nullptr, *rgba = nullptr;
    cr_status s = cr_cloud_device(cloud, &batches, &lo, &md, &hi, &rgba);
    if (s != CR_OK || !lo || !md || !hi || !rgba) return CR_ERR_INVALID_ARG;

    const int64_t bpp = laz->layout.bpp, task = CR_MAX_POINTS_PER_LOAD;
    const int nthreads = resolve_threads(threads, 1 << 20);
    // windows of whole load tasks holding about four chunks per thread, and at
    // least the largest chunk (so a chunk touches at most two windows)
    int64_t max_chunk = laz->chunk_points > 0 ? laz->chunk_points : CR_LAZ_DEFAULT_CHUNK;
    for (size_t c = 0; c + 1 < laz->chunk_first.size(); c++)
        max_chunk = std::max(max_chunk, laz->chunk_first[c + 1] - laz->chunk_first[c]);
    int64_t window = std::max<int64_t>(1, (4 * nthreads * max_chunk + task - 1) / task) * task;
    window = std::max(window, (max_chunk + task - 1) / task * task);
    window = std::min(window, (n + task - 1) / task * task);
    const int64_t nwin = (n + window - 1) / window;
    const bool pipelined = !laz->sequential && laz->info.compressor != CR_LAZ_POINTWISE && nwin > 1;
    const int R = pipelined ? 3 : 2;  // host window slots
    uint8_t* host[3] = {nullptr, nullptr, nullptr};
    uint8_t* staging = nullptr;
    cudaEvent_t copied[3] = {nullptr, nullptr, nullptr};
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cudaMalloc(&staging, (size_t)(window * bpp));
    for (int r = 0; r < R && e == cudaSuccess; r++) {
        e = cudaHostAlloc(&host[r], (size_t)(window * bpp), cudaHostAllocDefault);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&copied[r], cudaEventDisableTiming);
    }
    if (e != cudaSuccess) s = e == cudaErrorMemoryAllocation ? CR_ERR_OUT_OF_MEMORY : CR_ERR_CUDA;
    int64_t b = batch_offset;
    // window wi's records in host[slot]: copied to the device and encoded task by task
    auto ship = [&](int64_t wi, int slot) -> cr_status {
        const int64_t w0 = wi * window, cnt = std::min(window, n - w0);
        if (cudaMemcpyAsync(staging, host[slot], (size_t)(cnt * bpp), cudaMemcpyHostToDevice, st) != cudaSuccess ||
            cudaEventRecord(copied[slot], st) != cudaSuccess)
            return CR_ERR_CUDA;
        for (int64_t t0 = 0; t0 < cnt; t0 += task) {
            const int64_t tc = std::min(task, cnt - t0);
            const int64_t p = point_offset + w0 + t0;
            const cr_status es = cr::encode_records_device(
                staging + t0 * bpp, tc, (int32_t)bpp, laz->layout.rgb_offset, laz->info.las.scale,
                laz->info.las.offset, laz->info.las.min, p, file_index, batches + b, lo + p, md + p, hi + p,
                rgba + p, st);
            if (es != CR_OK) return es;
            b += cr_num_batches(tc);
        }
        return CR_OK;
    };
    if (s == CR_OK && !pipelined) {
        // one window at a time, decoded while the previous one is copied and encoded
        for (int64_t wi = 0; s == CR_OK && wi < nwin; wi++) {
            const int slot = (int)(wi % R);
            if (wi >= R && cudaEventSynchronize(copied[slot]) != cudaSuccess) {
                s = CR_ERR_CUDA;
                break;
            }
            s = decode_range(laz, wi * window, std::min(window, n - wi * window), host[slot], nthreads);
            if (s == CR_OK) s = ship(wi, slot);
        }
    } else if (s == CR_OK) {
        // Every thread decodes chunks in file order into the slot of their
        // window (a chunk across a window border into both); this thread ships
        // each window once all its points are decoded, and hands the slot to
        // window wi + R once the copy has read it.
        const auto& cf = laz->chunk_first;
        const int64_t nchunks = (int64_t)cf.size() - 1;
        std::mutex mu;
        std::condition_variable cv;
        std::vector<int64_t> owner(R), left(nwin);
        for (int r = 0; r < R; r++) owner[r] = r < nwin ? r : -1;
        for (int64_t wi = 0; wi < nwin; wi++) left[wi] = std::min(window, n - wi * window);
        bool failed = false;
        std::atomic<int64_t> next(0);
        const uint8_t* file_end = laz->file + laz->size;
        auto worker = [&]() {
            PointCodec codec(laz->layout, true);
            std::vector<uint8_t> tmp;
            for (int64_t c = next++; c < nchunks; c = next++) {
                const int64_t clo = cf[c], chi = std::min(cf[c + 1], n);
                if (clo >= chi) continue;
                const int64_t wa = clo / window, wb = (chi - 1) / window;
                {
                    std::unique_lock<std::mutex> lk(mu);
                    cv.wait(lk, [&] { return failed || (owner[wa % R] == wa && owner[wb % R] == wb); });
                    if (failed) return;
                }
                const int64_t count = cf[c + 1] - clo;
                uint8_t* dst;
                if (wa == wb) {
                    dst = host[wa % R] + (clo - wa * window) * bpp;
                } else {
                    tmp.resize((size_t)((chi - clo) * bpp));
                    dst = tmp.data();
                }
                const uint8_t* end = nullptr;
                const bool ok = codec.decode_chunk(laz->file + laz->chunk_start[c], file_end, count, 0, chi - clo,
                                                   chi - clo, dst, &end) &&
                                (chi - clo < count || end == laz->file + laz->chunk_start[c + 1]);
                if (ok && wa != wb) {  // split across the border
                    const int64_t border = wb * window;
                    std::memcpy(host[wa % R] + (clo - wa * window) * bpp, tmp.data(), (size_t)((border - clo) * bpp));
                    std::memcpy(host[wb % R], tmp.data() + (border - clo) * bpp, (size_t)((chi - border) * bpp));
                }
                std::lock_guard<std::mutex> lk(mu);
                if (!ok) failed = true;
                left[wa] -= std::min(chi, (wa + 1) * window) - clo;
                if (wb != wa) left[wb] -= chi - wb * window;
                cv.notify_all();
            }
        };
        std::vector<std::thread> pool;
        for (int t = 0; t < nthreads; t++) pool.emplace_back(worker);
        for (int64_t wi = 0; wi < nwin && s == CR_OK; wi++) {
            {
                std::unique_lock<std::mutex> lk(mu);
                cv.wait(lk, [&] { return failed || left[wi] == 0; });
                if (failed) s = CR_ERR_CORRUPT;
            }
            const int slot = (int)(wi % R);
            if (s == CR_OK) s = ship(wi, slot);
            if (s == CR_OK && cudaEventSynchronize(copied[slot]) != cudaSuccess) s = CR_ERR_CUDA;
            std::lock_guard<std::mutex> lk(mu);
            if (s != CR_OK) failed = true;
            else if (wi + R < nwin) owner[slot] = wi + R;
            cv.notify_all();
        }
        for (auto& th : pool) th.join();
    }
    if (cudaStreamSynchronize(st) != cudaSuccess && s == CR_OK) s = CR_ERR_CUDA;
    for (cudaEvent_t ev : copied)
        if (ev) cudaEventDestroy(ev);
    if (staging) cudaFree(staging);
    for (uint8_t* h : host)
        if (h) cudaFreeHost(h);
    cudaGetLastError();
    return s;
}

// laszip.cpp pack: compressor, coder, version, options, chunk size, special
// EVLR count and offset (-1: none), the items.  The version fields are those
// of the LASzip the reference vendors (3.4 r3), whose bytes the writer below
// reproduces.
cr_status cr_laz_vlr(int32_t point_format, int32_t bytes_per_point, int64_t chunk_size, uint8_t* out,
                     int64_t cap, int64_t* len) {
    Layout L;
    cr_status st = layout_for(point_format, bytes_per_point, &L);
    if (st != CR_OK) return st;
    if (!len || (chunk_size != CR_LAZ_VARIABLE_CHUNKS && (chunk_size <= 0 || chunk_size >= 0xFFFFFFFFll)))
        return CR_ERR_INVALID_ARG;
    const int64_t need = 34 + 6 * (int64_t)L.items.size();
    *len = need;
    if (!out || cap < need) return CR_ERR_INVALID_ARG;
    std::memset(out, 0, (size_t)need);
    st16(out, CR_LAZ_POINTWISE_CHUNKED);
    st16(out + 2, 0);
    out[4] = 3;
    out[5] = 4;
    st16(out + 6, 3);
    st32(out + 8, 0);
    st32(out + 12, chunk_size == CR_LAZ_VARIABLE_CHUNKS ? 0xFFFFFFFFu : (uint32_t)chunk_size);
    st64(out + 16, ~0ull);
    st64(out + 24, ~0ull);
    st16(out + 32, (uint16_t)L.items.size());
    for (size_t i = 0; i < L.items.size(); i++) {
        st16(out + 34 + 6 * i, (uint16_t)L.items[i].type);
        st16(out + 36 + 6 * i, (uint16_t)L.items[i].size);
        st16(out + 38 + 6 * i, (uint16_t)L.items[i].version);
    }
    return CR_OK;
}

int64_t cr_laz_compress_bound(int64_t n, int32_t bytes_per_point, int64_t chunk_size) {
    if (n < 0 || bytes_per_point <= 0) return -1;
    const int64_t chunks = chunk_size > 0 ? (n + chunk_size - 1) / chunk_size : n;
    return 64 + n * (2 * (int64_t)bytes_per_point + 32) + chunks * ((int64_t)bytes_per_point + 64);
}

// laswritepoint.cpp: the chunk table pointer, the chunks, the chunk table.
cr_status cr_laz_compress(const void* records, int64_t n, int32_t point_format, int32_t bytes_per_point,
                          int64_t chunk_size, int64_t var_chunk, int64_t points_at, uint8_t* out,
                          int64_t cap, int64_t* len, int32_t threads) {
    Layout L;
    cr_status st = layout_for(point_format, bytes_per_point, &L);
    if (st != CR_OK) return st;
    const bool variable = chunk_size == CR_LAZ_VARIABLE_CHUNKS;
    if (!len || n < 0 || (n > 0 && !records) || points_at < 0 || (variable && var_chunk <= 0) ||
        (!variable && (chunk_size <= 0 || chunk_size >= 0xFFFFFFFFll)))
        return CR_ERR_INVALID_ARG;
    const int64_t step = variable ? var_chunk : chunk_size;
    const int64_t chunks = (n + step - 1) / step;
    std::vector<std::vector<uint8_t>> parts((size_t)chunks);
    std::atomic<int64_t> next(0);
    const uint8_t* rec = static_cast<const uint8_t*>(records);
    run_workers(resolve_threads(threads, chunks), [&](int) {
        PointCodec codec(L, false);
        for (int64_t c = next++; c < chunks; c = next++) {
            const int64_t lo = c * step, count = std::min(step, n - lo);
            codec.encode_chunk(rec + lo * bytes_per_point, count, parts[(size_t)c]);
        }
    });
    std::vector<uint8_t> table;
    if (chunks > 0) {
        Encoder e;
        e.start(&table);
        IntCoder ic;
        ic.create(32, 2, false);
        ic.reset();
        for (int64_t c = 0; c < chunks; c++) {
            const int64_t count = std::min(step, n - c * step);
            const int64_t prev_count = c ? std::min(step, n - (c - 1) * step) : 0;
            if (variable) ic.encode(e, (int32_t)prev_count, (int32_t)count, 0);
            ic.encode(e, c ? (int32_t)parts[(size_t)c - 1].size() : 0, (int32_t)parts[(size_t)c].size(), 1);
        }
        e.finish();
    }
    int64_t body = 0;
    for (const auto& p : parts) body += (int64_t)p.size();
    const int64_t total = 8 + body + 8 + (int64_t)table.size();
    *len = total;
    if (!out || cap < total) return CR_ERR_INVALID_ARG;
    st64(out, (uint64_t)(points_at + 8 + body));
    uint8_t* w = out + 8;
    for (const auto& p : parts) {
        std::memcpy(w, p.data(), p.size());
        w += p.size();
    }
    st32(w, 0);
    st32(w + 4, (uint32_t)chunks);
    if (!table.empty()) std::memcpy(w + 8, table.data(), table.size());
    return CR_OK;
}

}  // extern "C"
