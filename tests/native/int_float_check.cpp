// Host check of lighthugger_gb300/csrc/int_float.cuh: the integer and FP32
// pipe conversions must equal the round-to-nearest-even conversion
// (static_cast<float>) for every 32-bit edge value class and for 64-bit
// values (signed, and non-negative below 2^46) around each power of two,
// halfway cases included.
#include <cstdio>
#include <cstring>
#include <random>

#include "int_float.cuh"

static uint32_t bits(float f) {
    uint32_t b;
    std::memcpy(&b, &f, 4);
    return b;
}

int main() {
    long long bad = 0, n = 0;
    auto check64 = [&](int64_t v) {
        n++;
        if (bits(lh::i64_to_f32_rn(v)) != bits(static_cast<float>(v))) {
            if (bad < 10) std::printf("i64 %lld: %a vs %a\n", (long long)v, lh::i64_to_f32_rn(v), static_cast<float>(v));
            bad++;
        }
    };
    auto check46 = [&](uint64_t v) {
        n++;
        if (bits(lh::u46_to_f32_rn(v)) != bits(static_cast<float>(v))) {
            if (bad < 10) std::printf("u46 %llu: %a vs %a\n", (unsigned long long)v, lh::u46_to_f32_rn(v), static_cast<float>(v));
            bad++;
        }
    };
    auto checku32 = [&](uint32_t v) {
        n++;
        if (bits(lh::u32_to_f32_rn(v)) != bits(static_cast<float>(v))) {
            if (bad < 10) std::printf("u32 %u: %a vs %a\n", v, lh::u32_to_f32_rn(v), static_cast<float>(v));
            bad++;
        }
    };
    auto check32 = [&](int32_t v) {
        n++;
        if (bits(lh::i32_to_f32_rn(v)) != bits(static_cast<float>(v))) {
            if (bad < 10) std::printf("i32 %d: %a vs %a\n", v, lh::i32_to_f32_rn(v), static_cast<float>(v));
            bad++;
        }
    };
    // every value near zero and around the fast-path limit 2^22
    for (int32_t v = -(1 << 20); v <= (1 << 20); v++) check32(v);
    for (int32_t d = -4096; d <= 4096; d++) {
        check32((1 << 22) + d);
        check32(-(1 << 22) + d);
        check32((1 << 24) + d);
        check32(-(1 << 24) + d);
    }
    check32(INT32_MAX);
    check32(INT32_MIN);
    // 64-bit: around every power of two, with the halfway and sticky bits
    for (int e = 0; e < 63; e++) {
        const int64_t p = (int64_t)1 << e;
        for (int64_t d = -70; d <= 70; d++) {
            check64(p + d);
            check64(-(p + d));
        }
        if (e > 24) {
            const int64_t ulp = (int64_t)1 << (e - 23);
            for (int64_t k = 1; k < 40; k++) {
                check64(p + k * ulp / 2);      // exact halves
                check64(p + k * ulp / 2 + 1);  // just above
                check64(p + k * ulp / 2 - 1);  // just below
                check64(-(p + k * ulp / 2));
            }
        }
    }
    check64(INT64_MAX);
    check64(INT64_MIN);
    // non-negative values below 2^46 (the covered edge values of chunks)
    for (uint64_t v = 0; v <= (1u << 20); v++) check46(v);
    for (int e = 1; e < 46; e++) {
        const uint64_t p = 1ull << e;
        for (int64_t d = -70; d <= 70; d++)
            if ((int64_t)p + d >= 0 && p + d < (1ull << 46)) check46(p + d);
        if (e > 24) {
            const uint64_t ulp = 1ull << (e - 23);
            for (uint64_t k = 1; k < 40; k++) {
                check46(p + k * ulp / 2);
                check46(p + k * ulp / 2 + 1);
                check46(p + k * ulp / 2 - 1);
            }
        }
    }
    check46((1ull << 46) - 1);
    for (int e = 0; e < 32; e++)
        for (int64_t d = -70; d <= 70; d++)
            if ((int64_t)(1ull << e) + d >= 0 && (1ull << e) + d <= 0xFFFFFFFFull) checku32((uint32_t)((1ull << e) + d));
    checku32(0xFFFFFFFFu);
    std::mt19937_64 rng(7);
    for (int i = 0; i < 2000000; i++) {
        const uint64_t r = rng();
        const int shift = (int)(r & 63);
        check64((int64_t)(rng() >> shift) * ((r >> 6) & 1 ? -1 : 1));
        check32((int32_t)(rng() >> (32 + (r >> 8) % 32)) * ((r >> 7) & 1 ? -1 : 1));
        check46(rng() >> (18 + (r >> 13) % 46));
        checku32((uint32_t)(rng() >> (32 + (r >> 19) % 32)));
    }
    std::printf("checked %lld bad %lld\n", n, bad);
    return bad == 0 ? 0 : 1;
}
