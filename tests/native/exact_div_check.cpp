// Host check of lighthugger_gb300/csrc/exact_div.cuh: div_by_count against
// the IEEE single-precision quotient for every integer pair
// 0 <= x <= n <= 16384 and every float 0 <= x <= 9 divided by 9.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <thread>
#include <vector>

#include "exact_div.cuh"

int main() {
    long long checked = 0, bad = 0;
    for (int n = 1; n <= lh::kExactDivMaxCount; n++) {
        const float nf = (float)n, rcp = 1.0f / nf;
        for (int x = 0; x <= n; x++) {
            const float xf = (float)x;
            const float q = lh::div_by_count(xf, nf, rcp), ref = xf / nf;
            uint32_t a, b;
            std::memcpy(&a, &q, 4);
            std::memcpy(&b, &ref, 4);
            checked++;
            if (a != b) {
                if (bad < 10) std::printf("n %d x %d: %a against %a\n", n, x, q, ref);
                bad++;
            }
        }
    }
    // every float in [0, 9] divided by 9 (16 threads over the bit patterns)
    {
        const float nine = 9.0f, rcp = 1.0f / nine;
        uint32_t hi;
        std::memcpy(&hi, &nine, 4);
        const uint32_t parts = 16;
        long long part_bad[parts] = {};
        std::vector<std::thread> pool;
        for (uint32_t t = 0; t < parts; t++)
            pool.emplace_back([&, t] {
                for (uint64_t b = t; b <= hi; b += parts) {
                    float x;
                    const uint32_t bits = (uint32_t)b;
                    std::memcpy(&x, &bits, 4);
                    const float q = lh::div_by_count(x, nine, rcp), ref = x / nine;
                    uint32_t qa, qb;
                    std::memcpy(&qa, &q, 4);
                    std::memcpy(&qb, &ref, 4);
                    if (qa != qb) part_bad[t]++;
                }
            });
        for (auto& th : pool) th.join();
        for (uint32_t t = 0; t < parts; t++) bad += part_bad[t];
        checked += (long long)hi + 1;
    }
    std::printf("checked %lld bad %lld\n", checked, bad);
    return bad == 0 ? 0 : 1;
}
