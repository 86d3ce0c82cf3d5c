// Host check of lighthugger_gb300/csrc/exact_div.cuh: div_by_count against
// the IEEE single-precision quotient for every 0 <= x <= n <= 16384.
#include <cstdint>
#include <cstdio>
#include <cstring>

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
    std::printf("checked %lld bad %lld\n", checked, bad);
    return bad == 0 ? 0 : 1;
}
