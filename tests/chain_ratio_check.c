/* The chaining kernel's diagonal test without division (ChainCtx::ratio_above in
 * strobealign_gb300/csrc/nams.cu) against the reference's f32 quotient
 * (src/chainer.rs:124-130: (max / min) as f32 > max_diagonal_ratio), for integer
 * differences below 2^24: R = M * 2^e with M the 24-bit significand; the quotient
 * rounds above R exactly when mx * 2^(1 - e) > mn * (2M + 1) (>= when M is odd),
 * and never when mx = 0 (0 / 0 is NaN). */
#include <math.h>
#include <stdint.h>
#include <stdio.h>

static int above_int(uint32_t mx, uint32_t mn, uint32_t shift, uint64_t num, int strict) {
    const uint64_t lhs = (uint64_t)mx << shift, rhs = (uint64_t)mn * num;
    return mx != 0 && (strict ? lhs > rhs : lhs >= rhs);
}

int main(void) {
    const float Rs[] = {10.0f, 1.5f, 3.0f, 7.3f, 2.0f, 1.0f, 100.0f, 0.7f, 12.345f};
    long bad = 0, tot = 0;
    for (unsigned t = 0; t < sizeof Rs / sizeof Rs[0]; t++) {
        const float R = Rs[t];
        int ex = 0;
        const float fr = frexpf(R, &ex);
        const uint64_t M = (uint64_t)ldexp((double)fr, 24);
        const int e = ex - 24, shift = 1 - e;
        const int strict = (M & 1) == 0;
        if (!(M >= (1u << 23) && M < (1u << 24) && shift >= 0 && shift <= 30)) continue;
        for (uint32_t mx = 0; mx < 2500; mx++)
            for (uint32_t mn = 0; mn <= mx; mn++) {
                volatile float a = (float)mx, b = (float)mn;
                const int ref = (a / b) > R;
                tot++;
                if (ref != above_int(mx, mn, (uint32_t)shift, 2 * M + 1, strict)) bad++;
            }
        for (uint32_t mn = 1; mn < 2000000; mn += 7919) {
            const uint32_t c = (uint32_t)(R * (float)mn);
            for (uint32_t mx = c > 3 ? c - 3 : 0; mx < c + 4 && mx < (1u << 24); mx++) {
                volatile float a = (float)mx, b = (float)mn;
                const int ref = (a / b) > R;
                tot++;
                if (ref != above_int(mx, mn, (uint32_t)shift, 2 * M + 1, strict)) bad++;
            }
        }
    }
    printf("checked %ld, mismatches %ld\n", tot, bad);
    return bad != 0;
}
