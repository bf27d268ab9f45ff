/* Exhaustive check of the correctly rounded division by the wavelength range
 * (470) that the device code computes with two fused multiply-adds (method of
 * Brisebarre, Muller and Raina, IEEE Trans. Computers 53(8), 2004): for every
 * float x in [2^-20, 2048], RN(q + RN(x - q * 470) * z) with z = RN(1/470)
 * and q = RN(x * z) must equal the IEEE quotient RN(x / 470).  Build with
 * -ffp-contract=off so that only the explicit fmaf calls fuse. */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

int main(void) {
    const float y = 470.0f;
    const float z = 1.0f / y;
    const float lo = 0x1p-20f, hi = 2048.0f;
    uint32_t ulo, uhi;
    memcpy(&ulo, &lo, 4);
    memcpy(&uhi, &hi, 4);
    unsigned long long bad = 0, n = 0;
    for (uint32_t u = ulo; u <= uhi; ++u) {
        float x;
        memcpy(&x, &u, 4);
        const float q = x * z;
        const float r = fmaf(-q, y, x);
        const float got = fmaf(r, z, q);
        const float want = x / y;
        ++n;
        if (memcmp(&got, &want, 4) != 0) {
            if (bad < 5) printf("x=%a got %a want %a\n", x, got, want);
            ++bad;
        }
    }
    {   /* zero divides exactly */
        const float x = 0.0f, q = x * z, got = fmaf(fmaf(-q, y, x), z, q);
        if (got != 0.0f) ++bad;
    }
    printf("checked %llu mismatches %llu\n", n, bad);
    return bad != 0;
}
