// Host restatement of the literal pair body's division (f2_neg_div_rn in
// compute_rasterizer_gb300/csrc/cr_device.cuh) on the quotients that
// cr_check_reciprocal draws (cr_divcheck.h), against C's correctly rounded
// division.  Prints "checked N hard H two_step_bad B one_step_bad O product_bad P":
// the two-step form must have no mismatch; the bare product RN(a * RN(1/x))
// must miss on the hard quotients, which shows that they sit where rounding
// is delicate.
#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "../../compute_rasterizer_gb300/csrc/cr_divcheck.h"

int main(int argc, char** argv) {
    const uint32_t stride = argc > 1 ? (uint32_t)strtoul(argv[1], nullptr, 10) : 97u;
    unsigned long long checked = 0, hard = 0, bad2 = 0, bad1 = 0, bad0 = 0;
    // every stride-th float with |x| in [2^-64, 2^64), both signs
    for (uint64_t i = (uint64_t)63u << 23; i < (uint64_t)191u << 23; i += stride) {
        for (uint32_t sign = 0; sign < 2; sign++) {
            const uint32_t xb = (uint32_t)i | (sign << 31);
            const float x = cr::divcheck_bits(xb);
            const float nr = -(1.0f / x);  // -RN(1/x)
            for (int k = 0; k < 2; k++) {
                const bool is_hard = k == 0 && (xb & 1u);
                const float a = cr::divcheck_numerator(xb, k == 0);
                const float q = a / x;
                const float nq0 = a * nr;
                const float nq1 = std::fmaf(std::fmaf(nq0, x, a), nr, nq0);
                const float nq2 = std::fmaf(std::fmaf(nq1, x, a), nr, nq1);
                checked++;
                hard += is_hard;
                bad2 += !cr::divcheck_quotient_ok(q, nq2);
                bad1 += !cr::divcheck_quotient_ok(q, nq1);
                bad0 += is_hard && !cr::divcheck_quotient_ok(q, nq0);
            }
        }
    }
    printf("checked %llu hard %llu two_step_bad %llu one_step_bad %llu product_bad %llu\n", checked,
           hard, bad2, bad1, bad0);
    return bad2 == 0 ? 0 : 1;
}
