// CPU check of the MPGOS_DF_TRIG_BOUNDED forms in csrc/perthread/dfloat.cuh
// (compiled for the host by tests/test_dfloat_cpu.py with -ffp-contract=off,
// once as is and once with -DMPGOS_DF_TRIG_BOUNDED).
//
// Arguments of random sign, magnitudes log-uniform over 2^-30 .. 2^20 (both
// sides of the bounds 2^14 and 2^16) with random low parts, plus zero,
// infinities and NaN. Prints one count per line:
//   bounded_in_differs   bounded sin/cos (sincospi) differ in some bit from the
//                        table path the default build takes inside the bound
//   bounded_out_not_nan  arguments outside the bound (or not finite) whose
//                        bounded result is not NaN in both parts
//   public_differs       the public sin, cos, sincos and sincospi differ from
//                        the bounded forms (counted in the bounded build only)
//   inside, outside      how many arguments fell on either side
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>

#include "dfloat.cuh"

using mpgos::df::dfloat;

static bool same_bits(dfloat a, dfloat b)
{
    return std::memcmp(&a.hi, &b.hi, sizeof(float)) == 0 && std::memcmp(&a.lo, &b.lo, sizeof(float)) == 0;
}

static bool both_nan(dfloat a) { return std::isnan(a.hi) && std::isnan(a.lo); }

int main()
{
    namespace D = mpgos::df::detail;
    std::mt19937_64 gen(20261204);
    std::uniform_real_distribution<double> expo(-30.0, 20.0), unit(-1.0, 1.0);
    long in_differs = 0, out_not_nan = 0, public_differs = 0, inside = 0, outside = 0;
    const int n = 400000;
    for (int i = 0; i < n + 6; i++) {
        dfloat x;
        if (i < n) {
            const float hi = static_cast<float>((unit(gen) < 0 ? -1.0 : 1.0) * std::exp2(expo(gen)));
            const float lo = static_cast<float>(unit(gen) * std::ldexp(1.0, std::ilogb(hi) - 25));
            x = mpgos::df::quick_two_sum(hi, lo);
        } else {
            const float special[6] = {0.0f, -0.0f, INFINITY, -INFINITY, NAN, 0x1p14f};
            x = dfloat(special[i - n], 0.0f);
        }
        dfloat sb, cb, pb_s, pb_c;
        D::sincos_bounded(x, &sb, &cb);
        D::sincospi_bounded(x, &pb_s, &pb_c);
        // sin / cos
        if (std::fabs(x.hi) < D::TRIG_TABLE_LIMIT) {
            inside++;
            int k;
            const dfloat r = D::reduce_pio128(x, k);
            dfloat s, c;
            D::sincos_table(r, k, &s, &c);
            if (!same_bits(s, sb) || !same_bits(c, cb)) in_differs++;
        } else {
            outside++;
            if (!both_nan(sb) || !both_nan(cb)) out_not_nan++;
        }
        // sincospi
        if (std::fabs(x.hi) < D::TRIGPI_TABLE_LIMIT) {
            dfloat s, c;
            D::sincospi_table(x, &s, &c);
            if (!same_bits(s, pb_s) || !same_bits(c, pb_c)) in_differs++;
        } else if (!both_nan(pb_s) || !both_nan(pb_c)) {
            out_not_nan++;
        }
#ifdef MPGOS_DF_TRIG_BOUNDED
        dfloat s2, c2, ps, pc;
        mpgos::df::sincos(x, &s2, &c2);
        mpgos::df::sincospi(x, &ps, &pc);
        const dfloat s1 = mpgos::df::sin(x), c1 = mpgos::df::cos(x);
        const bool nan_ok = both_nan(sb) && both_nan(s1) && both_nan(c1) && both_nan(s2) && both_nan(c2);
        if (!nan_ok && !(same_bits(s1, sb) && same_bits(c1, cb) && same_bits(s2, sb) && same_bits(c2, cb)))
            public_differs++;
        if (!(both_nan(pb_s) && both_nan(ps) && both_nan(pc)) && !(same_bits(ps, pb_s) && same_bits(pc, pb_c)))
            public_differs++;
#endif
    }
    std::printf("bounded_in_differs %ld\nbounded_out_not_nan %ld\npublic_differs %ld\ninside %ld\noutside %ld\n",
                in_differs, out_not_nan, public_differs, inside, outside);
    return 0;
}
