// CPU check of the double-float arithmetic in csrc/perthread/dfloat.cuh
// (compiled for the host by tests/test_dfloat_cpu.py with -ffp-contract=off).
// Random operands of mixed sign and magnitude; each operation is compared with
// the same operation in long double on the exact values hi + lo of the inputs.
// Prints one line per operation: name, max relative error (to the larger of
// the result and the operands' magnitude, the bound of a "sloppy" add).
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <random>
#include <string>
#include <vector>

#include "df_convert.cuh"

using mpgos::df::dfloat;

static long double val(dfloat a) { return (long double)a.hi + (long double)a.lo; }

// "eval" mode: read int32 op, int64 n, double a[n], double b[n] from stdin and
// write op(dfloat(a), dfloat(b)) as n pairs of doubles (hi, lo) to stdout; the
// same operation codes as mpgos_probe_df_math (the device build), so a test can
// compare the two builds bit for bit.
static int eval_mode()
{
    int32_t op = 0;
    int64_t n = 0;
    if (std::fread(&op, sizeof(op), 1, stdin) != 1 || std::fread(&n, sizeof(n), 1, stdin) != 1 || n < 0) return 2;
    std::vector<double> a(n), b(n), out(2 * n);
    if (std::fread(a.data(), sizeof(double), n, stdin) != (size_t)n ||
        std::fread(b.data(), sizeof(double), n, stdin) != (size_t)n)
        return 2;
    for (int64_t i = 0; i < n; i++) {
        if (op == 12) {   // the SPLIT mode's integer-pipe conversion of the double itself
            const dfloat r = mpgos::df::split(a[i]);
            out[2 * i] = r.hi;
            out[2 * i + 1] = r.lo;
            continue;
        }
        const dfloat x(a[i]), y(b[i]);
        dfloat r;
        switch (op) {
            case 0: r = mpgos::df::exp(x); break;
            case 1: r = mpgos::df::log(x); break;
            case 2: r = mpgos::df::pow(x, y); break;
            case 3: r = mpgos::df::sin(x); break;
            case 4: r = mpgos::df::cos(x); break;
            case 5: r = mpgos::df::sqrt(x); break;
            case 6: r = x / y; break;
            case 7: r = x * y; break;
            case 8: r = x + y; break;
            case 10: { dfloat c; mpgos::df::sincospi(x, &r, &c); break; }
            case 11: { dfloat s; mpgos::df::sincospi(x, &s, &r); break; }
            default: r = mpgos::df::pow(x, static_cast<int>(b[i])); break;
        }
        out[2 * i] = r.hi;
        out[2 * i + 1] = r.lo;
    }
    std::fwrite(out.data(), sizeof(double), out.size(), stdout);
    return 0;
}

int main(int argc, char** argv)
{
    if (argc > 1 && std::string(argv[1]) == "eval") return eval_mode();
    std::mt19937_64 rng(12345);
    std::uniform_real_distribution<double> u(-1.0, 1.0), e(-8.0, 8.0);
    auto draw = [&]() { return dfloat(u(rng) * std::pow(2.0, std::floor(e(rng)))); };
    double m_add = 0, m_mul = 0, m_div = 0, m_sqrt = 0, m_cvt = 0, m_cmp = 0, m_norm = 0, m_fma = 0, m_dot = 0;
    double m_psum = 0, m_paxpy = 0;
    for (int n = 0; n < 200000; n++) {
        const dfloat a = draw(), b = draw();
        const long double A = val(a), B = val(b);
        const long double scale_add = std::fabs(A) + std::fabs(B);
        const dfloat s = a + b, p = a * b, q = a / b, r = mpgos::df::sqrt(mpgos::df::abs(a));
        m_add = std::fmax(m_add, (double)(std::fabs(val(s) - (A + B)) / scale_add));
        m_mul = std::fmax(m_mul, (double)(std::fabs(val(p) - A * B) / std::fabs(A * B)));
        m_div = std::fmax(m_div, (double)(std::fabs(val(q) - A / B) / std::fabs(A / B)));
        m_sqrt = std::fmax(m_sqrt, (double)(std::fabs(val(r) - std::sqrt(std::fabs(A))) / std::sqrt(std::fabs(A))));
        // fused forms, error relative to the sum of the terms' magnitudes
        const dfloat c = draw(), dd = draw();
        const long double C = val(c), D = val(dd);
        const dfloat f = mpgos::df::fma(a, b, c), g = mpgos::df::dot2(a, b, c, dd);
        // five-term product sum and c + a * (sum), unnormalised in between
        {
            const dfloat e = draw(), h = draw(), q = draw(), w = draw(), z = draw(), y = draw();
            mpgos::df::prod_sum ps = mpgos::df::prod_sum_start(a, b);
            mpgos::df::prod_sum_add(ps, c, dd);
            mpgos::df::prod_sum_add(ps, e, h);
            mpgos::df::prod_sum_add(ps, q, w);
            mpgos::df::prod_sum_add(ps, z, y);
            const long double E = val(e), H = val(h), Q = val(q), W = val(w), Z = val(z), Y = val(y);
            const long double exact = A * B + C * D + E * H + Q * W + Z * Y;
            const long double mag = std::fabs(A * B) + std::fabs(C * D) + std::fabs(E * H) + std::fabs(Q * W) +
                                    std::fabs(Z * Y);
            m_psum = std::fmax(m_psum, (double)(std::fabs(val(mpgos::df::prod_sum_value(ps)) - exact) / mag));
            const dfloat ax = mpgos::df::prod_sum_axpy(e, ps, h);
            const long double ex2 = E * exact + H;
            m_paxpy = std::fmax(m_paxpy, (double)(std::fabs(val(ax) - ex2) / (std::fabs(E) * mag + std::fabs(H))));
        }
        m_fma = std::fmax(m_fma, (double)(std::fabs(val(f) - (A * B + C)) / (std::fabs(A * B) + std::fabs(C))));
        m_dot = std::fmax(m_dot, (double)(std::fabs(val(g) - (A * B + C * D)) / (std::fabs(A * B) + std::fabs(C * D))));
        // normalisation: |lo| <= ulp(hi) / 2 after every operation
        for (dfloat z : {s, p, q, r, f, g})
            if (z.hi != 0.0f) m_norm = std::fmax(m_norm, std::fabs(z.lo) / (std::nextafter(std::fabs(z.hi), INFINITY) - std::fabs(z.hi)));
        // conversion from double keeps 48 bits
        const double d = u(rng) * std::pow(2.0, std::floor(e(rng)));
        m_cvt = std::fmax(m_cvt, std::fabs((double)dfloat(d) - d) / std::fabs(d));
        // comparisons agree with the exact values
        if (((a < b) != (A < B)) || ((a > b) != (A > B)) || ((a <= b) != (A <= B))) m_cmp = 1;
    }
    // sin / cos: error relative to |x| 2^-48 + 2^-50 (the argument's own precision)
    double m_trig = 0, m_trig_small = 0;
    std::uniform_real_distribution<double> wide(-2000.0, 2000.0), narrow(-1.0, 1.0);
    for (int n = 0; n < 200000; n++) {
        const dfloat x = dfloat(n % 2 ? wide(rng) : narrow(rng));
        const long double X = val(x);
        const long double bound = std::fabs(X) * std::ldexp(1.0L, -48) + std::ldexp(1.0L, -50);
        const double es = (double)(std::fabs(val(mpgos::df::sin(x)) - std::sin(X)) / bound);
        const double ec = (double)(std::fabs(val(mpgos::df::cos(x)) - std::cos(X)) / bound);
        m_trig = std::fmax(m_trig, std::fmax(es, ec));
        if (std::fabs(X) < 1.0L)
            m_trig_small = std::fmax(m_trig_small, (double)std::fmax(std::fabs(val(mpgos::df::sin(x)) - std::sin(X)),
                                                                     std::fabs(val(mpgos::df::cos(x)) - std::cos(X))));
    }
    // sincospi: absolute error (the reduction by halves is exact, so it does not grow with |x|)
    double m_trigpi = 0;
    const long double PI = std::acos(-1.0L);
    for (int n = 0; n < 200000; n++) {
        const dfloat x = dfloat(n % 2 ? wide(rng) : narrow(rng));
        const long double X = val(x);
        dfloat s, c;
        mpgos::df::sincospi(x, &s, &c);
        // reduce X exactly by halves before the long double sin/cos
        const long double k = std::nearbyint(2.0L * X), f = X - 0.5L * k;
        const int q = (int)std::fmod(std::fmod(k, 4.0L) + 4.0L, 4.0L);
        const long double sf = std::sin(PI * f), cf = std::cos(PI * f);
        const long double S = q == 0 ? sf : q == 1 ? cf : q == 2 ? -sf : -cf;
        const long double C = q == 0 ? cf : q == 1 ? -sf : q == 2 ? -cf : sf;
        m_trigpi = std::fmax(m_trigpi, (double)std::fmax(std::fabs(val(s) - S), std::fabs(val(c) - C)));
    }
    // exp, log, pow: exp relative to 2^-48 (|x| + 1) (the argument's own
    // precision carried through; results above 2^-100, where the low float
    // is still normal), log relative to 2^-48 (|log a| + 1), pow relative to
    // 2^-48 (|b log a| + 1)
    double m_exp = 0, m_log = 0, m_pow = 0, m_powi = 0, m_fallback = 0;
    std::uniform_real_distribution<double> ex(-69.0, 80.0), small(-1.0, 1.0), lg(-30.0, 30.0), pb(-6.0, 6.0);
    for (int n = 0; n < 200000; n++) {
        const dfloat x = dfloat(n % 2 ? ex(rng) : small(rng));
        const long double X = val(x);
        const long double ulp48 = std::ldexp(1.0L, -48);
        m_exp = std::fmax(m_exp, (double)(std::fabs(val(mpgos::df::exp(x)) - std::exp(X)) / std::exp(X) /
                                          (ulp48 * (std::fabs(X) + 1.0L))));
        const dfloat a = dfloat(std::exp((double)lg(rng)) * (n % 3 ? 1.0 : 1.0 + 1e-3 * small(rng)));
        const long double A = val(a);
        m_log = std::fmax(m_log, (double)(std::fabs(val(mpgos::df::log(a)) - std::log(A)) /
                                          (ulp48 * (std::fabs(std::log(A)) + 1.0L))));
        const dfloat b = dfloat(pb(rng));
        const long double B = val(b);
        if (std::fabs(B * std::log(A)) < 69.0L) {
            const long double P = std::pow(A, B);
            m_pow = std::fmax(m_pow, (double)(std::fabs(val(mpgos::df::pow(a, b)) - P) / P /
                                              (ulp48 * (std::fabs(B * std::log(A)) + 1.0L))));
        }
        const int k = n % 13 - 6;
        const dfloat c = dfloat(0.5 + small(rng));
        const long double Pc = std::pow(val(c), (long double)k);
        m_powi = std::fmax(m_powi, (double)(std::fabs(val(mpgos::df::pow(c, k)) - Pc) / std::fabs(Pc)));
    }
    // arguments outside the FP32-pipe ranges take the FP64 path
    for (double v : {-100.0, 85.0, 100.0}) {
        const double got = (double)mpgos::df::exp(dfloat(v)), want = (double)dfloat(std::exp(v));
        if (!(got == want || (std::isinf(got) && std::isinf(want)))) m_fallback = 1;
    }
    if (!std::isnan((double)mpgos::df::log(dfloat(-1.0))) || !std::isinf((double)mpgos::df::log(dfloat(0.0))))
        m_fallback = 1;
    if ((double)mpgos::df::pow(dfloat(-2.0), dfloat(3.0)) != -8.0) m_fallback = 1;
    std::printf("add %.3e\nmul %.3e\ndiv %.3e\nsqrt %.3e\ncvt %.3e\ncmp %.0f\nnorm %.3f\ntrig %.3f\ntrig_small %.3e\n"
                "fma %.3e\ndot2 %.3e\nprod_sum %.3e\nprod_sum_axpy %.3e\nexp %.3f\nlog %.3f\npow %.3f\n"
                "pow_int %.3e\nfallback %.0f\ntrigpi %.3e\n",
                m_add, m_mul, m_div, m_sqrt, m_cvt, m_cmp, m_norm, m_trig, m_trig_small, m_fma, m_dot, m_psum,
                m_paxpy, m_exp, m_log, m_pow, m_powi, m_fallback, m_trigpi);
    return 0;
}
