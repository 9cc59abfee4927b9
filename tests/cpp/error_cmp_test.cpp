// The squared-error comparisons of csrc/isti_error_cmp.cuh against comparisons of the
// correctly rounded square roots (the reference's length(), src/renderer.cu:204-215), with
// FLT_MAX for a direction that was not searched.
//  - every finite pattern a: RN(sqrt(a)) < RN(sqrt(a + 3 floats)) (the fast path of err_lt);
//  - err_lt on specials (+0, +inf, NaN, the unsearched marker, FLT_MAX), on random
//    neighbours 0..63 floats apart over the whole range and on squares of adjacent floats;
//  - both encodings through the selectors err_pack / ERR_UNSEARCHED_OF / err_less /
//    err_below / err_eps, on special and random neighbouring squared sums at EPS_1;
//  - err_store of +-0, +inf, NaN and random values;
//  - err_threshold for EPS_1 at full and low resolution and for random eps: the float
//    below T has a root below eps, T itself does not; err_lt_eps around T and at random.
// Prints "ok <cases>" or the first mismatch and exits 1.
#include "isti_error_cmp.cuh"

#include <cfloat>
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

namespace
{
using isti::err_bits;
using isti::err_float;

static_assert(isti::err_threshold(0.002f) == 0x368637bdu);
static_assert(isti::err_threshold(0.008f) == 0x388637bdu);

float value(uint32_t q)
{
    if (q == isti::ERR_UNSEARCHED)
        return FLT_MAX;
    if (q == isti::ERR_INF)
        return INFINITY;
    return std::sqrt(err_float(q)); // NaN patterns stay NaN
}

long cases = 0;

bool check_pair(uint32_t a, uint32_t b)
{
    cases++;
    const bool want = value(a) < value(b), got = isti::err_lt(a, b);
    if (want != got)
    {
        std::printf("err_lt mismatch: %08x %08x got %d want %d\n", a, b, int(got), int(want));
        return false;
    }
    return true;
}

bool check_eps(uint32_t q, float eps)
{
    cases++;
    const bool want = value(q) < eps, got = isti::err_lt_eps(q, isti::err_threshold(eps));
    if (want != got)
    {
        std::printf("err_lt_eps mismatch: %08x eps %a got %d want %d\n", q, double(eps), int(got), int(want));
        return false;
    }
    return true;
}

// the selectors: err_pack / ERR_UNSEARCHED_OF / err_less / err_below / err_eps of either
// encoding against the error they stand for
template <bool SQ>
float sel_value(uint32_t q)
{
    return SQ ? value(q) : err_float(q);
}

template <bool SQ>
bool check_selectors(uint32_t sa, uint32_t sb, float eps)
{
    cases += 4;
    const float a = err_float(sa), b = err_float(sb);
    const uint32_t pa = isti::err_pack<SQ>(a), pb = isti::err_pack<SQ>(b), un = isti::ERR_UNSEARCHED_OF<SQ>;
    const bool ok = sel_value<SQ>(un) == FLT_MAX && isti::err_less<SQ>(pa, pb) == (std::sqrt(a) < std::sqrt(b)) &&
                    isti::err_less<SQ>(pa, un) == (std::sqrt(a) < FLT_MAX) && isti::err_less<SQ>(un, pa) == (FLT_MAX < std::sqrt(a)) &&
                    isti::err_below<SQ>(pa, isti::err_eps<SQ>(eps)) == (std::sqrt(a) < eps) &&
                    isti::err_below<SQ>(un, isti::err_eps<SQ>(eps)) == false;
    if (!ok)
        std::printf("selectors (SQ=%d) disagree for squared sums %08x %08x, eps %a\n", int(SQ), sa, sb, double(eps));
    return ok;
}

bool check_store(float s)
{
    cases++;
    const float want = std::sqrt(s), got = value(isti::err_store(s));
    const bool same = (std::isnan(want) && std::isnan(got)) || want == got; // -0 compares as +0
    if (!same)
    {
        std::printf("err_store mismatch: %a -> %08x\n", double(s), isti::err_store(s));
        return false;
    }
    return true;
}
} // namespace

int main()
{
    // the fast path, every finite a
    for (uint32_t a = 0; a + 3u <= 0x7f7fffffu; a++)
        if (!(std::sqrt(err_float(a)) < std::sqrt(err_float(a + 3u))))
        {
            std::printf("roots of %08x and 3 floats above round alike\n", a);
            return 1;
        }
    cases += 0x7f7fffffL - 2;

    std::mt19937_64 rng(99);
    const std::vector<uint32_t> specials = {0u,         1u,         2u,         3u,         0x00800000u,          0x0b800000u,
                                            0x3f800000u, 0x7f7ffffdu, 0x7f7ffffeu, 0x7f7fffffu, isti::ERR_UNSEARCHED, isti::ERR_INF,
                                            0x7fffffffu, 0x7fc00000u, 0x3b800000u, 0x1a000000u};
    for (uint32_t a : specials)
        for (uint32_t b : specials)
            if (!check_pair(a, b))
                return 1;
    for (int it = 0; it < 4000000; it++)
    {
        const uint32_t a = uint32_t(rng() % 0x7f800000u);
        const uint32_t k = uint32_t(rng() % 64);
        const uint32_t b = a + k < 0x7f800000u ? a + k : a;
        if (!check_pair(a, b) || !check_pair(b, a))
            return 1;
    }
    // both encodings through the selectors: squared sums from specials (finite, +inf, NaN)
    // and random neighbours, at the EPS_1 values and around them
    const uint32_t sums[] = {0u, 1u, 0x00800000u, 0x3f800000u, 0x7f7fffffu, 0x7f800000u, 0x7fc00000u,
                             isti::err_threshold(0.002f) - 1u, isti::err_threshold(0.002f), isti::err_threshold(0.008f)};
    for (uint32_t a : sums)
        for (uint32_t b : sums)
            for (float eps : {0.002f, 0.008f})
                if (!check_selectors<true>(a, b, eps) || !check_selectors<false>(a, b, eps))
                    return 1;
    for (int it = 0; it < 1000000; it++)
    {
        const uint32_t a = uint32_t(rng() % 0x7f800000u), b = a + uint32_t(rng() % 8) < 0x7f800000u ? a + uint32_t(rng() % 8) : a;
        const float eps = it & 1 ? 0.002f : 0.008f;
        if (!check_selectors<true>(a, b, eps) || !check_selectors<false>(a, b, eps) || !check_selectors<true>(b, a, eps) ||
            !check_selectors<false>(b, a, eps))
            return 1;
    }
    for (int it = 0; it < 2000000; it++)
    {
        const float x = std::ldexp(float(rng() % 0x1000000) / float(0x1000000) + 0.5f, int(rng() % 120) - 70);
        const float y = std::nextafter(x, 2.0f * x + 1.0f);
        const uint32_t a = isti::err_store(x * x), b = isti::err_store(y * y);
        if (!check_pair(a, b) || !check_pair(b, a))
            return 1;
    }

    const float store_specials[] = {0.0f, -0.0f, INFINITY, NAN, -NAN, FLT_MAX, FLT_MIN, 1e-45f};
    for (float s : store_specials)
        if (!check_store(s))
            return 1;
    for (int it = 0; it < 1000000; it++)
        if (!check_store(err_float(uint32_t(rng() % 0x7f800000u))))
            return 1;

    std::vector<float> epss = {0.002f, 0.008f, 1.0f, 0.25f, FLT_MIN};
    for (int it = 0; it < 200; it++)
        epss.push_back(err_float(uint32_t(0x00800000u + rng() % (0x5f000000u - 0x00800000u))));
    for (float eps : epss)
    {
        const uint32_t t = isti::err_threshold(eps);
        cases++;
        if (!(std::sqrt(err_float(t - 1u)) < eps) || !(std::sqrt(err_float(t)) >= eps))
        {
            std::printf("err_threshold(%a) = %08x is not the first float whose root reaches eps\n", double(eps), t);
            return 1;
        }
        for (int64_t d = -2000; d <= 2000; d++)
            if (!check_eps(uint32_t(int64_t(t) + d), eps))
                return 1;
        for (uint32_t q : specials)
            if (!check_eps(q, eps))
                return 1;
        for (int it = 0; it < 5000; it++)
            if (!check_eps(uint32_t(rng() % 0x7f800000u), eps))
                return 1;
    }
    std::printf("ok %ld\n", cases);
    return 0;
}
