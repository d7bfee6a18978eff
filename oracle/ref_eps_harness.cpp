// ref_eps_harness.cpp -- test infrastructure: prints the reference's own
// neighbour threshold (epsilonOneFunctorClass, cuda/SpecialFunctors.hcu:245-274)
// and its two- and three-hop bounds (epsilonTwoFunctorClass /
// epsilonThreeFunctorClass, :276-344) for a grid of thresholds and length
// pairs, compiled on the host from the reference header where it lies
// (oracle/build_ref.py).  The output becomes the
// golden table tests/golden/eps_reference.json.
//
// The header derives two functors from thrust::unary_function, which the
// Thrust of this toolkit no longer has; the two empty bases below stand in for
// it (they carry only typedefs and play no part in the computation).
#include <cstdio>
#include <cmath>
#include <thrust/functional.h>
namespace thrust {
template <class A, class R> struct unary_function { typedef A argument_type; typedef R result_type; };
template <class A1, class A2, class R> struct binary_function {
    typedef A1 first_argument_type; typedef A2 second_argument_type; typedef R result_type;
};
}
#include "SpecialFunctors.hcu"

int main() {
    const float ts[] = {0.0f, 0.01f, 0.05f, 0.08f, 0.1f, 0.12f, 0.125f, 0.15f, 0.2f, 0.25f,
                        0.29f, 0.3f, 1.0f / 3.0f, 0.35f, 0.4f, 0.5f, 0.6f, 0.7f, 0.9f, 1.0f,
                        1.5f, -0.1f};
    std::printf("{\"thresholds\": [");
    for (size_t k = 0; k < sizeof ts / sizeof ts[0]; ++k) std::printf("%s%.9g", k ? ", " : "", ts[k]);
    // every length pair up to 64, then the diagonal up to 1024
    std::printf("],\n \"max_len\": 64,\n \"levenshtein\": [\n");
    for (size_t k = 0; k < sizeof ts / sizeof ts[0]; ++k) {
        epsilonOneFunctorClass<false> f(ts[k]);
        std::printf("  [");
        for (unsigned q = 0; q <= 64; ++q) {
            std::printf("%s[", q ? ",\n   " : "");
            for (unsigned s = 0; s <= 64; ++s) std::printf("%s%d", s ? "," : "", f(q, s));
            std::printf("]");
        }
        std::printf("]%s\n", k + 1 < sizeof ts / sizeof ts[0] ? "," : "");
    }
    std::printf(" ],\n \"diag_len\": 1024,\n \"hamming\": [\n");
    for (size_t k = 0; k < sizeof ts / sizeof ts[0]; ++k) {
        epsilonOneFunctorClass<true> h(ts[k]);
        std::printf("  [");
        for (unsigned q = 0; q <= 1024; ++q) std::printf("%s%d", q ? "," : "", h(q, q));
        std::printf("]%s\n", k + 1 < sizeof ts / sizeof ts[0] ? "," : "");
    }
    // multi-hop bounds (cuda/SpecialFunctors.hcu:276-344): every length pair up to 64
    std::printf(" ],\n \"two_hop\": [\n");
    for (size_t k = 0; k < sizeof ts / sizeof ts[0]; ++k) {
        epsilonTwoFunctorClass<false> f(ts[k]);
        std::printf("  [");
        for (unsigned q = 0; q <= 64; ++q) {
            std::printf("%s[", q ? ",\n   " : "");
            for (unsigned s = 0; s <= 64; ++s) std::printf("%s%d", s ? "," : "", f(q, s));
            std::printf("]");
        }
        std::printf("]%s\n", k + 1 < sizeof ts / sizeof ts[0] ? "," : "");
    }
    std::printf(" ],\n \"three_hop\": [\n");
    for (size_t k = 0; k < sizeof ts / sizeof ts[0]; ++k) {
        epsilonThreeFunctorClass<false> f(ts[k]);
        std::printf("  [");
        for (unsigned q = 0; q <= 64; ++q) {
            std::printf("%s[", q ? ",\n   " : "");
            for (unsigned s = 0; s <= 64; ++s) std::printf("%s%d", s ? "," : "", f(q, s));
            std::printf("]");
        }
        std::printf("]%s\n", k + 1 < sizeof ts / sizeof ts[0] ? "," : "");
    }
    std::printf(" ],\n \"hamming_two_three\": [\n");
    for (size_t k = 0; k < sizeof ts / sizeof ts[0]; ++k) {
        epsilonTwoFunctorClass<true> f2(ts[k]);
        epsilonThreeFunctorClass<true> f3(ts[k]);
        std::printf("  [[");
        for (unsigned q = 0; q <= 256; ++q) std::printf("%s%d", q ? "," : "", f2(q, q));
        std::printf("], [");
        for (unsigned q = 0; q <= 256; ++q) std::printf("%s%d", q ? "," : "", f3(q, q));
        std::printf("]]%s\n", k + 1 < sizeof ts / sizeof ts[0] ? "," : "");
    }
    std::printf(" ]}\n");
    return 0;
}
