// Minimal stand-in for boost::math::beta, used only so the oracle can compile
// the reference's CPU tensor-voting functions where Boost is not installed.
// B(a, b) = Gamma(a) Gamma(b) / Gamma(a + b), evaluated through log-gamma.
// Test infrastructure, not part of the product.
#pragma once
#include <cmath>
namespace boost { namespace math {
inline double beta(double a, double b) {
    return std::exp(std::lgamma(a) + std::lgamma(b) - std::lgamma(a + b));
}
}}  // namespace boost::math
