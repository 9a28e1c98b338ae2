// Minimal stand-in for boost::math::hypergeometric_pFq, used only so the
// oracle can compile the reference's CPU tensor-voting functions where Boost
// is not installed.  Evaluates the generalised hypergeometric series
//   pFq(a; b; z) = sum_k prod_i (a_i)_k / prod_j (b_j)_k * z^k / k!
// term by term.  The tensor-voting path only calls it with a non-positive
// integer numerator parameter (a terminating polynomial) and |z| <= 1; the
// loop stops when a term becomes exactly zero or negligibly small.
// Test infrastructure, not part of the product.
#pragma once
#include <cmath>
#include <vector>
namespace boost { namespace math {
inline double hypergeometric_pFq(const std::vector<double>& a, const std::vector<double>& b, double z) {
    double sum = 1.0, term = 1.0;
    for (int k = 0; k < 100000; ++k) {
        double ratio = z / double(k + 1);
        for (double ai : a) ratio *= (ai + k);
        for (double bj : b) ratio /= (bj + k);
        term *= ratio;
        sum += term;
        if (term == 0.0 || std::fabs(term) < 1e-17 * std::fabs(sum)) break;
    }
    return sum;
}
}}  // namespace boost::math
