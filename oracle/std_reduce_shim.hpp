// ORACLE TEST INFRASTRUCTURE — not part of the product.
//
// BowTieFilter::normalizeData (beamfilters.hpp:88-92) sums its (angle, weight)
// pairs with std::reduce and a lambda (double, pair) -> double.  GCC 13's
// std::reduce asserts that the operation also takes (pair, pair) and
// (pair, double), which that lambda does not, so the constructors fail to
// compile.  The overload below, declared before the reference's headers, is
// more specialised for that iterator type and is chosen instead: a left fold
// from the initial value, the sum the reference's normalisation means.
#pragma once
#include <numeric>
#include <utility>
#include <vector>

namespace std {
template <class T, class Op>
double reduce(__gnu_cxx::__normal_iterator<pair<T, T>*, vector<pair<T, T>>> first,
    __gnu_cxx::__normal_iterator<pair<T, T>*, vector<pair<T, T>>> last, double init, Op op)
{
    for (; first != last; ++first)
        init = op(init, *first);
    return init;
}
} // namespace std
