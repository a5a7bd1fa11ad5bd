// Stand-in for boost/numeric/conversion/cast.hpp so that the reference's
// include/redux/math/helpers.hpp compiles into oracle/_ref: its bound_cast template names
// numeric_cast and the two overflow exceptions, none of which the minimiser calls.  Like
// the Boost header it brings in the C math declarations that helpers.hpp relies on.
#ifndef RDXG_REF_BOOST_NUMERIC_CAST_HPP
#define RDXG_REF_BOOST_NUMERIC_CAST_HPP
#include <math.h>

#include <cmath>
#include <limits>
#include <stdexcept>

namespace boost {
namespace numeric {
struct negative_overflow : std::range_error {
    negative_overflow() : std::range_error("negative overflow") {}
};
struct positive_overflow : std::range_error {
    positive_overflow() : std::range_error("positive overflow") {}
};
}  // namespace numeric
template <typename Target, typename Source>
Target numeric_cast(Source s) {
    if (s < static_cast<Source>(std::numeric_limits<Target>::lowest())) throw numeric::negative_overflow();
    if (s > static_cast<Source>(std::numeric_limits<Target>::max())) throw numeric::positive_overflow();
    return static_cast<Target>(s);
}
}  // namespace boost
#endif
