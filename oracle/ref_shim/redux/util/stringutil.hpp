// Stand-in for the reference's redux/util/stringutil.hpp, which conjugate_gradient.cpp
// includes but (outside its DEBUG_ printouts) does not use; the original pulls in Boost
// date_time.  It shadows the reference header only in the oracle/_ref build.
#ifndef RDXG_REF_STRINGUTIL_HPP
#define RDXG_REF_STRINGUTIL_HPP
#include <string>
#endif
