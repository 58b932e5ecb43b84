// CPU ORACLE -- test infrastructure only.
// Correctly rounded arc cosine in a given direction, as the reference computes it with MPFR
// (ivarp/src/interval_acos.cpp:29-34,52-66): acos_rounded(x, up) is acos(x) rounded down (up=false)
// or up (up=true) to the type T.
#pragma once

#include <stdexcept>

namespace sido {
template<class T> T acos_rounded(T, bool) {
    throw std::runtime_error("oracle: acos not available yet");
}
}
