// Directed arc cosine for intervals (declaration; the lemmas that use acos are built once the
// correctly rounded implementation is in place).
#pragma once

#include "interval.cuh"

namespace sid {
template<class T, bool CLAMP_LO, bool CLAMP_HI> __device__ Iv<T> iv_acos(Iv<T> x);
}
