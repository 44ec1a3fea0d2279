// Force-included into reference translation units that call
// thrust::make_pair / make_tuple with explicit template arguments on lvalues
// (src/tools/progressionMatrices/multiBadMatrix.cpp:16,30,124).  The Thrust
// the reference was written against took these arguments by value; CCCL's
// versions forward, which rejects lvalues for explicit non-reference types.
// The by-value versions below restore the original semantics for that file.
#pragma once
// every library header the translation unit uses is included first, so the
// macros at the end only touch the reference file's own code
#include <omp.h>
#include <thrust/binary_search.h>
#include <thrust/count.h>
#include <thrust/device_vector.h>
#include <thrust/host_vector.h>
#include <thrust/iterator/constant_iterator.h>
#include <thrust/iterator/counting_iterator.h>
#include <thrust/pair.h>
#include <thrust/sequence.h>
#include <thrust/sort.h>
#include <thrust/tuple.h>

#include <cassert>
#include <chrono>
#include <iostream>
#include <limits>
#include <map>
#include <random>
#include <sstream>
#include <stdexcept>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

namespace thrust {
template <class T1, class T2>
pair<T1, T2> psim_compat_make_pair(T1 a, T2 b) {
    return pair<T1, T2>(a, b);
}
template <class... T>
tuple<T...> psim_compat_make_tuple(T... a) {
    return tuple<T...>(a...);
}
}  // namespace thrust
namespace std {
template <class T1, class T2>
pair<T1, T2> psim_compat_make_pair(T1 a, T2 b) {
    return pair<T1, T2>(a, b);
}
}  // namespace std
#define make_pair psim_compat_make_pair
#define make_tuple psim_compat_make_tuple
