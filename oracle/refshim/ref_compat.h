// Force-included when the VEDAS reference sources are compiled with g++ for
// the reference-as-oracle build (test infrastructure only).  It supplies what
// the reference got implicitly from nvcc's headers and an older Thrust:
//  - <numeric>, <thrust/execution_policy.h>, <thrust/extrema.h> includes;
//  - thrust::unary_function (removed from current CCCL Thrust);
//  - a namespace-scope declaration of libstdc++'s vector<bool> reference
//    swap so that the reference's qualified std::swap call finds it.
#ifndef VEDAS_ORACLE_REF_COMPAT_H
#define VEDAS_ORACLE_REF_COMPAT_H

#include <numeric>
#include <vector>
#include <cassert>
#include <climits>
#include <limits>
#include <thrust/execution_policy.h>
#include <thrust/extrema.h>
#include <thrust/functional.h>

namespace thrust {
template <typename A, typename R>
struct unary_function {
  typedef A argument_type;
  typedef R result_type;
};
}  // namespace thrust

namespace std {
void swap(_Bit_reference, _Bit_reference) noexcept;
}

#endif
