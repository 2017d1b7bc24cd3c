// Integer division by run-time constants without the integer divide.
#pragma once

#include <cuda_runtime.h>

namespace deft {

// Division by a run-time constant d without the integer divide (which the
// GPU emulates in ~20 instructions): with l = ceil(log2 d) and
// mul = floor(2^32 (2^l - d) / d) + 1, n / d = (umulhi(n, mul) + n) >> l for
// every 0 <= n < 2^31 (Granlund & Montgomery, "Division by invariant
// integers using multiplication", 1994).  d = 1 gives mul = 1, l = 0.
struct FastDiv {
  unsigned int d, mul, shift;
};

inline FastDiv make_fastdiv(unsigned int d) {
  FastDiv f;
  f.d = d;
  if (d <= 1) {
    f.mul = 1;
    f.shift = 0;
    f.d = 1;
    return f;
  }
  unsigned int l = 0;
  while ((1u << l) < d) l++;
  f.shift = l;
  f.mul = (unsigned int)(((unsigned long long)1 << 32) * ((1ull << l) - d) / d + 1);
  return f;
}

__device__ __forceinline__ int fdiv(int n, const FastDiv &f) {
  return (int)((__umulhi((unsigned)n, f.mul) + (unsigned)n) >> f.shift);
}
// q = n / d, r = n - q d
__device__ __forceinline__ void fdivmod(int n, const FastDiv &f, int &q, int &r) {
  q = fdiv(n, f);
  r = n - q * (int)f.d;
}

}  // namespace deft
