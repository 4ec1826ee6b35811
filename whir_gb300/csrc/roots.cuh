// Device access to powers of Goldilocks roots of unity through two 2^16-entry tables of powers of
// w = 7^((p-1)/2^32): w_n^e = w^(e * 2^32/n) = lo[E mod 2^16] * hi[E >> 16] with E = e << (32 - log2 n).
// root(n) = 7^((p-1)/n) is the reference's NttEngine root (ntt/cooley_tukey.rs:53-79, 171-183).
#pragma once
#include "field.cuh"
#include "kernels.hpp"

namespace whir {

__device__ __forceinline__ Gl root_pow(const RootTab& rt, int logn, uint64_t e) {
  const uint64_t E = e << (32 - logn);
  return Gl{gl_mul(__ldg(rt.lo + (E & 0xFFFF)), __ldg(rt.hi + (E >> 16)))};
}

__device__ __forceinline__ uint32_t brev(uint32_t x, int bits) { return bits ? (__brev(x) >> (32 - bits)) : 0; }

}  // namespace whir
