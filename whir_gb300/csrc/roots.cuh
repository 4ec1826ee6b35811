// Device access to powers of a base field's roots of unity through two tables of powers of
// w = g^((p-1)/2^L) (L = RootTab::log_order): w_n^e = w^(e * 2^L/n) = lo[E mod 2^16] * hi[E >> 16]
// with E = e << (L - log2 n). root(n) = g^((p-1)/n) is the reference's NttEngine root
// (ntt/cooley_tukey.rs:53-79, 171-183): Goldilocks g = 7, L = 32; Field192 g = 3, L = 32 (of its
// 2-adicity 48); Field256 g = 5, L = 28.
#pragma once
#include "field.cuh"
#include "kernels.hpp"

namespace whir {

template <class B>
__device__ __forceinline__ B ldg_elem(const B* p) {
  B r;
  const unsigned long long* s = reinterpret_cast<const unsigned long long*>(p);
  unsigned long long* d = reinterpret_cast<unsigned long long*>(&r);
#pragma unroll
  for (int i = 0; i < (int)(sizeof(B) / 8); ++i) d[i] = __ldg(s + i);
  return r;
}

template <class B>
__device__ __forceinline__ B root_pow(const RootTab& rt, int logn, uint64_t e) {
  const uint64_t E = e << (rt.log_order - logn);
  const B* lo = reinterpret_cast<const B*>(rt.lo);
  const B* hi = reinterpret_cast<const B*>(rt.hi);
  return ldg_elem(lo + (E & 0xFFFF)) * ldg_elem(hi + (E >> 16));
}
template <>
__device__ __forceinline__ Gl root_pow<Gl>(const RootTab& rt, int logn, uint64_t e) {
  const uint64_t E = e << (rt.log_order - logn);
  return Gl{gl_mul(__ldg(rt.lo + (E & 0xFFFF)), __ldg(rt.hi + (E >> 16)))};
}

__device__ __forceinline__ uint32_t brev(uint32_t x, int bits) { return bits ? (__brev(x) >> (32 - bits)) : 0; }

}  // namespace whir
