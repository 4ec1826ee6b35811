// Unreduced (wide) accumulation of products for the sumcheck reductions.
//
// A sum of products a_k * b_k of Goldilocks-family elements is accumulated as exact 192-bit integers
// per product coefficient (three u64 words, 64x64 -> 128-bit multiply-adds with carry), and reduced
// mod p once at the end: x = w0 + w1 2^64 + w2 2^128 with 2^64 = 2^32 - 1 and 2^128 = -2^32 (mod p).
// Compared with reducing every product and adding canonically, this replaces two modular
// reductions and a modular add per coefficient product by three carry-chained multiply-adds. The
// result is the same field element (exact arithmetic). Fields without a specialisation (the
// Montgomery fields) accumulate reduced products.
#pragma once
#include <cstdint>

#include "field.cuh"

namespace whir {

struct Wide3 {
  uint64_t w0, w1, w2;
};
__device__ __forceinline__ void wide_zero(Wide3& a) { a.w0 = a.w1 = a.w2 = 0; }
// a += x * y (exact).
__device__ __forceinline__ void wide_madd(Wide3& a, uint64_t x, uint64_t y) {
  asm("mad.lo.cc.u64 %0, %3, %4, %0;\n\t"
      "madc.hi.cc.u64 %1, %3, %4, %1;\n\t"
      "addc.u64 %2, %2, 0;"
      : "+l"(a.w0), "+l"(a.w1), "+l"(a.w2)
      : "l"(x), "l"(y));
}
// Canonical value mod p; valid while w2 < 2^32 - 1 (fewer than 2^32 products accumulated).
__device__ __forceinline__ uint64_t wide_reduce(const Wide3& a) {
  return gl_sub(gl_reduce(a.w0, a.w1), a.w2 << 32);
}

template <class T>
struct WideAcc {
  T v;
  __device__ __forceinline__ void init() { v = T::zero(); }
  __device__ __forceinline__ void mac(const T& a, const T& b) { v += a * b; }
  template <class S>
  __device__ __forceinline__ void mac_mixed(const T& a, const S& s) {
    v += Embed<T, S>::mul(a, s);
  }
  __device__ __forceinline__ T get() const { return v; }
};

template <>
struct WideAcc<Gl> {
  Wide3 w;
  __device__ __forceinline__ void init() { wide_zero(w); }
  __device__ __forceinline__ void mac(const Gl& a, const Gl& b) { wide_madd(w, a.v, b.v); }
  template <class S>
  __device__ __forceinline__ void mac_mixed(const Gl& a, const S& s) {
    wide_madd(w, a.v, s.v);
  }
  __device__ __forceinline__ Gl get() const { return Gl{wide_reduce(w)}; }
};

// (a0 + a1 u)(b0 + b1 u) = a0 b0 + 7 a1 b1 + (a0 b1 + a1 b0) u
template <>
struct WideAcc<Gl2> {
  Wide3 w00, w11, w01;
  __device__ __forceinline__ void init() {
    wide_zero(w00);
    wide_zero(w11);
    wide_zero(w01);
  }
  __device__ __forceinline__ void mac(const Gl2& a, const Gl2& b) {
    wide_madd(w00, a.c0, b.c0);
    wide_madd(w11, a.c1, b.c1);
    wide_madd(w01, a.c0, b.c1);
    wide_madd(w01, a.c1, b.c0);
  }
  __device__ __forceinline__ void mac_mixed(const Gl2& a, const Gl2& b) { mac(a, b); }
  __device__ __forceinline__ void mac_mixed(const Gl2& a, const Gl& s) {
    wide_madd(w00, a.c0, s.v);
    wide_madd(w01, a.c1, s.v);
  }
  __device__ __forceinline__ Gl2 get() const {
    return Gl2{gl_add(wide_reduce(w00), gl_mul7(wide_reduce(w11))), wide_reduce(w01)};
  }
};

// (a0 + a1 u + a2 u^2)(b0 + b1 u + b2 u^2), u^3 = 2:
//   c0 = a0 b0 + 2 (a1 b2 + a2 b1), c1 = a0 b1 + a1 b0 + 2 a2 b2, c2 = a0 b2 + a1 b1 + a2 b0
template <>
struct WideAcc<Gl3> {
  Wide3 A, B, C, D, E;
  __device__ __forceinline__ void init() {
    wide_zero(A);
    wide_zero(B);
    wide_zero(C);
    wide_zero(D);
    wide_zero(E);
  }
  __device__ __forceinline__ void mac(const Gl3& a, const Gl3& b) {
    wide_madd(A, a.c0, b.c0);
    wide_madd(B, a.c1, b.c2);
    wide_madd(B, a.c2, b.c1);
    wide_madd(C, a.c0, b.c1);
    wide_madd(C, a.c1, b.c0);
    wide_madd(D, a.c2, b.c2);
    wide_madd(E, a.c0, b.c2);
    wide_madd(E, a.c1, b.c1);
    wide_madd(E, a.c2, b.c0);
  }
  __device__ __forceinline__ void mac_mixed(const Gl3& a, const Gl3& b) { mac(a, b); }
  __device__ __forceinline__ void mac_mixed(const Gl3& a, const Gl& s) {
    wide_madd(A, a.c0, s.v);
    wide_madd(C, a.c1, s.v);
    wide_madd(E, a.c2, s.v);
  }
  __device__ __forceinline__ Gl3 get() const {
    const uint64_t b = wide_reduce(B), d = wide_reduce(D);
    return Gl3{gl_add(wide_reduce(A), gl_add(b, b)), gl_add(wide_reduce(C), gl_add(d, d)), wide_reduce(E)};
  }
};

}  // namespace whir
