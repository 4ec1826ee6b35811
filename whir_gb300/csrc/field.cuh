// Finite-field arithmetic shared by the CUDA kernels and the host-side protocol code.
//
// Fields (reference src/algebra/fields.rs):
//   Gl   Goldilocks p = 2^64 - 2^32 + 1 (Field64, fields.rs:85-91), canonical u64 in [0, p)
//   Gl2  Fp2 = Fp[u]/(u^2 - 7) (Field64_2, fields.rs:93-106), coefficients c0 + c1 u
//   Gl3  Fp3 = Fp[u]/(u^3 - 2) (Field64_3, fields.rs:108-143)
// Values are stored canonically, so the in-memory little-endian bytes of a row are exactly the
// ArkFieldEncoder leaf bytes (matrix_commit.rs:130-156) and the C ABI layout.
//
// Goldilocks reduction uses 2^64 = 2^32 - 1 and 2^96 = -1 (mod p); on the device the 64x64->128
// product is lo = a*b, hi = __umul64hi(a, b) (both on the integer multiply pipe).
#pragma once
#include <cstdint>

#if defined(__CUDACC__)
#define WHIR_HD __host__ __device__ __forceinline__
#else
#define WHIR_HD inline
#endif

namespace whir {

static constexpr uint64_t GL_P = 0xFFFFFFFF00000001ULL;
static constexpr uint64_t GL_EPS = 0xFFFFFFFFULL;

#if defined(__CUDA_ARCH__)
// Device versions on 32-bit halves with PTX carry chains (fewer compare/select instructions on the
// ALU pipe than the 64-bit C expressions). Same canonical inputs and outputs as the host versions.
__device__ __forceinline__ uint64_t gl_add_ptx(uint64_t a, uint64_t b) {
  uint64_t r;
  // s = a + b (carry c); t = s + eps (carry c2). The canonical sum is t when c | c2, else s.
  asm("{\n\t"
      ".reg .u32 a0, a1, b0, b1, s0, s1, t0, t1, c, c2;\n\t"
      ".reg .pred p;\n\t"
      "mov.b64 {a0, a1}, %1;\n\t"
      "mov.b64 {b0, b1}, %2;\n\t"
      "add.cc.u32 s0, a0, b0;\n\t"
      "addc.cc.u32 s1, a1, b1;\n\t"
      "addc.u32 c, 0, 0;\n\t"
      "add.cc.u32 t0, s0, 0xffffffff;\n\t"
      "addc.cc.u32 t1, s1, 0;\n\t"
      "addc.u32 c2, 0, 0;\n\t"
      "or.b32 c, c, c2;\n\t"
      "setp.ne.u32 p, c, 0;\n\t"
      "selp.b32 s0, t0, s0, p;\n\t"
      "selp.b32 s1, t1, s1, p;\n\t"
      "mov.b64 %0, {s0, s1};\n\t"
      "}"
      : "=l"(r)
      : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ uint64_t gl_sub_ptx(uint64_t a, uint64_t b) {
  uint64_t r;
  // d = a - b; on borrow subtract eps as well (adding p modulo 2^64).
  asm("{\n\t"
      ".reg .u32 a0, a1, b0, b1, d0, d1, bw;\n\t"
      "mov.b64 {a0, a1}, %1;\n\t"
      "mov.b64 {b0, b1}, %2;\n\t"
      "sub.cc.u32 d0, a0, b0;\n\t"
      "subc.cc.u32 d1, a1, b1;\n\t"
      "subc.u32 bw, 0, 0;\n\t"
      "sub.cc.u32 d0, d0, bw;\n\t"
      "subc.u32 d1, d1, 0;\n\t"
      "mov.b64 %0, {d0, d1};\n\t"
      "}"
      : "=l"(r)
      : "l"(a), "l"(b));
  return r;
}
// 64x64 -> 128 product in four 32-bit limbs r3:r2:r1:r0, then
//   x = (r1:r0) + r2 * 2^64 + r3 * 2^96 = (r1:r0) - r3 + r2 * (2^32 - 1)   (mod p)
// with each borrow / carry folded back as -eps / +eps, and a final conditional subtraction of p.
__device__ __forceinline__ uint64_t gl_mul_ptx(uint64_t a, uint64_t b) {
  uint64_t r;
  asm("{\n\t"
      ".reg .u32 a0, a1, b0, b1, r0, r1, r2, r3, bw, y0, y1, c, t0, t1, z;\n\t"
      ".reg .pred p;\n\t"
      "mov.b64 {a0, a1}, %1;\n\t"
      "mov.b64 {b0, b1}, %2;\n\t"
      "mov.u32 z, 0;\n\t"
      "mul.lo.u32 r0, a0, b0;\n\t"
      "mul.hi.u32 r1, a0, b0;\n\t"
      "mad.lo.cc.u32 r1, a0, b1, r1;\n\t"
      "madc.hi.u32 r2, a0, b1, z;\n\t"
      "mad.lo.cc.u32 r1, a1, b0, r1;\n\t"
      "madc.hi.cc.u32 r2, a1, b0, r2;\n\t"
      "addc.u32 r3, z, z;\n\t"
      "mad.lo.cc.u32 r2, a1, b1, r2;\n\t"
      "madc.hi.u32 r3, a1, b1, r3;\n\t"
      // w = (r1:r0) - r3, minus eps on borrow
      "sub.cc.u32 r0, r0, r3;\n\t"
      "subc.cc.u32 r1, r1, z;\n\t"
      "subc.u32 bw, z, z;\n\t"
      "sub.cc.u32 r0, r0, bw;\n\t"
      "subc.u32 r1, r1, z;\n\t"
      // y = r2 * (2^32 - 1) = (r2 << 32) - r2
      "sub.cc.u32 y0, z, r2;\n\t"
      "subc.u32 y1, r2, z;\n\t"
      // w += y, plus eps on carry
      "add.cc.u32 r0, r0, y0;\n\t"
      "addc.cc.u32 r1, r1, y1;\n\t"
      "addc.u32 c, z, z;\n\t"
      "sub.u32 c, z, c;\n\t"
      "add.cc.u32 r0, r0, c;\n\t"
      "addc.u32 r1, r1, z;\n\t"
      // canonical: if w + eps carries, w >= p and the result is w + eps mod 2^64
      "add.cc.u32 t0, r0, 0xffffffff;\n\t"
      "addc.cc.u32 t1, r1, z;\n\t"
      "addc.u32 c, z, z;\n\t"
      "setp.ne.u32 p, c, 0;\n\t"
      "selp.b32 r0, t0, r0, p;\n\t"
      "selp.b32 r1, t1, r1, p;\n\t"
      "mov.b64 %0, {r0, r1};\n\t"
      "}"
      : "=l"(r)
      : "l"(a), "l"(b));
  return r;
}
#endif

WHIR_HD uint64_t gl_add(uint64_t a, uint64_t b) {
#if defined(__CUDA_ARCH__)
  return gl_add_ptx(a, b);
#else
  uint64_t s = a + b;
  uint64_t w = (s < a) ? GL_EPS : 0;  // wrapped past 2^64: add 2^64 mod p
  s += w;
  return (s >= GL_P) ? s - GL_P : s;
#endif
}
WHIR_HD uint64_t gl_sub(uint64_t a, uint64_t b) {
#if defined(__CUDA_ARCH__)
  return gl_sub_ptx(a, b);
#else
  uint64_t d = a - b;
  return (a < b) ? d - GL_EPS : d;
#endif
}
WHIR_HD uint64_t gl_neg(uint64_t a) { return a ? GL_P - a : 0; }

WHIR_HD uint64_t gl_reduce(uint64_t lo, uint64_t hi) {
  uint64_t hh = hi >> 32, hl = hi & GL_EPS;
  uint64_t t0 = lo - hh;
  if (lo < hh) t0 -= GL_EPS;
  uint64_t t1 = (hl << 32) - hl;  // hl * (2^32 - 1)
  uint64_t r = t0 + t1;
  if (r < t0) r += GL_EPS;
  return (r >= GL_P) ? r - GL_P : r;
}

WHIR_HD uint64_t gl_mul(uint64_t a, uint64_t b) {
#if defined(__CUDA_ARCH__)
  return gl_mul_ptx(a, b);
#else
  unsigned __int128 x = (unsigned __int128)a * b;
  return gl_reduce((uint64_t)x, (uint64_t)(x >> 64));
#endif
}
WHIR_HD uint64_t gl_sqr(uint64_t a) { return gl_mul(a, a); }
// 7 * a as 8a - a with modular additions (cheaper than a multiply).
WHIR_HD uint64_t gl_mul7(uint64_t a) {
  uint64_t a2 = gl_add(a, a), a4 = gl_add(a2, a2), a8 = gl_add(a4, a4);
  return gl_sub(a8, a);
}
WHIR_HD uint64_t gl_pow(uint64_t a, uint64_t e) {
  uint64_t r = 1;
  while (e) {
    if (e & 1) r = gl_mul(r, a);
    a = gl_mul(a, a);
    e >>= 1;
  }
  return r;
}
WHIR_HD uint64_t gl_inv(uint64_t a) { return gl_pow(a, GL_P - 2); }

// ---------------------------------------------------------------------------------------------
struct Gl {
  uint64_t v;
  static constexpr int DEG = 1;
  static constexpr int LIMBS = 1;  // u64 words per element (ABI and storage)
  typedef Gl Base;
  WHIR_HD static Gl zero() { return Gl{0}; }
  WHIR_HD static Gl one() { return Gl{1}; }
  WHIR_HD static Gl from_base(Gl b) { return b; }
  WHIR_HD Gl coeff(int) const { return *this; }
  WHIR_HD friend Gl operator+(Gl a, Gl b) { return Gl{gl_add(a.v, b.v)}; }
  WHIR_HD friend Gl operator-(Gl a, Gl b) { return Gl{gl_sub(a.v, b.v)}; }
  WHIR_HD friend Gl operator*(Gl a, Gl b) { return Gl{gl_mul(a.v, b.v)}; }
  WHIR_HD Gl operator-() const { return Gl{gl_neg(v)}; }
  WHIR_HD Gl& operator+=(Gl b) { v = gl_add(v, b.v); return *this; }
  WHIR_HD Gl& operator-=(Gl b) { v = gl_sub(v, b.v); return *this; }
  WHIR_HD Gl& operator*=(Gl b) { v = gl_mul(v, b.v); return *this; }
  WHIR_HD bool operator==(Gl b) const { return v == b.v; }
  WHIR_HD bool operator!=(Gl b) const { return v != b.v; }
  WHIR_HD bool is_zero() const { return v == 0; }
  WHIR_HD Gl mul_base(Gl b) const { return Gl{gl_mul(v, b.v)}; }
  WHIR_HD Gl dbl() const { return Gl{gl_add(v, v)}; }
  WHIR_HD Gl sqr() const { return Gl{gl_sqr(v)}; }
  WHIR_HD Gl inv() const { return Gl{gl_inv(v)}; }
  WHIR_HD Gl pow(uint64_t e) const { return Gl{gl_pow(v, e)}; }
};

struct Gl2 {
  uint64_t c0, c1;
  static constexpr int DEG = 2;
  static constexpr int LIMBS = 2;
  typedef Gl Base;
  WHIR_HD static Gl2 zero() { return Gl2{0, 0}; }
  WHIR_HD static Gl2 one() { return Gl2{1, 0}; }
  WHIR_HD static Gl2 from_base(Gl b) { return Gl2{b.v, 0}; }
  WHIR_HD Gl coeff(int i) const { return Gl{i == 0 ? c0 : c1}; }
  WHIR_HD friend Gl2 operator+(Gl2 a, Gl2 b) { return Gl2{gl_add(a.c0, b.c0), gl_add(a.c1, b.c1)}; }
  WHIR_HD friend Gl2 operator-(Gl2 a, Gl2 b) { return Gl2{gl_sub(a.c0, b.c0), gl_sub(a.c1, b.c1)}; }
  WHIR_HD friend Gl2 operator*(Gl2 a, Gl2 b) {
    // Karatsuba: (a0 + a1 u)(b0 + b1 u) = a0 b0 + 7 a1 b1 + ((a0+a1)(b0+b1) - a0 b0 - a1 b1) u
    uint64_t v0 = gl_mul(a.c0, b.c0), v1 = gl_mul(a.c1, b.c1);
    uint64_t s = gl_mul(gl_add(a.c0, a.c1), gl_add(b.c0, b.c1));
    return Gl2{gl_add(v0, gl_mul7(v1)), gl_sub(gl_sub(s, v0), v1)};
  }
  WHIR_HD Gl2 operator-() const { return Gl2{gl_neg(c0), gl_neg(c1)}; }
  WHIR_HD Gl2& operator+=(Gl2 b) { *this = *this + b; return *this; }
  WHIR_HD Gl2& operator-=(Gl2 b) { *this = *this - b; return *this; }
  WHIR_HD Gl2& operator*=(Gl2 b) { *this = *this * b; return *this; }
  WHIR_HD bool operator==(Gl2 b) const { return c0 == b.c0 && c1 == b.c1; }
  WHIR_HD bool operator!=(Gl2 b) const { return !(*this == b); }
  WHIR_HD bool is_zero() const { return (c0 | c1) == 0; }
  WHIR_HD Gl2 mul_base(Gl b) const { return Gl2{gl_mul(c0, b.v), gl_mul(c1, b.v)}; }
  WHIR_HD Gl2 dbl() const { return *this + *this; }
  WHIR_HD Gl2 sqr() const { return *this * *this; }
  WHIR_HD Gl2 inv() const {
    uint64_t norm = gl_sub(gl_sqr(c0), gl_mul7(gl_sqr(c1)));
    uint64_t ni = gl_inv(norm);
    return Gl2{gl_mul(c0, ni), gl_neg(gl_mul(c1, ni))};
  }
  WHIR_HD Gl2 pow(uint64_t e) const {
    Gl2 r = one(), a = *this;
    while (e) {
      if (e & 1) r = r * a;
      a = a * a;
      e >>= 1;
    }
    return r;
  }
};

struct Gl3 {
  uint64_t c0, c1, c2;
  static constexpr int DEG = 3;
  static constexpr int LIMBS = 3;
  typedef Gl Base;
  WHIR_HD static Gl3 zero() { return Gl3{0, 0, 0}; }
  WHIR_HD static Gl3 one() { return Gl3{1, 0, 0}; }
  WHIR_HD static Gl3 from_base(Gl b) { return Gl3{b.v, 0, 0}; }
  WHIR_HD Gl coeff(int i) const { return Gl{i == 0 ? c0 : (i == 1 ? c1 : c2)}; }
  WHIR_HD friend Gl3 operator+(Gl3 a, Gl3 b) {
    return Gl3{gl_add(a.c0, b.c0), gl_add(a.c1, b.c1), gl_add(a.c2, b.c2)};
  }
  WHIR_HD friend Gl3 operator-(Gl3 a, Gl3 b) {
    return Gl3{gl_sub(a.c0, b.c0), gl_sub(a.c1, b.c1), gl_sub(a.c2, b.c2)};
  }
  WHIR_HD friend Gl3 operator*(Gl3 a, Gl3 b) {
    // schoolbook with u^3 = 2
    uint64_t d0 = gl_mul(a.c0, b.c0);
    uint64_t d1 = gl_add(gl_mul(a.c0, b.c1), gl_mul(a.c1, b.c0));
    uint64_t d2 = gl_add(gl_add(gl_mul(a.c0, b.c2), gl_mul(a.c1, b.c1)), gl_mul(a.c2, b.c0));
    uint64_t d3 = gl_add(gl_mul(a.c1, b.c2), gl_mul(a.c2, b.c1));
    uint64_t d4 = gl_mul(a.c2, b.c2);
    return Gl3{gl_add(d0, gl_add(d3, d3)), gl_add(d1, gl_add(d4, d4)), d2};
  }
  WHIR_HD Gl3 operator-() const { return Gl3{gl_neg(c0), gl_neg(c1), gl_neg(c2)}; }
  WHIR_HD Gl3& operator+=(Gl3 b) { *this = *this + b; return *this; }
  WHIR_HD Gl3& operator-=(Gl3 b) { *this = *this - b; return *this; }
  WHIR_HD Gl3& operator*=(Gl3 b) { *this = *this * b; return *this; }
  WHIR_HD bool operator==(Gl3 b) const { return c0 == b.c0 && c1 == b.c1 && c2 == b.c2; }
  WHIR_HD bool operator!=(Gl3 b) const { return !(*this == b); }
  WHIR_HD bool is_zero() const { return (c0 | c1 | c2) == 0; }
  WHIR_HD Gl3 mul_base(Gl b) const { return Gl3{gl_mul(c0, b.v), gl_mul(c1, b.v), gl_mul(c2, b.v)}; }
  WHIR_HD Gl3 dbl() const { return *this + *this; }
  WHIR_HD Gl3 sqr() const { return *this * *this; }
  WHIR_HD Gl3 pow(uint64_t e) const {
    Gl3 r = one(), a = *this;
    while (e) {
      if (e & 1) r = r * a;
      a = a * a;
      e >>= 1;
    }
    return r;
  }
  WHIR_HD Gl3 inv() const {
    // Solve a * x = 1 with the multiplication matrix (columns a, a*u, a*u^2) by Cramer's rule.
    uint64_t m00 = c0, m01 = gl_add(c2, c2), m02 = gl_add(c1, c1);
    uint64_t m10 = c1, m11 = c0, m12 = gl_add(c2, c2);
    uint64_t m20 = c2, m21 = c1, m22 = c0;
    uint64_t a00 = gl_sub(gl_mul(m11, m22), gl_mul(m12, m21));
    uint64_t a10 = gl_sub(gl_mul(m12, m20), gl_mul(m10, m22));
    uint64_t a20 = gl_sub(gl_mul(m10, m21), gl_mul(m11, m20));
    uint64_t det = gl_add(gl_add(gl_mul(m00, a00), gl_mul(m01, a10)), gl_mul(m02, a20));
    uint64_t di = gl_inv(det);
    return Gl3{gl_mul(a00, di), gl_mul(a10, di), gl_mul(a20, di)};
  }
};

// Embedding helpers (reference src/algebra/embedding.rs:126-153).
template <class T, class S>
struct Embed {
  WHIR_HD static T map(const S& s) { return T::from_base(s); }
  WHIR_HD static T mul(const T& a, const S& s) { return a.mul_base(s); }
};
template <class T>
struct Embed<T, T> {
  WHIR_HD static T map(const T& s) { return s; }
  WHIR_HD static T mul(const T& a, const T& s) { return a * s; }
};

}  // namespace whir
