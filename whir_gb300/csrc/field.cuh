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
  // s = a + b (carry c); t = s + eps (carry c2). The canonical sum is t when c | c2, else s. The
  // carry chains are written as multiply-adds by 1, which moves part of the work to the integer
  // multiply pipe: measured 6.0 ALU + 2.2 FMA-pipe instructions per add against 7.0 + 0.3 for
  // add.cc chains (the carry-outs themselves stay on the ALU pipe).
  asm("{\n\t"
      ".reg .u32 a0, a1, b0, b1, s0, s1, t0, t1, c, c2;\n\t"
      ".reg .pred p;\n\t"
      "mov.b64 {a0, a1}, %1;\n\t"
      "mov.b64 {b0, b1}, %2;\n\t"
      "mad.lo.cc.u32 s0, a0, 1, b0;\n\t"
      "madc.lo.cc.u32 s1, a1, 1, b1;\n\t"
      "addc.u32 c, 0, 0;\n\t"
      "mad.lo.cc.u32 t0, s0, 1, 0xffffffff;\n\t"
      "madc.lo.cc.u32 t1, s1, 1, 0;\n\t"
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
      // y = r2 * (2^32 - 1) as one 32x32 -> 64 multiply (integer multiply pipe)
      "mul.lo.u32 y0, r2, 0xffffffff;\n\t"
      "mul.hi.u32 y1, r2, 0xffffffff;\n\t"
      // w += y, plus eps on carry (carry chains as multiply-adds by 1: integer multiply pipe)
      "mad.lo.cc.u32 r0, r0, 1, y0;\n\t"
      "madc.lo.cc.u32 r1, r1, 1, y1;\n\t"
      "addc.u32 c, z, z;\n\t"
      "mul.lo.u32 c, c, 0xffffffff;\n\t"
      "mad.lo.cc.u32 r0, r0, 1, c;\n\t"
      "madc.lo.u32 r1, r1, 1, z;\n\t"
      // canonical: if w + eps carries, w >= p and the result is w + eps mod 2^64
      "mad.lo.cc.u32 t0, r0, 1, 0xffffffff;\n\t"
      "madc.lo.cc.u32 t1, r1, 1, z;\n\t"
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
// 7 * a (the non-residue of Fp2). On the device a multiply: its products run on the integer
// multiply pipe, which the add/select-heavy field code leaves mostly idle.
WHIR_HD uint64_t gl_mul7(uint64_t a) {
#if defined(__CUDA_ARCH__)
  return gl_mul_ptx(a, 7);
#else
  uint64_t a2 = gl_add(a, a), a4 = gl_add(a2, a2), a8 = gl_add(a4, a4);
  return gl_sub(a8, a);
#endif
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

// ---------------------------------------------------------------------------------------------
// Multi-limb prime fields in Montgomery form (R = 2^(64N)), as ark-ff's MontBackend stores them:
//   Field192  p = 3801539170989320091464968600173246866371124347557388484609, generator 3
//   Field256  BN254 scalar field, generator 5 (fields.rs:65-77)
// Elements live in Montgomery form in memory (host and device); the C ABI, the transcript and leaf
// hashing use canonical little-endian limbs (to_canonical / from_canonical).
// ---------------------------------------------------------------------------------------------
typedef unsigned __int128 u128_t;

struct F192Params {
  static constexpr int N = 3;
  static constexpr int BYTES = 24;  // ceil(192 / 8)
  WHIR_HD static uint64_t p(int i) {
    return i == 0 ? 0x5887000000000001ULL : (i == 1 ? 0x0ad0a439abc2c817ULL : 0x9b09ebbd813f1e17ULL);
  }
  WHIR_HD static uint64_t r2(int i) {
    return i == 0 ? 0xe7d9d9a32bc43105ULL : (i == 1 ? 0x9b5537d38879c40aULL : 0x6c2a69f7d53e03c3ULL);
  }
  WHIR_HD static uint64_t one(int i) {
    return i == 0 ? 0xa778ffffffffffffULL : (i == 1 ? 0xf52f5bc6543d37e8ULL : 0x64f614427ec0e1e8ULL);
  }
  static constexpr uint64_t PINV = 0x5886ffffffffffffULL;  // -p^{-1} mod 2^64
  static constexpr uint64_t GENERATOR = 3;
  static constexpr int TWO_ADICITY = 48;
  static constexpr uint64_t SMALL_ORDER = 1;  // no 3-power subgroup used by the NTT engine
};
struct F256Params {
  static constexpr int N = 4;
  static constexpr int BYTES = 32;  // ceil(254 / 8)
  WHIR_HD static uint64_t p(int i) {
    switch (i) {
      case 0: return 0x43e1f593f0000001ULL;
      case 1: return 0x2833e84879b97091ULL;
      case 2: return 0xb85045b68181585dULL;
      default: return 0x30644e72e131a029ULL;
    }
  }
  WHIR_HD static uint64_t r2(int i) {
    switch (i) {
      case 0: return 0x1bb8e645ae216da7ULL;
      case 1: return 0x53fe3ab1e35c59e3ULL;
      case 2: return 0x8c49833d53bb8085ULL;
      default: return 0x0216d0b17f4e44a5ULL;
    }
  }
  WHIR_HD static uint64_t one(int i) {
    switch (i) {
      case 0: return 0xac96341c4ffffffbULL;
      case 1: return 0x36fc76959f60cd29ULL;
      case 2: return 0x666ea36f7879462eULL;
      default: return 0x0e0a77c19a07df2fULL;
    }
  }
  static constexpr uint64_t PINV = 0xc2e1f593efffffffULL;
  static constexpr uint64_t GENERATOR = 5;
  static constexpr int TWO_ADICITY = 28;
  static constexpr uint64_t SMALL_ORDER = 9;  // 3^2 (small_subgroup_base 3, power 2)
};

template <class P>
struct MontField {
  static constexpr int N = P::N;
  uint64_t l[N];
  static constexpr int DEG = 1;
  static constexpr int LIMBS = N;  // u64 words per element (storage)
  typedef MontField Base;

  WHIR_HD static MontField zero() {
    MontField r;
    for (int i = 0; i < N; ++i) r.l[i] = 0;
    return r;
  }
  WHIR_HD static MontField one() {
    MontField r;
    for (int i = 0; i < N; ++i) r.l[i] = P::one(i);
    return r;
  }
  WHIR_HD static MontField from_base(const MontField& b) { return b; }
  WHIR_HD MontField coeff(int) const { return *this; }

  WHIR_HD static bool geq_p(const uint64_t* a) {
    for (int i = N - 1; i >= 0; --i) {
      const uint64_t pi = P::p(i);
      if (a[i] != pi) return a[i] > pi;
    }
    return true;
  }
  WHIR_HD static void sub_p(uint64_t* a) {
    uint64_t borrow = 0;
#pragma unroll
    for (int i = 0; i < N; ++i) {
      const u128_t d = (u128_t)a[i] - P::p(i) - borrow;
      a[i] = (uint64_t)d;
      borrow = (uint64_t)(d >> 64) & 1;
    }
  }
  // CIOS Montgomery multiplication: a * b * R^{-1} mod p.
  WHIR_HD static MontField mont_mul(const uint64_t* a, const uint64_t* b) {
    uint64_t t[N + 2];
    for (int i = 0; i < N + 2; ++i) t[i] = 0;
#pragma unroll
    for (int i = 0; i < N; ++i) {
      uint64_t carry = 0;
#pragma unroll
      for (int j = 0; j < N; ++j) {
        const u128_t s = (u128_t)a[j] * b[i] + t[j] + carry;
        t[j] = (uint64_t)s;
        carry = (uint64_t)(s >> 64);
      }
      u128_t s = (u128_t)t[N] + carry;
      t[N] = (uint64_t)s;
      t[N + 1] = (uint64_t)(s >> 64);
      const uint64_t m = t[0] * P::PINV;
      u128_t s2 = (u128_t)m * P::p(0) + t[0];
      carry = (uint64_t)(s2 >> 64);
#pragma unroll
      for (int j = 1; j < N; ++j) {
        const u128_t s3 = (u128_t)m * P::p(j) + t[j] + carry;
        t[j - 1] = (uint64_t)s3;
        carry = (uint64_t)(s3 >> 64);
      }
      const u128_t s4 = (u128_t)t[N] + carry;
      t[N - 1] = (uint64_t)s4;
      t[N] = t[N + 1] + (uint64_t)(s4 >> 64);
    }
    MontField r;
    for (int i = 0; i < N; ++i) r.l[i] = t[i];
    if (t[N] || geq_p(r.l)) sub_p(r.l);
    return r;
  }
  WHIR_HD friend MontField operator*(const MontField& a, const MontField& b) { return mont_mul(a.l, b.l); }
  WHIR_HD friend MontField operator+(const MontField& a, const MontField& b) {
    MontField r;
    uint64_t carry = 0;
#pragma unroll
    for (int i = 0; i < N; ++i) {
      const u128_t s = (u128_t)a.l[i] + b.l[i] + carry;
      r.l[i] = (uint64_t)s;
      carry = (uint64_t)(s >> 64);
    }
    if (carry || geq_p(r.l)) sub_p(r.l);
    return r;
  }
  WHIR_HD friend MontField operator-(const MontField& a, const MontField& b) {
    MontField r;
    uint64_t borrow = 0;
#pragma unroll
    for (int i = 0; i < N; ++i) {
      const u128_t d = (u128_t)a.l[i] - b.l[i] - borrow;
      r.l[i] = (uint64_t)d;
      borrow = (uint64_t)(d >> 64) & 1;
    }
    if (borrow) {
      uint64_t carry = 0;
#pragma unroll
      for (int i = 0; i < N; ++i) {
        const u128_t s = (u128_t)r.l[i] + P::p(i) + carry;
        r.l[i] = (uint64_t)s;
        carry = (uint64_t)(s >> 64);
      }
    }
    return r;
  }
  WHIR_HD MontField operator-() const { return zero() - *this; }
  WHIR_HD MontField& operator+=(const MontField& b) { *this = *this + b; return *this; }
  WHIR_HD MontField& operator-=(const MontField& b) { *this = *this - b; return *this; }
  WHIR_HD MontField& operator*=(const MontField& b) { *this = *this * b; return *this; }
  WHIR_HD bool operator==(const MontField& b) const {
    for (int i = 0; i < N; ++i)
      if (l[i] != b.l[i]) return false;
    return true;
  }
  WHIR_HD bool operator!=(const MontField& b) const { return !(*this == b); }
  WHIR_HD bool is_zero() const {
    uint64_t o = 0;
    for (int i = 0; i < N; ++i) o |= l[i];
    return o == 0;
  }
  WHIR_HD MontField mul_base(const MontField& b) const { return *this * b; }
  WHIR_HD MontField dbl() const { return *this + *this; }
  WHIR_HD MontField sqr() const { return *this * *this; }
  WHIR_HD MontField pow(uint64_t e) const {
    MontField r = one(), a = *this;
    while (e) {
      if (e & 1) r = r * a;
      a = a * a;
      e >>= 1;
    }
    return r;
  }
  // base^e for a little-endian multi-limb exponent
  WHIR_HD MontField pow_limbs(const uint64_t* e, int ne) const {
    MontField r = one();
    for (int i = ne - 1; i >= 0; --i)
      for (int b = 63; b >= 0; --b) {
        r = r * r;
        if ((e[i] >> b) & 1) r = r * *this;
      }
    return r;
  }
  WHIR_HD MontField inv() const {
    uint64_t e[N];
    uint64_t borrow = 2;
    for (int i = 0; i < N; ++i) {
      const uint64_t pi = P::p(i);
      e[i] = pi - borrow;
      borrow = pi < borrow ? 1 : 0;
    }
    return pow_limbs(e, N);
  }
  WHIR_HD static MontField from_canonical(const uint64_t* c) {
    uint64_t r2[N];
    for (int i = 0; i < N; ++i) r2[i] = P::r2(i);
    return mont_mul(c, r2);
  }
  WHIR_HD void to_canonical(uint64_t* out) const {
    uint64_t one_c[N];
    for (int i = 0; i < N; ++i) one_c[i] = i == 0 ? 1 : 0;
    MontField r = mont_mul(l, one_c);
    for (int i = 0; i < N; ++i) out[i] = r.l[i];
  }
  WHIR_HD static bool canonical_ok(const uint64_t* c) { return !geq_p(c); }
};

typedef MontField<F192Params> F192;
typedef MontField<F256Params> F256;

// Canonical conversion for every field type: element -> F::LIMBS canonical u64 limbs and back
// (identity for the Goldilocks family, whose elements are stored canonically).
template <class F>
struct Canon {
  WHIR_HD static void to(const F& x, uint64_t* out) {
    const uint64_t* w = reinterpret_cast<const uint64_t*>(&x);
    for (int i = 0; i < F::LIMBS; ++i) out[i] = w[i];
  }
  WHIR_HD static F from(const uint64_t* in) {
    F x;
    uint64_t* w = reinterpret_cast<uint64_t*>(&x);
    for (int i = 0; i < F::LIMBS; ++i) w[i] = in[i];
    return x;
  }
  WHIR_HD static bool ok(const uint64_t* in) {
    for (int i = 0; i < F::LIMBS; ++i)
      if (in[i] >= GL_P) return false;
    return true;
  }
  static constexpr int BASE_BYTES = 8;  // encoded bytes per base coefficient
  static constexpr bool IDENTITY = true;
};
template <class P>
struct Canon<MontField<P>> {
  WHIR_HD static void to(const MontField<P>& x, uint64_t* out) { x.to_canonical(out); }
  WHIR_HD static MontField<P> from(const uint64_t* in) { return MontField<P>::from_canonical(in); }
  WHIR_HD static bool ok(const uint64_t* in) { return MontField<P>::canonical_ok(in); }
  static constexpr int BASE_BYTES = P::BYTES;
  static constexpr bool IDENTITY = false;
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
