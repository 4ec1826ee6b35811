// ORACLE — test infrastructure only. CPU restatement of the WHIR reference's field arithmetic.
// Nothing in the product library links or calls this code; parity tests compare the library with
// it, and it is the timed CPU baseline.
//
// Fields follow src/algebra/fields.rs of the reference:
//   Field64   Goldilocks p = 2^64 - 2^32 + 1, generator 7                (fields.rs:85-91)
//   Field64_2 Fp2 = Fp[u]/(u^2 - 7)                                       (fields.rs:93-106)
//   Field64_3 Fp3 = Fp[u]/(u^3 - 2)                                       (fields.rs:108-143)
//   Field192  3-limb prime, generator 3                                   (fields.rs:73-77)
//   Field256  BN254 scalar field, generator 5                             (fields.rs:65-71)
// Elements cross the C ABI in canonical (non-Montgomery) little-endian u64 limbs, one limb vector
// per base coefficient, extension coefficients in increasing degree.
#pragma once
#include <cstdint>
#include <cstring>
#include <cmath>
#include <string>
#include <vector>

namespace oracle {

typedef unsigned __int128 u128;

// ---------------------------------------------------------------------------------------------
// Goldilocks
// ---------------------------------------------------------------------------------------------
static constexpr uint64_t GL_P = 0xFFFFFFFF00000001ULL;
static constexpr uint64_t GL_EPS = 0xFFFFFFFFULL;  // 2^64 mod p = 2^32 - 1

inline uint64_t gl_add(uint64_t a, uint64_t b) {
  uint64_t s = a + b;
  // a, b < p; a + b < 2p < 2^65. On wrap, add 2^64 mod p = eps.
  if (s < a) s += GL_EPS;
  if (s >= GL_P) s -= GL_P;
  return s;
}
inline uint64_t gl_sub(uint64_t a, uint64_t b) {
  uint64_t d = a - b;
  if (a < b) d -= GL_EPS;  // subtract 2^64 mod p, i.e. add p in two's complement arithmetic
  return d;
}
inline uint64_t gl_neg(uint64_t a) { return a == 0 ? 0 : GL_P - a; }
// 128-bit reduction using 2^64 = eps and 2^96 = -1 (mod p).
inline uint64_t gl_reduce128(u128 x) {
  uint64_t lo = (uint64_t)x, hi = (uint64_t)(x >> 64);
  uint64_t hh = hi >> 32, hl = hi & GL_EPS;
  uint64_t t0 = lo - hh;
  if (lo < hh) t0 -= GL_EPS;
  uint64_t t1 = hl * GL_EPS;  // < 2^64
  uint64_t r = t0 + t1;
  if (r < t0) r += GL_EPS;
  if (r >= GL_P) r -= GL_P;
  return r;
}
inline uint64_t gl_mul(uint64_t a, uint64_t b) { return gl_reduce128((u128)a * b); }
inline uint64_t gl_pow(uint64_t a, uint64_t e) {
  uint64_t r = 1;
  while (e) {
    if (e & 1) r = gl_mul(r, a);
    a = gl_mul(a, a);
    e >>= 1;
  }
  return r;
}
inline uint64_t gl_inv(uint64_t a) { return gl_pow(a, GL_P - 2); }
inline uint64_t gl_canon(uint64_t a) { return a >= GL_P ? a - GL_P : a; }

// ---------------------------------------------------------------------------------------------
// Generic little-endian multi-limb helpers (for the Montgomery fields and byte decoding)
// ---------------------------------------------------------------------------------------------
template <int N>
struct Limbs {
  uint64_t l[N];
};

template <int N>
inline bool limbs_geq(const uint64_t* a, const uint64_t* b) {
  for (int i = N - 1; i >= 0; --i) {
    if (a[i] != b[i]) return a[i] > b[i];
  }
  return true;
}
template <int N>
inline uint64_t limbs_sub(uint64_t* r, const uint64_t* a, const uint64_t* b) {
  uint64_t borrow = 0;
  for (int i = 0; i < N; ++i) {
    u128 d = (u128)a[i] - b[i] - borrow;
    r[i] = (uint64_t)d;
    borrow = (uint64_t)(d >> 64) & 1;
  }
  return borrow;
}
template <int N>
inline uint64_t limbs_add(uint64_t* r, const uint64_t* a, const uint64_t* b) {
  uint64_t carry = 0;
  for (int i = 0; i < N; ++i) {
    u128 s = (u128)a[i] + b[i] + carry;
    r[i] = (uint64_t)s;
    carry = (uint64_t)(s >> 64);
  }
  return carry;
}

// Montgomery arithmetic with R = 2^(64N), the representation ark-ff's MontBackend uses.
template <int N>
struct MontParams {
  uint64_t p[N];
  uint64_t r2[N];   // R^2 mod p
  uint64_t one[N];  // R mod p
  uint64_t pinv;    // -p^{-1} mod 2^64
  int bits;
  uint64_t generator;
  std::string name;
};

template <int N>
inline void mont_mul(uint64_t* out, const uint64_t* a, const uint64_t* b, const MontParams<N>& P) {
  // CIOS Montgomery multiplication.
  uint64_t t[N + 2];
  for (int i = 0; i < N + 2; ++i) t[i] = 0;
  for (int i = 0; i < N; ++i) {
    uint64_t carry = 0;
    for (int j = 0; j < N; ++j) {
      u128 s = (u128)a[j] * b[i] + t[j] + carry;
      t[j] = (uint64_t)s;
      carry = (uint64_t)(s >> 64);
    }
    u128 s = (u128)t[N] + carry;
    t[N] = (uint64_t)s;
    t[N + 1] = (uint64_t)(s >> 64);
    uint64_t m = t[0] * P.pinv;
    u128 s2 = (u128)m * P.p[0] + t[0];
    carry = (uint64_t)(s2 >> 64);
    for (int j = 1; j < N; ++j) {
      u128 s3 = (u128)m * P.p[j] + t[j] + carry;
      t[j - 1] = (uint64_t)s3;
      carry = (uint64_t)(s3 >> 64);
    }
    u128 s4 = (u128)t[N] + carry;
    t[N - 1] = (uint64_t)s4;
    t[N] = t[N + 1] + (uint64_t)(s4 >> 64);
  }
  uint64_t r[N];
  for (int i = 0; i < N; ++i) r[i] = t[i];
  if (t[N] || limbs_geq<N>(r, P.p)) limbs_sub<N>(r, r, P.p);
  for (int i = 0; i < N; ++i) out[i] = r[i];
}

template <int N>
MontParams<N> make_mont_params(const uint64_t* p, uint64_t generator, const char* name) {
  MontParams<N> P;
  for (int i = 0; i < N; ++i) P.p[i] = p[i];
  // -p^{-1} mod 2^64 by Newton iteration.
  uint64_t inv = 1;
  for (int i = 0; i < 7; ++i) inv *= 2 - p[0] * inv;
  P.pinv = (uint64_t)0 - inv;
  // R mod p: start from 1 and double 64N times.
  uint64_t x[N];
  for (int i = 0; i < N; ++i) x[i] = 0;
  x[0] = 1;
  for (int k = 0; k < 64 * N * 2; ++k) {
    uint64_t c = limbs_add<N>(x, x, x);
    if (c || limbs_geq<N>(x, P.p)) limbs_sub<N>(x, x, P.p);
    if (k == 64 * N - 1) {
      for (int i = 0; i < N; ++i) P.one[i] = x[i];
    }
  }
  for (int i = 0; i < N; ++i) P.r2[i] = x[i];
  int bits = 64 * N;
  while (bits > 0 && !((p[(bits - 1) / 64] >> ((bits - 1) % 64)) & 1)) --bits;
  P.bits = bits;
  P.generator = generator;
  P.name = name;
  return P;
}

const MontParams<3>& f192_params();
const MontParams<4>& f256_params();

// ---------------------------------------------------------------------------------------------
// Field element types. Every type exposes the same static interface used by the templated
// protocol code:  zero(), one(), from_u64(), add/sub/mul/neg, inv(), eq, pow,
// DEG (extension degree), BASE_BYTES (ceil(bits/8) of the base prime field),
// to_limbs/from_limbs (canonical ABI form), base_coeff_bytes (ArkFieldEncoder form),
// from_bytes_mod (reduce a little-endian byte string), mul_base (multiply by base element).
// ---------------------------------------------------------------------------------------------

struct Gl {
  uint64_t v;
  typedef Gl Base;
  static constexpr int DEG = 1;
  static constexpr int LIMBS = 1;       // limbs per base coefficient
  static constexpr int BASE_BYTES = 8;  // ceil(64/8)
  static const char* name() { return "Field64"; }
  static Gl zero() { return {0}; }
  static Gl one() { return {1}; }
  static Gl from_u64(uint64_t x) { return {gl_canon(x)}; }
  friend Gl operator+(Gl a, Gl b) { return {gl_add(a.v, b.v)}; }
  friend Gl operator-(Gl a, Gl b) { return {gl_sub(a.v, b.v)}; }
  friend Gl operator*(Gl a, Gl b) { return {gl_mul(a.v, b.v)}; }
  Gl operator-() const { return {gl_neg(v)}; }
  Gl& operator+=(Gl b) { v = gl_add(v, b.v); return *this; }
  Gl& operator-=(Gl b) { v = gl_sub(v, b.v); return *this; }
  Gl& operator*=(Gl b) { v = gl_mul(v, b.v); return *this; }
  bool operator==(Gl b) const { return v == b.v; }
  bool operator!=(Gl b) const { return v != b.v; }
  bool is_zero() const { return v == 0; }
  Gl inv() const { return {gl_inv(v)}; }
  Gl pow(uint64_t e) const { return {gl_pow(v, e)}; }
  Gl dbl() const { return *this + *this; }
  void to_limbs(uint64_t* out) const { out[0] = v; }
  static Gl from_limbs(const uint64_t* in) { return {in[0]}; }
  static bool limbs_valid(const uint64_t* in) { return in[0] < GL_P; }
  void base_coeff_bytes(uint8_t* out) const {
    for (int i = 0; i < 8; ++i) out[i] = (uint8_t)(v >> (8 * i));
  }
  // Reduce an arbitrary little-endian byte string mod p (Horner over 8-byte words, high first).
  static Gl from_bytes_mod(const uint8_t* b, size_t n) {
    Gl acc = zero();
    Gl two64 = {GL_EPS};
    size_t words = (n + 7) / 8;
    for (size_t w = words; w-- > 0;) {
      uint64_t x = 0;
      for (int i = 7; i >= 0; --i) {
        size_t k = w * 8 + i;
        x = (x << 8) | (k < n ? b[k] : 0);
      }
      acc = acc * two64 + from_u64(x);
    }
    return acc;
  }
  static double modulus_f64() { return (double)GL_P; }
  static int modulus_bits() { return 64; }
  static uint64_t generator() { return 7; }
  // p - 1 as little-endian limbs.
  static void p_minus_1(uint64_t* out) { out[0] = GL_P - 1; }
  Gl coeff(int) const { return *this; }
  static Gl from_coeffs(const Gl* c) { return c[0]; }
  static Gl from_base(Gl x) { return x; }
  Gl mul_base(Gl b) const { return *this * b; }
};

// Fp2 = Fp[u]/(u^2 - 7)
struct Gl2 {
  Gl c0, c1;
  typedef Gl Base;
  static constexpr int DEG = 2;
  static constexpr int LIMBS = 1;
  static constexpr int BASE_BYTES = 8;
  static const char* name() { return "Field64_2"; }
  static Gl2 zero() { return {{0}, {0}}; }
  static Gl2 one() { return {{1}, {0}}; }
  static Gl2 from_u64(uint64_t x) { return {Gl::from_u64(x), {0}}; }
  static Gl2 from_base(Gl x) { return {x, {0}}; }
  friend Gl2 operator+(Gl2 a, Gl2 b) { return {a.c0 + b.c0, a.c1 + b.c1}; }
  friend Gl2 operator-(Gl2 a, Gl2 b) { return {a.c0 - b.c0, a.c1 - b.c1}; }
  friend Gl2 operator*(Gl2 a, Gl2 b) {
    Gl v0 = a.c0 * b.c0, v1 = a.c1 * b.c1;
    Gl seven = {7};
    return {v0 + seven * v1, a.c0 * b.c1 + a.c1 * b.c0};
  }
  Gl2 mul_base(Gl b) const { return {c0 * b, c1 * b}; }
  Gl2 operator-() const { return {-c0, -c1}; }
  Gl2& operator+=(Gl2 b) { *this = *this + b; return *this; }
  Gl2& operator-=(Gl2 b) { *this = *this - b; return *this; }
  Gl2& operator*=(Gl2 b) { *this = *this * b; return *this; }
  bool operator==(Gl2 b) const { return c0 == b.c0 && c1 == b.c1; }
  bool operator!=(Gl2 b) const { return !(*this == b); }
  bool is_zero() const { return c0.is_zero() && c1.is_zero(); }
  Gl2 dbl() const { return *this + *this; }
  Gl2 inv() const {
    // (c0 + c1 u)^-1 = (c0 - c1 u) / (c0^2 - 7 c1^2)
    Gl norm = c0 * c0 - Gl{7} * c1 * c1;
    Gl ni = norm.inv();
    return {c0 * ni, -(c1 * ni)};
  }
  Gl2 pow(uint64_t e) const {
    Gl2 r = one(), a = *this;
    while (e) {
      if (e & 1) r = r * a;
      a = a * a;
      e >>= 1;
    }
    return r;
  }
  void to_limbs(uint64_t* out) const { out[0] = c0.v; out[1] = c1.v; }
  static Gl2 from_limbs(const uint64_t* in) { return {{in[0]}, {in[1]}}; }
  static bool limbs_valid(const uint64_t* in) { return in[0] < GL_P && in[1] < GL_P; }
  Gl coeff(int i) const { return i == 0 ? c0 : c1; }
  static Gl2 from_coeffs(const Gl* c) { return {c[0], c[1]}; }
};

// Fp3 = Fp[u]/(u^3 - 2)
struct Gl3 {
  Gl c0, c1, c2;
  typedef Gl Base;
  static constexpr int DEG = 3;
  static constexpr int LIMBS = 1;
  static constexpr int BASE_BYTES = 8;
  static const char* name() { return "Field64_3"; }
  static Gl3 zero() { return {{0}, {0}, {0}}; }
  static Gl3 one() { return {{1}, {0}, {0}}; }
  static Gl3 from_u64(uint64_t x) { return {Gl::from_u64(x), {0}, {0}}; }
  static Gl3 from_base(Gl x) { return {x, {0}, {0}}; }
  friend Gl3 operator+(Gl3 a, Gl3 b) { return {a.c0 + b.c0, a.c1 + b.c1, a.c2 + b.c2}; }
  friend Gl3 operator-(Gl3 a, Gl3 b) { return {a.c0 - b.c0, a.c1 - b.c1, a.c2 - b.c2}; }
  friend Gl3 operator*(Gl3 a, Gl3 b) {
    Gl two = {2};
    Gl d0 = a.c0 * b.c0, d1 = a.c0 * b.c1 + a.c1 * b.c0, d2 = a.c0 * b.c2 + a.c1 * b.c1 + a.c2 * b.c0;
    Gl d3 = a.c1 * b.c2 + a.c2 * b.c1, d4 = a.c2 * b.c2;
    return {d0 + two * d3, d1 + two * d4, d2};
  }
  Gl3 mul_base(Gl b) const { return {c0 * b, c1 * b, c2 * b}; }
  Gl3 operator-() const { return {-c0, -c1, -c2}; }
  Gl3& operator+=(Gl3 b) { *this = *this + b; return *this; }
  Gl3& operator-=(Gl3 b) { *this = *this - b; return *this; }
  Gl3& operator*=(Gl3 b) { *this = *this * b; return *this; }
  bool operator==(Gl3 b) const { return c0 == b.c0 && c1 == b.c1 && c2 == b.c2; }
  bool operator!=(Gl3 b) const { return !(*this == b); }
  bool is_zero() const { return c0.is_zero() && c1.is_zero() && c2.is_zero(); }
  Gl3 dbl() const { return *this + *this; }
  Gl3 pow(uint64_t e) const {
    Gl3 r = one(), a = *this;
    while (e) {
      if (e & 1) r = r * a;
      a = a * a;
      e >>= 1;
    }
    return r;
  }
  Gl3 inv() const {
    // a^{-1} = a^(p^3 - 2), computed as a^(p^3-2) via the norm: use Frobenius-free generic pow.
    // p^3 - 2 = (p-1)(p^2+p+1) + (p^2 + p - 1)... use the standard formula with the adjugate.
    // For u^3 = 2: inverse via solving the 3x3 linear system of multiplication by a.
    Gl a0 = c0, a1 = c1, a2 = c2, two = {2};
    // Multiplication matrix M (columns = a*1, a*u, a*u^2):
    // a*1   = (a0, a1, a2)
    // a*u   = (2 a2, a0, a1)
    // a*u^2 = (2 a1, 2 a2, a0)
    Gl m00 = a0, m01 = two * a2, m02 = two * a1;
    Gl m10 = a1, m11 = a0, m12 = two * a2;
    Gl m20 = a2, m21 = a1, m22 = a0;
    // Solve M x = e0 by Cramer's rule.
    Gl det = m00 * (m11 * m22 - m12 * m21) - m01 * (m10 * m22 - m12 * m20) + m02 * (m10 * m21 - m11 * m20);
    Gl di = det.inv();
    Gl x0 = (m11 * m22 - m12 * m21) * di;
    Gl x1 = (m12 * m20 - m10 * m22) * di;
    Gl x2 = (m10 * m21 - m11 * m20) * di;
    return {x0, x1, x2};
  }
  void to_limbs(uint64_t* out) const { out[0] = c0.v; out[1] = c1.v; out[2] = c2.v; }
  static Gl3 from_limbs(const uint64_t* in) { return {{in[0]}, {in[1]}, {in[2]}}; }
  static bool limbs_valid(const uint64_t* in) { return in[0] < GL_P && in[1] < GL_P && in[2] < GL_P; }
  Gl coeff(int i) const { return i == 0 ? c0 : (i == 1 ? c1 : c2); }
  static Gl3 from_coeffs(const Gl* c) { return {c[0], c[1], c[2]}; }
};

// Montgomery-form prime field with N limbs; `Tag` selects the parameter set.
template <int N, const MontParams<N>& (*PARAMS)()>
struct MontField {
  uint64_t m[N];  // Montgomery form
  typedef MontField Base;
  static constexpr int DEG = 1;
  static constexpr int LIMBS = N;
  static const MontParams<N>& P() { return PARAMS(); }
  static const char* name() { return P().name.c_str(); }
  static MontField zero() {
    MontField r;
    for (int i = 0; i < N; ++i) r.m[i] = 0;
    return r;
  }
  static MontField one() {
    MontField r;
    for (int i = 0; i < N; ++i) r.m[i] = P().one[i];
    return r;
  }
  static MontField from_canonical(const uint64_t* c) {
    MontField r;
    mont_mul<N>(r.m, c, P().r2, P());
    return r;
  }
  static MontField from_u64(uint64_t x) {
    uint64_t c[N] = {0};
    c[0] = x;
    return from_canonical(c);
  }
  void to_limbs(uint64_t* out) const {
    uint64_t one_c[N] = {0};
    one_c[0] = 1;
    mont_mul<N>(out, m, one_c, P());
  }
  static MontField from_limbs(const uint64_t* in) { return from_canonical(in); }
  static bool limbs_valid(const uint64_t* in) { return !limbs_geq<N>(in, P().p); }
  friend MontField operator+(MontField a, MontField b) {
    MontField r;
    uint64_t c = limbs_add<N>(r.m, a.m, b.m);
    if (c || limbs_geq<N>(r.m, P().p)) limbs_sub<N>(r.m, r.m, P().p);
    return r;
  }
  friend MontField operator-(MontField a, MontField b) {
    MontField r;
    uint64_t br = limbs_sub<N>(r.m, a.m, b.m);
    if (br) limbs_add<N>(r.m, r.m, P().p);
    return r;
  }
  friend MontField operator*(MontField a, MontField b) {
    MontField r;
    mont_mul<N>(r.m, a.m, b.m, P());
    return r;
  }
  MontField operator-() const { return zero() - *this; }
  MontField& operator+=(MontField b) { *this = *this + b; return *this; }
  MontField& operator-=(MontField b) { *this = *this - b; return *this; }
  MontField& operator*=(MontField b) { *this = *this * b; return *this; }
  bool operator==(const MontField& b) const { return std::memcmp(m, b.m, sizeof(m)) == 0; }
  bool operator!=(const MontField& b) const { return !(*this == b); }
  bool is_zero() const {
    for (int i = 0; i < N; ++i)
      if (m[i]) return false;
    return true;
  }
  MontField dbl() const { return *this + *this; }
  MontField pow_limbs(const uint64_t* e, int ne) const {
    MontField r = one(), a = *this;
    for (int i = 0; i < ne; ++i) {
      uint64_t w = e[i];
      for (int b = 0; b < 64; ++b) {
        if (w & 1) r = r * a;
        a = a * a;
        w >>= 1;
      }
    }
    return r;
  }
  MontField pow(uint64_t e) const { return pow_limbs(&e, 1); }
  MontField inv() const {
    uint64_t e[N];
    uint64_t two[N] = {0};
    two[0] = 2;
    limbs_sub<N>(e, P().p, two);
    return pow_limbs(e, N);
  }
  MontField coeff(int) const { return *this; }
  static MontField from_coeffs(const MontField* c) { return c[0]; }
  static MontField from_base(MontField x) { return x; }
  MontField mul_base(MontField b) const { return *this * b; }
};

typedef MontField<3, f192_params> F192;
typedef MontField<4, f256_params> F256;

// Traits bridging the uniform interface for prime fields (DEG == 1).
template <class F>
struct PrimeTraits;

template <>
struct PrimeTraits<Gl> {
  static constexpr int BYTES = 8;
  static int bits() { return 64; }
  static void p_limbs(uint64_t* out) { out[0] = GL_P; }
  static uint64_t generator() { return 7; }
  static double modulus_f64() { return (double)GL_P; }
};
template <int N, const MontParams<N>& (*PARAMS)()>
struct PrimeTraits<MontField<N, PARAMS>> {
  static constexpr int BYTES = 8 * N;  // upper bound; actual is ceil(bits/8)
  static int bits() { return PARAMS().bits; }
  static void p_limbs(uint64_t* out) {
    for (int i = 0; i < N; ++i) out[i] = PARAMS().p[i];
  }
  static uint64_t generator() { return PARAMS().generator; }
  static double modulus_f64() {
    // Same evaluation order as the reference: most significant limb first, value*2^64 + limb.
    double m = 0.0;
    for (int i = N - 1; i >= 0; --i) m = m * 18446744073709551616.0 + (double)PARAMS().p[i];
    return m;
  }
};

}  // namespace oracle
