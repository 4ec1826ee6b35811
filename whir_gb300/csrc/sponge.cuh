// Fiat–Shamir duplex sponge and the element codecs the transcript uses (host and device callable).
//
// Duplex sponge over Keccak-f[1600], rate 136 bytes:
//   absorb  — XOR bytes into the rate, permuting before a byte that would overflow it;
//   squeeze — on the first squeeze after absorbing, XOR 0x01 at the current position and 0x80 at
//             rate byte 135, permute, then read rate bytes (permuting when exhausted).
// Prover messages are the ArkFieldEncoder bytes of each element: the canonical little-endian bytes
// of each base coefficient (8 per Goldilocks coefficient, 24 for Field192, 32 for Field256 — the
// canonical u64 limbs in every supported field). A verifier challenge squeezes, per base
// coefficient, (base bytes + 16) bytes read as a little-endian integer and reduced mod p.
#pragma once
#include <cstddef>
#include <cstdint>

#include "field.cuh"
#include "hash.cuh"

namespace whir {

struct Sponge {
  uint64_t st[25];
  uint32_t pos;
  uint32_t squeezing;
  static constexpr uint32_t RATE = 136;

  WHIR_HD void reset() {
    for (int i = 0; i < 25; ++i) st[i] = 0;
    pos = 0;
    squeezing = 0;
  }
  WHIR_HD uint8_t* bytes() { return reinterpret_cast<uint8_t*>(st); }
  WHIR_HD void absorb(const uint8_t* in, size_t n) {
    if (squeezing) {
      squeezing = 0;
      pos = 0;
    }
    for (size_t i = 0; i < n; ++i) {
      if (pos == RATE) {
        keccak_f1600(st);
        pos = 0;
      }
      bytes()[pos++] ^= in[i];
    }
  }
  WHIR_HD void squeeze(uint8_t* out, size_t n) {
    if (!squeezing) {
      if (pos == RATE) {
        keccak_f1600(st);
        pos = 0;
      }
      bytes()[pos] ^= 0x01;
      bytes()[RATE - 1] ^= 0x80;
      keccak_f1600(st);
      pos = 0;
      squeezing = 1;
    }
    for (size_t i = 0; i < n; ++i) {
      if (pos == RATE) {
        keccak_f1600(st);
        pos = 0;
      }
      out[i] = bytes()[pos++];
    }
  }
};

// Canonical little-endian message bytes of an element (8 * LIMBS bytes).
template <class F>
WHIR_HD void elem_bytes(const F& x, uint8_t* out) {
  static_assert(F::LIMBS * 8 == F::DEG * Canon<F>::BASE_BYTES, "encoded size must equal the limb size");
  uint64_t c[F::LIMBS];
  Canon<F>::to(x, c);
  for (int d = 0; d < F::LIMBS; ++d)
    for (int i = 0; i < 8; ++i) out[8 * d + i] = (uint8_t)(c[d] >> (8 * i));
}

WHIR_HD Gl gl_from_bytes_mod(const uint8_t* b, size_t n) {
  uint64_t acc = 0;
  const uint64_t two64 = GL_EPS;
  size_t words = (n + 7) / 8;
  for (size_t w = words; w-- > 0;) {
    uint64_t x = 0;
    for (int i = 7; i >= 0; --i) {
      size_t k = w * 8 + i;
      x = (x << 8) | (k < n ? b[k] : 0);
    }
    if (x >= GL_P) x -= GL_P;
    acc = gl_add(gl_mul(acc, two64), x);
  }
  return Gl{acc};
}
template <class P>
WHIR_HD MontField<P> mont_from_bytes_mod(const uint8_t* b, size_t n) {
  typedef MontField<P> M;
  uint64_t l[M::N];
  for (int i = 0; i < M::N; ++i) l[i] = i == 1 ? 1 : 0;
  const M two64 = M::from_canonical(l);
  M acc = M::zero();
  size_t words = (n + 7) / 8;
  for (size_t w = words; w-- > 0;) {
    uint64_t x = 0;
    for (int i = 7; i >= 0; --i) {
      size_t k = w * 8 + i;
      x = (x << 8) | (k < n ? b[k] : 0);
    }
    uint64_t xl[M::N];
    for (int i = 0; i < M::N; ++i) xl[i] = i == 0 ? x : 0;
    acc = acc * two64 + M::from_canonical(xl);
  }
  return acc;
}

// verifier_message<F> squeezed from the sponge.
template <class F>
struct ChallengeCodec {
  // Goldilocks family: DEG coefficients of 8 + 16 squeezed bytes each.
  WHIR_HD static F squeeze(Sponge& s) {
    uint64_t c[F::LIMBS];
    uint8_t buf[24];
    for (int d = 0; d < F::DEG; ++d) {
      s.squeeze(buf, 24);
      c[d] = gl_from_bytes_mod(buf, 24).v;
    }
    return Canon<F>::from(c);
  }
};
template <class P>
struct ChallengeCodec<MontField<P>> {
  WHIR_HD static MontField<P> squeeze(Sponge& s) {
    uint8_t buf[P::BYTES + 16];
    s.squeeze(buf, sizeof(buf));
    return mont_from_bytes_mod<P>(buf, sizeof(buf));
  }
};

}  // namespace whir
