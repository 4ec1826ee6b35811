// Hash primitives on the device (and host, for the transcript sponge): BLAKE3 compression
// (published BLAKE3 spec), Keccak-f[1600] (FIPS 202) and the SHA-256 compression (FIPS 180-4).
// These back the reference's hash engines (src/hash/mod.rs:28-36): Blake3 single-chunk hashing
// (blake3_engine.rs:83-160), SHA3-256 / Keccak-256 / SHA-256 (digest_engine.rs:122-141), Copy
// (copy_engine.rs:42-59).
#pragma once
#include <cstdint>

#include "field.cuh"

namespace whir {

enum HashKind : int { HASH_BLAKE3 = 0, HASH_SHA2 = 1, HASH_SHA3 = 2, HASH_KECCAK = 3, HASH_COPY = 4 };

#if defined(__CUDACC__)
#define WHIR_CONST __constant__
#else
#define WHIR_CONST
#endif

WHIR_HD uint32_t rotr32(uint32_t x, int n) {
#if defined(__CUDA_ARCH__)
  return __funnelshift_r(x, x, n);
#else
  return (x >> n) | (x << (32 - n));
#endif
}

static constexpr uint32_t B3_CHUNK_START = 1, B3_CHUNK_END = 2, B3_PARENT = 4, B3_ROOT = 8;

struct Blake3IV {
  static WHIR_HD uint32_t w(int i) {
    switch (i) {
      case 0: return 0x6A09E667u;
      case 1: return 0xBB67AE85u;
      case 2: return 0x3C6EF372u;
      case 3: return 0xA54FF53Au;
      case 4: return 0x510E527Fu;
      case 5: return 0x9B05688Cu;
      case 6: return 0x1F83D9ABu;
      default: return 0x5BE0CD19u;
    }
  }
};

#define WHIR_B3_G(a, b, c, d, x, y)      \
  do {                                   \
    a = a + b + (x);                     \
    d = rotr32(d ^ a, 16);               \
    c = c + d;                           \
    b = rotr32(b ^ c, 12);               \
    a = a + b + (y);                     \
    d = rotr32(d ^ a, 8);                \
    c = c + d;                           \
    b = rotr32(b ^ c, 7);                \
  } while (0)

// One BLAKE3 round over state s0..s15 with message words m[] given in the round's order.
#define WHIR_B3_ROUND(m0, m1, m2, m3, m4, m5, m6, m7, m8, m9, m10, m11, m12, m13, m14, m15) \
  do {                                                                                     \
    WHIR_B3_G(s0, s4, s8, s12, m0, m1);                                                    \
    WHIR_B3_G(s1, s5, s9, s13, m2, m3);                                                    \
    WHIR_B3_G(s2, s6, s10, s14, m4, m5);                                                   \
    WHIR_B3_G(s3, s7, s11, s15, m6, m7);                                                   \
    WHIR_B3_G(s0, s5, s10, s15, m8, m9);                                                   \
    WHIR_B3_G(s1, s6, s11, s12, m10, m11);                                                 \
    WHIR_B3_G(s2, s7, s8, s13, m12, m13);                                                  \
    WHIR_B3_G(s3, s4, s9, s14, m14, m15);                                                  \
  } while (0)

// BLAKE3 compression, chaining-value output only (first 8 words). The 7 rounds are unrolled with
// the message permutation folded into the word order of each round.
WHIR_HD void blake3_compress_cv(uint32_t cv[8], const uint32_t m[16], uint32_t counter_lo, uint32_t counter_hi,
                                uint32_t block_len, uint32_t flags) {
  uint32_t s0 = cv[0], s1 = cv[1], s2 = cv[2], s3 = cv[3], s4 = cv[4], s5 = cv[5], s6 = cv[6], s7 = cv[7];
  uint32_t s8 = Blake3IV::w(0), s9 = Blake3IV::w(1), s10 = Blake3IV::w(2), s11 = Blake3IV::w(3);
  uint32_t s12 = counter_lo, s13 = counter_hi, s14 = block_len, s15 = flags;
  // Message schedules: round r uses m[P^r(i)] with P = {2,6,3,10,7,0,4,13,1,11,12,5,9,14,15,8}.
  WHIR_B3_ROUND(m[0], m[1], m[2], m[3], m[4], m[5], m[6], m[7], m[8], m[9], m[10], m[11], m[12], m[13], m[14], m[15]);
  WHIR_B3_ROUND(m[2], m[6], m[3], m[10], m[7], m[0], m[4], m[13], m[1], m[11], m[12], m[5], m[9], m[14], m[15], m[8]);
  WHIR_B3_ROUND(m[3], m[4], m[10], m[12], m[13], m[2], m[7], m[14], m[6], m[5], m[9], m[0], m[11], m[15], m[8], m[1]);
  WHIR_B3_ROUND(m[10], m[7], m[12], m[9], m[14], m[3], m[13], m[15], m[4], m[0], m[11], m[2], m[5], m[8], m[1], m[6]);
  WHIR_B3_ROUND(m[12], m[13], m[9], m[11], m[15], m[10], m[14], m[8], m[7], m[2], m[5], m[3], m[0], m[1], m[6], m[4]);
  WHIR_B3_ROUND(m[9], m[14], m[11], m[5], m[8], m[12], m[15], m[1], m[13], m[3], m[0], m[10], m[2], m[6], m[4], m[7]);
  WHIR_B3_ROUND(m[11], m[15], m[5], m[0], m[1], m[9], m[8], m[6], m[14], m[10], m[2], m[12], m[3], m[4], m[7], m[13]);
  cv[0] = s0 ^ s8;
  cv[1] = s1 ^ s9;
  cv[2] = s2 ^ s10;
  cv[3] = s3 ^ s11;
  cv[4] = s4 ^ s12;
  cv[5] = s5 ^ s13;
  cv[6] = s6 ^ s14;
  cv[7] = s7 ^ s15;
}

WHIR_HD void blake3_iv(uint32_t cv[8]) {
  for (int i = 0; i < 8; ++i) cv[i] = Blake3IV::w(i);
}

// Hash of a 64-byte message (one block, CHUNK_START | CHUNK_END | ROOT): Merkle nodes and PoW.
WHIR_HD void blake3_64(const uint32_t m[16], uint32_t out[8]) {
  blake3_iv(out);
  blake3_compress_cv(out, m, 0, 0, 64, B3_CHUNK_START | B3_CHUNK_END | B3_ROOT);
}

// Proof-of-work blocks (proof_of_work.rs:81-104): m[0..8) = challenge, m[8..10) = nonce (LE),
// m[10..16) = 0, hashed as blake3_64. Round 1 reads the nonce only in its first diagonal G; the
// column step and the other three diagonal G's (disjoint state words, so their order is free) are
// the same for every nonce of a search and are computed once by blake3_pow_prefix. blake3_pow_tail
// finishes one nonce from that state and returns the first two output words.
WHIR_HD void blake3_pow_prefix(const uint32_t c[8], uint32_t pre[16]) {
  uint32_t s0 = Blake3IV::w(0), s1 = Blake3IV::w(1), s2 = Blake3IV::w(2), s3 = Blake3IV::w(3);
  uint32_t s4 = Blake3IV::w(4), s5 = Blake3IV::w(5), s6 = Blake3IV::w(6), s7 = Blake3IV::w(7);
  uint32_t s8 = Blake3IV::w(0), s9 = Blake3IV::w(1), s10 = Blake3IV::w(2), s11 = Blake3IV::w(3);
  uint32_t s12 = 0, s13 = 0, s14 = 64, s15 = B3_CHUNK_START | B3_CHUNK_END | B3_ROOT;
  WHIR_B3_G(s0, s4, s8, s12, c[0], c[1]);
  WHIR_B3_G(s1, s5, s9, s13, c[2], c[3]);
  WHIR_B3_G(s2, s6, s10, s14, c[4], c[5]);
  WHIR_B3_G(s3, s7, s11, s15, c[6], c[7]);
  WHIR_B3_G(s1, s6, s11, s12, 0u, 0u);
  WHIR_B3_G(s2, s7, s8, s13, 0u, 0u);
  WHIR_B3_G(s3, s4, s9, s14, 0u, 0u);
  const uint32_t v[16] = {s0, s1, s2, s3, s4, s5, s6, s7, s8, s9, s10, s11, s12, s13, s14, s15};
  for (int i = 0; i < 16; ++i) pre[i] = v[i];
}
WHIR_HD void blake3_pow_tail(const uint32_t pre[16], const uint32_t c[8], uint32_t n0, uint32_t n1, uint32_t& h0,
                             uint32_t& h1) {
  uint32_t s0 = pre[0], s1 = pre[1], s2 = pre[2], s3 = pre[3], s4 = pre[4], s5 = pre[5], s6 = pre[6], s7 = pre[7];
  uint32_t s8 = pre[8], s9 = pre[9], s10 = pre[10], s11 = pre[11], s12 = pre[12], s13 = pre[13], s14 = pre[14],
           s15 = pre[15];
  WHIR_B3_G(s0, s5, s10, s15, n0, n1);
  const uint32_t m[16] = {c[0], c[1], c[2], c[3], c[4], c[5], c[6], c[7], n0, n1, 0u, 0u, 0u, 0u, 0u, 0u};
  WHIR_B3_ROUND(m[2], m[6], m[3], m[10], m[7], m[0], m[4], m[13], m[1], m[11], m[12], m[5], m[9], m[14], m[15], m[8]);
  WHIR_B3_ROUND(m[3], m[4], m[10], m[12], m[13], m[2], m[7], m[14], m[6], m[5], m[9], m[0], m[11], m[15], m[8], m[1]);
  WHIR_B3_ROUND(m[10], m[7], m[12], m[9], m[14], m[3], m[13], m[15], m[4], m[0], m[11], m[2], m[5], m[8], m[1], m[6]);
  WHIR_B3_ROUND(m[12], m[13], m[9], m[11], m[15], m[10], m[14], m[8], m[7], m[2], m[5], m[3], m[0], m[1], m[6], m[4]);
  WHIR_B3_ROUND(m[9], m[14], m[11], m[5], m[8], m[12], m[15], m[1], m[13], m[3], m[0], m[10], m[2], m[6], m[4], m[7]);
  WHIR_B3_ROUND(m[11], m[15], m[5], m[0], m[1], m[9], m[8], m[6], m[14], m[10], m[2], m[12], m[3], m[4], m[7], m[13]);
  h0 = s0 ^ s8;
  h1 = s1 ^ s9;
}

// ------------------------------------------------------------------------------------------------
// Keccak-f[1600]
// ------------------------------------------------------------------------------------------------
WHIR_HD uint64_t rotl64(uint64_t x, int n) { return (x << n) | (x >> (64 - n)); }

WHIR_HD uint64_t keccak_rc(int r) {
  switch (r) {
    case 0: return 0x0000000000000001ULL;
    case 1: return 0x0000000000008082ULL;
    case 2: return 0x800000000000808AULL;
    case 3: return 0x8000000080008000ULL;
    case 4: return 0x000000000000808BULL;
    case 5: return 0x0000000080000001ULL;
    case 6: return 0x8000000080008081ULL;
    case 7: return 0x8000000000008009ULL;
    case 8: return 0x000000000000008AULL;
    case 9: return 0x0000000000000088ULL;
    case 10: return 0x0000000080008009ULL;
    case 11: return 0x000000008000000AULL;
    case 12: return 0x000000008000808BULL;
    case 13: return 0x800000000000008BULL;
    case 14: return 0x8000000000008089ULL;
    case 15: return 0x8000000000008003ULL;
    case 16: return 0x8000000000008002ULL;
    case 17: return 0x8000000000000080ULL;
    case 18: return 0x000000000000800AULL;
    case 19: return 0x800000008000000AULL;
    case 20: return 0x8000000080008081ULL;
    case 21: return 0x8000000000008080ULL;
    case 22: return 0x0000000080000001ULL;
    default: return 0x8000000080008008ULL;
  }
}

// In-place permutation of the 25-lane state (lane index x + 5y), fully unrolled theta/rho/pi/chi.
WHIR_HD void keccak_f1600(uint64_t a[25]) {
#if defined(__CUDA_ARCH__)
#pragma unroll 1
#endif
  for (int round = 0; round < 24; ++round) {
    uint64_t c0 = a[0] ^ a[5] ^ a[10] ^ a[15] ^ a[20];
    uint64_t c1 = a[1] ^ a[6] ^ a[11] ^ a[16] ^ a[21];
    uint64_t c2 = a[2] ^ a[7] ^ a[12] ^ a[17] ^ a[22];
    uint64_t c3 = a[3] ^ a[8] ^ a[13] ^ a[18] ^ a[23];
    uint64_t c4 = a[4] ^ a[9] ^ a[14] ^ a[19] ^ a[24];
    uint64_t d0 = c4 ^ rotl64(c1, 1), d1 = c0 ^ rotl64(c2, 1), d2 = c1 ^ rotl64(c3, 1);
    uint64_t d3 = c2 ^ rotl64(c4, 1), d4 = c3 ^ rotl64(c0, 1);
    // theta + rho + pi: b[y + 5*((2x+3y)%5)] = rot(a[x+5y] ^ d[x], r[x,y])
    uint64_t b0 = a[0] ^ d0;
    uint64_t b10 = rotl64(a[1] ^ d1, 1);
    uint64_t b20 = rotl64(a[2] ^ d2, 62);
    uint64_t b5 = rotl64(a[3] ^ d3, 28);
    uint64_t b15 = rotl64(a[4] ^ d4, 27);
    uint64_t b16 = rotl64(a[5] ^ d0, 36);
    uint64_t b1 = rotl64(a[6] ^ d1, 44);
    uint64_t b11 = rotl64(a[7] ^ d2, 6);
    uint64_t b21 = rotl64(a[8] ^ d3, 55);
    uint64_t b6 = rotl64(a[9] ^ d4, 20);
    uint64_t b7 = rotl64(a[10] ^ d0, 3);
    uint64_t b17 = rotl64(a[11] ^ d1, 10);
    uint64_t b2 = rotl64(a[12] ^ d2, 43);
    uint64_t b12 = rotl64(a[13] ^ d3, 25);
    uint64_t b22 = rotl64(a[14] ^ d4, 39);
    uint64_t b23 = rotl64(a[15] ^ d0, 41);
    uint64_t b8 = rotl64(a[16] ^ d1, 45);
    uint64_t b18 = rotl64(a[17] ^ d2, 15);
    uint64_t b3 = rotl64(a[18] ^ d3, 21);
    uint64_t b13 = rotl64(a[19] ^ d4, 8);
    uint64_t b14 = rotl64(a[20] ^ d0, 18);
    uint64_t b24 = rotl64(a[21] ^ d1, 2);
    uint64_t b9 = rotl64(a[22] ^ d2, 61);
    uint64_t b19 = rotl64(a[23] ^ d3, 56);
    uint64_t b4 = rotl64(a[24] ^ d4, 14);
    // chi
    a[0] = b0 ^ (~b1 & b2);
    a[1] = b1 ^ (~b2 & b3);
    a[2] = b2 ^ (~b3 & b4);
    a[3] = b3 ^ (~b4 & b0);
    a[4] = b4 ^ (~b0 & b1);
    a[5] = b5 ^ (~b6 & b7);
    a[6] = b6 ^ (~b7 & b8);
    a[7] = b7 ^ (~b8 & b9);
    a[8] = b8 ^ (~b9 & b5);
    a[9] = b9 ^ (~b5 & b6);
    a[10] = b10 ^ (~b11 & b12);
    a[11] = b11 ^ (~b12 & b13);
    a[12] = b12 ^ (~b13 & b14);
    a[13] = b13 ^ (~b14 & b10);
    a[14] = b14 ^ (~b10 & b11);
    a[15] = b15 ^ (~b16 & b17);
    a[16] = b16 ^ (~b17 & b18);
    a[17] = b17 ^ (~b18 & b19);
    a[18] = b18 ^ (~b19 & b15);
    a[19] = b19 ^ (~b15 & b16);
    a[20] = b20 ^ (~b21 & b22);
    a[21] = b21 ^ (~b22 & b23);
    a[22] = b22 ^ (~b23 & b24);
    a[23] = b23 ^ (~b24 & b20);
    a[24] = b24 ^ (~b20 & b21);
    a[0] ^= keccak_rc(round);
  }
}

// ------------------------------------------------------------------------------------------------
// SHA-256 compression
// ------------------------------------------------------------------------------------------------
WHIR_HD uint32_t sha256_k(int i) {
  switch (i) {
    case 0: return 0x428a2f98; case 1: return 0x71374491; case 2: return 0xb5c0fbcf; case 3: return 0xe9b5dba5;
    case 4: return 0x3956c25b; case 5: return 0x59f111f1; case 6: return 0x923f82a4; case 7: return 0xab1c5ed5;
    case 8: return 0xd807aa98; case 9: return 0x12835b01; case 10: return 0x243185be; case 11: return 0x550c7dc3;
    case 12: return 0x72be5d74; case 13: return 0x80deb1fe; case 14: return 0x9bdc06a7; case 15: return 0xc19bf174;
    case 16: return 0xe49b69c1; case 17: return 0xefbe4786; case 18: return 0x0fc19dc6; case 19: return 0x240ca1cc;
    case 20: return 0x2de92c6f; case 21: return 0x4a7484aa; case 22: return 0x5cb0a9dc; case 23: return 0x76f988da;
    case 24: return 0x983e5152; case 25: return 0xa831c66d; case 26: return 0xb00327c8; case 27: return 0xbf597fc7;
    case 28: return 0xc6e00bf3; case 29: return 0xd5a79147; case 30: return 0x06ca6351; case 31: return 0x14292967;
    case 32: return 0x27b70a85; case 33: return 0x2e1b2138; case 34: return 0x4d2c6dfc; case 35: return 0x53380d13;
    case 36: return 0x650a7354; case 37: return 0x766a0abb; case 38: return 0x81c2c92e; case 39: return 0x92722c85;
    case 40: return 0xa2bfe8a1; case 41: return 0xa81a664b; case 42: return 0xc24b8b70; case 43: return 0xc76c51a3;
    case 44: return 0xd192e819; case 45: return 0xd6990624; case 46: return 0xf40e3585; case 47: return 0x106aa070;
    case 48: return 0x19a4c116; case 49: return 0x1e376c08; case 50: return 0x2748774c; case 51: return 0x34b0bcb5;
    case 52: return 0x391c0cb3; case 53: return 0x4ed8aa4a; case 54: return 0x5b9cca4f; case 55: return 0x682e6ff3;
    case 56: return 0x748f82ee; case 57: return 0x78a5636f; case 58: return 0x84c87814; case 59: return 0x8cc70208;
    case 60: return 0x90befffa; case 61: return 0xa4506ceb; case 62: return 0xbef9a3f7; default: return 0xc67178f2;
  }
}

// w: 16 big-endian message words of one 64-byte block.
WHIR_HD void sha256_compress(uint32_t h[8], const uint32_t block_be[16]) {
  uint32_t w[16];
  for (int i = 0; i < 16; ++i) w[i] = block_be[i];
  uint32_t a = h[0], b = h[1], c = h[2], d = h[3], e = h[4], f = h[5], g = h[6], hh = h[7];
  for (int i = 0; i < 64; ++i) {
    uint32_t wi;
    if (i < 16) {
      wi = w[i];
    } else {
      uint32_t w15 = w[(i - 15) & 15], w2 = w[(i - 2) & 15];
      uint32_t s0 = rotr32(w15, 7) ^ rotr32(w15, 18) ^ (w15 >> 3);
      uint32_t s1 = rotr32(w2, 17) ^ rotr32(w2, 19) ^ (w2 >> 10);
      wi = w[i & 15] + s0 + w[(i - 7) & 15] + s1;
      w[i & 15] = wi;
    }
    uint32_t S1 = rotr32(e, 6) ^ rotr32(e, 11) ^ rotr32(e, 25);
    uint32_t ch = (e & f) ^ (~e & g);
    uint32_t t1 = hh + S1 + ch + sha256_k(i) + wi;
    uint32_t S0 = rotr32(a, 2) ^ rotr32(a, 13) ^ rotr32(a, 22);
    uint32_t mj = (a & b) ^ (a & c) ^ (b & c);
    uint32_t t2 = S0 + mj;
    hh = g; g = f; f = e; e = d + t1; d = c; c = b; b = a; a = t1 + t2;
  }
  h[0] += a; h[1] += b; h[2] += c; h[3] += d; h[4] += e; h[5] += f; h[6] += g; h[7] += hh;
}

WHIR_HD void sha256_init(uint32_t h[8]) {
  h[0] = 0x6a09e667; h[1] = 0xbb67ae85; h[2] = 0x3c6ef372; h[3] = 0xa54ff53a;
  h[4] = 0x510e527f; h[5] = 0x9b05688c; h[6] = 0x1f83d9ab; h[7] = 0x5be0cd19;
}

WHIR_HD uint32_t bswap32(uint32_t x) {
  return (x >> 24) | ((x >> 8) & 0xff00u) | ((x << 8) & 0xff0000u) | (x << 24);
}

// ------------------------------------------------------------------------------------------------
// Streaming message hasher: feed little-endian 32-bit words of a message whose total length is a
// multiple of 4 bytes and known in advance, get the 32-byte digest as 8 LE words. Used for leaf
// rows (message = concatenated canonical field-element bytes) for every engine.
// ------------------------------------------------------------------------------------------------
template <int KIND>
struct WordHasher;

template <>
struct WordHasher<HASH_BLAKE3> {
  // Single-chunk messages only (<= 1024 bytes); the caller checks the size.
  uint32_t cv[8];
  uint32_t blk[16];
  uint32_t total_words, fed, block_index;
  WHIR_HD void init(uint32_t msg_bytes) {
    blake3_iv(cv);
    total_words = msg_bytes / 4;
    fed = 0;
    block_index = 0;
  }
  WHIR_HD void push(uint32_t w) {
    blk[fed & 15] = w;
    ++fed;
    if ((fed & 15) == 0 && fed < total_words) {
      uint32_t flags = block_index == 0 ? B3_CHUNK_START : 0;
      blake3_compress_cv(cv, blk, 0, 0, 64, flags);
      ++block_index;
    }
  }
  WHIR_HD void finish(uint32_t out[8]) {
    uint32_t rem = fed - block_index * 16;  // words in the last block
    for (uint32_t i = rem; i < 16; ++i) blk[i] = 0;
    uint32_t flags = (block_index == 0 ? B3_CHUNK_START : 0) | B3_CHUNK_END | B3_ROOT;
    blake3_compress_cv(cv, blk, 0, 0, rem * 4, flags);
    for (int i = 0; i < 8; ++i) out[i] = cv[i];
  }
};

template <int PAD>
struct KeccakWordHasher {
  uint64_t st[25];
  uint32_t pos;  // words absorbed in the current rate block (rate 136 bytes = 34 words)
  bool hi;
  WHIR_HD void init(uint32_t) {
    for (int i = 0; i < 25; ++i) st[i] = 0;
    pos = 0;
  }
  WHIR_HD void push(uint32_t w) {
    st[pos >> 1] ^= (uint64_t)w << (32 * (pos & 1));
    if (++pos == 34) {
      keccak_f1600(st);
      pos = 0;
    }
  }
  WHIR_HD void finish(uint32_t out[8]) {
    // pad byte at byte offset 4*pos, 0x80 at byte 135
    uint32_t byte = pos * 4;
    st[byte >> 3] ^= (uint64_t)PAD << (8 * (byte & 7));
    st[135 >> 3] ^= (uint64_t)0x80 << (8 * (135 & 7));
    keccak_f1600(st);
    for (int i = 0; i < 4; ++i) {
      out[2 * i] = (uint32_t)st[i];
      out[2 * i + 1] = (uint32_t)(st[i] >> 32);
    }
  }
};
template <>
struct WordHasher<HASH_SHA3> : KeccakWordHasher<0x06> {};
template <>
struct WordHasher<HASH_KECCAK> : KeccakWordHasher<0x01> {};

template <>
struct WordHasher<HASH_SHA2> {
  uint32_t h[8];
  uint32_t blk[16];
  uint32_t fed;
  uint64_t total_bytes;
  WHIR_HD void init(uint32_t msg_bytes) {
    sha256_init(h);
    fed = 0;
    total_bytes = msg_bytes;
  }
  WHIR_HD void push(uint32_t w) {
    blk[fed & 15] = bswap32(w);
    ++fed;
    if ((fed & 15) == 0) sha256_compress(h, blk);
  }
  WHIR_HD void finish(uint32_t out[8]) {
    uint32_t rem = fed & 15;
    blk[rem] = 0x80000000u;
    for (uint32_t i = rem + 1; i < 16; ++i) blk[i] = 0;
    if (rem >= 14) {
      sha256_compress(h, blk);
      for (int i = 0; i < 16; ++i) blk[i] = 0;
    }
    uint64_t bits = total_bytes * 8;
    blk[14] = (uint32_t)(bits >> 32);
    blk[15] = (uint32_t)bits;
    sha256_compress(h, blk);
    for (int i = 0; i < 8; ++i) out[i] = bswap32(h[i]);
  }
};

template <>
struct WordHasher<HASH_COPY> {
  uint32_t buf[8];
  uint32_t fed;
  WHIR_HD void init(uint32_t) {
    fed = 0;
    for (int i = 0; i < 8; ++i) buf[i] = 0;
  }
  WHIR_HD void push(uint32_t w) {
    if (fed < 8) buf[fed] = w;
    ++fed;
  }
  WHIR_HD void finish(uint32_t out[8]) {
    for (int i = 0; i < 8; ++i) out[i] = buf[i];
  }
};

// Hash of one 64-byte message given as 16 LE words (Merkle nodes, PoW inputs) for every engine.
template <int KIND>
WHIR_HD void hash64(const uint32_t m[16], uint32_t out[8]) {
  if constexpr (KIND == HASH_BLAKE3) {
    blake3_64(m, out);
  } else {
    WordHasher<KIND> h;
    h.init(64);
    for (int i = 0; i < 16; ++i) h.push(m[i]);
    h.finish(out);
  }
}

}  // namespace whir
