// ORACLE — test infrastructure only (see hashes.hpp).
#include "hashes.hpp"

#include <vector>

namespace oracle {

// Values verified against hashlib.sha3_256 in the test suite; identical to the reference's
// constants in blake3_engine.rs:19, digest_engine.rs:11-19 and copy_engine.rs:9.
const uint8_t ENGINE_BLAKE3[32] = {0x03, 0xe0, 0x17, 0x49, 0xeb, 0xcc, 0x04, 0x77, 0x92, 0x42, 0x54,
                                   0xeb, 0x48, 0x20, 0x66, 0xb8, 0x64, 0xa8, 0xdd, 0x4d, 0x77, 0x25,
                                   0x24, 0x64, 0xca, 0x6f, 0x5b, 0x6f, 0x5c, 0xc0, 0x5b, 0x4c};
const uint8_t ENGINE_SHA2[32] = {0x01, 0x8e, 0xaa, 0x24, 0x7c, 0xb8, 0x95, 0x7a, 0xb1, 0xe9, 0xfd,
                                 0xac, 0x88, 0x54, 0x50, 0x40, 0x3c, 0x5e, 0x7b, 0xda, 0x1a, 0xca,
                                 0xaa, 0x50, 0x4e, 0x4c, 0xc8, 0xf2, 0xf7, 0x6b, 0xb0, 0x76};
const uint8_t ENGINE_SHA3[32] = {0xaa, 0x80, 0x2d, 0xcd, 0xab, 0xad, 0x8e, 0xa8, 0xa1, 0x43, 0x09,
                                 0x19, 0x89, 0x3b, 0x96, 0xc3, 0x0e, 0x31, 0xff, 0x57, 0x34, 0xb3,
                                 0x85, 0x99, 0x91, 0x08, 0xaa, 0x20, 0x2d, 0x27, 0xdc, 0x12};
const uint8_t ENGINE_KECCAK[32] = {0xdd, 0xd2, 0x48, 0x96, 0x4e, 0x32, 0x03, 0x12, 0xa6, 0x67, 0x75,
                                   0xae, 0xe8, 0xe1, 0x6c, 0x88, 0xc9, 0x27, 0x73, 0x4b, 0xe5, 0x9a,
                                   0xca, 0x09, 0xb7, 0xaf, 0x6d, 0xeb, 0x0a, 0xd0, 0x0e, 0x8c};
const uint8_t ENGINE_COPY[32] = {0x09, 0x45, 0x90, 0x20, 0xf4, 0x51, 0x87, 0x4a, 0x1b, 0x39, 0x98,
                                 0x19, 0xd0, 0x79, 0x63, 0x2c, 0xc0, 0xf9, 0x26, 0x3b, 0x14, 0x86,
                                 0xc4, 0x23, 0x17, 0x3c, 0x6e, 0x15, 0xd8, 0xe2, 0xd6, 0x1d};

HashKind hash_kind(const uint8_t id[32]) {
  if (!memcmp(id, ENGINE_BLAKE3, 32)) return HK_BLAKE3;
  if (!memcmp(id, ENGINE_SHA2, 32)) return HK_SHA2;
  if (!memcmp(id, ENGINE_SHA3, 32)) return HK_SHA3;
  if (!memcmp(id, ENGINE_KECCAK, 32)) return HK_KECCAK;
  if (!memcmp(id, ENGINE_COPY, 32)) return HK_COPY;
  return HK_INVALID;
}

// ------------------------------------------------------------------------------------------
// BLAKE3 (spec: 7 rounds of the ChaCha-style G function over a 4x4 word state, message word
// permutation between rounds, chunk/parent tree with flags).
// ------------------------------------------------------------------------------------------
static const uint32_t B3_IV[8] = {0x6A09E667u, 0xBB67AE85u, 0x3C6EF372u, 0xA54FF53Au,
                                  0x510E527Fu, 0x9B05688Cu, 0x1F83D9ABu, 0x5BE0CD19u};
static const int B3_PERM[16] = {2, 6, 3, 10, 7, 0, 4, 13, 1, 11, 12, 5, 9, 14, 15, 8};
enum : uint32_t { CHUNK_START = 1, CHUNK_END = 2, PARENT = 4, ROOT = 8 };

static inline uint32_t rotr32(uint32_t x, int n) { return (x >> n) | (x << (32 - n)); }

static inline void b3_g(uint32_t* s, int a, int b, int c, int d, uint32_t mx, uint32_t my) {
  s[a] = s[a] + s[b] + mx;
  s[d] = rotr32(s[d] ^ s[a], 16);
  s[c] = s[c] + s[d];
  s[b] = rotr32(s[b] ^ s[c], 12);
  s[a] = s[a] + s[b] + my;
  s[d] = rotr32(s[d] ^ s[a], 8);
  s[c] = s[c] + s[d];
  s[b] = rotr32(s[b] ^ s[c], 7);
}

void blake3_compress(const uint32_t cv[8], const uint8_t block[64], uint64_t counter, uint32_t block_len,
                     uint32_t flags, uint32_t out[16]) {
  uint32_t m[16];
  for (int i = 0; i < 16; ++i)
    m[i] = (uint32_t)block[4 * i] | ((uint32_t)block[4 * i + 1] << 8) | ((uint32_t)block[4 * i + 2] << 16) |
           ((uint32_t)block[4 * i + 3] << 24);
  uint32_t s[16] = {cv[0],     cv[1],     cv[2],     cv[3],     cv[4],     cv[5],
                    cv[6],     cv[7],     B3_IV[0],  B3_IV[1],  B3_IV[2],  B3_IV[3],
                    (uint32_t)counter, (uint32_t)(counter >> 32), block_len, flags};
  for (int r = 0; r < 7; ++r) {
    b3_g(s, 0, 4, 8, 12, m[0], m[1]);
    b3_g(s, 1, 5, 9, 13, m[2], m[3]);
    b3_g(s, 2, 6, 10, 14, m[4], m[5]);
    b3_g(s, 3, 7, 11, 15, m[6], m[7]);
    b3_g(s, 0, 5, 10, 15, m[8], m[9]);
    b3_g(s, 1, 6, 11, 12, m[10], m[11]);
    b3_g(s, 2, 7, 8, 13, m[12], m[13]);
    b3_g(s, 3, 4, 9, 14, m[14], m[15]);
    if (r < 6) {
      uint32_t t[16];
      for (int i = 0; i < 16; ++i) t[i] = m[B3_PERM[i]];
      memcpy(m, t, sizeof(m));
    }
  }
  for (int i = 0; i < 8; ++i) {
    out[i] = s[i] ^ s[i + 8];
    out[i + 8] = s[i + 8] ^ cv[i];
  }
}

// Chaining value of one chunk (<= 1024 bytes); `root` marks a single-chunk message.
static void b3_chunk(const uint8_t* in, size_t len, uint64_t chunk_counter, bool root, uint32_t cv_out[8]) {
  uint32_t cv[8];
  memcpy(cv, B3_IV, sizeof(cv));
  size_t nblocks = len == 0 ? 1 : (len + 63) / 64;
  for (size_t b = 0; b < nblocks; ++b) {
    uint8_t block[64] = {0};
    size_t off = b * 64;
    size_t blen = len - off < 64 ? len - off : 64;
    if (len == 0) blen = 0;
    if (blen) memcpy(block, in + off, blen);
    uint32_t flags = 0;
    if (b == 0) flags |= CHUNK_START;
    if (b == nblocks - 1) flags |= CHUNK_END | (root ? ROOT : 0);
    uint32_t out[16];
    blake3_compress(cv, block, chunk_counter, (uint32_t)blen, flags, out);
    memcpy(cv, out, sizeof(cv));
  }
  memcpy(cv_out, cv, sizeof(cv));
}

static void b3_parent(const uint32_t l[8], const uint32_t r[8], bool root, uint32_t cv_out[8]) {
  uint8_t block[64];
  for (int i = 0; i < 8; ++i)
    for (int k = 0; k < 4; ++k) {
      block[4 * i + k] = (uint8_t)(l[i] >> (8 * k));
      block[32 + 4 * i + k] = (uint8_t)(r[i] >> (8 * k));
    }
  uint32_t out[16];
  blake3_compress(B3_IV, block, 0, 64, PARENT | (root ? ROOT : 0), out);
  memcpy(cv_out, out, 32);
}

// Chaining value of the subtree covering chunks [first, first + n) of the message.
static void b3_subtree(const uint8_t* in, size_t len, uint64_t first_chunk, bool root, uint32_t cv[8]) {
  size_t nchunks = len == 0 ? 1 : (len + 1023) / 1024;
  if (nchunks == 1) {
    b3_chunk(in, len, first_chunk, root, cv);
    return;
  }
  // Left subtree holds the largest power of two number of chunks strictly less than nchunks.
  size_t left = 1;
  while (left * 2 < nchunks) left *= 2;
  uint32_t lcv[8], rcv[8];
  b3_subtree(in, left * 1024, first_chunk, false, lcv);
  b3_subtree(in + left * 1024, len - left * 1024, first_chunk + left, false, rcv);
  b3_parent(lcv, rcv, root, cv);
}

void blake3(const uint8_t* in, size_t len, uint8_t out[32]) {
  uint32_t cv[8];
  b3_subtree(in, len, 0, true, cv);
  for (int i = 0; i < 8; ++i)
    for (int k = 0; k < 4; ++k) out[4 * i + k] = (uint8_t)(cv[i] >> (8 * k));
}

// ------------------------------------------------------------------------------------------
// Keccak-f[1600] and the FIPS 202 sponge (SHA3-256, SHA3-512) plus original Keccak-256 padding.
// ------------------------------------------------------------------------------------------
static const uint64_t KECCAK_RC[24] = {
    0x0000000000000001ULL, 0x0000000000008082ULL, 0x800000000000808AULL, 0x8000000080008000ULL,
    0x000000000000808BULL, 0x0000000080000001ULL, 0x8000000080008081ULL, 0x8000000000008009ULL,
    0x000000000000008AULL, 0x0000000000000088ULL, 0x0000000080008009ULL, 0x000000008000000AULL,
    0x000000008000808BULL, 0x800000000000008BULL, 0x8000000000008089ULL, 0x8000000000008003ULL,
    0x8000000000008002ULL, 0x8000000000000080ULL, 0x000000000000800AULL, 0x800000008000000AULL,
    0x8000000080008081ULL, 0x8000000000008080ULL, 0x0000000080000001ULL, 0x8000000080008008ULL};
// Rotation offsets r[x][y] indexed as lane x + 5y.
static const int KECCAK_ROT[25] = {0,  1,  62, 28, 27, 36, 44, 6,  55, 20, 3,  10, 43,
                                   25, 39, 41, 45, 15, 21, 8,  18, 2,  61, 56, 14};

static inline uint64_t rotl64(uint64_t x, int n) { return n == 0 ? x : (x << n) | (x >> (64 - n)); }

void keccak_f1600(uint64_t a[25]) {
  for (int round = 0; round < 24; ++round) {
    uint64_t c[5], d[5], b[25];
    for (int x = 0; x < 5; ++x) c[x] = a[x] ^ a[x + 5] ^ a[x + 10] ^ a[x + 15] ^ a[x + 20];
    for (int x = 0; x < 5; ++x) d[x] = c[(x + 4) % 5] ^ rotl64(c[(x + 1) % 5], 1);
    for (int i = 0; i < 25; ++i) a[i] ^= d[i % 5];
    // rho and pi: B[y, 2x+3y] = rot(A[x,y], r[x,y])
    for (int x = 0; x < 5; ++x)
      for (int y = 0; y < 5; ++y) b[y + 5 * ((2 * x + 3 * y) % 5)] = rotl64(a[x + 5 * y], KECCAK_ROT[x + 5 * y]);
    // chi
    for (int x = 0; x < 5; ++x)
      for (int y = 0; y < 5; ++y)
        a[x + 5 * y] = b[x + 5 * y] ^ ((~b[(x + 1) % 5 + 5 * y]) & b[(x + 2) % 5 + 5 * y]);
    // iota
    a[0] ^= KECCAK_RC[round];
  }
}

static void keccak_sponge(const uint8_t* in, size_t len, size_t rate, uint8_t pad, uint8_t* out, size_t outlen) {
  uint64_t st[25] = {0};
  uint8_t* sb = (uint8_t*)st;  // little-endian lane layout (both build targets are little-endian)
  size_t off = 0;
  while (len - off >= rate) {
    for (size_t i = 0; i < rate; ++i) sb[i] ^= in[off + i];
    keccak_f1600(st);
    off += rate;
  }
  size_t rem = len - off;
  for (size_t i = 0; i < rem; ++i) sb[i] ^= in[off + i];
  sb[rem] ^= pad;
  sb[rate - 1] ^= 0x80;
  keccak_f1600(st);
  size_t done = 0;
  while (done < outlen) {
    size_t n = outlen - done < rate ? outlen - done : rate;
    memcpy(out + done, sb, n);
    done += n;
    if (done < outlen) keccak_f1600(st);
  }
}

void sha3_256(const uint8_t* in, size_t len, uint8_t out[32]) { keccak_sponge(in, len, 136, 0x06, out, 32); }
void sha3_512(const uint8_t* in, size_t len, uint8_t out[64]) { keccak_sponge(in, len, 72, 0x06, out, 64); }
void keccak_256(const uint8_t* in, size_t len, uint8_t out[32]) { keccak_sponge(in, len, 136, 0x01, out, 32); }

// ------------------------------------------------------------------------------------------
// SHA-256 (FIPS 180-4)
// ------------------------------------------------------------------------------------------
static const uint32_t SHA256_K[64] = {
    0x428a2f98, 0x71374491, 0xb5c0fbcf, 0xe9b5dba5, 0x3956c25b, 0x59f111f1, 0x923f82a4, 0xab1c5ed5,
    0xd807aa98, 0x12835b01, 0x243185be, 0x550c7dc3, 0x72be5d74, 0x80deb1fe, 0x9bdc06a7, 0xc19bf174,
    0xe49b69c1, 0xefbe4786, 0x0fc19dc6, 0x240ca1cc, 0x2de92c6f, 0x4a7484aa, 0x5cb0a9dc, 0x76f988da,
    0x983e5152, 0xa831c66d, 0xb00327c8, 0xbf597fc7, 0xc6e00bf3, 0xd5a79147, 0x06ca6351, 0x14292967,
    0x27b70a85, 0x2e1b2138, 0x4d2c6dfc, 0x53380d13, 0x650a7354, 0x766a0abb, 0x81c2c92e, 0x92722c85,
    0xa2bfe8a1, 0xa81a664b, 0xc24b8b70, 0xc76c51a3, 0xd192e819, 0xd6990624, 0xf40e3585, 0x106aa070,
    0x19a4c116, 0x1e376c08, 0x2748774c, 0x34b0bcb5, 0x391c0cb3, 0x4ed8aa4a, 0x5b9cca4f, 0x682e6ff3,
    0x748f82ee, 0x78a5636f, 0x84c87814, 0x8cc70208, 0x90befffa, 0xa4506ceb, 0xbef9a3f7, 0xc67178f2};

static void sha256_block(uint32_t h[8], const uint8_t* p) {
  uint32_t w[64];
  for (int i = 0; i < 16; ++i)
    w[i] = ((uint32_t)p[4 * i] << 24) | ((uint32_t)p[4 * i + 1] << 16) | ((uint32_t)p[4 * i + 2] << 8) | p[4 * i + 3];
  for (int i = 16; i < 64; ++i) {
    uint32_t s0 = rotr32(w[i - 15], 7) ^ rotr32(w[i - 15], 18) ^ (w[i - 15] >> 3);
    uint32_t s1 = rotr32(w[i - 2], 17) ^ rotr32(w[i - 2], 19) ^ (w[i - 2] >> 10);
    w[i] = w[i - 16] + s0 + w[i - 7] + s1;
  }
  uint32_t a = h[0], b = h[1], c = h[2], d = h[3], e = h[4], f = h[5], g = h[6], hh = h[7];
  for (int i = 0; i < 64; ++i) {
    uint32_t S1 = rotr32(e, 6) ^ rotr32(e, 11) ^ rotr32(e, 25);
    uint32_t ch = (e & f) ^ (~e & g);
    uint32_t t1 = hh + S1 + ch + SHA256_K[i] + w[i];
    uint32_t S0 = rotr32(a, 2) ^ rotr32(a, 13) ^ rotr32(a, 22);
    uint32_t mj = (a & b) ^ (a & c) ^ (b & c);
    uint32_t t2 = S0 + mj;
    hh = g; g = f; f = e; e = d + t1; d = c; c = b; b = a; a = t1 + t2;
  }
  h[0] += a; h[1] += b; h[2] += c; h[3] += d; h[4] += e; h[5] += f; h[6] += g; h[7] += hh;
}

void sha256(const uint8_t* in, size_t len, uint8_t out[32]) {
  uint32_t h[8] = {0x6a09e667, 0xbb67ae85, 0x3c6ef372, 0xa54ff53a, 0x510e527f, 0x9b05688c, 0x1f83d9ab, 0x5be0cd19};
  size_t off = 0;
  while (len - off >= 64) {
    sha256_block(h, in + off);
    off += 64;
  }
  uint8_t tail[128] = {0};
  size_t rem = len - off;
  memcpy(tail, in + off, rem);
  tail[rem] = 0x80;
  size_t tl = rem + 9 <= 64 ? 64 : 128;
  uint64_t bits = (uint64_t)len * 8;
  for (int i = 0; i < 8; ++i) tail[tl - 1 - i] = (uint8_t)(bits >> (8 * i));
  sha256_block(h, tail);
  if (tl == 128) sha256_block(h, tail + 64);
  for (int i = 0; i < 8; ++i)
    for (int k = 0; k < 4; ++k) out[4 * i + k] = (uint8_t)(h[i] >> (24 - 8 * k));
}

int hash_many(HashKind kind, size_t size, const uint8_t* in, size_t count, uint8_t* out) {
  for (size_t i = 0; i < count; ++i) {
    const uint8_t* m = in + i * size;
    uint8_t* o = out + i * 32;
    switch (kind) {
      case HK_BLAKE3: blake3(m, size, o); break;
      case HK_SHA2: sha256(m, size, o); break;
      case HK_SHA3: sha3_256(m, size, o); break;
      case HK_KECCAK: keccak_256(m, size, o); break;
      case HK_COPY:
        if (size > 32) return -1;
        memset(o, 0, 32);
        memcpy(o, m, size);
        break;
      default: return -1;
    }
  }
  if (count == 0 && kind == HK_COPY && size > 32) return -1;
  if (kind == HK_INVALID) return -1;
  return 0;
}

}  // namespace oracle
