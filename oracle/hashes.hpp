// ORACLE — test infrastructure only. CPU restatement of the hash engines the WHIR reference
// registers in src/hash/mod.rs:28-36: Blake3 (blake3_engine.rs), SHA2-256 / SHA3-256 / Keccak-256
// (digest_engine.rs) and Copy (copy_engine.rs). The algorithms are the published BLAKE3 spec,
// FIPS 202 (Keccak-f[1600], SHA3) and FIPS 180-4 (SHA-256), written from those documents.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cstring>

namespace oracle {

// Engine identifiers: SHA3-256("whir::hash" || oid-or-name), see src/hash/mod.rs:88-103.
extern const uint8_t ENGINE_BLAKE3[32];
extern const uint8_t ENGINE_SHA2[32];
extern const uint8_t ENGINE_SHA3[32];
extern const uint8_t ENGINE_KECCAK[32];
extern const uint8_t ENGINE_COPY[32];

enum HashKind { HK_INVALID = -1, HK_BLAKE3 = 0, HK_SHA2 = 1, HK_SHA3 = 2, HK_KECCAK = 3, HK_COPY = 4 };
HashKind hash_kind(const uint8_t id[32]);

// BLAKE3 (unkeyed, 32-byte output) of an arbitrary-length message.
void blake3(const uint8_t* in, size_t len, uint8_t out[32]);
// BLAKE3 compression function; writes the 16-word output state.
void blake3_compress(const uint32_t cv[8], const uint8_t block[64], uint64_t counter, uint32_t block_len,
                     uint32_t flags, uint32_t out[16]);

void keccak_f1600(uint64_t st[25]);
void sha3_256(const uint8_t* in, size_t len, uint8_t out[32]);
void sha3_512(const uint8_t* in, size_t len, uint8_t out[64]);
void keccak_256(const uint8_t* in, size_t len, uint8_t out[32]);
void sha256(const uint8_t* in, size_t len, uint8_t out[32]);

// HashEngine::hash_many (src/hash/mod.rs:79-85): `count` messages of `size` bytes each.
// Returns 0, or -1 for an unknown engine / unsupported size (Copy only supports size <= 32).
int hash_many(HashKind kind, size_t size, const uint8_t* in, size_t count, uint8_t* out);

}  // namespace oracle
