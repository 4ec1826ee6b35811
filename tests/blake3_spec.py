"""BLAKE3 in plain Python, restated from the published specification (J.-P. Aumasson, S. Neves,
Z. Wilcox-O'Hearn, J. O'Connor, "BLAKE3: one function, fast everywhere", 2020, section 2): the
compression function, chunk chaining (1024-byte chunks of 64-byte blocks, the last block zero-padded
with its true length) and the binary tree of parent nodes whose left subtree holds the largest power
of two of chunks that leaves at least one chunk on the right. Default hash mode, 32-byte output.

A test helper only: slow, written for clarity, and independent of the C++ oracle and the CUDA code
it is compared against."""

import struct

IV = (0x6A09E667, 0xBB67AE85, 0x3C6EF372, 0xA54FF53A, 0x510E527F, 0x9B05688C, 0x1F83D9AB, 0x5BE0CD19)
PERMUTATION = (2, 6, 3, 10, 7, 0, 4, 13, 1, 11, 12, 5, 9, 14, 15, 8)
CHUNK_START, CHUNK_END, PARENT, ROOT = 1, 2, 4, 8
BLOCK_LEN, CHUNK_LEN = 64, 1024
MASK = 0xFFFFFFFF


def _rotr(x, n):
    return ((x >> n) | (x << (32 - n))) & MASK


def _g(v, a, b, c, d, mx, my):
    v[a] = (v[a] + v[b] + mx) & MASK
    v[d] = _rotr(v[d] ^ v[a], 16)
    v[c] = (v[c] + v[d]) & MASK
    v[b] = _rotr(v[b] ^ v[c], 12)
    v[a] = (v[a] + v[b] + my) & MASK
    v[d] = _rotr(v[d] ^ v[a], 8)
    v[c] = (v[c] + v[d]) & MASK
    v[b] = _rotr(v[b] ^ v[c], 7)


def compress(cv, block, counter, block_len, flags):
    """The 16-word output of one compression (the first 8 words are the next chaining value)."""
    m = list(struct.unpack("<16I", block))
    v = list(cv) + list(IV[:4]) + [counter & MASK, (counter >> 32) & MASK, block_len, flags]
    for r in range(7):
        _g(v, 0, 4, 8, 12, m[0], m[1])
        _g(v, 1, 5, 9, 13, m[2], m[3])
        _g(v, 2, 6, 10, 14, m[4], m[5])
        _g(v, 3, 7, 11, 15, m[6], m[7])
        _g(v, 0, 5, 10, 15, m[8], m[9])
        _g(v, 1, 6, 11, 12, m[10], m[11])
        _g(v, 2, 7, 8, 13, m[12], m[13])
        _g(v, 3, 4, 9, 14, m[14], m[15])
        if r < 6:
            m = [m[PERMUTATION[i]] for i in range(16)]
    return [v[i] ^ v[i + 8] for i in range(8)] + [v[i + 8] ^ cv[i] for i in range(8)]


def _chunk_output(chunk, index):
    """(cv, last block, its length, flags) of a chunk: every block but the last is compressed here;
    the last one is left for the caller, which adds ROOT when the chunk is the whole input."""
    blocks = [chunk[i:i + BLOCK_LEN] for i in range(0, len(chunk), BLOCK_LEN)] or [b""]
    cv = list(IV)
    for k, blk in enumerate(blocks[:-1]):
        cv = compress(cv, blk, index, BLOCK_LEN, CHUNK_START if k == 0 else 0)[:8]
    last = blocks[-1]
    flags = CHUNK_END | (CHUNK_START if len(blocks) == 1 else 0)
    return cv, last.ljust(BLOCK_LEN, b"\0"), len(last), flags, index


def _node(data, first_chunk, root):
    """Chaining value (or, at the root, the root output words) of the subtree over `data`."""
    if len(data) <= CHUNK_LEN:
        cv, block, blen, flags, idx = _chunk_output(data, first_chunk)
        return compress(cv, block, idx, blen, flags | (ROOT if root else 0))[:8]
    chunks = (len(data) + CHUNK_LEN - 1) // CHUNK_LEN
    left_chunks = 1 << ((chunks - 1).bit_length() - 1)
    split = left_chunks * CHUNK_LEN
    left = _node(data[:split], first_chunk, False)
    right = _node(data[split:], first_chunk + left_chunks, False)
    block = struct.pack("<16I", *(left + right))
    return compress(list(IV), block, 0, BLOCK_LEN, PARENT | (ROOT if root else 0))[:8]


def blake3(data):
    """32-byte BLAKE3 hash of `data`."""
    return struct.pack("<8I", *_node(bytes(data), 0, True))
