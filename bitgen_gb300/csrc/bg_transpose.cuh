/* Byte -> basis-plane transpose of one 32-byte word, shared by the fused scan kernels and the
 * stand-alone transpose kernel.
 *
 * Layout produced (the reference's, bitgen/bitstream.py:228-258, kernel.cu:60-100): plane b
 * holds bit 7-b of every byte; character j of the word is bit 31-j of the plane word.
 *
 * Bytes 8r..8r+7 are read as an 8x8 bit matrix (row k = byte k, column c = bit c).  Flipping
 * it about the anti-diagonal moves bit c of byte k to bit 7-k of byte 7-c, so byte b of the
 * result is plane b of those 8 characters, first character in the high bit.  The flip is the
 * well-known three delta-swap anti-diagonal flip of a 64-bit bitboard (swap distances 36, 18,
 * 9).  Four byte permutes per half then gather byte b of the four pieces into plane word b.
 * Per 32 bytes this is about 100 integer instructions per thread, against 8 x 32 votes plus
 * bit extraction for a __ballot_sync transpose of the same bytes.
 */
#pragma once

namespace bg {
__device__ __forceinline__ unsigned long long flip_anti_diag(unsigned long long x) {
  const unsigned long long k1 = 0xaa00aa00aa00aa00ull, k2 = 0xcccc0000cccc0000ull,
                           k4 = 0xf0f0f0f00f0f0f0full;
  unsigned long long t = x ^ (x << 36);
  x ^= k4 & (t ^ (x >> 36));
  t = k2 & (x ^ (x << 18));
  x ^= t ^ (t >> 18);
  t = k1 & (x ^ (x << 9));
  x ^= t ^ (t >> 9);
  return x;
}

__device__ __forceinline__ void transpose32(const uint32_t u[8], uint32_t out[8]) {
  uint32_t L[4], H[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const unsigned long long y =
        flip_anti_diag((unsigned long long)u[2 * r] | ((unsigned long long)u[2 * r + 1] << 32));
    L[r] = (uint32_t)y;
    H[r] = (uint32_t)(y >> 32);
  }
  {
    const uint32_t A = __byte_perm(L[3], L[2], 0x5140), B = __byte_perm(L[3], L[2], 0x7362);
    const uint32_t C = __byte_perm(L[1], L[0], 0x5140), D = __byte_perm(L[1], L[0], 0x7362);
    out[0] = __byte_perm(A, C, 0x5410);
    out[1] = __byte_perm(A, C, 0x7632);
    out[2] = __byte_perm(B, D, 0x5410);
    out[3] = __byte_perm(B, D, 0x7632);
  }
  {
    const uint32_t A = __byte_perm(H[3], H[2], 0x5140), B = __byte_perm(H[3], H[2], 0x7362);
    const uint32_t C = __byte_perm(H[1], H[0], 0x5140), D = __byte_perm(H[1], H[0], 0x7362);
    out[4] = __byte_perm(A, C, 0x5410);
    out[5] = __byte_perm(A, C, 0x7632);
    out[6] = __byte_perm(B, D, 0x5410);
    out[7] = __byte_perm(B, D, 0x7632);
  }
}

/* The inverse: 8 plane words back to 32 bytes.  Byte m of plane word i (i < 4) is byte i of
 * the flipped piece L[3 - m] (of H[3 - m] for plane word 4 + i), a 4x4 byte transpose that the
 * same two byte-permute stages undo; the anti-diagonal flip is its own inverse. */
__device__ __forceinline__ void untranspose32(const uint32_t in[8], uint32_t u[8]) {
  uint32_t L[4], H[4];
  {
    const uint32_t P = __byte_perm(in[0], in[1], 0x5140), Q = __byte_perm(in[0], in[1], 0x7362);
    const uint32_t R = __byte_perm(in[2], in[3], 0x5140), T = __byte_perm(in[2], in[3], 0x7362);
    L[3] = __byte_perm(P, R, 0x5410);
    L[2] = __byte_perm(P, R, 0x7632);
    L[1] = __byte_perm(Q, T, 0x5410);
    L[0] = __byte_perm(Q, T, 0x7632);
  }
  {
    const uint32_t P = __byte_perm(in[4], in[5], 0x5140), Q = __byte_perm(in[4], in[5], 0x7362);
    const uint32_t R = __byte_perm(in[6], in[7], 0x5140), T = __byte_perm(in[6], in[7], 0x7362);
    H[3] = __byte_perm(P, R, 0x5410);
    H[2] = __byte_perm(P, R, 0x7632);
    H[1] = __byte_perm(Q, T, 0x5410);
    H[0] = __byte_perm(Q, T, 0x7632);
  }
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const unsigned long long x = flip_anti_diag((unsigned long long)L[r] | ((unsigned long long)H[r] << 32));
    u[2 * r] = (uint32_t)x;
    u[2 * r + 1] = (uint32_t)(x >> 32);
  }
}

}  // namespace bg
