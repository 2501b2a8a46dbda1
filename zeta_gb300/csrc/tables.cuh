/*
 * tables.cuh -- Zobrist keys and evaluation tables.
 *
 * These are the reference's constants (zeta.cl:258-359); bit-exact hashes
 * and scores need the same numbers.  Device code reads them from constant
 * memory, host code from a plain copy.
 */
#pragma once

#include "chess.cuh"

namespace zeta {

#define ZETA_ZOBRIST_INIT                                                                        \
  {0x9D39247E33776D41ULL, 0x2AF7398005AAA5C7ULL, 0x44DB015024623547ULL, 0x9C15F73E62A76AE2ULL, \
   0x75834465489C0C89ULL, 0x3290AC3A203001BFULL, 0x0FBBAD1F61042279ULL, 0xE83A908FF2FB60CAULL, \
   0x0D7E765D58755C10ULL, 0x1A083822CEAFE02DULL, 0x9605D5F0E25EC3B0ULL, 0xD021FF5CD13A2ED5ULL, \
   0x40BDF15D4A672E32ULL, 0x011355146FD56395ULL, 0x5DB4832046F3D9E5ULL, 0x239F8B2D7FF719CCULL, \
   0x05D1A1AE85B49AA1ULL, 0x679F848F6E8FC971ULL}

#if defined(__CUDACC__)
static __constant__ u64 kZobristDev[18] = ZETA_ZOBRIST_INIT;
#endif
static const u64 kZobristHost[18] = ZETA_ZOBRIST_INIT;

ZHD u64 zobrist(int i) {
#if defined(__CUDA_ARCH__)
  return kZobristDev[i];
#else
  return kZobristHost[i];
#endif
}

ZHD u64 rotl64(u64 z, int s) {
  s &= 63;
  return s ? (z << s) | (z >> (64 - s)) : z;
}

/* Full Zobrist hash of a position: computehash, src/bitboard.c:461-510. */
ZHD u64 compute_hash(const Pos &p, int stm) {
  u64 h = 0;
  u64 occ = p.p1 | p.p2 | p.p3;
  u64 w = occ;
  while (w) {
    int sq = ctz(w);
    w &= w - 1;
    int pc = piece_at(p, sq);
    h ^= rotl64(zobrist((pc & 1) * 6 + (pc >> 1) - 1), sq);
  }
  u64 cr = p.cr;
  if (~cr & ZETA_CR_WQ) h ^= zobrist(12);
  if (~cr & ZETA_CR_WK) h ^= zobrist(13);
  if (~cr & ZETA_CR_BQ) h ^= zobrist(14);
  if (~cr & ZETA_CR_BK) h ^= zobrist(15);
  u64 ep = ~cr & ZETA_EPMASK;
  if (ep) h ^= rotl64(zobrist(16), ctz(ep) & 7);
  if (stm) h ^= 1ULL;
  return h;
}

/* Half-move clock after a move (zeta.cl:2361-2373; kept in a u8). */
ZHD int next_hmc(int hmc, Move m) {
  int pf = m_pfrom(m) >> 1, f = m_from(m), t = m_to(m);
  int h = (hmc + 1) & 0xFF;
  if (pf == PAWN || (m_pcpt(m) >> 1) != PNONE) h = 0;
  if (pf == KING && (f - t == 2 || t - f == 2)) h = 0;
  return h;
}

}  // namespace zeta
