/*
 * movegen_fast.cuh -- move generation and hash updates for the search
 * kernels (full engine and pure search), where one thread works on one
 * node at a time and the cost per node is latency:
 *   - gen_engine: the legal moves of gen_legal (chess.cuh), same packing,
 *     emitted with the moving piece known (one capture test per move
 *     instead of three piece lookups);
 *   - zkey / cr_keys / piece_delta: the Zobrist hash of a child from its
 *     parent's, equal to hashing the child from scratch (the hash is an
 *     XOR over pieces plus castle, en-passant and side-to-move keys).
 * The perft kernels keep gen_legal: their fixed per-node operation count
 * is measured on it.
 */
#pragma once

#include "chess.cuh"
#include "tables.cuh"

namespace zeta {

#ifndef ZE
#define ZE __host__ __device__ __forceinline__
#endif

/* Zobrist key of piece pc on sq, as computehash adds it (zeta.cl:614-661) */
ZE u64 zkey(int pc, int sq) { return rotl64(zobrist((pc & 1) * 6 + (pc >> 1) - 1), sq); }
/* the castle and en-passant part of the hash, a function of the moved flags */
ZE u64 cr_keys(u64 cr) {
  u64 h = 0;
  if (~cr & ZETA_CR_WQ) h ^= zobrist(12);
  if (~cr & ZETA_CR_WK) h ^= zobrist(13);
  if (~cr & ZETA_CR_BQ) h ^= zobrist(14);
  if (~cr & ZETA_CR_BK) h ^= zobrist(15);
  const u64 ep = ~cr & ZETA_EPMASK;
  if (ep) h ^= rotl64(zobrist(16), ctz(ep) & 7);
  return h;
}
/* change of the piece part of the hash made by a (real) move: the hash is
 * an XOR over pieces, so the child's value is the parent's with the moved,
 * captured and castling-rook keys toggled -- equal to hashing the child
 * from scratch, as the reference does at every move (zeta.cl:2294-2359) */
ZE u64 piece_delta(Move m) {
  const int f = m_from(m), t = m_to(m), c = m_cpt(m), pf = m_pfrom(m), pt = m_pto(m), pc = m_pcpt(m);
  u64 x = zkey(pf, f) ^ zkey(pt, t);
  if (pc >> 1) x ^= zkey(pc, c);
  const int rook = (ROOK << 1) | (pf & 1);
  if ((pf >> 1) == KING && f - t == 2) x ^= zkey(rook, f - 4) ^ zkey(rook, t + 1);
  if ((pf >> 1) == KING && t - f == 2) x ^= zkey(rook, f + 3) ^ zkey(rook, t - 1);
  return x;
}

/* The same legal moves, in the same packing, as gen_legal; the emitters
 * know the moving piece, so a move costs one capture test instead of
 * three piece lookups.  The list order differs from gen_legal's: callers
 * order moves by score, not by list position. */
ZE Move mv_known(const Pos &p, const Sets &s, int from, int to, int pfrom) {
  const int pcpt = (s.them & bit(to)) ? piece_at(p, to) : PNONE;
  return make_move(from, to, to, pfrom, pfrom, pcpt);
}

template <int D>
ZE int emit_slider_k(const Pos &p, const Sets &s, const Guard &g, u64 tgt, int stm, Move *list, int n) {
  u64 t = slider_targets<D>(s, g, tgt);
  const u64 queens = s.rq & s.bq;
  while (t) {
    const int to = ctz(t);
    t &= t - 1;
    const int from = slider_from<D>(to, s.occ);
    const int type = (queens & bit(from)) ? QUEEN : (D < 4 ? ROOK : BISHOP);
    list[n++] = mv_known(p, s, from, to, (type << 1) | stm);
  }
  return n;
}

/* knights and pawn captures: a fixed shift back to the origin */
ZE int emit_shift_k(const Pos &p, const Sets &s, u64 t, int delta, int pfrom, Move *list, int n) {
  while (t) {
    const int to = ctz(t);
    t &= t - 1;
    list[n++] = mv_known(p, s, to - delta, to, pfrom);
  }
  return n;
}

/* pawn moves: queen promotion on the last rank; pushes capture nothing */
ZE int emit_pawn_k(const Pos &p, const Sets &s, u64 t, int delta, int stm, bool capture, Move *list, int n) {
  const int pawn = (PAWN << 1) | stm, queen = (QUEEN << 1) | stm, last = stm ? 0 : 7;
  while (t) {
    const int to = ctz(t);
    t &= t - 1;
    const int pto = (to >> 3) == last ? queen : pawn;
    const int pcpt = capture ? piece_at(p, to) : PNONE;
    list[n++] = make_move(to - delta, to, to, pawn, pto, pcpt);
  }
  return n;
}

ZE int gen_engine(const Pos &p, const Sets &s, u64 danger, int stm, bool qs,
                                                Move *list) {
  const Guard g = make_guard(s, stm);
  const u64 capmask = qs ? s.them : ~0ULL;
  const u64 tgt = ~s.us & g.cmask & capmask;
  int n = 0;
  n = emit_slider_k<0>(p, s, g, tgt, stm, list, n);
  n = emit_slider_k<1>(p, s, g, tgt, stm, list, n);
  n = emit_slider_k<2>(p, s, g, tgt, stm, list, n);
  n = emit_slider_k<3>(p, s, g, tgt, stm, list, n);
  n = emit_slider_k<4>(p, s, g, tgt, stm, list, n);
  n = emit_slider_k<5>(p, s, g, tgt, stm, list, n);
  n = emit_slider_k<6>(p, s, g, tgt, stm, list, n);
  n = emit_slider_k<7>(p, s, g, tgt, stm, list, n);
  const u64 empty = ~s.occ;
  const u64 P = s.pawns & s.us;
  const u64 free_ = ~g.pinned;
  const u64 pp = P & (free_ | g.pin[0]);
  const u64 pd = P & (free_ | g.pin[2]);
  const u64 pa = P & (free_ | g.pin[3]);
  if (stm) {
    const u64 s1 = (pp >> 8) & empty;
    const u64 s2 = ((s1 & ZETA_RANK6) >> 8) & empty;
    if (!qs) {
      n = emit_pawn_k(p, s, s1 & g.cmask, -8, stm, false, list, n);
      n = emit_pawn_k(p, s, s2 & g.cmask, -16, stm, false, list, n);
    }
    n = emit_pawn_k(p, s, ((pa >> 7) & ZETA_NOTA) & s.them & g.cmask, -7, stm, true, list, n);
    n = emit_pawn_k(p, s, ((pd >> 9) & ZETA_NOTH) & s.them & g.cmask, -9, stm, true, list, n);
  } else {
    const u64 s1 = (pp << 8) & empty;
    const u64 s2 = ((s1 & ZETA_RANK3) << 8) & empty;
    if (!qs) {
      n = emit_pawn_k(p, s, s1 & g.cmask, 8, stm, false, list, n);
      n = emit_pawn_k(p, s, s2 & g.cmask, 16, stm, false, list, n);
    }
    n = emit_pawn_k(p, s, ((pd << 9) & ZETA_NOTA) & s.them & g.cmask, 9, stm, true, list, n);
    n = emit_pawn_k(p, s, ((pa << 7) & ZETA_NOTH) & s.them & g.cmask, 7, stm, true, list, n);
  }
  const u64 N = s.knights & s.us & free_;
  const int knight = (KNIGHT << 1) | stm;
  n = emit_shift_k(p, s, ((N << 17) & ZETA_NOTA) & tgt, 17, knight, list, n);
  n = emit_shift_k(p, s, ((N << 15) & ZETA_NOTH) & tgt, 15, knight, list, n);
  n = emit_shift_k(p, s, ((N << 10) & ZETA_NOTAB) & tgt, 10, knight, list, n);
  n = emit_shift_k(p, s, ((N << 6) & ZETA_NOTGH) & tgt, 6, knight, list, n);
  n = emit_shift_k(p, s, ((N >> 17) & ZETA_NOTH) & tgt, -17, knight, list, n);
  n = emit_shift_k(p, s, ((N >> 15) & ZETA_NOTA) & tgt, -15, knight, list, n);
  n = emit_shift_k(p, s, ((N >> 10) & ZETA_NOTGH) & tgt, -10, knight, list, n);
  n = emit_shift_k(p, s, ((N >> 6) & ZETA_NOTAB) & tgt, -6, knight, list, n);
  const int king = (KING << 1) | stm;
  {
    u64 t = king_attacks(s.kbb) & ~s.us & ~danger & capmask;
    while (t) {
      const int to = ctz(t);
      t &= t - 1;
      list[n++] = mv_known(p, s, s.ksq, to, king);
    }
  }
  if (!qs) {
    const int c = castles(p, s, stm, danger);
    if (c & 1) list[n++] = make_move(s.ksq, (s.ksq - 2) & 63, (s.ksq - 2) & 63, king, king, PNONE);
    if (c & 2) list[n++] = make_move(s.ksq, (s.ksq + 2) & 63, (s.ksq + 2) & 63, king, king, PNONE);
  }
  int sqep;
  const int e = ep_legal(p, s, stm, sqep);
  if (e) {
    const int to = stm ? sqep - 8 : sqep + 8;
    const int pawn = (PAWN << 1) | stm;
    const int victim = piece_at(p, sqep);
    if (e & 1) list[n++] = make_move(sqep - 1, to, sqep, pawn, pawn, victim);
    if (e & 2) list[n++] = make_move(sqep + 1, to, sqep, pawn, pawn, victim);
  }
  return n;
}

}  // namespace zeta
