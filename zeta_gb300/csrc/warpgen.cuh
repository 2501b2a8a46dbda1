/*
 * warpgen.cuh -- the search kernels' legal-move list built by a whole warp.
 *
 * gen_engine (movegen_fast.cuh) runs 23 emitters in a fixed order -- eight
 * slider directions, four pawn sets, eight knight jumps, the king, castling
 * and en passant -- each turning one target bitboard into moves, lowest
 * square first.  The list is thus fully described by those 23 bitboards:
 * move j is the j-th set bit counted across the emitters in order.  Here
 * the bitboards are computed once with gen_engine's own set operations
 * (gen_plan), and then move j is built by lane j % 32 (gen_decode): a
 * 35-move list costs two parallel rounds instead of 35 serial emitter
 * iterations on one thread, and comes out identical to gen_engine's, in
 * the same order.
 *
 * gen_plan and gen_decode are plain functions (host and device): the CPU
 * tests compile them for the host and compare the decoded list with
 * gen_engine's on every node of full move trees.
 */
#pragma once

#include "movegen_fast.cuh"

namespace zeta {

#ifndef ZE
#define ZE __host__ __device__ __forceinline__
#endif

constexpr int kEmitters = 23;
/* emitter index: 0-7 slider directions, 8 pawn single push, 9 pawn double
 * push, 10-11 pawn captures, 12-19 knight jumps, 20 king, 21 castling
 * (target squares), 22 en passant (bit 0 the capturer on sqep-1, bit 1 on
 * sqep+1) */

/* pawn shifts of emitters 8-11 by side to move, knight shifts of 12-19:
 * gen_engine's emission order */
ZE int pawn_delta(int k, int stm) {
  return stm ? (k == 0 ? -8 : k == 1 ? -16 : k == 2 ? -7 : -9) : (k == 0 ? 8 : k == 1 ? 16 : k == 2 ? 9 : 7);
}
ZE int knight_delta(int k) {
  return k == 0 ? 17 : k == 1 ? 15 : k == 2 ? 10 : k == 3 ? 6 : k == 4 ? -17 : k == 5 ? -15 : k == 6 ? -10 : -6;
}

/* The 23 target sets of gen_engine for (p, stm), written to set[0..22];
 * returns the number of legal moves.  *in_check: the side to move is in
 * check; *sqep: the en-passant square (for emitter 22). */
ZE int gen_plan(const Pos &p, const Sets &s, u64 danger, int stm, bool qs, u64 *set, bool *in_check, int *sqep) {
  const Guard g = make_guard(s, stm);
  const u64 capmask = qs ? s.them : ~0ULL;
  const u64 tgt = ~s.us & g.cmask & capmask;
  set[0] = slider_targets<0>(s, g, tgt);
  set[1] = slider_targets<1>(s, g, tgt);
  set[2] = slider_targets<2>(s, g, tgt);
  set[3] = slider_targets<3>(s, g, tgt);
  set[4] = slider_targets<4>(s, g, tgt);
  set[5] = slider_targets<5>(s, g, tgt);
  set[6] = slider_targets<6>(s, g, tgt);
  set[7] = slider_targets<7>(s, g, tgt);
  const u64 empty = ~s.occ;
  const u64 P = s.pawns & s.us;
  const u64 free_ = ~g.pinned;
  const u64 pp = P & (free_ | g.pin[0]);
  const u64 pd = P & (free_ | g.pin[2]);
  const u64 pa = P & (free_ | g.pin[3]);
  if (stm) {
    const u64 s1 = (pp >> 8) & empty;
    const u64 s2 = ((s1 & ZETA_RANK6) >> 8) & empty;
    set[8] = qs ? 0ULL : s1 & g.cmask;
    set[9] = qs ? 0ULL : s2 & g.cmask;
    set[10] = ((pa >> 7) & ZETA_NOTA) & s.them & g.cmask;
    set[11] = ((pd >> 9) & ZETA_NOTH) & s.them & g.cmask;
  } else {
    const u64 s1 = (pp << 8) & empty;
    const u64 s2 = ((s1 & ZETA_RANK3) << 8) & empty;
    set[8] = qs ? 0ULL : s1 & g.cmask;
    set[9] = qs ? 0ULL : s2 & g.cmask;
    set[10] = ((pd << 9) & ZETA_NOTA) & s.them & g.cmask;
    set[11] = ((pa << 7) & ZETA_NOTH) & s.them & g.cmask;
  }
  const u64 N = s.knights & s.us & free_;
  set[12] = ((N << 17) & ZETA_NOTA) & tgt;
  set[13] = ((N << 15) & ZETA_NOTH) & tgt;
  set[14] = ((N << 10) & ZETA_NOTAB) & tgt;
  set[15] = ((N << 6) & ZETA_NOTGH) & tgt;
  set[16] = ((N >> 17) & ZETA_NOTH) & tgt;
  set[17] = ((N >> 15) & ZETA_NOTA) & tgt;
  set[18] = ((N >> 10) & ZETA_NOTGH) & tgt;
  set[19] = ((N >> 6) & ZETA_NOTAB) & tgt;
  set[20] = king_attacks(s.kbb) & ~s.us & ~danger & capmask;
  u64 cs = 0;
  if (!qs) {
    const int c = castles(p, s, stm, danger);
    if (c & 1) cs |= bit(s.ksq - 2);
    if (c & 2) cs |= bit(s.ksq + 2);
  }
  set[21] = cs;
  int ep_sq = 0;
  set[22] = (u64)ep_legal(p, s, stm, ep_sq);
  *sqep = ep_sq;
  *in_check = g.checkers != 0;
  int n = 0;
#pragma unroll
  for (int e = 0; e < kEmitters; e++) n += popc(set[e]);
  return n;
}

/* index of the k-th (0-based) set bit of x; k < popc(x) */
ZE int select_bit(u64 x, int k) {
  unsigned long long v = (unsigned long long)x;
  int base = 0;
  int c = popc(u64(v & 0xFFFFFFFFULL));
  if (k >= c) {
    k -= c;
    v >>= 32;
    base = 32;
  }
  c = popc(u64(v & 0xFFFFULL));
  if (k >= c) {
    k -= c;
    v >>= 16;
    base += 16;
  }
  c = popc(u64(v & 0xFFULL));
  if (k >= c) {
    k -= c;
    v >>= 8;
    base += 8;
  }
  c = popc(u64(v & 0xFULL));
  if (k >= c) {
    k -= c;
    v >>= 4;
    base += 4;
  }
  for (int i = 0; i < k; i++) v &= v - 1; /* k < 4 here */
  return base + ctz(u64(v));
}

/* Move `sq` of emitter e (sq: the target square; for e == 22 the variant
 * bit), exactly as gen_engine builds it. */
ZE Move gen_decode(const Pos &p, const Sets &s, int stm, int e, int sq, int sqep) {
  if (e < 8) {
    int from;
    switch (e) {
      case 0: from = slider_from<0>(sq, s.occ); break;
      case 1: from = slider_from<1>(sq, s.occ); break;
      case 2: from = slider_from<2>(sq, s.occ); break;
      case 3: from = slider_from<3>(sq, s.occ); break;
      case 4: from = slider_from<4>(sq, s.occ); break;
      case 5: from = slider_from<5>(sq, s.occ); break;
      case 6: from = slider_from<6>(sq, s.occ); break;
      default: from = slider_from<7>(sq, s.occ); break;
    }
    const u64 queens = s.rq & s.bq;
    const int type = (queens & bit(from)) ? QUEEN : (e < 4 ? ROOK : BISHOP);
    return mv_known(p, s, from, sq, (type << 1) | stm);
  }
  if (e < 12) {
    const int pawn = (PAWN << 1) | stm, queen = (QUEEN << 1) | stm, last = stm ? 0 : 7;
    const int pto = (sq >> 3) == last ? queen : pawn;
    const int pcpt = e >= 10 ? piece_at(p, sq) : PNONE;
    return make_move(sq - pawn_delta(e - 8, stm), sq, sq, pawn, pto, pcpt);
  }
  if (e < 20) return mv_known(p, s, sq - knight_delta(e - 12), sq, (KNIGHT << 1) | stm);
  const int king = (KING << 1) | stm;
  if (e == 20) return mv_known(p, s, s.ksq, sq, king);
  if (e == 21) return make_move(s.ksq, sq, sq, king, king, PNONE);
  const int pawn = (PAWN << 1) | stm;
  const int to = stm ? sqep - 8 : sqep + 8;
  return make_move(sq ? sqep + 1 : sqep - 1, to, sqep, pawn, pawn, piece_at(p, sqep));
}

/* Move j of the list (0 <= j < n): its emitter by the prefix counts
 * off[0..23] (off[e] = moves before emitter e), then the set bit. */
ZE Move gen_move_at(const Pos &p, const Sets &s, int stm, const u64 *set, const uint8_t *off, int sqep, int j) {
  int e = 0;
#pragma unroll 1
  while (e < kEmitters - 1 && off[e + 1] <= j) e++;
  return gen_decode(p, s, stm, e, select_bit(set[e], j - off[e]), sqep);
}

/* ---------------- rolled form ----------------
 * The same sets computed with loops over the eight directions (one ray
 * fill with a run-time shift instead of eight unrolled ones).  A few more
 * instructions are executed, but the code is several times smaller: the
 * warp-cooperative search kernel is limited by instruction fetch, and this
 * one copy serves both its move generation and its leaf legality test. */

/* shift of direction d (0 N +8, 1 S -8, 2 E +1, 3 W -1, 4 NE +9, 5 SW -9,
 * 6 NW +7, 7 SE -7) and the mask that keeps a step on the board */
ZE int dir_shift(int d) {
  const int a = (int)((0x07090108u >> ((d >> 1) * 8)) & 0xFFu);
  return (d & 1) ? -a : a;
}
ZE u64 dir_mask(int d) {
  return d < 2 ? ~0ULL : (((d == 2) | (d == 4) | (d == 7)) ? (u64)ZETA_NOTA : (u64)ZETA_NOTH);
}
ZE u64 shift_dyn(u64 x, int s) { return s >= 0 ? (x << s) : (x >> (-s)); }

/* ray_attacks<d> with d known only at run time */
ZE u64 ray_dyn(u64 gen, u64 pro, int d) {
  const int s = dir_shift(d);
  const u64 m = dir_mask(d);
  pro &= m;
  gen |= pro & shift_dyn(gen, s);
  pro &= shift_dyn(pro, s);
  gen |= pro & shift_dyn(gen, 2 * s);
  pro &= shift_dyn(pro, 2 * s);
  gen |= pro & shift_dyn(gen, 4 * s);
  return shift_dyn(gen, s) & m;
}

/* enemy_attacks, rolled */
ZE u64 enemy_attacks_rolled(const Sets &s, int stm) {
  const u64 pro = ~s.occ | s.kbb;
  const u64 erq = s.rq & s.them, ebq = s.bq & s.them;
  u64 a = 0;
#pragma unroll 1
  for (int d = 0; d < 8; d++) a |= ray_dyn(d < 4 ? erq : ebq, pro, d);
  a |= pawn_attacks(s.pawns & s.them, !stm);
  a |= knight_attacks(s.knights & s.them);
  a |= king_attacks(s.kings & s.them);
  return a;
}

/* make_guard, rolled */
ZE Guard make_guard_rolled(const Sets &s, int stm) {
  Guard g;
  u64 p0 = 0, p1 = 0, p2 = 0, p3 = 0, checkers = 0, cm = 0;
  const u64 erq = s.rq & s.them, ebq = s.bq & s.them;
#pragma unroll 1
  for (int d = 0; d < 8; d++) {
    const u64 r = ray_dyn(s.kbb, ~s.them, d);
    const u64 hit = r & s.them & (d < 4 ? erq : ebq);
    const u64 own = r & s.us;
    const bool has = hit != 0;
    const bool chk = has && own == 0;
    const bool pin = has && own != 0 && (own & (own - 1)) == 0;
    checkers |= chk ? hit : 0ULL;
    cm |= chk ? r : 0ULL;
    const u64 pn = pin ? own : 0ULL;
    const int ax = d >> 1;
    p0 |= ax == 0 ? pn : 0ULL;
    p1 |= ax == 1 ? pn : 0ULL;
    p2 |= ax == 2 ? pn : 0ULL;
    p3 |= ax == 3 ? pn : 0ULL;
  }
  g.pin[0] = p0;
  g.pin[1] = p1;
  g.pin[2] = p2;
  g.pin[3] = p3;
  const u64 pc = pawn_attacks(s.kbb, stm) & s.pawns & s.them;
  const u64 nc = knight_attacks(s.kbb) & s.knights & s.them;
  g.checkers = checkers | pc | nc;
  cm |= pc | nc;
  g.pinned = p0 | p1 | p2 | p3;
  const u64 c = g.checkers;
  g.cmask = (c == 0) ? ~0ULL : ((c & (c - 1)) ? 0ULL : cm);
  return g;
}

/* attacked_after, rolled: is `ksq` attacked once an en-passant capture
 * has changed the occupancy */
ZE bool attacked_after_rolled(int ksq, u64 occ, u64 them, const Sets &s, int stm) {
  const u64 k = bit(ksq);
  const u64 pro = ~occ;
  const u64 erq = s.rq & them, ebq = s.bq & them;
  u64 hit = 0;
#pragma unroll 1
  for (int d = 0; d < 8; d++) hit |= ray_dyn(k, pro, d) & (d < 4 ? erq : ebq);
  hit |= knight_attacks(k) & s.knights & them;
  hit |= pawn_attacks(k, stm) & s.pawns & them;
  hit |= king_attacks(k) & s.kings & them;
  return hit != 0;
}

/* ep_legal, rolled */
ZE int ep_legal_rolled(const Pos &p, const Sets &s, int stm, int &sqep_out) {
  const u64 ep = ~p.cr & ZETA_EPMASK;
  sqep_out = 0;
  if (!ep) return 0;
  const int sqep = ctz(ep);
  sqep_out = sqep;
  const u64 cand = s.pawns & s.us & (stm ? ZETA_RANK4 : ZETA_RANK5);
  int res = 0;
#pragma unroll 1
  for (int i = 0; i < 2; i++) {
    const int from = sqep + (i ? 1 : -1);
    if (!(cand & bit(from))) continue;
    const int to = stm ? sqep - 8 : sqep + 8;
    const u64 tb = bit(to);
    const u64 occ2 = (s.occ & ~bit(from) & ~bit(sqep) & ~tb) | tb;
    const u64 them2 = s.them & ~bit(sqep) & ~tb;
    if (!attacked_after_rolled(s.ksq, occ2, them2, s, stm)) res |= 1 << i;
  }
  return res;
}

/* gen_plan, rolled: the same 23 sets, the same count, the same flags */
ZE int gen_plan_rolled(const Pos &p, const Sets &s, u64 danger, int stm, bool qs, u64 *set, bool *in_check,
                       int *sqep) {
  const Guard g = make_guard_rolled(s, stm);
  const u64 capmask = qs ? s.them : ~0ULL;
  const u64 tgt = ~s.us & g.cmask & capmask;
  int n = 0;
#pragma unroll 1
  for (int d = 0; d < 8; d++) {
    const u64 sl = (d < 4 ? s.rq : s.bq) & s.us;
    const int ax = d >> 1;
    const u64 pin = ax == 0 ? g.pin[0] : ax == 1 ? g.pin[1] : ax == 2 ? g.pin[2] : g.pin[3];
    const u64 t = ray_dyn(sl & (~g.pinned | pin), ~s.occ, d) & tgt;
    set[d] = t;
    n += popc(t);
  }
  const u64 empty = ~s.occ;
  const u64 P = s.pawns & s.us;
  const u64 free_ = ~g.pinned;
  const u64 pp = P & (free_ | g.pin[0]);
  const u64 pd = P & (free_ | g.pin[2]);
  const u64 pa = P & (free_ | g.pin[3]);
  u64 s1, s2, ca, cb;
  if (stm) {
    s1 = (pp >> 8) & empty;
    s2 = ((s1 & ZETA_RANK6) >> 8) & empty;
    ca = ((pa >> 7) & ZETA_NOTA) & s.them & g.cmask;
    cb = ((pd >> 9) & ZETA_NOTH) & s.them & g.cmask;
  } else {
    s1 = (pp << 8) & empty;
    s2 = ((s1 & ZETA_RANK3) << 8) & empty;
    ca = ((pd << 9) & ZETA_NOTA) & s.them & g.cmask;
    cb = ((pa << 7) & ZETA_NOTH) & s.them & g.cmask;
  }
  set[8] = qs ? 0ULL : s1 & g.cmask;
  set[9] = qs ? 0ULL : s2 & g.cmask;
  set[10] = ca;
  set[11] = cb;
  const u64 N = s.knights & s.us & free_;
  set[12] = ((N << 17) & ZETA_NOTA) & tgt;
  set[13] = ((N << 15) & ZETA_NOTH) & tgt;
  set[14] = ((N << 10) & ZETA_NOTAB) & tgt;
  set[15] = ((N << 6) & ZETA_NOTGH) & tgt;
  set[16] = ((N >> 17) & ZETA_NOTH) & tgt;
  set[17] = ((N >> 15) & ZETA_NOTA) & tgt;
  set[18] = ((N >> 10) & ZETA_NOTGH) & tgt;
  set[19] = ((N >> 6) & ZETA_NOTAB) & tgt;
  set[20] = king_attacks(s.kbb) & ~s.us & ~danger & capmask;
  u64 cs = 0;
  if (!qs) {
    const int c = castles(p, s, stm, danger);
    if (c & 1) cs |= bit(s.ksq - 2);
    if (c & 2) cs |= bit(s.ksq + 2);
  }
  set[21] = cs;
  int ep_sq = 0;
  set[22] = (u64)ep_legal_rolled(p, s, stm, ep_sq);
  *sqep = ep_sq;
  *in_check = g.checkers != 0;
#pragma unroll 1
  for (int e = 8; e < kEmitters; e++) n += popc(set[e]);
  return n;
}

/* has_free_move (chess.cuh) with the rolled pin and check test: a legal
 * move exists when the side to move is out of check and an unpinned
 * knight, slider or pawn has a first step; false means "undecided" */
ZE bool has_free_move_rolled(const Pos &p, int stm, bool &in_check) {
  const Sets s = make_sets(p, stm);
  const Guard g = make_guard_rolled(s, stm);
  in_check = g.checkers != 0;
  if (in_check) return false;
  const u64 free_ = s.us & ~g.pinned, open = ~s.us, empty = ~s.occ;
  if (knight_attacks(s.knights & free_) & open) return true;
  const u64 R = s.rq & free_, B = s.bq & free_;
  const u64 rstep = (R << 8) | (R >> 8) | ((R << 1) & ZETA_NOTA) | ((R >> 1) & ZETA_NOTH);
  const u64 bstep = ((B << 9) & ZETA_NOTA) | ((B << 7) & ZETA_NOTH) | ((B >> 7) & ZETA_NOTA) | ((B >> 9) & ZETA_NOTH);
  if ((rstep | bstep) & open) return true;
  const u64 P = s.pawns & free_;
  const u64 push = stm ? (P >> 8) : (P << 8);
  return ((push & empty) | (pawn_attacks(P, stm) & s.them)) != 0;
}

/* has_free_move_rolled, then a king step: when no other piece proves a
 * legal move -- always the case in check -- a king step to a square the
 * enemy does not attack (the attack map made with the king off the board,
 * so it cannot step back along a checking ray) is one.  true proves a legal
 * move; false leaves the question to the exact count.  in_check is exact. */
ZE bool has_quick_move_rolled(const Pos &p, int stm, bool &in_check) {
  if (has_free_move_rolled(p, stm, in_check)) return true;
  const Sets s = make_sets(p, stm);
  return (king_attacks(s.kbb) & ~s.us & ~enemy_attacks_rolled(s, stm)) != 0;
}

/* gen_decode with the slider's origin from a run-time-direction ray */
ZE Move gen_decode_rolled(const Pos &p, const Sets &s, int stm, int e, int sq, int sqep) {
  if (e < 8) {
    const int from = ctz(ray_dyn(bit(sq), ~s.occ, e ^ 1) & s.occ); /* first piece behind, along -e */
    const u64 queens = s.rq & s.bq;
    const int type = (queens & bit(from)) ? QUEEN : (e < 4 ? ROOK : BISHOP);
    return mv_known(p, s, from, sq, (type << 1) | stm);
  }
  return gen_decode(p, s, stm, e, sq, sqep);
}

ZE Move gen_move_at_rolled(const Pos &p, const Sets &s, int stm, const u64 *set, const uint8_t *off, int sqep,
                           int j) {
  int e = 0;
#pragma unroll 1
  while (e < kEmitters - 1 && off[e + 1] <= j) e++;
  return gen_decode_rolled(p, s, stm, e, select_bit(set[e], j - off[e]), sqep);
}

}  // namespace zeta
