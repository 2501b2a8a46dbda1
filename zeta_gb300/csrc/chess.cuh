/*
 * chess.cuh -- quad-bitboard chess core for the GB300 kernels.
 *
 * The position layout is the reference's (src/types.h:59-66): black
 * pieces, three piece-type bit planes (piece = type<<1 | color, types
 * P=1 N=2 K=3 B=4 R=5 Q=6) and the "piece moved" flag word that carries
 * castle rights and the en-passant target.  Moves use the reference's
 * 32-bit packing (src/types.h:67-74,130-141).
 *
 * Move generation is set-wise instead of one work-item per square
 * (zetaperft.cl:1063-1311): every slider direction is one Kogge-Stone
 * occluded fill over all sliders of that direction at once, pins and
 * checks come from eight x-ray fills out of the king square, and a node
 * whose children are leaves is counted with popcounts instead of being
 * expanded.  The legal move set is the reference's exactly: queen-only
 * promotions (zetaperft.cl:1380-1384), castle rules keyed on the moved
 * flags with shift counts taken mod 64 (zetaperft.cl:1249-1297), and en
 * passant checked by making the capture (zetaperft.cl:1222-1248).
 */
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define ZHD __host__ __device__ __forceinline__
#else
#define ZHD static inline
#endif

/* The bitboard word.  The op counter (opcount.cc) compiles this file on
 * the host with a counting word type to measure the algorithmic integer
 * operations per node; every other build uses plain 64-bit integers. */
#ifndef ZETA_WORD_TYPE
#define ZETA_WORD_TYPE unsigned long long
#define ZETA_OPS(n) ((void)0)
#endif

namespace zeta {

typedef ZETA_WORD_TYPE u64;
typedef uint32_t Move;

/* piece types and flag masks (src/types.h:94-124) */
enum { PNONE = 0, PAWN = 1, KNIGHT = 2, KING = 3, BISHOP = 4, ROOK = 5, QUEEN = 6 };
#define ZETA_NOTA 0xFEFEFEFEFEFEFEFEULL
#define ZETA_NOTH 0x7F7F7F7F7F7F7F7FULL
#define ZETA_NOTAB 0xFCFCFCFCFCFCFCFCULL
#define ZETA_NOTGH 0x3F3F3F3F3F3F3F3FULL
#define ZETA_EPMASK 0x000000FFFF000000ULL
#define ZETA_CR_ALL 0x8900000000000091ULL
#define ZETA_CR_WQ 0x0000000000000011ULL
#define ZETA_CR_WK 0x0000000000000090ULL
#define ZETA_CR_BQ 0x1100000000000000ULL
#define ZETA_CR_BK 0x9000000000000000ULL
#define ZETA_RANK3 0x0000000000FF0000ULL
#define ZETA_RANK4 0x00000000FF000000ULL
#define ZETA_RANK5 0x000000FF00000000ULL
#define ZETA_RANK6 0x0000FF0000000000ULL
#define ZETA_RANK1 0x00000000000000FFULL
#define ZETA_RANK8 0xFF00000000000000ULL
#define ZETA_NULLMOVE 0x41u

/* A position without hash and clock: what move generation needs. */
struct Pos {
  u64 b0, p1, p2, p3; /* black, type bit planes */
  u64 cr;             /* moved flags (castle rights, ep target) */
};

ZHD int popc(u64 x) {
  ZETA_OPS(2);
#if defined(__CUDA_ARCH__)
  return __popcll(x);
#else
  return __builtin_popcountll((unsigned long long)x);
#endif
}
ZHD int ctz(u64 x) {
  ZETA_OPS(2);
#if defined(__CUDA_ARCH__)
  return __ffsll((long long)x) - 1;
#else
  return __builtin_ctzll((unsigned long long)x);
#endif
}
/* OpenCL shift semantics: counts mod 64 */
ZHD u64 bit(int sq) {
  ZETA_OPS(4); /* a variable shift */
  return u64(1ULL << (sq & 63));
}

/* The initial position as setboard leaves it (src/io.c:335-531): all
 * moved flags set except the six castle squares. */
ZHD Pos start_pos() {
  const u64 pawns = 0x00FF00000000FF00ULL, knights = 0x4200000000000042ULL, bishops = 0x2400000000000024ULL,
            rooks = 0x8100000000000081ULL, queens = 0x0800000000000008ULL, kings = 0x1000000000000010ULL;
  Pos p;
  p.b0 = 0xFFFF000000000000ULL;
  p.p1 = pawns | kings | rooks;    /* type bit 0: P K R */
  p.p2 = knights | kings | queens; /* type bit 1: N K Q */
  p.p3 = bishops | rooks | queens; /* type bit 2: B R Q */
  p.cr = ~(ZETA_CR_WQ | ZETA_CR_WK | ZETA_CR_BQ | ZETA_CR_BK);
  return p;
}

ZHD int piece_at(const Pos &p, int sq) {
  sq &= 63;
  ZETA_OPS(4 * 6 + 3 * 2); /* four variable shifts and masks, three ors */
  const unsigned long long b0 = (unsigned long long)p.b0, p1 = (unsigned long long)p.p1,
                           p2 = (unsigned long long)p.p2, p3 = (unsigned long long)p.p3;
  return (int)(((b0 >> sq) & 1) | (((p1 >> sq) & 1) << 1) | (((p2 >> sq) & 1) << 2) | (((p3 >> sq) & 1) << 3));
}

/* ---------------- directions ----------------
 * 0 N(+8) 1 S(-8) 2 E(+1) 3 W(-1) 4 NE(+9) 5 SW(-9) 6 NW(+7) 7 SE(-7)
 * axis(d) = d>>1: 0 file, 1 rank, 2 a1-h8 diagonal, 3 h1-a8 diagonal */
template <int D>
struct Dir;
template <> struct Dir<0> { static constexpr int s = 8;  static constexpr u64 m = ~0ULL; };
template <> struct Dir<1> { static constexpr int s = -8; static constexpr u64 m = ~0ULL; };
template <> struct Dir<2> { static constexpr int s = 1;  static constexpr u64 m = ZETA_NOTA; };
template <> struct Dir<3> { static constexpr int s = -1; static constexpr u64 m = ZETA_NOTH; };
template <> struct Dir<4> { static constexpr int s = 9;  static constexpr u64 m = ZETA_NOTA; };
template <> struct Dir<5> { static constexpr int s = -9; static constexpr u64 m = ZETA_NOTH; };
template <> struct Dir<6> { static constexpr int s = 7;  static constexpr u64 m = ZETA_NOTH; };
template <> struct Dir<7> { static constexpr int s = -7; static constexpr u64 m = ZETA_NOTA; };

template <int S>
ZHD u64 sh(u64 x) {
  if constexpr (S > 0) return x << S;
  else return x >> (-S);
}

/* Kogge-Stone occluded fill of `gen` through `pro`, then one step:
 * the squares attacked in direction D (first blocker included). */
template <int D>
ZHD u64 ray_attacks(u64 gen, u64 pro) {
  constexpr int s = Dir<D>::s;
  constexpr u64 m = Dir<D>::m;
  pro &= m;
  gen |= pro & sh<s>(gen);
  pro &= sh<s>(pro);
  gen |= pro & sh<2 * s>(gen);
  pro &= sh<2 * s>(pro);
  gen |= pro & sh<4 * s>(gen);
  return sh<s>(gen) & m;
}

ZHD u64 king_attacks(u64 k) {
  u64 a = ((k << 1) & ZETA_NOTA) | ((k >> 1) & ZETA_NOTH);
  u64 r = a | k;
  return a | (r << 8) | (r >> 8);
}
ZHD u64 knight_attacks(u64 n) {
  u64 l1 = (n >> 1) & ZETA_NOTH, l2 = (n >> 2) & ZETA_NOTGH;
  u64 r1 = (n << 1) & ZETA_NOTA, r2 = (n << 2) & ZETA_NOTAB;
  u64 h1 = l1 | r1, h2 = l2 | r2;
  return (h1 << 16) | (h1 >> 16) | (h2 << 8) | (h2 >> 8);
}
/* squares attacked by pawns of colour c */
ZHD u64 pawn_attacks(u64 p, int c) {
  return c ? (((p >> 7) & ZETA_NOTA) | ((p >> 9) & ZETA_NOTH))
           : (((p << 9) & ZETA_NOTA) | ((p << 7) & ZETA_NOTH));
}

/* Piece sets of one position seen from the side to move. */
struct Sets {
  u64 occ, us, them, pawns, knights, kings, rq, bq;
  u64 kbb;
  int ksq;
};

ZHD Sets make_sets(const Pos &p, int stm) {
  Sets s;
  s.occ = p.p1 | p.p2 | p.p3;
  u64 white = s.occ ^ p.b0;
  s.us = stm ? p.b0 : white;
  s.them = s.occ ^ s.us;
  s.pawns = p.p1 & ~p.p2 & ~p.p3;
  s.knights = p.p2 & ~p.p1 & ~p.p3;
  s.kings = p.p1 & p.p2 & ~p.p3;
  s.rq = p.p3 & (p.p1 ^ p.p2);
  s.bq = p.p3 & ~p.p1;
  s.kbb = s.kings & s.us;
  s.ksq = ctz(s.kbb | (1ULL << 63)); /* a king always exists in a legal position */
  return s;
}

/* Squares attacked by the side not to move, with our king taken off the
 * board so that it cannot hide behind itself (zetaperft.cl:1066-1169). */
ZHD u64 enemy_attacks(const Sets &s, int stm) {
  u64 pro = ~s.occ | s.kbb;
  u64 erq = s.rq & s.them, ebq = s.bq & s.them;
  u64 a = ray_attacks<0>(erq, pro) | ray_attacks<1>(erq, pro) | ray_attacks<2>(erq, pro) |
          ray_attacks<3>(erq, pro);
  a |= ray_attacks<4>(ebq, pro) | ray_attacks<5>(ebq, pro) | ray_attacks<6>(ebq, pro) |
       ray_attacks<7>(ebq, pro);
  a |= pawn_attacks(s.pawns & s.them, !stm);
  a |= knight_attacks(s.knights & s.them);
  a |= king_attacks(s.kings & s.them);
  return a;
}

/* Pins and checks from eight x-ray fills out of the king square: each
 * ray passes our own pieces and stops at the first enemy piece. */
struct Guard {
  u64 pin[4];    /* pinned own pieces, by pin axis */
  u64 pinned;    /* union */
  u64 cmask;     /* allowed targets for non-king moves (check evasion) */
  u64 checkers;
};

template <int D>
ZHD void xray_dir(const Sets &s, u64 sl, Guard &g, u64 &cm) {
  u64 r = ray_attacks<D>(s.kbb, ~s.them);
  u64 hit = r & s.them & sl;
  u64 own = r & s.us;
  bool has = hit != 0;
  bool chk = has && own == 0;
  bool pin = has && own != 0 && (own & (own - 1)) == 0;
  g.checkers |= chk ? hit : 0ULL;
  cm |= chk ? r : 0ULL;
  g.pin[D >> 1] |= pin ? own : 0ULL;
}

ZHD Guard make_guard(const Sets &s, int stm) {
  Guard g;
  g.pin[0] = g.pin[1] = g.pin[2] = g.pin[3] = 0;
  g.checkers = 0;
  u64 cm = 0;
  u64 erq = s.rq & s.them, ebq = s.bq & s.them;
  xray_dir<0>(s, erq, g, cm);
  xray_dir<1>(s, erq, g, cm);
  xray_dir<2>(s, erq, g, cm);
  xray_dir<3>(s, erq, g, cm);
  xray_dir<4>(s, ebq, g, cm);
  xray_dir<5>(s, ebq, g, cm);
  xray_dir<6>(s, ebq, g, cm);
  xray_dir<7>(s, ebq, g, cm);
  u64 pc = pawn_attacks(s.kbb, stm) & s.pawns & s.them;
  u64 nc = knight_attacks(s.kbb) & s.knights & s.them;
  g.checkers |= pc | nc;
  cm |= pc | nc;
  g.pinned = g.pin[0] | g.pin[1] | g.pin[2] | g.pin[3];
  u64 c = g.checkers;
  g.cmask = (c == 0) ? ~0ULL : ((c & (c - 1)) ? 0ULL : cm);
  return g;
}

/* Is `ksq` attacked after an en-passant capture?  post-move sets. */
ZHD bool attacked_after(int ksq, u64 occ, u64 them, const Sets &s, int stm) {
  u64 k = bit(ksq);
  u64 pro = ~occ;
  u64 erq = s.rq & them, ebq = s.bq & them;
  u64 a = ray_attacks<0>(k, pro) | ray_attacks<1>(k, pro) | ray_attacks<2>(k, pro) |
          ray_attacks<3>(k, pro);
  if (a & erq) return true;
  u64 b = ray_attacks<4>(k, pro) | ray_attacks<5>(k, pro) | ray_attacks<6>(k, pro) |
          ray_attacks<7>(k, pro);
  if (b & ebq) return true;
  if (knight_attacks(k) & s.knights & them) return true;
  if (pawn_attacks(k, stm) & s.pawns & them) return true;
  if (king_attacks(k) & s.kings & them) return true;
  return false;
}

/* En-passant captures that are legal: bit i set for the capturer on
 * sqep-1 (i=0) and sqep+1 (i=1).  zetaperft.cl:1222-1248. */
ZHD int ep_legal(const Pos &p, const Sets &s, int stm, int &sqep_out) {
  u64 ep = ~p.cr & ZETA_EPMASK;
  sqep_out = 0;
  if (!ep) return 0;
  int sqep = ctz(ep);
  sqep_out = sqep;
  u64 cand = s.pawns & s.us & (stm ? ZETA_RANK4 : ZETA_RANK5);
  int res = 0;
#pragma unroll
  for (int i = 0; i < 2; i++) {
    int from = sqep + (i ? 1 : -1);
    if (!(cand & bit(from))) continue;
    int to = stm ? sqep - 8 : sqep + 8;
    u64 tb = bit(to);
    u64 occ2 = (s.occ & ~bit(from) & ~bit(sqep) & ~tb) | tb;
    u64 them2 = s.them & ~bit(sqep) & ~tb;
    if (!attacked_after(s.ksq, occ2, them2, s, stm)) res |= 1 << i;
  }
  return res;
}

/* Castle moves allowed: bit 0 queenside, bit 1 kingside
 * (zetaperft.cl:1249-1297, shift counts mod 64). */
ZHD int castles(const Pos &p, const Sets &s, int stm, u64 danger) {
  u64 cr = p.cr;
  int k = s.ksq;
  int rook = (ROOK << 1) | stm;
  bool any = (cr & ZETA_CR_ALL) != 0;
  u64 q = stm ? ZETA_CR_BQ : ZETA_CR_WQ, kk = stm ? ZETA_CR_BK : ZETA_CR_WK;
  int res = 0;
  if (any && (~cr & q) == q && piece_at(p, k - 4) == rook &&
      !(s.occ & (bit(k - 1) | bit(k - 2) | bit(k - 3))) &&
      !(danger & (bit(k) | bit(k - 1) | bit(k - 2))))
    res |= 1;
  if (any && (~cr & kk) == kk && piece_at(p, k + 3) == rook && !(s.occ & (bit(k + 1) | bit(k + 2))) &&
      !(danger & (bit(k) | bit(k + 1) | bit(k + 2))))
    res |= 2;
  return res;
}

/* Movers of slider direction D: sliders of the right kind that are not
 * pinned, or pinned along D's own axis. */
template <int D>
ZHD u64 slider_targets(const Sets &s, const Guard &g, u64 tgt) {
  u64 sl = ((D < 4) ? s.rq : s.bq) & s.us;
  u64 mv = sl & (~g.pinned | g.pin[D >> 1]);
  return ray_attacks<D>(mv, ~s.occ) & tgt;
}

/* ---------------- bulk count ----------------
 * Number of legal moves: the leaf count of a node one ply above the
 * leaves, without expanding it.  ALLP: a pawn reaching the last rank
 * makes four moves (queen, rook, bishop, knight) instead of the
 * reference's one queen promotion. */
template <bool ALLP = false>
ZHD int count_legal_ex(const Pos &p, int stm, bool &in_check) {
  Sets s = make_sets(p, stm);
  Guard g = make_guard(s, stm);
  in_check = (bool)(g.checkers != 0);
  u64 danger = enemy_attacks(s, stm);
  u64 tgt = ~s.us & g.cmask;
  int n = popc(king_attacks(s.kbb) & ~s.us & ~danger);
  n += popc(slider_targets<0>(s, g, tgt)) + popc(slider_targets<1>(s, g, tgt)) +
       popc(slider_targets<2>(s, g, tgt)) + popc(slider_targets<3>(s, g, tgt)) +
       popc(slider_targets<4>(s, g, tgt)) + popc(slider_targets<5>(s, g, tgt)) +
       popc(slider_targets<6>(s, g, tgt)) + popc(slider_targets<7>(s, g, tgt));
  u64 empty = ~s.occ;
  u64 P = s.pawns & s.us;
  u64 free_ = ~g.pinned;
  u64 pp = P & (free_ | g.pin[0]);
  u64 pd = P & (free_ | g.pin[2]);  /* a1-h8 diagonal */
  u64 pa = P & (free_ | g.pin[3]);  /* h1-a8 diagonal */
  u64 s1, s2, c1, c2;
  if (stm) {
    s1 = (pp >> 8) & empty;
    s2 = ((s1 & ZETA_RANK6) >> 8) & empty;
    c1 = (pa >> 7) & ZETA_NOTA; /* SE */
    c2 = (pd >> 9) & ZETA_NOTH; /* SW */
  } else {
    s1 = (pp << 8) & empty;
    s2 = ((s1 & ZETA_RANK3) << 8) & empty;
    c1 = (pd << 9) & ZETA_NOTA; /* NE */
    c2 = (pa << 7) & ZETA_NOTH; /* NW */
  }
  n += popc(s1 & g.cmask) + popc(s2 & g.cmask) + popc(c1 & s.them & g.cmask) +
       popc(c2 & s.them & g.cmask);
  if (ALLP) {
    /* pushes land on empty squares, captures on enemy ones: s1 and c1 are
     * disjoint, but c1 and c2 may share a square (two pawns taking the same
     * piece), so c2 is counted on its own */
    const u64 last = g.cmask & (stm ? ZETA_RANK1 : ZETA_RANK8);
    n += 3 * (popc((s1 | (c1 & s.them)) & last) + popc(c2 & s.them & last));
  }
  u64 N = s.knights & s.us & free_;
  n += popc(((N << 17) & ZETA_NOTA) & tgt) + popc(((N << 15) & ZETA_NOTH) & tgt) +
       popc(((N << 10) & ZETA_NOTAB) & tgt) + popc(((N << 6) & ZETA_NOTGH) & tgt) +
       popc(((N >> 17) & ZETA_NOTH) & tgt) + popc(((N >> 15) & ZETA_NOTA) & tgt) +
       popc(((N >> 10) & ZETA_NOTGH) & tgt) + popc(((N >> 6) & ZETA_NOTAB) & tgt);
  int c = castles(p, s, stm, danger);
  n += (c & 1) + (c >> 1);
  int sqep;
  int e = ep_legal(p, s, stm, sqep);
  n += (e & 1) + (e >> 1);
  return n;
}

template <bool ALLP = false>
ZHD int count_legal(const Pos &p, int stm) {
  bool in_check;
  return count_legal_ex<ALLP>(p, stm, in_check);
}

/* A quick sufficient test for "the side to move has a legal move": out of
 * check, any move of a piece that is not pinned is legal, so a free
 * knight, pawn or slider with a first step it may take proves one without
 * the attack map.  True: a legal move exists.  False: undecided (in check,
 * or only the king, pinned pieces, en passant or castling could move) --
 * the exact count decides.  in_check is set either way. */
ZHD bool has_free_move(const Pos &p, int stm, bool &in_check) {
  const Sets s = make_sets(p, stm);
  const Guard g = make_guard(s, stm);
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

/* count_legal_ex(...) > 0, with the quick test first */
ZHD bool has_legal_ex(const Pos &p, int stm, bool &in_check) {
  if (has_free_move(p, stm, in_check)) return true;
  bool chk;
  return count_legal_ex(p, stm, chk) > 0;
}

/* ---------------- make ----------------
 * Pieces (domove, zetaperft.cl:464-552) and moved flags. */
ZHD Move make_move(int from, int to, int cpt, int pfrom, int pto, int pcpt) {
  return (Move)from | ((Move)to << 6) | ((Move)cpt << 12) | ((Move)pfrom << 18) |
         ((Move)pto << 22) | ((Move)pcpt << 26);
}
ZHD int m_from(Move m) { return m & 63; }
ZHD int m_to(Move m) { return (m >> 6) & 63; }
ZHD int m_cpt(Move m) { return (m >> 12) & 63; }
ZHD int m_pfrom(Move m) { return (m >> 18) & 15; }
ZHD int m_pto(Move m) { return (m >> 22) & 15; }
ZHD int m_pcpt(Move m) { return (m >> 26) & 15; }

ZHD void put_piece(Pos &p, int sq, int pc) {
  u64 b = bit(sq);
  p.b0 |= (pc & 1) ? b : 0ULL;
  p.p1 |= (pc & 2) ? b : 0ULL;
  p.p2 |= (pc & 4) ? b : 0ULL;
  p.p3 |= (pc & 8) ? b : 0ULL;
}

/* perft_flags: the perft kernel also flags the castle rook's square
 * (zetaperft.cl:1446-1449); the search kernel does not (zeta.cl:2330-2333). */
ZHD void play(Pos &p, Move m, bool perft_flags) {
  int f = m_from(m), t = m_to(m), c = m_cpt(m), pf = m_pfrom(m), pt = m_pto(m);
  if (m == 0 || m == ZETA_NULLMOVE) {
    /* pieces unchanged; flags still updated as the kernels do */
  } else {
    bool qc = ((pf >> 1) == KING) && (f - t == 2);
    bool kc = ((pf >> 1) == KING) && (t - f == 2);
    u64 clr = ~bit(f) & ~bit(c) & ~bit(t);
    clr &= qc ? ~bit(f - 4) : ~0ULL;
    clr &= kc ? ~bit(f + 3) : ~0ULL;
    p.b0 &= clr; p.p1 &= clr; p.p2 &= clr; p.p3 &= clr;
    put_piece(p, t, pt);
    int rook = (ROOK << 1) | (pf & 1);
    if (qc) put_piece(p, t + 1, rook);
    if (kc) put_piece(p, t - 1, rook);
  }
  u64 cr = p.cr | bit(f) | bit(t) | bit(c);
  if (perft_flags) {
    cr |= (((pf >> 1) == KING) && (f - t == 2)) ? bit(f - 4) : 0ULL;
    cr |= (((pf >> 1) == KING) && (t - f == 2)) ? bit(f + 3) : 0ULL;
  }
  int col = pf & 1;
  int rt = col ? ((t >> 3) ^ 7) : (t >> 3), rf = col ? ((f >> 3) ^ 7) : (f >> 3);
  bool dbl = ((pf >> 1) == PAWN) && (rt - rf == 2);
  cr |= ZETA_EPMASK;
  cr &= (dbl && t) ? ~bit(t) : ~0ULL;
  p.cr = cr;
}

/* ---------------- move list ----------------
 * Legal moves in the reference packing.  qs restricts to captures
 * (non-captures and castles dropped, zeta.cl:1356-1358).  Returns the
 * count; `list` needs room for 256 moves. */
ZHD Move encode(const Pos &p, int stm, int from, int to) {
  int pfrom = piece_at(p, from);
  int cpt = to;
  int pcpt = piece_at(p, to);
  bool pawn = (pfrom >> 1) == PAWN;
  int d = stm ? from - to : to - from;
  if (pawn && d != 8 && d != 16 && pcpt == PNONE) cpt = stm ? to + 8 : to - 8;
  pcpt = piece_at(p, cpt);
  int rr = stm ? ((to >> 3) ^ 7) : (to >> 3);
  int pto = (pawn && rr == 7) ? ((QUEEN << 1) | (pfrom & 1)) : pfrom;
  return make_move(from, to, cpt, pfrom, pto, pcpt);
}

/* from-square of a slider target: first piece behind it along -D */
template <int D>
ZHD int slider_from(int to, u64 occ) {
  constexpr int R = (D & 1) ? D - 1 : D + 1; /* opposite direction */
  u64 r = ray_attacks<R>(bit(to), ~occ);
  return ctz(r & occ);
}

template <int D>
ZHD int emit_slider(const Pos &p, const Sets &s, const Guard &g, u64 tgt, int stm, Move *list,
                    int n) {
  u64 t = slider_targets<D>(s, g, tgt);
  while (t) {
    int to = ctz(t);
    t &= t - 1;
    list[n++] = encode(p, stm, slider_from<D>(to, s.occ), to);
  }
  return n;
}

ZHD int emit_shift(const Pos &p, int stm, u64 t, int delta, Move *list, int n) {
  while (t) {
    int to = ctz(t);
    t &= t - 1;
    list[n++] = encode(p, stm, to - delta, to);
  }
  return n;
}

/* Single pushes and pawn captures.  encode() makes a pawn reaching the
 * last rank a queen, as the reference does; with ALLP the rook, bishop
 * and knight promotions follow it (same squares, pieces, capture). */
template <bool ALLP>
ZHD int emit_pawn(const Pos &p, int stm, u64 t, int delta, Move *list, int n) {
  if (ALLP) {
    const u64 last = stm ? ZETA_RANK1 : ZETA_RANK8;
    u64 pr = t & last;
    t &= ~last;
    while (pr) {
      const int to = ctz(pr);
      pr &= pr - 1;
      const Move q = encode(p, stm, to - delta, to);
      const Move rest = q & ~(15u << 22);
      list[n++] = q;
      list[n++] = rest | ((Move)((ROOK << 1) | stm) << 22);
      list[n++] = rest | ((Move)((BISHOP << 1) | stm) << 22);
      list[n++] = rest | ((Move)((KNIGHT << 1) | stm) << 22);
    }
  }
  return emit_shift(p, stm, t, delta, list, n);
}

/* the same with the side's piece sets and the enemy attack map already
 * computed (callers that also need the in-check test) */
template <bool ALLP = false>
ZHD int gen_legal_sd(const Pos &p, const Sets &s, u64 danger, int stm, bool qs, Move *list) {
  Guard g = make_guard(s, stm);
  u64 capmask = qs ? s.them : ~0ULL;
  u64 tgt = ~s.us & g.cmask & capmask;
  int n = 0;
  n = emit_slider<0>(p, s, g, tgt, stm, list, n);
  n = emit_slider<1>(p, s, g, tgt, stm, list, n);
  n = emit_slider<2>(p, s, g, tgt, stm, list, n);
  n = emit_slider<3>(p, s, g, tgt, stm, list, n);
  n = emit_slider<4>(p, s, g, tgt, stm, list, n);
  n = emit_slider<5>(p, s, g, tgt, stm, list, n);
  n = emit_slider<6>(p, s, g, tgt, stm, list, n);
  n = emit_slider<7>(p, s, g, tgt, stm, list, n);
  u64 empty = ~s.occ;
  u64 P = s.pawns & s.us;
  u64 free_ = ~g.pinned;
  u64 pp = P & (free_ | g.pin[0]);
  u64 pd = P & (free_ | g.pin[2]);
  u64 pa = P & (free_ | g.pin[3]);
  if (stm) {
    u64 s1 = (pp >> 8) & empty;
    u64 s2 = ((s1 & ZETA_RANK6) >> 8) & empty;
    if (!qs) {
      n = emit_pawn<ALLP>(p, stm, s1 & g.cmask, -8, list, n);
      n = emit_shift(p, stm, s2 & g.cmask, -16, list, n);
    }
    n = emit_pawn<ALLP>(p, stm, ((pa >> 7) & ZETA_NOTA) & s.them & g.cmask, -7, list, n);
    n = emit_pawn<ALLP>(p, stm, ((pd >> 9) & ZETA_NOTH) & s.them & g.cmask, -9, list, n);
  } else {
    u64 s1 = (pp << 8) & empty;
    u64 s2 = ((s1 & ZETA_RANK3) << 8) & empty;
    if (!qs) {
      n = emit_pawn<ALLP>(p, stm, s1 & g.cmask, 8, list, n);
      n = emit_shift(p, stm, s2 & g.cmask, 16, list, n);
    }
    n = emit_pawn<ALLP>(p, stm, ((pd << 9) & ZETA_NOTA) & s.them & g.cmask, 9, list, n);
    n = emit_pawn<ALLP>(p, stm, ((pa << 7) & ZETA_NOTH) & s.them & g.cmask, 7, list, n);
  }
  u64 N = s.knights & s.us & free_;
  n = emit_shift(p, stm, ((N << 17) & ZETA_NOTA) & tgt, 17, list, n);
  n = emit_shift(p, stm, ((N << 15) & ZETA_NOTH) & tgt, 15, list, n);
  n = emit_shift(p, stm, ((N << 10) & ZETA_NOTAB) & tgt, 10, list, n);
  n = emit_shift(p, stm, ((N << 6) & ZETA_NOTGH) & tgt, 6, list, n);
  n = emit_shift(p, stm, ((N >> 17) & ZETA_NOTH) & tgt, -17, list, n);
  n = emit_shift(p, stm, ((N >> 15) & ZETA_NOTA) & tgt, -15, list, n);
  n = emit_shift(p, stm, ((N >> 10) & ZETA_NOTGH) & tgt, -10, list, n);
  n = emit_shift(p, stm, ((N >> 6) & ZETA_NOTAB) & tgt, -6, list, n);
  {
    u64 t = king_attacks(s.kbb) & ~s.us & ~danger & capmask;
    while (t) {
      int to = ctz(t);
      t &= t - 1;
      list[n++] = encode(p, stm, s.ksq, to);
    }
  }
  if (!qs) {
    int c = castles(p, s, stm, danger);
    if (c & 1) list[n++] = encode(p, stm, s.ksq, (s.ksq - 2) & 63);
    if (c & 2) list[n++] = encode(p, stm, s.ksq, (s.ksq + 2) & 63);
  }
  int sqep;
  int e = ep_legal(p, s, stm, sqep);
  if (e) {
    int to = stm ? sqep - 8 : sqep + 8;
    int pawn = (PAWN << 1) | stm;
    int victim = piece_at(p, sqep);
    if (e & 1) list[n++] = make_move(sqep - 1, to, sqep, pawn, pawn, victim);
    if (e & 2) list[n++] = make_move(sqep + 1, to, sqep, pawn, pawn, victim);
  }
  return n;
}

template <bool ALLP = false>
ZHD int gen_legal(const Pos &p, int stm, bool qs, Move *list) {
  const Sets s = make_sets(p, stm);
  return gen_legal_sd<ALLP>(p, s, enemy_attacks(s, stm), stm, qs, list);
}

}  // namespace zeta
