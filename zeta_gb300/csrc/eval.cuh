/*
 * eval.cuh -- static evaluation of the reference (zeta.cl:1479-1544):
 * per piece +10, material, piece-square and square-control tables (black's
 * view; a white piece on sq reads sq^56), pawn structure (blocked -15,
 * diagonal support +10 each, -30 per own pawn further back on the file),
 * bishop pair +-25.  The reference sums one work-item per square; here the
 * piece terms are a loop over the occupied squares and the pawn terms are
 * set-wise shifts and popcounts.  Result in centipawns from white's view.
 *
 * The tables are the reference's values (they define the score); device
 * code keeps a copy in shared memory (EvalTables) so that lanes reading
 * different entries do not serialise on the constant cache.
 */
#pragma once

#include "chess.cuh"

namespace zeta {

struct EvalTables {
  int16_t pst[7][64];   /* piece-square, black's view */
  int16_t control[64];  /* square control, black's view */
  int16_t value[8];     /* pnone pawn knight king bishop rook queen */
};

#define ZETA_EVAL_VALUES {0, 100, 400, 0, 400, 600, 1200, 0}
#define ZETA_EVAL_CONTROL                                                                              \
  {0, 0, 5, 5, 5, 5, 0, 0, 5, 0, 5, 5, 5, 5, 0, 5, 0, 0, 10, 5, 5, 10, 0, 0, 0, 5, 5, 10, 10, 5, 5, 0, \
   0, 5, 5, 10, 10, 5, 5, 0, 0, 0, 10, 5, 5, 10, 0, 0, 0, 0, 5, 5, 5, 5, 0, 0, 0, 0, 5, 5, 5, 5, 0, 0}
#define ZETA_EVAL_PST                                                                                      \
  {{0},                                                                                                    \
   {0, 0, 0, 0, 0, 0, 0, 0, 50, 50, 50, 50, 50, 50, 50, 50, 30, 30, 30, 30, 30, 30, 30, 30, 5, 5, 5, 10,   \
    10, 5, 5, 5, 3, 3, 3, 8, 8, 3, 3, 3, 2, 2, 2, 2, 2, 2, 2, 2, 0, 0, 0, -5, -5, 0, 0, 0, 0, 0, 0, 0, 0,  \
    0, 0, 0},                                                                                              \
   {-50, -40, -30, -30, -30, -30, -40, -50, -40, -20, 0, 0, 0, 0, -20, -40, -30, 0, 10, 15, 15, 10, 0,     \
    -30, -30, 5, 15, 20, 20, 15, 5, -30, -30, 0, 15, 20, 20, 15, 0, -30, -30, 5, 10, 15, 15, 10, 5, -30,   \
    -40, -20, 0, 5, 5, 0, -20, -40, -50, -40, -30, -30, -30, -30, -40, -50},                               \
   {-1, -1, -1, -1, -1, -1, -1, -1, -1, 0, 0, 0, 0, 0, 0, -1, -1, 0, 0, 0, 0, 0, 0, -1, -1, 0, 0, 0, 0,   \
    0, 0, -1, -1, 0, 0, 0, 0, 0, 0, -1, -1, 0, 0, 0, 0, 0, 0, -1, -1, 0, 0, 0, 0, 0, 0, -1, -1, -1, -1,   \
    -1, -1, -1, -1, -1},                                                                                   \
   {-20, -10, -10, -10, -10, -10, -10, -20, -10, 0, 0, 0, 0, 0, 0, -10, -10, 0, 5, 10, 10, 5, 0, -10,     \
    -10, 5, 5, 10, 10, 5, 5, -10, -10, 0, 10, 10, 10, 10, 0, -10, -10, 10, 10, 10, 10, 10, 10, -10, -10,   \
    5, 0, 0, 0, 0, 5, -10, -20, -10, -10, -10, -10, -10, -10, -20},                                        \
   {0, 0, 0, 0, 0, 0, 0, 0, 5, 10, 10, 10, 10, 10, 10, 5, -5, 0, 0, 0, 0, 0, 0, -5, -5, 0, 0, 0, 0, 0,    \
    0, -5, -5, 0, 0, 0, 0, 0, 0, -5, -5, 0, 0, 0, 0, 0, 0, -5, -5, 0, 0, 0, 0, 0, 0, -5, 0, 0, 0, 5, 5, 0,  \
    0, 0},                                                                                                 \
   {-20, -10, -10, -5, -5, -10, -10, -20, -10, 0, 0, 0, 0, 0, 0, -10, -10, 0, 5, 5, 5, 5, 0, -10, -5, 0,  \
    5, 5, 5, 5, 0, -5, -5, 0, 5, 5, 5, 5, 0, -5, -10, 0, 5, 5, 5, 5, 0, -10, -10, 0, 0, 0, 0, 0, 0, -10,   \
    -20, -10, -10, -5, -5, -10, -10, -20}}

static const EvalTables kEvalHost = {ZETA_EVAL_PST, ZETA_EVAL_CONTROL, ZETA_EVAL_VALUES};
#if defined(__CUDACC__)
static __constant__ EvalTables kEvalDev = {ZETA_EVAL_PST, ZETA_EVAL_CONTROL, ZETA_EVAL_VALUES};
#endif

/* sum over the pieces of one side of +10, material, PST and control */
ZHD int eval_pieces(const Pos &p, u64 side, bool black, const EvalTables &T) {
  int s = 0;
  u64 w = side;
  while (w) {
    int sq = ctz(w);
    w &= w - 1;
    int t = piece_at(p, sq) >> 1;
    int v = black ? sq : (sq ^ 56);
    s += 10 + T.value[t] + T.pst[t][v] + T.control[v];
  }
  return s;
}

/* pawn structure of one side, own pawns `x`, opponent pieces `opp` */
ZHD int eval_pawns_white(u64 x, u64 opp) {
  int s = -15 * popc(x & (opp >> 8));
  s += 10 * (popc(x & ZETA_NOTH & (x << 7)) + popc(x & ZETA_NOTA & (x << 9)));
  u64 low = x & ~0xFFULL; /* the file loop stops at rank 2 (sq > 7) */
  int back = 0;
#pragma unroll
  for (int k = 1; k < 7; k++) back += popc(x & (low << (8 * k)));
  return s - 30 * back;
}
ZHD int eval_pawns_black(u64 x, u64 opp) {
  int s = -15 * popc(x & (opp << 8));
  s += 10 * (popc(x & ZETA_NOTA & (x >> 7)) + popc(x & ZETA_NOTH & (x >> 9)));
  u64 high = x & ~0xFF00000000000000ULL; /* the file loop stops at rank 7 (sq < 56) */
  int back = 0;
#pragma unroll
  for (int k = 1; k < 7; k++) back += popc(x & (high >> (8 * k)));
  return s - 30 * back;
}

/* white's view, as the reference's evalscore before the stm negation */
ZHD int eval_white(const Pos &p, const EvalTables &T) {
  u64 occ = p.p1 | p.p2 | p.p3;
  u64 black = p.b0, white = occ ^ p.b0;
  u64 pawns = p.p1 & ~p.p2 & ~p.p3;
  int s = eval_pieces(p, white, false, T) - eval_pieces(p, black, true, T);
  s += eval_pawns_white(pawns & white, black) - eval_pawns_black(pawns & black, white);
  u64 bishops = p.p3 & ~p.p1 & ~p.p2;
  if (popc(black & bishops) == 2) s -= 25;
  if (popc(white & bishops) == 2) s += 25;
  return s;
}

/* ---------------- incremental form ----------------
 * eval_white is the piece terms (a sum over pieces) plus the pawn-structure
 * and bishop-pair terms.  The piece terms of a child therefore equal its
 * parent's plus the change the move makes -- the mover leaves its square,
 * the moved (or promoted) piece arrives, a captured piece and a castling
 * rook's old square drop out, the rook's new square comes in -- so a leaf
 * is scored without the loop over its pieces.  Exact: every term is an
 * integer and the sum does not depend on its order. */

/* one piece's term in eval_pieces, signed from white's view */
ZHD int piece_term(int pc, int sq, const EvalTables &T) {
  const int t = pc >> 1;
  const bool black = pc & 1;
  const int v = black ? sq : (sq ^ 56);
  const int s = 10 + T.value[t] + T.pst[t][v] + T.control[v];
  return black ? -s : s;
}

/* the piece terms of eval_white */
ZHD int eval_piece_sum(const Pos &p, const EvalTables &T) {
  const u64 occ = p.p1 | p.p2 | p.p3;
  return eval_pieces(p, occ ^ p.b0, false, T) - eval_pieces(p, p.b0, true, T);
}

/* the rest of eval_white: pawn structure and bishop pair */
ZHD int eval_structure(const Pos &p) {
  const u64 occ = p.p1 | p.p2 | p.p3;
  const u64 black = p.b0, white = occ ^ p.b0;
  const u64 pawns = p.p1 & ~p.p2 & ~p.p3;
  int s = eval_pawns_white(pawns & white, black) - eval_pawns_black(pawns & black, white);
  const u64 bishops = p.p3 & ~p.p1 & ~p.p2;
  if (popc(black & bishops) == 2) s -= 25;
  if (popc(white & bishops) == 2) s += 25;
  return s;
}

/* eval_piece_sum(child) - eval_piece_sum(parent) for a real move m (not the
 * null move), as play() moves the pieces */
ZHD int piece_sum_delta(Move m, const EvalTables &T) {
  const int f = m_from(m), t = m_to(m), c = m_cpt(m), pf = m_pfrom(m), pt = m_pto(m), pc = m_pcpt(m);
  int d = piece_term(pt, t, T) - piece_term(pf, f, T);
  if (pc >> 1) d -= piece_term(pc, c, T);
  if ((pf >> 1) == KING && f - t == 2) {
    const int rook = (ROOK << 1) | (pf & 1);
    d += piece_term(rook, t + 1, T) - piece_term(rook, f - 4, T);
  }
  if ((pf >> 1) == KING && t - f == 2) {
    const int rook = (ROOK << 1) | (pf & 1);
    d += piece_term(rook, t - 1, T) - piece_term(rook, f + 3, T);
  }
  return d;
}

}  // namespace zeta
