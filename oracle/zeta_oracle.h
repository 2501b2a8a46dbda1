/*
 * zeta_oracle.h -- CPU oracle for the Zeta device path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of what the
 * reference OpenCL kernels compute (src/zetaperft.cl, src/zeta.cl) and of
 * the host board code that feeds them (src/io.c, src/bitboard.c).  It is
 * the checker for the CUDA kernels: only tests/, __graft_entry__.smoke()
 * and the cpu_baseline leg of bench.py may load it.  The product path
 * (libzeta_cuda.so, the zeta host binary) never links it.
 *
 * Parity pins: the 14 perft known-answer tests of src/test.c:43-73 and the
 * reference kernels themselves compiled under oracle/refshim (fixtures in
 * tests/golden/ made by tests/golden/make_golden.py).
 *
 * Board layout is the reference quad-bitboard (src/types.h:59-66):
 *   b[0] black pieces, b[1..3] piece-type bit planes (piece = type<<1|color),
 *   b[4] "piece moved" flags (castle rights, en-passant target),
 *   b[5] Zobrist hash, b[6] half-move clock.
 * Moves are the reference 32-bit packing (src/types.h:67-74,130-141).
 */
#ifndef ZETA_ORACLE_H
#define ZETA_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef uint64_t zo_u64;
typedef uint32_t zo_move;

#define ZO_MAXMOVES 256
#define ZO_INF 32000
#define ZO_MATESCORE 30000

/* FEN -> board; returns 1 on success, 0 on an invalid position.
 * Follows setboard() in src/io.c:335-531, including its handling of the
 * en-passant field (the FEN target square lies outside the engine's
 * rank 4/5 flag mask, so a FEN en-passant square never enables a capture). */
int zo_setboard(zo_u64 board[7], int *stm, const char *fen);

/* Zobrist hash of a board, src/bitboard.c:461-510 and zetaperft.cl:586-631. */
zo_u64 zo_computehash(const zo_u64 board[7], int stm);

/* Legal moves of the side to move, in the reference packing.
 * qs != 0 restricts to captures (zetaperft.cl:1297, zeta.cl:1356).
 * Order: lane (from-square) ascending, then to-square ascending. */
int zo_genmoves(const zo_u64 board[7], int stm, int qs, zo_move *moves);

/* The same with all_promotions != 0: each queen promotion is followed by
 * the same move promoting to a rook, a bishop and a knight.  The reference
 * generates queen promotions only; this rule has no reference output to
 * pin, so the tests pin it against an independent mailbox generator. */
int zo_genmoves_ex(const zo_u64 board[7], int stm, int qs, int all_promotions, zo_move *moves);

/* Number of legal moves and the reference's in-check flag. */
int zo_movecount(const zo_u64 board[7], int stm, int *in_check);

/* Play a move: quad bitboards + moved flags (+hash and hmc when
 * with_hash).  perft_flags selects the perft kernel's flag update
 * (zetaperft.cl:1440-1466, castle rook squares flagged) instead of the
 * search kernel's (zeta.cl:2330-2350). */
void zo_play(zo_u64 board[7], int stm, zo_move move, int perft_flags);

/* Leaf count of the legal tree (queen-only promotions), zetaperft.cl:801-1477. */
zo_u64 zo_perft(const zo_u64 board[7], int stm, int depth);
/* The same with all four promotions when all_promotions != 0. */
zo_u64 zo_perft_ex(const zo_u64 board[7], int stm, int depth, int all_promotions);

/* Static evaluation, white's view, zeta.cl:1479-1544 (x64 lanes + bishop pair). */
int zo_eval_white(const zo_u64 board[7]);

/* Plain fixed-depth negamax: legal moves, side-to-move relative eval at the
 * leaves, mate = -INF+ply, stalemate = 0, no quiescence, no extensions, no
 * pruning, no draw rules.  Root score; *bestmove gets the first move (in
 * zo_genmoves order) that reaches it.  nodes counts visited nodes. */
int zo_negamax(const zo_u64 board[7], int stm, int depth, zo_move *bestmove, zo_u64 *nodes);

/* Same value computed by full-window alpha-beta (no TT); equals zo_negamax. */
int zo_alphabeta(const zo_u64 board[7], int stm, int depth, zo_move *bestmove, zo_u64 *nodes);

/* The same alpha-beta value with moves reordered (iterative deepening
 * 1..depth, previous best move first, MVV-LVA captures, killers): only the
 * visited-node count differs.  *bestmove reaches the score. */
int zo_alphabeta_ordered(const zo_u64 board[7], int stm, int depth, zo_move *bestmove, zo_u64 *nodes);

/* Seeded random legal playout (splitmix64): plays `plies` moves from the
 * initial position, uniform over zo_genmoves order; returns 0 if the game
 * ended (no legal move) before that. */
int zo_playout(zo_u64 seed, int plies, zo_u64 board[7], int *stm);

/* Position i of a seeded synthetic batch (the benchmark workloads):
 *   s = seed ^ (0xD1B54A32D192ED03 * (i + 1)), splitmix64 steps;
 *   up to 64 attempts of: plies = min_plies + next % (max-min+1), play
 *   moves[next % n] from the (from,to)-ordered legal list; accept when
 *   the side to move has a legal move and >= min_pieces pieces remain;
 *   depth = min_depth + next % (max_depth-min_depth+1).
 * Returns 0 when all attempts fail.  Hash = zo_computehash. */
int zo_make_position(zo_u64 seed, int i, int min_plies, int max_plies, int min_pieces, int min_depth,
                     int max_depth, zo_u64 board[7], int *stm, int *depth);

/* splitmix64 step */
zo_u64 zo_splitmix64(zo_u64 *state);

/* Move <-> coordinate text (src/io.c:70-160). */
void zo_move2can(zo_move move, char out[6]);
zo_move zo_can2move(const char *can, const zo_u64 board[7], int stm);

/* Tables the oracle derives from chess geometry; exported so a test can
 * compare them with the reference's literal tables. */
const zo_u64 *zo_attack_tables(void);      /* [7*64], zetaperft.cl:650-670 */
const zo_u64 *zo_pawn_push_tables(void);   /* [2*64], zetaperft.cl:643-649 */
const zo_u64 *zo_inbetween_table(void);    /* [64*64], src/bitboard.c:52  */
const zo_u64 *zo_line_table(void);         /* [64*64], src/bitboard.c:119 */

#ifdef __cplusplus
}
#endif
#endif
