/*
 * board.h -- host-side board layer of the zeta host: FEN, move text,
 * Zobrist hash and playing a move on the quad-bitboard.
 *
 * Same board and move formats as the reference host (src/types.h:59-74)
 * and the same semantics as its src/io.c / src/bitboard.c functions, so a
 * board set here is the input the device path expects.
 */
#ifndef ZETA_HOST_BOARD_H
#define ZETA_HOST_BOARD_H

#include <stdbool.h>
#include <stdint.h>

typedef uint64_t Bitboard;
typedef uint32_t Move;

enum { QBBBLACK = 0, QBBP1 = 1, QBBP2 = 2, QBBP3 = 3, QBBPMVD = 4, QBBHASH = 5, QBBHMC = 6 };
enum { PNONE = 0, PAWN = 1, KNIGHT = 2, KING = 3, BISHOP = 4, ROOK = 5, QUEEN = 6 };
#define WHITE 0
#define BLACK 1
#define MAXPLY 64
#define MAXGAMEPLY 1024
#define INF 32000
#define MATESCORE 30000
#define ESTEBF 3 /* estimated effective branching factor (src/types.h:81) */
#define MOVENONE 0u
#define NULLMOVE 0x41u

#define GETSQFROM(m) ((int)((m)&0x3F))
#define GETSQTO(m) ((int)(((m) >> 6) & 0x3F))
#define GETSQCPT(m) ((int)(((m) >> 12) & 0x3F))
#define GETPFROM(m) ((int)(((m) >> 18) & 0xF))
#define GETPTO(m) ((int)(((m) >> 22) & 0xF))
#define GETPCPT(m) ((int)(((m) >> 26) & 0xF))
#define JUSTMOVE(m) ((m)&0x3FFFFFFFu)

/* setboard, src/io.c:335-531: returns false on an illegal position (not
 * exactly one king per side).  *stm gets the side to move, *fullmove the
 * FEN move number. */
bool board_setfen(Bitboard board[7], int *stm, int *fullmove, const char *fen);

/* createfen, src/io.c:227-333 */
void board_getfen(const Bitboard board[7], int stm, int fullmove, char *out, int outlen);

/* computehash, src/bitboard.c:461-510 */
Bitboard board_hash(const Bitboard board[7], int stm);

/* piece code at a square (type<<1 | colour) */
int board_piece(const Bitboard board[7], int sq);

/* play a move for the game (pieces, moved flags, hash, half-move clock),
 * as the search kernel's moveup does (zeta.cl:2269-2373) */
void board_play(Bitboard board[7], int stm, Move move);

/* move text, src/io.c:70-160 */
void move2can(Move move, char out[6]);
Move can2move(const char *can, const Bitboard board[7], int stm);
/* true when `can` is coordinate move text: from and to squares (a-h,
 * 1-8) and an optional promotion letter (q, r, b, n), nothing else */
bool move_text_ok(const char *can);

/* printboard, src/io.c:165-225 */
void board_print(const Bitboard board[7], int stm);

#endif
