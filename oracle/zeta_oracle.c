/*
 * zeta_oracle.c -- CPU oracle (test infrastructure only, see zeta_oracle.h).
 *
 * The move generator below restates the reference's "64 work-items, one
 * per square" generator as a loop over the 64 lanes followed by the same
 * reductions and per-lane legality filters, in the order the kernel runs
 * them (zetaperft.cl:911-1311; the search kernel zeta.cl:1023-1454 is the
 * same generator plus extension/LMR bookkeeping that does not change the
 * move set).  Shift counts are reduced mod 64 as OpenCL does.
 */
#include "zeta_oracle.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef zo_u64 u64;
typedef zo_move Move;

enum { BLACKBB = 0, P1 = 1, P2 = 2, P3 = 3, PMVD = 4, HASH = 5, HMC = 6 };
enum { PNONE = 0, PAWN = 1, KNIGHT = 2, KING = 3, BISHOP = 4, ROOK = 5, QUEEN = 6 };

#define NOTA 0xFEFEFEFEFEFEFEFEULL
#define NOTH 0x7F7F7F7F7F7F7F7FULL
#define EPMASK 0x000000FFFF000000ULL
/* castle-right flag masks, src/types.h:113-124 (SMCRALL keeps the
 * reference's 0x89 top byte, which includes d8 instead of e8) */
#define CR_ALL 0x8900000000000091ULL
#define CR_WQ 0x0000000000000011ULL
#define CR_WK 0x0000000000000090ULL
#define CR_BQ 0x1100000000000000ULL
#define CR_BK 0x9000000000000000ULL
#define NULLMOVE 0x41u

/* OpenCL shift semantics: count taken mod 64 */
static inline u64 bit(int sq) { return 1ULL << (sq & 63); }
static inline u64 shl(u64 x, int s) { return x << (s & 63); }
static inline u64 shr(u64 x, int s) { return x >> (s & 63); }
static inline int popc(u64 x) { return __builtin_popcountll(x); }
static inline int lsb(u64 x) { return __builtin_ctzll(x); }

#define SQFROM(m) ((int)((m) & 0x3F))
#define SQTO(m) ((int)(((m) >> 6) & 0x3F))
#define SQCPT(m) ((int)(((m) >> 12) & 0x3F))
#define PFROM(m) ((int)(((m) >> 18) & 0xF))
#define PTO(m) ((int)(((m) >> 22) & 0xF))
#define PCPT(m) ((int)(((m) >> 26) & 0xF))
#define PTYPE(p) (((p) >> 1) & 7)
#define MKMOVE(f, t, c, pf, pt, pc)                                            \
  ((Move)(f) | ((Move)(t) << 6) | ((Move)(c) << 12) | ((Move)(pf) << 18) |     \
   ((Move)(pt) << 22) | ((Move)(pc) << 26))
#define RRANK(sq, c) ((c) ? (((sq) >> 3) ^ 7) : ((sq) >> 3))

/* ------------------------------------------------------------------ */
/* Geometry tables, derived here (the reference ships them as literals:
 * zetaperft.cl:643-670, src/bitboard.c:52,119).  A test compares them. */
static u64 T_attack[7 * 64];  /* 0 white pawn, 1 black pawn, 2 N, 3 K, 4 B, 5 R, 6 Q */
static u64 T_push[2 * 64];
static u64 T_between[64 * 64];
static u64 T_line[64 * 64];
static int tables_ready = 0;

static int onboard(int f, int r) { return f >= 0 && f < 8 && r >= 0 && r < 8; }

static void init_tables(void) {
  if (tables_ready) return;
  static const int kn[8][2] = {{1, 2}, {2, 1}, {2, -1}, {1, -2}, {-1, -2}, {-2, -1}, {-2, 1}, {-1, 2}};
  static const int dirs[8][2] = {{1, 0}, {-1, 0}, {0, 1}, {0, -1}, {1, 1}, {1, -1}, {-1, 1}, {-1, -1}};
  for (int sq = 0; sq < 64; sq++) {
    int f = sq & 7, r = sq >> 3;
    u64 wp = 0, bp = 0, n = 0, k = 0, b = 0, rk = 0;
    if (onboard(f - 1, r + 1)) wp |= bit((r + 1) * 8 + f - 1);
    if (onboard(f + 1, r + 1)) wp |= bit((r + 1) * 8 + f + 1);
    if (onboard(f - 1, r - 1)) bp |= bit((r - 1) * 8 + f - 1);
    if (onboard(f + 1, r - 1)) bp |= bit((r - 1) * 8 + f + 1);
    for (int i = 0; i < 8; i++) {
      if (onboard(f + kn[i][0], r + kn[i][1])) n |= bit((r + kn[i][1]) * 8 + f + kn[i][0]);
      if (onboard(f + dirs[i][0], r + dirs[i][1])) k |= bit((r + dirs[i][1]) * 8 + f + dirs[i][0]);
      u64 ray = 0;
      for (int s = 1; onboard(f + s * dirs[i][0], r + s * dirs[i][1]); s++)
        ray |= bit((r + s * dirs[i][1]) * 8 + f + s * dirs[i][0]);
      if (i < 4) rk |= ray; else b |= ray;
    }
    /* the reference tables leave pawn attacks empty on the last rank */
    T_attack[0 * 64 + sq] = (r == 7) ? 0 : wp;
    T_attack[1 * 64 + sq] = (r == 0) ? 0 : bp;
    T_attack[2 * 64 + sq] = n;
    T_attack[3 * 64 + sq] = k;
    T_attack[4 * 64 + sq] = b;
    T_attack[5 * 64 + sq] = rk;
    T_attack[6 * 64 + sq] = b | rk;
    /* pawn pushes: single step, double step from the start rank */
    T_push[sq] = (r < 7) ? bit(sq + 8) : 0;
    if (r == 1) T_push[sq] |= bit(sq + 16);
    T_push[64 + sq] = (r > 0) ? bit(sq - 8) : 0;
    if (r == 6) T_push[64 + sq] |= bit(sq - 16);
  }
  for (int a = 0; a < 64; a++)
    for (int bsq = 0; bsq < 64; bsq++) {
      int fa = a & 7, ra = a >> 3, fb = bsq & 7, rb = bsq >> 3;
      u64 btw = 0, line = 0;
      int df = (fb > fa) - (fb < fa), dr = (rb > ra) - (rb < ra);
      int aligned = a != bsq && (fa == fb || ra == rb || abs(fa - fb) == abs(ra - rb));
      if (aligned) {
        for (int f = fa + df, r = ra + dr; f != fb || r != rb; f += df, r += dr) btw |= bit(r * 8 + f);
        for (int s = -1; s <= 1; s += 2)
          for (int f = fa, r = ra; onboard(f, r); f += s * df, r += s * dr) line |= bit(r * 8 + f);
      }
      T_between[a * 64 + bsq] = btw;
      T_line[a * 64 + bsq] = line;
    }
  tables_ready = 1;
}

const zo_u64 *zo_attack_tables(void) { init_tables(); return T_attack; }
const zo_u64 *zo_pawn_push_tables(void) { init_tables(); return T_push; }
const zo_u64 *zo_inbetween_table(void) { init_tables(); return T_between; }
const zo_u64 *zo_line_table(void) { init_tables(); return T_line; }

/* ------------------------------------------------------------------ */
/* Zobrist keys and evaluation tables: the reference's constants, which
 * bit-exact hashing and scoring require (zeta.cl:258-359). */
static const u64 ZOBRIST[18] = {
    0x9D39247E33776D41ULL, 0x2AF7398005AAA5C7ULL, 0x44DB015024623547ULL,
    0x9C15F73E62A76AE2ULL, 0x75834465489C0C89ULL, 0x3290AC3A203001BFULL,
    0x0FBBAD1F61042279ULL, 0xE83A908FF2FB60CAULL, 0x0D7E765D58755C10ULL,
    0x1A083822CEAFE02DULL, 0x9605D5F0E25EC3B0ULL, 0xD021FF5CD13A2ED5ULL,
    0x40BDF15D4A672E32ULL, 0x011355146FD56395ULL, 0x5DB4832046F3D9E5ULL,
    0x239F8B2D7FF719CCULL, 0x05D1A1AE85B49AA1ULL, 0x679F848F6E8FC971ULL};

static const int VALUE[7] = {0, 100, 400, 0, 400, 600, 1200};

/* indexed black's view; a white piece on sq reads index sq^56 */
static const int CONTROL[64] = {
    0, 0, 5, 5, 5, 5, 0, 0,  5, 0, 5, 5, 5, 5, 0, 5,  0, 0, 10, 5, 5, 10, 0, 0,
    0, 5, 5, 10, 10, 5, 5, 0, 0, 5, 5, 10, 10, 5, 5, 0, 0, 0, 10, 5, 5, 10, 0, 0,
    0, 0, 5, 5, 5, 5, 0, 0,  0, 0, 5, 5, 5, 5, 0, 0};

static const int PST[7][64] = {
    {0},
    {0, 0, 0, 0, 0, 0, 0, 0,    50, 50, 50, 50, 50, 50, 50, 50,
     30, 30, 30, 30, 30, 30, 30, 30, 5, 5, 5, 10, 10, 5, 5, 5,
     3, 3, 3, 8, 8, 3, 3, 3,    2, 2, 2, 2, 2, 2, 2, 2,
     0, 0, 0, -5, -5, 0, 0, 0,  0, 0, 0, 0, 0, 0, 0, 0},
    {-50, -40, -30, -30, -30, -30, -40, -50, -40, -20, 0, 0, 0, 0, -20, -40,
     -30, 0, 10, 15, 15, 10, 0, -30,      -30, 5, 15, 20, 20, 15, 5, -30,
     -30, 0, 15, 20, 20, 15, 0, -30,      -30, 5, 10, 15, 15, 10, 5, -30,
     -40, -20, 0, 5, 5, 0, -20, -40,      -50, -40, -30, -30, -30, -30, -40, -50},
    {-1, -1, -1, -1, -1, -1, -1, -1, -1, 0, 0, 0, 0, 0, 0, -1,
     -1, 0, 0, 0, 0, 0, 0, -1,      -1, 0, 0, 0, 0, 0, 0, -1,
     -1, 0, 0, 0, 0, 0, 0, -1,      -1, 0, 0, 0, 0, 0, 0, -1,
     -1, 0, 0, 0, 0, 0, 0, -1,      -1, -1, -1, -1, -1, -1, -1, -1},
    {-20, -10, -10, -10, -10, -10, -10, -20, -10, 0, 0, 0, 0, 0, 0, -10,
     -10, 0, 5, 10, 10, 5, 0, -10,   -10, 5, 5, 10, 10, 5, 5, -10,
     -10, 0, 10, 10, 10, 10, 0, -10, -10, 10, 10, 10, 10, 10, 10, -10,
     -10, 5, 0, 0, 0, 0, 5, -10,     -20, -10, -10, -10, -10, -10, -10, -20},
    {0, 0, 0, 0, 0, 0, 0, 0,       5, 10, 10, 10, 10, 10, 10, 5,
     -5, 0, 0, 0, 0, 0, 0, -5,     -5, 0, 0, 0, 0, 0, 0, -5,
     -5, 0, 0, 0, 0, 0, 0, -5,     -5, 0, 0, 0, 0, 0, 0, -5,
     -5, 0, 0, 0, 0, 0, 0, -5,     0, 0, 0, 5, 5, 0, 0, 0},
    {-20, -10, -10, -5, -5, -10, -10, -20, -10, 0, 0, 0, 0, 0, 0, -10,
     -10, 0, 5, 5, 5, 5, 0, -10,    -5, 0, 5, 5, 5, 5, 0, -5,
     -5, 0, 5, 5, 5, 5, 0, -5,      -10, 0, 5, 5, 5, 5, 0, -10,
     -10, 0, 0, 0, 0, 0, 0, -10,    -20, -10, -10, -5, -5, -10, -10, -20}};

/* ------------------------------------------------------------------ */
static inline int piece_at(const u64 *b, int sq) {
  return (int)((shr(b[BLACKBB], sq) & 1) | ((shr(b[P1], sq) & 1) << 1) |
               ((shr(b[P2], sq) & 1) << 2) | ((shr(b[P3], sq) & 1) << 3));
}
static inline u64 occupancy(const u64 *b) { return b[P1] | b[P2] | b[P3]; }
static inline u64 side_bb(const u64 *b, int side) {
  return side ? b[BLACKBB] : (b[BLACKBB] ^ occupancy(b));
}
static inline u64 rooks_queens(const u64 *b) { return (b[P1] & ~b[P2] & b[P3]) | (~b[P1] & b[P2] & b[P3]); }
static inline u64 bishops_queens(const u64 *b) { return (~b[P1] & ~b[P2] & b[P3]) | (~b[P1] & b[P2] & b[P3]); }

/* One Dumb7Fill ray, as the reference writes it per direction: six
 * propagation steps through `pro`, then one more shift masked by `wrap`. */
static u64 d7ray(u64 start, u64 pro, int s, u64 wrap) {
  pro &= wrap;
  u64 gen = start, acc = start;
  for (int i = 0; i < 6; i++) {
    gen = (s > 0 ? shl(gen, s) : shr(gen, -s)) & pro;
    acc |= gen;
  }
  return (s > 0 ? shl(acc, s) : shr(acc, -s)) & wrap;
}
static u64 rays_ortho(u64 start, u64 pro) {
  return d7ray(start, pro, 1, NOTA) | d7ray(start, pro, 8, ~0ULL) | d7ray(start, pro, -1, NOTH) |
         d7ray(start, pro, -8, ~0ULL);
}
static u64 rays_diag(u64 start, u64 pro) {
  return d7ray(start, pro, 9, NOTA) | d7ray(start, pro, 7, NOTH) | d7ray(start, pro, -9, NOTH) |
         d7ray(start, pro, -7, NOTA);
}

/* squareunderattack(), zetaperft.cl:681-797: is sq attacked by side `by` */
static int square_attacked(const u64 *b, int by, int sq) {
  init_tables();
  u64 occ = occupancy(b), me = side_bb(b, by);
  if (rays_ortho(bit(sq), ~occ) & me & rooks_queens(b)) return 1;
  if (rays_diag(bit(sq), ~occ) & me & bishops_queens(b)) return 1;
  if (T_attack[128 + sq] & me & (~b[P1] & b[P2] & ~b[P3])) return 1;
  if (T_attack[(!by) * 64 + sq] & me & (b[P1] & ~b[P2] & ~b[P3])) return 1;
  if (T_attack[192 + sq] & me & (b[P1] & b[P2] & ~b[P3])) return 1;
  return 0;
}
static int king_square(const u64 *b, int side) {
  u64 k = side_bb(b, side) & b[P1] & b[P2] & ~b[P3];
  return k ? lsb(k) : 0;
}

/* domovequick/undomovequick, zetaperft.cl:391-462 (no castle rook) */
static void quick_play(u64 *b, Move m) {
  int f = SQFROM(m), t = SQTO(m), c = SQCPT(m), pt = PTO(m);
  u64 clr = ~bit(f) & ~bit(c) & ~bit(t);
  for (int i = 0; i < 4; i++) b[i] &= clr;
  for (int i = 0; i < 4; i++) b[i] |= (u64)((pt >> i) & 1) << t;
}

/* domove, zetaperft.cl:464-552: pieces only, castle rook included */
static void do_pieces(u64 *b, Move m) {
  if (m == 0 || m == NULLMOVE) return;
  int f = SQFROM(m), t = SQTO(m), c = SQCPT(m), pf = PFROM(m), pt = PTO(m);
  u64 clr = ~bit(f) & ~bit(c) & ~bit(t);
  int qcastle = PTYPE(pf) == KING && f - t == 2;
  int kcastle = PTYPE(pf) == KING && t - f == 2;
  if (qcastle) clr &= ~bit(f - 4);
  if (kcastle) clr &= ~bit(f + 3);
  for (int i = 0; i < 4; i++) b[i] &= clr;
  for (int i = 0; i < 4; i++) b[i] |= (u64)((pt >> i) & 1) << t;
  int rook = (ROOK << 1) | (pf & 1);
  if (qcastle)
    for (int i = 0; i < 4; i++) b[i] |= (u64)((rook >> i) & 1) << (t + 1);
  if (kcastle)
    for (int i = 0; i < 4; i++) b[i] |= (u64)((rook >> i) & 1) << (t - 1);
}

/* ------------------------------------------------------------------ */
/* The 64-lane generator.  lanes[lid] = legal to-squares of the piece on
 * lid.  Returns the move count; *kic gets the in-check flag. */
static int gen_lanes(const u64 *bin, int stm, int qs, u64 cr, u64 lanes[64], int *kic) {
  init_tables();
  u64 b[4] = {bin[0], bin[1], bin[2], bin[3]};
  u64 blockers = occupancy(b);
  u64 me = stm ? b[BLACKBB] : (b[BLACKBB] ^ blockers);
  u64 opp = (!stm) ? b[BLACKBB] : (b[BLACKBB] ^ blockers);
  int sqking = lsb(me & b[P1] & b[P2] & ~b[P3]);  /* zetaperft.cl:928-931 */

  /* superking rays on an empty board find pinners; a lone blocker between
   * pinner and king is pinned (zetaperft.cl:933-1061) */
  u64 pinned = 0;
  u64 work = rays_ortho(bit(sqking), ~0ULL) & opp & rooks_queens(b);
  while (work) {
    int s = lsb(work); work &= work - 1;
    u64 t = T_between[s * 64 + sqking] & blockers;
    if (popc(t) == 1) pinned |= t;
  }
  work = rays_diag(bit(sqking), ~0ULL) & opp & bishops_queens(b);
  while (work) {
    int s = lsb(work); work &= work - 1;
    u64 t = T_between[s * 64 + sqking] & blockers;
    if (popc(t) == 1) pinned |= t;
  }

  /* per-lane pseudo moves and opposite attacks (zetaperft.cl:1063-1169) */
  u64 mv[64];
  u64 attacks = 0, checkers = 0;
  int sqchecker = 0;
  for (int lid = 0; lid < 64; lid++) {
    int p = piece_at(b, lid), color = p & 1, type = PTYPE(p);
    u64 pro = (color == stm) ? ~blockers : ~(blockers ^ bit(sqking));
    u64 gen = blockers & bit(lid);
    u64 w = rays_ortho(gen, pro) | rays_diag(gen, pro);
    if (type == KNIGHT) w = ~0ULL;
    int n = (color == stm) ? stm : !stm;
    n = (type == PAWN) ? n : type;
    u64 mask = T_attack[n * 64 + lid];
    u64 moves = (color == stm) ? (mask & w & opp) : (mask & w);
    if (type == PAWN) mask = T_push[stm * 64 + lid];
    if (color == stm && !qs) moves |= mask & w & ~blockers;
    mv[lid] = moves;
    if (color != stm) attacks |= moves;
  }
  for (int lid = 0; lid < 64; lid++)
    if (mv[lid] & bit(sqking)) { sqchecker = lid; checkers |= bit(lid); }
  *kic = checkers != 0;

  /* per-lane legality filters (zetaperft.cl:1201-1297) */
  int ncheck = popc(checkers);
  u64 epw = ~cr & EPMASK;
  int sqep = epw ? lsb(epw) : 0;
  u64 eppawns = me & (b[P1] & ~b[P2] & ~b[P3]) & (stm ? 0xFF000000ULL : 0xFF00000000ULL);
  u64 epcap = eppawns & (bit(sqep + 1) | bit(sqep - 1));
  int count = 0;
  for (int lid = 0; lid < 64; lid++) {
    int p = piece_at(b, lid), color = p & 1, type = PTYPE(p);
    u64 moves = (color == stm) ? mv[lid] : 0;
    if (ncheck >= 2 && type != KING) moves = 0;
    if (bit(lid) & pinned) moves &= T_line[lid * 64 + sqking];
    if (type == KING) moves &= ~attacks;
    if (ncheck == 1 && type != KING) moves &= T_between[sqchecker * 64 + sqking] | checkers;
    if (epcap & bit(lid)) {
      int sqto = stm ? sqep - 8 : sqep + 8;
      Move m = MKMOVE(lid, sqto, sqep, p, p, piece_at(b, sqep));
      u64 tb[4] = {b[0], b[1], b[2], b[3]};
      quick_play(tb, m);
      if (!square_attacked(tb, !stm, king_square(tb, stm))) moves |= bit(sqto);
    }
    /* castles: flags, rook present, empty path, unattacked path */
    int canq = lid == sqking && !qs && (cr & CR_ALL) &&
               ((stm && ((~cr & CR_BQ) == CR_BQ)) || (!stm && ((~cr & CR_WQ) == CR_WQ)));
    int rookq = piece_at(b, lid - 4) == ((ROOK << 1) | color);
    u64 emptq = (blockers & bit(lid - 1)) | (blockers & bit(lid - 2)) | (blockers & bit(lid - 3));
    u64 attq = (attacks & bit(lid)) | (attacks & bit(lid - 1)) | (attacks & bit(lid - 2));
    if (canq && rookq && !emptq && !attq) moves |= bit(lid - 2);
    int cank = lid == sqking && !qs && (cr & CR_ALL) &&
               ((stm && ((~cr & CR_BK) == CR_BK)) || (!stm && ((~cr & CR_WK) == CR_WK)));
    int rookk = piece_at(b, lid + 3) == ((ROOK << 1) | color);
    u64 emptk = (blockers & bit(lid + 1)) | (blockers & bit(lid + 2));
    u64 attk = (attacks & bit(lid)) | (attacks & bit(lid + 1)) | (attacks & bit(lid + 2));
    if (cank && rookk && !emptk && !attk) moves |= bit(lid + 2);
    lanes[lid] = moves;
    count += popc(moves);
  }
  return count;
}

/* Turn (lane, to-square) into a packed move, zetaperft.cl:1359-1384:
 * en-passant capture square, queen-only promotion. */
static Move decode_move(const u64 *b, int stm, int lid, int sqto) {
  int pfrom = piece_at(b, lid);
  int sqcpt = sqto;
  int pcpt = piece_at(b, sqcpt);
  if (PTYPE(pfrom) == PAWN && stm && lid - sqto != 8 && lid - sqto != 16 && pcpt == PNONE)
    sqcpt = sqto + 8;
  if (PTYPE(pfrom) == PAWN && !stm && sqto - lid != 8 && sqto - lid != 16 && pcpt == PNONE)
    sqcpt = sqto - 8;
  pcpt = piece_at(b, sqcpt);
  int pto = (PTYPE(pfrom) == PAWN && RRANK(sqto, stm) == 7) ? ((QUEEN << 1) | (pfrom & 1)) : pfrom;
  return MKMOVE(lid, sqto, sqcpt, pfrom, pto, pcpt);
}

/* Append move m and, when all_promotions is set and m is a promotion,
 * the same move promoting to a rook, a bishop and a knight (the
 * reference stops at the queen, zetaperft.cl:1380-1384). */
static int push_move(Move *moves, int n, Move m, int all_promotions) {
  moves[n++] = m;
  if (all_promotions && PTYPE(PFROM(m)) == PAWN && PTYPE(PTO(m)) == QUEEN) {
    const int side = PFROM(m) & 1;
    const int under[3] = {ROOK, BISHOP, KNIGHT};
    for (int i = 0; i < 3; i++)
      moves[n++] = MKMOVE(SQFROM(m), SQTO(m), SQCPT(m), PFROM(m), (under[i] << 1) | side, PCPT(m));
  }
  return n;
}

int zo_genmoves_ex(const zo_u64 board[7], int stm, int qs, int all_promotions, zo_move *moves) {
  u64 lanes[64];
  int kic;
  gen_lanes(board, stm, qs, board[PMVD], lanes, &kic);
  int n = 0;
  for (int lid = 0; lid < 64; lid++) {
    u64 t = lanes[lid];
    while (t) {
      int to = lsb(t); t &= t - 1;
      n = push_move(moves, n, decode_move(board, stm, lid, to), all_promotions);
    }
  }
  return n;
}

int zo_genmoves(const zo_u64 board[7], int stm, int qs, zo_move *moves) {
  return zo_genmoves_ex(board, stm, qs, 0, moves);
}

int zo_movecount(const zo_u64 board[7], int stm, int *in_check) {
  u64 lanes[64];
  int kic;
  int n = gen_lanes(board, stm, 0, board[PMVD], lanes, &kic);
  if (in_check) *in_check = kic;
  return n;
}

/* ------------------------------------------------------------------ */
static inline u64 rotl(u64 z, int s) { s &= 63; return s ? (z << s) | (z >> (64 - s)) : z; }

zo_u64 zo_computehash(const zo_u64 board[7], int stm) {
  u64 hash = 0;
  for (int side = 0; side <= 1; side++) {
    u64 w = side_bb(board, side);
    while (w) {
      int sq = lsb(w); w &= w - 1;
      int p = piece_at(board, sq);
      hash ^= rotl(ZOBRIST[(p & 1) * 6 + PTYPE(p) - 1], sq);
    }
  }
  u64 cr = board[PMVD];
  if (~cr & CR_WQ) hash ^= ZOBRIST[12];
  if (~cr & CR_WK) hash ^= ZOBRIST[13];
  if (~cr & CR_BQ) hash ^= ZOBRIST[14];
  if (~cr & CR_BK) hash ^= ZOBRIST[15];
  u64 ep = ~cr & EPMASK;
  int sqep = ep ? lsb(ep) : 0;
  if (sqep) hash ^= rotl(ZOBRIST[16], sqep & 7);
  if (stm) hash ^= 1ULL;
  return hash;
}

/* Moved flags after a move: zetaperft.cl:1440-1466 (perft) or
 * zeta.cl:2330-2343 (search, no castle rook squares). */
static u64 next_flags(u64 cr, Move m, int perft_flags) {
  int f = SQFROM(m), t = SQTO(m), pf = PFROM(m);
  cr |= bit(f) | bit(t) | bit(SQCPT(m));
  if (perft_flags) {
    if (PTYPE(pf) == KING && f - t == 2) cr |= bit(f - 4);
    if (PTYPE(pf) == KING && t - f == 2) cr |= bit(f + 3);
  }
  int sqep = (PTYPE(pf) == PAWN && RRANK(t, pf & 1) - RRANK(f, pf & 1) == 2) ? t : 0;
  cr |= EPMASK;
  if (sqep) cr &= ~bit(sqep);
  return cr;
}

/* Incremental hash of the search kernel's moveup, zeta.cl:2297-2359:
 * full piece rehash, ep key from the move, stm key, castle keys from the
 * new flags, and the extra stm flip of a null move. */
static u64 search_hash(const u64 *b, int stm_after, Move m, u64 cr_after) {
  u64 h = 0;
  for (int sq = 0; sq < 64; sq++) {
    int p = piece_at(b, sq);
    if (PTYPE(p)) h ^= rotl(ZOBRIST[(p & 1) * 6 + PTYPE(p) - 1], sq);
  }
  int pf = PFROM(m), f = SQFROM(m), t = SQTO(m);
  int sqto = (PTYPE(pf) == PAWN && RRANK(t, pf & 1) - RRANK(f, pf & 1) == 2) ? t : 0;
  if (sqto) h ^= rotl(ZOBRIST[16], sqto & 7);
  if (stm_after) h ^= 1ULL;
  if (~cr_after & CR_WQ) h ^= ZOBRIST[12];
  if (~cr_after & CR_WK) h ^= ZOBRIST[13];
  if (~cr_after & CR_BQ) h ^= ZOBRIST[14];
  if (~cr_after & CR_BK) h ^= ZOBRIST[15];
  if (m == NULLMOVE) h ^= 1ULL;
  return h;
}

void zo_play(zo_u64 board[7], int stm, zo_move m, int perft_flags) {
  do_pieces(board, m);
  u64 cr = next_flags(board[PMVD], m, perft_flags);
  board[PMVD] = cr;
  if (!perft_flags) {
    board[HASH] = search_hash(board, !stm, m, cr);
    u64 hmc = board[HMC] + 1;
    int pf = PFROM(m), f = SQFROM(m), t = SQTO(m);
    if (PTYPE(pf) == PAWN || PTYPE(PCPT(m)) != PNONE) hmc = 0;
    if (PTYPE(pf) == KING && (f - t == 2 || t - f == 2)) hmc = 0;
    board[HMC] = hmc & 0xFF; /* the kernel keeps it in a u8 */
  }
}

/* ------------------------------------------------------------------ */
/* perft_gpu leaf count: a leaf is a node reached after `depth` moves
 * (sd > search_depth, zetaperft.cl:1316-1324). */
static u64 perft_rec(u64 *b, int stm, int depth, int all_promotions) {
  if (depth == 0) return 1;
  u64 lanes[64];
  int kic;
  gen_lanes(b, stm, 0, b[PMVD], lanes, &kic);
  u64 total = 0;
  for (int lid = 0; lid < 64; lid++) {
    u64 t = lanes[lid];
    while (t) {
      int to = lsb(t); t &= t - 1;
      Move ms[4];
      const int k = push_move(ms, 0, decode_move(b, stm, lid, to), all_promotions);
      for (int i = 0; i < k; i++) {
        u64 c[7];
        memcpy(c, b, sizeof c);
        zo_play(c, stm, ms[i], 1);
        total += perft_rec(c, !stm, depth - 1, all_promotions);
      }
    }
  }
  return total;
}

zo_u64 zo_perft_ex(const zo_u64 board[7], int stm, int depth, int all_promotions) {
  u64 b[7];
  memcpy(b, board, sizeof b);
  return perft_rec(b, stm, depth, all_promotions);
}

zo_u64 zo_perft(const zo_u64 board[7], int stm, int depth) { return zo_perft_ex(board, stm, depth, 0); }

/* ------------------------------------------------------------------ */
/* Evaluation x64 + bishop pair, zeta.cl:1479-1531 (white's view). */
int zo_eval_white(const zo_u64 board[7]) {
  u64 blockers = occupancy(board);
  u64 pawns = board[P1] & ~board[P2] & ~board[P3];
  int total = 0;
  for (int lid = 0; lid < 64; lid++) {
    int p = piece_at(board, lid), color = p & 1, type = PTYPE(p);
    u64 me = color ? board[BLACKBB] : (board[BLACKBB] ^ blockers);
    u64 opp = color ? (board[BLACKBB] ^ blockers) : board[BLACKBB];
    int score = 0;
    int sqv = color ? lid : (lid ^ 56);
    if (type != PNONE) score += 10 + VALUE[type] + PST[type][sqv] + CONTROL[sqv];
    if (type == PAWN && color == 0) {
      if ((lid >> 3) < 7 && (opp & bit(lid + 8))) score -= 15;
      if ((lid & 7) < 7 && (pawns & me & bit(lid - 7))) score += 10;
      if ((lid & 7) > 0 && (pawns & me & bit(lid - 9))) score += 10;
      /* the kernel's loop variable is a u8 square */
      for (unsigned char s = (unsigned char)(lid - 8); s > 7; s -= 8)
        if (pawns & me & bit(s)) score -= 30;
    }
    if (type == PAWN && color == 1) {
      if ((lid >> 3) > 0 && (opp & bit(lid - 8))) score -= 15;
      if ((lid & 7) > 0 && (pawns & me & bit(lid + 7))) score += 10;
      if ((lid & 7) < 7 && (pawns & me & bit(lid + 9))) score += 10;
      for (unsigned char s = (unsigned char)(lid + 8); s < 56; s += 8)
        if (pawns & me & bit(s)) score -= 30;
    }
    total += color ? -score : score;
  }
  u64 bishops = ~board[P1] & ~board[P2] & board[P3];
  if (popc(board[BLACKBB] & bishops) == 2) total -= 25;
  if (popc((board[BLACKBB] ^ blockers) & bishops) == 2) total += 25;
  return total;
}

/* ------------------------------------------------------------------ */
static int negamax_rec(u64 *b, int stm, int depth, int ply, Move *best, u64 *nodes) {
  (*nodes)++;
  Move moves[ZO_MAXMOVES];
  int n = zo_genmoves(b, stm, 0, moves);
  if (n == 0) {
    int kic;
    zo_movecount(b, stm, &kic);
    return kic ? -ZO_INF + ply : 0;
  }
  if (depth == 0) {
    int e = zo_eval_white(b);
    return stm ? -e : e;
  }
  int bestv = -ZO_INF - 1;
  for (int i = 0; i < n; i++) {
    u64 c[7];
    memcpy(c, b, sizeof c);
    zo_play(c, stm, moves[i], 0);
    int v = -negamax_rec(c, !stm, depth - 1, ply + 1, NULL, nodes);
    if (v > bestv) { bestv = v; if (best) *best = moves[i]; }
  }
  return bestv;
}

int zo_negamax(const zo_u64 board[7], int stm, int depth, zo_move *bestmove, zo_u64 *nodes) {
  u64 b[7];
  memcpy(b, board, sizeof b);
  u64 cnt = 0;
  Move bm = 0;
  int v = negamax_rec(b, stm, depth, 0, &bm, &cnt);
  if (bestmove) *bestmove = bm;
  if (nodes) *nodes = cnt;
  return v;
}

static int ab_rec(u64 *b, int stm, int depth, int ply, int alpha, int beta, Move *best, u64 *nodes) {
  (*nodes)++;
  Move moves[ZO_MAXMOVES];
  int n = zo_genmoves(b, stm, 0, moves);
  if (n == 0) {
    int kic;
    zo_movecount(b, stm, &kic);
    return kic ? -ZO_INF + ply : 0;
  }
  if (depth == 0) {
    int e = zo_eval_white(b);
    return stm ? -e : e;
  }
  int bestv = -ZO_INF - 1;
  for (int i = 0; i < n; i++) {
    u64 c[7];
    memcpy(c, b, sizeof c);
    zo_play(c, stm, moves[i], 0);
    int v = -ab_rec(c, !stm, depth - 1, ply + 1, -beta, -alpha, NULL, nodes);
    if (v > bestv) { bestv = v; if (best) *best = moves[i]; }
    if (v > alpha) alpha = v;
    if (alpha >= beta) break;
  }
  return bestv;
}

int zo_alphabeta(const zo_u64 board[7], int stm, int depth, zo_move *bestmove, zo_u64 *nodes) {
  u64 b[7];
  memcpy(b, board, sizeof b);
  u64 cnt = 0;
  Move bm = 0;
  int v = ab_rec(b, stm, depth, 0, -ZO_INF - 1, ZO_INF + 1, &bm, &cnt);
  if (bestmove) *bestmove = bm;
  if (nodes) *nodes = cnt;
  return v;
}

/* ------------------------------------------------------------------ */
/* The same full-window alpha-beta with the moves of every node reordered:
 * the best move found at that node by the previous iteration (a move-only
 * table indexed by the board's hash, checked against the node's own list,
 * so a collision only changes the order), then captures by MVV-LVA
 * (V[captured] * 16 - V[mover], the reference's capture order,
 * zeta.cl:2039-2110), then two killer moves per ply.  Alpha-beta returns
 * the negamax value for any move order, so this equals zo_alphabeta and
 * zo_negamax; it only visits fewer nodes, which makes depth-7 fixtures of
 * middlegame positions affordable on host cores. */
typedef struct {
  u64 key;
  Move move;
} OrderSlot;
#define ORDER_BITS 20
#define ZO_MAXPLY_ORDERED 64

static int ab_ord_rec(u64 *b, int stm, int depth, int ply, int alpha, int beta, Move *best, u64 *nodes,
                      OrderSlot *tab, Move (*killers)[2]) {
  (*nodes)++;
  Move moves[ZO_MAXMOVES];
  int n = zo_genmoves(b, stm, 0, moves);
  if (n == 0) {
    int kic;
    zo_movecount(b, stm, &kic);
    return kic ? -ZO_INF + ply : 0;
  }
  if (depth == 0) {
    int e = zo_eval_white(b);
    return stm ? -e : e;
  }
  const u64 key = b[HASH] ^ (u64)stm;
  OrderSlot *slot = &tab[key & ((1u << ORDER_BITS) - 1)];
  const Move hashmove = slot->key == key ? slot->move : 0;
  int score[ZO_MAXMOVES];
  for (int i = 0; i < n; i++) {
    const Move m = moves[i];
    int s = 0;
    if (m == hashmove) s = 1 << 30;
    else if (PTYPE(PCPT(m)) != PNONE) s = (1 << 20) + VALUE[PTYPE(PCPT(m))] * 16 - VALUE[PTYPE(PFROM(m))];
    else if (m == killers[ply][0]) s = 1 << 19;
    else if (m == killers[ply][1]) s = 1 << 18;
    score[i] = s;
  }
  int bestv = -ZO_INF - 1;
  Move bm = 0;
  for (int i = 0; i < n; i++) {
    int k = i; /* selection of the highest remaining score, stable */
    for (int j = i + 1; j < n; j++)
      if (score[j] > score[k]) k = j;
    if (k != i) {
      Move tm = moves[k]; int ts = score[k];
      memmove(&moves[i + 1], &moves[i], (size_t)(k - i) * sizeof(Move));
      memmove(&score[i + 1], &score[i], (size_t)(k - i) * sizeof(int));
      moves[i] = tm; score[i] = ts;
    }
    u64 c[7];
    memcpy(c, b, sizeof c);
    zo_play(c, stm, moves[i], 0);
    int v = -ab_ord_rec(c, !stm, depth - 1, ply + 1, -beta, -alpha, NULL, nodes, tab, killers);
    if (v > bestv) { bestv = v; bm = moves[i]; }
    if (v > alpha) alpha = v;
    if (alpha >= beta) {
      if (PTYPE(PCPT(moves[i])) == PNONE && killers[ply][0] != moves[i]) {
        killers[ply][1] = killers[ply][0];
        killers[ply][0] = moves[i];
      }
      break;
    }
  }
  slot->key = key;
  slot->move = bm;
  if (best) *best = bm;
  return bestv;
}

int zo_alphabeta_ordered(const zo_u64 board[7], int stm, int depth, zo_move *bestmove, zo_u64 *nodes) {
  OrderSlot *tab = calloc((size_t)1 << ORDER_BITS, sizeof(OrderSlot));
  Move (*killers)[2] = calloc(ZO_MAXPLY_ORDERED, sizeof *killers);
  if (!tab || !killers) {
    free(tab);
    free(killers);
    return zo_alphabeta(board, stm, depth, bestmove, nodes);
  }
  u64 b[7];
  memcpy(b, board, sizeof b);
  b[HASH] = zo_computehash(b, stm);
  u64 cnt = 0;
  Move bm = 0;
  int v = 0;
  for (int d = 1; d <= depth; d++) v = ab_ord_rec(b, stm, d, 0, -ZO_INF - 1, ZO_INF + 1, &bm, &cnt, tab, killers);
  free(tab);
  free(killers);
  if (depth <= 0) v = ab_rec(b, stm, depth, 0, -ZO_INF - 1, ZO_INF + 1, &bm, &cnt);
  if (bestmove) *bestmove = bm;
  if (nodes) *nodes = cnt;
  return v;
}

/* ------------------------------------------------------------------ */
zo_u64 zo_splitmix64(zo_u64 *state) {
  u64 z = (*state += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

int zo_make_position(zo_u64 seed, int i, int min_plies, int max_plies, int min_pieces, int min_depth,
                     int max_depth, zo_u64 board[7], int *stm, int *depth) {
  u64 s = seed ^ (0xD1B54A32D192ED03ULL * (u64)(i + 1));
  for (int attempt = 0; attempt < 64; attempt++) {
    int plies = min_plies + (int)(zo_splitmix64(&s) % (u64)(max_plies - min_plies + 1));
    int side;
    zo_setboard(board, &side, "rnbqkbnr/pppppppp/8/8/8/8/PPPPPPPP/RNBQKBNR w KQkq - 0 1");
    int ok = 1;
    for (int k = 0; k < plies; k++) {
      Move moves[ZO_MAXMOVES];
      int n = zo_genmoves(board, side, 0, moves); /* (from,to) order */
      if (n == 0) { ok = 0; break; }
      zo_play(board, side, moves[zo_splitmix64(&s) % (u64)n], 0);
      side = !side;
    }
    if (!ok || zo_movecount(board, side, NULL) == 0 || popc(occupancy(board)) < min_pieces) continue;
    board[HASH] = zo_computehash(board, side);
    *stm = side;
    *depth = min_depth + (int)(zo_splitmix64(&s) % (u64)(max_depth - min_depth + 1));
    return 1;
  }
  return 0;
}

int zo_playout(zo_u64 seed, int plies, zo_u64 board[7], int *stm) {
  int side;
  zo_setboard(board, &side, "rnbqkbnr/pppppppp/8/8/8/8/PPPPPPPP/RNBQKBNR w KQkq - 0 1");
  u64 st = seed;
  for (int i = 0; i < plies; i++) {
    Move moves[ZO_MAXMOVES];
    int n = zo_genmoves(board, side, 0, moves);
    if (n == 0) { *stm = side; return 0; }
    Move m = moves[zo_splitmix64(&st) % (u64)n];
    zo_play(board, side, m, 0);
    side = !side;
  }
  *stm = side;
  return 1;
}

/* ------------------------------------------------------------------ */
/* setboard(), src/io.c:335-531 */
int zo_setboard(zo_u64 board[7], int *stm, const char *fen) {
  init_tables();
  char pos[1024] = {0}, side[16] = {0}, castle[16] = {0}, ep[16] = {0};
  unsigned long long hmc = 0, fullmove = 1;
  if (sscanf(fen, "%1023s %15s %15s %15s %llu %llu", pos, side, castle, ep, &hmc, &fullmove) < 1)
    return 0;
  (void)fullmove;
  memset(board, 0, 7 * sizeof(u64));
  board[PMVD] = ~0ULL;
  static const char map[] = " PNKBRQ pnkbrq/12345678";
  int file = 0, rank = 7;
  for (const char *c = pos; *c && !(rank <= 0 && file >= 8); c++) {
    const char *hit = strchr(map, *c);
    if (!hit || *c == ' ') continue;
    int j = (int)(hit - map);
    if (j == 14) { rank--; file = 0; }
    else if (j >= 15) file += j - 14;
    else {
      int p = (j >= 7) ? (((j - 7) << 1) | 1) : (j << 1);
      int sq = rank * 8 + file;
      if (sq >= 0 && sq < 64)
        for (int i = 0; i < 4; i++) board[i] |= (u64)((p >> i) & 1) << sq;
      file++;
    }
  }
  *stm = (side[0] == 'b' || side[0] == 'B') ? 1 : 0;
  u64 cr = 0;
  if (castle[0] != '-')
    for (const char *c = castle; *c; c++) {
      if (*c == 'Q') cr |= CR_WQ;
      if (*c == 'K') cr |= CR_WK;
      if (*c == 'q') cr |= CR_BQ;
      if (*c == 'k') cr |= CR_BK;
    }
  board[PMVD] ^= cr;
  board[HMC] = hmc;
  if (ep[0] && ep[0] != '-') {
    int sq = (ep[1] - '1') * 8 + (ep[0] - 'a');
    if (sq > 0 && sq < 64) board[PMVD] &= ~bit(sq);
  }
  board[HASH] = zo_computehash(board, *stm);
  /* isvalid(): one king per side, src/bitboard.c:448-459 */
  u64 kings = board[P1] & board[P2] & ~board[P3];
  if (popc(board[BLACKBB] & kings) != 1 || popc((board[BLACKBB] ^ occupancy(board)) & kings) != 1)
    return 0;
  return 1;
}

void zo_move2can(zo_move m, char out[6]) {
  out[0] = (char)('a' + (SQFROM(m) & 7));
  out[1] = (char)('1' + (SQFROM(m) >> 3));
  out[2] = (char)('a' + (SQTO(m) & 7));
  out[3] = (char)('1' + (SQTO(m) >> 3));
  out[4] = 0;
  int pf = PTYPE(PFROM(m)), pt = PTYPE(PTO(m));
  if (pf == PAWN && pt != PAWN) {
    out[4] = pt == QUEEN ? 'q' : pt == ROOK ? 'r' : pt == BISHOP ? 'b' : 'n';
    out[5] = 0;
  }
}

zo_move zo_can2move(const char *s, const zo_u64 board[7], int stm) {
  int from = (s[1] - '1') * 8 + (s[0] - 'a');
  int to = (s[3] - '1') * 8 + (s[2] - 'a');
  int pfrom = piece_at(board, from), pto = pfrom, sqcpt = to;
  int pcpt = piece_at(board, to);
  if (PTYPE(pfrom) == PAWN && !stm && (from >> 3) == 4 && to - from != 8 && pcpt == PNONE) sqcpt = to - 8;
  if (PTYPE(pfrom) == PAWN && stm && (from >> 3) == 3 && from - to != 8 && pcpt == PNONE) sqcpt = to + 8;
  pcpt = piece_at(board, sqcpt);
  switch (s[4]) {
    case 'q': case 'Q': pto = (QUEEN << 1) | stm; break;
    case 'n': case 'N': pto = (KNIGHT << 1) | stm; break;
    case 'b': case 'B': pto = (BISHOP << 1) | stm; break;
    case 'r': case 'R': pto = (ROOK << 1) | stm; break;
    default: break;
  }
  return MKMOVE(from, to, sqcpt, pfrom, pto, pcpt);
}
