/*
 * board.c -- host-side board layer (see board.h).
 */
#include "board.h"

#include <stdio.h>
#include <string.h>

#define EPMASK 0x000000FFFF000000ULL
#define CR_WQ 0x0000000000000011ULL
#define CR_WK 0x0000000000000090ULL
#define CR_BQ 0x1100000000000000ULL
#define CR_BK 0x9000000000000000ULL

/* Zobrist keys of the reference (zeta.cl:258-265), needed for identical hashes */
static const Bitboard ZOB[18] = {
    0x9D39247E33776D41ULL, 0x2AF7398005AAA5C7ULL, 0x44DB015024623547ULL, 0x9C15F73E62A76AE2ULL,
    0x75834465489C0C89ULL, 0x3290AC3A203001BFULL, 0x0FBBAD1F61042279ULL, 0xE83A908FF2FB60CAULL,
    0x0D7E765D58755C10ULL, 0x1A083822CEAFE02DULL, 0x9605D5F0E25EC3B0ULL, 0xD021FF5CD13A2ED5ULL,
    0x40BDF15D4A672E32ULL, 0x011355146FD56395ULL, 0x5DB4832046F3D9E5ULL, 0x239F8B2D7FF719CCULL,
    0x05D1A1AE85B49AA1ULL, 0x679F848F6E8FC971ULL};

static inline Bitboard sqbit(int sq) { return 1ULL << (sq & 63); }
static inline Bitboard rotl(Bitboard z, int s) {
  s &= 63;
  return s ? (z << s) | (z >> (64 - s)) : z;
}

int board_piece(const Bitboard b[7], int sq) {
  sq &= 63;
  return (int)(((b[0] >> sq) & 1) | (((b[1] >> sq) & 1) << 1) | (((b[2] >> sq) & 1) << 2) |
               (((b[3] >> sq) & 1) << 3));
}

static void put(Bitboard b[7], int sq, int pc) {
  for (int i = 0; i < 4; i++) b[i] |= (Bitboard)((pc >> i) & 1) << sq;
}

Bitboard board_hash(const Bitboard b[7], int stm) {
  Bitboard h = 0, occ = b[1] | b[2] | b[3];
  while (occ) {
    int sq = __builtin_ctzll(occ);
    occ &= occ - 1;
    int pc = board_piece(b, sq);
    h ^= rotl(ZOB[(pc & 1) * 6 + (pc >> 1) - 1], sq);
  }
  Bitboard cr = b[QBBPMVD];
  if (~cr & CR_WQ) h ^= ZOB[12];
  if (~cr & CR_WK) h ^= ZOB[13];
  if (~cr & CR_BQ) h ^= ZOB[14];
  if (~cr & CR_BK) h ^= ZOB[15];
  Bitboard ep = ~cr & EPMASK;
  if (ep) h ^= rotl(ZOB[16], __builtin_ctzll(ep) & 7);
  if (stm) h ^= 1ULL;
  return h;
}

bool board_setfen(Bitboard b[7], int *stm, int *fullmove, const char *fen) {
  char pos[1024] = {0}, side[16] = {0}, castle[16] = {0}, ep[16] = {0};
  unsigned long long hmc = 0, full = 1;
  if (sscanf(fen, "%1023s %15s %15s %15s %llu %llu", pos, side, castle, ep, &hmc, &full) < 1) return false;
  memset(b, 0, 7 * sizeof(Bitboard));
  b[QBBPMVD] = ~0ULL;
  static const char map[] = " PNKBRQ pnkbrq/12345678";
  int file = 0, rank = 7;
  for (const char *c = pos; *c && !(rank <= 0 && file >= 8); c++) {
    const char *hit = strchr(map, *c);
    if (!hit || *c == ' ') continue;
    int j = (int)(hit - map);
    if (j == 14) {
      rank--;
      file = 0;
    } else if (j >= 15) {
      file += j - 14;
    } else {
      int pc = (j >= 7) ? (((j - 7) << 1) | BLACK) : (j << 1);
      int sq = rank * 8 + file;
      if (sq >= 0 && sq < 64) put(b, sq, pc);
      file++;
    }
  }
  *stm = (side[0] == 'b' || side[0] == 'B') ? BLACK : WHITE;
  Bitboard cr = 0;
  if (castle[0] != '-')
    for (const char *c = castle; *c; c++) {
      if (*c == 'Q') cr |= CR_WQ;
      if (*c == 'K') cr |= CR_WK;
      if (*c == 'q') cr |= CR_BQ;
      if (*c == 'k') cr |= CR_BK;
    }
  b[QBBPMVD] ^= cr;
  b[QBBHMC] = hmc;
  /* the reference clears the FEN target square's flag (rank 3/6), which
   * lies outside its rank-4/5 en-passant mask (src/io.c:495-505) */
  if (ep[0] && ep[0] != '-') {
    int sq = (ep[1] - '1') * 8 + (ep[0] - 'a');
    if (sq > 0 && sq < 64) b[QBBPMVD] &= ~sqbit(sq);
  }
  b[QBBHASH] = board_hash(b, *stm);
  if (fullmove) *fullmove = (int)full;
  Bitboard kings = b[1] & b[2] & ~b[3], occ = b[1] | b[2] | b[3];
  return __builtin_popcountll(b[0] & kings) == 1 && __builtin_popcountll((b[0] ^ occ) & kings) == 1;
}

void board_getfen(const Bitboard b[7], int stm, int fullmove, char *out, int outlen) {
  static const char pcs[] = " PNKBRQ pnkbrq";
  char buf[128];
  int n = 0;
  for (int rank = 7; rank >= 0; rank--) {
    int empty = 0;
    for (int file = 0; file < 8; file++) {
      int pc = board_piece(b, rank * 8 + file);
      if (!(pc >> 1)) {
        empty++;
        continue;
      }
      if (empty) buf[n++] = (char)('0' + empty);
      empty = 0;
      buf[n++] = pcs[(pc & 1) * 7 + (pc >> 1)];
    }
    if (empty) buf[n++] = (char)('0' + empty);
    if (rank) buf[n++] = '/';
  }
  buf[n++] = ' ';
  buf[n++] = stm ? 'b' : 'w';
  buf[n++] = ' ';
  int c0 = n;
  Bitboard cr = b[QBBPMVD];
  if ((~cr & CR_WK) == CR_WK) buf[n++] = 'K';
  if ((~cr & CR_WQ) == CR_WQ) buf[n++] = 'Q';
  if ((~cr & CR_BK) == CR_BK) buf[n++] = 'k';
  if ((~cr & CR_BQ) == CR_BQ) buf[n++] = 'q';
  if (n == c0) buf[n++] = '-';
  buf[n++] = ' ';
  Bitboard ep = ~cr & EPMASK;
  if (ep) {
    int sq = __builtin_ctzll(ep) + (stm ? -8 : 8);
    buf[n++] = (char)('a' + (sq & 7));
    buf[n++] = (char)('1' + (sq >> 3));
  } else {
    buf[n++] = '-';
  }
  buf[n] = 0;
  snprintf(out, outlen, "%s %llu %d", buf, (unsigned long long)b[QBBHMC], fullmove);
}

void board_play(Bitboard b[7], int stm, Move m) {
  int f = GETSQFROM(m), t = GETSQTO(m), c = GETSQCPT(m), pf = GETPFROM(m), pt = GETPTO(m);
  if (m != MOVENONE && m != NULLMOVE) {
    Bitboard clr = ~sqbit(f) & ~sqbit(c) & ~sqbit(t);
    int qc = (pf >> 1) == KING && f - t == 2, kc = (pf >> 1) == KING && t - f == 2;
    if (qc) clr &= ~sqbit(f - 4);
    if (kc) clr &= ~sqbit(f + 3);
    for (int i = 0; i < 4; i++) b[i] &= clr;
    put(b, t, pt);
    if (qc) put(b, t + 1, (ROOK << 1) | (pf & 1));
    if (kc) put(b, t - 1, (ROOK << 1) | (pf & 1));
  }
  Bitboard cr = b[QBBPMVD] | sqbit(f) | sqbit(t) | sqbit(c);
  int col = pf & 1;
  int rt = col ? ((t >> 3) ^ 7) : (t >> 3), rf = col ? ((f >> 3) ^ 7) : (f >> 3);
  cr |= EPMASK;
  if ((pf >> 1) == PAWN && rt - rf == 2 && t) cr &= ~sqbit(t);
  b[QBBPMVD] = cr;
  unsigned hmc = (unsigned)(b[QBBHMC] + 1) & 0xFF;
  if ((pf >> 1) == PAWN || (GETPCPT(m) >> 1) != PNONE) hmc = 0;
  if ((pf >> 1) == KING && (f - t == 2 || t - f == 2)) hmc = 0;
  b[QBBHMC] = hmc;
  b[QBBHASH] = board_hash(b, !stm) ^ (m == NULLMOVE ? 1ULL : 0ULL);
}

void move2can(Move m, char out[6]) {
  out[0] = (char)('a' + (GETSQFROM(m) & 7));
  out[1] = (char)('1' + (GETSQFROM(m) >> 3));
  out[2] = (char)('a' + (GETSQTO(m) & 7));
  out[3] = (char)('1' + (GETSQTO(m) >> 3));
  out[4] = 0;
  int pf = GETPFROM(m) >> 1, pt = GETPTO(m) >> 1;
  if (pf == PAWN && pt != PAWN) {
    out[4] = pt == QUEEN ? 'q' : pt == ROOK ? 'r' : pt == BISHOP ? 'b' : 'n';
    out[5] = 0;
  }
}

bool move_text_ok(const char *s) {
  if (!s) return false;
  const size_t n = strlen(s);
  if (n != 4 && n != 5) return false;
  for (int i = 0; i < 4; i += 2)
    if (s[i] < 'a' || s[i] > 'h' || s[i + 1] < '1' || s[i + 1] > '8') return false;
  return n == 4 || strchr("qrbnQRBN", s[4]) != NULL;
}

Move can2move(const char *s, const Bitboard b[7], int stm) {
  int from = (s[1] - '1') * 8 + (s[0] - 'a'), to = (s[3] - '1') * 8 + (s[2] - 'a');
  from &= 63;
  to &= 63;
  int pfrom = board_piece(b, from), pto = pfrom, cpt = to;
  int pcpt = board_piece(b, to);
  if ((pfrom >> 1) == PAWN && !stm && (from >> 3) == 4 && to - from != 8 && !(pcpt >> 1)) cpt = to - 8;
  if ((pfrom >> 1) == PAWN && stm && (from >> 3) == 3 && from - to != 8 && !(pcpt >> 1)) cpt = to + 8;
  pcpt = board_piece(b, cpt);
  switch (s[4]) {
    case 'q': case 'Q': pto = (QUEEN << 1) | stm; break;
    case 'n': case 'N': pto = (KNIGHT << 1) | stm; break;
    case 'b': case 'B': pto = (BISHOP << 1) | stm; break;
    case 'r': case 'R': pto = (ROOK << 1) | stm; break;
    default: break;
  }
  return (Move)from | ((Move)to << 6) | ((Move)cpt << 12) | ((Move)pfrom << 18) | ((Move)pto << 22) |
         ((Move)pcpt << 26);
}

void board_print(const Bitboard b[7], int stm) {
  static const char pcs[] = " PNKBRQ pnkbrq";
  printf("###ABCDEFGH###\n");
  for (int rank = 7; rank >= 0; rank--) {
    printf("#%d ", rank + 1);
    for (int file = 0; file < 8; file++) {
      int pc = board_piece(b, rank * 8 + file);
      putchar((pc >> 1) ? pcs[(pc & 1) * 7 + (pc >> 1)] : '-');
    }
    printf("\n");
  }
  printf("# %s to move, hash 0x%016llx\n", stm ? "black" : "white", (unsigned long long)b[QBBHASH]);
}
