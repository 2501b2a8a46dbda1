"""A second, independent move generator for the tests: a 64-square mailbox
walked square by square (pseudo-legal moves, then "is my king attacked
after the move"), written from the rules of chess.  It shares no code and
no method with the oracle (set-wise bitboard lanes) or the device
generators, and exists to pin a rule the reference cannot: promotion to a
rook, bishop or knight, which the reference never generates
(zetaperft.cl:1380-1384 makes every promotion a queen).  With
all_promotions=False it must reproduce the oracle's (reference-pinned)
counts, which checks the mailbox itself.

Only the formats are the reference's, so that results compare move for
move:
  * board: 7 x u64 quad bitboard (src/types.h:59-66) -- b[0] black,
    b[1..3] piece-type bit planes, b[4] the "moved" flags from which castle
    rights and the en-passant square follow;
  * piece code type << 1 | colour (colour 1 = black), types PAWN 1,
    KNIGHT 2, KING 3, BISHOP 4, ROOK 5, QUEEN 6;
  * moves: from | to << 6 | capture square << 12 | piece from << 18 |
    piece to << 22 | captured piece << 26 (src/types.h:67-74);
  * castling needs the king's and the rook's squares unflagged and, as the
    reference tests it, at least one of the squares of its castle mask
    flagged (zetaperft.cl:1249-1297); a move flags its from, to and capture
    squares, a castle also the rook's square, and a double push leaves its
    square unflagged as the en-passant mark (zetaperft.cl:1440-1466).

Pure Python: small positions and depths only (test infrastructure).
"""
from __future__ import annotations

PAWN, KNIGHT, KING, BISHOP, ROOK, QUEEN = 1, 2, 3, 4, 5, 6
EPMASK = 0x000000FFFF000000
CR_ALL = 0x8900000000000091
CR_WQ, CR_WK = 0x11, 0x90
CR_BQ, CR_BK = 0x1100000000000000, 0x9000000000000000
M64 = (1 << 64) - 1

KNIGHT_STEPS = ((1, 2), (2, 1), (2, -1), (1, -2), (-1, -2), (-2, -1), (-2, 1), (-1, 2))
KING_STEPS = ((1, 0), (1, 1), (0, 1), (-1, 1), (-1, 0), (-1, -1), (0, -1), (1, -1))
ORTHO = ((1, 0), (-1, 0), (0, 1), (0, -1))
DIAG = ((1, 1), (1, -1), (-1, 1), (-1, -1))


def squares_from_board(b) -> list[int]:
    """64 piece codes (0 = empty) from a quad bitboard."""
    b = [int(x) for x in b]
    return [((b[0] >> q) & 1) | (((b[1] >> q) & 1) << 1) | (((b[2] >> q) & 1) << 2) | (((b[3] >> q) & 1) << 3)
            for q in range(64)]


def _at(f: int, r: int) -> int:
    return r * 8 + f if 0 <= f < 8 and 0 <= r < 8 else -1


def attacked(sq: list[int], target: int, by: int) -> bool:
    """Is square `target` attacked by a piece of colour `by`?"""
    f0, r0 = target & 7, target >> 3
    for df, dr in KNIGHT_STEPS:
        q = _at(f0 + df, r0 + dr)
        if q >= 0 and sq[q] == (KNIGHT << 1 | by):
            return True
    for df, dr in KING_STEPS:
        q = _at(f0 + df, r0 + dr)
        if q >= 0 and sq[q] == (KING << 1 | by):
            return True
    # a white pawn attacks upward, so it stands one rank below its target
    pr = r0 - 1 if by == 0 else r0 + 1
    for df in (-1, 1):
        q = _at(f0 + df, pr)
        if q >= 0 and sq[q] == (PAWN << 1 | by):
            return True
    for dirs, kinds in ((ORTHO, (ROOK, QUEEN)), (DIAG, (BISHOP, QUEEN))):
        for df, dr in dirs:
            f, r = f0 + df, r0 + dr
            while 0 <= f < 8 and 0 <= r < 8:
                p = sq[r * 8 + f]
                if p:
                    if (p & 1) == by and (p >> 1) in kinds:
                        return True
                    break
                f += df
                r += dr
    return False


def _pack(frm: int, to: int, cpt: int, pfrom: int, pto: int, pcpt: int) -> int:
    return frm | to << 6 | cpt << 12 | pfrom << 18 | pto << 22 | pcpt << 26


def _apply(sq: list[int], m: int) -> list[int]:
    """Pieces after move m (castles move the rook too)."""
    frm, to, cpt, pfrom, pto = m & 63, (m >> 6) & 63, (m >> 12) & 63, (m >> 18) & 15, (m >> 22) & 15
    s = list(sq)
    s[frm] = 0
    s[cpt] = 0
    s[to] = pto
    if pfrom >> 1 == KING and abs(to - frm) == 2:
        rook_from, rook_to = (frm + 3, frm + 1) if to > frm else (frm - 4, frm - 1)
        s[rook_to] = s[rook_from]
        s[rook_from] = 0
    return s


def _flags_after(cr: int, m: int) -> int:
    frm, to, cpt, pfrom = m & 63, (m >> 6) & 63, (m >> 12) & 63, (m >> 18) & 15
    cr |= (1 << frm) | (1 << to) | (1 << cpt)
    if pfrom >> 1 == KING and to - frm == 2:
        cr |= 1 << (frm + 3)
    if pfrom >> 1 == KING and frm - to == 2:
        cr |= 1 << (frm - 4)
    cr |= EPMASK
    if pfrom >> 1 == PAWN and abs(to - frm) == 16:
        cr &= ~(1 << to) & M64
    return cr


def _king(sq: list[int], side: int) -> int:
    return sq.index(KING << 1 | side)


def pseudo_moves(sq: list[int], cr: int, stm: int, all_promotions: bool) -> list[int]:
    """Every move of the side to move that ignores its own king's safety
    (castling already requires the king's path to be unattacked)."""
    out = []
    them = stm ^ 1
    promo_types = (QUEEN, ROOK, BISHOP, KNIGHT) if all_promotions else (QUEEN,)
    fwd = 1 if stm == 0 else -1
    last = 7 if stm == 0 else 0
    start = 1 if stm == 0 else 6
    for frm in range(64):
        p = sq[frm]
        if not p or (p & 1) != stm:
            continue
        kind, f0, r0 = p >> 1, frm & 7, frm >> 3
        if kind == PAWN:
            targets = []
            one = _at(f0, r0 + fwd)
            if one >= 0 and not sq[one]:
                targets.append((one, 0))
                two = _at(f0, r0 + 2 * fwd)
                if r0 == start and not sq[two]:
                    targets.append((two, 0))
            for df in (-1, 1):
                q = _at(f0 + df, r0 + fwd)
                if q >= 0 and sq[q] and (sq[q] & 1) == them:
                    targets.append((q, sq[q]))
            for to, victim in targets:
                if to >> 3 == last:
                    for t in promo_types:
                        out.append(_pack(frm, to, to, p, t << 1 | stm, victim))
                else:
                    out.append(_pack(frm, to, to, p, p, victim))
            continue
        if kind in (KNIGHT, KING):
            for df, dr in (KNIGHT_STEPS if kind == KNIGHT else KING_STEPS):
                q = _at(f0 + df, r0 + dr)
                if q >= 0 and (not sq[q] or (sq[q] & 1) == them):
                    out.append(_pack(frm, q, q, p, p, sq[q]))
            continue
        dirs = ORTHO if kind == ROOK else DIAG if kind == BISHOP else ORTHO + DIAG
        for df, dr in dirs:
            f, r = f0 + df, r0 + dr
            while 0 <= f < 8 and 0 <= r < 8:
                q = r * 8 + f
                if sq[q] and (sq[q] & 1) == stm:
                    break
                out.append(_pack(frm, q, q, p, p, sq[q]))
                if sq[q]:
                    break
                f += df
                r += dr
    # en passant: the enemy pawn that just made a double push stands on the
    # one unflagged square of ranks 4-5
    ep = ~cr & EPMASK
    if ep:
        victim_sq = (ep & -ep).bit_length() - 1
        to = victim_sq + 8 * fwd
        for df in (-1, 1):
            frm = _at((victim_sq & 7) + df, victim_sq >> 3)
            if frm >= 0 and sq[frm] == (PAWN << 1 | stm) and (frm >> 3) == (4 if stm == 0 else 3):
                out.append(_pack(frm, to, victim_sq, sq[frm], sq[frm], sq[victim_sq]))
    # castling
    k = _king(sq, stm)
    if cr & CR_ALL:
        rook = ROOK << 1 | stm
        qmask, kmask = (CR_WQ, CR_WK) if stm == 0 else (CR_BQ, CR_BK)
        if (~cr & qmask) == qmask and k - 4 >= 0 and sq[k - 4] == rook and not (sq[k - 1] or sq[k - 2] or sq[k - 3]):
            if not any(attacked(sq, s, them) for s in (k, k - 1, k - 2)):
                out.append(_pack(k, k - 2, k - 2, sq[k], sq[k], 0))
        if (~cr & kmask) == kmask and k + 3 < 64 and sq[k + 3] == rook and not (sq[k + 1] or sq[k + 2]):
            if not any(attacked(sq, s, them) for s in (k, k + 1, k + 2)):
                out.append(_pack(k, k + 2, k + 2, sq[k], sq[k], 0))
    return out


def legal_moves(sq: list[int], cr: int, stm: int, all_promotions: bool = False) -> list[int]:
    out = []
    for m in pseudo_moves(sq, cr, stm, all_promotions):
        after = _apply(sq, m)
        if not attacked(after, _king(after, stm), stm ^ 1):
            out.append(m)
    return out


def perft(sq: list[int], cr: int, stm: int, depth: int, all_promotions: bool = False) -> int:
    if depth == 0:
        return 1
    moves = legal_moves(sq, cr, stm, all_promotions)
    if depth == 1:
        return len(moves)
    return sum(perft(_apply(sq, m), _flags_after(cr, m), stm ^ 1, depth - 1, all_promotions) for m in moves)


def board_perft(board, stm: int, depth: int, all_promotions: bool = False) -> int:
    return perft(squares_from_board(board), int(board[4]), int(stm), depth, all_promotions)


def board_moves(board, stm: int, all_promotions: bool = False) -> list[int]:
    return legal_moves(squares_from_board(board), int(board[4]), int(stm), all_promotions)
