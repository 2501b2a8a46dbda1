/*
 * legal_test_check.cc -- host build of the device chess core (chess.cuh,
 * movegen_fast.cuh, tables.cuh) for the CPU tests.  Walks full move trees
 * and checks at every node that
 *   - the quick free-move test (has_free_move, used at pure-search leaves)
 *     and its king-step extension (has_quick_move_rolled) never claim a
 *     legal move where the exact count (count_legal_ex) finds none,
 *     has_legal_ex equals "count > 0", and all report the same in-check
 *     flag;
 *   - the search kernels' generator (gen_engine) gives the perft
 *     generator's (gen_legal) move set, all moves and captures only;
 *   - with all four promotions, the perft generator (gen_legal<true>)
 *     gives the oracle's zo_genmoves_ex set and its bulk count
 *     (count_legal_ex<true>) that set's size;
 *   - the warp generator's plan and per-move decode (warpgen.cuh), in
 *     both their unrolled and rolled forms, give gen_engine's list move for
 *     move, in the same order, and the same in-check flag;
 *   - the incremental Zobrist update of the search kernels (parent hash ^
 *     side toggle ^ castle / en-passant keys ^ piece_delta) equals hashing
 *     every child from scratch (compute_hash), and compute_hash equals the
 *     oracle's zo_computehash;
 *   - the device evaluation source (eval.cuh) equals the oracle's
 *     zo_eval_white, and its incremental form (piece terms of the parent
 *     plus the move's change, plus the structure terms) equals it on every
 *     child.
 * Linked with the oracle (oracle/zeta_oracle.c) as the checker.
 * Arguments: b0:p1:p2:p3:cr:stm:depth per root.  Prints one line per
 * root; exit status 1 on any disagreement.
 */
#include <algorithm>
#include <cstdio>
#include <cstdlib>

#define ZE static inline
#include "../../oracle/zeta_oracle.h"
#include "../../zeta_gb300/csrc/chess.cuh"
#include "../../zeta_gb300/csrc/eval.cuh"
#include "../../zeta_gb300/csrc/movegen_fast.cuh"
#include "../../zeta_gb300/csrc/tables.cuh"
#include "../../zeta_gb300/csrc/warpgen.cuh"

using namespace zeta;

static unsigned long long g_nodes = 0, g_bad = 0, g_quick = 0, g_king = 0;

static void walk(const Pos &p, int stm, int depth) {
  bool c1, c2, c3;
  const int n = count_legal_ex(p, stm, c1);
  const bool quick = has_free_move(p, stm, c2);
  {
    bool cr, ck;
    if (has_free_move_rolled(p, stm, cr) != quick || cr != c2) {
      if (g_bad < 5) printf("rolled quick test differs\n");
      g_bad++;
    }
    const bool qk = has_quick_move_rolled(p, stm, ck);
    g_king += qk && !quick;
    if ((qk && n == 0) || ck != c1) {
      if (g_bad < 5) printf("king-step quick test claims a move the count does not find\n");
      g_bad++;
    }
  }
  const bool has = has_legal_ex(p, stm, c3);
  g_nodes++;
  g_quick += quick;
  if ((quick && n == 0) || has != (n > 0) || c1 != c2 || c1 != c3) {
    if (g_bad < 5) printf("disagreement: count %d quick %d has %d check %d/%d/%d\n", n, quick, has, c1, c2, c3);
    g_bad++;
  }
  const zo_u64 b7[7] = {p.b0, p.p1, p.p2, p.p3, p.cr, 0, 0};
  if (eval_white(p, kEvalHost) != zo_eval_white(b7) || compute_hash(p, stm) != zo_computehash(b7, stm)) {
    if (g_bad < 5) printf("evaluation or hash differs from the oracle's\n");
    g_bad++;
  }
  const Sets sets = make_sets(p, stm);
  const u64 danger = enemy_attacks(sets, stm);
  for (int qs = 0; qs < 2; qs++) {
    Move a[256], b[256];
    const int na = gen_legal(p, stm, qs != 0, a);
    const int nb = gen_engine(p, sets, danger, stm, qs != 0, b);
    {
      u64 set[kEmitters];
      bool chk = false;
      int sqep = 0;
      const int nw = gen_plan(p, sets, danger, stm, qs != 0, set, &chk, &sqep);
      uint8_t off[kEmitters + 1];
      off[0] = 0;
      for (int e = 0; e < kEmitters; e++) off[e + 1] = (uint8_t)(off[e] + popc(set[e]));
      bool same = nw == nb && chk == c1 && off[kEmitters] == nw;
      for (int j = 0; same && j < nw; j++) same = gen_move_at(p, sets, stm, set, off, sqep, j) == b[j];
      /* the rolled form: the same attack map, sets, flags and list */
      u64 setr[kEmitters];
      bool chkr = false;
      int sqepr = -1;
      same = same && enemy_attacks_rolled(sets, stm) == danger;
      const int nr = gen_plan_rolled(p, sets, danger, stm, qs != 0, setr, &chkr, &sqepr);
      same = same && nr == nw && chkr == chk && sqepr == sqep;
      for (int e = 0; same && e < kEmitters; e++) same = setr[e] == set[e];
      for (int j = 0; same && j < nw; j++) same = gen_move_at_rolled(p, sets, stm, setr, off, sqep, j) == b[j];
      if (!same) {
        if (g_bad < 5) printf("warp generator differs (qs %d): %d vs %d moves\n", qs, nw, nb);
        g_bad++;
      }
    }
    std::sort(a, a + na);
    std::sort(b, b + nb);
    if (na != nb || !std::equal(a, a + na, b)) {
      if (g_bad < 5) printf("generators differ (qs %d): %d vs %d moves\n", qs, na, nb);
      g_bad++;
    }
  }
  /* all four promotions: the perft generator and its bulk count against
   * the oracle's all-promotions mode */
  for (int qs = 0; qs < 2; qs++) {
    Move a[256];
    zo_move o[256];
    const int na = gen_legal<true>(p, stm, qs != 0, a);
    const int no = zo_genmoves_ex(b7, stm, qs, 1, o);
    bool ck;
    std::sort(a, a + na);
    std::sort(o, o + no);
    if (na != no || !std::equal(a, a + na, o) || (!qs && count_legal_ex<true>(p, stm, ck) != na)) {
      if (g_bad < 5) printf("all-promotions generator differs (qs %d): %d vs %d moves\n", qs, na, no);
      g_bad++;
    }
  }
  const int psum = eval_piece_sum(p, kEvalHost);
  if (psum + eval_structure(p) != eval_white(p, kEvalHost)) {
    if (g_bad < 5) printf("piece terms + structure differ from the evaluation\n");
    g_bad++;
  }
  if (depth == 0) return;
  Move list[256];
  const int k = gen_legal(p, stm, false, list);
  const u64 th = compute_hash(p, stm);
  for (int i = 0; i < k; i++) {
    Pos q = p;
    play(q, list[i], false);
    if (psum + piece_sum_delta(list[i], kEvalHost) != eval_piece_sum(q, kEvalHost)) {
      if (g_bad < 5) printf("incremental piece terms differ after move %08x\n", list[i]);
      g_bad++;
    }
    const u64 inc = th ^ 1ULL ^ cr_keys(p.cr) ^ cr_keys(q.cr) ^ piece_delta(list[i]);
    if (inc != compute_hash(q, stm ^ 1)) {
      if (g_bad < 5) printf("incremental hash differs after move %08x\n", list[i]);
      g_bad++;
    }
    walk(q, stm ^ 1, depth - 1);
  }
}

int main(int argc, char **argv) {
  for (int r = 1; r < argc; r++) {
    unsigned long long v[7];
    char *s = argv[r];
    for (int i = 0; i < 7; i++) {
      v[i] = strtoull(s, &s, 0);
      if (*s == ':') s++;
    }
    const Pos p{v[0], v[1], v[2], v[3], v[4]};
    walk(p, (int)v[5], (int)v[6]);
    printf("root %d: %llu nodes, %llu decided by the quick test, %llu more by the king step, %llu disagreements\n", r,
           g_nodes, g_quick, g_king, g_bad);
  }
  return g_bad != 0;
}
