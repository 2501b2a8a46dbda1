/*
 * opcount.cc -- algorithmic integer operations per node of the perft
 * kernel, measured by running the kernel's own move-generation code
 * (chess.cuh) on the host with a counting 64-bit word.
 *
 * Counting rule (one u64 operation = two 32-bit instructions on the GPU):
 * and/or/xor/not/add/sub/compare 2, shift by a constant 2, shift by a
 * variable 4, popcount/count-trailing-zeros 2.  Branch, select and address
 * arithmetic are not counted.  The result is the roofline numerator of the
 * benchmark: achieved int32 ops/s = nodes/s x ops/node.
 *
 * Usage: opcount <out.json>   -- counts over the initial position's depth-5
 * tree and over the first 64 positions of the batched-perft workload.
 * Built and run by zeta_gb300/build.py on request (build_opcount()).
 */
#include <cstdint>
#include <cstdio>
#include <cstring>

namespace opc {
struct Counter {
  static inline unsigned long long ops = 0;
};
/* 64-bit word that counts its operations */
struct W {
  unsigned long long v;
  W() = default;
  constexpr W(unsigned long long x) : v(x) {}
  constexpr W(long long x) : v((unsigned long long)x) {}
  constexpr W(int x) : v((unsigned long long)(long long)x) {}
  constexpr W(unsigned x) : v(x) {}
  explicit operator bool() const { Counter::ops += 2; return v != 0; }
  explicit operator unsigned long long() const { return v; }
  W operator~() const { Counter::ops += 2; return W(~v); }
  W &operator&=(W b) { Counter::ops += 2; v &= b.v; return *this; }
  W &operator|=(W b) { Counter::ops += 2; v |= b.v; return *this; }
  W &operator^=(W b) { Counter::ops += 2; v ^= b.v; return *this; }
};
inline W operator&(W a, W b) { Counter::ops += 2; return W(a.v & b.v); }
inline W operator|(W a, W b) { Counter::ops += 2; return W(a.v | b.v); }
inline W operator^(W a, W b) { Counter::ops += 2; return W(a.v ^ b.v); }
inline W operator+(W a, W b) { Counter::ops += 2; return W(a.v + b.v); }
inline W operator-(W a, W b) { Counter::ops += 2; return W(a.v - b.v); }
inline W operator<<(W a, int s) { Counter::ops += 2; return W(a.v << s); }
inline W operator>>(W a, int s) { Counter::ops += 2; return W(a.v >> s); }
inline bool operator==(W a, W b) { Counter::ops += 2; return a.v == b.v; }
inline bool operator!=(W a, W b) { Counter::ops += 2; return a.v != b.v; }
}  // namespace opc

#define ZETA_WORD_TYPE ::opc::W
#define ZETA_OPS(n) (::opc::Counter::ops += (n))
#include "chess.cuh"
#include "eval.cuh"
#include "tables.cuh"

using namespace zeta;
using opc::Counter;

struct Tally {
  unsigned long long count_nodes = 0, count_ops = 0, gen_nodes = 0, gen_ops = 0;
};

/* The kernel's task walk: expand interior nodes, count the last ply.
 * make_ops: operations of the move that produced this node. */
static unsigned long long walk(const Pos &p, int stm, int depth, Tally &t, unsigned long long make_ops) {
  if (depth == 0) return 1;
  if (depth == 1) {
    unsigned long long before = Counter::ops;
    int n = count_legal(p, stm);
    t.count_ops += Counter::ops - before + make_ops;
    t.count_nodes++;
    return (unsigned long long)n;
  }
  Move list[256];
  unsigned long long before = Counter::ops;
  int n = gen_legal(p, stm, false, list);
  t.gen_ops += Counter::ops - before + make_ops;
  t.gen_nodes++;
  unsigned long long total = 0;
  for (int i = 0; i < n; i++) {
    Pos c = p;
    unsigned long long b = Counter::ops;
    play(c, list[i], true);
    total += walk(c, stm ^ 1, depth - 1, t, Counter::ops - b);
  }
  return total;
}

/* Search nodes: the per-node work of the fixed-depth search kernel --
 * make the move, hash the child; at the horizon test for a legal move
 * (mate / stalemate: the quick free-move test, then the count when it
 * cannot decide, as the search kernels do) and evaluate, elsewhere
 * generate the moves.  Walked
 * as plain alpha-beta (no table) so that the mix of horizon and interior
 * nodes is that of a searched tree.  The full engine's node also tests
 * for check, generates (captures only in quiescence) and evaluates at
 * every node: engine_ops adds that work for each visited node. */
struct STally {
  unsigned long long leaves = 0, leaf_ops = 0, interior = 0, int_ops = 0, engine_ops = 0, engine_nodes = 0;
};

static int sab(const Pos &p, int stm, int depth, int alpha, int beta, int ply, STally &t, unsigned long long make_ops) {
  unsigned long long before = Counter::ops;
  (void)compute_hash(p, stm);
  if (depth == 0) {
    bool chk = false;
    const bool n = has_legal_ex(p, stm, chk);
    int v = n ? (stm ? -eval_white(p, kEvalHost) : eval_white(p, kEvalHost)) : (chk ? -32000 + ply : 0);
    t.leaf_ops += Counter::ops - before + make_ops;
    t.leaves++;
    return v;
  }
  Move list[256];
  int n = gen_legal(p, stm, false, list);
  t.int_ops += Counter::ops - before + make_ops;
  t.interior++;
  if (!n) {
    bool chk = false;
    count_legal_ex(p, stm, chk);
    return chk ? -32000 + ply : 0;
  }
  for (int i = 0; i < n; i++) {
    Pos c = p;
    unsigned long long b = Counter::ops;
    play(c, list[i], false);
    int v = -sab(c, stm ^ 1, depth - 1, -beta, -alpha, ply + 1, t, Counter::ops - b);
    if (v > alpha) alpha = v;
    if (alpha >= beta) break;
  }
  return alpha;
}

/* the engine's node work on one position: in-check test, generation,
 * evaluation, hash and the make that led to it */
static unsigned long long engine_node_ops(const Pos &p, int stm, bool qs) {
  unsigned long long before = Counter::ops;
  const Sets s = make_sets(p, stm);
  (void)(enemy_attacks(s, stm) & s.kbb);
  Move list[256];
  (void)gen_legal(p, stm, qs, list);
  (void)eval_white(p, kEvalHost);
  (void)compute_hash(p, stm);
  return Counter::ops - before;
}

static unsigned long long splitmix(unsigned long long &s) {
  unsigned long long z = (s += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

int main(int argc, char **argv) {
  const char *out = argc > 1 ? argv[1] : "opcount.json";
  Tally a;
  unsigned long long leaves = walk(start_pos(), 0, 5, a, 0);
  if (leaves != 4865609ULL) {
    fprintf(stderr, "opcount: startpos depth 5 gave %llu leaves\n", leaves);
    return 1;
  }
  /* a sample of the batched-perft workload's kind of positions: seeded
   * random playouts of 10-60 plies, two plies deep from each */
  Tally b;
  unsigned long long s = 0x5A17A0000000003ULL;
  for (int i = 0; i < 64; i++) {
    Pos p = start_pos();
    int stm = 0, plies = 10 + (int)(splitmix(s) % 51);
    bool ok = true;
    for (int k = 0; k < plies && ok; k++) {
      Move list[256];
      int n = gen_legal(p, stm, false, list);
      if (!n) { ok = false; break; }
      play(p, list[splitmix(s) % (unsigned)n], true);
      stm ^= 1;
    }
    if (ok) walk(p, stm, 3, b, 0);
  }
  /* search nodes: 16 positions like the search workload (20-40 plies,
   * >= 20 pieces), depth 5 */
  STally st;
  unsigned long long ss = 0x5A17A0000000004ULL;
  int done = 0;
  while (done < 16) {
    Pos p = start_pos();
    int stm = 0, plies = 20 + (int)(splitmix(ss) % 21);
    bool ok = true;
    for (int k = 0; k < plies && ok; k++) {
      Move list[256];
      int n = gen_legal(p, stm, false, list);
      if (!n) { ok = false; break; }
      play(p, list[splitmix(ss) % (unsigned)n], false);
      stm ^= 1;
    }
    if (!ok || popc(p.p1 | p.p2 | p.p3) < 20) continue;
    Move list[256];
    if (!gen_legal(p, stm, false, list)) continue;
    sab(p, stm, 5, -32000, 32000, 0, st, 0);
    /* engine node work on the root and its children, the children
     * alternately as full-width and as quiescence nodes */
    int n = gen_legal(p, stm, false, list);
    st.engine_ops += engine_node_ops(p, stm, false);
    for (int i = 0; i < n; i++) {
      Pos c = p;
      unsigned long long b = Counter::ops;
      play(c, list[i], false);
      const unsigned long long mk = Counter::ops - b;
      st.engine_ops += engine_node_ops(c, stm ^ 1, (i & 1) != 0) + mk;
    }
    st.engine_nodes += (unsigned long long)n + 1;
    done++;
  }
  const double s_leaf = (double)st.leaf_ops / st.leaves, s_int = (double)st.int_ops / st.interior;
  const double s_node = (double)(st.leaf_ops + st.int_ops) / (double)(st.leaves + st.interior);
  const double e_node = (double)st.engine_ops / (double)st.engine_nodes;
  FILE *f = fopen(out, "w");
  if (!f) return 1;
  fprintf(f,
          "{\n \"rule\": \"u64 and/or/xor/not/add/sub/compare = 2, constant shift = 2, variable shift = 4, "
          "popc/ctz = 2 int32 ops; make-move counted with the node it feeds\",\n"
          " \"startpos_d5\": {\"counted_nodes\": %llu, \"ops_per_counted_node\": %.2f, \"interior_nodes\": %llu, "
          "\"ops_per_interior_node\": %.2f},\n"
          " \"workload_sample\": {\"positions\": 64, \"depth\": 3, \"counted_nodes\": %llu, "
          "\"ops_per_counted_node\": %.2f, \"interior_nodes\": %llu, \"ops_per_interior_node\": %.2f},\n"
          " \"ops_per_counted_node\": %.2f,\n \"ops_per_interior_node\": %.2f,\n"
          " \"search_sample\": {\"positions\": 16, \"depth\": 5, \"horizon_nodes\": %llu, \"ops_per_horizon_node\": %.2f, "
          "\"interior_nodes\": %llu, \"ops_per_interior_node\": %.2f},\n"
          " \"ops_per_search_node\": %.2f,\n \"ops_per_engine_node\": %.2f,\n"
          " \"search_rule\": \"search node = make + hash + (horizon: legal-move test (free-move test, count "
          "when undecided) + evaluation | interior: "
          "generation), averaged over a plain alpha-beta walk to depth 5 of 16 search-workload positions; engine "
          "node = make + in-check test + generation + evaluation + hash (move ordering and table work not "
          "counted)\"\n}\n",
          a.count_nodes, (double)a.count_ops / a.count_nodes, a.gen_nodes, (double)a.gen_ops / a.gen_nodes,
          b.count_nodes, (double)b.count_ops / b.count_nodes, b.gen_nodes, (double)b.gen_ops / b.gen_nodes,
          (double)a.count_ops / a.count_nodes, (double)a.gen_ops / a.gen_nodes, st.leaves, s_leaf, st.interior, s_int,
          s_node, e_node);
  fclose(f);
  printf("search node: %.1f ops (horizon %.1f, interior %.1f); engine node: %.1f ops\n", s_node, s_leaf, s_int, e_node);
  printf("counted node: %.1f ops (startpos d5 %.1f); interior node: %.1f ops\n", (double)b.count_ops / b.count_nodes,
         (double)a.count_ops / a.count_nodes, (double)b.gen_ops / b.gen_nodes);
  return 0;
}
