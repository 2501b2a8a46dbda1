/*
 * search.cu -- batched fixed-depth alpha-beta on GB300 ("pure" mode).
 *
 * The reference has no pure search: its alphabeta_gpu (zeta.cl:852-2512)
 * always runs quiescence, extensions, null move, LMR and IID.  This kernel
 * is the plain fixed-depth negamax the project defines for exact parity:
 * legal moves (queen-only promotions), the reference's evaluation at the
 * leaves from the side to move, mate = -INF+ply, stalemate = 0, no
 * quiescence, extensions, pruning or draw rules.  The root value equals
 * plain negamax exactly; alpha-beta, the transposition table and ABDADA
 * only change how much of the tree is visited.
 *
 * Layout and parallelism
 *  - A batch of N positions runs with W workers each; worker t works on
 *    position t % N, so the workers of one position sit in different warps
 *    (ABDADA across warps).  Three launch forms: dense (k_search_pure, one
 *    worker per thread: 32 positions per warp), sparse (k_search_pure, one
 *    worker per warp on lane 0) and warp-cooperative (k_search_warp, one
 *    worker per warp whose 32 lanes score the children of every node with
 *    one ply left).
 *  - Workers of a position share a 16-byte-entry transposition table in
 *    HBM (1 GiB by default, 2^26 entries, shared by the whole batch):
 *    {key ^ data, data}, data = move | score<<32 | depth<<48 | bound<<56,
 *    written and read as one 16-byte access; a torn entry fails the XOR
 *    check (the reference's lockless scheme, zeta.cl:1631,1891).  An entry
 *    is used only at exactly the same remaining depth, which keeps the
 *    result equal to plain negamax.
 *  - ABDADA (Weill 1996; the reference's variant is zeta.cl:1648-1782): a
 *    node of remaining depth >= 2 counts the workers inside it in a busy
 *    table; a worker asked to search a younger brother exclusively skips it
 *    while another worker is inside and comes back to it in a second pass.
 *  - The first worker to finish a root publishes score, best move and
 *    node counts; the others of that position see the flag and stop
 *    (the reference's early-bird `finito`, zeta.cl:1790-1792).
 *  - Every per-thread loop has a node budget; running out sets
 *    ZETA_ERR_BUDGET in the status word instead of spinning.
 */
#include <cstdio>
#include <cstring>
#include <vector>

#include "context.cuh"
#include "eval.cuh"
#include "movegen_fast.cuh"
#include "tables.cuh"
#include "warpgen.cuh"

namespace zeta {

namespace {

constexpr int kSearchInf = 32000;       /* INF, zeta.cl:131 */
constexpr int kMate = 30000;            /* MATESCORE */
constexpr int kOnEval = 32500;          /* "searched by another worker" */
constexpr int kMaxSearchDepth = 16;
constexpr int kMaxMoves = 218;
constexpr size_t kSearchStatusBytes = 24; /* status word, pad, table probes (u64), table stores (u64) */
constexpr int kAbdadaMinDepth = 2;
constexpr uint32_t kDone = 1u << 30;    /* move flags above the 30-bit packing */
constexpr uint32_t kDefer = 1u << 31;
constexpr uint32_t kMoveBits = (1u << 30) - 1;

constexpr uint32_t SST_BUDGET = 1u;

enum Bound : uint32_t { B_NONE = 0, B_LOWER = 1, B_UPPER = 2, B_EXACT = 3 };

/* exact castle rights and the en-passant square mixed into the reference
 * Zobrist hash: its castle keys depend on either of the king and rook
 * flags, which two positions with different rights can share */
__device__ __forceinline__ u64 search_key(const Pos &p, u64 hash) {
  u64 k = hash; /* the reference hash of (p, side to move) */
  u64 cr = ~p.cr;
  uint32_t rights = ((cr & ZETA_CR_WQ) == ZETA_CR_WQ) | (((cr & ZETA_CR_WK) == ZETA_CR_WK) << 1) |
                    (((cr & ZETA_CR_BQ) == ZETA_CR_BQ) << 2) | (((cr & ZETA_CR_BK) == ZETA_CR_BK) << 3);
  return k ^ ((u64)rights * 0x9E3779B97F4A7C15ULL);
}

struct TTEntry {
  unsigned long long kx, data;
};

__device__ __forceinline__ bool tt_probe(const TTEntry *tt, u64 mask, u64 key, int &score, int &depth, int &bound,
                                         Move &move) {
  const longlong2 e = __ldcg((const longlong2 *)&tt[key & mask]);
  const u64 kx = (u64)e.x, data = (u64)e.y;
  if ((kx ^ data) != key) return false;
  move = (Move)(data & 0xFFFFFFFFu);
  score = (int)(int16_t)((data >> 32) & 0xFFFF);
  depth = (int)((data >> 48) & 0xFF);
  bound = (int)(data >> 56);
  return true;
}

__device__ __forceinline__ void tt_store(TTEntry *tt, u64 mask, u64 key, int score, int depth, int bound, Move move) {
  u64 data = (u64)(move & kMoveBits) | ((u64)(uint16_t)(int16_t)score << 32) | ((u64)(depth & 0xFF) << 48) |
             ((u64)bound << 56);
  longlong2 e;
  e.x = (long long)(key ^ data);
  e.y = (long long)data;
  __stcg((longlong2 *)&tt[key & mask], e);
}

/* mate scores are kept relative to the node in the table */
__device__ __forceinline__ int to_tt(int s, int ply) { return s > kMate ? s + ply : (s < -kMate ? s - ply : s); }
__device__ __forceinline__ int from_tt(int s, int ply) { return s > kMate ? s - ply : (s < -kMate ? s + ply : s); }

/* Move ordering: TT move, captures by MVV-LVA, queen promotions, the two
 * killers of the ply, then quiet moves by piece-square gain -- the
 * reference's scheme (zeta.cl:2039-2110) without the counter-move and
 * randomisation terms. */
__device__ __forceinline__ int order_score(Move m, int stm, Move ttmove, Move k0, Move k1, const EvalTables &T) {
  if (m == ttmove) return 1 << 20;
  int pf = m_pfrom(m) >> 1, pt = m_pto(m) >> 1, pc = m_pcpt(m) >> 1;
  if (pc) return (1 << 18) + T.value[pc] * 16 - T.value[pt];
  if (pt != pf) return (1 << 17);
  if (m == k0) return (1 << 16) + 1;
  if (m == k1) return (1 << 16);
  int to = m_to(m), from = m_from(m);
  int vt = stm ? to : (to ^ 56), vf = stm ? from : (from ^ 56);
  return T.pst[pt][vt] + T.control[vt] - T.pst[pf][vf] - T.control[vf];
}

/* one ply of a worker's explicit stack */
struct Frame {
  Pos pos;
  u64 th; /* reference Zobrist hash of (pos, stm), updated move by move */
  u64 key;
  int alpha, beta, alpha0, best;
  Move bestmove;
  int n, i, iter, searched;
  int depth;
  uint8_t stm, exclusive, deferred, busy;
  Move moves[kMaxMoves];
};

struct SearchOut {
  int score;
  Move bestmove;
  unsigned long long nodes;
  unsigned long long tthits;
};


/* single out-of-line copies (instruction cache, as in perft.cu) */
__device__ __noinline__ int s_count(Pos p, int stm, bool *chk) {
  bool c;
  int n = count_legal_ex(p, stm, c);
  *chk = c;
  return n;
}
__device__ __noinline__ int s_gen(Pos p, int stm, Move *list) {
  const Sets s = make_sets(p, stm);
  return gen_engine(p, s, enemy_attacks(s, stm), stm, false, list);
}
__device__ __noinline__ int s_eval(Pos p, const EvalTables *T) { return eval_white(p, *T); }
/* whether the side to move has a legal move, and whether it is in check:
 * the quick test, then the exact count when it cannot decide */
__device__ __noinline__ bool s_has_move(Pos p, int stm, bool *chk) {
  bool c;
  if (has_free_move(p, stm, c)) {
    *chk = c;
    return true;
  }
  return s_count(p, stm, chk) > 0;
}

/* value of a node with no depth left, from the side to move */
__device__ __forceinline__ int leaf_value(const Pos &p, int stm, int ply, const EvalTables *T) {
  bool chk;
  if (!s_has_move(p, stm, &chk)) return chk ? -kSearchInf + ply : 0;
  int e = s_eval(p, T);
  return stm ? -e : e;
}

struct Worker {
  TTEntry *tt;
  u64 tt_mask;
  uint32_t *busy;
  u64 busy_mask;
  const EvalTables *T;
  unsigned long long nodes, tthits;
  unsigned long long probes, stores; /* table operations over the worker's life */
  Move killer[kMaxSearchDepth + 1][2];
  int scores[kMaxMoves];
  /* learned ordering */
  int learned, learned_top, learned_quiet;
  OrderEntry *ocache;
  u64 ocache_mask;
  OrderRequest *oreq;
  uint32_t *noreq;
  uint32_t oreq_cap;
};

struct LearnArgs {
  int learned;
  int top;   /* how many of the network's best moves are used */
  int quiet; /* 0: they go right after the TT move; 1: they order the quiet moves only */
  OrderEntry *cache;
  u64 mask;
  OrderRequest *req;
  uint32_t *nreq;
  uint32_t cap;
};

/* rank of move m in a cached network ordering, or -1 */
__device__ __forceinline__ int learned_rank(const uint16_t *mv, Move m) {
  const uint16_t k = (uint16_t)(m_from(m) | (m_to(m) << 6));
#pragma unroll
  for (int r = 0; r < kOrderTop; r++)
    if (mv[r] == k) return r;
  return -1;
}

/* Set up frame f at `ply`; false when the node is decided on entry (TT
 * hit, busy elsewhere, no legal move), with its value in `value` (kOnEval
 * for an exclusive request on a busy node). */
__device__ bool node_enter(Worker &W, Frame &f, int ply, int &value) {
  W.nodes++;
  f.key = search_key(f.pos, f.th);
  Move ttm = 0;
  int ts, td, tb;
  Move tm;
  W.probes++;
  if (tt_probe(W.tt, W.tt_mask, f.key, ts, td, tb, tm)) {
    ttm = tm; /* a move from any depth orders; only an equal depth cuts */
    if (td == f.depth) {
      int s = from_tt(ts, ply);
      if (ply > 0 && (tb == B_EXACT || (tb == B_LOWER && s >= f.beta) || (tb == B_UPPER && s <= f.alpha))) {
        W.tthits++;
        value = s;
        return false;
      }
    }
  }
  const u64 bidx = (f.key >> 32) & W.busy_mask;
  if (f.exclusive && f.depth >= kAbdadaMinDepth && ((volatile uint32_t *)W.busy)[bidx] > 0) {
    value = kOnEval;
    return false;
  }
  f.n = s_gen(f.pos, f.stm, f.moves);
  if (f.n == 0) {
    bool chk;
    s_count(f.pos, f.stm, &chk);
    value = chk ? -kSearchInf + ply : 0;
    return false;
  }
  /* the network's ordering at nodes with >= 3 plies left: from the cache,
   * or requested for the next kernel step from nodes with >= 2 left */
  uint16_t lmv[kOrderTop];
  bool have_l = false;
  if (W.learned && f.depth >= 2) {
    OrderEntry *e = &W.ocache[f.key & W.ocache_mask];
    const unsigned long long ek = ((volatile unsigned long long *)&e->key)[0];
    if (ek == f.key) {
      if (f.depth >= 3) {
#pragma unroll
        for (int r = 0; r < kOrderTop; r++) lmv[r] = e->mv[r];
        have_l = true;
      }
    } else {
      const uint32_t idx = atomicAdd(W.noreq, 1u);
      if (idx < W.oreq_cap) {
        OrderRequest q;
        q.key = f.key;
        q.b[0] = f.pos.b0;
        q.b[1] = f.pos.p1;
        q.b[2] = f.pos.p2;
        q.b[3] = f.pos.p3;
        q.b[4] = f.pos.cr;
        q.stm = f.stm;
        q.pad = 0;
        W.oreq[idx] = q;
        /* mark as requested so other workers do not ask again */
        OrderEntry pend;
        pend.key = f.key;
#pragma unroll
        for (int r = 0; r < kOrderTop; r++) pend.mv[r] = 0xFFFF;
        *e = pend;
      }
    }
  }
  /* order once: insertion sort by score, best first */
  const Move k0 = W.killer[ply][0], k1 = W.killer[ply][1];
  for (int i = 0; i < f.n; i++) {
    Move m = f.moves[i];
    int s = order_score(m, f.stm, ttm, k0, k1, *W.T);
    if (have_l && m != ttm) {
      const int r = learned_rank(lmv, m);
      if (r >= 0 && r < W.learned_top) {
        if (!W.learned_quiet)
          s = (1 << 19) - r;
        else if (s < (1 << 16))
          s = (1 << 15) - r; /* below captures, promotions and killers */
      }
    }
    int j = i;
    while (j > 0 && W.scores[j - 1] < s) {
      W.scores[j] = W.scores[j - 1];
      f.moves[j] = f.moves[j - 1];
      j--;
    }
    W.scores[j] = s;
    f.moves[j] = m;
  }
  f.busy = f.depth >= kAbdadaMinDepth;
  if (f.busy) atomicAdd(&W.busy[bidx], 1u);
  f.best = -kSearchInf - 1;
  f.bestmove = 0;
  f.alpha0 = f.alpha;
  f.i = f.iter = f.searched = 0;
  f.deferred = 0;
  return true;
}

/* all moves searched or cut: store and return the value */
__device__ __forceinline__ int node_finish(Worker &W, Frame &f, int ply) {
  if (f.busy) atomicSub(&W.busy[(f.key >> 32) & W.busy_mask], 1u);
  int bound = f.best <= f.alpha0 ? B_UPPER : (f.best >= f.beta ? B_LOWER : B_EXACT);
  W.stores++;
  tt_store(W.tt, W.tt_mask, f.key, to_tt(f.best, ply), f.depth, bound, f.bestmove);
  return f.best;
}

template <int TPB>
__global__ void __launch_bounds__(TPB) k_search_pure(const uint64_t *__restrict__ boards, const uint8_t *__restrict__ stm,
                                                     int N, int nworkers, int depth, TTEntry *tt, u64 tt_mask,
                                                     uint32_t *busy, u64 busy_mask, uint32_t *done, SearchOut *out,
                                                     unsigned long long budget, uint32_t *status, uint32_t *active,
                                                     int max_per_pos, LearnArgs la, int sparse,
                                                     unsigned long long *ttops) {
  __shared__ EvalTables sT;
  for (int i = threadIdx.x; i < (int)(sizeof(EvalTables) / 4); i += TPB)
    ((uint32_t *)&sT)[i] = ((const uint32_t *)&kEvalDev)[i];
  __syncthreads();
  /* dense: one worker per thread; sparse: one worker per warp (lane 0),
   * when every worker fits on the GPU with a warp of its own */
  long long t = (long long)blockIdx.x * TPB + threadIdx.x;
  if (sparse) {
    if (threadIdx.x & 31) return;
    t >>= 5;
  }
  if (t >= (long long)N * nworkers) return;
  int p = (int)(t % N);

  Frame F[kMaxSearchDepth + 1];
  Worker W;
  W.tt = tt;
  W.tt_mask = tt_mask;
  W.busy = busy;
  W.busy_mask = busy_mask;
  W.T = &sT;
  W.learned = la.learned;
  W.learned_top = la.top;
  W.learned_quiet = la.quiet;
  W.ocache = la.cache;
  W.ocache_mask = la.mask;
  W.oreq = la.req;
  W.noreq = la.nreq;
  W.oreq_cap = la.cap;
  W.probes = W.stores = 0;
  unsigned long long steps = 0;

  /* A worker searches its own position, then helps unfinished ones: it
   * joins them as one more ABDADA worker from their root, so the largest
   * trees of the batch end up with every thread of the grid. */
  for (int job = 0;; job++) {
    if (job > 0) {
      if (max_per_pos <= nworkers) break; /* helping disabled */
      const unsigned h = (unsigned)(t * 0x9E3779B1u + (unsigned)job * 0x85EBCA6Bu);
      int q = -1;
      for (int k = 0; k < N; k++) {
        int c = (int)((h + (unsigned)k) % (unsigned)N);
        if (((volatile uint32_t *)done)[c]) continue;
        if (atomicAdd(&active[c], 1u) < (unsigned)max_per_pos) {
          q = c;
          break;
        }
        atomicSub(&active[c], 1u);
      }
      if (q < 0) break;
      p = q;
    } else {
      atomicAdd(&active[p], 1u);
    }
    W.nodes = W.tthits = 0;
    for (int i = 0; i <= kMaxSearchDepth; i++) W.killer[i][0] = W.killer[i][1] = 0;
    const uint64_t *b = boards + 7 * (size_t)p;
    F[0].pos.b0 = b[0];
    F[0].pos.p1 = b[1];
    F[0].pos.p2 = b[2];
    F[0].pos.p3 = b[3];
    F[0].pos.cr = b[4];
    F[0].th = compute_hash(F[0].pos, stm[p] & 1);
    F[0].stm = stm[p] & 1;
    F[0].depth = depth;
    F[0].alpha = -kSearchInf - 1;
    F[0].beta = kSearchInf + 1;
    F[0].exclusive = 0;
    int v;
    if (!node_enter(W, F[0], 0, v)) {
      /* no legal move at the root: the game is over */
      if (atomicCAS(&done[p], 0u, 1u) == 0u) {
        out[p].score = v;
        out[p].bestmove = 0;
      }
      atomicAdd(&out[p].nodes, W.nodes);
      atomicSub(&active[p], 1u);
      continue;
    }
    int ply = 0;
    for (;;) {
    if (++steps > budget) {
      atomicOr(status, SST_BUDGET);
      return;
    }
    if ((steps & 15) == 0 && ((volatile uint32_t *)done)[p]) break; /* another worker finished */
    Frame &f = F[ply];
    int val = 0;
    bool deferred = false;
    /* next move of this node: skip searched ones, and in the second pass
     * everything that was not deferred */
    while (f.i < f.n && ((f.moves[f.i] & kDone) || (f.iter == 1 && !(f.moves[f.i] & kDefer)))) f.i++;
    if (f.i >= f.n) {
      if (f.iter == 0 && f.deferred) {
        f.iter = 1;
        f.i = 0;
        f.deferred = 0;
        continue;
      }
      int r = node_finish(W, f, ply);
      if (ply == 0) {
        if (atomicCAS(&done[p], 0u, 1u) == 0u) {
          out[p].score = r;
          out[p].bestmove = f.bestmove;
        }
        break;
      }
      ply--;
      val = -r;
    } else {
      const Move m = f.moves[f.i] & kMoveBits;
      Pos c = f.pos;
      play(c, m, false);
      if (f.depth == 1) {
        W.nodes++;
        val = -leaf_value(c, f.stm ^ 1, ply + 1, W.T);
      } else {
        Frame &g = F[ply + 1];
        g.pos = c;
        g.th = f.th ^ 1ULL ^ cr_keys(f.pos.cr) ^ cr_keys(c.cr) ^ piece_delta(m);
        g.stm = f.stm ^ 1;
        g.depth = f.depth - 1;
        g.alpha = -f.beta;
        g.beta = -(f.alpha > f.best ? f.alpha : f.best);
        g.exclusive = (f.iter == 0 && f.searched > 0);
        int cv;
        if (node_enter(W, g, ply + 1, cv)) {
          ply++;
          continue;
        }
        if (cv == kOnEval) deferred = true;
        else val = -cv;
      }
    }
    /* a child of F[ply] returned `val` (or was deferred) */
    Frame &h = F[ply];
    if (deferred) {
      h.moves[h.i] |= kDefer;
      h.deferred = 1;
      h.i++;
      continue;
    }
    const Move m = h.moves[h.i] & kMoveBits;
    h.moves[h.i] = (h.moves[h.i] & kMoveBits) | kDone;
    h.i++;
    h.searched++;
    if (val > h.best) {
      h.best = val;
      h.bestmove = m;
    }
    if (h.best > h.alpha) h.alpha = h.best;
    if (h.best >= h.beta) {
      if (!(m_pcpt(m) >> 1) && (m_pto(m) == m_pfrom(m)) && W.killer[ply][0] != m) {
        W.killer[ply][1] = W.killer[ply][0];
        W.killer[ply][0] = m;
      }
      h.i = h.n; /* cut: nothing else to search here */
      h.deferred = 0;
    }
    }
    atomicAdd(&out[p].nodes, W.nodes);
    atomicAdd(&out[p].tthits, W.tthits);
    atomicSub(&active[p], 1u);
  }
  atomicAdd(ttops, W.probes);
  atomicAdd(ttops + 1, W.stores);
}

/* Hand-off from a warp's tree walker (lane 0) to all 32 lanes: a node with
 * one ply left, and after its moves are generated, its legal moves (in
 * shared memory). */
struct LeafBatch {
  Pos pos;
  int n, ply, beta;
  uint32_t stm;
  int psum; /* eval_piece_sum of pos (carried down the walk): each leaf adds its move's change */
  Move moves[kMaxMoves];
};

/* Hand-off for generating and ordering the moves of an interior node:
 * lane 0 puts the position and what orders its moves here; the warp
 * builds the list (warpgen.cuh), scores it and writes it, best first, to
 * the node's move array. */
struct WarpGen {
  Pos pos;
  uint32_t stm;
  Move ttm, k0, k1;
  int have_l;
  uint16_t lmv[kOrderTop];
  int n, chk;
  u64 set[kEmitters];
  uint8_t off[kEmitters + 1];
  int sc[kMaxMoves];
  Move mv[kMaxMoves];
  Move srt[kMaxMoves]; /* the ordered list, best first */
};

constexpr unsigned kFull = 0xFFFFFFFFu;

/* The warp kernel's generator in its rolled form (warpgen.cuh), one
 * out-of-line copy each: the piece sets, the enemy attack map and the 23
 * emitter sets of (pos, stm) -- returns the number of legal moves -- and
 * move j of the list. */
__device__ __noinline__ int w_plan(const Pos &pos, int stm, bool qs, u64 *set, bool *chk, int *sqep, Sets *sets) {
  const Sets s = make_sets(pos, stm);
  *sets = s;
  return gen_plan_rolled(pos, s, enemy_attacks_rolled(s, stm), stm, qs, set, chk, sqep);
}
__device__ __noinline__ Move w_move_at(const Pos &p, const Sets &s, int stm, const u64 *set, const uint8_t *off,
                                       int sqep, int j) {
  return gen_move_at_rolled(p, s, stm, set, off, sqep, j);
}

/* the legal moves of n positions, one warp each, with the warp-cooperative
 * search's generator -- the same plan and per-lane decode as warp_plan and
 * warp_gen_order (test entry: the list must equal gen_engine's, in the
 * same order) */
__global__ void k_genmoves_warp(const uint64_t *__restrict__ boards, const uint8_t *__restrict__ stm, int n, int qs,
                                uint32_t *__restrict__ moves, int32_t *__restrict__ counts) {
  __shared__ u64 wset[4][kEmitters];
  __shared__ uint8_t woff[4][kEmitters + 1];
  const int lane = threadIdx.x & 31, wi = threadIdx.x >> 5;
  const int i = blockIdx.x * 4 + wi;
  if (i >= n) return; /* whole warps */
  const uint64_t *b = boards + 7 * (size_t)i;
  Pos p;
  p.b0 = b[0];
  p.p1 = b[1];
  p.p2 = b[2];
  p.p3 = b[3];
  p.cr = b[4];
  const int side = stm[i] & 1;
  Sets s;
  bool chk;
  int sqep;
  int cnt = w_plan(p, side, qs != 0, wset[wi], &chk, &sqep, &s);
  __syncwarp();
  int c = lane < kEmitters ? popc(wset[wi][lane]) : 0;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xFFFFFFFFu, c, o);
    if (lane >= o) c += y;
  }
  if (lane < kEmitters) woff[wi][lane + 1] = (uint8_t)min(c, 255);
  if (lane == 0) woff[wi][0] = 0;
  __syncwarp();
  cnt = cnt < 256 ? cnt : 256;
  for (int j = lane; j < cnt; j += 32) moves[(size_t)i * 256 + j] = w_move_at(p, s, side, wset[wi], woff[wi], sqep, j);
  if (lane == 0) counts[i] = cnt;
}

/* whether the side to move has a legal move, and whether it is in check:
 * the quick free-move and king-step tests, then the legal-move count of
 * w_plan (the generator's own code, so the leaf test adds no second copy
 * of it).  The count is needed for well under 1% of the leaves: a warp
 * whose lanes all decide quickly skips it. */
__device__ __noinline__ bool w_has_move(const Pos &p, int stm, bool *chk) {
  bool c;
  if (has_quick_move_rolled(p, stm, c)) {
    *chk = c;
    return true;
  }
  u64 set[kEmitters];
  int sqep;
  Sets s;
  const int n = w_plan(p, stm, false, set, chk, &sqep, &s);
  return n > 0;
}

/* value of a node with no depth left, from the side to move; psum: its
 * piece terms (eval.cuh, incremental form) */
__device__ __forceinline__ int leaf_value_w(const Pos &p, int stm, int ply, int psum) {
  bool chk;
  if (!w_has_move(p, stm, &chk)) return chk ? -kSearchInf + ply : 0;
  const int e = psum + eval_structure(p);
  return stm ? -e : e;
}

/* one ply of a warp worker's stack (lane 0's local memory: its move
 * flags are written at every visited child, and local memory is cached
 * write-back) */
struct WFrame {
  Pos pos;
  u64 th;
  u64 key;
  int alpha, beta, alpha0, best;
  Move bestmove;
  int n, i, iter, searched;
  int depth;
  uint8_t stm, exclusive, deferred, busy;
  int psum; /* eval_piece_sum of pos (eval.cuh, incremental form) */
  Move moves[kMaxMoves];
};

/* All lanes: the 23 emitter sets of (pos, stm) and their prefix counts into
 * G; returns the number of legal moves (at most kMaxMoves).  Every lane
 * computes the same sets (no lane-dependent branch) and writes the same
 * values to G.set.  One out-of-line copy: the kernel calls it from two
 * places, and the instruction cache is the search kernels' tightest
 * resource. */
__device__ __noinline__ int warp_plan(WarpGen &G, const Pos &pos, int stm, Sets &s, int &sqep, int lane) {
  bool chk = false;
  int n = w_plan(pos, stm, false, G.set, &chk, &sqep, &s);
  __syncwarp();
  int c = lane < kEmitters ? popc(G.set[lane]) : 0;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(kFull, c, o);
    if (lane >= o) c += y;
  }
  if (lane < kEmitters) G.off[lane + 1] = (uint8_t)min(c, 255);
  if (lane == 0) {
    G.off[0] = 0;
    G.chk = chk;
  }
  __syncwarp();
  return n < kMaxMoves ? n : kMaxMoves; /* a legal position has at most 218 */
}

/* All lanes: the moves of G.pos scored as node_enter orders them (table
 * move, captures by MVV-LVA, promotions, killers, learned ranks, then
 * piece-square gain) and written to G.srt best first -- a stable sort,
 * the same order as node_enter's insertion sort: move j goes to the number
 * of moves with a higher score, or an equal score and a smaller index. */
__device__ __forceinline__ int warp_gen_order(WarpGen &G, const EvalTables &T, int learned_top, int learned_quiet,
                                              int lane) {
  Sets s;
  int sqep = 0;
  const Pos pos = G.pos;
  const int stm = G.stm;
  const int n = warp_plan(G, pos, stm, s, sqep, lane);
  const Move ttm = G.ttm, k0 = G.k0, k1 = G.k1;
  const int have_l = G.have_l;
  for (int j = lane; j < n; j += 32) {
    const Move m = w_move_at(pos, s, stm, G.set, G.off, sqep, j);
    int sc = order_score(m, stm, ttm, k0, k1, T);
    if (have_l && m != ttm) {
      const int r = learned_rank(G.lmv, m);
      if (r >= 0 && r < learned_top) {
        if (!learned_quiet)
          sc = (1 << 19) - r;
        else if (sc < (1 << 16))
          sc = (1 << 15) - r; /* below captures, promotions and killers */
      }
    }
    G.sc[j] = sc;
    G.mv[j] = m;
  }
  __syncwarp();
  for (int j = lane; j < n; j += 32) {
    const int sj = G.sc[j];
    int r = 0;
    for (int i = 0; i < n; i++) {
      const int si = G.sc[i];
      r += (si > sj) || (si == sj && i < j);
    }
    G.srt[r] = G.mv[j];
  }
  if (lane == 0) G.n = n;
  __syncwarp(); /* the list and G.n are visible to lane 0 */
  return n;
}

/* All lanes: the legal moves of B.pos into B.moves, captures and
 * promotions first when they take more than one scoring round (each group
 * in generation order). */
__device__ __forceinline__ int warp_gen_batch(WarpGen &G, LeafBatch &B, int lane) {
  Sets s;
  int sqep = 0;
  const Pos pos = B.pos;
  const int stm = B.stm;
  const int n = warp_plan(G, pos, stm, s, sqep, lane);

  if (n <= 32) {
    if (lane < n) B.moves[lane] = w_move_at(pos, s, stm, G.set, G.off, sqep, lane);
  } else {
    int ncap = 0;
    for (int base = 0; base < n; base += 32) {
      const int j = base + lane;
      bool cap = false;
      if (j < n) {
        const Move m = w_move_at(pos, s, stm, G.set, G.off, sqep, j);
        cap = (m_pcpt(m) >> 1) || m_pto(m) != m_pfrom(m);
        G.mv[j] = m;
      }
      ncap += __popc(__ballot_sync(kFull, cap));
    }
    __syncwarp();
    const unsigned lt = (1u << lane) - 1u;
    int ci = 0, qi = ncap;
    for (int base = 0; base < n; base += 32) {
      const int j = base + lane;
      const Move m = j < n ? G.mv[j] : 0u;
      const bool cap = j < n && ((m_pcpt(m) >> 1) || m_pto(m) != m_pfrom(m));
      const unsigned bc = __ballot_sync(kFull, cap), bq = __ballot_sync(kFull, j < n && !cap);
      if (j < n) B.moves[cap ? ci + __popc(bc & lt) : qi + __popc(bq & lt)] = m;
      ci += __popc(bc);
      qi += __popc(bq);
    }
  }
  if (lane == 0) B.n = n;
  __syncwarp();
  return n;
}

/* lane 0: node entry up to move generation -- table probe (a move from any
 * depth orders, only an equal depth cuts), the ABDADA busy check, the
 * learned-ordering lookup or request.  false: decided here (`value`;
 * kOnEval for a busy node asked exclusively).  true: the moves must be
 * generated; the request is in G. */
__device__ bool wnode_pre(Worker &W, WFrame &f, int ply, int &value, WarpGen &G) {
  W.nodes++;
  f.key = search_key(f.pos, f.th);
  Move ttm = 0;
  int ts, td, tb;
  Move tm;
  W.probes++;
  if (tt_probe(W.tt, W.tt_mask, f.key, ts, td, tb, tm)) {
    ttm = tm;
    if (td == f.depth) {
      const int s = from_tt(ts, ply);
      if (ply > 0 && (tb == B_EXACT || (tb == B_LOWER && s >= f.beta) || (tb == B_UPPER && s <= f.alpha))) {
        W.tthits++;
        value = s;
        return false;
      }
    }
  }
  const u64 bidx = (f.key >> 32) & W.busy_mask;
  if (f.exclusive && f.depth >= kAbdadaMinDepth && ((volatile uint32_t *)W.busy)[bidx] > 0) {
    value = kOnEval;
    return false;
  }
  G.have_l = 0;
  if (W.learned && f.depth >= 2) {
    OrderEntry *e = &W.ocache[f.key & W.ocache_mask];
    const unsigned long long ek = ((volatile unsigned long long *)&e->key)[0];
    if (ek == f.key) {
      if (f.depth >= 3) {
#pragma unroll
        for (int r = 0; r < kOrderTop; r++) G.lmv[r] = e->mv[r];
        G.have_l = 1;
      }
    } else {
      const uint32_t idx = atomicAdd(W.noreq, 1u);
      if (idx < W.oreq_cap) {
        OrderRequest q;
        q.key = f.key;
        q.b[0] = f.pos.b0;
        q.b[1] = f.pos.p1;
        q.b[2] = f.pos.p2;
        q.b[3] = f.pos.p3;
        q.b[4] = f.pos.cr;
        q.stm = f.stm;
        q.pad = 0;
        W.oreq[idx] = q;
        OrderEntry pend;
        pend.key = f.key;
#pragma unroll
        for (int r = 0; r < kOrderTop; r++) pend.mv[r] = 0xFFFF;
        *e = pend;
      }
    }
  }
  G.pos = f.pos;
  G.stm = f.stm;
  G.ttm = ttm;
  G.k0 = W.killer[ply][0];
  G.k1 = W.killer[ply][1];
  return true;
}

/* lane 0: node entry after the warp generated and ordered n moves.  false:
 * no legal move (`value` = mate or stalemate score). */
__device__ bool wnode_post(Worker &W, WFrame &f, int ply, const Move *srt, int n, bool chk, int &value) {
  f.n = n;
  for (int i = 0; i < n; i++) f.moves[i] = srt[i];
  if (n == 0) {
    value = chk ? -kSearchInf + ply : 0;
    return false;
  }
  f.busy = f.depth >= kAbdadaMinDepth;
  if (f.busy) atomicAdd(&W.busy[(f.key >> 32) & W.busy_mask], 1u);
  f.best = -kSearchInf - 1;
  f.bestmove = 0;
  f.alpha0 = f.alpha;
  f.i = f.iter = f.searched = 0;
  f.deferred = 0;
  return true;
}

__device__ __forceinline__ int wnode_finish(Worker &W, WFrame &f, int ply) {
  if (f.busy) atomicSub(&W.busy[(f.key >> 32) & W.busy_mask], 1u);
  const int bound = f.best <= f.alpha0 ? B_UPPER : (f.best >= f.beta ? B_LOWER : B_EXACT);
  W.stores++;
  tt_store(W.tt, W.tt_mask, f.key, to_tt(f.best, ply), f.depth, bound, f.bestmove);
  return f.best;
}

/* Warp-cooperative form: one warp is one ABDADA worker.  Lane 0 walks the
 * tree with the control flow of k_search_pure (same ordering, table,
 * ABDADA, killers, learned ordering); all 32 lanes do the per-node work:
 *  - at a node with two or more plies left, the warp generates the legal
 *    moves (warpgen.cuh), scores them and sorts them into the node's move
 *    array -- the same list, in the same order, as k_search_pure's;
 *  - at a node with one ply left, the warp generates its moves and then
 *    plays and scores the children, 32 per round (lane i takes move r*32+i
 *    in round r), with a warp reduction after each round.  A round whose
 *    best value reaches the node's beta ends the node with that lower
 *    bound; a node whose moves were all scored has its exact value.
 *    Either is stored in the table as such, so only the number of leaves
 *    visited changes and the root value is plain negamax.
 * Lane 0 hands work to the warp with a command: 2 generate and order the
 * moves of the node in G (lane 0 then copies the list into its frame), 3
 * generate and score the batch in B, 0 stop. */
template <int TPB>
__global__ void __launch_bounds__(TPB, 4) k_search_warp(const uint64_t *__restrict__ boards, const uint8_t *__restrict__ stm,
                                                     int N, int nworkers, int depth, TTEntry *tt, u64 tt_mask,
                                                     uint32_t *busy, u64 busy_mask, uint32_t *done, SearchOut *out,
                                                     unsigned long long budget, uint32_t *status, uint32_t *active,
                                                     int max_per_pos, LearnArgs la, unsigned long long *ttops) {
  __shared__ EvalTables sT;
  __shared__ LeafBatch LB[TPB / 32];
  __shared__ WarpGen WG[TPB / 32];
  for (int i = threadIdx.x; i < (int)(sizeof(EvalTables) / 4); i += TPB)
    ((uint32_t *)&sT)[i] = ((const uint32_t *)&kEvalDev)[i];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const long long t = ((long long)blockIdx.x * TPB + threadIdx.x) >> 5; /* worker = warp */
  if (t >= (long long)N * nworkers) return;                              /* whole warps leave */
  LeafBatch &B = LB[threadIdx.x >> 5];
  WarpGen &G = WG[threadIdx.x >> 5];

  WFrame F[kMaxSearchDepth + 1]; /* lane 0's stack; the other lanes never touch theirs */
  Worker W;
  W.tt = tt;
  W.tt_mask = tt_mask;
  W.busy = busy;
  W.busy_mask = busy_mask;
  W.T = &sT;
  W.learned = la.learned;
  W.learned_top = la.top;
  W.learned_quiet = la.quiet;
  W.ocache = la.cache;
  W.ocache_mask = la.mask;
  W.oreq = la.req;
  W.noreq = la.nreq;
  W.oreq_cap = la.cap;
  W.probes = W.stores = 0;
  unsigned long long steps = 0;
  int p = (int)(t % N), job = 0, ply = 0;
  int phase = 0; /* lane 0: 0 take a job, 1 walk, 2 take a batch's value, 3 finish a node entry */
  int pend = 0;  /* the batch is 1: the child F[ply + 1], 2: the root */
  int gq = 0;    /* phase 3: the frame whose moves the warp generated */
  int bval = 0, bidx = 0, bdone = 0;

  for (;;) {
    int cmd = 0; /* 0: the worker stops; 2: generate and order frame gq; 3: generate and score B */
    if (lane == 0) {
      for (;;) {
        if (++steps > budget) {
          atomicOr(status, SST_BUDGET);
          break;
        }
        int val = 0;
        bool deferred = false;
        if (phase == 0) {
          /* the worker's own position first, then unfinished ones, joining
           * them as one more ABDADA worker from their root */
          if (job > 0) {
            if (max_per_pos <= nworkers) break; /* helping disabled */
            const unsigned hsh = (unsigned)(t * 0x9E3779B1u + (unsigned)job * 0x85EBCA6Bu);
            int q = -1;
            for (int k = 0; k < N; k++) {
              int c = (int)((hsh + (unsigned)k) % (unsigned)N);
              if (((volatile uint32_t *)done)[c]) continue;
              if (atomicAdd(&active[c], 1u) < (unsigned)max_per_pos) {
                q = c;
                break;
              }
              atomicSub(&active[c], 1u);
            }
            if (q < 0) break;
            p = q;
          } else {
            atomicAdd(&active[p], 1u);
          }
          job++;
          W.nodes = W.tthits = 0;
          for (int i = 0; i <= kMaxSearchDepth; i++) W.killer[i][0] = W.killer[i][1] = 0;
          const uint64_t *b = boards + 7 * (size_t)p;
          F[0].pos.b0 = b[0];
          F[0].pos.p1 = b[1];
          F[0].pos.p2 = b[2];
          F[0].pos.p3 = b[3];
          F[0].pos.cr = b[4];
          F[0].th = compute_hash(F[0].pos, stm[p] & 1);
          F[0].psum = eval_piece_sum(F[0].pos, sT);
          F[0].stm = stm[p] & 1;
          F[0].depth = depth;
          F[0].alpha = -kSearchInf - 1;
          F[0].beta = kSearchInf + 1;
          F[0].exclusive = 0;
          if (depth == 1) {
            W.nodes++;
            F[0].key = search_key(F[0].pos, F[0].th);
            B.pos = F[0].pos;
            B.psum = F[0].psum;
            B.stm = F[0].stm;
            B.ply = 0;
            B.beta = kSearchInf + 1;
            pend = 2;
            phase = 2;
            cmd = 3;
            break;
          }
          int v = 0;
          if (wnode_pre(W, F[0], 0, v, G)) {
            gq = 0;
            phase = 3;
            cmd = 2;
            break;
          }
          /* the root is never cut or deferred on entry */
          atomicAdd(&out[p].nodes, W.nodes);
          atomicSub(&active[p], 1u);
          continue;
        }
        if (phase == 3) {
          /* the warp generated and ordered frame gq's moves */
          phase = 1;
          int v = 0;
          const bool open = wnode_post(W, F[gq], gq, G.srt, G.n, G.chk != 0, v);
          if (gq == 0) {
            if (!open) {
              /* no legal move at the root: the game is over */
              if (atomicCAS(&done[p], 0u, 1u) == 0u) {
                out[p].score = v;
                out[p].bestmove = 0;
              }
              atomicAdd(&out[p].nodes, W.nodes);
              atomicSub(&active[p], 1u);
              phase = 0;
            }
            ply = 0;
            continue;
          }
          if (open) {
            ply = gq;
            continue;
          }
          val = -v; /* a child with no legal move: falls through to its parent F[ply] */
        } else if (phase == 2) {
          /* the lanes scored every child of the batch node (or it has none) */
          phase = 1;
          W.nodes += bdone;
          if (B.n == 0) {
            const int mate = G.chk ? -kSearchInf + B.ply : 0;
            if (pend == 2) {
              if (atomicCAS(&done[p], 0u, 1u) == 0u) {
                out[p].score = mate;
                out[p].bestmove = 0;
              }
              atomicAdd(&out[p].nodes, W.nodes);
              atomicSub(&active[p], 1u);
              phase = 0;
              continue;
            }
            val = -mate;
          } else {
            const Move bm = B.moves[bidx];
            if (pend == 2) {
              W.stores++;
              tt_store(W.tt, W.tt_mask, F[0].key, bval, 1, B_EXACT, bm);
              if (atomicCAS(&done[p], 0u, 1u) == 0u) {
                out[p].score = bval;
                out[p].bestmove = bm;
              }
              atomicAdd(&out[p].nodes, W.nodes);
              atomicAdd(&out[p].tthits, W.tthits);
              atomicSub(&active[p], 1u);
              phase = 0;
              continue;
            }
            W.stores++;
            tt_store(W.tt, W.tt_mask, F[ply + 1].key, to_tt(bval, ply + 1), 1, bdone == B.n ? B_EXACT : B_LOWER,
                     bm);
            val = -bval;
          }
        } else {
          if ((steps & 15) == 0 && ((volatile uint32_t *)done)[p]) {
            /* another worker finished this position */
            atomicAdd(&out[p].nodes, W.nodes);
            atomicAdd(&out[p].tthits, W.tthits);
            atomicSub(&active[p], 1u);
            phase = 0;
            continue;
          }
          WFrame &f = F[ply];
          while (f.i < f.n && ((f.moves[f.i] & kDone) || (f.iter == 1 && !(f.moves[f.i] & kDefer)))) f.i++;
          if (f.i >= f.n) {
            if (f.iter == 0 && f.deferred) {
              f.iter = 1;
              f.i = 0;
              f.deferred = 0;
              continue;
            }
            const int r = wnode_finish(W, f, ply);
            if (ply == 0) {
              if (atomicCAS(&done[p], 0u, 1u) == 0u) {
                out[p].score = r;
                out[p].bestmove = f.bestmove;
              }
              atomicAdd(&out[p].nodes, W.nodes);
              atomicAdd(&out[p].tthits, W.tthits);
              atomicSub(&active[p], 1u);
              phase = 0;
              continue;
            }
            ply--;
            val = -r;
          } else {
            const Move m = f.moves[f.i] & kMoveBits;
            WFrame &g = F[ply + 1];
            g.pos = f.pos;
            play(g.pos, m, false);
            g.th = f.th ^ 1ULL ^ cr_keys(f.pos.cr) ^ cr_keys(g.pos.cr) ^ piece_delta(m);
            g.psum = f.psum + piece_sum_delta(m, sT); /* the child's piece terms */
            g.stm = f.stm ^ 1;
            g.depth = f.depth - 1;
            g.alpha = -f.beta;
            g.beta = -(f.alpha > f.best ? f.alpha : f.best);
            g.exclusive = (f.iter == 0 && f.searched > 0);
            if (g.depth == 1) {
              /* one ply left: a table hit, or a batch for the warp */
              W.nodes++;
              g.key = search_key(g.pos, g.th);
              int ts, td, tb;
              Move tm;
              bool hit = false;
              W.probes++;
              if (tt_probe(W.tt, W.tt_mask, g.key, ts, td, tb, tm) && td == 1) {
                const int s = from_tt(ts, ply + 1);
                if (tb == B_EXACT || (tb == B_LOWER && s >= g.beta) || (tb == B_UPPER && s <= g.alpha)) {
                  W.tthits++;
                  val = -s;
                  hit = true;
                }
              }
              if (!hit) {
                B.pos = g.pos;
                B.psum = g.psum;
                B.stm = g.stm;
                B.ply = ply + 1;
                B.beta = g.beta;
                pend = 1;
                phase = 2;
                cmd = 3;
                break;
              }
            } else {
              int cv = 0;
              if (wnode_pre(W, g, ply + 1, cv, G)) {
                gq = ply + 1;
                phase = 3;
                cmd = 2;
                break;
              }
              if (cv == kOnEval) deferred = true;
              else val = -cv;
            }
          }
        }
        /* a child of F[ply] returned `val` (or was deferred) */
        WFrame &h = F[ply];
        if (deferred) {
          h.moves[h.i] |= kDefer;
          h.deferred = 1;
          h.i++;
          continue;
        }
        const Move m = h.moves[h.i] & kMoveBits;
        h.moves[h.i] = m | kDone;
        h.i++;
        h.searched++;
        if (val > h.best) {
          h.best = val;
          h.bestmove = m;
        }
        if (h.best > h.alpha) h.alpha = h.best;
        if (h.best >= h.beta) {
          if (!(m_pcpt(m) >> 1) && (m_pto(m) == m_pfrom(m)) && W.killer[ply][0] != m) {
            W.killer[ply][1] = W.killer[ply][0];
            W.killer[ply][0] = m;
          }
          h.i = h.n;
          h.deferred = 0;
        }
      }
    }
    cmd = __shfl_sync(kFull, cmd, 0);
    if (!cmd) break;
    __syncwarp(); /* lane 0's request in G or B is visible to the warp */
    if (cmd == 2) {
      warp_gen_order(G, sT, W.learned_top, W.learned_quiet, lane);
      continue;
    }
    /* cmd 3: generate the batch node's moves, then score its children */
    const int n = warp_gen_batch(G, B, lane);
    const int beta = B.beta;
    int best = -kSearchInf - 1, bi = 0, scored = 0;
    for (int base = 0; base < n; base += 32) {
      const int i = base + lane;
      if (i < n) {
        Pos c = B.pos;
        const Move m = B.moves[i];
        play(c, m, false);
        const int v = -leaf_value_w(c, B.stm ^ 1, B.ply + 1, B.psum + piece_sum_delta(m, sT));
        if (v > best) {
          best = v;
          bi = i;
        }
      }
      /* the best value so far, the first move in list order on ties;
       * every lane ends with the same pair */
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const int ov = __shfl_xor_sync(kFull, best, o);
        const int oi = __shfl_xor_sync(kFull, bi, o);
        if (ov > best || (ov == best && oi < bi)) {
          best = ov;
          bi = oi;
        }
      }
      scored = min(n, base + 32);
      if (best >= beta) break; /* warp-uniform: the node fails high */
    }
    bval = best;
    bidx = bi;
    bdone = scored;
    __syncwarp(); /* B is read by every lane before lane 0 writes it again */
  }
  if (lane == 0) {
    atomicAdd(ttops, W.probes);
    atomicAdd(ttops + 1, W.stores);
  }
}

/* the static evaluation (white's view) of n boards, for the parity test */
__global__ void k_eval(const uint64_t *__restrict__ boards, int n, int32_t *__restrict__ scores) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint64_t *b = boards + 7 * (size_t)i;
  Pos p;
  p.b0 = b[0];
  p.p1 = b[1];
  p.p2 = b[2];
  p.p3 = b[3];
  p.cr = b[4];
  scores[i] = eval_white(p, kEvalDev);
}

__global__ void k_search_scatter(const SearchOut *out, int n, int32_t *scores, uint32_t *moves,
                                 unsigned long long *nodes) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (scores) scores[i] = out[i].score;
  if (moves) moves[i] = out[i].bestmove;
  if (nodes) nodes[i] = out[i].nodes;
}

}  // namespace

/* search buffers: outputs per position, the ABDADA busy table, the
 * transposition table (zeta_init's tt1, else a 64 MiB table of our own) */
static int search_buffers(int n) {
  Context &c = ctx();
  if (n > c.s_cap) {
    cudaFree(c.s_out);
    cudaFree(c.s_done);
    c.s_out = nullptr;
    c.s_done = nullptr;
    c.s_cap = 0;
    ZCHECK(cudaMalloc(&c.s_out, (size_t)n * sizeof(SearchOut)));
    /* done flags, then active-worker counts */
    ZCHECK(cudaMalloc(&c.s_done, (size_t)2 * n * sizeof(uint32_t)));
    c.s_cap = n;
  }
  if (!c.s_busy) {
    c.s_busy_entries = 1ull << 22;
    ZCHECK(cudaMalloc(&c.s_busy, c.s_busy_entries * sizeof(uint32_t)));
  }
  /* status word, then (8-byte aligned) the table probes and stores */
  if (!c.s_status) ZCHECK(cudaMalloc(&c.s_status, kSearchStatusBytes));
  if (!c.tt1 && !c.s_tt) {
    c.s_tt_entries = 1ull << 22; /* 64 MiB of 16-byte entries */
    ZCHECK(cudaMalloc(&c.s_tt, c.s_tt_entries * sizeof(TTEntry)));
    ZCHECK(cudaMemset(c.s_tt, 0, c.s_tt_entries * sizeof(TTEntry)));
  }
  return ZETA_OK;
}

int warp_genmoves_launch(const uint64_t *d_boards, const uint8_t *d_stm, int n, int qs, uint32_t *d_moves,
                         int32_t *d_counts, cudaStream_t s) {
  k_genmoves_warp<<<(n + 3) / 4, 128, 0, s>>>(d_boards, d_stm, n, qs, d_moves, d_counts);
  ZCHECK(cudaGetLastError());
  ZCHECK(cudaStreamSynchronize(s));
  return ZETA_OK;
}

int eval_launch(const uint64_t *d_boards, int n, int32_t *d_scores, cudaStream_t s) {
  k_eval<<<(n + 127) / 128, 128, 0, s>>>(d_boards, n, d_scores);
  ZCHECK(cudaGetLastError());
  ZCHECK(cudaStreamSynchronize(s));
  return ZETA_OK;
}

int search_tt_clear(cudaStream_t s) {
  Context &c = ctx();
  if (c.tt1) ZCHECK(cudaMemsetAsync(c.tt1, 0, c.tt1_entries * 16, s));
  if (c.s_tt) ZCHECK(cudaMemsetAsync(c.s_tt, 0, c.s_tt_entries * sizeof(TTEntry), s));
  return ZETA_OK;
}

/* ordering cache and request log of the learned ordering */
int learn_buffers() {
  Context &c = ctx();
  if (!c.s_ocache) {
    c.s_ocache_entries = 1ull << 22; /* 128 MiB of 32-byte entries */
    ZCHECK(cudaMalloc(&c.s_ocache, c.s_ocache_entries * sizeof(OrderEntry)));
    ZCHECK(cudaMemset(c.s_ocache, 0, c.s_ocache_entries * sizeof(OrderEntry)));
    c.s_oreq_cap = 1u << 20;
    ZCHECK(cudaMalloc(&c.s_oreq, (size_t)c.s_oreq_cap * sizeof(OrderRequest)));
    ZCHECK(cudaMalloc(&c.s_noreq, sizeof(uint32_t)));
    ZCHECK(cudaMemset(c.s_noreq, 0, sizeof(uint32_t)));
  }
  return ZETA_OK;
}

int search_pure_launch(const uint64_t *d_boards, const uint8_t *d_stm, int n, int depth, int workers, int32_t *d_scores,
                       uint32_t *d_moves, unsigned long long *d_nodes, cudaStream_t s, int learned) {
  Context &c = ctx();
  LearnArgs la{0, 0, 0, nullptr, 0, nullptr, nullptr, 0};
  if (learned) {
    int rc = learn_buffers();
    if (rc) return rc;
    la = LearnArgs{1, c.s_learned_top, c.s_learned_quiet, (OrderEntry *)c.s_ocache, c.s_ocache_entries - 1, (OrderRequest *)c.s_oreq,
                   c.s_noreq, c.s_oreq_cap};
  }
  if (n <= 0 || workers <= 0 || depth < 1 || depth > kMaxSearchDepth - 1)
    return set_error(ZETA_ERR_ARG, "search: need n > 0, workers > 0, depth 1..%d", kMaxSearchDepth - 1);
  if ((long long)n * workers > (1ll << 31)) return set_error(ZETA_ERR_ARG, "search: too many workers");
  int rc = search_buffers(n);
  if (rc) return rc;
  if (c.tt_owner != 1 && c.tt1) {
    /* the full engine keeps a different entry format in the same table */
    ZCHECK(cudaMemsetAsync(c.tt1, 0, c.tt1_entries * 16, s));
  }
  c.tt_owner = 1;
  TTEntry *tt = (TTEntry *)(c.tt1 ? c.tt1 : c.s_tt);
  u64 entries = c.tt1 ? c.tt1_entries : c.s_tt_entries;
  ZCHECK(cudaMemsetAsync(c.s_out, 0, (size_t)n * sizeof(SearchOut), s));
  ZCHECK(cudaMemsetAsync(c.s_done, 0, (size_t)2 * n * sizeof(uint32_t), s));
  ZCHECK(cudaMemsetAsync(c.s_busy, 0, c.s_busy_entries * sizeof(uint32_t), s));
  ZCHECK(cudaMemsetAsync(c.s_status, 0, kSearchStatusBytes, s));
  unsigned long long *ttops = (unsigned long long *)(c.s_status + 2);
  const long long total = (long long)n * workers;
  const int tpb = 128;
  /* automatic form: warp-cooperative when every worker can have a resident
   * warp of its own (it is the sparse form's walk with the last ply scored
   * by the whole warp), else dense */
  static int resident_blocks = 0;
  if (!resident_blocks) {
    int per_sm = 0;
    ZCHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_search_warp<128>, tpb, 0));
    resident_blocks = (per_sm > 0 ? per_sm : 1) * c.sms;
  }
  const int form = c.s_launch_form ? c.s_launch_form
                                   : (total <= (long long)resident_blocks * (tpb / 32) ? 3 : 1);
  const long long threads = form == 1 ? total : total * 32;
  const unsigned blocks = (unsigned)((threads + tpb - 1) / tpb);
  const unsigned long long budget = 1ull << 40;
  ZCHECK(cudaEventRecord(c.ev[1], s));
  if (form == 3)
    k_search_warp<128><<<blocks, tpb, 0, s>>>(d_boards, d_stm, n, workers, depth, tt, entries - 1, c.s_busy,
                                              c.s_busy_entries - 1, c.s_done, (SearchOut *)c.s_out, budget,
                                              c.s_status, c.s_done + n, c.s_helpers_cap, la, ttops);
  else
    k_search_pure<128><<<blocks, tpb, 0, s>>>(d_boards, d_stm, n, workers, depth, tt, entries - 1, c.s_busy,
                                              c.s_busy_entries - 1, c.s_done, (SearchOut *)c.s_out, budget,
                                              c.s_status, c.s_done + n, c.s_helpers_cap, la, form == 2, ttops);
  ZCHECK(cudaGetLastError());
  ZCHECK(cudaEventRecord(c.ev[2], s));
  k_search_scatter<<<(n + 127) / 128, 128, 0, s>>>((const SearchOut *)c.s_out, n, d_scores, d_moves, d_nodes);
  ZCHECK(cudaGetLastError());
  uint32_t st[kSearchStatusBytes / 4] = {0};
  ZCHECK(cudaMemcpyAsync(st, c.s_status, kSearchStatusBytes, cudaMemcpyDeviceToHost, s));
  ZCHECK(cudaStreamSynchronize(s));
  const uint32_t status = st[0];
  memcpy(&c.s_probes, st + 2, 8);
  memcpy(&c.s_stores, st + 4, 8);
  float ms = -1.f;
  if (cudaEventElapsedTime(&ms, c.ev[1], c.ev[2]) != cudaSuccess) ms = -1.f;
  (void)cudaGetLastError();
  c.sstats.kernel_ms = ms;
  if (status & SST_BUDGET) return set_error(ZETA_ERR_BUDGET, "search: a worker ran out of its node budget");
  return ZETA_OK;
}

/* Iterative deepening 1..depth over a batch, the transposition table
 * kept between iterations (src/search.c:77-198 does the same per launch).
 * With ordering > 0 every iteration is one kernel step of the learned
 * ordering: the search logs the nodes that have no network ordering yet,
 * then one batched tensor-core inference (BF16, or FP8 when ordering == 2)
 * scores them all and the next iteration orders by the result.  Host
 * outputs: final scores and best moves, nodes summed over all iterations,
 * wall time, search-kernel time and network time (ms). */
int search_id(const uint64_t *boards, const uint8_t *stm, int n, int depth, int workers, int ordering, int32_t *scores,
              uint32_t *moves, uint64_t *nodes, float *ms_total, float *ms_search, float *ms_mlp) {
  Context &c = ctx();
  const int learned = ordering > 0;
  if (learned && !mlp_ready_for_search())
    return set_error(ZETA_ERR_STATE, "learned ordering needs zeta_mlp_init (and training or parameters)");
  cudaStream_t s = c.stream;
  uint64_t *db = nullptr, *dn = nullptr;
  uint8_t *ds = nullptr;
  int32_t *dsc = nullptr;
  uint32_t *dm = nullptr;
  cudaError_t e = cudaMalloc(&db, (size_t)n * 56);
  if (e == cudaSuccess) e = cudaMalloc(&ds, n);
  if (e == cudaSuccess) e = cudaMalloc(&dsc, (size_t)n * 4);
  if (e == cudaSuccess) e = cudaMalloc(&dm, (size_t)n * 4);
  if (e == cudaSuccess) e = cudaMalloc(&dn, (size_t)n * 8);
  if (e == cudaSuccess) e = cudaMemcpy(db, boards, (size_t)n * 56, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(ds, stm, n, cudaMemcpyHostToDevice);
  int rc = e == cudaSuccess ? ZETA_OK : cuda_fail(e, "search_id buffers");
  if (!rc && learned) rc = learn_buffers();
  if (!rc && learned) {
    e = cudaMemsetAsync(c.s_ocache, 0, c.s_ocache_entries * sizeof(OrderEntry), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(c.s_noreq, 0, 4, s);
    if (e != cudaSuccess) rc = cuda_fail(e, "search_id cache");
  }
  std::vector<uint64_t> it(n);
  if (nodes) memset(nodes, 0, (size_t)n * 8);
  float t_search = 0.f, t_mlp = 0.f;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, s);
  for (int d = 1; d <= depth && !rc; d++) {
    rc = search_pure_launch(db, ds, n, d, workers, dsc, dm, (unsigned long long *)dn, s, learned);
    if (rc) break;
    t_search += c.sstats.kernel_ms;
    if (cudaMemcpy(it.data(), dn, (size_t)n * 8, cudaMemcpyDeviceToHost) != cudaSuccess) {
      rc = set_error(ZETA_ERR_CUDA, "search_id read-back");
      break;
    }
    if (nodes)
      for (int i = 0; i < n; i++) nodes[i] += it[i];
    if (learned && d < depth) {
      uint32_t nreq = 0;
      cudaMemcpy(&nreq, c.s_noreq, 4, cudaMemcpyDeviceToHost);
      if (nreq > c.s_oreq_cap) nreq = c.s_oreq_cap;
      cudaEvent_t m0, m1;
      cudaEventCreate(&m0);
      cudaEventCreate(&m1);
      cudaEventRecord(m0, s);
      if (nreq) rc = mlp_fill_order_cache((const OrderRequest *)c.s_oreq, nreq, (OrderEntry *)c.s_ocache,
                                          c.s_ocache_entries - 1, ordering == 2, s);
      cudaEventRecord(m1, s);
      cudaEventSynchronize(m1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, m0, m1);
      t_mlp += ms;
      cudaEventDestroy(m0);
      cudaEventDestroy(m1);
      cudaMemsetAsync(c.s_noreq, 0, 4, s);
    }
  }
  cudaEventRecord(e1, s);
  cudaEventSynchronize(e1);
  float tot = 0.f;
  cudaEventElapsedTime(&tot, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (!rc) {
    if (scores) cudaMemcpy(scores, dsc, (size_t)n * 4, cudaMemcpyDeviceToHost);
    if (moves) cudaMemcpy(moves, dm, (size_t)n * 4, cudaMemcpyDeviceToHost);
  }
  cudaFree(db);
  cudaFree(ds);
  cudaFree(dsc);
  cudaFree(dm);
  cudaFree(dn);
  if (ms_total) *ms_total = tot;
  if (ms_search) *ms_search = t_search;
  if (ms_mlp) *ms_mlp = t_mlp;
  return rc;
}

}  // namespace zeta

