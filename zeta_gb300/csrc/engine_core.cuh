/*
 * engine_core.cuh -- the full-engine alpha-beta search: the reference's
 * alphabeta_gpu (src/zeta.cl:852-2511) with all of its heuristics, as a
 * per-thread state machine.
 *
 * The reference runs one worker per 64-lane work-group: every lane owns a
 * square, move generation and evaluation are 64-way, and the tree walk
 * (an explicit stack of per-ply arrays in local memory) runs on lane 0
 * between barriers.  Here one thread is one worker: move generation and
 * evaluation are the set-wise forms of chess.cuh / eval.cuh in that
 * thread's registers, and the per-ply arrays are a frame stack in global
 * memory.  The walk itself follows the reference step for step, so one
 * worker visits exactly the reference's tree:
 *
 *   node entry   LMR undo for checking moves, check / promotion
 *                extension, quiescence when depth <= 0 (captures only,
 *                stand pat), mate / stalemate, repetition, fifty-move and
 *                bare-kings draws, TT1 lower-bound probe, ABDADA TT2 probe
 *                and lock (zeta.cl:1316-1723);
 *   move down    TT2 store, negamax backup, LMR re-search, IID completion,
 *                TT1 store with the reference's replacement rule, killer
 *                and counter moves (zeta.cl:1724-1951);
 *   move picker  null move (R=2, depth >= 4), TT move > IID move > killer
 *                > counter move > MVV-LVA captures > piece-square gain,
 *                first the ITER1 moves, then the moves ABDADA deferred
 *                (zeta.cl:1955-2268);
 *   move up      make, hash, castle / en-passant flags, half-move clock,
 *                child window, IID start, null-move window, LMR
 *                (zeta.cl:2269-2451);
 *   PV           the finishing worker walks TT1 from the root
 *                (zeta.cl:2452-2511).
 *
 * The reference's move picker takes, among the remaining moves, the one
 * with the highest score; ties go to the lowest from-square and, within
 * one from-square, to the highest to-square (zeta.cl:2087-2124 with the
 * serial lane reduction).  The move lists here keep the same order key.
 *
 * Batches: position p's workers are threads w*N + p (different warps);
 * each position owns a power-of-two slice of TT1 and TT2, so a batched
 * search of a position equals a single search with that table size.
 * Every loop is bounded; an exhausted budget sets a status bit.
 */
#pragma once

#include <cstring>

#include "context.cuh"
#include "eval.cuh"
#include "movegen_fast.cuh"
#include "tables.cuh"

namespace zeta {

namespace {

constexpr int kEPly = 64;              /* MAXPLY */
constexpr int kEFrames = kEPly + 2;    /* frames 0..64 (+1 for the child window at 64) */
constexpr int kGamePly = 1024;         /* MAXGAMEPLY */
constexpr int kEMoves = 218;           /* most legal moves of a chess position */
constexpr int E_INF = 32000;           /* INF */
constexpr int E_MATE = 30000;          /* MATESCORE */
constexpr int E_LMRR = 1, E_NULLR = 2; /* LMRR, NULLR */
constexpr int E_INFMS = 0x7FFFFFFF;    /* INFMOVESCORE */
constexpr Move E_NULLMOVE = 0x41;

/* node states and search modes (zeta.cl:87-101) */
constexpr uint8_t ST_KIC = 1, ST_QS = 2, ST_EXT = 4, ST_LMR = 8, ST_IID = 16, ST_IIDDONE = 32, ST_ITER1 = 64,
                  ST_ITER2 = 128;
constexpr uint8_t MD_SEARCH = 1, MD_NULL = 2, MD_LMR = 4, MD_IID = 8;
constexpr int F_LOW = 0, F_EXACT = 1, F_HIGH = 2;

constexpr uint32_t EST_BUDGET = 1u; /* a worker ran out of loop iterations */

#define ZE __host__ __device__ __forceinline__

ZE bool is_mate(int v) { return (v > E_MATE && v < E_INF) || (v < -E_MATE && v > -E_INF); }
ZE bool is_inf(int v) { return v == E_INF || v == -E_INF; }

/* TT1 entry, the reference's TTE (src/types.h:207-214): 16 bytes */
struct __align__(16) TT1E {
  unsigned long long hash; /* position hash ^ move ^ score ^ depth */
  uint32_t move;
  int16_t score;
  uint8_t flag; /* bound | age << 2 */
  uint8_t depth;
};
/* TT2 entry, the reference's ABDADATTE (src/types.h:216-224): 24 bytes */
struct __align__(8) TT2E {
  unsigned long long hash; /* hash ^ score ^ depth */
  int lock, ply, sd;
  int16_t score, depth;
};
static_assert(sizeof(TT1E) == 16, "TT1 entry is 16 bytes");
static_assert(sizeof(TT2E) == 24, "TT2 entry is 24 bytes");

/* one ply of a worker (the reference's local per-ply arrays) */
struct EFrame {
  Pos pos;      /* the board at this ply (copy-make instead of undo) */
  u64 hash;     /* localHashHistory */
  u64 th;       /* hash of the position itself (without the null-move toggle) */
  u64 m1[4];    /* ITER1 moves not yet searched (bits over the move list) */
  u64 m2[4];    /* ITER2: moves deferred by ABDADA */
  int alpha, beta, depth, todo, mc;
  Move mh, iid; /* localMoveHistory, localIIDMoves */
  uint8_t state, mode, hmc, mi; /* node state, search mode, half-move clock, list index of mh */
  u64 lmask[4];                 /* list indices of the network's best moves */
  uint8_t lidx[kOrderTop];      /* their list indices, best first (0xFF = none) */
};

struct EngineArgs {
  const uint64_t *boards; /* N x 7 */
  const uint8_t *stm;
  const u64 *hist_in;      /* N x kGamePly, or null: entry ply_init = the root hash */
  const int *ply_init;     /* N, or null: 0 */
  const uint8_t *active;   /* N, or null: all */
  int N, W, depth;
  unsigned long long max_nodes;   /* stop when worker 0 of the position has made more moves */
  unsigned long long iter_budget; /* main-loop iterations per worker */
  TT1E *tt1;
  u64 tt1_slice; /* entries per position (power of two), <= 1 disables */
  TT2E *tt2;
  u64 tt2_slice;
  EFrame *frames;      /* N*W x kEFrames */
  Move *moves;         /* N*W x kEFrames x kEMoves */
  u64 *hist;           /* N*W x kGamePly */
  Move *killers;       /* N*W x kEPly */
  Move *cmoves;        /* N*W x 64 x 64 */
  unsigned long long *cnt; /* N*W x 4: nodes, TT-move hits, TT-score hits, IID hits */
  uint32_t *finito;    /* N: gid+1 of the first worker back at the root */
  uint32_t *pv;        /* N x 64: PV[0] score, PV[1..] moves */
  uint32_t *status;
  /* learned ordering (no reference counterpart): null cache = off */
  OrderEntry *ocache;
  u64 ocache_mask;
  OrderRequest *oreq;
  uint32_t *noreq;
  uint32_t oreq_cap;
  int learned_top;
  /* lazy SMP (no TT2) helper depths, no reference counterpart: with k >= 2,
   * helpers w = k-1, 2k-1, ... search one ply deeper than the iteration;
   * 0 = every worker at the iteration depth (the reference's search) */
  int deep_every;
};

/* the move-ordering score of the reference's picker (zeta.cl:2087-2124) */
ZE int pick_score(Move m, int stm, const EvalTables &T) {
  const int from = m_from(m), to = m_to(m);
  const int pf = m_pfrom(m) >> 1, pt = m_pto(m) >> 1, pc = m_pcpt(m) >> 1;
  const int vt = stm ? to : (to ^ 56), vf = stm ? from : (from ^ 56);
  int s = T.value[pt] + T.pst[pt][vt] + T.control[vt];
  s -= T.value[pf] + T.pst[pf][vf] + T.control[vf];
  if (pc) s = T.value[pc] * 16 - T.value[pt];
  return s;
}

/* TT1 verification: the stored hash is hash ^ move ^ score ^ depth with
 * the score sign-extended (zeta.cl:1632, 2021) */
ZE bool tt1_ok(const TT1E &e, u64 h) {
  return e.hash == (h ^ (u64)e.move ^ (u64)(long long)e.score ^ (u64)e.depth);
}

/* Table entries are read and written whole, through L2 (shared by the
 * workers on every SM); the host versions serve host-side test builds. */
ZE TT1E tt1_load(const TT1E *p) {
  TT1E e;
#if defined(__CUDA_ARCH__)
  longlong2 v = __ldcg((const longlong2 *)p);
  memcpy(&e, &v, 16);
#else
  e = *p;
#endif
  return e;
}
ZE void tt1_store(TT1E *p, const TT1E &e) {
#if defined(__CUDA_ARCH__)
  longlong2 v;
  memcpy(&v, &e, 16);
  __stcg((longlong2 *)p, v);
#else
  *p = e;
#endif
}
ZE TT2E tt2_load(const TT2E *p) {
  TT2E e;
#if defined(__CUDA_ARCH__)
  const unsigned long long *q = (const unsigned long long *)p;
  unsigned long long w[3] = {__ldcg(q), __ldcg(q + 1), __ldcg(q + 2)};
  memcpy(&e, w, 24);
#else
  e = *p;
#endif
  return e;
}
ZE void tt2_store(TT2E *p, const TT2E &e) {
#if defined(__CUDA_ARCH__)
  unsigned long long w[3];
  memcpy(w, &e, 24);
  unsigned long long *q = (unsigned long long *)p;
  __stcg(q, w[0]);
  __stcg(q + 1, w[1]);
  __stcg(q + 2, w[2]);
#else
  *p = e;
#endif
}

/* start moving a table entry into L2 (the child's entry, probed when the
 * child is entered); no effect on host builds */
ZE void prefetch_l2(const void *p) {
#if defined(__CUDA_ARCH__)
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
#else
  (void)p;
#endif
}

/* 32-bit atomics of the ABDADA table and the early-bird flag */
ZE int e_cas(int *p, int cmp, int val) {
#if defined(__CUDA_ARCH__)
  return atomicCAS(p, cmp, val);
#else
  int old = *p;
  if (old == cmp) *p = val;
  return old;
#endif
}
ZE uint32_t e_casu(uint32_t *p, uint32_t cmp, uint32_t val) {
#if defined(__CUDA_ARCH__)
  return atomicCAS(p, cmp, val);
#else
  uint32_t old = *p;
  if (old == cmp) *p = val;
  return old;
#endif
}
ZE void e_xchg(int *p, int val) {
#if defined(__CUDA_ARCH__)
  atomicExch(p, val);
#else
  *p = val;
#endif
}
ZE void e_or(uint32_t *p, uint32_t v) {
#if defined(__CUDA_ARCH__)
  atomicOr(p, v);
#else
  *p |= v;
#endif
}

}  // namespace

namespace {

/* The reference picker over one move set (zeta.cl:2039-2124): highest
 * score, ties to the lowest from-square, then to the highest to-square.
 * Returns the list index or -1.  Counts TT-move and IID-move sightings as
 * the reference's COUNTERS[3] / [5] do. */
__host__ __device__ int pick_move(const Move *L, const u64 *mask, int stm, Move killer, Move counter, Move iid, Move ttm,
                         bool randomize, uint32_t &prn, const EvalTables &T, unsigned long long *C,
                         const EFrame *lf, int ltop) {
  int best = -1, bs = 0, bf = 0, bt = 0;
  for (int wd = 0; wd < 4; wd++) {
    u64 b = mask[wd];
    while (b) {
      const int i = wd * 64 + ctz(b);
      b &= b - 1;
      const Move m = L[i];
      int s = pick_score(m, stm, T);
      if (lf && ((lf->lmask[i >> 6] >> (i & 63)) & 1) && (m_pcpt(m) >> 1) == PNONE) {
        /* learned: the network's quiet moves right after the counter move */
        for (int r = 0; r < ltop; r++)
          if (lf->lidx[r] == i) {
            s = T.value[QUEEN] + T.value[PAWN] - 1 - r;
            break;
          }
      }
      if (m == counter) s = T.value[QUEEN] + T.value[PAWN];
      if (m == killer) s = T.value[QUEEN] + 2 * T.value[PAWN];
      if (randomize) {
        prn ^= prn << 13;
        prn ^= prn >> 17;
        prn ^= prn << 5;
        s += (int)(prn % (uint32_t)E_INF);
      }
      if (m == iid) {
        s = E_INFMS - 200;
        C[3]++;
      }
      if (m == ttm) {
        s = E_INFMS - 100;
        C[1]++;
      }
      const int f = m_from(m), t = m_to(m);
      if (best < 0 || s > bs || (s == bs && (f < bf || (f == bf && t > bt)))) {
        best = i;
        bs = s;
        bf = f;
        bt = t;
      }
    }
  }
  return best;
}

ZE int mate_from_tt(int s, int ply) {
  s = (is_mate(s) && s > 0) ? s - ply : s;
  s = (is_mate(s) && s < 0) ? s + ply : s;
  return s;
}
ZE int mate_to_tt(int s, int ply) {
  s = (is_mate(s) && s > 0) ? s + ply : s;
  s = (is_mate(s) && s < 0) ? s - ply : s;
  return s;
}

/* the side's piece sets and the enemy attack map of a node, computed once
 * for both the in-check test and the move generation */
struct NodeSets {
  Sets s;
  u64 danger;
};
__host__ __device__ __noinline__ void e_sets(const Pos &p, int stm, NodeSets &ns) {
  ns.s = make_sets(p, stm);
  ns.danger = enemy_attacks(ns.s, stm);
}
__host__ __device__ __noinline__ int e_gen(const Pos &p, const NodeSets &ns, int stm, bool qs, Move *L) {
  return gen_engine(p, ns.s, ns.danger, stm, qs, L);
}
__host__ __device__ __noinline__ int e_eval(const Pos &p, const EvalTables *T) { return eval_white(p, *T); }


/* One worker (thread t = w * N + p) of the full-engine search. */
__host__ __device__ void engine_worker(const EngineArgs &a, long long t, const EvalTables &sT) {
  const int p = (int)(t % a.N), w = (int)(t / a.N);
  if (a.active && !a.active[p]) return;

  EFrame *F = a.frames + t * kEFrames;
  Move *MV = a.moves + t * (long long)kEFrames * kEMoves;
  u64 *H = a.hist + t * kGamePly;
  Move *KIL = a.killers + t * kEPly;
  Move *CM = a.cmoves + t * 4096;
  unsigned long long *C = a.cnt + t * 4;
  const unsigned long long *C0 = a.cnt + (long long)p * 4; /* worker 0 of this position */
  TT1E *tt1 = a.tt1_slice > 1 ? a.tt1 + (u64)p * a.tt1_slice : nullptr;
  TT2E *tt2 = a.tt2_slice > 1 ? a.tt2 + (u64)p * a.tt2_slice : nullptr;
  const u64 mask1 = a.tt1_slice - 1, mask2 = a.tt2_slice - 1;
  const int gid1 = w + 1;
  /* a deeper helper never ends the search (the result is a worker's at the
   * iteration depth); its table entries serve the next iteration */
  const bool deeper = !tt2 && a.deep_every >= 2 && w > 0 && w % a.deep_every == a.deep_every - 1;
  const int D = a.depth + (deeper ? 1 : 0);
  const int ply_init = a.ply_init ? a.ply_init[p] : 0;
  const int ttage = ply_init & 0x3F;
  const uint64_t *B = a.boards + (long long)p * 7;
  const int stm0 = a.stm[p] & 1;
  uint32_t prn = 0x9E3779B9u ^ (uint32_t)(t * 0x85EBCA6Bu) ^ 1u;

  C[0] = C[1] = C[2] = C[3] = 0;
  for (int k = 0; k <= ply_init && k < kGamePly; k++)
    H[k] = a.hist_in ? a.hist_in[(long long)p * kGamePly + k] : (k == ply_init ? B[5] : 0ULL);

  Pos root;
  root.b0 = B[0];
  root.p1 = B[1];
  root.p2 = B[2];
  root.p3 = B[3];
  root.cr = B[4];
  const u64 root_th = compute_hash(root, stm0); /* children hash from this, the root keeps B[5] */
  for (int k = 0; k < 2; k++) {
    EFrame *f = F + k;
    f->pos = root;
    f->hash = B[5];
    f->th = root_th;
    f->alpha = -E_INF;
    f->beta = E_INF;
    f->todo = 0;
    f->mc = 0;
    f->mh = 0;
    f->iid = 0;
    f->hmc = (uint8_t)B[6];
    f->depth = k == 0 ? D + 1 : D;
    f->state = ST_ITER1;
    f->mode = MD_SEARCH;
    f->mi = 0;
    for (int j = 0; j < 4; j++) f->m1[j] = f->m2[j] = 0;
  }

  int sd = 1, ply = 0, stm = stm0;
  Move bestmove = 0;
  int bestscore = 0;
  bool out_of_budget = false;
  unsigned long long iters = 0;

  for (;;) {
    if (++iters > a.iter_budget) {
      e_or(a.status, EST_BUDGET);
      out_of_budget = true;
      break;
    }
    bool brandomize = false, bresearch = false, bforward = false;

    /* ---------------- node entry (zeta.cl:1316-1723) ---------------- */
    {
      EFrame *f = F + sd, *up = F + sd - 1;
      const Pos pos = f->pos;
      NodeSets ns;
      e_sets(pos, stm, ns);
      const bool kic = (ns.danger & ns.s.kbb) != 0;
      if (kic && (up->state & ST_LMR)) { /* no reduction of checking moves */
        f->depth += E_LMRR;
        up->state ^= ST_LMR;
        f->mode = up->mode;
      }
      const Move um = up->mh;
      if (f->depth >= 0 && !(up->state & ST_QS) &&
          (kic || ((m_pfrom(um) >> 1) == PAWN && (m_pto(um) >> 1) == QUEEN))) {
        f->depth++;
        f->state |= ST_EXT;
      }
      const bool qs = f->depth <= 0;
      Move *L = MV + sd * kEMoves;
      const int ngen = e_gen(pos, ns, stm, qs, L);
      int movecount = ngen;
      f->state |= (qs ? ST_QS : 0) | (kic ? ST_KIC : 0);
      /* the static score is used only by quiescence (stand pat, no capture
       * left) and at the ply limit: mates, stalemates and draws set their
       * own score below, and other nodes overwrite it by searching */
      int score = 0;
      if (qs || sd >= kEPly) {
        const int ev = e_eval(pos, &sT);
        score = stm ? -ev : ev;
      }
      if (!qs && kic && movecount == 0) score = -E_INF + ply;
      if (!qs && !kic && movecount == 0) score = 0;
      for (int k = ply + ply_init - 2; movecount > 0 && !qs && sd > 1 && k >= 0 && k >= ply + ply_init - (int)f->hmc;
           k -= 2) {
        if (k < kGamePly && f->hash == H[k]) {
          movecount = 0;
          score = 0;
          break;
        }
      }
      if (sd > 1 && f->hmc >= 100) {
        movecount = 0;
        score = 0;
      }
      if (sd > 1 && popc(pos.p1 | pos.p2 | pos.p3) <= 2) {
        movecount = 0;
        score = 0;
      }
      if (sd >= kEPly) movecount = 0;
      if (movecount == 0) f->alpha = score;
      if (movecount > 0 && qs && !kic && score >= f->beta) {
        f->alpha = score; /* stand pat, fail soft */
        movecount = 0;
      }
      if (movecount > 0 && qs && !kic && score > f->alpha) f->alpha = score;
      /* TT1: lower bounds raise alpha (zeta.cl:1611-1646) */
      if (movecount > 0 && !qs && sd > 1 && !(f->mode & MD_NULL) && tt1) {
        const TT1E e = tt1_load(tt1 + (f->hash & mask1));
        const int s = mate_from_tt(e.score, ply);
        if (tt1_ok(e, f->hash) && (int)e.depth >= f->depth && (e.flag & 3) > F_LOW && !is_inf(s) && s > f->alpha) {
          f->alpha = s;
          if (f->alpha >= f->beta) movecount = 0;
          C[2]++;
        }
      }
      /* ABDADA TT2 (zeta.cl:1648-1717) */
      if (movecount > 1 && !qs && sd > 1 && !(f->mode & MD_NULL) && !(f->mode & MD_IID) && up->todo > 1 &&
          up->mc > 1 && tt2 && f->depth > 0) {
        TT2E *e2 = tt2 + (f->hash & mask2);
        int nl = 0;
        if (e_cas(&e2->ply, 0, ply_init + 1) != ply_init + 1 || e_cas(&e2->sd, 0, D + 1) != D + 1) {
          e_xchg(&e2->ply, ply_init + 1);
          e_xchg(&e2->sd, D + 1);
          e_xchg(&e2->lock, 0);
        }
        if (up->state & ST_ITER1) {
          nl = e_cas(&e2->lock, 0, gid1);
          nl = e_cas(&e2->lock, gid1, gid1);
        }
        const TT2E e = tt2_load(e2);
        const int s = mate_from_tt(e.score, ply);
        if (nl != gid1 && e.hash == (f->hash ^ (u64)(long long)e.score ^ (u64)(long long)e.depth) &&
            e.depth >= (int16_t)f->depth && !is_inf(s) && s > f->alpha) {
          f->alpha = s;
          if (f->alpha >= f->beta) movecount = 0;
        } else if (nl != gid1 && nl > 0 && (up->state & ST_ITER1)) {
          /* searched by another worker: defer the parent's move to ITER2 */
          up->m2[up->mi >> 6] |= 1ULL << (up->mi & 63);
          up->todo--;
          movecount = 0;
          f->alpha = E_INF; /* the parent ignores this score */
        }
      }
      f->mc = movecount;
      if (a.ocache) {
        /* the network's ordering of this node: from the cache at >= 3 plies
         * left, else requested for the next iteration from >= 2 plies */
        for (int j = 0; j < 4; j++) f->lmask[j] = 0;
        for (int r = 0; r < kOrderTop; r++) f->lidx[r] = 0xFF;
        if (movecount > 1 && !qs && f->depth >= 2) {
          OrderEntry *oe = a.ocache + (f->hash & a.ocache_mask);
          const unsigned long long ek = ((volatile unsigned long long *)&oe->key)[0];
          if (ek == f->hash) {
            if (f->depth >= 3)
              for (int r = 0; r < a.learned_top && r < kOrderTop; r++) {
                const uint16_t k = oe->mv[r];
                if (k == 0xFFFF) break;
                for (int j = 0; j < ngen; j++)
                  if ((uint16_t)(m_from(L[j]) | (m_to(L[j]) << 6)) == k) {
                    f->lidx[r] = (uint8_t)j;
                    f->lmask[j >> 6] |= 1ULL << (j & 63);
                    break;
                  }
              }
          } else {
#if defined(__CUDA_ARCH__)
            const uint32_t idx = atomicAdd(a.noreq, 1u);
#else
            const uint32_t idx = (*a.noreq)++;
#endif
            if (idx < a.oreq_cap) {
              OrderRequest q;
              q.key = f->hash;
              q.b[0] = pos.b0;
              q.b[1] = pos.p1;
              q.b[2] = pos.p2;
              q.b[3] = pos.p3;
              q.b[4] = pos.cr;
              q.stm = stm;
              q.pad = 0;
              a.oreq[idx] = q;
              OrderEntry pend; /* requested: other workers do not ask again */
              pend.key = f->hash;
              for (int r = 0; r < kOrderTop; r++) pend.mv[r] = 0xFFFF;
              *oe = pend;
            }
          }
        }
      }
      for (int j = 0; j < 4; j++) {
        const int lo = j * 64;
        f->m1[j] = ngen <= lo ? 0ULL : (ngen >= lo + 64 ? ~0ULL : ((1ULL << (ngen - lo)) - 1));
        f->m2[j] = 0;
      }
    }

    /* ---------------- move down (zeta.cl:1724-1951) ---------------- */
    while ((F[sd].todo >= F[sd].mc || F[sd].alpha >= F[sd].beta) && !bresearch && !bforward) {
      if (sd > 1 && tt2 && (F[sd - 1].state & ST_ITER1)) {
        EFrame *f = F + sd;
        TT2E *e2 = tt2 + (f->hash & mask2);
        const int s = mate_to_tt(f->alpha, ply);
        const int nl = e_cas(&e2->lock, gid1, gid1);
        if (nl == gid1 && !is_inf(s) && !(f->state & ST_QS) && !(f->mode & MD_NULL) && !(f->mode & MD_IID)) {
          TT2E e;
          e.hash = f->hash ^ (u64)(long long)s ^ (u64)(long long)f->depth;
          e.score = (int16_t)s;
          e.depth = (int16_t)f->depth;
          e.lock = gid1;
          e.ply = ply_init + 1;
          e.sd = D + 1;
          tt2_store(e2, e);
        }
      }
      sd--;
      ply--;
      stm ^= 1;
      if (sd < 1) {
        if (!deeper) e_casu(a.finito + p, 0u, (uint32_t)gid1); /* early bird */
        break;
      }
      EFrame *g = F + sd;
      int flag = F_LOW;
      const Move move = g->mh;
      int score = -F[sd + 1].alpha;
      if (move == E_NULLMOVE && score < g->beta) score = -E_INF; /* null move: only a fail high counts */
      if ((g->state & ST_LMR) && score > g->alpha) {               /* reduced move beat alpha: re-search */
        score = -E_INF;
        bresearch = true;
        g->state ^= ST_LMR;
      }
      if (score > g->alpha) {
        g->alpha = score;
        flag = F_EXACT;
        if (sd == 1 && move != 0 && move != E_NULLMOVE) {
          bestscore = score;
          bestmove = move;
        }
      }
      if (score >= g->beta) flag = F_HIGH;
      if ((g->state & ST_IID) && flag > F_LOW) g->iid = move;
      if ((g->state & ST_IID) && (g->alpha >= g->beta || g->todo >= g->mc)) {
        /* internal iterative deepening done: search the node again */
        bforward = true;
        g->mh = 0;
        g->mc = 0;
        g->todo = 0;
        g->alpha = -F[sd - 1].beta;
        g->beta = -F[sd - 1].alpha;
        g->depth = F[sd - 1].depth - 1;
        g->mode = F[sd - 1].mode;
        g->state = ST_IIDDONE | ST_ITER1;
      }
      if (flag > F_LOW && move != 0 && move != E_NULLMOVE && !(g->state & ST_QS) && !(g->mode & MD_NULL) &&
          !(g->mode & MD_IID) && !(g->state & ST_LMR) && g->depth >= 0 && !bforward && !bresearch && tt1) {
        TT1E *ep = tt1 + (g->hash & mask1);
        const int s = mate_to_tt(score, ply);
        const u64 key = g->hash ^ (u64)move ^ (u64)(long long)s ^ (u64)(long long)g->depth;
        TT1E e = tt1_load(ep);
        const int age = e.flag >> 2;
        if ((uint8_t)g->depth > e.depth || ((uint8_t)g->depth >= e.depth && tt1_ok(e, g->hash) && s > (int)e.score) ||
            (ttage != age && ttage != age + 2)) {
          e.hash = key;
          e.move = move;
          e.score = (int16_t)s;
          e.flag = (uint8_t)(flag | (ttage & 0x3F) << 2);
          e.depth = (uint8_t)g->depth;
          tt1_store(ep, e);
        }
      }
      if (flag == F_HIGH && move != 0 && move != E_NULLMOVE && (m_pcpt(move) >> 1) == PNONE && !(g->state & ST_QS) &&
          !(g->mode & MD_NULL) && !bforward && !bresearch) {
        KIL[sd] = move;
        const Move pm = F[sd - 1].mh;
        CM[m_from(pm) * 64 + m_to(pm)] = move;
      }
      if (g->state & ST_LMR) g->state ^= ST_LMR;
    }
    {
      bool bexit = sd < 1;
      if (((volatile const unsigned long long *)C0)[0] > a.max_nodes) bexit = true;
      if (((volatile const uint32_t *)a.finito)[p] > 0) bexit = true;
      if (bexit) break;
    }
    if (bforward) continue;

    /* ---------------- move picker (zeta.cl:1955-2268) ---------------- */
    EFrame *g = F + sd;
    Move lmove = 0;
    if (!bresearch && sd > 1 && g->mh == 0 && !(g->state & (ST_QS | ST_KIC | ST_EXT | ST_IIDDONE)) &&
        !(g->mode & (MD_NULL | MD_IID)) && g->depth >= 4)
      lmove = E_NULLMOVE;
    if (bresearch) lmove = g->mh;
    if (lmove == 0 && (tt1 && !tt2) && w > 0 && !(g->state & (ST_QS | ST_KIC | ST_EXT)) &&
        !(g->mode & (MD_NULL | MD_LMR | MD_IID)) && g->depth > 0 && g->todo >= 1)
      brandomize = true; /* lazy SMP helpers without TT2 */
    const Move pm = F[sd - 1].mh;
    const Move killer = KIL[sd];
    const Move counter = CM[m_from(pm) * 64 + m_to(pm)];
    Move ttmove = 0;
    if (tt1) {
      const TT1E e = tt1_load(tt1 + (g->hash & mask1));
      if (tt1_ok(e, g->hash)) ttmove = e.move;
    }
    const Move *L = MV + sd * kEMoves;
    int pick = -1;
    if (lmove == 0 && !bresearch) {
      pick = pick_move(L, g->m1, stm, killer, counter, g->iid, ttmove, brandomize, prn, sT, C,
                       a.ocache ? g : nullptr, a.learned_top);
      if (pick >= 0) lmove = L[pick];
    }
    if (lmove == 0 && (g->state & ST_ITER1)) {
      g->state ^= ST_ITER1;
      g->state |= ST_ITER2;
    }
    if (lmove == 0 && !bresearch) {
      pick = pick_move(L, g->m2, stm, killer, counter, g->iid, ttmove, brandomize, prn, sT, C,
                       a.ocache ? g : nullptr, a.learned_top);
      if (pick >= 0) lmove = L[pick];
    }

    /* ---------------- move up (zeta.cl:2269-2451) ---------------- */
    const Move move = lmove;
    if (!bresearch) {
      if (move != E_NULLMOVE && move != 0) {
        if (g->state & ST_ITER1) g->m1[pick >> 6] &= ~(1ULL << (pick & 63));
        else g->m2[pick >> 6] &= ~(1ULL << (pick & 63));
        C[0]++;
      }
      g->todo++;
      g->mh = move;
      if (pick >= 0) g->mi = (uint8_t)pick;
    }
    EFrame *c = F + sd + 1;
    Pos np = g->pos;
    play(np, move, false);
    stm ^= 1;
    sd++;
    ply++;
    c->pos = np;
    u64 th = g->th ^ 1ULL ^ cr_keys(g->pos.cr) ^ cr_keys(np.cr); /* side to move, flags */
    if (move != 0 && move != E_NULLMOVE) th ^= piece_delta(move);
    c->th = th;
    const u64 h = th ^ (move == E_NULLMOVE ? 1ULL : 0ULL); /* the null move toggles once more */
    c->hash = h;
    if (tt1) prefetch_l2(tt1 + (h & mask1));
    if (tt2) prefetch_l2(tt2 + (h & mask2));
    if (ply + ply_init < kGamePly) H[ply + ply_init] = h;
    c->hmc = (uint8_t)next_hmc(g->hmc, move);
    c->mh = 0;
    c->iid = 0;
    c->mc = 0;
    c->todo = 0;
    c->alpha = -g->beta;
    c->beta = -g->alpha;
    c->depth = g->depth - 1;
    c->mode = g->mode;
    c->state = ST_ITER1;
    c->mi = 0;
    if (!bresearch && sd > 2 && !brandomize && move != E_NULLMOVE && move != 0 && ttmove == 0 && g->todo == 1 &&
        g->mc > 1 && g->depth > 5 && !(g->state & (ST_IID | ST_IIDDONE | ST_QS))) {
      /* internal iterative deepening: a shallow full-window pass first */
      g->state |= ST_IID;
      g->alpha = -E_INF;
      g->beta = E_INF;
      c->alpha = -E_INF;
      c->beta = E_INF;
    }
    if (g->state & ST_IID) {
      c->mode |= MD_IID;
      c->depth = g->depth / 5;
    }
    if (move == E_NULLMOVE) {
      g->todo--;
      c->mode |= MD_NULL;
      c->depth -= E_NULLR;
      c->alpha = -g->beta;
      c->beta = -g->beta + 1;
    }
    if (!bresearch && sd > 2 && move != E_NULLMOVE && move != 0 && (m_pcpt(move) >> 1) == PNONE &&
        !(g->state & (ST_IID | ST_QS | ST_KIC | ST_EXT)) && g->todo > 2 && g->depth >= 2 && popc(np.b0) >= 2 &&
        popc(np.b0 ^ (np.p1 | np.p2 | np.p3)) >= 2) {
      c->depth -= E_LMRR; /* late move reduction */
      g->state |= ST_LMR;
      c->mode |= MD_LMR;
    }
    if (sd == 2 && g->todo == 1) bestmove = move;
  }

  /* ---------------- PV (zeta.cl:2452-2511) ---------------- */
  if (!out_of_budget && ((volatile const uint32_t *)a.finito)[p] == (uint32_t)gid1) {
    uint32_t *PV = a.pv + (long long)p * kEPly;
    PV[0] = (uint32_t)bestscore;
    Pos b = root;
    int s = stm0;
    Move bm = bestmove;
    for (int k = 1; k < kEPly; k++) {
      PV[k] = bm;
      play(b, bm, false);
      s ^= 1;
      const u64 hh = compute_hash(b, s);
      bm = 0;
      int bsc = -E_INF;
      if (tt1) {
        const TT1E e = tt1_load(tt1 + (hh & mask1));
        if (tt1_ok(e, hh)) {
          bsc = e.score;
          bm = e.move;
        }
      }
      if (bm == 0 || is_inf(bsc)) break;
    }
  }
}

}  // namespace
}  // namespace zeta
