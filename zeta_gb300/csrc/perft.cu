/*
 * perft.cu -- batched perft on GB300.
 *
 * Replaces the reference's perft_gpu (zetaperft.cl:801-1477), which walks
 * one tree with one 64-work-item group, ten barriers per node and a move
 * stack in global memory.  Here one launch sequence handles a whole batch
 * of positions of any depth:
 *
 *   k_roots     batch -> level-0 tasks
 *   k_split     breadth-first split, one launch per level: a node becomes
 *               a subtree task when its remaining depth is <= task_depth
 *               (lower only while a level holds fewer than min_tasks
 *               nodes), otherwise its children go to the next level
 *   k_perft_ws  persistent kernel, one worker per thread block: tasks are
 *               dealt out as contiguous per-block ranges; a block takes
 *               from its own range and, when that is empty, steals from
 *               the other blocks' ranges (one atomic cursor per range, so
 *               every task is taken exactly once and nothing waits).
 *
 * A block runs its task breadth-first: the task root's children go to
 * shared memory, their children (the nodes one ply above the leaves) to a
 * per-block scratch area that stays in L2, and then every thread of the
 * block counts those nodes' legal moves with popcounts (count_legal)
 * instead of expanding them.  The counting phase, which is nearly all of
 * the work, runs with no divergence between threads.
 *
 * Promotions follow the reference (queen only) unless the caller asks for
 * all four pieces (zeta_perft_set_promotions): every kernel that generates
 * or counts moves is compiled in both forms (template flag ALLP), so the
 * reference's form pays nothing for the other.
 *
 * The sequence is captured in a CUDA graph and replayed while the batch
 * shape stays the same.  Leaf counts are u64 and summed with atomics, so
 * the result does not depend on scheduling.
 */
#include <algorithm>
#include <cstdio>
#include <mutex>

#include "context.cuh"
#include "movegen_fast.cuh"

namespace zeta {

namespace {

constexpr uint32_t ST_CAPACITY = 1u;
constexpr uint32_t ST_DEPTH = 2u;
constexpr uint32_t ST_BOUNDS = 4u; /* a write fell outside its buffer: skipped, reported */
constexpr int kMaxChildren = 218; /* most legal moves of any chess position */

__device__ __forceinline__ Pos load_pos(const uint64_t *b) {
  Pos p;
  p.b0 = b[0];
  p.p1 = b[1];
  p.p2 = b[2];
  p.p3 = b[3];
  p.cr = b[4];
  return p;
}

__global__ void k_roots(const uint64_t *__restrict__ boards, const uint8_t *__restrict__ stm,
                        const uint8_t *__restrict__ depth, int n, Task *__restrict__ out,
                        uint64_t *__restrict__ leaves, PerftCounters *pc) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) pc->level_n[0] = (uint32_t)n;
  if (i >= n) return;
  Task t;
  t.pos = load_pos(boards + 7 * (size_t)i);
  t.root = (uint32_t)i;
  t.stm = stm[i] & 1;
  uint8_t d = depth[i];
  if (d > kMaxDepth) {
    atomicOr(&pc->status, ST_DEPTH);
    d = 0;
  }
  t.depth = d;
  t.pad = 0;
  out[i] = t;
  leaves[i] = 0;
}

/* One split level: see the file comment. */
template <bool ALLP>
__global__ void __launch_bounds__(128) k_split(int level, const Task *__restrict__ in, Task *__restrict__ out,
                                               Task *__restrict__ fin, uint32_t cap_lvl, uint32_t cap_fin,
                                               uint32_t min_tasks, int rmax, PerftCounters *pc) {
  /* After an overflow (ST_CAPACITY, set by an earlier level) the call's
   * result is void and the host reports it; stop here.  A level that
   * overflowed holds an unwritten gap below its capacity (the reservation
   * that crossed the end was dropped whole), so its slots must not be read
   * as tasks. */
  if (pc->status & ST_CAPACITY) return;
  const uint32_t n_in = min(pc->level_n[level], cap_lvl);
  const bool last = level == kMaxLevels - 1;
  Move list[256];
  unsigned long long interior = 0;
  for (uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n_in; idx += gridDim.x * blockDim.x) {
    Task t = in[idx];
    int d = t.depth;
    bool split = (d > rmax) || (n_in < min_tasks && d > 1);
    if (split && last) {
      atomicOr(&pc->status, ST_DEPTH);
      continue;
    }
    if (!split) {
      uint32_t k = atomicAdd(&pc->n_final, 1u);
      if (k < cap_fin) fin[k] = t;
      else atomicOr(&pc->status, ST_CAPACITY);
      continue;
    }
    int nm = gen_legal<ALLP>(t.pos, t.stm, false, list);
    interior++;
    if (nm == 0) continue;
    uint32_t k = atomicAdd(&pc->level_n[level + 1], (uint32_t)nm);
    if (k + (uint32_t)nm > cap_lvl) {
      atomicOr(&pc->status, ST_CAPACITY);
      continue;
    }
    for (int j = 0; j < nm; j++) {
      Task c;
      c.pos = t.pos;
      play(c.pos, list[j], true);
      c.root = t.root;
      c.stm = t.stm ^ 1;
      c.depth = (uint8_t)(d - 1);
      c.pad = 0;
      out[k + j] = c;
    }
  }
  if (interior) atomicAdd(&pc->interior, interior);
}

/* Work-stealing deal: block b owns tasks [b*n/B, (b+1)*n/B).  `victim`
 * only moves forward, so a worker gives up after at most B empty ranges. */
__device__ __forceinline__ bool take_task(uint32_t *cursors, uint32_t n, uint32_t B, uint32_t &victim,
                                          uint32_t &idx, unsigned long long &steals) {
  while (victim < B) {
    uint32_t v = blockIdx.x + victim;
    v = v >= B ? v - B : v;
    uint64_t begin = (uint64_t)v * n / B, end = (uint64_t)(v + 1) * n / B;
    if (begin < end) {
      uint32_t i = atomicAdd(&cursors[v], 1u);
      if (begin + i < end) {
        idx = (uint32_t)(begin + i);
        steals += victim != 0;
        return true;
      }
    }
    victim++;
  }
  return false;
}

/* exclusive prefix sum over the block; returns the block total */
template <int TPB>
__device__ __forceinline__ int block_exclusive_scan(int v, int &excl, int *warp_tot) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xFFFFFFFFu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[warp] = x;
  __syncthreads();
  int before = 0, total = 0;
#pragma unroll
  for (int w = 0; w < TPB / 32; w++) {
    int t = warp_tot[w];
    before += (w < warp) ? t : 0;
    total += t;
  }
  excl = before + x - v;
  __syncthreads();
  return total;
}

template <int TPB>
__device__ __forceinline__ unsigned long long block_sum(unsigned long long v, unsigned long long *red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xFFFFFFFFu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  unsigned long long s = 0;
  if (threadIdx.x == 0)
#pragma unroll
    for (int w = 0; w < TPB / 32; w++) s += red[w];
  __syncthreads();
  return s;
}

/* One copy of each generator in the kernel's code: the kernels call them
 * from several places, and inlining every call overflows the
 * instruction cache. */
template <bool ALLP>
__device__ __noinline__ int count_node(Pos p, int stm) { return count_legal<ALLP>(p, stm); }
template <bool ALLP>
__device__ __noinline__ int expand_node(Pos p, int stm, Move *list) { return gen_legal<ALLP>(p, stm, false, list); }

/* Expand src[0..nsrc) (nsrc <= TPB, one node per thread) into dst,
 * children of a node contiguous; returns the number written.  Block-wide:
 * every thread must call it. */
template <int TPB, bool ALLP>
__device__ __forceinline__ int expand_round(const Pos *src, int nsrc, int stm, Pos *dst, int dst_cap, int *s_warp,
                                            Move *list, unsigned long long &interior, uint32_t *status) {
  const int tid = threadIdx.x;
  int k = 0;
  if (tid < nsrc) {
    k = expand_node<ALLP>(src[tid], stm, list);
    interior++;
  }
  int off;
  const int total = block_exclusive_scan<TPB>(k, off, s_warp);
  if (off + k > dst_cap) {
    atomicOr(status, ST_BOUNDS);
    k = off < dst_cap ? dst_cap - off : 0;
  }
  for (int j = 0; j < k; j++) {
    Pos c = src[tid];
    play(c, list[j], true);
    dst[off + j] = c;
  }
  __syncthreads();
  return total < dst_cap ? total : dst_cap;
}

/* sum of the legal-move counts of src[0..n): the leaf count below them */
template <int TPB, bool ALLP>
__device__ __forceinline__ unsigned long long count_range(const Pos *src, int n, int stm, unsigned long long &counted) {
  unsigned long long acc = 0;
  for (int j = threadIdx.x; j < n; j += TPB) {
    acc += (unsigned)count_node<ALLP>(src[j], stm);
    counted++;
  }
  return acc;
}

/* Per-block scratch: `cap2` positions for a depth-4 task's second level
 * (218*218 covers any position) and `cap3` for the nodes one ply above the
 * leaves; each round expands at most cap3/218 parents, so it never
 * overflows. */
template <int TPB, int MINB, bool ALLP>
__global__ void __launch_bounds__(TPB, MINB) k_perft_ws(const Task *__restrict__ tasks, uint32_t *cursors,
                                                  uint64_t *__restrict__ leaves, PerftCounters *pc,
                                                  Pos *__restrict__ scratch, uint32_t cap2, uint32_t cap3,
                                                  uint32_t cap_fin, uint32_t n_roots) {
  __shared__ Pos s_l1[256];
  __shared__ Pos s_root;
  __shared__ int s_warp[TPB / 32];
  __shared__ unsigned long long s_red[TPB / 32];
  __shared__ uint32_t s_task;

  const int tid = threadIdx.x;
  /* a split level overflowed: the task set is incomplete and the host
   * reports the call as failed; every block leaves at once (uniformly: only
   * the split kernels set this bit) */
  if (pc->status & ST_CAPACITY) return;
  const uint32_t n = min(pc->n_final, cap_fin); /* tasks beyond the array were not stored */
  const uint32_t B = gridDim.x;
  const int per_round = min(TPB, (int)(cap3 / kMaxChildren));
  Pos *b2 = scratch + (size_t)blockIdx.x * (cap2 + cap3);
  Pos *b3 = b2 + cap2;
  uint32_t victim = 0;
  unsigned long long steals = 0, interior = 0, counted = 0;
  Move list[256];

  for (;;) {
    if (tid == 0) {
      uint32_t idx;
      s_task = take_task(cursors, n, B, victim, idx, steals) ? idx : 0xFFFFFFFFu;
    }
    __syncthreads();
    const uint32_t ti = s_task;
    if (ti == 0xFFFFFFFFu) break;
    const Task t = tasks[ti];
    const int R = t.depth;
    unsigned long long acc = 0;
    if (tid == 0) s_root = t.pos;
    __syncthreads();
    if (R == 0) {
      acc = tid == 0;
    } else if (R == 1) {
      acc = count_range<TPB, ALLP>(&s_root, 1, t.stm, counted);
    } else {
      /* level 1: the task root's children, in shared memory */
      const int n1 = expand_round<TPB, ALLP>(&s_root, 1, t.stm, s_l1, 256, s_warp, list, interior, &pc->status);
      if (R == 2) {
        acc = count_range<TPB, ALLP>(s_l1, n1, t.stm ^ 1, counted);
      } else {
        /* R == 4: level 2 in full into the block's level-2 buffer */
        const Pos *par = s_l1;
        int npar = n1, spar = t.stm ^ 1;
        if (R == 4) {
          int n2 = 0;
          for (int base = 0; base < n1; base += TPB)
            n2 += expand_round<TPB, ALLP>(s_l1 + base, min(TPB, n1 - base), t.stm ^ 1, b2 + n2, (int)cap2 - n2, s_warp,
                                    list, interior, &pc->status);
          par = b2;
          npar = n2;
          spar = t.stm;
        }
        /* the nodes one ply above the leaves, a round at a time, then count */
        for (int base = 0; base < npar; base += per_round) {
          const int total = expand_round<TPB, ALLP>(par + base, min(per_round, npar - base), spar, b3, (int)cap3, s_warp,
                                              list, interior, &pc->status);
          acc += count_range<TPB, ALLP>(b3, total, spar ^ 1, counted);
          __syncthreads();
        }
      }
    }
    const unsigned long long sum = block_sum<TPB>(acc, s_red);
    if (tid == 0 && sum) {
      if (t.root < n_roots) atomicAdd((unsigned long long *)&leaves[t.root], sum);
      else atomicOr(&pc->status, ST_BOUNDS);
    }
  }
  /* warp-aggregate the statistics */
  for (int o = 16; o > 0; o >>= 1) {
    steals += __shfl_down_sync(0xFFFFFFFFu, steals, o);
    interior += __shfl_down_sync(0xFFFFFFFFu, interior, o);
    counted += __shfl_down_sync(0xFFFFFFFFu, counted, o);
  }
  if ((tid & 31) == 0) {
    if (steals) atomicAdd(&pc->steals, steals);
    atomicAdd(&pc->interior, interior);
    atomicAdd(&pc->counted, counted);
  }
}

/* one thread per position: gen 0 the perft generator (gen_legal; allp:
 * all four promotions), 1 the search engine's (gen_engine) */
__global__ void k_genmoves(const uint64_t *__restrict__ boards, const uint8_t *__restrict__ stm, int n, int qs,
                           int gen, int allp, uint32_t *__restrict__ moves, int32_t *__restrict__ counts) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  Move list[256];
  Pos p = load_pos(boards + 7 * (size_t)i);
  int k;
  if (gen == 1) {
    const Sets sets = make_sets(p, stm[i] & 1);
    k = gen_engine(p, sets, enemy_attacks(sets, stm[i] & 1), stm[i] & 1, qs != 0, list);
  } else if (allp) {
    k = gen_legal<true>(p, stm[i] & 1, qs != 0, list);
  } else {
    k = gen_legal(p, stm[i] & 1, qs != 0, list);
  }
  counts[i] = k;
  for (int j = 0; j < k; j++) moves[(size_t)i * 256 + j] = list[j];
}

typedef void (*WsKernel)(const Task *, uint32_t *, uint64_t *, PerftCounters *, Pos *, uint32_t, uint32_t,
                         uint32_t, uint32_t);

/* Compiled variants: threads per block x minimum resident blocks per SM
 * (the second number caps registers per thread at 65536/(TPB*MINB));
 * blocks_per_sm == 0 selects the uncapped variant.  Caps of 64 registers
 * (128x8, 256x4, 512x2) are not built: 128x8 raised an illegal-address
 * fault on GB300 at task depth 3 with its bounds checks silent. */
template <bool ALLP>
WsKernel ws_kernel_of(int tpb, int minb) {
  switch (tpb * 100 + minb) {
    case 6400: return k_perft_ws<64, 1, ALLP>;
    case 6408: return k_perft_ws<64, 8, ALLP>;
    case 6412: return k_perft_ws<64, 12, ALLP>;
    case 12800: return k_perft_ws<128, 1, ALLP>;
    case 12804: return k_perft_ws<128, 4, ALLP>;
    case 12806: return k_perft_ws<128, 6, ALLP>;
    case 25600: return k_perft_ws<256, 1, ALLP>;
    case 25603: return k_perft_ws<256, 3, ALLP>;
    case 51200: return k_perft_ws<512, 1, ALLP>;
    default: return nullptr;
  }
}
WsKernel ws_kernel(int tpb, int minb, bool allp) {
  return allp ? ws_kernel_of<true>(tpb, minb) : ws_kernel_of<false>(tpb, minb);
}
typedef void (*SplitKernel)(int, const Task *, Task *, Task *, uint32_t, uint32_t, uint32_t, int, PerftCounters *);
SplitKernel split_kernel(bool allp) { return allp ? k_split<true> : k_split<false>; }

}  // namespace

int perft_ensure_arena(uint64_t tasks_cap) {
  Context &c = ctx();
  if (tasks_cap <= c.cap_fin) return ZETA_OK;
  if (tasks_cap > 0xF0000000ull) return set_error(ZETA_ERR_CAPACITY, "perft arena request too large");
  for (int i = 0; i < 2; i++)
    if (c.lvl[i]) cudaFree(c.lvl[i]);
  if (c.fin) cudaFree(c.fin);
  c.lvl[0] = c.lvl[1] = c.fin = nullptr;
  c.cap_lvl = c.cap_fin = 0;
  ZCHECK(cudaMalloc(&c.lvl[0], tasks_cap * sizeof(Task)));
  ZCHECK(cudaMalloc(&c.lvl[1], tasks_cap * sizeof(Task)));
  ZCHECK(cudaMalloc(&c.fin, tasks_cap * sizeof(Task)));
  c.cap_lvl = c.cap_fin = (uint32_t)tasks_cap;
  if (c.graph) {
    cudaGraphExecDestroy(c.graph);
    c.graph = nullptr;
  }
  return ZETA_OK;
}

int perft_run(const uint64_t *d_boards, const uint8_t *d_stm, const uint8_t *d_depth, int n, uint64_t *d_leaves,
              cudaStream_t s);

/* Per-thread stack for kernel k.  Every perft kernel keeps a 256-move list
 * on its stack and the register-capped variants spill next to it (1024 to
 * 1152 bytes; the 64-register variants, which are not built, needed 1264),
 * above CUDA's 1 KB default.  The driver grows the stack when a kernel is
 * launched directly; this path replays its launches from a CUDA graph, so
 * the stack is sized here, before the sequence is captured, instead of
 * relying on that. */
static int ensure_stack(const void *k) {
  cudaFuncAttributes fa;
  ZCHECK(cudaFuncGetAttributes(&fa, k));
  size_t cur = 0;
  ZCHECK(cudaDeviceGetLimit(&cur, cudaLimitStackSize));
  if (fa.localSizeBytes > cur) ZCHECK(cudaDeviceSetLimit(cudaLimitStackSize, fa.localSizeBytes));
  return ZETA_OK;
}

/* grid of the work-stealing kernel, cursors and per-block scratch */
static int ws_geometry(int &blocks, int &tpb, WsKernel &k) {
  Context &c = ctx();
  tpb = c.pcfg.threads_per_block;
  k = ws_kernel(tpb, c.pcfg.blocks_per_sm, c.perft_allp != 0);
  if (!k)
    return set_error(ZETA_ERR_ARG, "no perft kernel variant for %d threads x %d blocks per SM", tpb,
                     c.pcfg.blocks_per_sm);
  int rc = ensure_stack((const void *)k);
  if (!rc) rc = ensure_stack((const void *)split_kernel(c.perft_allp != 0));
  if (rc) return rc;
  int bps = 0;
  ZCHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k, tpb, 0));
  if (bps < 1) bps = 1;
  blocks = c.sms * bps;
  const uint32_t cap2 = c.pcfg.task_depth >= 4 ? (uint32_t)(kMaxChildren * kMaxChildren) : 0u;
  const uint32_t cap = cap2 + (uint32_t)tpb * kMaxChildren;
  bool regrow = blocks > c.cursors_cap || (uint64_t)blocks * cap > c.scratch_cap;
  if (regrow) {
    if (c.cursors) cudaFree(c.cursors);
    if (c.scratch) cudaFree(c.scratch);
    c.cursors = nullptr;
    c.scratch = nullptr;
    c.cursors_cap = 0;
    c.scratch_cap = 0;
    ZCHECK(cudaMalloc(&c.cursors, blocks * sizeof(uint32_t)));
    c.cursors_cap = blocks;
    ZCHECK(cudaMalloc(&c.scratch, (size_t)blocks * cap * sizeof(Pos)));
    c.scratch_cap = (uint64_t)blocks * cap;
    if (c.graph) {
      cudaGraphExecDestroy(c.graph);
      c.graph = nullptr;
    }
  }
  return ZETA_OK;
}

/* enqueue the whole launch sequence on `s` */
static int perft_enqueue(const uint64_t *d_boards, const uint8_t *d_stm, const uint8_t *d_depth, int n,
                         uint64_t *d_leaves, cudaStream_t s, int blocks, int tpb, WsKernel k, bool capturing) {
  Context &c = ctx();
  const uint32_t min_tasks = c.pcfg.min_tasks; /* 0: never split below task_depth */
  ZCHECK(cudaMemsetAsync(c.pc, 0, sizeof(PerftCounters), s));
  ZCHECK(cudaMemsetAsync(c.cursors, 0, blocks * sizeof(uint32_t), s));
  k_roots<<<(n + 127) / 128, 128, 0, s>>>(d_boards, d_stm, d_depth, n, c.lvl[0], d_leaves, c.pc);
  ZCHECK(cudaGetLastError());
  const SplitKernel split = split_kernel(c.perft_allp != 0);
  for (int lv = 0; lv < kMaxLevels; lv++) {
    split<<<c.sms * 4, 128, 0, s>>>(lv, c.lvl[lv & 1], c.lvl[(lv + 1) & 1], c.fin, c.cap_lvl, c.cap_fin,
                                    min_tasks, c.pcfg.task_depth, c.pc);
    ZCHECK(cudaGetLastError());
  }
  /* external records: inside a stream capture they become event-record
   * nodes of the graph, so the kernel is timed on every replay */
  ZCHECK(capturing ? cudaEventRecordWithFlags(c.ev[1], s, cudaEventRecordExternal) : cudaEventRecord(c.ev[1], s));
  const uint32_t cap2 = c.pcfg.task_depth >= 4 ? (uint32_t)(kMaxChildren * kMaxChildren) : 0u;
  k<<<blocks, tpb, 0, s>>>(c.fin, c.cursors, d_leaves, c.pc, c.scratch, cap2, (uint32_t)tpb * kMaxChildren,
                           c.cap_fin, (uint32_t)n);
  ZCHECK(cudaGetLastError());
  ZCHECK(capturing ? cudaEventRecordWithFlags(c.ev[2], s, cudaEventRecordExternal) : cudaEventRecord(c.ev[2], s));
  return ZETA_OK;
}

int perft_launch(const uint64_t *d_boards, const uint8_t *d_stm, const uint8_t *d_depth, int n, uint64_t *d_leaves,
                 cudaStream_t user) {
  Context &c = ctx();
  if (n <= 0) return set_error(ZETA_ERR_ARG, "batch size must be positive");
  /* the legacy default stream cannot be captured: run on the library's
   * stream, ordered after the caller's work and before its next work */
  cudaStream_t s = user;
  bool joined = false;
  if (user == nullptr || user == cudaStreamLegacy || user == cudaStreamPerThread) {
    s = c.stream;
    joined = true;
    ZCHECK(cudaEventRecord(c.ev_join[0], user));
    ZCHECK(cudaStreamWaitEvent(s, c.ev_join[0], 0));
  }
  int rc = perft_run(d_boards, d_stm, d_depth, n, d_leaves, s);
  if (joined) {
    ZCHECK(cudaEventRecord(c.ev_join[1], s));
    ZCHECK(cudaStreamWaitEvent(user, c.ev_join[1], 0));
  }
  return rc;
}

int perft_run(const uint64_t *d_boards, const uint8_t *d_stm, const uint8_t *d_depth, int n, uint64_t *d_leaves,
              cudaStream_t s) {
  Context &c = ctx();
  if (c.pcfg.task_depth < 1 || c.pcfg.task_depth > 4) return set_error(ZETA_ERR_ARG, "task_depth must be 1..4");
  int blocks, tpb;
  WsKernel k;
  int rc = ws_geometry(blocks, tpb, k);
  if (rc) return rc;
  if (c.cap_fin == 0 || (uint32_t)n > c.cap_lvl) {
    rc = perft_ensure_arena(std::max<uint64_t>(8u << 20, (uint64_t)n + n / 4)); /* the roots fit level 0 */
    if (rc) return rc;
  }
  ZCHECK(cudaEventRecord(c.ev[0], s));
  bool same = c.graph && c.g_boards == d_boards && c.g_stm == d_stm && c.g_depth == d_depth &&
              c.g_leaves == d_leaves && c.g_n == n && c.g_stream == s &&
              c.g_cfg.threads_per_block == c.pcfg.threads_per_block &&
              c.g_cfg.blocks_per_sm == c.pcfg.blocks_per_sm && c.g_cfg.min_tasks == c.pcfg.min_tasks &&
              c.g_cfg.task_depth == c.pcfg.task_depth && c.g_allp == c.perft_allp;
  if (c.pcfg.use_graph) {
    if (!same) {
      if (c.graph) {
        cudaGraphExecDestroy(c.graph);
        c.graph = nullptr;
      }
      cudaGraph_t g;
      ZCHECK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
      rc = perft_enqueue(d_boards, d_stm, d_depth, n, d_leaves, s, blocks, tpb, k, true);
      cudaError_t e = cudaStreamEndCapture(s, &g);
      if (rc) return rc;
      if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
      e = cudaGraphInstantiate(&c.graph, g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
      c.g_boards = d_boards;
      c.g_stm = d_stm;
      c.g_depth = d_depth;
      c.g_leaves = d_leaves;
      c.g_n = n;
      c.g_stream = s;
      c.g_cfg = c.pcfg;
      c.g_allp = c.perft_allp;
    }
    ZCHECK(cudaGraphLaunch(c.graph, s));
  } else {
    rc = perft_enqueue(d_boards, d_stm, d_depth, n, d_leaves, s, blocks, tpb, k, false);
    if (rc) return rc;
  }
  ZCHECK(cudaEventRecord(c.ev[3], s));
  PerftCounters h;
  ZCHECK(cudaMemcpyAsync(&h, c.pc, sizeof h, cudaMemcpyDeviceToHost, s));
  ZCHECK(cudaStreamSynchronize(s));
  c.pstats.tasks = h.n_final;
  c.pstats.steals = h.steals;
  c.pstats.interior_nodes = h.interior;
  c.pstats.counted_nodes = h.counted;
  if (cudaEventElapsedTime(&c.pstats.kernel_ms, c.ev[1], c.ev[2]) != cudaSuccess) c.pstats.kernel_ms = -1.f;
  if (cudaEventElapsedTime(&c.pstats.total_ms, c.ev[0], c.ev[3]) != cudaSuccess) c.pstats.total_ms = -1.f;
  (void)cudaGetLastError(); /* a failed timing query must not poison the next call */
  if (h.status & ST_CAPACITY) {
    /* grow the arena for the next call and report */
    uint64_t need = h.n_final;
    for (int i = 0; i <= kMaxLevels; i++) need = std::max<uint64_t>(need, h.level_n[i]);
    perft_ensure_arena(need + need / 4 + 1024);
    return set_error(ZETA_ERR_CAPACITY, "perft task arena too small (%llu tasks needed); grown, retry",
                     (unsigned long long)need);
  }
  if (h.status & ST_DEPTH) return set_error(ZETA_ERR_ARG, "perft depth above %d", kMaxDepth);
  if (h.status & ST_BOUNDS) return set_error(ZETA_ERR_DEVICE, "perft: a buffer bound was hit (write skipped)");
  return ZETA_OK;
}

int genmoves_launch(const uint64_t *d_boards, const uint8_t *d_stm, int n, int flags, uint32_t *d_moves,
                    int32_t *d_counts, cudaStream_t s) {
  const int qs = flags & 1, gen = (flags >> 1) & 3, allp = (flags >> 3) & 1;
  if (gen > 2) return set_error(ZETA_ERR_ARG, "genmoves: unknown generator");
  if (allp && gen != 0) return set_error(ZETA_ERR_ARG, "genmoves: all promotions only with the perft generator");
  if (gen == 2) return warp_genmoves_launch(d_boards, d_stm, n, qs, d_moves, d_counts, s);
  k_genmoves<<<(n + 127) / 128, 128, 0, s>>>(d_boards, d_stm, n, qs, gen, allp, d_moves, d_counts);
  ZCHECK(cudaGetLastError());
  ZCHECK(cudaStreamSynchronize(s));
  return ZETA_OK;
}

/* ------------------------------------------------------------------ */
/* Batched perft for callers that cannot allocate device memory.
 *
 * Some programs that embed the engine own every byte of device memory
 * themselves (a host application with a fixed memory budget and its own
 * pool), or run a latency-critical loop in which a cudaMalloc -- which
 * may synchronise the whole device -- is not acceptable.  For them,
 * zeta_perft_batch_noalloc runs the same launch sequence as
 * zeta_perft_batch_device with all of its scratch (task arrays, counters,
 * work-stealing cursors, per-block node buffers) in one fixed file-scope
 * device array instead of buffers allocated by the library.  The caller
 * passes the inputs and outputs, already in device memory. */
namespace {
constexpr uint32_t kNoAllocMaxTasks = 1u << 17; /* per task array: 131072 subtrees */
constexpr int kNoAllocMaxBlocks = 256;          /* worker blocks */
constexpr uint32_t kNoAllocNodesPerBlock = 1024; /* per-block node buffer */

struct NoAllocScratch {
  PerftCounters pc;
  uint32_t cursors[kNoAllocMaxBlocks];
  Task lvl[2][kNoAllocMaxTasks];
  Task fin[kNoAllocMaxTasks];
  Pos nodes[kNoAllocMaxBlocks * kNoAllocNodesPerBlock];
};

/* about 29 MB; every GPU that loads the library holds it until exit */
static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(NoAllocScratch)];

constexpr int kNoAllocMaxDevices = 64;
/* per-device set-up results, written and read under g_noalloc_mu so that
 * a host thread never sees the address without the launch geometry */
std::mutex g_noalloc_mu;
NoAllocScratch *g_noalloc_ptr[kNoAllocMaxDevices] = {nullptr};
int g_noalloc_sms[kNoAllocMaxDevices] = {0};
int g_noalloc_blocks[kNoAllocMaxDevices] = {0};
}  // namespace

}  // namespace zeta

using namespace zeta;

extern "C" int zeta_perft_batch_noalloc(const uint64_t *d_boards, const uint8_t *d_stm, const uint8_t *d_depth,
                                        int n, uint64_t *d_leaves, void *stream) {
  if (!d_boards || !d_stm || !d_depth || !d_leaves) return set_error(ZETA_ERR_ARG, "null buffer");
  if (n <= 0 || (uint32_t)n > kNoAllocMaxTasks)
    return set_error(ZETA_ERR_NOALLOC, "batch of %d positions outside 1..%u (fixed scratch)", n, kNoAllocMaxTasks);
  int dev = 0;
  ZCHECK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kNoAllocMaxDevices) return set_error(ZETA_ERR_ARG, "device %d out of range", dev);
  /* set-up, once per device, with that device current: the host-side name
   * of the array is not a device address, so look the address up */
  NoAllocScratch *S = nullptr;
  int blocks = 0, sms = 0;
  {
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
      void *p = nullptr;
      ZCHECK(cudaGetSymbolAddress(&p, g_noalloc_scratch));
      int nsm = 0, bps = 0;
      ZCHECK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
      ZCHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_perft_ws<128, 1, false>, 128, 0));
      int nb = nsm * (bps > 0 ? bps : 1);
      if (nb > kNoAllocMaxBlocks) nb = kNoAllocMaxBlocks;
      g_noalloc_sms[dev] = nsm;
      g_noalloc_blocks[dev] = nb;
      g_noalloc_ptr[dev] = (NoAllocScratch *)p;
    }
    S = g_noalloc_ptr[dev];
    blocks = g_noalloc_blocks[dev];
    sms = g_noalloc_sms[dev];
  }
  cudaStream_t s = (cudaStream_t)stream;
  /* the array keeps the previous call's contents: clear what must start at zero */
  ZCHECK(cudaMemsetAsync(&S->pc, 0, sizeof(PerftCounters), s));
  ZCHECK(cudaMemsetAsync(S->cursors, 0, blocks * sizeof(uint32_t), s));
  const bool allp = ctx().perft_allp != 0;
  k_roots<<<(n + 127) / 128, 128, 0, s>>>(d_boards, d_stm, d_depth, n, S->lvl[0], d_leaves, &S->pc);
  ZCHECK(cudaGetLastError());
  const SplitKernel split = split_kernel(allp);
  for (int lv = 0; lv < kMaxLevels; lv++) {
    split<<<sms * 4, 128, 0, s>>>(lv, S->lvl[lv & 1], S->lvl[(lv + 1) & 1], S->fin, kNoAllocMaxTasks,
                                  kNoAllocMaxTasks, 0u, 3, &S->pc);
    ZCHECK(cudaGetLastError());
  }
  /* blocks_per_sm 0 names the uncapped variant, k_perft_ws<128, 1, allp> */
  const WsKernel ws = ws_kernel(128, 0, allp);
  if (!ws) return set_error(ZETA_ERR_ARG, "no perft kernel variant for the allocation-free entry");
  ws<<<blocks, 128, 0, s>>>(S->fin, S->cursors, d_leaves, &S->pc, S->nodes, 0u, kNoAllocNodesPerBlock,
                            kNoAllocMaxTasks, (uint32_t)n);
  ZCHECK(cudaGetLastError());
  uint32_t status = 0;
  ZCHECK(cudaMemcpyAsync(&status, &S->pc.status, sizeof status, cudaMemcpyDeviceToHost, s));
  ZCHECK(cudaStreamSynchronize(s));
  if (status & ST_CAPACITY)
    return set_error(ZETA_ERR_NOALLOC, "the split needs more than %u subtree tasks (fixed scratch)", kNoAllocMaxTasks);
  if (status & ST_DEPTH) return set_error(ZETA_ERR_ARG, "perft depth above %d", kMaxDepth);
  if (status & ST_BOUNDS) return set_error(ZETA_ERR_DEVICE, "perft: a buffer bound was hit (write skipped)");
  return ZETA_OK;
}
