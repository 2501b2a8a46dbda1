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
 *               a subtree task when it is shallow enough (remaining depth
 *               <= task_depth, or <= 2 once a level holds min_tasks nodes),
 *               otherwise its children go to the next level
 *   k_perft_ws  persistent kernel, one worker per thread: tasks are dealt
 *               out as contiguous per-block ranges; a worker takes from its
 *               block's range and, when that is empty, steals from the
 *               other blocks' ranges (each range has one atomic cursor, so
 *               every task is taken exactly once and no wait is needed).
 *               A task is a depth-first walk whose last ply is counted with
 *               popcounts (count_legal), never expanded.
 *
 * The sequence is captured in a CUDA graph and replayed while the batch
 * shape stays the same.  Leaf counts are u64 and summed with atomics, so
 * the result does not depend on scheduling.
 */
#include <algorithm>
#include <cstdio>

#include "context.cuh"

namespace zeta {

namespace {

constexpr uint32_t ST_CAPACITY = 1u;
constexpr uint32_t ST_DEPTH = 2u;

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
__global__ void __launch_bounds__(128) k_split(int level, const Task *__restrict__ in, Task *__restrict__ out,
                                               Task *__restrict__ fin, uint32_t cap_lvl, uint32_t cap_fin,
                                               uint32_t min_tasks, int rmax, PerftCounters *pc) {
  const uint32_t n_in = pc->level_n[level];
  const int rmin = rmax < 2 ? rmax : 2;
  const bool last = level == kMaxLevels - 1;
  Move list[256];
  unsigned long long interior = 0;
  for (uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n_in; idx += gridDim.x * blockDim.x) {
    Task t = in[idx];
    int d = t.depth;
    bool split = (d > rmax) || (n_in < min_tasks && d > rmin);
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
    int nm = gen_legal(t.pos, t.stm, false, list);
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

template <int TPB>
__global__ void __launch_bounds__(TPB) k_perft_ws(const Task *__restrict__ tasks, uint32_t *cursors,
                                                  uint64_t *__restrict__ leaves, PerftCounters *pc) {
  const uint32_t n = min(pc->n_final, 0xFFFFFFFFu);
  const uint32_t B = gridDim.x;
  uint32_t victim = 0;
  unsigned long long steals = 0, interior = 0, counted = 0;

  Move l0[256], l1[256];
  int n0 = 0, i0 = 0, n1 = 0, i1 = 0;
  int R = -1;         /* remaining depth of the current task; -1 none, -2 count then finish */
  Pos base, mid;
  int sb = 0;
  uint32_t root = 0;
  unsigned long long acc = 0;

  for (;;) {
    Pos leaf;
    int sl = 0;
    bool have = false;
    /* advance to the next node whose children are the leaves */
    for (;;) {
      if (R == -1) {
        uint32_t idx;
        if (!take_task(cursors, n, B, victim, idx, steals)) break;
        Task t = tasks[idx];
        base = t.pos;
        sb = t.stm;
        root = t.root;
        R = t.depth;
        acc = 0;
        if (R == 0) {
          atomicAdd((unsigned long long *)&leaves[root], 1ULL);
          R = -1;
          continue;
        }
        if (R == 1) {
          leaf = base;
          sl = sb;
          R = -2;
          have = true;
          break;
        }
        n0 = gen_legal(base, sb, false, l0);
        interior++;
        i0 = 0;
        n1 = 0;
        i1 = 0;
      }
      if (R == 2) {
        if (i0 < n0) {
          leaf = base;
          play(leaf, l0[i0++], true);
          sl = sb ^ 1;
          have = true;
          break;
        }
      } else if (R == 3) {
        if (i1 < n1) {
          leaf = mid;
          play(leaf, l1[i1++], true);
          sl = sb;
          have = true;
          break;
        }
        if (i0 < n0) {
          mid = base;
          play(mid, l0[i0++], true);
          n1 = gen_legal(mid, sb ^ 1, false, l1);
          interior++;
          i1 = 0;
          continue;
        }
      }
      /* task done */
      if (acc) atomicAdd((unsigned long long *)&leaves[root], acc);
      R = -1;
    }
    if (!have) break;
    acc += (unsigned)count_legal(leaf, sl);
    counted++;
    if (R == -2) {
      if (acc) atomicAdd((unsigned long long *)&leaves[root], acc);
      R = -1;
    }
  }
  /* warp-aggregate the statistics */
  for (int o = 16; o > 0; o >>= 1) {
    steals += __shfl_down_sync(0xFFFFFFFFu, steals, o);
    interior += __shfl_down_sync(0xFFFFFFFFu, interior, o);
    counted += __shfl_down_sync(0xFFFFFFFFu, counted, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&pc->steals, steals);
    atomicAdd(&pc->interior, interior);
    atomicAdd(&pc->counted, counted);
  }
}

__global__ void k_genmoves(const uint64_t *__restrict__ boards, const uint8_t *__restrict__ stm, int n, int qs,
                           uint32_t *__restrict__ moves, int32_t *__restrict__ counts) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  Move list[256];
  Pos p = load_pos(boards + 7 * (size_t)i);
  int k = gen_legal(p, stm[i] & 1, qs != 0, list);
  counts[i] = k;
  for (int j = 0; j < k; j++) moves[(size_t)i * 256 + j] = list[j];
}

typedef void (*WsKernel)(const Task *, uint32_t *, uint64_t *, PerftCounters *);

WsKernel ws_kernel(int tpb) {
  switch (tpb) {
    case 64: return k_perft_ws<64>;
    case 128: return k_perft_ws<128>;
    case 256: return k_perft_ws<256>;
    case 512: return k_perft_ws<512>;
    default: return nullptr;
  }
}

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

static int ws_geometry(int &blocks, int &tpb) {
  Context &c = ctx();
  tpb = c.pcfg.threads_per_block;
  WsKernel k = ws_kernel(tpb);
  if (!k) return set_error(ZETA_ERR_ARG, "threads_per_block must be 64, 128, 256 or 512");
  int bps = c.pcfg.blocks_per_sm;
  if (bps <= 0) {
    ZCHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k, tpb, 0));
    if (bps < 1) bps = 1;
  }
  blocks = c.sms * bps;
  if (blocks > c.cursors_cap) {
    if (c.cursors) cudaFree(c.cursors);
    c.cursors = nullptr;
    ZCHECK(cudaMalloc(&c.cursors, blocks * sizeof(uint32_t)));
    c.cursors_cap = blocks;
    if (c.graph) {
      cudaGraphExecDestroy(c.graph);
      c.graph = nullptr;
    }
  }
  return ZETA_OK;
}

/* enqueue the whole launch sequence on `s` */
static int perft_enqueue(const uint64_t *d_boards, const uint8_t *d_stm, const uint8_t *d_depth, int n,
                         uint64_t *d_leaves, cudaStream_t s, int blocks, int tpb, bool timed, bool capturing) {
  Context &c = ctx();
  uint32_t min_tasks = c.pcfg.min_tasks ? c.pcfg.min_tasks : (uint32_t)(4ull * blocks * tpb);
  ZCHECK(cudaMemsetAsync(c.pc, 0, sizeof(PerftCounters), s));
  ZCHECK(cudaMemsetAsync(c.cursors, 0, blocks * sizeof(uint32_t), s));
  k_roots<<<(n + 127) / 128, 128, 0, s>>>(d_boards, d_stm, d_depth, n, c.lvl[0], d_leaves, c.pc);
  ZCHECK(cudaGetLastError());
  for (int lv = 0; lv < kMaxLevels; lv++) {
    k_split<<<c.sms * 4, 128, 0, s>>>(lv, c.lvl[lv & 1], c.lvl[(lv + 1) & 1], c.fin, c.cap_lvl, c.cap_fin,
                                      min_tasks, c.pcfg.task_depth, c.pc);
    ZCHECK(cudaGetLastError());
  }
  /* external records: inside a stream capture they become event-record
   * nodes of the graph, so the kernel can be timed on every replay */
  if (timed) ZCHECK(capturing ? cudaEventRecordWithFlags(c.ev[1], s, cudaEventRecordExternal) : cudaEventRecord(c.ev[1], s));
  ws_kernel(tpb)<<<blocks, tpb, 0, s>>>(c.fin, c.cursors, d_leaves, c.pc);
  ZCHECK(cudaGetLastError());
  if (timed) ZCHECK(capturing ? cudaEventRecordWithFlags(c.ev[2], s, cudaEventRecordExternal) : cudaEventRecord(c.ev[2], s));
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
  if (c.pcfg.task_depth < 1 || c.pcfg.task_depth > 3) return set_error(ZETA_ERR_ARG, "task_depth must be 1..3");
  int blocks, tpb;
  int rc = ws_geometry(blocks, tpb);
  if (rc) return rc;
  if (c.cap_fin == 0) {
    rc = perft_ensure_arena(8u << 20);
    if (rc) return rc;
  }
  ZCHECK(cudaEventRecord(c.ev[0], s));
  bool same = c.graph && c.g_boards == d_boards && c.g_stm == d_stm && c.g_depth == d_depth &&
              c.g_leaves == d_leaves && c.g_n == n && c.g_stream == s &&
              c.g_cfg.threads_per_block == c.pcfg.threads_per_block &&
              c.g_cfg.blocks_per_sm == c.pcfg.blocks_per_sm && c.g_cfg.min_tasks == c.pcfg.min_tasks &&
              c.g_cfg.task_depth == c.pcfg.task_depth;
  if (c.pcfg.use_graph) {
    if (!same) {
      if (c.graph) {
        cudaGraphExecDestroy(c.graph);
        c.graph = nullptr;
      }
      cudaGraph_t g;
      ZCHECK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
      rc = perft_enqueue(d_boards, d_stm, d_depth, n, d_leaves, s, blocks, tpb, true, true);
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
    }
    ZCHECK(cudaGraphLaunch(c.graph, s));
  } else {
    rc = perft_enqueue(d_boards, d_stm, d_depth, n, d_leaves, s, blocks, tpb, true, false);
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
    uint64_t need = std::max<uint64_t>(h.n_final, 0);
    for (int i = 0; i <= kMaxLevels; i++) need = std::max<uint64_t>(need, h.level_n[i]);
    perft_ensure_arena(need + need / 4 + 1024);
    return set_error(ZETA_ERR_CAPACITY, "perft task arena too small (%llu tasks needed); grown, retry",
                     (unsigned long long)need);
  }
  if (h.status & ST_DEPTH) return set_error(ZETA_ERR_ARG, "perft depth above %d", kMaxDepth);
  return ZETA_OK;
}

int genmoves_launch(const uint64_t *d_boards, const uint8_t *d_stm, int n, int qs, uint32_t *d_moves,
                    int32_t *d_counts, cudaStream_t s) {
  k_genmoves<<<(n + 127) / 128, 128, 0, s>>>(d_boards, d_stm, n, qs, d_moves, d_counts);
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
 * work-stealing cursors) in one fixed file-scope device array instead of
 * buffers allocated by the library.  The caller passes the inputs and
 * outputs, already in device memory. */
namespace {
constexpr uint32_t kNoAllocMaxTasks = 1u << 17; /* per task array: 131072 subtrees */
constexpr int kNoAllocMaxBlocks = 4096;         /* work-stealing cursors */

struct NoAllocScratch {
  PerftCounters pc;
  uint32_t cursors[kNoAllocMaxBlocks];
  Task lvl[2][kNoAllocMaxTasks];
  Task fin[kNoAllocMaxTasks];
};

/* about 19 MB; every GPU that loads the library holds it until exit */
static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(NoAllocScratch)];

constexpr int kNoAllocMaxDevices = 64;
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
  if (!g_noalloc_ptr[dev]) {
    void *p = nullptr;
    ZCHECK(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    int sms = 0, bps = 0;
    ZCHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    ZCHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_perft_ws<128>, 128, 0));
    int blocks = sms * (bps > 0 ? bps : 1);
    if (blocks > kNoAllocMaxBlocks) blocks = kNoAllocMaxBlocks;
    g_noalloc_sms[dev] = sms;
    g_noalloc_blocks[dev] = blocks;
    g_noalloc_ptr[dev] = (NoAllocScratch *)p;
  }
  NoAllocScratch *S = g_noalloc_ptr[dev];
  const int blocks = g_noalloc_blocks[dev], sms = g_noalloc_sms[dev];
  cudaStream_t s = (cudaStream_t)stream;
  /* the array keeps the previous call's contents: clear what must start at zero */
  ZCHECK(cudaMemsetAsync(&S->pc, 0, sizeof(PerftCounters), s));
  ZCHECK(cudaMemsetAsync(S->cursors, 0, blocks * sizeof(uint32_t), s));
  /* stop splitting early enough that the next level (about 35 children per
   * node) still fits the fixed task arrays */
  uint32_t min_tasks = (uint32_t)(4ull * blocks * 128);
  if (min_tasks > kNoAllocMaxTasks / 64) min_tasks = kNoAllocMaxTasks / 64;
  k_roots<<<(n + 127) / 128, 128, 0, s>>>(d_boards, d_stm, d_depth, n, S->lvl[0], d_leaves, &S->pc);
  ZCHECK(cudaGetLastError());
  for (int lv = 0; lv < kMaxLevels; lv++) {
    k_split<<<sms * 4, 128, 0, s>>>(lv, S->lvl[lv & 1], S->lvl[(lv + 1) & 1], S->fin, kNoAllocMaxTasks,
                                    kNoAllocMaxTasks, min_tasks, 3, &S->pc);
    ZCHECK(cudaGetLastError());
  }
  k_perft_ws<128><<<blocks, 128, 0, s>>>(S->fin, S->cursors, d_leaves, &S->pc);
  ZCHECK(cudaGetLastError());
  uint32_t status = 0;
  ZCHECK(cudaMemcpyAsync(&status, &S->pc.status, sizeof status, cudaMemcpyDeviceToHost, s));
  ZCHECK(cudaStreamSynchronize(s));
  if (status & ST_CAPACITY)
    return set_error(ZETA_ERR_NOALLOC, "the split needs more than %u subtree tasks (fixed scratch)", kNoAllocMaxTasks);
  if (status & ST_DEPTH) return set_error(ZETA_ERR_ARG, "perft depth above %d", kMaxDepth);
  return ZETA_OK;
}
